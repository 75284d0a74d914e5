"""The MLP oracle's gradients against central finite differences (CPU)."""
import numpy as np

from oracle import mlp_oracle as mo


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    sizes = [7, 11, 9, 5]
    params = [(rng.standard_normal((o, i)) * 0.5, rng.standard_normal(o) * 0.1) for i, o in zip(sizes, sizes[1:])]
    X = rng.standard_normal((6, sizes[0]))
    T = rng.standard_normal((6, sizes[-1]))
    _, grads = mo.loss_and_grads(params, X, T)
    h = 1e-6
    for li, (W, b) in enumerate(params):
        for arr, g in ((W, grads[li][0]), (b, grads[li][1])):
            flat = arr.reshape(-1)
            for idx in rng.choice(flat.size, size=min(8, flat.size), replace=False):
                old = flat[idx]
                flat[idx] = old + h
                lp, _ = mo.loss_and_grads(params, X, T)
                flat[idx] = old - h
                lm, _ = mo.loss_and_grads(params, X, T)
                flat[idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - g.reshape(-1)[idx]) <= 1e-6 * max(1.0, abs(fd)), (li, idx, fd, g.reshape(-1)[idx])


def test_oracle_adam_matches_closed_form_first_step():
    p, g = np.array([1.0, -2.0]), np.array([0.5, -0.25])
    p1, m, v = mo.adam(p, g, np.zeros(2), np.zeros(2), 0.1, 0.9, 0.999, 1e-8, 1)
    # first bias-corrected step moves each parameter by lr * sign(g)
    assert np.allclose(p1, p - 0.1 * np.sign(g), atol=1e-6)
