"""The compressor's conjugate-gradient iteration (zcg_grid_kernel,
carcassonne_gb300/csrc/cg.cu; the host form in compression._cg_host)
restated in numpy, to show on the CPU why it keeps its best iterate.

The normal equations G x = c of the product compressor are singular and, once
formed in floating point, slightly inconsistent: c has a rounding-level part
outside the range of G.  Plain CG then steps along G's near-null directions
with huge step sizes: the iterate grows far beyond the least-squares solution
and the residual rises, until p^H G p <= 0 stops it.  The kernel keeps the
iterate with the smallest residual, stops once the residual is 1e8 above it,
and reports the true residual of what it returns.  No GPU is used."""
import numpy as np
import pytest


def cg(G, c, tol=1e-12, max_iter=None, keep_best=True):
    """(x, true relative residual, iterations) under the kernel's rules, or
    plain CG's (``keep_best=False``)."""
    n = len(c)
    max_iter = max_iter or max(10 * n, 500)
    x = np.zeros(n, complex)
    r = c.copy()
    p = r.copy()
    rr = c2 = float(np.vdot(r, r).real)
    best, xb, last = rr, x.copy(), rr
    it = 0
    while it < max_iter:
        gp = G @ p
        pgp = float(np.vdot(p, gp).real)
        if not pgp > 0.0:
            break
        alpha = rr / pgp
        x = x + alpha * p
        r = r - alpha * gp
        rn = float(np.vdot(r, r).real)
        it += 1
        last = rn
        if rn < best:
            best, xb = rn, x.copy()
        if rn <= tol * tol * c2:
            break
        if keep_best and rn > 1e8 * best:
            break
        p = r + (rn / rr) * p
        rr = rn
    out = xb if (keep_best and best < last) else x
    return out, float(np.linalg.norm(c - G @ out) / np.sqrt(c2)), it


def _system(n, rank, outside, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, rank)) + 1j * rng.standard_normal((n, rank))
    G = a @ a.conj().T / rank
    c = G @ (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    if outside:
        w, v = np.linalg.eigh(G)
        z = v[:, : n - rank] @ (rng.standard_normal(n - rank) + 1j * rng.standard_normal(n - rank))
        c = c + outside * np.linalg.norm(c) * z / np.linalg.norm(z)
    return G, c


@pytest.mark.parametrize("n,rank", [(64, 16), (128, 24)])
def test_plain_cg_grows_on_an_inconsistent_singular_system(n, rank):
    G, c = _system(n, rank, 1e-9, n)
    x_ls = np.linalg.pinv(G, rcond=1e-12) @ c
    x, res, _ = cg(G, c, keep_best=False)
    assert np.linalg.norm(x) > 1e3 * np.linalg.norm(x_ls)
    assert res > 1e-6


@pytest.mark.parametrize("n,rank", [(64, 16), (128, 24)])
def test_best_iterate_is_the_least_squares_solution(n, rank):
    G, c = _system(n, rank, 1e-9, n)
    x_ls = np.linalg.pinv(G, rcond=1e-12) @ c
    x, res, _ = cg(G, c)
    assert 5e-10 <= res <= 2e-9  # the part of c outside G's range, and no more
    assert np.linalg.norm(x - x_ls) <= 1e-6 * np.linalg.norm(x_ls)


def test_consistent_systems_converge_to_the_tolerance():
    for n, rank in ((64, 64), (64, 16)):
        G, c = _system(n, rank, 0.0, 7 + rank)
        x, res, it = cg(G, c)
        assert res <= 1e-11 and it <= 10 * n
