"""Learned Lanczos start vector for the center-site solve.

The reference starts each center solve from the previous center (the gauge-
moved old iterate, system/_2d.py:435-439 and :491-492).  Here a small fully
connected network proposes the start instead, from compressed boundary
features: the top-k singular values of the Identity tag of each of the four
corners and four sides (k = 16), plus the field h.  Its target is the
converged center of the plain FP64 solve, normalized and phase-fixed against a
fixed reference vector, as 2N real numbers (real, imaginary parts).

Training (FP32) and inference (BF16 weights and activations, FP32
accumulation) run on the project's own kernels (csrc/mlp.cu): no framework
autograd.  The eigensolver judges the proposal: the start only changes how
many Lanczos iterations the solve takes, never its result, and the plain
previous-iterate or fixed start remains the fallback (``x0=None``).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib, linalg, workloads
from .data import TorchData
from .engine import CDT, current_stream_handle
from .tensors._2d import sparse as tsp
from .sparse import Identity


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class StartMLP:
    """3-layer MLP (n_in -> width -> width -> n_out), ReLU hidden layers."""

    def __init__(self, n_in, n_out, width=256, depth=3, seed=0, device="cuda"):
        g = torch.Generator().manual_seed(seed)
        sizes = [n_in] + [width] * (depth - 1) + [n_out]
        self.sizes = sizes
        self.W, self.b = [], []
        for i, o in zip(sizes, sizes[1:]):
            self.W.append((torch.randn(o, i, generator=g) * (2.0 / i) ** 0.5).float().to(device))
            self.b.append(torch.zeros(o, dtype=torch.float32, device=device))
        self.m = [torch.zeros_like(p) for p in self.params()]
        self.v = [torch.zeros_like(p) for p in self.params()]
        self.steps = 0
        self._bf16 = None
        self.x_mean = None
        self.x_std = None

    def params(self):
        out = []
        for W, b in zip(self.W, self.b):
            out += [W, b]
        return out

    # -- FP32 training path ------------------------------------------------
    def forward(self, X):
        lib = _lib.load()
        acts = [X.contiguous().float()]
        for li, (W, b) in enumerate(zip(self.W, self.b)):
            B, K = acts[-1].shape
            N = W.shape[0]
            Y = torch.empty((B, N), dtype=torch.float32, device=X.device)
            relu = 1 if li + 1 < len(self.W) else 0
            _lib.check(lib.carc_mlp_linear_forward(B, K, N, _vp(acts[-1]), _vp(W), _vp(b), relu, _vp(Y),
                                                   current_stream_handle()))
            acts.append(Y)
        return acts

    def loss_and_grads(self, X, T):
        """MSE loss (a device scalar) and the gradients of every parameter."""
        lib = _lib.load()
        acts = self.forward(X)
        Y = acts[-1]
        B = Y.shape[0]
        dY = torch.empty_like(Y)
        loss = torch.zeros((), dtype=torch.float32, device=Y.device)
        _lib.check(lib.carc_mlp_mse(Y.numel(), B, _vp(Y), _vp(T.contiguous().float()), _vp(dY), _vp(loss),
                                    current_stream_handle()))
        grads = [None] * (2 * len(self.W))
        g = dY
        for li in range(len(self.W) - 1, -1, -1):
            W = self.W[li]
            N, K = W.shape
            relu = 1 if li + 1 < len(self.W) else 0
            dZ = torch.empty_like(g) if relu else None
            dX = torch.empty((B, K), dtype=torch.float32, device=Y.device) if li > 0 else None
            dW = torch.empty_like(W)
            db = torch.empty_like(self.b[li])
            _lib.check(lib.carc_mlp_linear_backward(B, K, N, _vp(acts[li]), _vp(W), _vp(acts[li + 1]), _vp(g), relu,
                                                    _vp(dZ), _vp(dX), _vp(dW), _vp(db), current_stream_handle()))
            grads[2 * li], grads[2 * li + 1] = dW, db
            g = dX
        return loss, grads

    def step(self, grads, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        lib = _lib.load()
        self.steps += 1
        for p, g, m, v in zip(self.params(), grads, self.m, self.v):
            _lib.check(lib.carc_mlp_adam(p.numel(), _vp(p), _vp(g), _vp(m), _vp(v), lr, beta1, beta2, eps,
                                         self.steps, current_stream_handle()))
        self._bf16 = None

    # -- BF16 inference ----------------------------------------------------
    def infer_bf16(self, X):
        lib = _lib.load()
        if self._bf16 is None:
            self._bf16 = []
            for W in self.W:
                Wb = torch.empty(W.shape, dtype=torch.bfloat16, device=W.device)
                _lib.check(lib.carc_mlp_to_bf16(W.numel(), _vp(W), _vp(Wb), current_stream_handle()))
                self._bf16.append(Wb)
        x = X.contiguous().float()
        h = torch.empty(x.shape, dtype=torch.bfloat16, device=x.device)
        _lib.check(lib.carc_mlp_to_bf16(x.numel(), _vp(x), _vp(h), current_stream_handle()))
        B = x.shape[0]
        out = None
        for li, (Wb, b) in enumerate(zip(self._bf16, self.b)):
            N, K = Wb.shape
            last = li + 1 == len(self._bf16)
            if last:
                out = torch.empty((B, N), dtype=torch.float32, device=x.device)
                _lib.check(lib.carc_mlp_linear_bf16(B, K, N, _vp(h), _vp(Wb), _vp(b), 0, None, _vp(out),
                                                    current_stream_handle()))
            else:
                hn = torch.empty((B, N), dtype=torch.bfloat16, device=x.device)
                _lib.check(lib.carc_mlp_linear_bf16(B, K, N, _vp(h), _vp(Wb), _vp(b), 1, _vp(hn), None,
                                                    current_stream_handle()))
                h = hn
        return out

    def normalize(self, X):
        return (X - self.x_mean) / self.x_std if self.x_mean is not None else X


# ---------------------------------------------------------------------------
# features, targets and data
# ---------------------------------------------------------------------------
def boundary_features(corners, sides, h, k=16):
    """Top-k singular values of the Identity tag of the 4 corners and 4 sides
    (each matricized as (left ket, left bra) x rest), then h: 8 k + 1 floats.
    The singular values are the square roots of the eigenvalues of the Gram
    matrices m m^H (c0 c1 square), all eight in one batched Jacobi
    eigensolve when the boundaries share c0 c1."""
    from . import engine
    bounds = list(corners) + list(sides)
    grams = []
    for t in bounds:
        a = t[Identity()]._t
        c0, c1 = a.shape[0], a.shape[1]
        m = a.reshape(c0 * c1, -1).contiguous()
        r = m.shape[0]
        grams.append(engine.contract("ik,jk->ij", m, m, (r, r), conj_b=True))
    dev = grams[0].device
    feats = []
    if len({g.shape[0] for g in grams}) == 1 and grams[0].shape[0] <= 512:
        r = grams[0].shape[0]
        A = torch.stack(grams).contiguous()
        lib = _lib.load()
        W = torch.empty((len(grams), r), dtype=torch.float64, device=dev)
        V = torch.empty((len(grams), r, r), dtype=CDT, device=dev)
        status = torch.zeros((), dtype=torch.int32, device=dev)
        ws_bytes = lib.carc_zheev_jacobi_workspace_size(r, len(grams))
        from .engine import Workspace
        ws = Workspace.get(ws_bytes, dev)
        _lib.call("carc_zheev_jacobi", r, len(grams), _vp(A), _vp(W), _vp(V), _vp(status), _vp(ws), ws_bytes,
                  current_stream_handle())
        sv = W.clamp_min(0).sqrt().flip(1).float()  # descending
        for i in range(len(grams)):
            v = torch.zeros(k, dtype=torch.float32, device=dev)
            v[: min(k, r)] = sv[i, :k]
            feats.append(v)
    else:
        for g in grams:
            w, _ = linalg.eigh_small(TorchData(g))
            sv = w.clamp_min(0).sqrt().flip(0).float()
            v = torch.zeros(k, dtype=torch.float32, device=dev)
            v[: min(k, sv.numel())] = sv[:k]
            feats.append(v)
    feats.append(torch.tensor([float(h)], dtype=torch.float32, device=dev))
    return torch.cat(feats)


def _reference_vector(n, device):
    r = np.random.default_rng(12345).standard_normal((n, 2))
    return torch.as_tensor(r[:, 0] + 1j * r[:, 1]).to(CDT).to(device)


def center_target(x):
    """Unit-norm center with its phase fixed by the overlap with a fixed
    reference vector, as 2N reals (real parts, then imaginary parts)."""
    v = x.reshape(-1).to(CDT)
    v = v / torch.linalg.vector_norm(v)
    ov = torch.vdot(_reference_vector(v.numel(), v.device), v)
    v = v * (ov.conj() / ov.abs())
    return torch.cat([v.real, v.imag]).float()


def center_from_output(y, shape):
    n = y.numel() // 2
    return torch.complex(y[:n].double(), y[n:].double()).reshape(shape)


def problem(seed, D, c, h_range=(2.0, 4.0)):
    """A transverse-Ising center-site problem (Hermitian-definite synthetic
    boundaries) with h drawn from h_range by the seed."""
    h = float(np.random.default_rng(seed).uniform(*h_range))
    cc, ss, oo = workloads.hermitian_problem_arrays(D=D, c=c, seed=seed, op_arrays=workloads.ti_operator_arrays(h=h))
    corners, sides, op = workloads.to_device(cc, ss, oo)
    H, N = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    return h, corners, sides, H, N


def make_dataset(seeds, D, c, h_range=(2.0, 4.0), tol=1e-12):
    """Features and converged centers from the plain FP64 solve of each seed."""
    X, T = [], []
    for seed in seeds:
        h, corners, sides, H, N = problem(seed, D, c, h_range)
        _, x, _ = linalg.hegv_lowest(H.formMatrix(), N.formMatrix(), tol=tol)
        X.append(boundary_features(corners, sides, h))
        T.append(center_target(x._t))
    return torch.stack(X), torch.stack(T)


def train(X, T, width=256, epochs=200, batch=128, lr=1e-3, seed=0):
    """Adam on the MSE between network outputs and phase-fixed centers;
    features standardized with the training set's statistics."""
    mlp = StartMLP(X.shape[1], T.shape[1], width=width, seed=seed, device=X.device)
    mlp.x_mean = X.mean(0, keepdim=True)
    mlp.x_std = X.std(0, keepdim=True).clamp_min(1e-6)
    Xn = mlp.normalize(X)
    g = torch.Generator().manual_seed(seed)
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(X.shape[0], generator=g).to(X.device)
        for i in range(0, X.shape[0], batch):
            idx = perm[i:i + batch]
            loss, grads = mlp.loss_and_grads(Xn[idx], T[idx])
            mlp.step(grads, lr=lr)
        losses.append(float(loss.item()))
    return mlp, losses


def predict_start(mlp, corners, sides, h, shape):
    f = mlp.normalize(boundary_features(corners, sides, h)[None])
    return center_from_output(mlp.infer_bf16(f)[0], shape)


def evaluate(mlp, seeds, D, c, h_range=(2.0, 4.0), tol=1e-10):
    """Lanczos iterations and wall time to residual tol from the learned start,
    a seeded random start, the solver's fixed start (x0 = None) and the
    previous problem's center (the previous-iterate start of independent
    problems), on the same problems; the eigenvalues must agree.  The learned
    start's wall time includes its features (8 boundary SVDs) and the BF16
    inference."""
    out = {k: dict(iterations=[], seconds=[]) for k in ("learned", "random", "fixed", "previous")}
    prev = None
    for seed in seeds:
        h, corners, sides, H, N = problem(seed, D, c, h_range)
        Hm, Nm = H.formMatrix(), N.formMatrix()
        shape = H.operator.in_shape
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        learned_x0 = predict_start(mlp, corners, sides, h, shape)
        torch.cuda.synchronize()
        t_infer = time.perf_counter() - t0
        rng = np.random.default_rng(seed + 7777)
        rand_x0 = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).to(CDT).cuda()
        starts = dict(learned=learned_x0, random=rand_x0, fixed=None, previous=prev)
        lams = {}
        ground = None
        for name, x0 in starts.items():
            if name == "previous" and x0 is None:
                continue
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lam, x, it = linalg.hegv_lowest(Hm, Nm, x0=None if x0 is None else TorchData(x0), tol=tol)
            torch.cuda.synchronize()
            out[name]["iterations"].append(it)
            out[name]["seconds"].append(time.perf_counter() - t0 + (t_infer if name == "learned" else 0.0))
            lams[name] = lam
            if name == "fixed":
                prev = x._t.reshape(shape)
                ground = x._t.reshape(-1)
        # start quality: |<x0, N g>| / sqrt(<x0, N x0> <g, N g>) against the converged center g
        from . import engine
        Nt = Nm._t
        nn = Nt.shape[0]
        Nmul = lambda u: engine.contract("ij,j->i", Nt, u, (nn,))  # noqa: E731
        dot = lambda a_, b_: TorchData(a_)._dot(TorchData(b_))  # noqa: E731
        Ng = Nmul(ground)
        gNg = float(dot(ground, Ng).real.item())
        for name, x0 in starts.items():
            if x0 is None:
                continue
            v = x0.reshape(-1).to(CDT).contiguous()
            ov = abs(complex(dot(v, Ng).item())) / float(np.sqrt(float(dot(v, Nmul(v)).real.item()) * gNg))
            out[name].setdefault("overlap", []).append(float(ov))
        vals = list(lams.values())
        out.setdefault("max_eigenvalue_spread", 0.0)
        out["max_eigenvalue_spread"] = max(out["max_eigenvalue_spread"],
                                           (max(vals) - min(vals)) / max(abs(vals[0]), 1e-300))
    summary = {k: dict(mean_iterations=float(np.mean(v["iterations"])), mean_ms=1e3 * float(np.mean(v["seconds"])),
                       mean_overlap=float(np.mean(v["overlap"])) if v.get("overlap") else None,
                       n=len(v["iterations"]))
               for k, v in out.items() if isinstance(v, dict) and v["iterations"]}
    summary["max_eigenvalue_spread"] = out["max_eigenvalue_spread"]
    return summary


def main(argv=None):
    """The configured learned-start experiment: plain-solve centers of
    transverse-Ising problems (D=3, c=7 so chi=49, h in [2, 4]) for the
    training seeds 1000, 1001, ... and the held-out seeds 30000, ...; train,
    then evaluate iterations and wall time to residual 1e-10 against random,
    fixed and previous-iterate starts.  Prints one JSON line."""
    import argparse
    import json
    p = argparse.ArgumentParser(prog="python -m carcassonne_gb300.learned")
    p.add_argument("--D", type=int, default=3)
    p.add_argument("--c", type=int, default=7)
    p.add_argument("--train", type=int, default=20000)
    p.add_argument("--eval", type=int, default=512)
    p.add_argument("--epochs", type=int, default=60)
    a = p.parse_args(argv)
    t0 = time.perf_counter()
    X, T = make_dataset(range(1000, 1000 + a.train), a.D, a.c)
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    mlp, losses = train(X, T, epochs=a.epochs, batch=256, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    res = evaluate(mlp, range(30000, 30000 + a.eval), a.D, a.c)
    print(json.dumps(dict(D=a.D, c=a.c, chi=a.c * a.c, train=a.train, eval=a.eval, epochs=a.epochs,
                          dataset_seconds=t_data, train_seconds=t_train, loss_first=losses[0],
                          loss_last=losses[-1], evaluation=res)), flush=True)


__all__ = ["StartMLP", "boundary_features", "center_target", "center_from_output", "make_dataset", "train",
           "predict_start", "evaluate", "problem", "main"]

if __name__ == "__main__":
    main()
