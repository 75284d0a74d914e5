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
    (each matricized as (left ket, left bra) x rest), then h: 8 k + 1 floats."""
    feats = []
    for t in list(corners) + list(sides):
        a = t[Identity()]._t
        c0, c1 = a.shape[0], a.shape[1]
        m = a.reshape(c0 * c1, -1)
        _, S, _ = linalg.svd(TorchData(m))
        s = (S._t.real if S._t.is_complex() else S._t).float()
        v = torch.zeros(k, dtype=torch.float32, device=a.device)
        v[: min(k, s.numel())] = s[:k]
        feats.append(v)
    feats.append(torch.tensor([float(h)], dtype=torch.float32, device=feats[0].device))
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
    the fixed start (no previous center) and the previous problem's center
    (previous-iterate), on the same problems; the eigenvalues must agree."""
    out = {k: dict(iterations=[], seconds=[]) for k in ("learned", "fixed", "previous")}
    prev = None
    for seed in seeds:
        h, corners, sides, H, N = problem(seed, D, c, h_range)
        Hm, Nm = H.formMatrix(), N.formMatrix()
        shape = H.operator.in_shape
        starts = dict(learned=predict_start(mlp, corners, sides, h, shape), fixed=None, previous=prev)
        lams = {}
        for name, x0 in starts.items():
            if name == "previous" and x0 is None:
                continue
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lam, x, it = linalg.hegv_lowest(Hm, Nm, x0=None if x0 is None else TorchData(x0), tol=tol)
            torch.cuda.synchronize()
            out[name]["iterations"].append(it)
            out[name]["seconds"].append(time.perf_counter() - t0)
            lams[name] = lam
            if name == "fixed":
                prev = x._t.reshape(shape)
        vals = list(lams.values())
        out.setdefault("max_eigenvalue_spread", 0.0)
        out["max_eigenvalue_spread"] = max(out["max_eigenvalue_spread"],
                                           (max(vals) - min(vals)) / max(abs(vals[0]), 1e-300))
    summary = {k: dict(mean_iterations=float(np.mean(v["iterations"])), mean_ms=1e3 * float(np.mean(v["seconds"])),
                       n=len(v["iterations"]))
               for k, v in out.items() if isinstance(v, dict) and v["iterations"]}
    summary["max_eigenvalue_spread"] = out["max_eigenvalue_spread"]
    return summary


__all__ = ["StartMLP", "boundary_features", "center_target", "center_from_output", "make_dataset", "train",
           "predict_start", "evaluate", "problem"]
