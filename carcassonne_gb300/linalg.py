"""GPU dense linear algebra behind the Data protocol (FP64 complex).

svd / unitize / normalize_axis restate NDArrayData.svd, unitize and
normalizeAxis (data/__init__.py:263-346, utils.py:879-882) on the one-sided
Jacobi SVD kernel; eigh_small carries computeCompressor's eigh
(utils.py:268-302); hegv_lowest is the lowest generalized eigenpair used by
minimizeExpectation (system/_2d.py:489-502).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib, engine
from .data import TorchData
from .engine import CDT, current_stream_handle


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _status_check(status, what):
    s = int(status.item())
    if s != _lib.CARC_OK:
        raise _lib.CarcNotConverged(s, what) if s == _lib.CARC_NOT_CONVERGED else _lib.CarcError(s, what)


def svd(data, full_matrices=True, deferred=None):
    """(U, S, Vh) of a matrix; the economic form (full_matrices is accepted
    for signature compatibility; only the economic factors are produced).
    ``deferred``: a list to which the device status word is appended instead
    of being read here (the caller checks it later with check_deferred, so a
    sequence of calls synchronises once)."""
    t = data._t if isinstance(data, TorchData) else TorchData(data)._t
    if t.dim() != 2:
        raise ValueError("svd needs a matrix")
    m, n = t.shape
    if m < n:
        # A^H = V S U^H
        U2, S2, Vh2 = svd(TorchData(engine.permute(t, [1, 0], conj=True)), deferred=deferred)
        return (TorchData(engine.permute(Vh2._t, [1, 0], conj=True)), S2,
                TorchData(engine.permute(U2._t, [1, 0], conj=True)))
    lib = _lib.load()
    a = t.contiguous()
    U = torch.empty((m, n), dtype=CDT, device=a.device)
    S = torch.empty((n,), dtype=torch.float64, device=a.device)
    Vh = torch.empty((n, n), dtype=CDT, device=a.device)
    status = torch.zeros((), dtype=torch.int32, device=a.device)
    ws_bytes = lib.carc_zgesvd_jacobi_workspace_size(m, n, 1)
    ws = engine.Workspace.get(ws_bytes, a.device)
    _lib.call("carc_zgesvd_jacobi", m, n, 1, _vp(a), _vp(U), _vp(S), _vp(Vh), _vp(status), _vp(ws), ws_bytes,
              current_stream_handle())
    if deferred is None:
        _status_check(status, "Jacobi SVD did not converge")
    else:
        deferred.append(status)
    return TorchData(U), TorchData(S), TorchData(Vh)


def check_deferred(statuses, what="Jacobi SVD did not converge"):
    """Read the status words collected by ``deferred`` calls (one device sync)."""
    if statuses:
        vals = torch.stack([s.reshape(()) for s in statuses]).cpu().numpy()
        for v in vals:
            if int(v) != _lib.CARC_OK:
                raise (_lib.CarcNotConverged(int(v), what) if int(v) == _lib.CARC_NOT_CONVERGED
                       else _lib.CarcError(int(v), what))


def unitize(data, deferred=None):
    """Polar factor U Vh (utils.py:879-882)."""
    U, _, Vh = svd(data, deferred=deferred)
    return U.contractWith(Vh, (1,), (0,))


def normalize_axis(data, axis, sqrt_svals=False, dont_recip_under=1e-14):
    """NDArrayData.normalizeAxis (data/__init__.py:263-301) on the GPU."""
    shape = data.shape
    if shape[axis] == 1:
        n = data.norm()
        if sqrt_svals:
            n = math.sqrt(n)
            return TorchData(np.array([[1 / n]])), TorchData(np.array([[n]]))
        return data * (1.0 / n), TorchData(np.array([[1 / n]])), TorchData(np.array([[n]]))
    others = [i for i in range(data.ndim) if i != axis]
    M = data.join(others, axis)
    if M.shape[0] < M.shape[1]:
        raise ValueError("the total number of degrees of freedom in all other axes ({}) are not enough to normalize "
                         "axis ({}) with dimension ({})".format(M.shape[0], axis, M.shape[1]))
    U, S, Vh = svd(M)
    n = S.shape[0]
    a = torch.empty((n, n), dtype=CDT, device=S._t.device)
    b = torch.empty((n, n), dtype=CDT, device=S._t.device)
    s_real = S._t.real.contiguous() if S._t.is_complex() else S._t.contiguous()
    thresh = float(dont_recip_under) if dont_recip_under else 0.0
    _lib.call("carc_normalize_axis_finish", n, _vp(s_real), _vp(Vh._t), thresh, int(bool(sqrt_svals)), _vp(a), _vp(b),
              current_stream_handle())
    if sqrt_svals:
        return TorchData(a), TorchData(b)
    iso = U.contractWith(Vh, (1,), (0,))
    split = [shape[i] for i in others] + [n]
    inv = list(range(data.ndim - 1))
    inv.insert(axis, data.ndim - 1)
    return iso.split(*split).join(*inv), TorchData(a), TorchData(b)


def qr(data, mode="full"):
    """Q, R of a matrix; only the economic factorisation is computed (mode
    'full' is accepted for tall matrices whose economic Q is what callers use)."""
    t = (data._t if isinstance(data, TorchData) else TorchData(data)._t).contiguous()
    m, n = t.shape
    if m < n:
        raise ValueError("qr on the GPU needs rows >= columns")
    Q = torch.empty((m, n), dtype=CDT, device=t.device)
    R = torch.empty((n, n), dtype=CDT, device=t.device)
    _lib.call("carc_zgeqr_economic", m, n, _vp(t), _vp(Q), _vp(R), current_stream_handle())
    return TorchData(Q), TorchData(R)


def qr_economic(data):
    return qr(data, "economic")[0]


def eigh_small(matrix):
    """(W ascending, V) of a small Hermitian matrix (Jacobi, n <= 512)."""
    t = matrix._t if isinstance(matrix, TorchData) else TorchData(matrix)._t
    n = t.shape[0]
    lib = _lib.load()
    a = t.contiguous()
    W = torch.empty((n,), dtype=torch.float64, device=a.device)
    V = torch.empty((n, n), dtype=CDT, device=a.device)
    status = torch.zeros((), dtype=torch.int32, device=a.device)
    ws_bytes = lib.carc_zheev_jacobi_workspace_size(n, 1)
    ws = engine.Workspace.get(ws_bytes, a.device)
    _lib.call("carc_zheev_jacobi", n, 1, _vp(a), _vp(W), _vp(V), _vp(status), _vp(ws), ws_bytes,
              current_stream_handle())
    _status_check(status, "Jacobi eigensolver did not converge")
    return W, TorchData(V)


def cholesky(matrix):
    t = matrix._t if isinstance(matrix, TorchData) else TorchData(matrix)._t
    n = t.shape[0]
    lib = _lib.load()
    L = t.contiguous().clone()
    status = torch.zeros((), dtype=torch.int32, device=L.device)
    ws_bytes = lib.carc_zpotrf_workspace_size(n)
    ws = engine.Workspace.get(ws_bytes, L.device)
    _lib.call("carc_zpotrf", n, _vp(L), _vp(status), _vp(ws), ws_bytes, current_stream_handle())
    s = int(status.item())
    if s != _lib.CARC_OK:
        raise np.linalg.LinAlgError("matrix is not positive definite")
    return TorchData(L)


def tri_inverse_lower(L):
    t = L._t.contiguous()
    n = t.shape[0]
    lib = _lib.load()
    X = torch.empty_like(t)
    ws_bytes = lib.carc_ztrtri_lower_workspace_size(n)
    ws = engine.Workspace.get(ws_bytes, t.device)
    _lib.call("carc_ztrtri_lower", n, _vp(t), _vp(X), _vp(ws), ws_bytes, current_stream_handle())
    return TorchData(X)


def hegv_lowest(H, N, x0=None, tol=1e-13, max_krylov=256, max_restarts=8, tensor_core=False, with_second=False,
                factors=None, single=False):
    """Lowest eigenpair of H x = l N x; returns (l, x, iterations), x N-normalized
    (with_second: (l, x, iterations, l2), l2 the second-lowest Ritz value, a
    gap estimate to about 1e-6).  factors: a complex128 device tensor of
    2 n^2 + n elements that receives [C = L^-1 H L^-H | L^-1 | u].
    tensor_core: reduce the pencil with the split-BF16 tensor-core GEMM
    (~1e-5 relative; for pencils that are tensor-core approximations).
    single: also factor, invert and iterate in complex64 (residual test
    clamped to tol >= 2e-6); for the same pencils."""
    Ht = (H._t if isinstance(H, TorchData) else TorchData(H)._t).contiguous()
    Nt = (N._t if isinstance(N, TorchData) else TorchData(N)._t).contiguous()
    n = Ht.shape[0]
    lib = _lib.load()
    x = torch.empty((n,), dtype=CDT, device=Ht.device)
    x0t = None
    if x0 is not None:
        x0t = (x0._t if isinstance(x0, TorchData) else TorchData(x0)._t).reshape(-1).contiguous()
    flags = (_lib.CARC_HEGV_TENSOR_CORE if tensor_core else 0) | (_lib.CARC_HEGV_SINGLE if single else 0)
    ws_bytes = lib.carc_zhegv_lowest_workspace_size(n, max_krylov, flags)
    ws = engine.Workspace.get(ws_bytes, Ht.device)
    lam = (ctypes.c_double * 2)(0.0, 0.0)
    iters = ctypes.c_int32(0)
    st = lib.carc_zhegv_lowest(n, _vp(Ht), _vp(Nt), _vp(x0t) if x0t is not None else None, _vp(x), lam,
                               max_krylov, max_restarts, float(tol), flags, ctypes.byref(iters),
                               _vp(factors) if factors is not None else None, _vp(ws), ws_bytes,
                               current_stream_handle())
    if st == _lib.CARC_NOT_POSDEF:
        raise np.linalg.LinAlgError(lib.carc_last_error_string().decode())
    _lib.check(st)
    if with_second:
        return lam[0], TorchData(x), iters.value, lam[1]
    return lam[0], TorchData(x), iters.value


def hegv_lowest_projected(H, N, cut=1e-12):
    """Lowest eigenpair of H x = l N x on the range of N, for an N whose
    Cholesky factorisation fails (nearly singular, with rounding-level
    negative eigenvalues).  Canonical orthogonalisation: N = V diag(w) V^H
    (Jacobi), X = V_k diag(w_k^-1/2) over the eigenvalues w_k > cut max(w),
    then the lowest eigenpair (l, c) of the Hermitian X^H H X and x = X c,
    N-normalized.  The same pencil as scipy.linalg.eigh(H, N) where N is
    definite, with N's near-null directions dropped where it is not.  Returns
    (l, x, kept dimension); n <= 512."""
    Ht = (H._t if isinstance(H, TorchData) else TorchData(H)._t).contiguous()
    Nt = (N._t if isinstance(N, TorchData) else TorchData(N)._t).contiguous()
    n = Ht.shape[0]
    W, V = eigh_small(TorchData(Nt))
    w = W.cpu().numpy()
    wmax = float(np.abs(w).max()) if n else 0.0
    k0 = int(np.searchsorted(w, cut * wmax, side="right")) if wmax > 0 else n
    kept = n - k0
    if kept == 0:
        raise np.linalg.LinAlgError("hegv: the normalization matrix is zero")
    scale = torch.from_numpy(w[k0:] ** -0.5).to(device=Ht.device, dtype=CDT)
    X = engine.contract("ij,jk->ik", V._t[:, k0:].contiguous(), torch.diag(scale), (n, kept))
    HX = engine.contract("ij,jk->ik", Ht, X, (n, kept))
    C = engine.contract("ji,jk->ik", X, HX, (kept, kept), conj_a=True)
    W2, V2 = eigh_small(TorchData(C))
    x = engine.contract("ij,jk->ik", X, V2._t[:, :1].contiguous(), (n, 1)).reshape(-1)
    return float(W2[0].item()), TorchData(x), kept


def minres_projected(C, u, shift, b, maxit=60, rtol=1e-3):
    """z solving P (C - shift) P z = P b, P = I - u u^H (u unit), C dense
    Hermitian: MINRES on the device.  Returns (z, iterations)."""
    Ct = (C._t if isinstance(C, TorchData) else C).contiguous()
    ut = (u._t if isinstance(u, TorchData) else u).reshape(-1).contiguous()
    bt = (b._t if isinstance(b, TorchData) else b).reshape(-1).contiguous()
    n = Ct.shape[0]
    lib = _lib.load()
    z = torch.empty((n,), dtype=CDT, device=Ct.device)
    ws_bytes = lib.carc_zminres_projected_workspace_size(n)
    ws = engine.Workspace.get(ws_bytes, Ct.device)
    iters = ctypes.c_int32(0)
    _lib.check(lib.carc_zminres_projected(n, _vp(Ct), _vp(ut), float(shift), _vp(bt), _vp(z), int(maxit), float(rtol),
                                          ctypes.byref(iters), _vp(ws), ws_bytes, current_stream_handle()))
    return z, iters.value


__all__ = ["svd", "unitize", "normalize_axis", "qr", "qr_economic", "eigh_small", "cholesky", "tri_inverse_lower",
           "hegv_lowest", "hegv_lowest_projected", "minres_projected"]
