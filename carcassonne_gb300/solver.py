"""GPU numerics with the reference's names: relaxOver, unitize, computeCompressor.

relaxOver        utils.py:805-878  (carc_relax_over: restarted Krylov / Rayleigh-Ritz)
unitize          utils.py:879-882  (Jacobi SVD polar factor)
computeCompressor utils.py:268-302 (Jacobi eigh of the Gram matrix; the
                 reference's ARPACK branch for new < old//2 computes the same
                 top eigenvectors, so one dense eigensolver serves both)
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, engine, linalg
from .data import TorchData
from .engine import CDT, current_stream_handle
from .utils import Multiplier, RelaxFailed


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _dense(m):
    """Device matrix of a Multiplier / TorchData."""
    if isinstance(m, Multiplier):
        m = m.formMatrix()
    if isinstance(m, TorchData):
        return m._t.contiguous()
    return TorchData(np.asarray(m))._t.contiguous()


def relaxOver(initial, expectation_multiplier, normalization_multiplier=None, maximum_number_of_multiplications=None,
              tolerance=1e-7, dimension_of_krylov_space=None):
    """Lowest Ritz vector of N^{-1} H starting from ``initial`` (utils.py:805-878).

    The operators are formed densely (the reference does the same whenever it
    is cheaper, which covers the center-site sizes).  The normalization
    matrix is factored by Cholesky where the reference uses LU; both solve the
    same systems.  N enters the reference's iteration only through the
    product N^{-1} (H v), so where Cholesky rejects N (nearly singular, with
    rounding-level negative eigenvalues, as right after a bandwidth increase)
    the iteration runs on the formed N^{-1} H instead, N^{-1} taken from N's
    Hermitian eigendecomposition: the exact inverse LU also computes.  Raises
    RelaxFailed like the reference when the Rayleigh value rises."""
    shape = initial.shape
    x0 = (initial._t if isinstance(initial, TorchData) else TorchData(initial)._t).reshape(-1).contiguous()
    n = x0.numel()
    k = 3 if dimension_of_krylov_space is None else int(dimension_of_krylov_space)
    k = min(k, n)
    H = _dense(expectation_multiplier)
    N = _dense(normalization_multiplier) if normalization_multiplier is not None else None
    lib = _lib.load()
    x = torch.empty((n,), dtype=CDT, device=x0.device)
    ws_bytes = lib.carc_relax_over_workspace_size(n, k)
    ws = engine.Workspace.get(ws_bytes, x0.device)
    lam = (ctypes.c_double * 2)()
    vals = (ctypes.c_double * 4)()
    mults = ctypes.c_int32(0)
    mm = -1 if maximum_number_of_multiplications is None else int(maximum_number_of_multiplications)
    st = lib.carc_relax_over(n, _vp(H), _vp(N) if N is not None else None, _vp(x0), _vp(x), k, mm, float(tolerance),
                             lam, ctypes.byref(mults), vals, _vp(ws), ws_bytes, current_stream_handle())
    if st == _lib.CARC_NOT_POSDEF and N is not None:
        W, V = linalg.eigh_small(TorchData(N))
        Vt = V._t
        VinvW = engine.contract("ij,jk->ik", Vt, torch.diag((1.0 / W).to(CDT)), (n, n))  # V diag(1/w)
        Ninv = engine.contract("ij,kj->ik", VinvW, Vt, (n, n), conj_b=True)
        M = engine.contract("ij,jk->ik", Ninv, H, (n, n))
        st = lib.carc_relax_over(n, _vp(M), None, _vp(x0), _vp(x), k, mm, float(tolerance), lam,
                                 ctypes.byref(mults), vals, _vp(ws), ws_bytes, current_stream_handle())
    if st == _lib.CARC_RELAX_FAILED:
        raise RelaxFailed(complex(vals[0], vals[1]), complex(vals[2], vals[3]))
    if st == _lib.CARC_NOT_POSDEF:
        raise np.linalg.LinAlgError(lib.carc_last_error_string().decode())
    _lib.check(st)
    out = TorchData(x.reshape(shape))
    out.relax_info = dict(eigenvalue=complex(lam[0], lam[1]), multiplications=mults.value)
    return out


def unitize(matrix):
    return linalg.unitize(matrix if isinstance(matrix, TorchData) else TorchData(np.asarray(matrix)))


def computeCompressor(old_dimension, new_dimension, multiplier, dtype=None, normalize=False):
    """Top ``new_dimension`` eigenvectors of a Hermitian Gram operator, rows of
    the returned (compressor, inverse_compressor_conj) (utils.py:268-302)."""
    if new_dimension < 0:
        raise ValueError("New dimension ({}) must be non-negative.".format(new_dimension))
    if new_dimension > old_dimension:
        raise ValueError("New dimension ({}) must be less than or equal to the old dimension ({}).".format(
            new_dimension, old_dimension))
    if new_dimension == 0:
        z = TorchData.newZeros((0, old_dimension))
        return z, z
    matrix = multiplier.formMatrix() if hasattr(multiplier, "formMatrix") else multiplier
    m = matrix if isinstance(matrix, TorchData) else TorchData(np.asarray(matrix))
    if m.shape != (old_dimension, old_dimension):
        raise ValueError("Multiplier matrix has shape {} but the old dimension is {}.".format(m.shape, old_dimension))
    W, V = linalg.eigh_small(m)
    evals = W[-new_dimension:].cpu().numpy()
    evecs_t = V._t[:, -new_dimension:].transpose(0, 1)  # (new, old), rows = eigenvectors
    while new_dimension > 0 and abs(evals[new_dimension - 1]) < 1e-15:
        new_dimension -= 1
    if new_dimension == 0:
        raise ValueError("Input is filled with near-zero elements.")
    evals = evals[:new_dimension]
    evecs = TorchData(evecs_t[:new_dimension].contiguous())
    if normalize:
        s = np.sqrt(evals.astype(np.complex128)).reshape(new_dimension, 1)
        scale = TorchData(np.broadcast_to(s, (new_dimension, old_dimension)).copy())
        inv = TorchData(np.broadcast_to(1.0 / s, (new_dimension, old_dimension)).copy())
        return evecs * scale, evecs * inv
    return evecs, evecs


def computeCompressorForMatrixTimesItsDagger(old_dimension, new_dimension, matrix, normalize=False):
    m = matrix if isinstance(matrix, TorchData) else TorchData(np.asarray(matrix))
    gram = m.conj().contractWith(m, (0,), (0,))  # M^H M
    return computeCompressor(old_dimension, new_dimension, Multiplier((old_dimension,) * 2, None, 0, lambda: gram, 0),
                             None, normalize)


__all__ = ["relaxOver", "unitize", "computeCompressor", "computeCompressorForMatrixTimesItsDagger"]
