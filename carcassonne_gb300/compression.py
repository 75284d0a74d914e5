"""Boundary compression: computeProductCompressor (compression.py:11-46).

Finds an isometry P (old x new) such that inserting P P^H between the two
halves L (l,old,old,op) and R (old,old,op,r) of a boundary reproduces L.R,
by four rounds of: form the linear map A(P) of the reference's five-tensor
contractor, solve the normal equations A^H A x = A^H b, and take the polar
factor of x.  The reference solves the normal equations with GMRES; here
they are solved on the GPU by conjugate gradients (the system is Hermitian
positive semi-definite and consistent) to a relative residual of 1e-12
within an iteration budget, raising AssertionError where GMRES would report
non-convergence (compression.py:43).  Returns P^T (new, old).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, engine, linalg
from .data import TorchData
from .engine import CDT, current_stream_handle


def _A_matrix(Lt, Rt, P):
    """A[(l,r),(a,i)] = sum L[l,a,b,o] conj(P[b,j]) conj(P[c,i]) P[e,j] R[c,e,o,r]."""
    l, old, _, op = Lt.shape
    r = Rt.shape[3]
    new = P.shape[1]
    t1 = engine.contract("labo,bj->laoj", Lt, P, (l, old, op, new), conj_b=True)
    t2 = engine.contract("ej,ceor->jcor", P, Rt, (new, old, op, r))
    t3 = engine.contract("ci,jcor->ijor", P, t2, (new, new, op, r), conj_a=True)
    return engine.contract("laoj,ijor->lrai", t1, t3, (l, r, old, new)).reshape(l * r, old * new)


def _dot(x, y):
    return TorchData(x)._dot(TorchData(y))


def _cg(G, c, tol=1e-12, max_iter=None):
    """Conjugate gradients on G x = c from x = 0 (G Hermitian PSD, device)."""
    n = c.numel()
    max_iter = max_iter or max(4 * n, 50)
    x = torch.zeros(n, dtype=CDT, device=c.device)
    r = c.clone()
    p = r.clone()
    rr = float(_dot(r, r).real.item())
    c2 = rr
    if c2 == 0.0:
        return x, 0
    for it in range(max_iter):
        Gp = engine.contract("pq,q->p", G, p, (n,))
        pGp = float(_dot(p, Gp).real.item())
        if pGp <= 0.0:
            return x, it
        alpha = rr / pGp
        x = TorchData(x)._axpby(1.0, TorchData(x), alpha, TorchData(p))._t
        r = TorchData(r)._axpby(1.0, TorchData(r), -alpha, TorchData(Gp))._t
        rr_new = float(_dot(r, r).real.item())
        if rr_new <= tol * tol * c2:
            return x, it + 1
        p = TorchData(r)._axpby(1.0, TorchData(r), rr_new / rr, TorchData(p))._t
        rr = rr_new
    raise AssertionError("normal equations of the product compressor did not converge "
                         "(residual %.3e after %d iterations)" % (np.sqrt(rr / c2), max_iter))


def computeProductCompressor(L, R, new_dimension, rounds=4, initial=None):
    if L.shape[1] != L.shape[2]:
        raise ValueError("left inward dimensions do not match (given " + str(L.shape) + ")")
    if R.shape[0] != R.shape[1]:
        raise ValueError("right inward dimensions do not match (given " + str(R.shape) + ")")
    if L.shape[1] != R.shape[1]:
        raise ValueError("left and right shapes are incompatible (given " + str(L.shape) + " and " + str(R.shape) + ")")
    old = L.shape[1]
    Lt = L._t.contiguous()
    Rt = R._t.contiguous()
    l, r = Lt.shape[0], Rt.shape[3]
    b = engine.contract("labo,abor->lr", Lt, Rt, (l, r)).reshape(-1)
    if initial is None:
        initial = TorchData.newRandom(old, new_dimension)  # numpy's global generator, as the reference
    P = linalg.unitize(initial if isinstance(initial, TorchData) else TorchData(np.asarray(initial)))
    for _ in range(rounds):
        A = _A_matrix(Lt, Rt, P._t)
        G = engine.contract("pq,pr->qr", A, A, (old * new_dimension, old * new_dimension), conj_a=True)
        c = engine.contract("pq,p->q", A, b, (old * new_dimension,), conj_a=True)
        x, _ = _cg(G, c)
        P = linalg.unitize(TorchData(x.reshape(old, new_dimension)))
    return P.transpose()


__all__ = ["computeProductCompressor"]
