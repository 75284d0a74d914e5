"""The product compressor's normal equations formed without the A matrix.

computeProductCompressor (compression.py:12-43 of the reference) forms
A[(l,r),(a,i)] = sum L[l,a,b,o] conj(P[b,j]) conj(P[c,i]) P[e,j] R[c,e,o,r]
and solves A^H A x = A^H b.  The GPU path forms G = A^H A and A^H b from the
factors t1 = L . conj(P) and t3 = conj(P) . P . R instead; this CPU test
restates that factorisation in numpy and checks it against the oracle's
explicit A (oracle/carc_oracle.py product_compressor_matrix) on random
complex boundaries, with a non-unit operator axis.
"""
import numpy as np
import pytest

from oracle import carc_oracle as orc


def _factored(Lt, Rt, P, b2):
    t1 = np.einsum("labo,bj->laoj", Lt, P.conj())
    t2 = np.einsum("ej,ceor->jcor", P, Rt)
    t3 = np.einsum("ci,jcor->ijor", P.conj(), t2)
    X = np.einsum("laoj,lbpk->aojbpk", t1.conj(), t1)
    Y = np.einsum("ijor,xkpr->ijoxkp", t3.conj(), t3)
    old, new = P.shape
    G = np.einsum("aojbpk,ijoxkp->aibx", X, Y).reshape(old * new, old * new)
    u = np.einsum("ijor,lr->lijo", t3.conj(), b2)
    c = np.einsum("laoj,lijo->ai", t1.conj(), u).reshape(old * new)
    return G, c


@pytest.mark.parametrize("l,old,new,op,r,seed", [(5, 4, 2, 1, 3, 0), (7, 6, 3, 2, 4, 1), (3, 5, 5, 3, 2, 2)])
def test_factored_normal_equations_equal_explicit(l, old, new, op, r, seed):
    rng = np.random.default_rng(seed)
    cn = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    Lt, Rt = cn(l, old, old, op), cn(old, old, op, r)
    P = orc.unitize(cn(old, new))
    b2 = np.tensordot(Lt, Rt, ((1, 2, 3), (0, 1, 2)))
    A = orc.product_compressor_matrix(Lt, Rt, P)
    G, c = _factored(Lt, Rt, P, b2)
    Ge, ce = A.conj().T @ A, A.conj().T @ b2.ravel()
    assert np.abs(G - Ge).max() <= 1e-12 * np.abs(Ge).max()
    assert np.abs(c - ce).max() <= 1e-12 * np.abs(ce).max()
