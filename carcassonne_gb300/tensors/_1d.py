"""Contractors of the 1D chain (tensors/_1d.py:12-93): environment
absorption of a center site with or without the operator, and the expectation
multiplier of the center.

Index conventions (fixed by the reference's join tables):
  left environment  L[o, s, t]   (operator bond, ket bond, bra bond)
  right environment R[o, s, t]
  operator center   O[o_left, o_right, p_bra, q_ket]
  state center      S[s_left, s_right, q]   (bra copy Sc = conj(S))
Each contractor is a fixed sequence of pairwise contractions on the GPU
engine (TorchData.contractWith); run on CostTracker objects the same sequence
gives the cost in complex MACs.
"""
from __future__ import annotations

from ..data.cost_tracker import computeCostOfContracting
from ..utils import Multiplier


def absorbCenterOSSIntoLeftEnvironment(L, O, S, Sc):
    """L'[o, s, t] = sum L[x, y, z] O[o, x, p, q] S[s, y, q] Sc[t, z, p]  (tensors/_1d.py:12-25)."""
    t = L.contractWith(S, (1,), (1,))          # x z s q
    t = t.contractWith(O, (0, 3), (1, 3))      # z s o p
    t = t.contractWith(Sc, (0, 3), (1, 2))     # s o t
    return t.transpose(1, 0, 2)


def absorbCenterOSSIntoRightEnvironment(R, O, S, Sc):
    """R'[o, s, t] = sum R[x, y, z] O[x, o, p, q] S[y, s, q] Sc[z, t, p]  (tensors/_1d.py:26-39)."""
    t = R.contractWith(S, (1,), (0,))          # x z s q
    t = t.contractWith(O, (0, 3), (0, 3))      # z s o p
    t = t.contractWith(Sc, (0, 3), (0, 2))     # s o t
    return t.transpose(1, 0, 2)


def absorbCenterSSIntoLeftEnvironment(L, S, Sc):
    """L'[s, t] = sum L[y, z] S[s, y, p] Sc[t, z, p]  (tensors/_1d.py:40-49)."""
    t = L.contractWith(S, (0,), (1,))          # z s p
    return t.contractWith(Sc, (0, 2), (1, 2))  # s t


def absorbCenterSSIntoRightEnvironment(R, S, Sc):
    """R'[s, t] = sum R[y, z] S[y, s, p] Sc[z, t, p]  (tensors/_1d.py:50-59)."""
    t = R.contractWith(S, (0,), (0,))          # z s p
    return t.contractWith(Sc, (0, 2), (0, 2))  # s t


def _multiply(R, L, O, S):
    # y[r, l, o] = sum R[x, r', r] L[u, l', l] O[x, u, o, q] S[r', l', q], in
    # the reference's pairwise order (R.O, then S, then L), so that the
    # CostTracker count is the reference's
    t = R.contractWith(O, (0,), (0,))          # r' r u o q
    t = t.contractWith(S, (0, 4), (0, 2))      # r u o l'
    t = t.contractWith(L, (1, 3), (0, 1))      # r o l
    return t.transpose(0, 2, 1)


def _formMatrix(R, L, O):
    # M[(r, l, o), (r', l', q)] = sum_{x, u} R[x, r', r] L[u, l', l] O[x, u, o, q]
    t = R.contractWith(O, (0,), (0,))          # r' r u o q
    t = t.contractWith(L, (2,), (0,))          # r' r o q l' l
    return t.join((1, 5, 2), (0, 4, 3))


def formExpectationMultiplier(R, L, O):
    """The center's expectation operator as a Multiplier on states of shape
    (R.shape[1], L.shape[1], O.shape[2]) (tensors/_1d.py:61-93)."""
    s_shape = (R.shape[1], L.shape[1], O.shape[2])
    n = s_shape[0] * s_shape[1] * s_shape[2]
    return Multiplier(
        (n, n),
        lambda S: _multiply(R, L, O, S),
        computeCostOfContracting(_multiply, R, L, O, s_shape),
        lambda: _formMatrix(R, L, O),
        computeCostOfContracting(_formMatrix, R, L, O),
    )


__all__ = ["absorbCenterOSSIntoLeftEnvironment", "absorbCenterOSSIntoRightEnvironment",
           "absorbCenterSSIntoLeftEnvironment", "absorbCenterSSIntoRightEnvironment", "formExpectationMultiplier"]
