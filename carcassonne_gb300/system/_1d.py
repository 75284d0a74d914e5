"""The 1D chain system (carcassonne/system/_1d.py:14-190) on the GPU: left and
right environments (operator bond x ket bond x bra bond), an MPO-like
operator center O[o_left, o_right, p, q] and a state center S[s_left,
s_right, q]; the same driver loop and policies as the 2D system.

Every contraction runs on the device through the 1D contractors
(tensors/_1d.py); the center solve uses relaxOver or the Jacobi eigensolver;
the one-site expectation (the energy per site as the limiting linear
coefficient of the operator transfer map) uses device SVDs and reads back
only 2 x 2 scalars.
"""
from __future__ import annotations

from copy import copy

import numpy as np
import torch

from .. import linalg
from ..data import TorchData
from ..engine import CDT
from ..tensors._1d import (absorbCenterOSSIntoLeftEnvironment, absorbCenterOSSIntoRightEnvironment,
                           absorbCenterSSIntoRightEnvironment, formExpectationMultiplier)
from ..utils import buildProductTensor, crand
from .base import BaseSystem


def _data(x):
    return x if isinstance(x, TorchData) else TorchData(np.asarray(x, dtype=np.complex128))


def computeAbsoluteLimitingLinearCoefficient(O, Sn, Sc, left_boundary, right_boundary, env_shape):
    """|e| where the operator transfer map T (right environments of shape
    env_shape, one center absorbed) acts on its dominant generalized
    eigenspace {v1, v2} as lambda + e-coupling (utils.py:333-361):
    numerator sqrt(tr(Om^H Om) - 2) with Om the 2 x 2 restriction of T,
    denominator sqrt(tr(Nm^H Nm)) with Nm the state-transfer overlaps of the
    two vectors seen through the left and right boundaries.

    T is formed densely on the device (one contraction); its dominant
    eigenvalue lambda is that of the state transfer E (the MPO's first and
    last channels carry the identity, so T is block triangular with E on
    those diagonal blocks), by power iteration from the identity; the
    generalized eigenspace is the two right singular vectors of (T^T -
    lambda)^2 with the smallest singular values (the reference's ovecs)."""
    o, s, t = env_shape
    n = o * s * t
    # T[(o', s', t'), (x, y, z)] = sum_{p, q} O[x, o', p, q] S[y, s', q] Sc[z, t', p]
    a = O.contractWith(Sn, (3,), (2,))            # x o' p y s'
    a = a.contractWith(Sc, (2,), (2,))            # x o' y s' z t'
    T = a.join((1, 3, 5), (0, 2, 4))              # n x n
    # dominant eigenvalue of the state transfer E by power iteration from I
    rho = TorchData(torch.eye(s, t, dtype=CDT, device=T._t.device))
    lam = 1.0 + 0j
    for _ in range(200):
        nxt = absorbCenterSSIntoRightEnvironment(rho, Sn, Sc)
        new = complex(rho.ravel()._dot(nxt.ravel()).item()) / float(rho.ravel()._dot(rho.ravel()).item().real)
        nrm = float(nxt.norm())
        rho = nxt * (1.0 / nrm) if nrm > 0 else nxt
        done = abs(new - lam) <= 1e-14 * max(1.0, abs(new))
        lam = new
        if done:
            break
    # the reference's matrix has rows T(e_i): T^T; its ovecs are the rows of
    # Vh of (T^T - lambda)^2 for the two smallest singular values
    tm = TorchData(T.transpose(1, 0)._t - lam * torch.eye(n, dtype=CDT, device=T._t.device))
    _, S, Vh = linalg.svd(tm.contractWith(tm, (1,), (0,)))
    sv = S._t.real if S._t.is_complex() else S._t
    order = torch.argsort(sv)[:2].flip(0)         # second smallest, smallest: Vh[-2:]
    ovecs = TorchData(Vh._t[order].contiguous())  # 2 x n
    Tv = ovecs.contractWith(T, (1,), (1,))        # rows T(ovecs[j])
    Om = ovecs.conj().contractWith(Tv, (1,), (1,))  # Om[i, j] = ovecs[i]^H T ovecs[j]
    numerator = np.sqrt(complex(Om.conj().contractWith(Om, (0, 1), (0, 1)).extractScalar()) - 2)
    # through the boundaries: contract each vector's operator bond with the boundary vector
    vs = ovecs.split(2, o, s * t)
    ln = left_boundary.contractWith(vs, (0,), (1,))   # 2 x (s t)
    rn = right_boundary.contractWith(vs, (0,), (1,))
    nvecs = [absorbCenterSSIntoRightEnvironment(TorchData(rn._t[j].reshape(s, t).contiguous()), Sn, Sc).ravel()
             for j in range(2)]
    Nm = np.array([[complex(TorchData(ln._t[i].contiguous())._dot(nvecs[j]).item()) for j in range(2)]
                   for i in range(2)])
    denominator = np.sqrt(np.trace(Nm.conj().T @ Nm))
    return numerator / denominator


class System(BaseSystem):
    @classmethod
    def newRandom(cls, operator_dimension, state_dimension, physical_dimension):
        h = crand(operator_dimension, operator_dimension, physical_dimension, physical_dimension)
        return cls(crand(operator_dimension), crand(operator_dimension), h + h.transpose(0, 1, 3, 2).conj(),
                   crand(state_dimension, state_dimension, physical_dimension), crand(state_dimension),
                   crand(state_dimension))

    def __init__(self, right_operator_boundary, left_operator_boundary, operator_center_data, state_center_data=None,
                 right_state_boundary=None, left_state_boundary=None):
        BaseSystem.__init__(self)
        rob = np.asarray(right_operator_boundary, dtype=np.complex128)
        lob = np.asarray(left_operator_boundary, dtype=np.complex128)
        self.right_operator_boundary = TorchData(rob)
        self.left_operator_boundary = TorchData(lob)
        if right_state_boundary is None:
            self.right_environment = TorchData(buildProductTensor(rob, [1], [1]))
        else:
            rsb = np.asarray(right_state_boundary, dtype=np.complex128)
            self.right_environment = TorchData(buildProductTensor(rob, rsb, rsb.conj()))
        if left_state_boundary is None:
            self.left_environment = TorchData(buildProductTensor(lob, [1], [1]))
        else:
            lsb = np.asarray(left_state_boundary, dtype=np.complex128)
            self.left_environment = TorchData(buildProductTensor(lob, lsb, lsb.conj()))
        self.operator_center_data = _data(operator_center_data)
        if state_center_data is None:
            self.setStateCenter(TorchData.newTrivial((1, 1, self.operator_center_data.shape[2])))
        else:
            self.setStateCenter(_data(state_center_data))
        assert self.left_operator_boundary.ndim == 1
        assert self.right_operator_boundary.ndim == 1
        assert self.left_environment.ndim == 3
        assert self.right_environment.ndim == 3
        assert self.operator_center_data.ndim == 4
        assert self.state_center_data.ndim == 3

    def __copy__(self):
        new = object.__new__(type(self))
        new.__dict__.update(self.__dict__)
        return new

    # -- expectations (system/_1d.py:64-110) -------------------------------
    def computeExpectation(self):
        return self.computeScalarUsingMultiplier(self.formExpectationMultiplier()).real

    def computeOneSiteExpectation(self):
        assert self.left_environment.size() >= 2
        assert self.left_operator_boundary.size() >= 2
        normalized = self.state_center_data.normalizeAxis(1)[0]
        return float(abs(computeAbsoluteLimitingLinearCoefficient(
            self.operator_center_data, normalized, normalized.conj(), self.left_operator_boundary,
            self.right_operator_boundary, tuple(self.right_environment.shape))))

    def computeScalarUsingMultiplier(self, multiply):
        return self.state_center_data_conj.ravel().contractWith(multiply(self.state_center_data).ravel(), (0,),
                                                                (0,)).extractScalar()

    # -- absorption (system/_1d.py:111-160) --------------------------------
    def contractLeftNormalized(self, state_center_data):
        if state_center_data.shape[1] != self.left_environment.shape[1]:
            raise ValueError("state dimension of the left environment ({}) does not match the left dimension of the "
                             "center state ({})".format(self.left_environment.shape[1], state_center_data.shape[1]))
        self.contractLeftUnnormalized(state_center_data.normalizeAxis(0)[0])

    def contractLeftUnnormalized(self, state_center_data):
        self.left_environment = absorbCenterOSSIntoLeftEnvironment(
            self.left_environment, self.operator_center_data, state_center_data, state_center_data.conj())

    def contractRightNormalized(self, state_center_data):
        if state_center_data.shape[0] != self.right_environment.shape[1]:
            raise ValueError("state dimension of the right environment ({}) does not match the right dimension of "
                             "the center state ({})".format(self.right_environment.shape[1],
                                                            state_center_data.shape[0]))
        self.contractRightUnnormalized(state_center_data.normalizeAxis(1)[0])

    def contractRightUnnormalized(self, state_center_data=None):
        if state_center_data is None:
            state_center_data = self.state_center_data
        self.right_environment = absorbCenterOSSIntoRightEnvironment(
            self.right_environment, self.operator_center_data, state_center_data, state_center_data.conj())

    def contractTowards(self, direction):
        tensor_to_contract, _, matrix_to_absorb = self.state_center_data.normalizeAxis(1 - direction)
        self.contractUnnormalizedTowards(direction, tensor_to_contract)
        self.setStateCenter(self.state_center_data.normalizeAxis(direction)[0].absorbMatrixAt(direction,
                                                                                              matrix_to_absorb))

    def contractNormalizedTowards(self, direction, state_center_data=None):
        if state_center_data is None:
            state_center_data = self.state_center_data
        if direction == 0:
            self.contractRightNormalized(state_center_data)
        elif direction == 1:
            self.contractLeftNormalized(state_center_data)
        else:
            raise ValueError("Direction must be 0 for right or 1 for left, not {}.".format(direction))

    def contractUnnormalizedTowards(self, direction, state_center_data=None):
        if state_center_data is None:
            state_center_data = self.state_center_data
        if direction == 0:
            self.contractRightUnnormalized(state_center_data)
        elif direction == 1:
            self.contractLeftUnnormalized(state_center_data)
        else:
            raise ValueError("Direction must be 0 for right or 1 for left, not {}.".format(direction))

    # -- the center (system/_1d.py:161-190) --------------------------------
    def formExpectationMatrix(self):
        return self.formExpectationMultiplier().formMatrix()

    def formExpectationMultiplier(self):
        return formExpectationMultiplier(self.right_environment, self.left_environment, self.operator_center_data)

    def increaseBandwidth(self, direction=0, by=None, to=None, do_as_much_as_possible=False, enlargeners=None):
        if direction != 0:
            raise ValueError("Direction for bandwidth increase must be 0, not {}.".format(direction))
        return self._increaseBandwidth(0, by, to, do_as_much_as_possible, enlargeners)

    def minimizeExpectation(self):
        from ..solver import relaxOver
        self.setStateCenter(relaxOver(initial=self.state_center_data,
                                      expectation_multiplier=self.formExpectationMultiplier(),
                                      maximum_number_of_multiplications=100))

    def minimizeExpectationUsingFullEigensolver(self):
        _, V = linalg.eigh_small(self.formExpectationMultiplier().formMatrix())
        self.setStateCenter(TorchData(V._t[:, 0].reshape(self.state_center_data.shape).contiguous()))

    def setStateCenter(self, state_center_data, state_center_data_conj=None):
        self.state_center_data = state_center_data
        if state_center_data_conj is None:
            state_center_data_conj = state_center_data.conj()
        self.state_center_data_conj = state_center_data_conj


__all__ = ["System", "computeAbsoluteLimitingLinearCoefficient"]
