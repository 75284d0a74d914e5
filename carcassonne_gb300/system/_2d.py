"""The 2D center-site system (carcassonne/system/_2d.py:19-574) on the GPU.

State: four corners and four sides (tag-keyed boundaries of TorchData), the
state center (D,D,D,D,d) and the operator center {tag: (d,d)}.  Every
numerical step runs in libcarcgb300: grouped stage-1/2 contractions, the
stage-3 operator, the absorption kernels, the Jacobi SVD gauge, the product
compressor and the generalized eigensolver.

minimizeExpectation(): as the reference, relaxOver (utils.py:805-878) with a
budget of 100 multiplications, on the GPU (``solver="relax"``, the default).
``solver="lanczos"`` instead finds the lowest generalized eigenpair of
(H_eff, N_eff) to ~1e-13 relative with a Cholesky-reduced restarted Lanczos
started from the current center (for well-conditioned N_eff: right after a
bandwidth increase N_eff is nearly singular, and the exact pencil's lowest
pair can lie in its near-null space, where relaxOver, started from the
previous center, does not go);
``solver="mixed"`` runs the mixed-precision solve (H_eff, N_eff formed on the
tensor cores from split-BF16 operands, complex64 Lanczos, one FP64 Newton
correction: FP64-level energies, solve.solve_center) from the current center.
"""
from __future__ import annotations

import math
from copy import copy
from random import randint

import numpy as np

from ..compression import absorb_matrices, computeProductCompressor
from ..data import TorchData
from ..sparse import (Identity, OneSiteOperator, TwoSiteOperator, TwoSiteOperatorCompressed, makeSimpleSparseOperator,
                      makeSparseOperator, mapOverSparseData, stripAllButIdentityFrom)
from ..tensors._2d.dense import formNormalizationMultiplier, formNormalizationSubmatrix
from ..tensors._2d.sparse import (absorbSparseCenterSOSIntoSide, absorbSparseSideIntoCornerFromLeft,
                                  absorbSparseSideIntoCornerFromRight, formExpectationAndNormalizationMultipliers)
from ..utils import InvariantViolatedError, Multiplier, L, O, R
from .base import BaseSystem


def sideFromCorner(corner_id, direction):
    """system/_2d.py:573-574."""
    return (corner_id + 1 - direction) % 4


class System(BaseSystem):
    solver = "relax"

    # -- construction ----------------------------------------------------
    def __init__(self, corners, sides, state_center_data, operator_center_tensor, state_center_data_conj=None):
        BaseSystem.__init__(self)
        self.corners = list(corners)
        self.sides = list(sides)
        self.operator_center_tensor = operator_center_tensor
        self.state_center_data = state_center_data
        self.state_center_data_conj = state_center_data.conj() if state_center_data_conj is None \
            else state_center_data_conj
        self.just_increased_bandwidth = False
        self.last_solve = None

    @classmethod
    def newTrivial(cls, operator_center_tensor, DataClass=TorchData):
        """All-ones boundaries and the uniform center 1/sqrt(d) (system/_2d.py:72-86)."""
        physical_dimension = None
        for data in operator_center_tensor.values():
            if data is not None:
                physical_dimension = data.shape[0]
                break
        if physical_dimension is None:
            raise ValueError("Operator tensor must have at least one non-identity component.")
        return cls(
            tuple({Identity(): DataClass.newTrivial((1,) * 6)} for _ in range(4)),
            tuple({Identity(): DataClass.newTrivial((1,) * 8)} for _ in range(4)),
            DataClass.newFilled((1, 1, 1, 1, physical_dimension), 1.0 / math.sqrt(physical_dimension)),
            operator_center_tensor)

    @classmethod
    def newTrivialWithSimpleSparseOperator(cls, O=None, OO_UD=None, OO_LR=None):
        return cls.newTrivial(makeSimpleSparseOperator(O=O, OO_UD=OO_UD, OO_LR=OO_LR))

    @classmethod
    def newTrivialWithSparseOperator(cls, Os=[], OO_UDs=[], OO_LRs=[]):
        return cls.newTrivial(makeSparseOperator(Os=Os, OO_UDs=OO_UDs, OO_LRs=OO_LRs))

    @classmethod
    def newRandom(cls, makeOperator=None, DataClass=TorchData, maximum_dimension=2, O=None):
        """Random Hermitian boundaries (system/_2d.py:38-70)."""
        assert not (makeOperator is not None and O is not None)
        rd = lambda: randint(1, maximum_dimension)
        spokes = (rd(), rd()) * 2
        side_dims = [rd() for _ in range(4)]
        sides = []
        for i in range(4):
            s = DataClass.newRandom(*((side_dims[i],) * 2 + (1,)) * 2 + (spokes[i],) * 2)
            s += s.join(1, 0, 2, 4, 3, 5, 7, 6).conj()
            sides.append(s)
        corners = []
        for i in range(4):
            c = DataClass.newRandom(*(sides[L(i)].shape[3],) * 2 + (1,) + (sides[i].shape[0],) * 2 + (1,))
            c += c.join(1, 0, 2, 4, 3, 5).conj()
            corners.append(c)
        d = O.shape[0] if O is not None else max(2, rd())
        center = DataClass.newRandom(*spokes + (d,))
        if O is None:
            if makeOperator is None:
                O = DataClass.newRandom(d, d)
                O += O.join(1, 0).conj()
            else:
                O = makeOperator(d)
        system = cls(tuple({Identity(): c} for c in corners), tuple({Identity(): s} for s in sides), center,
                     {Identity(): DataClass.newIdentity(d), OneSiteOperator(None): O})
        system.assertDimensionsAreConsistent()
        system.assertNormalizationIsHermitian()
        system.assertHasNoNaNs()
        return system

    def __copy__(self):
        return System(copy(self.corners), copy(self.sides), self.state_center_data, copy(self.operator_center_tensor),
                      self.state_center_data_conj)

    # -- invariants (system/_2d.py:132-190) ------------------------------
    def assertDimensionsAreConsistent(self):
        s = self.state_center_data.shape
        assert s == self.state_center_data_conj.shape
        if s[0] != s[2]:
            raise AssertionError("state center's left and right dimensions do not agree ({} != {})".format(s[0], s[2]))
        if s[1] != s[3]:
            raise AssertionError("state center's up and down dimensions do not agree ({} != {})".format(s[1], s[3]))
        for i, side in enumerate(self.sides):
            ref = side[Identity()]
            if ref.ndim != 8:
                raise AssertionError("for side {} the normalization data has rank {} instead of rank 8".format(i, ref.ndim))
            for tag, data in side.items():
                if data.shape != ref.shape:
                    raise AssertionError("for side {} the data tagged with {} does not match the shape of the data "
                                         "tagged with Identity() ({} != {})".format(i, tag, data.shape, ref.shape))
            sh = ref.shape
            for d in (0, 3, 6):
                if sh[d] != sh[d + 1]:
                    raise AssertionError("side {}'s dimension {} does not match its dimension {} ({} != {})".format(
                        i, d, d + 1, sh[d], sh[d + 1]))
            if sh[0] != sh[3]:
                raise AssertionError("side {}'s left and right dimensions do not agree ({} != {})".format(i, sh[0], sh[3]))
            if sh[6] != s[i]:
                raise AssertionError("side {}'s center-facing dimensions do not match the corresponding state "
                                     "dimension ({} != {})".format(i, sh[6], s[i]))
        for i, corner in enumerate(self.corners):
            ref = corner[Identity()]
            if ref.ndim != 6:
                raise AssertionError("for corner {} the normalization data has rank {} instead of rank 6".format(i, ref.ndim))
            for tag, data in corner.items():
                if data.shape != ref.shape:
                    raise AssertionError("for corner {} the data tagged with {} does not match the shape of the data "
                                         "tagged with Identity() ({} != {})".format(i, tag, data.shape, ref.shape))
            sh = ref.shape
            for d in (0, 3):
                if sh[d] != sh[d + 1]:
                    raise AssertionError("corner {}'s dimension {} does not match its dimension {} ({} != {})".format(
                        i, d, d + 1, sh[d], sh[d + 1]))
            if sh[3] != self.sides[i][Identity()].shape[0]:
                raise AssertionError("corner {}'s right dimensions do not match side {}'s left dimensions".format(i, i))
            if sh[0] != self.sides[L(i)][Identity()].shape[3]:
                raise AssertionError("corner {}'s left dimensions do not match side {}'s right dimensions".format(i, L(i)))

    def assertHasNoNaNs(self):
        for i, corner in enumerate(self.corners):
            for tag, data in corner.items():
                if data.hasNaN():
                    raise AssertionError("corner {} has a NaN in component {}".format(i, tag))
        for i, side in enumerate(self.sides):
            for tag, data in side.items():
                if data.hasNaN():
                    raise AssertionError("side {} has a NaN in component {}".format(i, tag))
        if self.state_center_data.hasNaN():
            raise AssertionError("state center has a NaN")
        for tag, data in self.operator_center_tensor.items():
            if data is not None and data.hasNaN():
                raise AssertionError("operator center has a NaN in component {}".format(tag))

    def assertNormalizationIsHermitian(self):
        for i in range(4):
            s = self.sides[i][Identity()]
            if not s.allcloseTo(s.join(1, 0, 2, 4, 3, 5, 7, 6).conj()):
                raise AssertionError("side {} is not hermitian".format(i))
            c = self.corners[i][Identity()]
            if not c.allcloseTo(c.join(1, 0, 2, 4, 3, 5).conj()):
                raise AssertionError("corner {} is not hermitian".format(i))

    # -- compression (system/_2d.py:191-363) -----------------------------
    def compressCornerStateTowards(self, corner_id, direction, new_dimension):
        if direction == 0:
            return self.compressCornerStateTowardsLeft(corner_id, new_dimension)
        if direction == 1:
            return self.compressCornerStateTowardsRight(corner_id, new_dimension)
        raise ValueError("compression direction must be 0 or 1, not " + str(direction))

    def compressCornerStateTowardsLeft(self, corner_id, new_dimension):
        side = self.sides[L(corner_id)][Identity()].join((0, 1, 2, 6, 7), 3, 4, 5)
        corner = self.corners[corner_id][Identity()].join(0, 1, 2, (3, 4, 5))
        P = computeProductCompressor(side, corner, new_dimension)
        Pc = P.conj()
        self.sides[L(corner_id)] = absorb_matrices(self.sides[L(corner_id)], 3, P, 4, Pc)
        self.corners[corner_id] = absorb_matrices(self.corners[corner_id], 0, Pc, 1, P)
        return P

    def compressCornerStateTowardsRight(self, corner_id, new_dimension):
        corner = self.corners[corner_id][Identity()].join((0, 1, 2), 3, 4, 5)
        side = self.sides[corner_id][Identity()].join(0, 1, 2, (3, 4, 5, 6, 7))
        P = computeProductCompressor(corner, side, new_dimension)
        Pc = P.conj()
        self.corners[corner_id] = absorb_matrices(self.corners[corner_id], 3, P, 4, Pc)
        self.sides[corner_id] = absorb_matrices(self.sides[corner_id], 0, Pc, 1, P)
        return P

    def compressCornerTwoSiteOperatorTowards(self, corner_id, direction, new_dimension, normalize=False):
        """Truncate the two-site operator terms running along one direction of a
        corner and its matching side to ``new_dimension`` combinations
        (system/_2d.py:229-363), via the top eigenvectors of their Gram matrix."""
        from ..solver import computeCompressor
        axis = 3 * direction + 2
        new_corner = {}
        sparse_data = []
        position_index = {}
        old_compressed = None
        for tag, data in self.corners[corner_id].items():
            if isinstance(tag, TwoSiteOperator) and tag.direction == direction:
                assert tag.position not in position_index
                position_index[tag.position] = len(sparse_data)
                sparse_data.append(data)
            elif isinstance(tag, TwoSiteOperatorCompressed) and tag.direction == direction:
                assert old_compressed is None
                old_compressed = data
            else:
                new_corner[tag] = data
        n1 = len(sparse_data)
        old_dimension = n1 + (old_compressed.shape[axis] if old_compressed is not None else 0)
        if old_dimension == 0:
            return
        # Gram matrix, block diagonal: collected terms | old compressed axis
        blocks = []
        if n1:
            collected = TorchData.newCollected([d.ravel() for d in sparse_data])  # (n1, size)
            g1 = collected.conj().contractWith(collected, (1,), (1,))
        else:
            collected = None
            g1 = None
        if old_compressed is not None:
            folded = old_compressed.fold(axis)
            g2 = folded.conj().contractWith(folded, (1,), (1,))
        else:
            g2 = None
        # block-diagonal Gram matrix assembled on the device (no host round trip)
        gram_d = TorchData.newZeros((old_dimension, old_dimension))
        if g1 is not None:
            gram_d._t[:n1, :n1] = g1._t
        if g2 is not None:
            gram_d._t[n1:, n1:] = g2._t
        corner_mult, side_mult_conj = computeCompressor(old_dimension, new_dimension,
                                                        Multiplier((old_dimension,) * 2, None, 0, lambda: gram_d, 0),
                                                        None, normalize)
        side_mult = side_mult_conj.conj()
        # new corner
        cshape = list(self.corners[corner_id][Identity()].shape)
        del cshape[axis]
        perm = list(range(1, 6))
        perm.insert(axis, 0)
        new_data = None
        if collected is not None:
            cd = collected.split(*([n1] + cshape))
            new_data = cd.absorbMatrixAt(0, corner_mult[:, :n1]).transpose(*perm)
        if old_compressed is not None:
            oc = old_compressed.absorbMatrixAt(axis, corner_mult[:, n1:])
            new_data = oc if new_data is None else oc + new_data
        new_corner[TwoSiteOperatorCompressed(direction)] = new_data
        self.corners[corner_id] = new_corner
        # new side
        side_id = sideFromCorner(corner_id, direction)
        sdir = 1 - direction
        saxis = 3 * sdir + 2
        collected_side = [None] * n1
        old_side = None
        new_side = {}
        for tag, data in self.sides[side_id].items():
            if isinstance(tag, TwoSiteOperator) and tag.direction == sdir:
                collected_side[position_index[tag.position]] = data
            elif isinstance(tag, TwoSiteOperatorCompressed) and tag.direction == sdir:
                assert old_compressed is not None and old_side is None
                old_side = data
            else:
                new_side[tag] = data
        assert None not in collected_side
        sshape = list(self.sides[side_id][Identity()].shape)
        del sshape[saxis]
        sperm = list(range(1, 8))
        sperm.insert(saxis, 0)
        new_sdata = None
        if n1:
            cs = TorchData.newCollected(collected_side).dropUnitAxis(saxis + 1)
            new_sdata = cs.absorbMatrixAt(0, side_mult[:, :n1]).transpose(*sperm)
        if old_side is not None:
            os_ = old_side.absorbMatrixAt(saxis, side_mult[:, n1:])
            new_sdata = os_ if new_sdata is None else os_ + new_sdata
        new_side[TwoSiteOperatorCompressed(sdir)] = new_sdata
        self.sides[side_id] = new_side

    # -- expectations (system/_2d.py:364-434) ----------------------------
    def computeCenterSiteExpectation(self):
        return self.computeExpectation() - self.computeExpectationWithoutCenter()

    def computeExpectation(self, operator_center_tensor=None):
        return self.computeExpectationAndNormalization(operator_center_tensor)[0]

    def computeExpectationWithoutCenter(self):
        return self.computeExpectationAndNormalizationWithoutCenter()[0]

    def computeExpectationAndNormalization(self, operator_center_tensor=None):
        H, N = self.formExpectationAndNormalizationMultipliers(operator_center_tensor)
        e = self.computeScalarUsingMultiplier(H)
        n = self.computeScalarUsingMultiplier(N)
        return e / n, n

    def computeExpectationAndNormalizationWithoutCenter(self):
        return self.computeExpectationAndNormalization({
            tag: value for tag, value in self.operator_center_tensor.items()
            if tag is Identity() or (isinstance(tag, TwoSiteOperator) and tag.position == 0 and tag.direction in (2, 3))
        })

    def computeNormalization(self):
        return self.computeScalarUsingMultiplier(self.formNormalizationMultiplier())

    def computeNormalizationMatrixConditionNumber(self):
        from ..linalg import svd
        _, S, _ = svd(self.formNormalizationMatrix())
        s = S.toArray().real
        return float(s[0] / s[-1]) if s[-1] > 0 else float("inf")

    def computeOneSiteExpectation(self):
        expectation = 0
        stripped = self.stripExpectationEnvironment()
        for tag, value in self.operator_center_tensor.items():
            if isinstance(tag, OneSiteOperator):
                system = copy(stripped)
                system.operator_center_tensor[tag] = value
                expectation += system.computeExpectation()
            if isinstance(tag, TwoSiteOperator) and tag.position == 0 and tag.direction in (0, 1):
                other = tag.withNewDirectionAndPosition(tag.direction + 2, 0)
                system = copy(stripped)
                system.operator_center_tensor[tag] = value
                system.operator_center_tensor[other] = self.operator_center_tensor[other]
                system.contractTowards(tag.direction)
                expectation += system.computeExpectation()
        return expectation

    def computeScalarUsingMultiplier(self, multiply):
        return self.state_center_data_conj.contractWith(multiply(self.state_center_data), range(5),
                                                        range(5)).extractScalar()

    # -- absorption (system/_2d.py:435-454) ------------------------------
    def contractTowards(self, direction):
        tensor_to_contract, _, matrix_to_absorb = self.state_center_data.normalizeAxis(O(direction))
        self.contractUnnormalizedTowards(direction, tensor_to_contract)
        self.setStateCenter(self.state_center_data.normalizeAxis(direction)[0].absorbMatrixAt(direction,
                                                                                              matrix_to_absorb))

    def contractNormalizedTowards(self, direction, state_center_data):
        self.contractUnnormalizedTowards(direction, state_center_data.normalizeAxis(O(direction))[0])

    def contractUnnormalizedTowards(self, direction, state_center_data=None, state_center_data_conj=None):
        if state_center_data is None:
            state_center_data = self.state_center_data
            state_center_data_conj = self.state_center_data_conj
        if state_center_data_conj is None:
            state_center_data_conj = state_center_data.conj()
        self.corners[direction] = absorbSparseSideIntoCornerFromLeft(self.corners[direction], self.sides[L(direction)])
        self.sides[direction] = absorbSparseCenterSOSIntoSide(direction, self.sides[direction], state_center_data,
                                                              self.operator_center_tensor, state_center_data_conj)
        self.corners[R(direction)] = absorbSparseSideIntoCornerFromRight(self.corners[R(direction)],
                                                                         self.sides[R(direction)])
        if self.just_increased_bandwidth:
            raise InvariantViolatedError("Contracting the current center would blow up the condition number of the "
                                         "normalization matrix;  optimize it or replace it first.")

    # -- operators (system/_2d.py:455-479) -------------------------------
    def formExpectationAndNormalizationMultipliers(self, operator_center_tensor=None):
        if operator_center_tensor is None:
            operator_center_tensor = self.operator_center_tensor
        return formExpectationAndNormalizationMultipliers(self.corners, self.sides, operator_center_tensor)

    def formExpectationMatrix(self):
        return self.formExpectationMultiplier().formMatrix()

    def formExpectationMultiplier(self):
        return self.formExpectationAndNormalizationMultipliers()[0]

    def formNormalizationMatrix(self):
        return self.formNormalizationMultiplier().formMatrix()

    def formNormalizationMultiplier(self):
        return formNormalizationMultiplier(tuple(c[Identity()] for c in self.corners),
                                           tuple(s[Identity()] for s in self.sides),
                                           self.operator_center_tensor[Identity()])

    def formNormalizationSubmatrix(self):
        return formNormalizationSubmatrix(tuple(c[Identity()] for c in self.corners),
                                          tuple(s[Identity()] for s in self.sides))

    # -- bandwidth ---------------------------------------------------------
    def increaseBandwidth(self, direction, by=None, to=None, do_as_much_as_possible=False, enlargeners=None):
        if direction not in (0, 1):
            raise ValueError("Direction for bandwidth increase must be either 0 (for horizontal axes) or 1 (for "
                             "vertical axes), not {}.".format(direction))
        return self._increaseBandwidth(direction, by, to, do_as_much_as_possible, enlargeners)

    def increaseBandwidthAndThenNormalize(self, direction, by=None, to=None):
        self.increaseBandwidth(direction, by, to)
        self.normalize()

    # -- optimisation (system/_2d.py:489-502) ----------------------------
    def minimizeExpectation(self):
        H, N = self.formExpectationAndNormalizationMultipliers()
        if self.solver == "relax":
            from ..solver import relaxOver
            self.setStateCenter(relaxOver(self.state_center_data, H, N, maximum_number_of_multiplications=100))
            return
        if self.solver == "mixed":
            from ..solve import solve_center
            out = solve_center(H, N, x0=self.state_center_data, precision="mixed")
            self.last_solve = dict(eigenvalue=out["energy"], iterations=out["iterations"])
            self.setStateCenter(TorchData(out["center"]._t.reshape(self.state_center_data.shape)))
            return
        from ..linalg import hegv_lowest
        lam, x, iters = hegv_lowest(H.formMatrix(), N.formMatrix(), x0=self.state_center_data)
        self.last_solve = dict(eigenvalue=lam, iterations=iters)
        self.setStateCenter(TorchData(x._t.reshape(self.state_center_data.shape)))

    def minimizeExpectationUsingFullEigensolver(self):
        from ..linalg import hegv_lowest
        lam, x, iters = hegv_lowest(self.formExpectationMultiplier().formMatrix(),
                                    self.formNormalizationMultiplier().formMatrix())
        self.last_solve = dict(eigenvalue=lam, iterations=iters)
        self.setStateCenter(TorchData(x._t.reshape(self.state_center_data.shape)))

    # -- gauge (system/_2d.py:503-549) -----------------------------------
    def normalize(self):
        for corner_id in range(4):
            for direction in range(2):
                self.normalizeCornerAndDenormalizeSide(corner_id, direction)
        for side_id in range(4):
            self.normalizeSideAndDenormalizeCenter(side_id)

    def normalizeCenterAndDenormalizeSide(self, direction):
        normalizer, denormalizer_1 = self.state_center_data.normalizeAxis(direction, True)
        self.state_center_data = self.state_center_data.absorbMatrixAt(direction, normalizer)
        self.state_center_data_conj = self.state_center_data.conj()
        denormalizer_2 = denormalizer_1.conj()
        self.sides[direction] = {tag: d.absorbMatrixAt(6, denormalizer_1).absorbMatrixAt(7, denormalizer_2)
                                 for tag, d in self.sides[direction].items()}

    def normalizeCornerAndDenormalizeSide(self, corner_id, direction):
        side_id = sideFromCorner(corner_id, direction)
        c1, c2 = direction * 3, direction * 3 + 1
        s1, s2 = (1 - direction) * 3, (1 - direction) * 3 + 1
        corner_data = self.corners[corner_id][Identity()]
        normalizer_1, denormalizer_1 = corner_data.normalizeAxis(c1, True)
        normalizer_2, denormalizer_2 = normalizer_1.conj(), denormalizer_1.conj()
        self.corners[corner_id] = {tag: d.absorbMatrixAt(c1, normalizer_1).absorbMatrixAt(c2, normalizer_2)
                                   for tag, d in self.corners[corner_id].items()}
        self.sides[side_id] = {tag: d.absorbMatrixAt(s1, denormalizer_1).absorbMatrixAt(s2, denormalizer_2)
                               for tag, d in self.sides[side_id].items()}

    def normalizeSideAndDenormalizeCenter(self, side_id):
        side_data = self.sides[side_id][Identity()]
        normalizer_1, denormalizer = side_data.normalizeAxis(6, True)
        normalizer_2 = normalizer_1.conj()
        self.sides[side_id] = {tag: d.absorbMatrixAt(6, normalizer_1).absorbMatrixAt(7, normalizer_2)
                               for tag, d in self.sides[side_id].items()}
        self.state_center_data = self.state_center_data.absorbMatrixAt(side_id, denormalizer)
        self.state_center_data_conj = self.state_center_data.conj()

    def setStateCenter(self, state_center_data, state_center_data_conj=None):
        self.state_center_data = state_center_data
        self.state_center_data_conj = state_center_data.conj() if state_center_data_conj is None \
            else state_center_data_conj
        self.just_increased_bandwidth = False

    def stripExpectationEnvironment(self):
        return type(self)(map(stripAllButIdentityFrom, self.corners), map(stripAllButIdentityFrom, self.sides),
                          self.state_center_data, stripAllButIdentityFrom(self.operator_center_tensor),
                          self.state_center_data_conj)


__all__ = ["System", "sideFromCorner"]
