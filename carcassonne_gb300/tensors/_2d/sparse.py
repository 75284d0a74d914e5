"""Tag-level (sparse) operations of the 2D path (tensors/_2d/sparse.py:12-161).

The rule tables are the reference's: which tag pairs contract and which tag
the result carries.  Each function compiles its table into a schedule and
runs the dense work as one grouped launch; formExpectationStage3 turns the
whole term list into a single device operator (one launch sequence per
matvec instead of one Python-level multiplier per term).
"""
from __future__ import annotations

import itertools

import numpy as np

from .dense import (Stage3Operator, absorbDenseSideIntoCornerFromLeft, absorbDenseSideIntoCornerFromRight,
                    center_pair, center_pairs, formNormalizationStage1, formNormalizationStage2, _absorb_pairs)
from .dense import *  # noqa: F401,F403  (the dense contractors are reachable from this module too)
from ...sparse import (Complete, Identity, OneSiteOperator, TwoSiteOperator, TwoSiteOperatorCompressed,
                       addStandardCompleteAndIdentityTerms, compileSparseSchedule, contractSparseTensors,
                       getInformationFromOperatorCenter)
from ...utils import Multiplier

T, TC, I, C, OS = TwoSiteOperator, TwoSiteOperatorCompressed, Identity, Complete, OneSiteOperator


def _absorb_corner_left_rules():
    terms = {}
    f = absorbDenseSideIntoCornerFromLeft
    addStandardCompleteAndIdentityTerms(terms, f)
    terms.update({
        (T, I): lambda corner, side: (corner.matchesSideIdentityOnLeft(), f),
        (I, T): lambda corner, side: (side.matchesCornerIdentityOnRight(), f),
        (T, T): lambda corner, side: (side.matches(corner), f),
        (TC, TC): lambda corner, side: (side.matches(corner), f),
    })
    return terms


def _absorb_corner_right_rules():
    terms = {}
    f = absorbDenseSideIntoCornerFromRight
    addStandardCompleteAndIdentityTerms(terms, f)
    terms.update({
        (T, I): lambda corner, side: (corner.matchesSideIdentityOnRight(), f),
        (I, T): lambda corner, side: (side.matchesCornerIdentityOnLeft(), f),
        (T, T): lambda corner, side: (corner.matches(side), f),
        (TC, TC): lambda corner, side: (side.matches(corner), f),
    })
    return terms


def absorbSparseSideIntoCornerFromLeft(corner, side):
    """tensors/_2d/sparse.py:12-23."""
    return contractSparseTensors(_absorb_corner_left_rules(), corner, side)


def absorbSparseSideIntoCornerFromRight(corner, side):
    """tensors/_2d/sparse.py:24-35."""
    return contractSparseTensors(_absorb_corner_right_rules(), corner, side)


_SS, _SOS = "SS", "SOS"


def _center_rules(direction):
    return {
        (I, I): lambda s, c: (Identity(), _SS),
        (C, I): lambda s, c: (Complete(), _SS),
        (I, OS): lambda s, c: (Complete(), _SOS),
        (T, I): lambda s, c: (s.matchesCenterIdentity(), _SS),
        (I, T): lambda s, c: (c.matchesSideIdentityOutward(direction), _SOS),
        (T, T): lambda s, c: (s.matchesCenter(direction, c), _SOS),
        (TC, I): lambda s, c: (s, _SS),
    }


def absorbSparseCenterSOSIntoSide(direction, side, state_center_data, operator_center_data,
                                  state_center_data_conj=None):
    """tensors/_2d/sparse.py:36-58: every (side tag, operator tag) pair of the
    rule table adds side (x) center-pair into the result tag; the center pairs
    (one without operator, one per operator tag used) are formed once and all
    side contractions run as one grouped launch."""
    side_tags, op_tags = list(side), list(operator_center_data)
    sched = compileSparseSchedule(_center_rules(direction), side_tags, op_tags)
    if not sched.entries:
        return {}
    e_slot = {}
    e_ops = []
    table = []
    for i_side, i_op, slot, kind in sched.entries:
        key = None if kind == _SS else i_op
        if key not in e_slot:
            e_slot[key] = len(e_ops)
            e_ops.append(None if key is None else operator_center_data[op_tags[key]])
        table.append((i_side, e_slot[key], slot))
    e_list = center_pairs(direction, state_center_data, e_ops, state_center_data_conj)
    outs = _absorb_pairs(direction, [side[t] for t in side_tags], e_list, table, len(sched.result_tags))
    return dict(zip(sched.result_tags, outs))


def _stage1_rules():
    terms = {}
    f = formNormalizationStage1
    addStandardCompleteAndIdentityTerms(terms, f)
    terms.update({
        (T, I): lambda c, s: (c.matchesSideIdentityOnRightForStage1(), f),
        (I, T): lambda c, s: (s.matchesCornerIdentityOnLeftForStage1(), f),
        (T, T): lambda c, s: (c.matches(s), f),
        (TC, I): lambda c, s: (c.matchesSideIdentityOnRightForStage1(), f),
        (I, TC): lambda c, s: (s.matchesCornerIdentityOnLeftForStage1(), f),
        (TC, TC): lambda c, s: (c.matches(s), f),
    })
    return terms


def formExpectationStage1(corner, side):
    """tensors/_2d/sparse.py:72-85."""
    return contractSparseTensors(_stage1_rules(), corner, side)


def _stage2_rules():
    terms = {}
    f = formNormalizationStage2
    addStandardCompleteAndIdentityTerms(terms, f)
    terms.update({
        (T, I): lambda r, l: (r.matchesStage1IdentityOnLeft(), f),
        (I, T): lambda r, l: (l.matchesStage1IdentityOnRight(), f),
        (T, T): lambda r, l: (l.matches(r), f),
        (TC, I): lambda r, l: (r.matchesStage1IdentityOnLeft(), f),
        (I, TC): lambda r, l: (l.matchesStage1IdentityOnRight(), f),
        (TC, TC): lambda r, l: (l.matches(r), f),
    })
    return terms


def formExpectationStage2(right, left):
    """tensors/_2d/sparse.py:86-99."""
    return contractSparseTensors(_stage2_rules(), right, left)


RULES = {
    "stage1": _stage1_rules,
    "stage2": _stage2_rules,
    "absL": _absorb_corner_left_rules,
    "absR": _absorb_corner_right_rules,
}


_STAGE3_RULES = {
    (C, I, I): lambda x, y, z: True,
    (I, C, I): lambda x, y, z: True,
    (I, I, OS): lambda x, y, z: True,
    (T, I, T): lambda x, y, z: x.matchesCenterForStage3(0, z),
    (I, T, T): lambda x, y, z: y.matchesCenterForStage3(1, z),
    (T, T, I): lambda x, y, z: x.matchesForStage3(y),
    (TC, TC, I): lambda x, y, z: x.matchesForStage3(y),
}


def stage3TermTable(tags_0, tags_1, tags_op):
    """(i0, i1, iop, is_identity) for every matching tag triple, in
    itertools.product order (tensors/_2d/sparse.py:101-127)."""
    out = []
    for (i0, x), (i1, y), (io, z) in itertools.product(enumerate(tags_0), enumerate(tags_1), enumerate(tags_op)):
        rule = _STAGE3_RULES.get((type(x), type(y), type(z)))
        if rule is None or not rule(x, y, z):
            continue
        out.append((i0, i1, io, z == Identity()))
    return out


def formExpectationStage3(stage2_0, stage2_1, operator_center):
    """Expectation and normalization multipliers (tensors/_2d/sparse.py:100-161)."""
    k0, k1, ko = list(stage2_0), list(stage2_1), list(operator_center)
    table = stage3TermTable(k0, k1, ko)
    d, _, _ = getInformationFromOperatorCenter(operator_center)
    terms = [(i0, i1, -1 if is_id else io) for i0, i1, io, is_id in table]
    ops = [operator_center[t] for t in ko]
    expectation = Stage3Operator([stage2_0[t] for t in k0], [stage2_1[t] for t in k1], ops, terms, d) \
        if terms else None
    i0, i1 = k0.index(Identity()), k1.index(Identity())
    normalization_op = Stage3Operator([stage2_0[Identity()]], [stage2_1[Identity()]], [], [(0, 0, -1)], d)
    normalization = normalization_op.multiplier()
    normalization.operator = normalization_op
    if expectation is None:
        zero = _ZeroOperator(normalization_op)
        em = Multiplier(normalization.shape, zero, 0, zero.formMatrix, 0)
        em.operator = None  # no term of the operator reaches the center: H_eff = 0
        return em, normalization
    em = expectation.multiplier()
    em.operator = expectation
    return em, normalization


class _ZeroOperator:
    def __init__(self, like):
        self.like = like

    def __call__(self, v):
        return v.newZeros(v.shape) if hasattr(v, "newZeros") else v * 0

    def formMatrix(self):
        from ...data import TorchData
        n = self.like.n
        return TorchData.newZeros((n, n))


def formExpectationAndNormalizationMultipliers(corners, sides, operator_center_data):
    """tensors/_2d/sparse.py:59-71."""
    return formExpectationStage3(
        formExpectationStage2(formExpectationStage1(corners[0], sides[0]),
                              formExpectationStage1(corners[1], sides[1])),
        formExpectationStage2(formExpectationStage1(corners[2], sides[2]),
                              formExpectationStage1(corners[3], sides[3])),
        operator_center_data)


__all__ = [
    "absorbSparseSideIntoCornerFromLeft", "absorbSparseSideIntoCornerFromRight", "absorbSparseCenterSOSIntoSide",
    "formExpectationAndNormalizationMultipliers", "formExpectationStage1", "formExpectationStage2",
    "formExpectationStage3", "stage3TermTable",
]
