"""Sparse operator algebra: symbolic tags keyed boundaries and their contraction.

Same public surface as carcassonne/sparse.py: the tag classes and their
matching rules (sparse.py:23-208), the direction constants (:211-215) and the
helpers (:218-345).  The difference is execution: ``contractSparseTensors``
first compiles the tag pairs into an integer schedule -- (index in tensor_1,
index in tensor_2, result slot) in the reference's iteration order -- and then
runs every dense contraction of the call in ONE grouped kernel launch when the
dense contractor supports it (all contractors of tensors/_2d/dense.py do).
"""
from __future__ import annotations

from functools import partial

import numpy as np

from .utils import L, R, O

LEFT = 0
RIGHT = 1
CENTER = 2


class _Unique:
    """Tags with a single instance (sparse.py:9-21)."""

    __slots__ = []
    _instances = {}

    def __new__(cls):
        inst = _Unique._instances.get(cls)
        if inst is None:
            inst = object.__new__(cls)
            _Unique._instances[cls] = inst
        return inst

    def __hash__(self):
        return hash(type(self).__name__)

    def __eq__(self, other):
        return self is other

    def __reduce__(self):
        return (type(self), ())


Singleton = _Unique


class Identity(_Unique):
    __slots__ = []

    def __repr__(self):
        return "Identity()"


class Complete(_Unique):
    __slots__ = []

    def __repr__(self):
        return "Complete()"


class OneSiteOperator:
    """One-site operator tag.  As in the reference (sparse.py:35-38) the id is
    not stored, so every OneSiteOperator is the same key; operators built from
    several one-site terms therefore keep only the last of them."""

    __slots__ = ["id"]

    def __init__(self, id):
        self.id = None

    def __eq__(self, other):
        return isinstance(other, OneSiteOperator) and other.id == self.id

    def __hash__(self):
        return hash(("OneSiteOperator", self.id))

    def __repr__(self):
        return "OneSiteOperator({})".format(self.id)


class TwoSiteOperator:
    """Half of a two-site operator term travelling through the boundaries
    (sparse.py:56-166).  ``direction`` is LEFT/RIGHT/CENTER within a boundary
    (or 0..3 on the operator center), ``position`` how far it has moved out."""

    __slots__ = ["id", "direction", "position"]

    def __init__(self, id, direction, position=None):
        self.id = id
        self.direction = direction
        self.position = position

    def _key(self):
        return (self.id, self.direction, self.position)

    def __eq__(self, other):
        return isinstance(other, TwoSiteOperator) and other._key() == self._key()

    def __hash__(self):
        return hash(("TwoSiteOperator",) + self._key())

    def __repr__(self):
        return "TwoSiteOperator({},{},{})".format(self.id, self.direction, self.position)

    def withNewDirectionAndPosition(self, direction, position=None):
        return TwoSiteOperator(self.id, direction, position)

    def moveOut(self):
        return TwoSiteOperator(self.id, self.direction, self.position + 1)

    # -- pair rules ----------------------------------------------------------
    def matches(left, right):
        """A right-moving half meets its left-moving partner: the term is complete."""
        if (left.id, left.direction, left.position) == (right.id, RIGHT, right.position) and right.direction == LEFT:
            return Complete()
        return None

    def matchesCenter(self, side_direction, center):
        if self.id == center.id and self.direction == CENTER and center.direction == side_direction:
            return Complete()
        return None

    def matchesCenterForStage3(self, direction, other):
        return self.id == other.id and self.direction == CENTER and self.position + 2 * direction == other.direction

    def matchesForStage3(x, y):
        return x.id == y.id and x.position == y.position and {x.direction, y.direction} == {LEFT, RIGHT}

    # -- rules against an Identity partner -----------------------------------
    def matchesCenterIdentity(self):
        return None if self.direction == CENTER else self.moveOut()

    def matchesCornerIdentityOnLeft(self):
        return {RIGHT: self, CENTER: TwoSiteOperator(self.id, LEFT, 0)}.get(self.direction)

    def matchesCornerIdentityOnRight(self):
        return {LEFT: self, CENTER: TwoSiteOperator(self.id, RIGHT, 0)}.get(self.direction)

    def matchesCornerIdentityOnLeftForStage1(self):
        return self if self.direction in (RIGHT, CENTER) else None

    def matchesSideIdentityOnLeft(self):
        return self.moveOut() if self.direction == RIGHT else None

    def matchesSideIdentityOnRight(self):
        return self.moveOut() if self.direction == LEFT else None

    def matchesSideIdentityOnRightForStage1(self):
        return self if self.direction == LEFT else None

    def matchesSideIdentityOutward(self, direction):
        if self.direction == L(direction):
            return TwoSiteOperator(self.id, LEFT, 0)
        if self.direction == R(direction):
            return TwoSiteOperator(self.id, RIGHT, 0)
        if self.direction == O(direction):
            return TwoSiteOperator(self.id, CENTER)
        return None

    def matchesStage1IdentityOnLeft(self):
        return {RIGHT: self, CENTER: TwoSiteOperator(self.id, CENTER, LEFT)}.get(self.direction)

    def matchesStage1IdentityOnRight(self):
        return {LEFT: self, CENTER: TwoSiteOperator(self.id, CENTER, RIGHT)}.get(self.direction)


class TwoSiteOperatorCompressed:
    """A compressed bundle of two-site halves along one direction (sparse.py:167-208)."""

    __slots__ = ["direction"]

    def __init__(self, direction):
        self.direction = direction

    def __eq__(self, other):
        return isinstance(other, TwoSiteOperatorCompressed) and other.direction == self.direction

    def __hash__(self):
        return hash(("TwoSiteOperatorCompressed", self.direction))

    def __repr__(self):
        return "TwoSiteOperatorCompressed({})".format(self.direction)

    def matches(left, right):
        return Complete() if (left.direction, right.direction) == (RIGHT, LEFT) else None

    def matchesCornerIdentityOnLeftForStage1(self):
        return self if self.direction == RIGHT else None

    def matchesSideIdentityOnRightForStage1(self):
        return self if self.direction == LEFT else None

    def matchesStage1IdentityOnLeft(self):
        return self if self.direction == RIGHT else None

    def matchesStage1IdentityOnRight(self):
        return self if self.direction == LEFT else None

    def matchesForStage3(x, y):
        return {x.direction, y.direction} == {LEFT, RIGHT}


# ---------------------------------------------------------------------------
# schedules
# ---------------------------------------------------------------------------
class Schedule:
    """Integer form of one contractSparseTensors call: the result tags in
    first-insertion order and the (i1, i2, slot, dense) entries in the
    reference's nested-loop order (sparse.py:223-240)."""

    __slots__ = ["result_tags", "entries", "dense"]

    def __init__(self, result_tags, entries, dense):
        self.result_tags = result_tags
        self.entries = entries
        self.dense = dense

    def table(self):
        return [(i, j, k) for i, j, k, _ in self.entries]


def compileSparseSchedule(dense_contractors, tags_1, tags_2):
    result_tags = []
    slot_of = {}
    entries = []
    for i1, t1 in enumerate(tags_1):
        for i2, t2 in enumerate(tags_2):
            rule = dense_contractors.get((type(t1), type(t2)))
            if rule is None:
                continue
            handled = rule(t1, t2)
            if handled is None:
                continue
            result_tag, dense = handled
            if result_tag is None:
                continue
            slot = slot_of.get(result_tag)
            if slot is None:
                slot = len(result_tags)
                slot_of[result_tag] = slot
                result_tags.append(result_tag)
            entries.append((i1, i2, slot, dense))
    return Schedule(result_tags, entries, None)


def contractSparseTensors(dense_contractors, tensor_1, tensor_2):
    """Contract two tag-keyed tensors (sparse.py:223-240).

    When every matching pair uses the same dense contractor and that
    contractor offers a ``grouped`` form, all pairs run as one launch that
    accumulates each result tag in the reference's order; otherwise the dense
    contractors are called pair by pair."""
    keys_1, keys_2 = list(tensor_1), list(tensor_2)
    sched = compileSparseSchedule(dense_contractors, keys_1, keys_2)
    if not sched.entries:
        return {}
    denses = {id(e[3]) for e in sched.entries}
    first = sched.entries[0][3]
    grouped = getattr(first, "grouped", None)
    if len(denses) == 1 and grouped is not None:
        outs = grouped([tensor_1[k] for k in keys_1], [tensor_2[k] for k in keys_2], sched.table(),
                       len(sched.result_tags))
        return dict(zip(sched.result_tags, outs))
    result = {}
    for i1, i2, slot, dense in sched.entries:
        tag = sched.result_tags[slot]
        data = dense(tensor_1[keys_1[i1]], tensor_2[keys_2[i2]])
        if tag in result:
            result[tag] += data
        else:
            result[tag] = data
    return result


def addStandardCompleteAndIdentityTerms(terms, dense):
    """Identity x Identity -> Identity, Complete x Identity -> Complete and back (sparse.py:218-222)."""
    terms[Identity, Identity] = lambda x, y: (Identity(), dense)
    terms[Complete, Identity] = lambda x, y: (Complete(), dense)
    terms[Identity, Complete] = lambda x, y: (Complete(), dense)


def formSparseContractor(dense_contractors):
    return partial(contractSparseTensors, dense_contractors)


def getInformationFromOperatorCenter(operator_center):
    for matrix in operator_center.values():
        return matrix.shape[0], matrix.dtype, type(matrix)
    raise ValueError("operator tensor has no term from which to extract the physical dimension")


def makeSparseOperator(Os=[], OO_UDs=[], OO_LRs=[]):
    """Operator center from one-site terms and up/down, left/right two-site
    pairs (sparse.py:295-338): tags OneSiteOperator, TwoSiteOperator(id,3|1,0)
    for up/down halves, TwoSiteOperator(id,0|2,0) for left/right halves, and
    the Identity."""
    operator = {}
    reference_shape = None

    def register(O_):
        nonlocal reference_shape
        if reference_shape is None:
            reference_shape = tuple(O_.shape)
        elif tuple(O_.shape) != reference_shape:
            raise ValueError("incompatible site matrix shapes: {} and {}".format(reference_shape, tuple(O_.shape)))

    first = None
    for i, O_ in enumerate(Os):
        operator[OneSiteOperator(i)] = O_
        register(O_)
        first = O_ if first is None else first
    for i, (up, down) in enumerate(OO_UDs):
        operator[TwoSiteOperator(i, 3, 0)] = up
        operator[TwoSiteOperator(i, 1, 0)] = down
        register(up)
        register(down)
        first = up if first is None else first
    for i, (left, right) in enumerate(OO_LRs):
        operator[TwoSiteOperator(i, 0, 0)] = left
        operator[TwoSiteOperator(i, 2, 0)] = right
        register(left)
        register(right)
        first = left if first is None else first
    if first is None:
        raise ValueError("No terms have been specified.")
    operator[Identity()] = first.newIdentity(reference_shape[0])
    return operator


def makeSimpleSparseOperator(O=None, OO_UD=None, OO_LR=None):
    return makeSparseOperator([O] if O is not None else [], [OO_UD] if OO_UD is not None else [],
                              [OO_LR] if OO_LR is not None else [])


def mapOverSparseData(f, sparse):
    return {tag: f(data) for tag, data in sparse.items()}


def stripAllButIdentityFrom(sparse):
    return {Identity(): sparse[Identity()]}


def makeMPO(I, Os=(), OOs=()):
    """Chain operator sum_i Os[i] + sum_j OOs[j][0] (x) OOs[j][1] as a
    matrix-product operator (sparse.py:265-287): an (n, n, d, d) tensor with
    n = 2 + len(OOs) channels, channel 0 the identity still to the right,
    channel n - 1 the identity after the term, channel j + 1 term j half
    applied; returns (tensor, right boundary, right tags, left boundary, left
    tags).  The arguments are not modified (the one-site terms are summed
    into a new array)."""
    from .utils import buildTensor
    I = np.asarray(I)
    size = 2 + len(OOs)
    last = size - 1
    components = {(0, 0): I, (last, last): I}
    if len(Os):
        components[(0, last)] = sum(np.asarray(o, dtype=np.complex128) for o in Os)
    for k, (first, second) in enumerate(OOs):
        components[(0, k + 1)] = second
        components[(k + 1, last)] = first
    d = len(I)
    two_site = [TwoSiteOperator(k, 2) for k in range(len(OOs))]
    return (buildTensor((size, size, d, d), components),
            [1] + [0] * (size - 1), [Identity()] + two_site + [Complete()],
            [0] * (size - 1) + [1], [Complete()] + list(two_site) + [Identity()])


__all__ = [
    "Identity", "Complete", "OneSiteOperator", "TwoSiteOperator", "TwoSiteOperatorCompressed",
    "LEFT", "RIGHT", "CENTER", "Schedule", "compileSparseSchedule",
    "addStandardCompleteAndIdentityTerms", "contractSparseTensors", "formSparseContractor",
    "getInformationFromOperatorCenter", "makeSimpleSparseOperator", "makeSparseOperator", "mapOverSparseData",
    "stripAllButIdentityFrom", "makeMPO", "Singleton",
]
