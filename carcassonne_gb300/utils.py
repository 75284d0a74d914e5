"""Helpers shared by the center-site path: index maps, exceptions, Multiplier.

Public names follow carcassonne/utils.py.  The numerical routines
(relaxOver, unitize, computeCompressor) run on the GPU and live in
``linalg``/``solver``; they are re-exported here under the reference's names.
"""
from __future__ import annotations

import numpy as np


# -- exceptions (utils.py:13-41) ---------------------------------------------
class DimensionMismatchError(ValueError):
    def __init__(self, left_tensor_number, left_index, left_dimension, right_tensor_number, right_index,
                 right_dimension):
        self.left_tensor_number = left_tensor_number
        self.left_index = left_index
        self.left_dimension = left_dimension
        self.right_tensor_number = right_tensor_number
        self.right_index = right_index
        self.right_dimension = right_dimension
        ValueError.__init__(self, "tensor {}'s index {} has dimension {}, whereas tensor {}'s index {} has "
                                  "dimension {}".format(left_tensor_number, left_index, left_dimension,
                                                        right_tensor_number, right_index, right_dimension))


class InvariantViolatedError(Exception):
    pass


class RelaxFailed(Exception):
    def __init__(self, initial_value, final_value):
        Exception.__init__(self)
        self.initial_value = initial_value
        self.final_value = final_value

    def __str__(self):
        return "{} --> {}".format(self.initial_value, self.final_value)

    def __repr__(self):
        return "RelaxFailed({},{})".format(self.initial_value, self.final_value)


class UnexpectedTensorRankError(ValueError):
    def __init__(self, tensor_number, expected_rank, actual_rank):
        self.tensor_number = tensor_number
        self.expected_rank = expected_rank
        self.actual_rank = actual_rank
        ValueError.__init__(self, "tensor {} was expected to have rank {} but actually has rank {}".format(
            tensor_number, expected_rank, actual_rank))


# -- index maps (utils.py:886-892) -------------------------------------------
def O(i):
    """Opposite direction."""
    return (i + 2) % 4


def L(i):
    """Direction to the left (counter-clockwise)."""
    return (i + 1) % 4


def R(i):
    """Direction to the right (clockwise)."""
    return (i - 1) % 4


def A(d, i):
    """Position of axis i among the remaining axes once axis d is removed."""
    return i - 1 if i > d else i


def OA(i):
    return A(i, O(i))


def LA(i):
    return A(i, L(i))


def RA(i):
    return A(i, R(i))


def dropAt(iterable, index):
    values = list(iterable)
    del values[index]
    return type(iterable)(values) if isinstance(iterable, tuple) else values


def replaceAt(iterable, index, new_value):
    values = [new_value if i == index else v for i, v in enumerate(iterable)]
    try:
        return type(iterable)(values)
    except TypeError:
        return tuple(values)


def computeNewDimension(old_dimension, by=None, to=None):
    if by is None and to is None:
        raise ValueError("Either 'by' or 'to' must be specified.")
    if by is not None and to is not None:
        raise ValueError("Only one of 'by' or 'to' may be specified.")
    if to is not None:
        if to < old_dimension:
            raise ValueError("The new dimension ({}) is smaller than the old dimension ({}).".format(to, old_dimension))
        return to
    if by < 0:
        raise ValueError("Increment ({}) must be non-negative.".format(by))
    return old_dimension + by


# -- random samples (utils.py:254-255, :795-796) -----------------------------
def buildProductTensor(*factors):
    """Outer product of the factors as a complex128 numpy array (utils.py:241-243)."""
    from functools import reduce
    return reduce(np.multiply.outer, (np.asarray(f, dtype=np.complex128) for f in factors))


def buildTensor(dimensions, components):
    """Zero complex128 array with the given {index: value} components (utils.py:244-249)."""
    t = np.zeros(dimensions, dtype=np.complex128)
    for index, value in components.items():
        t[index] = value
    return t


def crand(*shape):
    return np.random.rand(*shape) * 2 - 1 + np.random.rand(*shape) * 2j - 1j


def randomComplexSample(shape):
    return np.random.random_sample(shape) * 2 - 1 + np.random.random_sample(shape) * 2j - 1j


class Pauli:
    I = np.identity(2, dtype=np.complex128)
    X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)


# -- Multiplier (utils.py:180-207) -------------------------------------------
class Multiplier:
    """An implicit linear operator: shape, how to apply it, what that costs,
    how to form it densely and what that costs (all costs in complex MACs)."""

    def __init__(self, shape, multiply, cost_of_multiply, formMatrix, cost_of_formMatrix):
        self.shape = shape
        self.multiply = multiply
        self.cost_of_multiply = cost_of_multiply
        self.formMatrix = formMatrix
        self.cost_of_formMatrix = cost_of_formMatrix

    def __call__(self, vector):
        return self.multiply(vector)

    @classmethod
    def fromMatrix(cls, matrix):
        m, n = matrix.shape
        return cls(matrix.shape, lambda v: matrix.matvecWith(v), m * n, lambda: matrix, 0)

    def isCheaperToFormMatrix(self, estimated_number_of_applications):
        n = estimated_number_of_applications
        return n * self.cost_of_multiply > self.cost_of_formMatrix + n * self.shape[0] * self.shape[1]


# -- decorators (utils.py:208-222) -------------------------------------------
class prepend:
    def __init__(self, *args, **keywords):
        self.args = args
        self.keywords = keywords

    def __call__(self, f):
        from functools import partial
        return partial(f, *self.args, **self.keywords)


def checkForNaNsIn(data):
    assert not data.hasNaN()
    return data


def multiplyBySingleSiteOperator(state, operator):
    return state.absorbMatrixAt(4, operator)


# -- contractor builder (utils.py:45-101, :562-711) ---------------------------
def _index_list(indices):
    if isinstance(indices, str) or not hasattr(indices, "__len__"):
        return [indices]
    return list(indices)


class Join:
    """Axes of two argument tensors of a contractor to be summed together
    (utils.py:45-101): one index or a sequence per side, kept with the lower
    tensor number on the left; a join of a tensor with itself is an error."""

    def __init__(self, left_tensor_number, left_tensor_indices, right_tensor_number, right_tensor_indices):
        left, right = _index_list(left_tensor_indices), _index_list(right_tensor_indices)
        if len(left) != len(right):
            raise ValueError("number of left indices does not match number of right indices (len({}) != len({}))"
                             .format(left, right))
        self.left_tensor_number = left_tensor_number
        self.left_tensor_indices = left
        self.right_tensor_number = right_tensor_number
        self.right_tensor_indices = right
        self._order()

    def __repr__(self):
        return "Join({},{},{},{})".format(self.left_tensor_number, self.left_tensor_indices, self.right_tensor_number,
                                          self.right_tensor_indices)

    def _order(self):
        if self.left_tensor_number == self.right_tensor_number:
            raise ValueError("attempted to create a self-join for tensor {} (indices = {},{})".format(
                self.left_tensor_number, self.left_tensor_indices, self.right_tensor_indices))
        if self.right_tensor_number < self.left_tensor_number:
            self.left_tensor_number, self.right_tensor_number = self.right_tensor_number, self.left_tensor_number
            self.left_tensor_indices, self.right_tensor_indices = self.right_tensor_indices, self.left_tensor_indices

    def mergeWith(self, other):
        assert (self.left_tensor_number, self.right_tensor_number) == \
            (other.left_tensor_number, other.right_tensor_number)
        self.left_tensor_indices = self.left_tensor_indices + other.left_tensor_indices
        self.right_tensor_indices = self.right_tensor_indices + other.right_tensor_indices

    def update(self, old_tensor_number, new_tensor_number, index_map):
        """Point the side that referred to old_tensor_number at the tensor that
        replaced it, its indices renumbered by index_map."""
        if self.left_tensor_number == old_tensor_number:
            self.left_tensor_number = new_tensor_number
            self.left_tensor_indices = [index_map[i] for i in self.left_tensor_indices]
            self._order()
        elif self.right_tensor_number == old_tensor_number:
            self.right_tensor_number = new_tensor_number
            self.right_tensor_indices = [index_map[i] for i in self.right_tensor_indices]
            self._order()

    def _copy(self):
        new = object.__new__(Join)
        new.__dict__.update(self.__dict__)
        new.left_tensor_indices = list(self.left_tensor_indices)
        new.right_tensor_indices = list(self.right_tensor_indices)
        return new


def computeLengthAndCheckForGaps(indices, error_message):
    """1 + the largest index, after checking that 0..largest all occur (utils.py:322-332)."""
    return _length_without_gaps(list(indices), error_message)


def _length_without_gaps(indices, message):
    if not indices:
        return 0
    length = max(indices) + 1
    missing = set(range(length)) - set(indices)
    if missing:
        raise ValueError(message + ": " + str(missing))
    return length


def computePostContractionIndexMap(rank, contracted_indices, offset=0):
    """Old index -> index after the contracted ones are removed (utils.py:407-416)."""
    return _surviving_index_map(rank, contracted_indices, offset)


def invertPermutation(permutation):
    permutation = list(permutation)
    return [permutation.index(i) for i in range(len(permutation))]


def applyPermutation(permutation, values):
    return [values[i] for i in permutation]


def applyIndexMapTo(index_map, indices):
    return [index_map[i] for i in indices]


def _surviving_index_map(rank, contracted, offset=0):
    """Old index -> index in the contraction's result, for the indices that survive."""
    contracted = set(contracted)
    out, new = {}, 0
    for old in range(rank):
        if old not in contracted:
            out[old] = new + offset
            new += 1
    return out


def formDataContractor(joins, final_groups, tensor_ranks=None):
    """A function contracting its argument tensors (any objects of the Data
    protocol: TorchData, CostTracker) by the given joins (utils.py:562-711).

    The joins are carried out pairwise in the order given, each by
    ``contractWith`` into a new tensor whose axes are the left tensor's
    remaining axes followed by the right tensor's; later joins that come to
    connect the same two tensors are merged into the earlier one.  Tensors no
    join touches are combined by outer products in tensor-number order.  The
    result is ``join``-ed into ``final_groups`` (lists of (tensor number,
    index) pairs), or reduced to a scalar when there are none.  The argument
    lists are not modified.  The returned function checks ranks
    (UnexpectedTensorRankError) and joined dimensions (DimensionMismatchError)
    and carries its plan as ``.source``."""
    joins = [j._copy() for j in joins]
    final_groups = [list(g) for g in final_groups]
    observed = {}
    pairs = set()

    def observe(tensor_number, *indices):
        if tensor_number < 0:
            raise ValueError("tensor numbers must be non-negative, not {}".format(tensor_number))
        seen = observed.setdefault(tensor_number, set())
        for index in indices:
            if index in seen:
                raise ValueError("index {} of tensor {} appears twice".format(index, tensor_number))
            seen.add(index)

    for j in joins:
        observe(j.left_tensor_number, *j.left_tensor_indices)
        observe(j.right_tensor_number, *j.right_tensor_indices)
        pair = (j.left_tensor_number, j.right_tensor_number)
        if pair in pairs:
            raise ValueError("two joins appear between tensors {} and {} (recall that specified joins can contain "
                             "multiple indices)".format(*pair))
        pairs.add(pair)
    for group in final_groups:
        for tensor_number, index in group:
            observe(tensor_number, index)
    n = _length_without_gaps(list(observed), "the following tensor numbers were expected but not observed")
    if n == 0:
        raise ValueError("no tensors have been specified to be contracted")
    ranks = [_length_without_gaps(list(observed[t]),
                                  "the following indices of tensor {} were expected but not observed".format(t))
             for t in range(n)]
    if tensor_ranks is not None and list(tensor_ranks) != ranks:
        raise ValueError("the ranks of the arguments were specified to be {}, but inferred to be {}".format(
            list(tensor_ranks), ranks))
    checks = [(j.left_tensor_number, li, j.right_tensor_number, ri)
              for j in joins for li, ri in zip(j.left_tensor_indices, j.right_tensor_indices)]

    steps = []
    ranks = list(ranks)
    active = set(range(n))
    pending = list(joins)
    new_number = n
    while pending:
        j = pending.pop(0)
        lt, rt = j.left_tensor_number, j.right_tensor_number
        li, ri = list(j.left_tensor_indices), list(j.right_tensor_indices)
        active -= {lt, rt}
        active.add(new_number)
        ranks.append(ranks[lt] + ranks[rt] - 2 * len(li))
        steps.append((new_number, lt, rt, li, ri))
        lmap = _surviving_index_map(ranks[lt], li)
        rmap = _surviving_index_map(ranks[rt], ri, len(lmap))
        merged = {}
        kept = []
        for other in pending:
            other.update(lt, new_number, lmap)
            other.update(rt, new_number, rmap)
            pair = (other.left_tensor_number, other.right_tensor_number)
            if pair in merged:
                merged[pair].mergeWith(other)
            else:
                merged[pair] = other
                kept.append(other)
        pending = kept
        for group in final_groups:
            for k, (t, index) in enumerate(group):
                if t == lt:
                    group[k] = (new_number, lmap[index])
                elif t == rt:
                    group[k] = (new_number, rmap[index])
        new_number += 1
    order = sorted(active)
    final = order[0]
    offsets, off = {}, 0
    for t in order:
        offsets[t] = off
        off += ranks[t]
    groups = [[offsets[t] + index for t, index in group] for group in final_groups]

    lines = ["_{} = _{}.contractWith(_{},{},{})".format(*st) for st in steps]
    lines += ["_{0} = _{0}.contractWith(_{1},[],[])".format(final, t) for t in order[1:]]
    lines.append("return _{}.join(*{})".format(final, groups) if groups else "return _{}.extractScalar()".format(final))
    n_args, arg_ranks = n, ranks[:n]

    def contract(*tensors):
        if len(tensors) != n_args:
            raise TypeError("contractor takes {} tensors, got {}".format(n_args, len(tensors)))
        for t, (tensor, rank) in enumerate(zip(tensors, arg_ranks)):
            if tensor.ndim != rank:
                raise UnexpectedTensorRankError(t, rank, tensor.ndim)
        for lt, li, rt, ri in checks:
            if tensors[lt].shape[li] != tensors[rt].shape[ri]:
                raise DimensionMismatchError(lt, li, tensors[lt].shape[li], rt, ri, tensors[rt].shape[ri])
        slots = dict(enumerate(tensors))
        for new, lt, rt, li, ri in steps:
            slots[new] = slots.pop(lt).contractWith(slots.pop(rt), li, ri)
        result = slots.pop(final)
        for t in order[1:]:
            result = result.contractWith(slots.pop(t), [], [])
        return result.join(*groups) if groups else result.extractScalar()

    contract.source = "\n".join(lines)
    return contract


def prependDataContractor(*args, **keywords):
    """Decorator: the function receives formDataContractor(*args, **keywords)
    as its first argument (utils.py:221-223)."""
    return prepend(formDataContractor(*args, **keywords))


def maximumNewBandwidth(direction, shape):
    return int(np.prod(dropAt(shape, direction)))


def computeAndCheckNewDimension(shape, direction, by=None, to=None, do_as_much_as_possible=False):
    """(old, new, increment) of a bandwidth increase of axis ``direction``
    (utils.py:257-267): the new dimension may not exceed the product of the
    other axes; with do_as_much_as_possible it is clipped to it instead."""
    old_dimension = shape[direction]
    new_dimension = computeNewDimension(old_dimension, by=by, to=to)
    maximum = maximumNewBandwidth(direction, shape)
    if new_dimension > maximum:
        if not do_as_much_as_possible:
            raise ValueError("New dimension {} is greater than the current maximum dimension for direction {}, "
                             "which is {} (shape = {}).".format(new_dimension, direction, maximum, tuple(shape)))
        new_dimension = maximum
    return old_dimension, new_dimension, new_dimension - old_dimension


def __getattr__(name):
    # GPU numerics are imported lazily so that the tag algebra works without CUDA
    if name in ("relaxOver", "unitize", "computeCompressor", "computeCompressorForMatrixTimesItsDagger"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)


__all__ = [
    "DimensionMismatchError", "InvariantViolatedError", "RelaxFailed", "UnexpectedTensorRankError",
    "Multiplier", "prepend", "Pauli", "O", "L", "R", "A", "OA", "LA", "RA", "dropAt", "replaceAt",
    "computeNewDimension", "crand", "randomComplexSample", "checkForNaNsIn", "multiplyBySingleSiteOperator",
    "buildProductTensor", "buildTensor", "Join", "formDataContractor", "prependDataContractor",
    "computeAndCheckNewDimension", "computeLengthAndCheckForGaps", "computePostContractionIndexMap",
    "invertPermutation", "applyPermutation", "applyIndexMapTo",
    "maximumNewBandwidth", "relaxOver", "unitize", "computeCompressor", "computeCompressorForMatrixTimesItsDagger",
]
