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


def maximumNewBandwidth(direction, shape):
    return int(np.prod(dropAt(shape, direction)))


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
    "buildProductTensor", "buildTensor",
    "maximumNewBandwidth", "relaxOver", "unitize", "computeCompressor", "computeCompressorForMatrixTimesItsDagger",
]
