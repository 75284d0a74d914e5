"""Host-side builders and index helpers of the public API on the CPU:
makeMPO (sparse.py:265-287), computeAndCheckNewDimension (utils.py:257-267),
the permutation and index-map helpers, prependDataContractor."""
import numpy as np
import pytest

from carcassonne_gb300.data.cost_tracker import CostTracker
from carcassonne_gb300.sparse import Complete, Identity, Singleton, TwoSiteOperator, makeMPO
from carcassonne_gb300.utils import (Join, Pauli, applyIndexMapTo, applyPermutation, computeAndCheckNewDimension,
                                     computeLengthAndCheckForGaps, computePostContractionIndexMap, invertPermutation,
                                     prependDataContractor)


def test_make_mpo_channels():
    Z, X, Y = Pauli.Z.copy(), Pauli.X.copy(), Pauli.Y.copy()
    keep = [Z.copy(), X.copy(), Y.copy()]
    T, rb, rt, lb, lt = makeMPO(Pauli.I, [Z, X], [(X, -X), (Y, 2 * Y)])
    assert T.shape == (4, 4, 2, 2) and T.dtype == np.complex128
    want = np.zeros((4, 4, 2, 2), np.complex128)
    want[0, 0] = want[3, 3] = Pauli.I
    want[0, 3] = Z + X                     # one-site terms summed
    want[0, 1], want[1, 3] = -X, X         # term 0: second half from channel 0, first half into the end channel
    want[0, 2], want[2, 3] = 2 * Y, Y
    assert np.array_equal(T, want)
    assert rb == [1, 0, 0, 0] and lb == [0, 0, 0, 1]
    assert rt == [Identity(), TwoSiteOperator(0, 2), TwoSiteOperator(1, 2), Complete()]
    assert lt == [Complete(), TwoSiteOperator(0, 2), TwoSiteOperator(1, 2), Identity()]
    assert all(np.array_equal(a, b) for a, b in zip([Z, X, Y], keep))  # arguments untouched


def test_make_mpo_field_only():
    T, rb, rt, lb, lt = makeMPO(Pauli.I, [Pauli.Z])
    assert T.shape == (2, 2, 2, 2)
    assert np.array_equal(T[0, 1], Pauli.Z) and np.array_equal(T[1, 0], np.zeros((2, 2)))
    assert rt == [Identity(), Complete()] and lt == [Complete(), Identity()]
    assert isinstance(Identity(), Singleton) and Identity() is Identity()


def test_compute_and_check_new_dimension():
    assert computeAndCheckNewDimension((2, 3, 4), 0, by=3) == (2, 5, 3)
    assert computeAndCheckNewDimension((2, 3, 4), 1, to=8) == (3, 8, 5)
    assert computeAndCheckNewDimension((2, 3, 4), 0, by=20, do_as_much_as_possible=True) == (2, 12, 10)
    with pytest.raises(ValueError):
        computeAndCheckNewDimension((2, 3, 4), 0, by=20)
    with pytest.raises(ValueError):
        computeAndCheckNewDimension((2, 3, 4), 0, to=1)


def test_index_helpers():
    p = [2, 0, 3, 1]
    q = invertPermutation(p)
    assert applyPermutation(p, applyPermutation(q, list("abcd"))) == list("abcd")
    assert computePostContractionIndexMap(5, [1, 3]) == {0: 0, 2: 1, 4: 2}
    assert computePostContractionIndexMap(3, [0], offset=4) == {1: 4, 2: 5}
    assert applyIndexMapTo({0: 5, 2: 7}, [2, 0]) == [7, 5]
    assert computeLengthAndCheckForGaps({0, 1, 2}, "gap") == 3
    with pytest.raises(ValueError):
        computeLengthAndCheckForGaps({0, 2}, "gap")


def test_prepend_data_contractor():
    @prependDataContractor([Join(0, 1, 1, 0)], [[(0, 0)], [(1, 1)]])
    def matmul_cost(contract, a, b):
        return contract(a, b).cost

    assert matmul_cost(CostTracker((2, 3)), CostTracker((3, 5))) == 30
