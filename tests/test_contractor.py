"""formDataContractor and Join (utils.py:45-101, :562-711) on the CPU.

Cost: the contractor run on CostTracker operands gives the multiply-add counts
of the reference's cost-model tests (tests/test_data_cost_tracker.py), which
fix the pairwise order (joins in the order given, joins between the same two
tensors merged, outer products last).  Values: the same contractors on a
numpy-backed stand-in of the Data protocol against einsum."""
import random
from functools import reduce
from operator import mul

import numpy as np
import pytest

from carcassonne_gb300.data.cost_tracker import CostTracker
from carcassonne_gb300.utils import DimensionMismatchError, Join, UnexpectedTensorRankError, formDataContractor

prod = lambda xs: reduce(mul, xs, 1)  # noqa: E731
CASES = 25


class NDStandIn:
    """The parts of the Data protocol a contractor uses, on numpy arrays."""

    def __init__(self, a):
        self.a = np.asarray(a)
        self.shape = self.a.shape
        self.ndim = self.a.ndim

    def contractWith(self, other, self_axes, other_axes):
        return NDStandIn(np.tensordot(self.a, other.a, (list(self_axes), list(other_axes))))

    def join(self, *groups):
        groups = [[g] if isinstance(g, (int, np.integer)) else list(g) for g in groups]
        t = self.a.transpose([i for g in groups for i in g])
        return NDStandIn(t.reshape([prod(self.a.shape[i] for i in g) for g in groups]))

    def extractScalar(self):
        return self.a.item()


def _shape(rng, ndim, hi=3):
    return tuple(rng.randint(1, hi) for _ in range(ndim))


def test_outer_product():
    rng = random.Random(1)
    for _ in range(CASES):
        tensors = [CostTracker(_shape(rng, rng.randint(1, 3))) for _ in range(rng.randint(1, 5))]
        groups = [[(t, i)] for t, x in enumerate(tensors) for i in range(x.ndim)]
        got = formDataContractor([], groups)(*tensors).cost
        want, size = 0, prod(tensors[0].shape)
        for x in tensors[1:]:
            size *= prod(x.shape)
            want += size
        assert got == want


def test_inner_product_to_scalar():
    rng = random.Random(2)
    for _ in range(CASES):
        ndim = rng.randint(1, 5)
        shape = _shape(rng, ndim, 5)
        perm = list(range(ndim))
        rng.shuffle(perm)
        inv = [perm.index(i) for i in range(ndim)]
        pairs = list(zip(range(ndim), inv))
        rng.shuffle(pairs)
        a_axes, b_axes = zip(*pairs)
        f = formDataContractor([Join(0, list(a_axes), 1, list(b_axes))], [])
        assert f(CostTracker(shape), CostTracker([shape[p] for p in perm])).cost == prod(shape)
        a = np.random.default_rng(0).standard_normal(shape)
        b = a.transpose(perm).copy()
        assert np.isclose(f(NDStandIn(a), NDStandIn(b)), np.sum(a * a))


def test_inner_product_to_tensor():
    rng = random.Random(3)
    for _ in range(CASES):
        left, middle, right = (_shape(rng, rng.randint(1, 3)) for _ in range(3))
        na, nb = len(left) + len(middle), len(middle) + len(right)
        pa = list(range(na))
        rng.shuffle(pa)
        pb = list(range(nb))
        rng.shuffle(pb)
        a_shape = [(left + middle)[p] for p in pa]
        b_shape = [(middle + right)[p] for p in pb]
        a_pos = [pa.index(i) for i in range(na)]  # where logical axis i sits in A
        b_pos = [pb.index(i) for i in range(nb)]
        a_left, a_mid = sorted(a_pos[:len(left)]), a_pos[len(left):]
        b_mid, b_right = b_pos[:len(middle)], sorted(b_pos[len(middle):])
        f = formDataContractor([Join(0, a_mid, 1, b_mid)], [[(0, i)] for i in a_left] + [[(1, i)] for i in b_right])
        assert f(CostTracker(a_shape), CostTracker(b_shape)).cost == prod(left) * prod(middle) * prod(right)


def test_matrix_products():
    rng = random.Random(4)
    for _ in range(CASES):
        a, b, c, d, e = (rng.randint(1, 10) for _ in range(5))
        f2 = formDataContractor([Join(0, 1, 1, 0)], [[(0, 0)], [(1, 1)]])
        assert f2(CostTracker((a, b)), CostTracker((b, c))).cost == a * b * c
        f3 = formDataContractor([Join(0, 1, 1, 0), Join(1, 1, 2, 0)], [[(0, 0)], [(2, 1)]])
        assert f3(*(CostTracker(s) for s in ((a, b), (b, c), (c, d)))).cost == a * b * c + a * c * d
        f4 = formDataContractor([Join(0, 1, 1, 0), Join(2, 1, 3, 0), Join(1, 1, 2, 0)], [[(0, 0)], [(3, 1)]])
        assert f4(*(CostTracker(s) for s in ((a, b), (b, c), (c, d), (d, e)))).cost == a * b * c + c * d * e + a * c * e
        mats = [np.random.default_rng(a).standard_normal(s) for s in ((a, b), (b, c), (c, d), (d, e))]
        got = f4(*(NDStandIn(m) for m in mats)).a
        assert np.allclose(got, mats[0] @ mats[1] @ mats[2] @ mats[3])


def test_chain_of_matrices():
    rng = random.Random(5)
    for _ in range(CASES):
        k = rng.randint(1, 10)
        dims = [rng.randint(1, 10) for _ in range(k + 1)]
        f = formDataContractor([Join(i, 1, i + 1, 0) for i in range(k - 1)], [[(0, 0)], [(k - 1, 1)]])
        want, b = 0, dims[1]
        for i in range(1, k):
            want += dims[0] * b * dims[i + 1]
            b = dims[i + 1]
        assert f(*(CostTracker((dims[i], dims[i + 1])) for i in range(k))).cost == want


def test_triangle():
    rng = random.Random(6)
    f = formDataContractor([Join(0, 0, 2, 1), Join(0, 2, 1, 1), Join(1, 0, 2, 2)], [[(0, 1)], [(1, 2)], [(2, 0)]])
    for _ in range(CASES):
        a, b, c, d, e, g = (rng.randint(1, 6) for _ in range(6))
        shapes = ((a, e, b), (c, b, g), (d, a, c))
        assert f(*(CostTracker(s) for s in shapes)).cost == a * b * c * d * e + b * c * d * e * g
        ts = [np.random.default_rng(7).standard_normal(s) for s in shapes]
        assert np.allclose(f(*(NDStandIn(t) for t in ts)).a, np.einsum("aeb,cbf,dac->efd", *ts))


def test_merged_groups():
    rng = random.Random(7)
    f1 = formDataContractor([Join(0, 2, 1, 2)], [[(0, 0), (1, 0)], [(0, 1), (1, 1)], [(1, 3)]])
    f2 = formDataContractor([Join(0, 3, 1, 2)], [[(0, 0), (1, 0)], [(0, 1), (1, 1)], [(0, 2), (1, 3)], [(1, 4)]])
    for _ in range(CASES):
        a, b, c, d, e, g, h, k = (rng.randint(1, 5) for _ in range(8))
        assert f1(CostTracker((a, b, c)), CostTracker((d, e, c, g))).cost == a * b * c * d * e * g
        assert f2(CostTracker((a, b, c, d)), CostTracker((e, g, d, h, k))).cost == a * b * c * d * e * g * h * k
        A = np.random.default_rng(1).standard_normal((a, b, c))
        B = np.random.default_rng(2).standard_normal((d, e, c, g))
        want = np.einsum("abc,decf->adbef", A, B).reshape(a * d, b * e, g)
        assert np.allclose(f1(NDStandIn(A), NDStandIn(B)).a, want)


def test_argument_checks():
    f = formDataContractor([Join(0, 1, 1, 0)], [[(0, 0)], [(1, 1)]])
    with pytest.raises(UnexpectedTensorRankError):
        f(CostTracker((2, 3, 4)), CostTracker((3, 5)))
    with pytest.raises(DimensionMismatchError):
        f(CostTracker((2, 3)), CostTracker((4, 5)))
    with pytest.raises(ValueError):
        Join(1, 0, 1, 1)                       # self-join
    with pytest.raises(ValueError):
        formDataContractor([Join(0, 0, 1, 0), Join(1, 1, 0, 1)], [])   # two joins between one pair
    with pytest.raises(ValueError):
        formDataContractor([Join(0, 1, 2, 0)], [[(0, 0)], [(2, 1)]])    # tensor 1 never observed
    joins, groups = [Join(0, 1, 1, 0)], [[(0, 0)], [(1, 1)]]
    formDataContractor(joins, groups)
    assert repr(joins[0]) == "Join(0,[1],1,[0])" and groups == [[(0, 0)], [(1, 1)]]  # arguments untouched
