"""A stage-3 operator's library calls (Stage3Operator._pack): one group per
shape class of (S2_0, S2_1) pairs, split where a class has more tags of
either half or more terms than one call takes.  Host logic on CPU tensors
(the groups hold only pointer and index tables), no GPU."""
import random

import torch

from carcassonne_gb300 import _lib
from carcassonne_gb300.data import TorchData
from carcassonne_gb300.tensors._2d.dense import Stage3Operator


def _cpu(shape):
    d = TorchData.__new__(TorchData)
    d._t = torch.zeros(shape, dtype=torch.complex128)
    return d


def test_groups_respect_the_call_limits_and_cover_every_term():
    rng = random.Random(3)
    # class A: S2_0 (1,2,...) with S2_1 (2,1,...); class B: S2_0 (2,1,...) with S2_1 (1,2,...)
    s2_0 = [_cpu((1, 2, 1, 1, 1, 1)) for _ in range(100)] + [_cpu((2, 1, 1, 1, 1, 1)) for _ in range(20)]
    s2_1 = [_cpu((2, 1, 1, 1, 1, 1)) for _ in range(90)] + [_cpu((1, 2, 1, 1, 1, 1)) for _ in range(15)]
    ops = [_cpu((1, 1)) for _ in range(3)]
    terms = []
    for _ in range(900):
        if rng.random() < 0.8:
            terms.append((rng.randrange(100), rng.randrange(90), rng.randrange(-1, 3)))
        else:
            terms.append((100 + rng.randrange(20), 90 + rng.randrange(15), rng.randrange(-1, 3)))
    op = Stage3Operator(s2_0, s2_1, ops, terms, 1)
    ptr0 = {t.data_ptr(): i for i, t in enumerate(op.s2_0)}
    ptr1 = {t.data_ptr(): i for i, t in enumerate(op.s2_1)}
    seen = []
    for g in op._groups:
        assert 1 <= g["n0"] <= _lib.MAX_SLOTS and 1 <= g["n1"] <= _lib.MAX_SLOTS
        assert 1 <= len(g["terms"]) <= _lib.MAX_ENTRIES
        t0 = [ptr0[int(p)] for p in g["k0"][: g["n0"]]]
        t1 = [ptr1[int(p)] for p in g["k1"][: g["n1"]]]
        assert all(tuple(op.s2_0[i].shape) == g["shape0"] for i in t0)
        assert all(tuple(op.s2_1[i].shape) == g["shape1"] for i in t1)
        seen.extend((t0[a], t1[b], c) for a, b, c in g["terms"])
    assert len(op._groups) > 2  # class A needed more than one call
    # every term once, and each shape class in its original order
    in_a = lambda t: t[0] < 100
    assert [t for t in seen if in_a(t)] == [t for t in terms if in_a(t)]
    assert [t for t in seen if not in_a(t)] == [t for t in terms if not in_a(t)]
