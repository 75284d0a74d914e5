"""Absorptions on the tensor cores (absorption_precision("tc")).

absorbDenseSideIntoCornerFromLeft/Right (tensors/_2d/dense.py:10-21) and
absorbDenseCenterSS/SOSIntoSide (:22-81) with every tag pair on tcgen05
(split-BF16 operands, FP32 accumulation, FP64 reduction) against the
reference's recorded outputs (tests/golden/dense.npz) and against the FP64
path at the growth runs' sizes (c = 8 boundaries, D = 4 centers), within
5e-5 of the result's scale; a whole contractTowards of a grown Heisenberg
system in both precisions.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TC_TOL = 5e-5


@pytest.fixture(scope="module")
def dense():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300.tensors._2d import dense as d
    return d


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_golden_absorptions_on_tensor_cores(dense):
    from carcassonne_gb300.data import TorchData
    g = np.load(os.path.join(GOLD, "dense.npz"))
    D = lambda k: TorchData(g[k])
    with dense.absorption_precision("tc"):
        for case in range(4):
            assert rel(dense.absorbDenseSideIntoCornerFromLeft(D(f"absL_{case}_C"), D(f"absL_{case}_S")).toArray(),
                       g[f"absL_{case}_out"]) < TC_TOL
            assert rel(dense.absorbDenseSideIntoCornerFromRight(D(f"absR_{case}_C"), D(f"absR_{case}_S")).toArray(),
                       g[f"absR_{case}_out"]) < TC_TOL
            for direction in range(4):
                key = f"center_{case}_{direction}"
                out = dense.absorbDenseCenterSOSIntoSide(direction, D(key + "_side"), D(key + "_S"), D(key + "_O"))
                assert rel(out.toArray(), g[key + "_SOS"]) < TC_TOL
                out = dense.absorbDenseCenterSSIntoSide(direction, D(key + "_side"), D(key + "_S"))
                assert rel(out.toArray(), g[key + "_SS"]) < TC_TOL


@pytest.mark.parametrize("direction", range(4))
def test_config_size_absorptions(dense, direction):
    from carcassonne_gb300.data import TorchData
    rng = np.random.default_rng(direction)
    cn = lambda *s: TorchData(rng.standard_normal(s) + 1j * rng.standard_normal(s))
    c, D, d = 8, 4, 2
    corner = cn(c, c, 1, c, c, 1)
    side = cn(c, c, 1, c, c, 1, D, D)
    state = cn(D, D, D, D, d)
    op = cn(d, d)
    fns = [lambda: dense.absorbDenseSideIntoCornerFromLeft(corner, side),
           lambda: dense.absorbDenseSideIntoCornerFromRight(corner, side),
           lambda: dense.absorbDenseCenterSOSIntoSide(direction, side, state, op)]
    for fn in fns:
        ref = fn().toArray()
        with dense.absorption_precision("tc"):
            got = fn().toArray()
        assert rel(got, ref) < TC_TOL


def test_contract_towards_tc_matches_fp64(dense):
    """One contractTowards of a grown Heisenberg system (D = 4) in both
    precisions: every corner and side tag within 5e-5."""
    from copy import copy
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.data import TorchData
    system = workloads.bond_start_system("heis", 4, 2)
    for step in range(5):
        system.setStateCenter(TorchData(workloads.growth_center((4, 4, 4, 4, 2), 900 + step)))
        system.contractTowards(step % 4)
    system.setStateCenter(TorchData(workloads.growth_center((4, 4, 4, 4, 2), 905)))
    a, b = copy(system), copy(system)
    a.contractTowards(1)
    with dense.absorption_precision("tc"):
        b.contractTowards(1)
    for ca, cb in zip(a.corners + a.sides, b.corners + b.sides):
        assert list(ca) == list(cb)
        for t in ca:
            assert rel(cb[t].toArray(), ca[t].toArray()) < TC_TOL, t
