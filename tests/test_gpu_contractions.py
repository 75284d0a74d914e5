"""GPU parity of the FP64 contraction path against the reference's golden
vectors and the CPU oracle (bit-exact schedules, 1e-12 relative on values)."""
import json
import os

import numpy as np
import pytest
import torch

from oracle import carc_oracle as orc
from tests.product_tags import parse

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def mods():
    _need_gpu()
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.tensors._2d import dense, sparse
    return TorchData, dense, sparse


def rel(a, b):
    a = a.toArray() if hasattr(a, "toArray") else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("case", range(4))
def test_dense_contractors_match_golden(mods, case):
    TorchData, dense, _ = mods
    g = np.load(os.path.join(GOLD, "dense.npz"))
    D = lambda k: TorchData(g[k])
    assert rel(dense.formNormalizationStage1(D(f"stage1_{case}_C"), D(f"stage1_{case}_S")), g[f"stage1_{case}_out"]) < TOL
    assert rel(dense.absorbDenseSideIntoCornerFromLeft(D(f"absL_{case}_C"), D(f"absL_{case}_S")),
               g[f"absL_{case}_out"]) < TOL
    assert rel(dense.absorbDenseSideIntoCornerFromRight(D(f"absR_{case}_C"), D(f"absR_{case}_S")),
               g[f"absR_{case}_out"]) < TOL
    assert rel(dense.formNormalizationStage2(D(f"stage2_{case}_A"), D(f"stage2_{case}_B")), g[f"stage2_{case}_out"]) < TOL
    s20, s21, op, v = (D(f"stage3_{case}_{k}") for k in ("s20", "s21", "op", "v"))
    m = dense.formDenseStage3(s20, s21, op)
    assert rel(m(v), g[f"stage3_{case}_Hv"]) < TOL
    assert rel(m.formMatrix(), g[f"stage3_{case}_H"]) < TOL
    assert (m.cost_of_multiply, m.cost_of_formMatrix) == tuple(int(x) for x in g[f"stage3_{case}_cost"])
    nm = dense.formNormalizationStage3(s20, s21, TorchData.newIdentity(op.shape[0]))
    assert rel(nm(v), g[f"stage3_{case}_Nv"]) < TOL
    assert rel(nm.formMatrix(), g[f"stage3_{case}_N"]) < TOL
    assert (nm.cost_of_multiply, nm.cost_of_formMatrix) == tuple(int(x) for x in g[f"stage3_{case}_ncost"])
    for direction in range(4):
        key = f"center_{case}_{direction}"
        side, st, o = D(key + "_side"), D(key + "_S"), D(key + "_O")
        assert rel(dense.absorbDenseCenterSSIntoSide(direction, side, st), g[key + "_SS"]) < TOL
        assert rel(dense.absorbDenseCenterSOSIntoSide(direction, side, st, o), g[key + "_SOS"]) < TOL


def _load_traj():
    with open(os.path.join(GOLD, "tables.json")) as f:
        tables = json.load(f)
    return tables, np.load(os.path.join(GOLD, "trajectory.npz"))


def _boundaries(TorchData, traj, rec, name, step):
    corners, sides = [], []
    for i in range(4):
        corners.append({parse(t): TorchData(traj[f"{name}_{step}_corner{i}_{j}"]) for j, t in enumerate(rec["corners"][i])})
        sides.append({parse(t): TorchData(traj[f"{name}_{step}_side{i}_{j}"]) for j, t in enumerate(rec["sides"][i])})
    op_tags = [parse(str(t)) for t in traj[f"{name}_op_tags"]]
    op = {t: TorchData(traj[f"{name}_op_{k}"]) for k, t in enumerate(op_tags)}
    return corners, sides, op


@pytest.mark.parametrize("name", ["ti", "heis", "ising_ud"])
def test_trajectory_operator_and_absorption(mods, name):
    TorchData, dense, sparse = mods
    tables, traj = _load_traj()
    steps = tables[name]["steps"]
    rng = np.random.default_rng(11)
    for step, direction in enumerate(steps):
        rec = tables[name]["records"][step]
        corners, sides, op = _boundaries(TorchData, traj, rec, name, step)
        H, N = sparse.formExpectationAndNormalizationMultipliers(corners, sides, op)
        Hg, Ng = traj[f"{name}_{step}_H"], traj[f"{name}_{step}_N"]
        assert rel(H.formMatrix(), Hg) < 1e-11
        assert rel(N.formMatrix(), Ng) < 1e-11
        shape = traj[f"{name}_{step}_state"].shape
        v = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        assert rel(H(TorchData(v)), (Hg @ v.ravel()).reshape(shape)) < 1e-11
        assert rel(N(TorchData(v)), (Ng @ v.ravel()).reshape(shape)) < 1e-11
        # absorption towards `direction` with the reference's minimized center
        if step + 1 < len(steps):
            iso, _, _ = orc.normalize_axis(traj[f"{name}_{step}_minstate"], orc.O(direction))
            iso_d = TorchData(iso)
            L, R = orc.L(direction), orc.R(direction)
            new_corner_d = sparse.absorbSparseSideIntoCornerFromLeft(corners[direction], sides[L])
            new_side = sparse.absorbSparseCenterSOSIntoSide(direction, sides[direction], iso_d, op)
            new_corner_r = sparse.absorbSparseSideIntoCornerFromRight(corners[R], sides[R])
            nxt = tables[name]["records"][step + 1]
            for got, idx, kind in ((new_corner_d, direction, "corner"), (new_side, direction, "side"),
                                   (new_corner_r, R, "corner")):
                tags = nxt[kind + "s"][idx]
                assert [repr(t) for t in got] == tags
                for j, t in enumerate(tags):
                    want = traj[f"{name}_{step + 1}_{kind}{idx}_{j}"]
                    assert rel(got[parse(t)], want) < 1e-10, (kind, idx, t)


def test_grouped_table_above_the_slot_limits():
    """A grouped FP64 table with more operands, outputs and entries than one
    library call takes (64 slots, 512 entries) is split by the planner and
    still gives every output its sum; an output fed by more than 64 operands
    is accumulated over consecutive calls."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import engine
    rng = np.random.default_rng(21)
    cplx = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    A = [cplx(8, 6) for _ in range(90)]
    B = [cplx(6, 5) for _ in range(75)]
    n_c = 100
    entries = [(int(rng.integers(90)), int(rng.integers(75)), int(rng.integers(n_c - 1))) for _ in range(700)]
    entries += [(i, i % 75, n_c - 1) for i in range(90)]  # the last output: 90 distinct A operands
    outs = [torch.full((8, 5), 7.0 + 0j, dtype=torch.complex128, device="cuda") for _ in range(n_c)]
    engine.contract_grouped("ij,jk->ik", [torch.as_tensor(a).cuda() for a in A], [torch.as_tensor(b).cuda() for b in B],
                            outs, entries)
    ref = [np.zeros((8, 5), complex) for _ in range(n_c)]
    for a, b, c in entries:
        ref[c] += A[a] @ B[b]
    for c in range(n_c):
        got = outs[c].cpu().numpy()
        assert np.abs(got - ref[c]).max() <= 1e-13 * max(1.0, np.abs(ref[c]).max()), c
