"""Pin the CPU oracle against golden vectors produced by the reference itself.

The fixtures under tests/golden/ were written by tests/golden/make_golden.py,
which runs the reference implementation; these tests need no GPU.
"""
import json
import os

import numpy as np
import pytest

from oracle import carc_oracle as orc
from tests.tagrepr import parse_tag, tag_repr

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def dense():
    return np.load(os.path.join(GOLD, "dense.npz"))


@pytest.fixture(scope="module")
def tables():
    with open(os.path.join(GOLD, "tables.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def traj():
    return np.load(os.path.join(GOLD, "trajectory.npz"))


@pytest.fixture(scope="module")
def numerics():
    return np.load(os.path.join(GOLD, "numerics.npz"))


def close(a, b, tol=1e-11):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= tol * scale, np.abs(a - b).max() / scale


CASES = range(4)


@pytest.mark.parametrize("case", CASES)
def test_dense_contractors(dense, case):
    g = dense
    close(orc.stage1(g[f"stage1_{case}_C"], g[f"stage1_{case}_S"]), g[f"stage1_{case}_out"])
    close(orc.absorb_side_into_corner_from_left(g[f"absL_{case}_C"], g[f"absL_{case}_S"]), g[f"absL_{case}_out"])
    close(orc.absorb_side_into_corner_from_right(g[f"absR_{case}_C"], g[f"absR_{case}_S"]), g[f"absR_{case}_out"])
    close(orc.stage2(g[f"stage2_{case}_A"], g[f"stage2_{case}_B"]), g[f"stage2_{case}_out"])
    s20, s21, op, v = (g[f"stage3_{case}_{k}"] for k in ("s20", "s21", "op", "v"))
    close(orc.stage3_matvec(s20, s21, op, v), g[f"stage3_{case}_Hv"])
    close(orc.stage3_matvec(s20, s21, None, v), g[f"stage3_{case}_Nv"])
    close(orc.stage3_matrix(s20, s21, op), g[f"stage3_{case}_H"])
    close(orc.stage3_matrix(s20, s21, np.eye(op.shape[0])), g[f"stage3_{case}_N"])
    cm, cf = orc.stage3_costs(s20, s21, op.shape[0], False)
    assert (cm, cf) == tuple(int(x) for x in g[f"stage3_{case}_cost"])
    cm, cf = orc.stage3_costs(s20, s21, op.shape[0], True)
    assert (cm, cf) == tuple(int(x) for x in g[f"stage3_{case}_ncost"])
    for direction in range(4):
        key = f"center_{case}_{direction}"
        side, st, o = g[key + "_side"], g[key + "_S"], g[key + "_O"]
        close(orc.absorb_center_into_side(direction, side, st), g[key + "_SS"])
        close(orc.absorb_center_into_side(direction, side, st, o), g[key + "_SOS"])


def _rules_for(call_kind, direction=None):
    return {
        "stage1": orc.rules_stage1,
        "stage2": orc.rules_stage2,
        "absL": orc.rules_absorb_corner_left,
        "absR": orc.rules_absorb_corner_right,
    }[call_kind]()


def _center_table(direction, tags_side, tags_op):
    rules = orc.rules_absorb_center(direction)
    out_tags, entries = [], []
    for i, s in enumerate(tags_side):
        for j, c in enumerate(tags_op):
            rule = rules.get((s[0], c[0]))
            if rule is None:
                continue
            tag, _ = rule(s, c)
            if tag is None:
                continue
            if tag not in out_tags:
                out_tags.append(tag)
            entries.append((i, j, out_tags.index(tag)))
    return out_tags, entries


def _check_call(call, kind, direction=None):
    t1 = [parse_tag(t) for t in call["tags1"]]
    t2 = [parse_tag(t) for t in call["tags2"]]
    if kind == "center":
        out_tags, entries = _center_table(direction, t1, t2)
    else:
        out_tags, entries = orc.sparse_table(_rules_for(kind), t1, t2)
    got = [[i, j, tag_repr(out_tags[k])] for i, j, k in entries]
    assert got == call["entries"]
    assert [tag_repr(t) for t in out_tags] == call["result"]


@pytest.mark.parametrize("name", ["ti", "heis", "ising_ud"])
def test_tag_tables_bit_exact(tables, name):
    for rec in tables[name]["records"]:
        calls = rec["stage_calls"]
        # argument evaluation order of tensors/_2d/sparse.py:59-71:
        # stage1, stage1, stage2, stage1, stage1, stage2
        assert len(calls) == 6
        for k, c in enumerate(calls):
            _check_call(c, "stage2" if k in (2, 5) else "stage1")
        d = rec["direction"]
        a = rec["absorb_calls"]
        assert len(a) == 3
        _check_call(a[0], "absL")
        _check_call(a[1], "center", d)
        _check_call(a[2], "absR")
        s3 = rec["stage3"]
        terms = orc.stage3_terms([parse_tag(t) for t in s3["s2_0"]], [parse_tag(t) for t in s3["s2_1"]],
                                 [parse_tag(t) for t in s3["op"]])
        assert [[a_, b_, c_, int(e_)] for a_, b_, c_, e_ in terms] == s3["terms"]


def _system_at(traj, name, step, tables):
    rec = tables[name]["records"][step]
    corners = []
    sides = []
    for i in range(4):
        corners.append({parse_tag(t): traj[f"{name}_{step}_corner{i}_{j}"] for j, t in enumerate(rec["corners"][i])})
        sides.append({parse_tag(t): traj[f"{name}_{step}_side{i}_{j}"] for j, t in enumerate(rec["sides"][i])})
    op_tags = [parse_tag(str(t)) for t in traj[f"{name}_op_tags"]]
    op = {t: traj[f"{name}_op_{k}"] for k, t in enumerate(op_tags)}
    return orc.OracleSystem(corners, sides, traj[f"{name}_{step}_state"], op)


@pytest.mark.parametrize("name", ["ti", "heis", "ising_ud"])
def test_trajectory_matrices_and_energies(traj, tables, name):
    nsteps = len(tables[name]["steps"])
    for step in range(nsteps):
        sysm = _system_at(traj, name, step, tables)
        H, N, _ = sysm.multipliers()
        close(H.formMatrix(), traj[f"{name}_{step}_H"], 1e-10)
        close(N.formMatrix(), traj[f"{name}_{step}_N"], 1e-10)
        e, n = sysm.expectation_and_normalization()
        ref = traj[f"{name}_{step}_E"]
        assert abs(e - ref[1]) <= 1e-9 * max(1, abs(ref[1]))
        w = sysm.minimize_full()
        assert abs(w - ref[0].real) <= 1e-9 * max(1, abs(ref[0]))
        # the absorbed boundaries of the next step come from the reference's contractTowards
        if step + 1 < nsteps:
            sysm.state = traj[f"{name}_{step}_minstate"]
            sysm.contract_towards(tables[name]["steps"][step])
            nxt = _system_at(traj, name, step + 1, tables)
            for i in range(4):
                for t, v in nxt.corners[i].items():
                    close(sysm.corners[i][t], v, 1e-9)
                for t, v in nxt.sides[i].items():
                    close(sysm.sides[i][t], v, 1e-9)
            close(sysm.state, traj[f"{name}_{step}_after_state"], 1e-8)


def test_normalize_axis(numerics):
    g = numerics
    keys = sorted({k.rsplit("_", 1)[0] for k in g.files if k.startswith("nax_") and k.endswith("_in")})
    assert keys
    for key in keys:
        axis = int(key.split("_")[2])
        t = g[key + "_in"]
        iso, nz, dz = orc.normalize_axis(t, axis)
        close(iso, g[key + "_iso"], 1e-10)
        close(nz, g[key + "_norm"], 1e-10)
        close(dz, g[key + "_denorm"], 1e-10)
        a, b = orc.normalize_axis(t, axis, True)
        close(a, g[key + "_sq_a"], 1e-10)
        close(b, g[key + "_sq_b"], 1e-10)


def test_unitize_and_compressor(numerics):
    g = numerics
    for case in range(3):
        close(orc.unitize(g[f"unitize_{case}_in"]), g[f"unitize_{case}_out"], 1e-10)
    for case in range(3):
        old, new = (int(x) for x in g[f"cc_{case}_meta"])
        c, _ = orc.compute_compressor(old, new, g[f"cc_{case}_in"])
        ref = g[f"cc_{case}_c"]
        # eigenvectors are defined up to a phase per row: compare projectors
        close(c.conj().T @ c, ref.conj().T @ ref, 1e-9)
        cn_, icn = orc.compute_compressor(old, new, g[f"cc_{case}_in"], True)
        close(cn_.conj().T @ icn, g[f"cc_{case}_cn"].conj().T @ g[f"cc_{case}_icn"], 1e-9)


def test_product_compressor_invariant(numerics):
    g = numerics
    rng = np.random.default_rng(3)
    for case in range(2):
        Lf, Rf, Pref = g[f"pc_{case}_L"], g[f"pc_{case}_R"], g[f"pc_{case}_P"]
        new = Pref.shape[0]
        init = rng.standard_normal((Lf.shape[1], new)) + 0j
        P = orc.product_compressor(Lf, Rf, new, init)
        for PP in (P, Pref):
            Lc = orc.absorb_matrix_at(orc.absorb_matrix_at(Lf, 1, PP), 2, PP.conj())
            Rc = orc.absorb_matrix_at(orc.absorb_matrix_at(Rf, 0, PP.conj()), 1, PP)
            close(np.tensordot(Lc, Rc, ((1, 2, 3), (0, 1, 2))), g[f"pc_{case}_exact"], 1e-8)


def test_relax_over(numerics):
    g = numerics
    for case in range(3):
        h, nm, v0 = g[f"relax_{case}_H"], g[f"relax_{case}_N"], g[f"relax_{case}_v0"]
        x, lam, count = orc.relax_over(v0.copy(), h, nm)
        close(x, g[f"relax_{case}_x"], 1e-7)
