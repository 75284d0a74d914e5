"""Host-side (no GPU) checks of the product: the tag-pair schedules and
stage-3 term tables must equal the reference's, bit for bit, and the C ABI
library must load and export every symbol its header declares."""
import json
import os
import re

import pytest

from carcassonne_gb300 import _lib
from carcassonne_gb300.sparse import compileSparseSchedule
from carcassonne_gb300.tensors._2d import sparse as tsp
from tests.product_tags import parse

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def tables():
    with open(os.path.join(GOLD, "tables.json")) as f:
        return json.load(f)


def _check(call, rules):
    t1 = [parse(t) for t in call["tags1"]]
    t2 = [parse(t) for t in call["tags2"]]
    sched = compileSparseSchedule(rules, t1, t2)
    got = [[i, j, repr(sched.result_tags[k])] for i, j, k, _ in sched.entries]
    assert got == call["entries"]
    assert [repr(t) for t in sched.result_tags] == call["result"]


@pytest.mark.parametrize("name", ["ti", "heis", "ising_ud"])
def test_schedules_bit_exact(tables, name):
    for rec in tables[name]["records"]:
        for k, c in enumerate(rec["stage_calls"]):
            _check(c, tsp.RULES["stage2" if k in (2, 5) else "stage1"]())
        a = rec["absorb_calls"]
        _check(a[0], tsp.RULES["absL"]())
        _check(a[1], tsp._center_rules(rec["direction"]))
        _check(a[2], tsp.RULES["absR"]())
        s3 = rec["stage3"]
        terms = tsp.stage3TermTable([parse(t) for t in s3["s2_0"]], [parse(t) for t in s3["s2_1"]],
                                    [parse(t) for t in s3["op"]])
        assert [[a_, b_, c_, int(e_)] for a_, b_, c_, e_ in terms] == s3["terms"]


def _declared_functions():
    names = []
    with open(os.path.join(ROOT, "include", "carcassonne_gb300.h")) as f:
        src = f.read()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(carc_\w+)\s*\(", src, re.M):
        names.append(m.group(1))
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _declared_functions()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name
    assert lib.carc_version() >= 100


def test_error_path_without_gpu_work():
    # a descriptor with a bad extent is rejected on the host, before any launch
    import ctypes
    d = _lib.ContractDesc()
    d.nm = 1
    d.m_ext[0] = 0
    assert _lib.load().carc_zcontract_workspace_size(ctypes.byref(d), 1) < 0


def _ru(a, b):
    return -(-a // b) * b


def _pow2_rows(n):
    """Vin rows: one power-of-two N tile up to 256, whole 256-row tiles above."""
    if n > 256:
        return _ru(n, 256)
    t = 16
    while t < n:
        t *= 2
    return t


def _equal_tile_rows(n):
    """W rows: ceil(n / 256) equal N tiles of a multiple of 16."""
    nt = -(-n // 256)
    return nt * _ru(-(-n // nt), 16)


def _tile_n(n):
    nt = -(-n // 256)
    if n % nt == 0 and (n // nt) % 16 == 0:
        return n // nt
    return next(b for b in (256, 128, 64, 32, 16) if n % b == 0)


def _effective_ksplit(k, ks):
    kb = k // 64
    ks = max(1, min(ks, kb))
    per = -(-kb // ks)
    return -(-kb // per)


# shapes outside the fused kernel's range (l0 l1 = 25, 36, 9): the two-kernel
# layout [Vin per group | W | split-K planes | reduction scratch]
@pytest.mark.parametrize("D,chi,nvec,d,group_sizes", [(5, 8, 8, 2, (2, 1, 3)), (6, 4, 8, 2, (1, 2)),
                                                      (3, 6, 3, 3, (1, 1)), (5, 3, 2, 4, (4,))])
def test_two_kernel_workspace_layout(D, chi, nvec, d, group_sizes):
    """The tensor-core matvec's workspace size (host arithmetic behind the C
    ABI, no GPU) against the layout it documents: W padded to equal N tiles
    of a multiple of 16 (400 rows -> 416, 576 -> 576), Vin to a power-of-two
    tile, split-K planes sized by the one-wave heuristic."""
    import ctypes
    L = _lib.load()
    assert L.carc_tc_autotune_clear() == 0
    s0 = (ctypes.c_int64 * 6)(chi, chi, D, D, D, D)  # x0 x1 k0 k1 l0 l1
    s1 = (ctypes.c_int64 * 6)(chi, chi, D, D, D, D)  # x1 x0 k2 k3 l2 l3
    trip = []
    for g, n in enumerate(group_sizes):
        trip += [(len(trip), g, 0) for _ in range(n)]
    terms = (ctypes.c_int32 * (3 * len(trip)))(*[v for t in trip for v in t])
    got = L.carc_stage3_matvec_tc_workspace_size(s0, s1, d, terms, len(trip), nvec)

    a256 = lambda x: _ru(x, 256)  # noqa: E731
    rows_vin = _pow2_rows(nvec * D * D * d)
    reg_a = _ru(4 * D * D, 64)
    vin = sum(a256(rows_vin * reg_a * n * 2) for n in group_sizes)
    kc_b = chi * chi * D * D
    kp_b = _ru(4 * kc_b, 64) * len(group_sizes)
    rows_w = _equal_tile_rows(nvec * D * D * d)
    rows_sb = _ru(4 * D * D, 128)
    tiles = (rows_sb // 128) * (rows_w // _tile_n(rows_w))
    ks = _effective_ksplit(kp_b, max(1, min(1 if tiles >= 152 else 152 // tiles, kp_b // 64)))
    want = a256(vin) + a256(rows_w * kp_b * 2) + a256(ks * rows_sb * rows_w * 4) + 256
    assert got == want, (got, want)
    if (D, d, nvec) == (5, 2, 8):
        assert rows_w == 416
