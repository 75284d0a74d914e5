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
