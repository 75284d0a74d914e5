"""Pin the CPU oracle at the benchmark's configured sizes (CPU only).

tests/golden/configs.npz holds the reference's own outputs (make_golden.py
configs): H v / N v of the matvec microbenchmark's operator (D=4, chi=32 =
8x4, 9 terms, seed 1) and the transverse-Ising growth run (h=3, D=2,
boundaries compressed to 8 per layer, 20 absorptions, seed 0): per step the
lowest generalized eigenvalue of the reference's dense H_eff / N_eff, the
seeded center it absorbed and the compressor matrices it applied.  The oracle
replays the run with the same centers and compressors and must reach the
same energies.
"""
import os

import numpy as np
import pytest

from oracle import carc_oracle as orc
from tests.tagrepr import parse_tag

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(GOLD, "configs.npz")))


def _oracle_problem(corners, sides, op):
    oc = [{parse_tag(repr(t)): a for t, a in lst} for lst in corners]
    osd = [{parse_tag(repr(t)): a for t, a in lst} for lst in sides]
    oo = {parse_tag(repr(t)): a for t, a in op}
    return oc, osd, oo


def test_matvec_config_operator_oracle(gold):
    from carcassonne_gb300 import workloads
    c, s, o = workloads.matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=1)
    H, N, _ = orc.expectation_and_normalization_multipliers(*_oracle_problem(c, s, o))
    x = gold["mv_x"]
    for i in range(2):
        for mult, key in ((H, "mv_Hx"), (N, "mv_Nx")):
            want = gold[key][i]
            assert np.abs(mult(x[i]) - want).max() <= 1e-12 * np.abs(want).max()


def test_ti_growth_run_oracle(gold):
    from carcassonne_gb300 import workloads
    c, s, st = workloads.bond_start_arrays(2, 2, 0)
    X, Z = orc.PAULI_X, orc.PAULI_Z
    op = orc.make_sparse_operator(Os=[-3.0 * Z], OO_UDs=[(X, -1.0 * X)], OO_LRs=[(X, -1.0 * X)])
    osys = orc.OracleSystem([{orc.I_TAG: a} for a in c], [{orc.I_TAG: a} for a in s], st, op)
    E = gold["ti20_E"]
    comps = [tuple(int(v) for v in r) for r in gold["ti20_comps"]]
    k = 0
    for step in range(E.shape[0]):
        H, N, _ = osys.multipliers()
        w, _ = orc.lowest_generalized(H.formMatrix(), N.formMatrix())
        assert abs(w - E[step, 0]) <= 1e-10 * abs(E[step, 0]), (step, w, E[step, 0])
        osys.state = gold[f"ti20_{step}_absorbed"]
        osys.contract_towards(step % 4)
        while k < len(comps) and comps[k][0] == step:
            _, corner, cdir, _ = comps[k]
            osys.compress_corner_state_towards(corner, cdir, 8, None, P=gold[f"ti20_P{k}"])
            k += 1
    assert k == len(comps)
