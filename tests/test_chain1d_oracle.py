"""The oracle's 1D-chain contractions against the reference's own outputs
(tests/golden/chain1d.npz, written by tests/golden/make_golden.py from the
reference's tensors/_1d.py)."""
import os

import numpy as np
import pytest

from oracle import carc_oracle as orc

GOLD = os.path.join(os.path.dirname(__file__), "golden", "chain1d.npz")


@pytest.mark.parametrize("case", range(4))
def test_chain_contractions_match_reference(case):
    z = np.load(GOLD)
    L, R, O, S = (z[f"c{case}_{k}"] for k in "LROS")
    L2, R2 = z[f"c{case}_L2"], z[f"c{case}_R2"]
    Sc = S.conj()
    close = lambda a, b: np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())  # noqa: E731
    assert close(orc.chain_absorb_oss_left(L, O, S, Sc), z[f"c{case}_ossL"])
    assert close(orc.chain_absorb_oss_right(R, O, S, Sc), z[f"c{case}_ossR"])
    assert close(orc.chain_absorb_ss_left(L2, S, Sc), z[f"c{case}_ssL"])
    assert close(orc.chain_absorb_ss_right(R2, S, Sc), z[f"c{case}_ssR"])
    # the multiplier takes the environments in the system's order (right, left)
    assert close(orc.chain_multiply(R, L, O, S), z[f"c{case}_y"])
    assert close(orc.chain_form_matrix(R, L, O), z[f"c{case}_M"])


@pytest.mark.parametrize("case", range(4))
def test_chain_costs_match_reference(case):
    from carcassonne_gb300.data.cost_tracker import CostTracker, computeCostOfContracting
    from carcassonne_gb300.tensors import _1d as t1
    z = np.load(GOLD)
    R, L, O = (CostTracker(z[f"c{case}_{k}"].shape) for k in "RLO")
    shape = (R.shape[1], L.shape[1], O.shape[2])
    assert computeCostOfContracting(t1._multiply, R, L, O, shape) == int(z[f"c{case}_cost"][0])
    assert computeCostOfContracting(t1._formMatrix, R, L, O) == int(z[f"c{case}_cost"][1])
