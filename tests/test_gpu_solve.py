"""Center-site solves: the plain FP64 solve and the mixed-precision solve
(tensor-core split-BF16 H_eff/N_eff, complex64 reduction and Lanczos, exact
FP64 H x / N x with or without the Newton correction) all reach the
reference's ground-state energy on the golden trajectories to 1e-8
relative."""
import json
import os

import numpy as np
import pytest
import torch

from tests.test_gpu_system import GOLD, _system_at, env  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu

CASES = [("ti", s) for s in range(1, 6)] + [("heis", s) for s in range(5)] + [("ising_ud", s) for s in range(0, 8, 2)]


@pytest.mark.parametrize("precision,newton", [("plain", True), ("mixed", True), ("mixed", False)])
def test_solve_center_energy(env, precision, newton):
    """newton=False: the mixed energy is the Rayleigh quotient of the
    tensor-core eigenvector with exact H x, N x (no correction step); its
    error is second order in the eigenvector's error, which grows as the
    spectral gap shrinks (3.7e-8 on heis step 4), so it is held to 1e-6
    here and the Newton-corrected solve to 1e-8."""
    from carcassonne_gb300.solve import solve_center
    with open(os.path.join(GOLD, "tables.json")) as f:
        tables = json.load(f)
    traj = np.load(os.path.join(GOLD, "trajectory.npz"))
    for name, step in CASES:
        system = _system_at(env, traj, tables[name]["records"][step], name, step)
        H, N = system.formExpectationAndNormalizationMultipliers()
        out = solve_center(H, N, precision=precision, newton=newton)
        exact = traj[f"{name}_{step}_E"][0].real
        err = abs(out["energy"] - exact) / max(1.0, abs(exact))
        assert err <= (1e-8 if newton else 1e-6), (name, step, precision, out["energy"], exact,
                                                   out["lanczos_eigenvalue"])
        # the returned center is N-normalized and its FP64 Rayleigh quotient is the energy
        x = out["center"]
        hx, nx = H(x)._t, N(x)._t
        xh = x._t.reshape(-1).conj()
        nn = torch.dot(xh, nx.reshape(-1)).real.item()
        ee = torch.dot(xh, hx.reshape(-1)).real.item() / nn
        assert abs(nn - 1.0) < 1e-8
        assert abs(ee - out["energy"]) <= 1e-10 * max(1.0, abs(exact))


@pytest.mark.parametrize("D,c", [(2, 3), (3, 2)])
def test_solve_center_hermitian_workload(env, D, c):
    """Synthetic Hermitian-definite pencils with the Heisenberg term structure:
    plain and mixed solves both land on the oracle's lowest generalized
    eigenvalue (dense scipy eigh of the oracle's H_eff, N_eff) to 1e-8."""
    import scipy.linalg as sl
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.solve import solve_center
    from carcassonne_gb300.tensors._2d import sparse as tsp
    from oracle import carc_oracle as orc
    from tests.tagrepr import parse_tag
    cc, ss, oo = workloads.hermitian_problem_arrays(D=D, c=c, seed=2)
    conv = lambda t: parse_tag(repr(t))  # noqa: E731
    H_o, N_o, _ = orc.expectation_and_normalization_multipliers(
        [{conv(t): a for t, a in lst} for lst in cc], [{conv(t): a for t, a in lst} for lst in ss],
        {conv(t): a for t, a in oo})
    exact = sl.eigh(H_o.formMatrix(), N_o.formMatrix(), eigvals_only=True)[0]
    corners, sides, op = workloads.to_device(cc, ss, oo)
    H, N = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    for precision, newton in (("plain", True), ("mixed", True), ("mixed", False)):
        out = solve_center(H, N, precision=precision, newton=newton)
        tol = 1e-8 if newton else 1e-6
        assert abs(out["energy"] - exact) <= tol * abs(exact), (precision, newton, out["energy"], exact)
