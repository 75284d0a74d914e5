"""The batched block eigensolver (blocksolve.py, csrc/lobpcg.cu) on
Hermitian-definite transverse-Ising center problems of uneven shape.

* Every problem's lowest eigenvalue agrees with the dense FP64 generalized
  eigensolve of its H_eff, N_eff (formMatrix, scipy.linalg.eigh) to the
  split-BF16 tolerance, and the returned vector's fresh residual is small.
* The batched solve and the per-problem loop give the same energies and
  iteration counts: each problem's arithmetic is independent of the batch.
* Two batched runs are bitwise identical.
"""
import numpy as np
import pytest
import scipy.linalg
import torch

pytestmark = pytest.mark.gpu

SPECS = [(2, 4, 2.5, 101), (3, 4, 3.2, 102), (2, 5, 3.9, 103), (3, 5, 2.1, 104), (2, 6, 2.8, 105)]
E_TOL = 2e-4   # split-BF16 operands, ~1e-5 relative per product; residual tolerance 1e-4


@pytest.fixture(scope="module")
def pencils():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import batched
    return [batched.build_pencil(*s) for s in SPECS]


def _dense_lowest(Hop, Nop):
    Hm = Hop.form_matrix().cpu().numpy()
    Nm = Nop.form_matrix().cpu().numpy()
    Hm, Nm = 0.5 * (Hm + Hm.conj().T), 0.5 * (Nm + Nm.conj().T)
    return scipy.linalg.eigh(Hm, Nm, eigvals_only=True)[0]


@pytest.mark.parametrize("m", [8, 4, 2, 1])
def test_batched_energies_match_dense_fp64(pencils, m):
    from carcassonne_gb300 import blocksolve
    seeds = [7 + i for i in range(len(pencils))]
    solver = blocksolve.BlockEigensolver(pencils, m)
    out = solver.solve(seeds, tol=1e-4, max_iter=400)
    assert out["converged"].all(), out
    for b, (Hop, Nop) in enumerate(pencils):
        e_ref = _dense_lowest(Hop, Nop)
        assert abs(out["energy"][b] - e_ref) <= E_TOL * abs(e_ref), (b, out["energy"][b], e_ref)
    for e, r in solver.verify():
        assert r <= 1e-3, r


def test_batched_equals_per_problem_loop(pencils):
    from carcassonne_gb300 import blocksolve
    seeds = [11 + i for i in range(len(pencils))]
    rb = blocksolve.solve_batch(pencils, seeds, m=8, tol=1e-4)
    rl = blocksolve.solve_each(pencils, seeds, m=8, tol=1e-4)
    assert np.array_equal(rb["iterations"], rl["iterations"]), (rb["iterations"], rl["iterations"])
    assert np.array_equal(rb["energy"], rl["energy"]), (rb["energy"], rl["energy"])


def test_batched_solve_is_deterministic(pencils):
    from carcassonne_gb300 import blocksolve
    seeds = [3 + i for i in range(len(pencils))]
    a = blocksolve.solve_batch(pencils, seeds, m=8)
    b = blocksolve.solve_batch(pencils, seeds, m=8)
    assert np.array_equal(a["energy"], b["energy"]) and np.array_equal(a["iterations"], b["iterations"])


def test_run_solves_small(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import batched
    out = batched.run_solves(count=6, m=4, seed=5, mem_budget=1 << 30, tune_file=str(tmp_path / "t.json"))
    assert out["problems"] == 6 and out["converged"] == 6
    assert out["batched_solves_per_s"] > 0 and out["loop_solves_per_s"] > 0
    assert out["iterations_equal_batched_vs_loop"] and out["max_energy_diff_batched_vs_loop"] == 0.0
