"""Parity at the benchmark's configured sizes, against the reference's own outputs.

Fixtures (tests/golden/configs.npz, written by ``make_golden.py configs`` from
the reference run on the same seeded inputs):

* the matvec microbenchmark's operator (transverse Ising after one absorption
  round, 9 terms, D=4, chi=32 = 8x4, seed 1): H v and N v for a block of 8
  centers, columns and diagonal of the dense H_eff / N_eff
  (formDenseStage3 / formNormalizationStage3 multiply and formMatrix,
  tensors/_2d/dense.py:114-225), and the CostTracker counts;
* the same shapes with the Heisenberg operator and complex boundaries
  (20 terms, complex S2 tensors through the tensor-core path);
* the center solve pencil (Heisenberg, D=4, chi=64 = 8x8, Hermitian-definite,
  seed 2): the lowest generalized eigenpair of the reference's dense H_eff,
  N_eff (minimizeExpectationUsingFullEigensolver, system/_2d.py:498-502);
* two growth runs: transverse Ising h=3 (D=2, per-layer boundary dimension
  compressed to 8, i.e. chi=64, 20 absorptions, seed 0) and Heisenberg (D=4,
  compressed to 8, the first 8 absorptions, seed 2): per step the reference's
  lowest generalized eigenvalue, the seeded random unit center absorbed
  (workloads.growth_center), and the compressor matrices
  computeProductCompressor returned (compression.py:26-46) with the seed of
  their random start.

The growth runs are replayed step by step on the same environments: the GPU
solves each step's center problem (plain FP64 to 1e-10, the mixed-precision
solve to 1e-8 relative of the reference's energy), absorbs the same center
(contractTowards, system/_2d.py:435-439) and applies the reference's
compressor (compressCornerStateTowards, system/_2d.py:191-228); the GPU's own
compressor is run on the same inputs from the same random start and must fit
the boundary product at least as well as the reference's, in FP64 and with
its big contractions on the tensor cores.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

TC_TOL = 5e-5  # split-BF16 operands (about 16 significant bits), FP32 accumulation, FP64 reductions
FP64_TOL = 1e-12
PLAIN_E_TOL = 1e-10
MIXED_E_TOL = 1e-8


@pytest.fixture(scope="module")
def gold():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return dict(np.load(os.path.join(GOLD, "configs.npz")))


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _multipliers(corners, sides, op):
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.tensors._2d import sparse as tsp
    c, s, o = workloads.to_device(corners, sides, op)
    return tsp.formExpectationAndNormalizationMultipliers(c, s, o)


def _check_fp64_multiply(gold, key, H, N):
    from carcassonne_gb300.data import TorchData
    x = gold[key + "_x"]
    for i in range(x.shape[0]):
        assert rel(H(TorchData(x[i])).toArray(), gold[key + "_Hx"][i]) < FP64_TOL
        assert rel(N(TorchData(x[i])).toArray(), gold[key + "_Nx"][i]) < FP64_TOL


def _check_operator(gold, key, corners, sides, op):
    H, N = _multipliers(corners, sides, op)
    x = gold[key + "_x"]
    cost = gold[key + "_cost"]
    assert (H.cost_of_multiply, H.cost_of_formMatrix, N.cost_of_multiply) == tuple(int(v) for v in cost)
    # FP64: one center at a time through the Multiplier, and the dense matrices
    _check_fp64_multiply(gold, key, H, N)
    Hm, Nm = H.formMatrix().toArray(), N.formMatrix().toArray()
    assert rel(Hm[:, :8], gold[key + "_H_cols"]) < FP64_TOL
    assert rel(np.diag(Hm), gold[key + "_H_diag"]) < FP64_TOL
    assert rel(Nm[:, :8], gold[key + "_N_cols"]) < FP64_TOL
    assert abs(np.linalg.norm(Hm) / gold[key + "_H_fro"][0] - 1) < FP64_TOL
    assert abs(np.linalg.norm(Nm) / gold[key + "_H_fro"][1] - 1) < FP64_TOL
    # tensor cores: the whole block in one application, and the dense H_eff
    xb = torch.as_tensor(x).cuda()
    yb = H.operator.apply_tc(xb, nvec=x.shape[0]).cpu().numpy()
    H.operator.check_status()
    assert rel(yb, gold[key + "_Hx"]) < TC_TOL
    nb = N.operator.apply_tc(xb, nvec=x.shape[0]).cpu().numpy()
    N.operator.check_status()
    assert rel(nb, gold[key + "_Nx"]) < TC_TOL
    Ht = H.operator.form_matrix_tc().cpu().numpy()
    assert rel(Ht[:, :8], gold[key + "_H_cols"]) < TC_TOL
    assert rel(np.diag(Ht), gold[key + "_H_diag"]) < TC_TOL


def test_matvec_config_operator(gold):
    from carcassonne_gb300 import workloads
    c, s, o = workloads.matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=1)
    _check_operator(gold, "mv", c, s, o)


def test_matvec_config_shapes_complex_heisenberg(gold):
    from carcassonne_gb300 import workloads
    c, s, o = workloads.matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=4,
                                              op_arrays=workloads.heisenberg_operator_arrays(), complex_=True)
    _check_operator(gold, "mvz", c, s, o)


@pytest.mark.parametrize("precision,tol", [("plain", PLAIN_E_TOL), ("mixed", MIXED_E_TOL)])
def test_solve_pencil_energy(gold, precision, tol):
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.solve import solve_center
    c, s, o = workloads.hermitian_problem_arrays(D=4, c=8, seed=2)
    H, N = _multipliers(c, s, o)
    _check_fp64_multiply(gold, "pencil", H, N)
    out = solve_center(H, N, precision=precision)
    e_ref = gold["pencil_E"][0]
    assert abs(out["energy"] - e_ref) <= tol * abs(e_ref), (out["energy"], e_ref)
    # the eigenvector, up to its phase, in the N-norm
    v = out["center"].toArray().ravel()
    vr = gold["pencil_v"]
    Nm = N.formMatrix().toArray()
    ov = abs(np.vdot(vr, Nm @ v)) / np.sqrt(abs(np.vdot(vr, Nm @ vr)) * abs(np.vdot(v, Nm @ v)))
    assert 1 - ov < (1e-9 if precision == "plain" else 1e-7), 1 - ov


# -- growth runs ---------------------------------------------------------------
GROWTH = {
    # name: (operator, D, seed, steps, new_dimension)
    "ti20": ("ti", 2, 0, 20, 8),
    "heis8": ("heis", 4, 2, 8, 8),
}


def _fit_residual(Lt, Rt, P):
    """|| L P-compressed . R P-compressed - L . R || / || L . R || with P (new, old)
    applied as compressCornerStateTowards does (ket by P, bra by conj P)."""
    exact = np.tensordot(Lt, Rt, ((1, 2, 3), (0, 1, 2)))
    Lc = np.einsum("na,mb,labo->lnmo", P, P.conj(), Lt, optimize=True)
    Rc = np.einsum("nc,me,ceor->nmor", P.conj(), P, Rt, optimize=True)
    approx = np.tensordot(Lc, Rc, ((1, 2, 3), (0, 1, 2)))
    return float(np.linalg.norm(approx - exact) / np.linalg.norm(exact))


@pytest.mark.parametrize("name", sorted(GROWTH))
@pytest.mark.parametrize("solver,tol", [("lanczos", PLAIN_E_TOL), ("mixed", MIXED_E_TOL)])
def test_growth_run_replay(gold, name, solver, tol, monkeypatch):
    from carcassonne_gb300 import compression, workloads
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.sparse import Identity
    import carcassonne_gb300.system._2d as sys2d
    kind, D, seed, steps, new_dim = GROWTH[name]
    system = workloads.bond_start_system(kind, D, seed)
    system.solver = solver
    E = gold[f"{name}_E"]
    comps = [tuple(int(v) for v in c) for c in gold[f"{name}_comps"]]
    queue = [(c, gold[f"{name}_P{i}"]) for i, c in enumerate(comps)]
    fits = []

    def replay_compressor(Ld, Rd, nd):
        (step, corner, cdir, cseed), P = queue.pop(0)
        assert P.shape == (nd, Ld.shape[1])
        np.random.seed(cseed)
        ours = compression.computeProductCompressor(Ld, Rd, nd).toArray()
        np.random.seed(cseed)
        with compression.compression_precision("tc"):
            ours_tc = compression.computeProductCompressor(Ld, Rd, nd).toArray()
        Lt, Rt = Ld.toArray(), Rd.toArray()
        fits.append((_fit_residual(Lt, Rt, ours), _fit_residual(Lt, Rt, P), _fit_residual(Lt, Rt, ours_tc)))
        return TorchData(P)

    monkeypatch.setattr(sys2d, "computeProductCompressor", replay_compressor)
    worst = 0.0
    for step in range(steps):
        e_ref = E[step, 0]
        system.minimizeExpectation()
        lam = system.last_solve["eigenvalue"]
        # a step whose effective Hamiltonian has no terms (a Heisenberg center's
        # first) has E = 0 exactly: compared absolutely
        err = abs(lam - e_ref) / abs(e_ref) if e_ref != 0 else abs(lam)
        worst = max(worst, err)
        assert err <= tol, (name, solver, step, lam, e_ref, err)
        absorbed = gold[f"{name}_{step}_absorbed"]
        # the fixture's center is the seeded one (up to the last bit of the norm,
        # which numpy may round differently on another machine)
        seed_c = workloads.GROWTH_CENTER_SEED[kind] + step
        assert np.abs(absorbed - workloads.growth_center(absorbed.shape, seed_c)).max() < 1e-15
        system.setStateCenter(TorchData(absorbed))
        system.contractTowards(step % 4)
        for corner in range(4):
            for cdir, axis in ((0, 0), (1, 3)):
                if system.corners[corner][Identity()].shape[axis] > new_dim:
                    assert queue and queue[0][0][:3] == (step, corner, cdir), (step, corner, cdir, queue[:1])
                    system.compressCornerStateTowards(corner, cdir, new_dim)
    assert not queue
    # the GPU's compressor fits each boundary product at least as well as the
    # reference's (both start from the same random isometry; the reference
    # solves the normal equations by GMRES to 1e-5, the GPU by CG to 1e-12),
    # also with the normal equations' big contractions on the tensor cores
    # (split-BF16, ~1e-5 relative: the size of the reference's GMRES tolerance)
    for ours, ref, ours_tc in fits:
        assert ours <= ref * 1.05 + 1e-10, fits
        assert ours_tc <= ref * 1.05 + 1e-8, fits
    print(name, solver, "worst relative energy error %.2e over %d steps, %d compressions" % (worst, steps, len(fits)))
