"""The compact-operand fused matvec kernel against the first fused kernel and FP64.

The compact kernel is the default tensor-core path where it takes the shape;
the autotune cache selects the first fused kernel (entry -1) or forces the
compact one (entry -2) for the same shape.  Every case compares both with the
FP64 path (formDenseStage3 multiply, tensors/_2d/dense.py:145-174) to the
split-BF16 tolerance 5e-5 of the result's scale, including the accumulate
path and complex operators.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TC_TOL = 5e-5


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    return _lib


def _site_operators(d, seed):
    from carcassonne_gb300 import workloads
    rng = np.random.default_rng(seed)
    out = []
    for tag, _ in workloads.ti_operator_arrays():
        if type(tag).__name__ == "Identity":
            out.append((tag, np.eye(d, dtype=np.complex128)))
            continue
        a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        out.append((tag, (a + a.conj().T) / 2))
    return out


def _operator(D, c_ket, c_bra, d, complex_, seed):
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.tensors._2d import sparse as tsp
    ops = None if d == 2 and not complex_ else _site_operators(d, seed)
    c, s, o = workloads.matvec_problem_arrays(D=D, c_ket=c_ket, c_bra=c_bra, seed=seed, op_arrays=ops,
                                              complex_=complex_)
    corners, sides, op = workloads.to_device(c, s, o)
    H, _ = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    return H.operator


def _force(lib, opr, nvec, value):
    L = lib.load()
    for g in opr._groups:
        groups = len({t[1] for t in g["terms"]})
        lib.check(L.carc_tc_autotune_set(g["s0"], g["s1"], opr.d, nvec, groups, value))


# (D, c_ket, c_bra, nvec, d, complex): D = 4 at the benchmark's chi = 32 and
# at chi = 16 (one and two vector parts), D = 2 with step-A column counts 16,
# 48 (a partial 32-column chunk) and 64, site dimensions 1, 4, 8
CASES = [(4, 8, 4, 8, 2, False), (4, 8, 4, 8, 2, True), (4, 4, 4, 2, 2, True), (4, 4, 4, 4, 1, True),
         (2, 2, 2, 8, 2, False), (2, 2, 2, 2, 2, True), (2, 2, 2, 6, 2, True), (2, 4, 2, 8, 4, True),
         (2, 2, 2, 4, 8, True), (4, 4, 2, 6, 2, True)]


@pytest.mark.parametrize("D,c_ket,c_bra,nvec,d,cplx", CASES)
def test_compact_fused_matvec(lib, D, c_ket, c_bra, nvec, d, cplx):
    L = lib.load()
    opr = _operator(D, c_ket, c_bra, d, cplx, seed=10 * D + d)
    rng = np.random.default_rng(D + nvec)
    shape = (nvec,) + opr.in_shape
    x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).cuda()
    y64 = opr.apply(x, nvec=nvec).cpu().numpy()
    scale = np.abs(y64).max()
    try:
        _force(lib, opr, nvec, -2)
        y2 = opr.apply_tc(x, nvec=nvec).cpu().numpy()
        opr.check_status()
        # accumulate onto a non-zero y
        y0 = torch.as_tensor(rng.standard_normal(y64.shape) + 1j * rng.standard_normal(y64.shape)).cuda()
        yacc = y0.clone()
        opr.apply_tc(x, yacc, nvec=nvec, accumulate=True)
        opr.check_status()
        yacc = yacc.cpu().numpy()
        _force(lib, opr, nvec, -1)
        y1 = opr.apply_tc(x, nvec=nvec).cpu().numpy()
        opr.check_status()
    finally:
        lib.check(L.carc_tc_autotune_clear())
    assert np.isfinite(y2).all()
    assert np.abs(y2 - y64).max() / scale < TC_TOL
    assert np.abs(y1 - y64).max() / scale < TC_TOL
    assert np.abs(yacc - (y0.cpu().numpy() + y64)).max() / scale < TC_TOL
    # dropping the lo x lo product costs about 2^-16 relative, below the split's own error
    assert np.abs(y2 - y1).max() / scale < 2e-5


def test_compact_fused_repeated_calls_deterministic(lib):
    """Two applications of the compact kernel to the same block give the same
    bits (fixed-order reductions)."""
    opr = _operator(4, 8, 4, 2, False, seed=1)
    rng = np.random.default_rng(0)
    shape = (8,) + opr.in_shape
    x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).cuda()
    a = opr.apply_tc(x, nvec=8).cpu().numpy()
    b = opr.apply_tc(x, nvec=8).cpu().numpy()
    opr.check_status()
    assert np.array_equal(a, b)
