"""The tcgen05 tensor-core path: the raw BF16 GEMM against an FP32 torch
reference of the same BF16 inputs, and the split-BF16 complex contraction
against numpy complex128 (tolerance 5e-5 of the result's scale: operands are
carried with ~16 significant bits)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    return _lib


@pytest.mark.parametrize("M,N,K,ksplit", [(128, 16, 64, 1), (256, 64, 256, 1), (128, 256, 512, 3),
                                          (384, 48, 192, 2), (128, 128, 1024, 4),
                                          # N tiles that are not powers of two: 2 x 208, 3 x 192, 1 x 144
                                          (128, 416, 256, 2), (256, 576, 128, 1), (128, 144, 192, 1)])
def test_raw_bf16_gemm(lib, M, N, K, ksplit):
    L = lib.load()
    g = torch.Generator().manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    ks = ksplit
    out = torch.full((ks, M, N), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros((), dtype=torch.int32, device="cuda")
    lib.check(L.carc_gemm_bf16_tn(_vp(A), M, _vp(B), N, K, ctypes.cast(ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p), N, ks, _vp(status), _stream()))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = A.float() @ B.float().T
    got = out.sum(0)
    err = (got - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


def _desc_matrix(lib, M, N, K, a_strides, b_strides):
    d = lib.ContractDesc()
    d.nm, d.nn, d.nk = 1, 1, 1
    d.m_ext[0], d.n_ext[0], d.k_ext[0] = M, N, K
    d.a_m[0], d.a_k[0] = a_strides
    d.b_n[0], d.b_k[0] = b_strides
    d.c_m[0], d.c_n[0] = N, 1
    return d


@pytest.mark.parametrize("M,N,K,transpose_b,ksplit", [(32, 16, 16, False, 1), (100, 70, 300, True, 2),
                                                      (256, 256, 1024, False, 4), (5, 3, 7, True, 1)])
def test_split_bf16_complex_contraction(lib, M, N, K, transpose_b, ksplit):
    L = lib.load()
    rng = np.random.default_rng(M * N + K)
    a = rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))
    b = rng.standard_normal((N, K)) + 1j * rng.standard_normal((N, K))
    A = torch.as_tensor(a).cuda()
    if transpose_b:
        Bt = torch.as_tensor(np.ascontiguousarray(b.T)).cuda()  # stored (K, N)
        bstr = (1, N)
        Bp = Bt
    else:
        Bp = torch.as_tensor(b).cuda()
        bstr = (K, 1)
    d = _desc_matrix(lib, M, N, K, (K, 1), bstr)
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    ws_bytes = L.carc_zcontract_tc_workspace_size(ctypes.byref(d), ksplit)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    status = torch.zeros((), dtype=torch.int32, device="cuda")
    lib.check(L.carc_zcontract_tc(ctypes.byref(d), _vp(A), _vp(Bp), _vp(C), 1.0, 0.0, 0, ksplit, _vp(ws), ws_bytes,
                                  _vp(status), _stream()))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = a @ b.T
    err = np.abs(C.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 5e-5, err


@pytest.mark.parametrize("D,c_ket,c_bra,nvec", [(2, 2, 2, 1), (2, 4, 2, 3), (4, 8, 4, 8), (3, 3, 3, 2)])
def test_stage3_tensorcore_matches_fp64(lib, D, c_ket, c_bra, nvec):
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.tensors._2d import sparse as tsp
    corners_a, sides_a, op_a = workloads.matvec_problem_arrays(D=D, c_ket=c_ket, c_bra=c_bra, seed=D + c_ket)
    corners, sides, op = workloads.to_device(corners_a, sides_a, op_a)
    H, N = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    for m in (H, N):
        opr = m.operator if hasattr(m, "operator") else None
        if opr is None:
            continue
        rng = np.random.default_rng(nvec)
        shape = (nvec,) + opr.in_shape
        x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).cuda()
        y64 = opr.apply(x, nvec=nvec).cpu().numpy()
        ytc = opr.apply_tc(x, nvec=nvec).cpu().numpy()
        opr.check_status()
        err = np.abs(ytc - y64).max() / np.abs(y64).max()
        assert err < 5e-5, err
        if opr.n <= 1296:
            H64 = opr.form_matrix().cpu().numpy()
            Htc = opr.form_matrix_tc().cpu().numpy()
            opr.check_status()
            err = np.abs(Htc - H64).max() / np.abs(H64).max()
            assert err < 5e-5, err


# (2, 2, 2, 2) and (2, 2, 2, 6): step-A column counts 16 and 48, a partial
# 32-column chunk in the fold
@pytest.mark.parametrize("D,c_ket,c_bra,nvec", [(2, 2, 2, 8), (4, 4, 4, 2), (4, 8, 4, 8), (2, 2, 2, 2), (2, 2, 2, 6)])
def test_fused_matvec_matches_unfused_and_fp64(lib, D, c_ket, c_bra, nvec):
    """The fused step-A/step-B kernel (W kept on chip) against the two-kernel
    path (forced through the autotune cache) and the FP64 path."""
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.tensors._2d import sparse as tsp
    L = lib.load()
    corners_a, sides_a, op_a = workloads.matvec_problem_arrays(D=D, c_ket=c_ket, c_bra=c_bra, seed=7)
    corners, sides, op = workloads.to_device(corners_a, sides_a, op_a)
    H, _ = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    opr = H.operator
    rng = np.random.default_rng(3)
    shape = (nvec,) + opr.in_shape
    x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).cuda()
    y64 = opr.apply(x, nvec=nvec).cpu().numpy()
    y_fused = opr.apply_tc(x, nvec=nvec).cpu().numpy()
    opr.check_status()
    for g in opr._groups:  # force the two-kernel path for this shape
        groups = len({t[1] for t in g["terms"]})
        lib.check(L.carc_tc_autotune_set(g["s0"], g["s1"], opr.d, nvec, groups, 152))
    y_two = opr.apply_tc(x, nvec=nvec).cpu().numpy()
    opr.check_status()
    lib.check(L.carc_tc_autotune_clear())
    scale = np.abs(y64).max()
    assert np.abs(y_fused - y64).max() / scale < 5e-5
    assert np.abs(y_two - y64).max() / scale < 5e-5
    assert np.abs(y_fused - y_two).max() / scale < 2e-5


def _random_site_operators(d, seed):
    """The transverse-Ising tag set with random Hermitian d x d site matrices
    (the identity tag keeps the identity)."""
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


# D = 5, 6: W has 400 / 576 rows, tiled 2 x 208 / 3 x 192 by step B; d = 1,
# 3, 4, 8: the folding epilogue's staged column order (p-major for 2, 4, 8,
# column order otherwise)
@pytest.mark.parametrize("D,c_ket,c_bra,nvec,d", [(5, 2, 2, 8, 2), (6, 2, 1, 8, 2), (3, 2, 2, 2, 4),
                                                  (3, 2, 2, 3, 1), (3, 2, 1, 2, 3), (2, 2, 2, 4, 8)])
def test_two_kernel_matvec_shapes(lib, D, c_ket, c_bra, nvec, d):
    """The two-kernel tensor-core path (step A with the folding epilogue, W
    through HBM, split-K step B), forced through the autotune cache, against
    the FP64 path."""
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.tensors._2d import sparse as tsp
    L = lib.load()
    ops = _random_site_operators(d, seed=D + d)
    corners_a, sides_a, op_a = workloads.matvec_problem_arrays(D=D, c_ket=c_ket, c_bra=c_bra, seed=11,
                                                               op_arrays=ops)
    corners, sides, op = workloads.to_device(corners_a, sides_a, op_a)
    H, _ = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    opr = H.operator
    assert opr.d == d
    rng = np.random.default_rng(5)
    shape = (nvec,) + opr.in_shape
    x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).cuda()
    y64 = opr.apply(x, nvec=nvec).cpu().numpy()
    try:
        for g in opr._groups:
            groups = len({t[1] for t in g["terms"]})
            lib.check(L.carc_tc_autotune_set(g["s0"], g["s1"], opr.d, nvec, groups, 152))
        y_two = opr.apply_tc(x, nvec=nvec).cpu().numpy()
        opr.check_status()
    finally:
        lib.check(L.carc_tc_autotune_clear())
    assert np.abs(y_two - y64).max() / np.abs(y64).max() < 5e-5
