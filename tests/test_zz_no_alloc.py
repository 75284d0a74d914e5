"""The allocation-free stage-3 matvec against the workspace-taking one.

carc_stage3_matvec_f64_noalloc serves callers that may not allocate device
memory while they run (a host that owns the whole GPU, or a loop that cannot
afford the synchronisation an allocation may cause); it takes its scratch from
a fixed array inside the library.  Both entry points are called through the C
ABI with ctypes on the same inputs; two calls in a row check that the shared
scratch left by one call does not leak into the next.  This file is collected
last so that a failure here does not hide any other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _problem(rng, dev):
    x0, x1, k, l, d = 6, 5, 3, 3, 2
    s0_shape = (x0, x1, k, k, l, l)
    s1_shape = (x1, x0, k, k, l, l)
    cplx = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s)).to(dev)
    s0 = [cplx(*s0_shape) for _ in range(3)]
    s1 = [cplx(*s1_shape) for _ in range(4)]
    ops = [cplx(d, d) for _ in range(2)]
    terms = [(0, 0, -1), (1, 2, 0), (2, 1, 1), (0, 3, 0), (1, 1, -1)]
    return s0_shape, s1_shape, d, s0, s1, ops, terms


def test_noalloc_matches_workspace_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(2024)
    s0_shape, s1_shape, d, s0, s1, ops, terms = _problem(rng, dev)
    p0, k0 = _lib.ptr_array([t.data_ptr() for t in s0])
    p1, k1 = _lib.ptr_array([t.data_ptr() for t in s1])
    po, ko = _lib.ptr_array([t.data_ptr() for t in ops])
    pt, kt = _lib.i32_array([v for t in terms for v in t])
    sh0, ks0 = _lib.i64_array(s0_shape)
    sh1, ks1 = _lib.i64_array(s1_shape)
    nvec = 2
    in_shape = (nvec, s0_shape[2], s0_shape[3], s1_shape[2], s1_shape[3], d)
    out_shape = (nvec, s0_shape[4], s0_shape[5], s1_shape[4], s1_shape[5], d)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws_bytes = lib.carc_stage3_matvec_f64_workspace_size(sh0, sh1, d, len(terms), nvec)
    assert 0 < ws_bytes <= (16 << 20)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    for call in range(2):
        x = torch.as_tensor(rng.standard_normal(in_shape) + 1j * rng.standard_normal(in_shape)).to(dev)
        y_ref = torch.empty(out_shape, dtype=torch.complex128, device=dev)
        y_new = torch.full(out_shape, float("nan"), dtype=torch.complex128, device=dev)
        _lib.check(lib.carc_stage3_matvec_f64(sh0, sh1, d, p0, len(s0), p1, len(s1), po, len(ops), pt, len(terms),
                                              _vp(x), _vp(y_ref), nvec, 0, _vp(ws), ws_bytes, stream))
        _lib.check(lib.carc_stage3_matvec_f64_noalloc(sh0, sh1, d, p0, len(s0), p1, len(s1), po, len(ops), pt,
                                                      len(terms), _vp(x), _vp(y_new), nvec, 0, stream))
        torch.cuda.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.isfinite(a).all(), call
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= 1e-12, (call, err)


def test_noalloc_rejects_oversized_problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    lib = _lib.load()
    # a shape whose scratch exceeds the fixed array; rejected before any launch
    s0_shape, s1_shape = (64, 64, 4, 4, 4, 4), (64, 64, 4, 4, 4, 4)
    sh0, ks0 = _lib.i64_array(s0_shape)
    sh1, ks1 = _lib.i64_array(s1_shape)
    assert lib.carc_stage3_matvec_f64_workspace_size(sh0, sh1, 2, 9, 8) > (16 << 20)
    dummy = torch.empty(1, dtype=torch.complex128, device="cuda")
    p, k = _lib.ptr_array([dummy.data_ptr()])
    pt, kt = _lib.i32_array([0, 0, -1])
    st = lib.carc_stage3_matvec_f64_noalloc(sh0, sh1, 2, p, 1, p, 1, p, 0, pt, 1, _vp(dummy), _vp(dummy), 8, 0,
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.CARC_TOO_LARGE
    assert b"fixed" in lib.carc_last_error_string()
