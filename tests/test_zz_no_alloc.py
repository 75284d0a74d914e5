"""The allocation-free stage-3 matvec against the workspace-taking one.

carc_stage3_matvec_f64_noalloc serves callers that may not allocate device
memory while they run (a host that owns the whole GPU, or a loop that cannot
afford the synchronisation an allocation may cause); it takes its scratch from
a fixed array inside the library.  Both entry points are called through the C
ABI with ctypes on the same inputs; two calls in a row check that the shared
scratch left by one call does not leak into the next.  The output is also
checked against the reference's own H v (golden vectors recorded from
formDenseStage3 / formNormalizationStage3, tensors/_2d/dense.py:114-174), the
accumulate path against the workspace entry point, and the device memory in
use is checked to stay the same across calls.  This file is collected last so
that a failure here does not hide any other test.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
LIMIT = 16 << 20  # CARC_NOALLOC_SCRATCH_BYTES


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


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


class _Args:
    """ctypes argument arrays of one problem (kept alive with the object)."""

    def __init__(self, s0_shape, s1_shape, s0, s1, ops, terms):
        from carcassonne_gb300 import _lib
        self.p0, self._k0 = _lib.ptr_array([t.data_ptr() for t in s0])
        self.p1, self._k1 = _lib.ptr_array([t.data_ptr() for t in s1])
        self.po, self._ko = _lib.ptr_array([t.data_ptr() for t in ops] or [0])
        self.pt, self._kt = _lib.i32_array([v for t in terms for v in t])
        self.sh0, self._ks0 = _lib.i64_array(s0_shape)
        self.sh1, self._ks1 = _lib.i64_array(s1_shape)
        self.n0, self.n1, self.nop, self.nt = len(s0), len(s1), len(ops), len(terms)


def _call_ws(lib, a, d, x, y, nvec, acc, ws):
    from carcassonne_gb300 import _lib
    _lib.check(lib.carc_stage3_matvec_f64(a.sh0, a.sh1, d, a.p0, a.n0, a.p1, a.n1, a.po, a.nop, a.pt, a.nt,
                                          _vp(x), _vp(y), nvec, acc, _vp(ws), ws.numel(), _stream()))


def _call_noalloc(lib, a, d, x, y, nvec, acc):
    return lib.carc_stage3_matvec_f64_noalloc(a.sh0, a.sh1, d, a.p0, a.n0, a.p1, a.n1, a.po, a.nop, a.pt, a.nt,
                                              _vp(x), _vp(y), nvec, acc, _stream())


def _lib_or_skip():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    torch.cuda.set_device(0)
    return _lib, _lib.load()


def test_noalloc_matches_workspace_entry_point_twice():
    _lib, lib = _lib_or_skip()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(2024)
    s0_shape, s1_shape, d, s0, s1, ops, terms = _problem(rng, dev)
    a = _Args(s0_shape, s1_shape, s0, s1, ops, terms)
    nvec = 2
    in_shape = (nvec, s0_shape[2], s0_shape[3], s1_shape[2], s1_shape[3], d)
    out_shape = (nvec, s0_shape[4], s0_shape[5], s1_shape[4], s1_shape[5], d)
    ws_bytes = lib.carc_stage3_matvec_f64_workspace_size(a.sh0, a.sh1, d, a.nt, nvec)
    assert 0 < ws_bytes <= LIMIT
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    # two plain calls, then one that accumulates into a non-zero y
    for call, acc in ((0, 0), (1, 0), (2, 1)):
        x = torch.as_tensor(rng.standard_normal(in_shape) + 1j * rng.standard_normal(in_shape)).to(dev)
        if acc:
            y0 = torch.as_tensor(rng.standard_normal(out_shape) + 1j * rng.standard_normal(out_shape)).to(dev)
            y_ref, y_new = y0.clone(), y0.clone()
        else:
            y_ref = torch.empty(out_shape, dtype=torch.complex128, device=dev)
            y_new = torch.full(out_shape, float("nan"), dtype=torch.complex128, device=dev)
        _call_ws(lib, a, d, x, y_ref, nvec, acc, ws)
        _lib.check(_call_noalloc(lib, a, d, x, y_new, nvec, acc))
        torch.cuda.synchronize()
        got, want = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.isfinite(got).all(), call
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err <= 1e-12, (call, err)


def test_noalloc_matches_reference_golden_vectors():
    """H v and N v of the reference's single-term stage-3 multipliers."""
    _lib, lib = _lib_or_skip()
    dev = torch.device("cuda", 0)
    g = np.load(os.path.join(HERE, "golden", "dense.npz"))
    for case in range(4):
        s20, s21, op, v = (torch.as_tensor(g[f"stage3_{case}_{k}"]).to(dev) for k in ("s20", "s21", "op", "v"))
        d = op.shape[0]
        for io, key in ((0, "Hv"), (-1, "Nv")):
            a = _Args(tuple(s20.shape), tuple(s21.shape), [s20], [s21], [op] if io >= 0 else [], [(0, 0, io)])
            want = g[f"stage3_{case}_{key}"]
            for call in range(2):
                y = torch.full(want.shape, float("nan"), dtype=torch.complex128, device=dev)
                _lib.check(_call_noalloc(lib, a, d, v.contiguous(), y, 1, 0))
                torch.cuda.synchronize()
                got = y.cpu().numpy()
                err = np.abs(got - want).max() / np.abs(want).max()
                assert err <= 1e-12, (case, key, call, err)


def test_noalloc_allocates_no_device_memory():
    _lib, lib = _lib_or_skip()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(7)
    s0_shape, s1_shape, d, s0, s1, ops, terms = _problem(rng, dev)
    a = _Args(s0_shape, s1_shape, s0, s1, ops, terms)
    nvec = 3
    in_shape = (nvec, s0_shape[2], s0_shape[3], s1_shape[2], s1_shape[3], d)
    out_shape = (nvec, s0_shape[4], s0_shape[5], s1_shape[4], s1_shape[5], d)
    x = torch.as_tensor(rng.standard_normal(in_shape) + 1j * rng.standard_normal(in_shape)).to(dev)
    y = torch.empty(out_shape, dtype=torch.complex128, device=dev)
    # the first call looks the array's address up and loads the kernels
    _lib.check(_call_noalloc(lib, a, d, x, y, nvec, 0))
    torch.cuda.synchronize()
    torch_before = torch.cuda.memory_allocated(dev)
    free_before = torch.cuda.mem_get_info(dev)[0]
    for acc in (0, 1, 0):
        _lib.check(_call_noalloc(lib, a, d, x, y, nvec, acc))
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated(dev) == torch_before
    assert torch.cuda.mem_get_info(dev)[0] == free_before


def test_noalloc_rejects_oversized_problem():
    _lib, lib = _lib_or_skip()
    dev = torch.device("cuda", 0)
    # a shape whose scratch exceeds the fixed array; rejected before any launch
    s0_shape, s1_shape = (64, 64, 4, 4, 4, 4), (64, 64, 4, 4, 4, 4)
    sh0, ks0 = _lib.i64_array(s0_shape)
    sh1, ks1 = _lib.i64_array(s1_shape)
    assert lib.carc_stage3_matvec_f64_workspace_size(sh0, sh1, 2, 1, 8) > LIMIT
    dummy = torch.empty(1, dtype=torch.complex128, device=dev)
    p, k = _lib.ptr_array([dummy.data_ptr()])
    pt, kt = _lib.i32_array([0, 0, -1])
    st = lib.carc_stage3_matvec_f64_noalloc(sh0, sh1, 2, p, 1, p, 1, p, 0, pt, 1, _vp(dummy), _vp(dummy), 8, 0,
                                            _stream())
    assert st == _lib.CARC_TOO_LARGE
    assert b"fixed" in lib.carc_last_error_string()


def test_noalloc_limit_boundary():
    """The largest block of vectors that fits the array runs and matches the
    workspace entry point; one more vector is rejected."""
    _lib, lib = _lib_or_skip()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(11)
    x0, x1, k, l, d = 8, 8, 3, 3, 2
    s0_shape, s1_shape = (x0, x1, k, k, l, l), (x1, x0, k, k, l, l)
    sh0, ks0 = _lib.i64_array(s0_shape)
    sh1, ks1 = _lib.i64_array(s1_shape)
    size = lambda nv: lib.carc_stage3_matvec_f64_workspace_size(sh0, sh1, d, 1, nv)
    nvec = 1
    while size(nvec + 1) <= LIMIT:
        nvec += 1
    assert size(nvec) <= LIMIT < size(nvec + 1)
    cplx = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s)).to(dev)
    s0, s1, op = cplx(*s0_shape), cplx(*s1_shape), cplx(d, d)
    a = _Args(s0_shape, s1_shape, [s0], [s1], [op], [(0, 0, 0)])
    for nv, ok in ((nvec, True), (nvec + 1, False)):
        x = cplx(nv, k, k, k, k, d)
        y = torch.full((nv, l, l, l, l, d), float("nan"), dtype=torch.complex128, device=dev)
        st = _call_noalloc(lib, a, d, x, y, nv, 0)
        if not ok:
            assert st == _lib.CARC_TOO_LARGE
            continue
        _lib.check(st)
        ws = torch.empty(size(nv), dtype=torch.uint8, device=dev)
        y_ref = torch.empty_like(y)
        _call_ws(lib, a, d, x, y_ref, nv, 0, ws)
        torch.cuda.synchronize()
        got, want = y.cpu().numpy(), y_ref.cpu().numpy()
        assert np.abs(got - want).max() / np.abs(want).max() <= 1e-12
