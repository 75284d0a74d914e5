"""Conjugate gradients for the compressor's normal equations on the device:
the cooperative-grid solver (carc_zcg_hpsd_grid) against the one-block
solver (carc_zcg_hpsd) and a direct solve, on Hermitian positive definite and
rank-deficient consistent systems of several sizes (rows that do not divide
among the CTAs included), a zero right-hand side, and two runs bitwise
equal."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import _lib
    return _lib


def _system(n, rank, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, rank)) + 1j * rng.standard_normal((n, rank))
    G = a @ a.conj().T / rank + (1e-3 * np.eye(n) if rank == n else 0)
    x_true = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return G, G @ x_true


def _run(lib, name, G, c, tol=1e-12, max_iter=None):
    n = c.shape[0]
    Gd = torch.as_tensor(G).cuda()
    cd = torch.as_tensor(c).cuda()
    x = torch.empty(n, dtype=torch.complex128, device="cuda")
    st = torch.zeros(2, dtype=torch.int32, device="cuda")
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    max_iter = max_iter or max(10 * n, 500)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if name == "grid":
        wsb = lib.load().carc_zcg_hpsd_grid_workspace_size(n)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        lib.call("carc_zcg_hpsd_grid", n, _vp(Gd), _vp(cd), _vp(x), tol, max_iter, _vp(st), _vp(res), _vp(ws), wsb,
                 stream)
    else:
        lib.call("carc_zcg_hpsd", n, _vp(Gd), _vp(cd), _vp(x), tol, max_iter, _vp(st), _vp(res), stream)
    torch.cuda.synchronize()
    return x.cpu().numpy(), st.cpu().numpy(), float(res.item())


@pytest.mark.parametrize("n,rank,seed", [(256, 256, 0), (250, 250, 1), (256, 40, 2), (3, 3, 3), (1000, 1000, 4),
                                         (2048, 300, 5)])
def test_grid_cg_solves_and_matches_one_block(lib, n, rank, seed):
    G, c = _system(n, rank, seed)
    xg, stg, rg = _run(lib, "grid", G, c)
    assert stg[0] >= 0 and stg[1] == 1 and rg <= 1e-10, (stg, rg)
    assert np.linalg.norm(G @ xg - c) <= 1e-9 * np.linalg.norm(c)
    if n <= 2048:
        xb, stb, rb = _run(lib, "block", G, c)
        assert np.linalg.norm(xg - xb) <= 1e-7 * np.linalg.norm(xb), (stg, stb)
    if rank == n:
        x_direct = np.linalg.solve(G, c)
        assert np.linalg.norm(xg - x_direct) <= 1e-7 * np.linalg.norm(x_direct)


def test_grid_cg_zero_rhs_and_determinism(lib):
    G, c = _system(300, 300, 7)
    x0, st0, r0 = _run(lib, "grid", G, np.zeros(300, complex))
    assert st0[1] == 1 and st0[0] == 0 and not x0.any() and r0 == 0.0
    a = _run(lib, "grid", G, c)
    b = _run(lib, "grid", G, c)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_grid_cg_reports_an_exhausted_budget(lib):
    G, c = _system(512, 512, 9)
    x, st, r = _run(lib, "grid", G, c, max_iter=3)
    assert st[0] == 3 and st[1] == 0 and r > 1e-10


@pytest.mark.parametrize("name", ["grid"])
def test_grid_cg_inconsistent_singular_system_stays_bounded(lib, name):
    """A rank-deficient G and a right-hand side with a part of 1e-9 outside
    its range (the rounding of formed normal equations): no x reaches the
    tolerance, and past the least-squares residual the steps along G's
    near-null directions would grow without bound.  The solver returns its
    best iterate, bounded, whose true residual is the unreachable part, and
    reports it."""
    n, rank = 256, 40
    G, c = _system(n, rank, 11)
    rng = np.random.default_rng(12)
    w, v = np.linalg.eigh(G)
    null = v[:, : n - rank] @ (rng.standard_normal(n - rank) + 1j * rng.standard_normal(n - rank))
    c_bad = c + 1e-9 * np.linalg.norm(c) * null / np.linalg.norm(null)
    x, st, r = _run(lib, name, G, c_bad)
    assert st[0] >= 0 and st[1] == 0
    true = np.linalg.norm(G @ x - c_bad) / np.linalg.norm(c_bad)
    assert abs(r - true) <= 1e-3 * true + 1e-14, (r, true)
    assert 5e-10 <= r <= 1e-8, r
    x_ls = np.linalg.pinv(G, rcond=1e-12) @ c_bad
    assert np.linalg.norm(x) <= 1e3 * np.linalg.norm(x_ls)
