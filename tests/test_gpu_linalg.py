"""GPU parity of the dense linear algebra against the reference's golden
vectors and the CPU oracle."""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from oracle import carc_oracle as orc

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300 import linalg, solver, compression
    return TorchData, linalg, solver, compression


def rel(a, b):
    a = a.toArray() if hasattr(a, "toArray") else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def cn(rng, *s):
    return rng.standard_normal(s) + 1j * rng.standard_normal(s)


@pytest.mark.parametrize("shape", [(7, 3), (40, 6), (432, 6), (64, 64), (3, 9), (100, 37)])
def test_svd_reconstructs_and_matches_scipy(env, shape):
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(sum(shape))
    a = cn(rng, *shape)
    U, S, Vh = linalg.svd(TorchData(a))
    u, s, vh = U.toArray(), S.toArray().real, Vh.toArray()
    s_ref = sla.svd(a, compute_uv=False)
    assert np.abs(s - s_ref).max() <= 1e-12 * s_ref.max()
    assert np.abs((u * s) @ vh - a).max() <= 1e-12 * np.abs(a).max()
    k = min(shape)
    assert np.abs(u.conj().T @ u - np.eye(k)).max() <= 1e-12
    assert np.abs(vh @ vh.conj().T - np.eye(k)).max() <= 1e-12


def test_normalize_axis_matches_golden(env):
    TorchData, linalg, _, _ = env
    g = np.load(os.path.join(GOLD, "numerics.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in g.files if k.startswith("nax_") and k.endswith("_in")})
    assert keys
    for key in keys:
        axis = int(key.split("_")[2])
        t = TorchData(g[key + "_in"])
        iso, nz, dz = t.normalizeAxis(axis)
        assert rel(iso, g[key + "_iso"]) < 1e-11, key
        assert rel(nz, g[key + "_norm"]) < 1e-11, key
        assert rel(dz, g[key + "_denorm"]) < 1e-11, key
        a, b = t.normalizeAxis(axis, True)
        # sqrt-singular-value factors are defined up to a unitary gauge: compare a^T b and products
        ga, gb = g[key + "_sq_a"], g[key + "_sq_b"]
        assert rel(a.toArray().T @ b.toArray(), ga.T @ gb) < 1e-10, key
        assert rel(b.toArray().conj().T @ b.toArray(), gb.conj().T @ gb) < 1e-10, key


def test_unitize_and_compute_compressor(env):
    TorchData, linalg, solver, _ = env
    g = np.load(os.path.join(GOLD, "numerics.npz"))
    for case in range(3):
        assert rel(solver.unitize(TorchData(g[f"unitize_{case}_in"])), g[f"unitize_{case}_out"]) < 1e-11
    from carcassonne_gb300.utils import Multiplier
    for case in range(3):
        old, new = (int(x) for x in g[f"cc_{case}_meta"])
        gm = TorchData(g[f"cc_{case}_in"])
        c, ic = solver.computeCompressor(old, new, Multiplier((old, old), None, 0, lambda: gm, 0), None)
        ref = g[f"cc_{case}_c"]
        c = c.toArray()
        assert rel(c.conj().T @ c, ref.conj().T @ ref) < 1e-9
        cn_, icn = solver.computeCompressor(old, new, Multiplier((old, old), None, 0, lambda: gm, 0), None, True)
        assert rel(cn_.toArray().conj().T @ icn.toArray(),
                   g[f"cc_{case}_cn"].conj().T @ g[f"cc_{case}_icn"]) < 1e-9


@pytest.mark.parametrize("n", [1, 5, 32, 100, 200])
def test_hermitian_jacobi_eigh(env, n):
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(n)
    a = cn(rng, n, n)
    a = a + a.conj().T
    W, V = linalg.eigh_small(TorchData(a))
    w = W.cpu().numpy()
    assert np.abs(w - np.linalg.eigvalsh(a)).max() <= 1e-11 * np.abs(w).max()
    v = V.toArray()
    assert np.abs(a @ v - v * w).max() <= 1e-10 * np.abs(a).max()


@pytest.mark.parametrize("n,rank", [(96, 24), (162, 40)])
def test_jacobi_eigh_nearly_hermitian_rank_deficient(env, n, rank):
    """A normalization matrix near a product state: rank-deficient, tiny, and
    Hermitian only up to an anti-Hermitian residue of 1e-11 of its norm (a
    rounded X^H M X).  The eigensolver works on the Hermitian part; rotations
    driven by one triangle of the raw matrix never bring its off-diagonal
    mass down to the stopping level."""
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(n + rank)
    x = cn(rng, n, rank)
    m = (x @ x.conj().T) * 1e-15
    e = cn(rng, n, n)
    e = e - e.conj().T
    m = m + e * (1e-11 * np.linalg.norm(m) / np.linalg.norm(e))
    h = 0.5 * (m + m.conj().T)
    W, V = linalg.eigh_small(TorchData(m))
    w = W.cpu().numpy()
    ref = np.linalg.eigvalsh(h)
    assert np.abs(w - ref).max() <= 1e-12 * np.abs(ref).max()
    v = V.toArray()
    assert np.abs(h @ v - v * w).max() <= 1e-11 * np.abs(h).max()
    assert np.abs(v.conj().T @ v - np.eye(n)).max() <= 1e-12


@pytest.mark.parametrize("n,rank", [(64, 40), (200, 150)])
def test_hegv_projected_on_singular_normalization(env, n, rank):
    """N of rank < n with rounding-level negative eigenvalues: Cholesky
    rejects it, and the projected solve returns the lowest eigenpair of the
    pencil on N's range (canonical orthogonalisation restated in numpy)."""
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(n + 3 * rank)
    x = cn(rng, n, rank)
    nm = x @ x.conj().T
    e = cn(rng, n, n)
    nm = nm + 1e-14 * np.abs(nm).max() * 0.5 * (e + e.conj().T) / np.abs(e).max()
    h = cn(rng, n, n)
    h = h + h.conj().T
    with pytest.raises(np.linalg.LinAlgError):
        linalg.hegv_lowest(TorchData(h), TorchData(nm))
    lam, xv, kept = linalg.hegv_lowest_projected(TorchData(h), TorchData(nm))
    w, v = np.linalg.eigh(0.5 * (nm + nm.conj().T))
    keep = w > 1e-12 * np.abs(w).max()
    X = v[:, keep] / np.sqrt(w[keep])
    cw = np.linalg.eigvalsh(X.conj().T @ h @ X)
    ref, scale = cw[0], np.abs(cw).max()
    assert kept == int(keep.sum()) == rank
    assert abs(lam - ref) <= 1e-10 * scale
    xa = xv.toArray()
    assert abs((xa.conj() @ nm @ xa).real - 1.0) < 1e-9
    # the residual vanishes on N's range
    r = X.conj().T @ (h @ xa - lam * (nm @ xa))
    assert np.abs(r).max() <= 1e-9 * scale


@pytest.mark.parametrize("n", [1, 31, 33, 100, 512])
def test_cholesky_and_generalized_lowest(env, n):
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(3 * n + 1)
    b = cn(rng, n, n)
    N = b.conj().T @ b + n * np.eye(n)
    h = cn(rng, n, n)
    H = h + h.conj().T
    L = linalg.cholesky(TorchData(N)).toArray()
    assert np.abs(L @ L.conj().T - N).max() <= 1e-12 * np.abs(N).max()
    lam, x, iters = linalg.hegv_lowest(TorchData(H), TorchData(N))
    w_ref = sla.eigh(H, N, eigvals_only=True)[0]
    assert abs(lam - w_ref) <= 1e-10 * max(1.0, abs(w_ref)), (lam, w_ref)
    xv = x.toArray()
    assert np.abs(H @ xv - lam * (N @ xv)).max() <= 1e-8 * np.abs(H).max() * np.abs(xv).max()
    assert abs(np.vdot(xv, N @ xv) - 1) <= 1e-10


@pytest.mark.parametrize("n", [1, 33, 100, 512])
def test_generalized_lowest_single_precision(env, n):
    """CARC_HEGV_SINGLE (complex64 factorization, inverse and Lanczos on a
    tensor-core reduction) lands within the pencil's own 1e-5 of the FP64
    eigenvalue, with an N-normalized eigenvector to the same accuracy."""
    TorchData, linalg, _, _ = env
    rng = np.random.default_rng(5 * n + 2)
    b = cn(rng, n, n)
    N = b.conj().T @ b + n * np.eye(n)
    h = cn(rng, n, n)
    H = h + h.conj().T
    w_ref = sla.eigh(H, N, eigvals_only=True)
    lam, x, iters = linalg.hegv_lowest(TorchData(H), TorchData(N), tol=1e-7, tensor_core=True, single=True)
    scale = max(np.abs(w_ref).max(), 1e-300)
    assert abs(lam - w_ref[0]) <= 2e-5 * scale, (lam, w_ref[0])
    xv = x.toArray()
    assert abs(np.vdot(xv, N @ xv) - 1) <= 1e-4
    # the Rayleigh quotient of the returned vector is second-order accurate
    rq = (np.vdot(xv, H @ xv) / np.vdot(xv, N @ xv)).real
    assert abs(rq - w_ref[0]) <= 1e-6 * scale, (rq, w_ref[0])


def test_cholesky_rejects_indefinite(env):
    TorchData, linalg, _, _ = env
    a = np.diag([1.0, -1.0, 2.0]).astype(np.complex128)
    with pytest.raises(np.linalg.LinAlgError):
        linalg.cholesky(TorchData(a))


def test_relax_over_matches_oracle_and_reference(env):
    TorchData, linalg, solver, _ = env
    from carcassonne_gb300.utils import Multiplier
    g = np.load(os.path.join(GOLD, "numerics.npz"))
    for case in range(3):
        h, nm, v0 = g[f"relax_{case}_H"], g[f"relax_{case}_N"], g[f"relax_{case}_v0"]
        x = solver.relaxOver(TorchData(v0.copy()), Multiplier.fromMatrix(TorchData(h)),
                             Multiplier.fromMatrix(TorchData(nm))).toArray()
        ref = g[f"relax_{case}_x"]
        # same Krylov iteration up to the global phase of each Ritz vector
        ov = abs(np.vdot(x, ref)) / (np.linalg.norm(x) * np.linalg.norm(ref))
        assert abs(ov - 1) <= 1e-9, (case, ov)
        xo, lam, count = orc.relax_over(v0.copy(), h, nm)
        assert abs(abs(np.vdot(x, xo)) - 1) <= 1e-9


def test_product_compressor_exact_recovery(env):
    TorchData, linalg, solver, compression = env
    g = np.load(os.path.join(GOLD, "numerics.npz"))
    for case in range(2):
        Lf, Rf = g[f"pc_{case}_L"], g[f"pc_{case}_R"]
        new = g[f"pc_{case}_P"].shape[0]
        np.random.seed(5 + case)
        P = compression.computeProductCompressor(TorchData(Lf), TorchData(Rf), new).toArray()
        Lc = orc.absorb_matrix_at(orc.absorb_matrix_at(Lf, 1, P), 2, P.conj())
        Rc = orc.absorb_matrix_at(orc.absorb_matrix_at(Rf, 0, P.conj()), 1, P)
        assert rel(np.tensordot(Lc, Rc, ((1, 2, 3), (0, 1, 2))), g[f"pc_{case}_exact"]) < 1e-8
        # same seed, same starting compressor as the reference: the projector agrees too
        Pr = g[f"pc_{case}_P"]
        assert rel(P.conj().T @ P, Pr.conj().T @ Pr) < 1e-6


@pytest.mark.parametrize("n,shift", [(40, 0.3), (130, -1.7)])
def test_minres_projected(n, shift):
    """MINRES on P (C - shift) P z = P b (P = I - u u^H) against numpy: the
    residual of the projected system and z's orthogonality to u."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import linalg
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    C = (a + a.conj().T) / 2
    u = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    u /= np.linalg.norm(u)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    z, its = linalg.minres_projected(torch.as_tensor(C).cuda(), torch.as_tensor(u).cuda(), shift,
                                     torch.as_tensor(b).cuda(), maxit=4 * n, rtol=1e-10)
    z = z.cpu().numpy()
    P = np.eye(n) - np.outer(u, u.conj())
    res = P @ (C - shift * np.eye(n)) @ P @ z - P @ b
    assert np.linalg.norm(res) <= 1e-8 * np.linalg.norm(P @ b), (np.linalg.norm(res), its)
    assert abs(np.vdot(u, z)) <= 1e-10 * np.linalg.norm(z)
