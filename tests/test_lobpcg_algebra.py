"""The batched block eigensolver's algebra (csrc/lobpcg.cu) restated in numpy.

Each step mirrors one kernel: the block inner products, the orthonormalising
coefficients of R and P (Gram B - A^H A, unit-diagonal scaling, eigen-drop),
the scaled Rayleigh-Ritz reduction with dropped directions raised above the
spectrum, and the block update with the residual norms.  On random
Hermitian-definite pencils the iteration reaches the lowest generalized
eigenvalue (scipy.linalg.eigh), also when every matvec carries a relative
perturbation of the size of the split-BF16 tensor-core rounding, and it does
not fall below the true eigenvalue.
"""
import numpy as np
import pytest
import scipy.linalg


def _herm(a):
    return 0.5 * (a + a.conj().T)


def _eig_drop(G, drop):
    """Mirror of rr_scale + Jacobi + the keep rule: (d, V, s)."""
    dg = np.real(np.diag(G))
    d = np.where(dg > 0, 1.0 / np.sqrt(np.where(dg > 0, dg, 1.0)), 0.0)
    Gs = d[:, None] * _herm(G) * d[None, :]
    w, V = np.linalg.eigh(Gs)
    keep = (w > drop * max(w.max(), 0.0)) & (w > 0)
    s = np.where(keep, 1.0 / np.sqrt(np.where(keep, w, 1.0)), 0.0)
    return d, V, s


def lobpcg(H, N, m, rng, tol=1e-4, max_iter=200, drop=1e-8, floor=1e-10, noise=0.0, refresh=20):
    n = H.shape[0]

    def mv(A, Z):  # columns of Z; a relative perturbation per product like the split-BF16 rounding
        Y = A @ Z
        if noise:
            Y = Y + noise * np.linalg.norm(A, 2) * np.linalg.norm(Z, axis=0) * (
                rng.standard_normal(Y.shape) + 1j * rng.standard_normal(Y.shape)) / np.sqrt(2 * n)
        return Y

    k = 3 * m
    S = np.zeros((n, k), complex)
    S[:, :m] = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    HS, NS = np.zeros_like(S), np.zeros_like(S)
    HS[:, :m], NS[:, :m] = mv(H, S[:, :m]), mv(N, S[:, :m])
    theta = None
    for it in range(max_iter):
        if refresh and it > 0 and it % refresh == 0:
            # fresh images of X, P restarted from zero (refresh)
            HS[:, :m], NS[:, :m] = mv(H, S[:, :m]), mv(N, S[:, :m])
            S[:, 2 * m:] = HS[:, 2 * m:] = NS[:, 2 * m:] = 0
        if it > 0:
            # orthonormalise R and P against X (orth_prepare / orth_finish / orth_apply)
            NS[:, m:2 * m] = mv(N, S[:, m:2 * m])
            Q = S.conj().T @ NS[:, m:3 * m]
            Ms = []
            for z in range(2):
                A = Q[:m, z * m:(z + 1) * m]
                Bz = Q[(z + 1) * m:(z + 2) * m, z * m:(z + 1) * m]
                Bp = Bz - A.conj().T @ A
                r0, r = np.real(np.diag(Bz)), np.real(np.diag(Bp))
                d = np.where((r0 > 0) & (r > floor * r0), 1.0 / np.sqrt(np.abs(r) + (r <= 0)), 0.0)
                w, V = np.linalg.eigh(d[:, None] * _herm(Bp) * d[None, :])
                keep = (w > drop * max(w.max(), 0.0)) & (w > 0)
                s = np.where(keep, 1.0 / np.sqrt(np.where(keep, w, 1.0)), 0.0)
                M1 = d[:, None] * V * s[None, :]
                Ms.append((M1, -A @ M1))
            X = S[:, :m].copy()
            S[:, m:2 * m] = S[:, m:2 * m] @ Ms[0][0] + X @ Ms[0][1]
            for pool in (S, HS, NS):
                pool[:, 2 * m:] = pool[:, 2 * m:] @ Ms[1][0] + pool[:, :m] @ Ms[1][1]
            HS[:, m:2 * m] = mv(H, S[:, m:2 * m])
            NS[:, m:2 * m] = mv(N, S[:, m:2 * m])
        # Rayleigh-Ritz (inner / rr_scale / rr_reduce / rr_combine)
        GH, GN = S.conj().T @ HS, S.conj().T @ NS
        d, V, s = _eig_drop(GN, drop)
        Tp = V * s[None, :]
        G = Tp.conj().T @ (d[:, None] * _herm(GH) * d[None, :]) @ Tp
        G = _herm(G)
        big = 10 * np.linalg.norm(G) + 1
        for j in np.flatnonzero(s == 0):
            G[j, j] = big
        theta, Y = np.linalg.eigh(G)
        C = (d[:, None] * Tp) @ Y[:, :m]
        # update
        S2, HS2, NS2 = np.zeros_like(S), np.zeros_like(S), np.zeros_like(S)
        for src, dst in ((S, S2), (HS, HS2), (NS, NS2)):
            dst[:, 2 * m:] = src[:, m:] @ C[m:]
            dst[:, :m] = src @ C
        S2[:, m:2 * m] = HS2[:, :m] - NS2[:, :m] * theta[None, :m]
        r = np.linalg.norm(S2[:, m]) / (np.linalg.norm(HS2[:, 0]) + abs(theta[0]) * np.linalg.norm(NS2[:, 0]))
        S, HS, NS = S2, HS2, NS2
        if r <= tol:
            return theta[0], S[:, 0], it + 1, r
    return theta[0], S[:, 0], max_iter, r


def _pencil(n, rng, cond=10.0):
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = _herm(a)
    b = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    N = b @ b.conj().T / n + np.eye(n) / cond
    return H, N


@pytest.mark.parametrize("n,m,seed", [(32, 8, 0), (162, 8, 1), (200, 4, 2), (64, 2, 3), (40, 1, 4)])
def test_lobpcg_reaches_lowest_generalized_eigenvalue(n, m, seed):
    rng = np.random.default_rng(seed)
    H, N = _pencil(n, rng)
    e_ref = scipy.linalg.eigh(H, N, eigvals_only=True)[0]
    e, x, iters, r = lobpcg(H, N, m, rng, tol=1e-8, max_iter=400)
    assert r <= 1e-8, (iters, r)
    assert abs(e - e_ref) <= 1e-9 * abs(e_ref), (e, e_ref)
    # the returned vector is N-normalised
    assert abs(np.vdot(x, N @ x) - 1) < 1e-6


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_lobpcg_under_split_precision_sized_noise(seed):
    """Matvecs perturbed by 1e-5 of |A| |z| (the tensor-core rounding): with
    X's images recomputed and P restarted every 20 iterations the iteration
    reaches a residual of 1e-4 and a Ritz value within 1e-4 of the true one."""
    rng = np.random.default_rng(100 + seed)
    H, N = _pencil(300, rng)
    e_ref = scipy.linalg.eigh(H, N, eigvals_only=True)[0]
    e, x, iters, r = lobpcg(H, N, 8, rng, tol=1e-4, max_iter=300, noise=1e-5)
    assert r <= 1e-4, (iters, r)
    assert abs(e - e_ref) <= 1e-4 * abs(e_ref), (e, e_ref)


def test_lobpcg_without_refresh_drifts_below_the_eigenvalue():
    """The failure the refresh prevents: without it the implicitly updated
    images of X and P drift under the same noise and the Ritz value falls
    well below the true lowest eigenvalue."""
    rng = np.random.default_rng(101)
    H, N = _pencil(300, rng)
    e_ref = scipy.linalg.eigh(H, N, eigvals_only=True)[0]
    e, x, iters, r = lobpcg(H, N, 8, rng, tol=1e-4, max_iter=200, noise=1e-5, refresh=0)
    assert e < e_ref - 1e-2 * abs(e_ref), (e, e_ref)
