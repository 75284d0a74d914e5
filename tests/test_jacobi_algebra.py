"""The Hermitian Jacobi eigensolver's iteration (heev_jacobi_kernel,
carcassonne_gb300/csrc/linalg.cu) restated in numpy, to show on the CPU why
the kernel works on the Hermitian part of its input.

The restatement follows the kernel: round-robin tournament pairs, each round's
disjoint pairs rotated together (all column updates, then all row updates),
a pair skipped when its coupling is negligible against its diagonal or
below 1e-16 of the matrix norm, and a sweep-level stop once the off-diagonal
mass is below 1e-30 of the diagonal's.  A matrix formed by contractions (N =
X^H M X) is Hermitian only to a few ulps.  Unitary rotations keep the
Frobenius norm of that anti-Hermitian residue, so when it is larger than the
stopping level the off-diagonal mass never reaches it.  On a rank-deficient
matrix, the residue then dominates the near-zero eigenvalues and the
rotations computed from one triangle keep cycling.  The Hermitian part
converges in a few sweeps.  No GPU is used."""
import numpy as np
import pytest


def _pair(n_even, r, k):
    if k == 0:
        a, b = n_even - 1, r % (n_even - 1)
    else:
        a, b = (r + k) % (n_even - 1), (r - k + n_even - 1) % (n_even - 1)
    return min(a, b), max(a, b)


def jacobi_sweeps(A, max_sweeps=40):
    """(sweeps used, stopped, A after the last sweep) of the kernel's iteration."""
    A = np.array(A, dtype=complex)
    n = A.shape[0]
    n_even = n + (n & 1)
    for sweep in range(max_sweeps):
        diag = np.diag(A).real
        dn = float(diag @ diag)
        on = float((np.abs(A - np.diag(np.diag(A))) ** 2).sum())  # the kernel sums the off-diagonal directly
        if on <= 1e-30 * (dn + 1e-300):
            return sweep, True, A
        rotated = False
        for r in range(n_even - 1):
            rots = []
            for k in range(n_even // 2):
                p, q = _pair(n_even, r, k)
                if q >= n:
                    continue
                g = abs(A[p, q])
                app, aqq = A[p, p].real, A[q, q].real
                if g <= 1e-300 or g <= 1e-17 * np.sqrt(abs(app * aqq)) or g <= 1e-16 * np.sqrt(on + dn):
                    continue
                rotated = True
                zeta = (aqq - app) / (2.0 * g)
                t = (1.0 if zeta >= 0 else -1.0) / (abs(zeta) + np.sqrt(1.0 + zeta * zeta))
                c = 1.0 / np.sqrt(1.0 + t * t)
                rots.append((p, q, c, c * t, A[p, q] / g))
            for p, q, c, s, ph in rots:  # columns: A <- A J (column q phased by conj(ph))
                a, b = A[:, p].copy(), A[:, q] * np.conj(ph)
                A[:, p], A[:, q] = c * a - s * b, s * a + c * b
            for p, q, c, s, ph in rots:  # rows: A <- J^H A
                a, b = A[p, :].copy(), A[q, :] * ph
                A[p, :], A[q, :] = c * a - s * b, s * a + c * b
        if not rotated:
            return sweep, True, A
    return max_sweeps, False, A


def _nearly_hermitian(n, rank, residue, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, rank)) + 1j * rng.standard_normal((n, rank))
    m = (x @ x.conj().T) * 1e-15
    e = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    e = e - e.conj().T
    return m + e * (residue * np.linalg.norm(m) / np.linalg.norm(e))


@pytest.mark.parametrize("n,rank", [(16, 4), (24, 6)])
def test_raw_nearly_hermitian_input_does_not_converge(n, rank):
    m = _nearly_hermitian(n, rank, 1e-11, n + rank)
    sweeps, stopped, _ = jacobi_sweeps(m)
    assert not stopped and sweeps == 40


@pytest.mark.parametrize("n,rank", [(16, 4), (24, 6)])
def test_hermitian_part_converges_to_eigvalsh(n, rank):
    m = _nearly_hermitian(n, rank, 1e-11, n + rank)
    h = 0.5 * (m + m.conj().T)
    sweeps, stopped, a = jacobi_sweeps(h)
    assert stopped and sweeps <= 10
    ref = np.linalg.eigvalsh(h)
    assert np.abs(np.sort(np.diag(a).real) - ref).max() <= 1e-13 * np.abs(ref).max()


def test_random_hermitian_converges():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((20, 20)) + 1j * rng.standard_normal((20, 20))
    a = a + a.conj().T
    sweeps, stopped, b = jacobi_sweeps(a)
    assert stopped and sweeps <= 12
    assert np.abs(np.sort(np.diag(b).real) - np.linalg.eigvalsh(a)).max() <= 1e-12 * np.abs(a).max()
