// FP64 complex dense linear algebra of the center-site path, all on the GPU:
//  * one-sided (Hestenes) Jacobi SVD of small matrices, one CTA per matrix
//    (NDArrayData.normalizeAxis / svd / unitize, data/__init__.py:263-346,
//    utils.py:879-882);
//  * parallel two-sided Jacobi eigensolver of small Hermitian matrices
//    (computeCompressor's eigh, utils.py:268-302);
//  * blocked Cholesky factorisation and triangular inverse of the
//    normalization matrix, and a Lanczos eigensolver with full
//    reorthogonalisation for the lowest generalized eigenpair of
//    (H_eff, N_eff) (minimizeExpectation / minimizeExpectationUsingFullEigensolver,
//    system/_2d.py:489-502).
// Every iterative routine has an iteration budget and reports
// CARC_NOT_CONVERGED through a status word instead of looping on.
#include "common.cuh"
#include "contract.cuh"
#include "linalg.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace carc {

namespace {

constexpr int SVD_THREADS = 256;
constexpr int SVD_WARPS = SVD_THREADS / 32;

// Pair (p,q) of the round-robin tournament over n (even) players in round r.
__device__ __forceinline__ void tournament_pair(int n, int r, int k, int* p, int* q) {
  // player n-1 is fixed; the others rotate
  int a, b;
  if (k == 0) {
    a = n - 1;
    b = r % (n - 1);
  } else {
    a = (r + k) % (n - 1);
    b = (r - k + (n - 1)) % (n - 1);
  }
  *p = min(a, b);
  *q = max(a, b);
}

// One-sided Jacobi on the columns of W (m x n, column j at W + j, row stride ldw)
// accumulating the right rotations into V (n x n, column-major in the same way).
__global__ __launch_bounds__(SVD_THREADS) void svd_jacobi_kernel(int m, int n, int n_even, double2* __restrict__ Wall,
                                                                  int64_t w_stride, double2* __restrict__ Vall,
                                                                  int64_t v_stride, double* __restrict__ Sall,
                                                                  int* __restrict__ status, int max_sweeps, double tol) {
  double2* W = Wall + blockIdx.x * w_stride;  // row-major m x n
  double2* V = Vall + blockIdx.x * v_stride;  // row-major n x n
  double* S = Sall + blockIdx.x * (int64_t)n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int rotated;
  // V = I
  for (int i = threadIdx.x; i < n * n; i += SVD_THREADS) V[i] = make_double2((i / n) == (i % n) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < n_even - 1; ++r) {
      for (int k = warp; k < n_even / 2; k += SVD_WARPS) {
        int p, q;
        tournament_pair(n_even, r, k, &p, &q);
        if (q >= n) continue;  // padding column
        double alpha = 0.0, beta = 0.0;
        double2 gamma = make_double2(0.0, 0.0);
        for (int i = lane; i < m; i += 32) {
          double2 a = W[(int64_t)i * n + p], b = W[(int64_t)i * n + q];
          alpha += cabs2(a);
          beta += cabs2(b);
          gamma = cadd(gamma, cmulc(a, b));
        }
        alpha = warp_sum(alpha);
        beta = warp_sum(beta);
        gamma = warp_sum2(gamma);
        double g = sqrt(cabs2(gamma));
        // converged pair: orthogonal to tol, or the smaller column negligible
        // (norm below 1e-14 of the larger: rounding noise of a rank-deficient
        // input, which no rotation makes orthogonal; its U column is replaced by
        // the orthonormal completion of svd_complete_kernel)
        if (g == 0.0 || g <= tol * sqrt(alpha * beta) || fmin(alpha, beta) <= 1e-28 * fmax(alpha, beta)) continue;
        if (lane == 0) rotated = 1;
        double zeta = (beta - alpha) / (2.0 * g);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        double2 ph = make_double2(gamma.x / g, -gamma.y / g);  // e^{-i phi}
        for (int i = lane; i < m; i += 32) {
          double2 a = W[(int64_t)i * n + p], b = cmul(W[(int64_t)i * n + q], ph);
          W[(int64_t)i * n + p] = make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
          W[(int64_t)i * n + q] = make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
        }
        for (int i = lane; i < n; i += 32) {
          double2 a = V[i * n + p], b = cmul(V[i * n + q], ph);
          V[i * n + p] = make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
          V[i * n + q] = make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
        }
      }
      __syncthreads();
    }
    __syncthreads();
    if (!rotated) break;
    __syncthreads();
  }
  if (threadIdx.x == 0 && sweep >= max_sweeps) atomicExch(status, CARC_NOT_CONVERGED);
  // column norms
  for (int j = warp; j < n; j += SVD_WARPS) {
    double s = 0.0;
    for (int i = lane; i < m; i += 32) s += cabs2(W[(int64_t)i * n + j]);
    s = warp_sum(s);
    if (lane == 0) S[j] = sqrt(s);
  }
}

// Sort singular values descending and write U = W[:,perm]/S, Vh = V[:,perm]^H.
__global__ void svd_finish_kernel(int m, int n, const double2* __restrict__ Wall, int64_t w_stride,
                                  const double2* __restrict__ Vall, int64_t v_stride, const double* __restrict__ Sraw,
                                  double2* __restrict__ Uall, int64_t u_stride, double* __restrict__ Sout,
                                  double2* __restrict__ Vhall, int64_t vh_stride) {
  extern __shared__ int perm[];
  const double2* W = Wall + blockIdx.x * w_stride;
  const double2* V = Vall + blockIdx.x * v_stride;
  const double* S = Sraw + blockIdx.x * (int64_t)n;
  double2* U = Uall + blockIdx.x * u_stride;
  double2* Vh = Vhall + blockIdx.x * vh_stride;
  if (threadIdx.x == 0) {
    for (int j = 0; j < n; ++j) perm[j] = j;
    for (int a = 0; a < n; ++a) {  // selection sort, descending, stable on ties
      int best = a;
      for (int b = a + 1; b < n; ++b)
        if (S[perm[b]] > S[perm[best]]) best = b;
      int t = perm[best];
      for (int b = best; b > a; --b) perm[b] = perm[b - 1];
      perm[a] = t;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) Sout[blockIdx.x * (int64_t)n + j] = S[perm[j]];
  for (int64_t idx = threadIdx.x; idx < (int64_t)m * n; idx += blockDim.x) {
    int i = (int)(idx / n), j = (int)(idx % n);
    double s = S[perm[j]];
    double2 w = W[(int64_t)i * n + perm[j]];
    U[idx] = s > 0 ? make_double2(w.x / s, w.y / s) : make_double2(0.0, 0.0);
  }
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx / n, j = idx % n;  // Vh[i][j] = conj(V[j][perm[i]])
    Vh[idx] = cconj(V[j * n + perm[i]]);
  }
}

// Columns of U whose singular value is negligible (<= tiny * S_max) are
// replaced by an orthonormal completion (Gram-Schmidt, twice, of the standard
// basis vectors against the columns already present), so that U stays an
// isometry for rank-deficient input, as LAPACK's U does.
__global__ void svd_complete_kernel(int m, int n, double2* __restrict__ Uall, int64_t u_stride,
                                    const double* __restrict__ Sall, double tiny) {
  double2* U = Uall + blockIdx.x * u_stride;
  const double* S = Sall + blockIdx.x * (int64_t)n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ double2 coef[SVD_WARPS * 4];
  __shared__ double nrm;
  __shared__ int cand;
  const double smax = S[0];
  for (int j = 0; j < n; ++j) {
    if (S[j] > tiny * smax && S[j] > 0.0) continue;
    if (threadIdx.x == 0) cand = 0;
    __syncthreads();
    for (int tries = 0; tries < m; ++tries) {
      // column j = e_cand
      for (int i = threadIdx.x; i < m; i += blockDim.x) U[(int64_t)i * n + j] = make_double2(i == cand ? 1.0 : 0.0, 0.0);
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        for (int c = 0; c < n; ++c) {
          if (c == j || (c > j && !(S[c] > tiny * smax && S[c] > 0.0))) continue;  // only valid/completed columns
          double2 acc = make_double2(0.0, 0.0);
          for (int i = threadIdx.x; i < m; i += blockDim.x) acc = cadd(acc, cmulc(U[(int64_t)i * n + c], U[(int64_t)i * n + j]));
          acc = warp_sum2(acc);
          if (lane == 0) coef[warp] = acc;
          __syncthreads();
          double2 h = make_double2(0.0, 0.0);
          for (int w = 0; w < SVD_WARPS; ++w) h = cadd(h, coef[w]);
          for (int i = threadIdx.x; i < m; i += blockDim.x)
            U[(int64_t)i * n + j] = csub(U[(int64_t)i * n + j], cmul(h, U[(int64_t)i * n + c]));
          __syncthreads();
        }
      }
      double a = 0.0;
      for (int i = threadIdx.x; i < m; i += blockDim.x) a += cabs2(U[(int64_t)i * n + j]);
      a = warp_sum(a);
      if (lane == 0) coef[warp] = make_double2(a, 0.0);
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < SVD_WARPS; ++w) t += coef[w].x;
        nrm = sqrt(t);
      }
      __syncthreads();
      if (nrm > 0.5) break;
      if (threadIdx.x == 0) cand = cand + 1;
      __syncthreads();
    }
    const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) U[(int64_t)i * n + j] = cscale(U[(int64_t)i * n + j], inv);
    __syncthreads();
  }
}

}  // namespace

int64_t svd_workspace_size(int m, int n, int batch) {
  return ((int64_t)m * n + (int64_t)n * n) * batch * 16 + (int64_t)n * batch * 8 + 256;
}

int svd_jacobi(int m, int n, int batch, const void* A, void* U, void* S, void* Vh, void* status, void* ws,
               int64_t ws_bytes, cudaStream_t stream) {
  if (m < 1 || n < 1 || batch < 1) return fail(CARC_BAD_SHAPE, "svd: bad shape %d x %d (batch %d)", m, n, batch);
  if (m < n) return fail(CARC_BAD_SHAPE, "svd: needs m >= n (got %d x %d); factor the adjoint instead", m, n);
  if (ws_bytes < svd_workspace_size(m, n, batch)) return fail(CARC_BAD_ARG, "svd: workspace too small");
  char* p = static_cast<char*>(ws);
  double2* W = reinterpret_cast<double2*>(p);
  double2* V = W + (int64_t)m * n * batch;
  double* Sraw = reinterpret_cast<double*>(V + (int64_t)n * n * batch);
  CARC_CHECK_CUDA(cudaMemcpyAsync(W, A, (int64_t)m * n * batch * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), stream));
  const int n_even = n + (n & 1);
  svd_jacobi_kernel<<<batch, SVD_THREADS, 0, stream>>>(m, n, n_even, W, (int64_t)m * n, V, (int64_t)n * n, Sraw,
                                                      static_cast<int*>(status), 60, 4e-16 * sqrt((double)m) + 1e-15);
  CARC_CHECK_LAUNCH();
  svd_finish_kernel<<<batch, 256, n * sizeof(int), stream>>>(m, n, W, (int64_t)m * n, V, (int64_t)n * n, Sraw,
                                                              static_cast<double2*>(U), (int64_t)m * n,
                                                              static_cast<double*>(S), static_cast<double2*>(Vh),
                                                              (int64_t)n * n);
  CARC_CHECK_LAUNCH();
  svd_complete_kernel<<<batch, SVD_THREADS, 0, stream>>>(m, n, static_cast<double2*>(U), (int64_t)m * n,
                                                        static_cast<const double*>(S), 1e-13 * (double)std::max(m, n));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// Hermitian Jacobi eigensolver (small n, one CTA per matrix)
// ---------------------------------------------------------------------------
namespace {

constexpr int HEEV_THREADS = 256;

// A is n x n row-major (overwritten), V accumulates eigenvectors (columns).
__global__ __launch_bounds__(HEEV_THREADS) void heev_jacobi_kernel(int n, int n_even, double2* __restrict__ Aall,
                                                                    double2* __restrict__ Vall, int* status,
                                                                    int max_sweeps) {
  double2* A = Aall + blockIdx.x * (int64_t)n * n;
  double2* V = Vall + blockIdx.x * (int64_t)n * n;
  extern __shared__ double rot[];  // per pair: c, s, ph.x, ph.y, p, q  (6 doubles)
  __shared__ double off_norm, diag_norm;
  for (int i = threadIdx.x; i < n * n; i += HEEV_THREADS) V[i] = make_double2((i / n) == (i % n) ? 1.0 : 0.0, 0.0);
  // the Hermitian part (A + A^H) / 2: the rotations are computed from the
  // upper triangle, and any anti-Hermitian residue of the input (a product
  // such as X^H M X rounds to a matrix that is Hermitian only to a few ulps of
  // its largest entries) survives every unitary rotation with its Frobenius
  // norm intact, so on a matrix whose small eigenvalues lie below that residue
  // the off-diagonal mass would never fall to the stopping level
  for (int idx = threadIdx.x; idx < n * n; idx += HEEV_THREADS) {
    const int i = idx / n, j = idx % n;
    if (i > j) continue;
    const double2 u = A[i * n + j], l = A[j * n + i];
    const double2 h = make_double2(0.5 * (u.x + l.x), i == j ? 0.0 : 0.5 * (u.y - l.y));
    A[i * n + j] = h;
    A[j * n + i] = cconj(h);
  }
  __syncthreads();
  const int npairs = n_even / 2;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int rotated = 0;  // this thread's rotations in this sweep
    if (threadIdx.x == 0) {
      double on = 0.0, dn = 0.0;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double a = cabs2(A[i * n + j]);
          if (i == j) dn += a; else on += a;
        }
      off_norm = on;
      diag_norm = dn;
    }
    __syncthreads();
    if (off_norm <= 1e-30 * (diag_norm + 1e-300)) break;
    for (int r = 0; r < n_even - 1; ++r) {
      // rotation parameters for the disjoint pairs of this round
      for (int k = threadIdx.x; k < npairs; k += HEEV_THREADS) {
        int p, q;
        tournament_pair(n_even, r, k, &p, &q);
        double* R = rot + 6 * k;
        R[4] = p;
        R[5] = q;
        R[0] = 1.0;
        R[1] = 0.0;
        R[2] = 1.0;
        R[3] = 0.0;
        if (q >= n) continue;
        double2 apq = A[p * n + q];
        double g = sqrt(cabs2(apq));
        double app = A[p * n + p].x, aqq = A[q * n + q].x;
        // converged pair: negligible against its diagonal, or against the
        // matrix (1e-16 of the Frobenius norm: the rounding level of a nearly
        // singular matrix, whose small diagonal entries alone would keep
        // noise-level pairs rotating forever)
        if (g <= 1e-300 || g <= 1e-17 * sqrt(fabs(app * aqq)) || g <= 1e-16 * sqrt(off_norm + diag_norm)) continue;
        rotated = 1;
        // phase-rotate so the off-diagonal is real, then a real Jacobi rotation
        double zeta = (aqq - app) / (2.0 * g);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        R[0] = c;
        R[1] = s;
        R[2] = apq.x / g;  // e^{i phi}
        R[3] = apq.y / g;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J  with J acting on (p, q)
      for (int idx = threadIdx.x; idx < npairs * n; idx += HEEV_THREADS) {
        int k = idx / n, i = idx % n;
        const double* R = rot + 6 * k;
        int p = (int)R[4], q = (int)R[5];
        if (q >= n || R[1] == 0.0) continue;
        double c = R[0], s = R[1];
        double2 ph = make_double2(R[2], R[3]);
        double2 ph_c = cconj(ph);
        // column q is first phased by e^{-i phi}
        double2 a = A[i * n + p], b = cmul(A[i * n + q], ph_c);
        A[i * n + p] = make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
        A[i * n + q] = make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
        double2 va = V[i * n + p], vb = cmul(V[i * n + q], ph_c);
        V[i * n + p] = make_double2(c * va.x - s * vb.x, c * va.y - s * vb.y);
        V[i * n + q] = make_double2(s * va.x + c * vb.x, s * va.y + c * vb.y);
      }
      __syncthreads();
      // rows: A <- J^H A
      for (int idx = threadIdx.x; idx < npairs * n; idx += HEEV_THREADS) {
        int k = idx / n, j = idx % n;
        const double* R = rot + 6 * k;
        int p = (int)R[4], q = (int)R[5];
        if (q >= n || R[1] == 0.0) continue;
        double c = R[0], s = R[1];
        double2 ph = make_double2(R[2], R[3]);
        double2 a = A[p * n + j], b = cmul(A[q * n + j], ph);
        A[p * n + j] = make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
        A[q * n + j] = make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
      }
      __syncthreads();
    }
    // one barrier both joins the threads' flags and ends the sweep, so no
    // thread can read a flag that the next sweep has already reset
    if (!__syncthreads_or(rotated)) break;
  }
  if (threadIdx.x == 0 && sweep >= max_sweeps) atomicExch(status, CARC_NOT_CONVERGED);
}

// eigenvalues ascending; W[j] = A[perm j][perm j], Vout[:, j] = V[:, perm j]
__global__ void heev_finish_kernel(int n, const double2* __restrict__ Aall, const double2* __restrict__ Vall,
                                   double* __restrict__ Wout, double2* __restrict__ Vout) {
  extern __shared__ int perm[];
  const double2* A = Aall + blockIdx.x * (int64_t)n * n;
  const double2* V = Vall + blockIdx.x * (int64_t)n * n;
  if (threadIdx.x == 0) {
    for (int j = 0; j < n; ++j) perm[j] = j;
    for (int a = 0; a < n; ++a) {
      int best = a;
      for (int b = a + 1; b < n; ++b)
        if (A[perm[b] * n + perm[b]].x < A[perm[best] * n + perm[best]].x) best = b;
      int t = perm[best];
      for (int b = best; b > a; --b) perm[b] = perm[b - 1];
      perm[a] = t;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) Wout[blockIdx.x * (int64_t)n + j] = A[perm[j] * n + perm[j]].x;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx / n, j = idx % n;
    Vout[blockIdx.x * (int64_t)n * n + idx] = V[i * n + perm[j]];
  }
}

}  // namespace

int64_t heev_workspace_size(int n, int batch) { return 2 * (int64_t)n * n * batch * 16 + 256; }

int heev_jacobi(int n, int batch, const void* A, void* W, void* V, void* status, void* ws, int64_t ws_bytes,
                cudaStream_t stream) {
  if (n < 1 || batch < 1) return fail(CARC_BAD_SHAPE, "heev: bad shape");
  if (n > 512) return fail(CARC_TOO_LARGE, "heev: Jacobi eigensolver limited to n <= 512 (got %d)", n);
  if (ws_bytes < heev_workspace_size(n, batch)) return fail(CARC_BAD_ARG, "heev: workspace too small");
  double2* Aw = static_cast<double2*>(ws);
  double2* Vw = Aw + (int64_t)n * n * batch;
  CARC_CHECK_CUDA(cudaMemcpyAsync(Aw, A, (int64_t)n * n * batch * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), stream));
  const int n_even = n + (n & 1);
  heev_jacobi_kernel<<<batch, HEEV_THREADS, 6 * sizeof(double) * (n_even / 2), stream>>>(
      n, n_even, Aw, Vw, static_cast<int*>(status), 40);
  CARC_CHECK_LAUNCH();
  heev_finish_kernel<<<batch, 256, n * sizeof(int), stream>>>(n, Aw, Vw, static_cast<double*>(W),
                                                               static_cast<double2*>(V));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// Blocked Cholesky  A = L L^H  (lower, in place; the strict upper part is zeroed)
// ---------------------------------------------------------------------------
namespace {

constexpr int NB = 32;

// Factor the nb x nb diagonal block at (k0,k0) in shared memory.
__global__ void potrf_diag_kernel(int n, double2* __restrict__ A, int k0, int nb, int* status, double scale) {
  __shared__ double2 T[NB][NB + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 32
  for (int i = ty; i < nb; i += blockDim.y)
    if (tx < nb) T[i][tx] = A[(int64_t)(k0 + i) * n + k0 + tx];
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    __shared__ double djj;
    if (tx == 0 && ty == 0) {
      double d = T[j][j].x;
      if (!(d > 1e-300 * scale) || isnan(d)) {
        atomicExch(status, CARC_NOT_POSDEF);
        d = 1.0;
      }
      djj = sqrt(d);
      T[j][j] = make_double2(djj, 0.0);
    }
    __syncthreads();
    // column below the pivot
    if (ty == 0 && tx > j && tx < nb) T[tx][j] = cscale(T[tx][j], 1.0 / djj);
    __syncthreads();
    // trailing update of the lower triangle: T[i][c] -= T[i][j] conj(T[c][j])
    for (int i = ty; i < nb; i += blockDim.y)
      if (i > j && tx > j && tx <= i) T[i][tx] = csub(T[i][tx], cmul(T[i][j], cconj(T[tx][j])));
    __syncthreads();
  }
  for (int i = ty; i < nb; i += blockDim.y)
    if (tx < nb) A[(int64_t)(k0 + i) * n + k0 + tx] = tx <= i ? T[i][tx] : make_double2(0.0, 0.0);
}

// L21 = A21 L11^{-H}: each warp solves one row x with x L11^H = a (forward substitution).
__global__ void potrf_panel_kernel(int n, double2* __restrict__ A, int k0, int nb) {
  __shared__ double2 L11[NB][NB + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int i = idx / nb, j = idx % nb;
    L11[i][j] = A[(int64_t)(k0 + i) * n + k0 + j];
  }
  __syncthreads();
  for (int row = k0 + nb + blockIdx.x * nwarps + warp; row < n; row += gridDim.x * nwarps) {
    double2* a = A + (int64_t)row * n + k0;
    double2 x = lane < nb ? a[lane] : make_double2(0.0, 0.0);
    // x_j = (a_j - sum_{c<j} x_c conj(L[j][c])) / L[j][j]
    for (int j = 0; j < nb; ++j) {
      double2 xj = make_double2(__shfl_sync(0xffffffffu, x.x, j), __shfl_sync(0xffffffffu, x.y, j));
      xj = cscale(xj, 1.0 / L11[j][j].x);
      if (lane == j) x = xj;
      if (lane > j && lane < nb) x = csub(x, cmul(xj, cconj(L11[lane][j])));
    }
    if (lane < nb) a[lane] = x;
  }
}

// zero the strict upper triangle
__global__ void zero_upper_kernel(int n, double2* __restrict__ A) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / n), j = (int)(idx % n);
    if (j > i) A[idx] = make_double2(0.0, 0.0);
  }
}

__global__ void max_diag_kernel(int n, const double2* __restrict__ A, double* out) {
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(A[(int64_t)i * n + i].x));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double w[32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmax(r, w[i]);
    *out = r;
  }
}

}  // namespace

int64_t potrf_workspace_size(int n) {
  // trailing update scratch of the GETT (split-K never triggers for K = NB, but query anyway)
  carc_contract_desc d = DescBuilder().m(n, n, n).n(n, n, 1).k(NB, 1, 1).d;
  return std::max<int64_t>(gett_workspace_size(d, 1), 0) + 256;
}

int potrf(int n, void* Av, void* status, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  if (n < 1) return fail(CARC_BAD_SHAPE, "potrf: n = %d", n);
  double2* A = static_cast<double2*>(Av);
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), stream));
  for (int k0 = 0; k0 < n; k0 += NB) {
    int nb = std::min(NB, n - k0);
    potrf_diag_kernel<<<1, dim3(32, 32), 0, stream>>>(n, A, k0, nb, static_cast<int*>(status), 1.0);
    CARC_CHECK_LAUNCH();
    int rest = n - k0 - nb;
    if (rest <= 0) break;
    int warps_needed = rest;
    int blocks = (int)std::min<int64_t>(ceil_div(warps_needed, 8), 4 * 152);
    potrf_panel_kernel<<<blocks, 256, 0, stream>>>(n, A, k0, nb);
    CARC_CHECK_LAUNCH();
    // A22 -= L21 L21^H   (rows/cols k0+nb .. n-1), full square; upper part zeroed at the end
    double2* L21 = A + (int64_t)(k0 + nb) * n + k0;
    double2* A22 = A + (int64_t)(k0 + nb) * n + k0 + nb;
    carc_contract_desc d = DescBuilder().m(rest, n, n).n(rest, n, 1).k(nb, 1, 1).d;
    d.conj_b = 1;
    const void* pa[1] = {L21};
    const void* pb[1] = {L21};
    void* pc[1] = {A22};
    int32_t e[3] = {0, 0, 0};
    CARC_RETURN_IF(gett_launch(d, pa, 1, pb, 1, pc, 1, e, 1, make_double2(-1.0, 0.0), 1, ws, ws_bytes, stream));
  }
  zero_upper_kernel<<<(int)std::min<int64_t>(ceil_div((int64_t)n * n, 256), 1216), 256, 0, stream>>>(n, A);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// Inverse of a lower-triangular matrix:  X = L^{-1}  (blocked forward substitution)
// ---------------------------------------------------------------------------
namespace {

// X[k0:k0+nb, :] = L_kk^{-1} X[k0:k0+nb, :] for columns col < k0+nb (X is
// lower), in place.  Each block inverts the nb x nb diagonal block in shared
// memory (one thread per column of the inverse, forward substitution with the
// diagonal's reciprocals) and applies it to its 16 columns of X, 16 row groups
// of threads sharing the work: the columns are independent, so the whole
// update is parallel over (row, column).
constexpr int TRSM_COLS = 16, TRSM_ROWG = 16;
__global__ __launch_bounds__(TRSM_COLS * TRSM_ROWG) void trsm_diag_kernel(int n, const double2* __restrict__ Lm,
                                                                          double2* __restrict__ X, int k0, int nb) {
  __shared__ double2 Lk[NB][NB + 1];
  __shared__ double2 Li[NB][NB + 1];
  __shared__ double2 dinv[NB];
  __shared__ double2 Xs[NB][TRSM_COLS + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int i = idx / nb, j = idx % nb;
    Lk[i][j] = Lm[(int64_t)(k0 + i) * n + k0 + j];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const double2 d = Lk[i][i];
    const double den = cabs2(d);
    dinv[i] = make_double2(d.x / den, -d.y / den);
  }
  __syncthreads();
  // column c of L_kk^{-1}: solve L y = e_c (rows < c are zero)
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    for (int i = 0; i < c; ++i) Li[i][c] = make_double2(0.0, 0.0);
    Li[c][c] = dinv[c];
    for (int i = c + 1; i < nb; ++i) {
      double2 acc = make_double2(0.0, 0.0);
      for (int j = c; j < i; ++j) acc = cadd(acc, cmul(Lk[i][j], Li[j][c]));
      Li[i][c] = cmul(dinv[i], make_double2(-acc.x, -acc.y));
    }
  }
  const int tc = threadIdx.x % TRSM_COLS, tr = threadIdx.x / TRSM_COLS;
  const int cols = k0 + nb;
  for (int c0 = blockIdx.x * TRSM_COLS; c0 < cols; c0 += gridDim.x * TRSM_COLS) {
    const int col = c0 + tc;
    __syncthreads();
    for (int i = tr; i < nb; i += TRSM_ROWG)
      Xs[i][tc] = col < cols ? X[(int64_t)(k0 + i) * n + col] : make_double2(0.0, 0.0);
    __syncthreads();
    if (col < cols) {
      for (int i = tr; i < nb; i += TRSM_ROWG) {
        double2 acc = make_double2(0.0, 0.0);
        for (int j = 0; j <= i; ++j) cfma(acc, Li[i][j], Xs[j][tc]);
        X[(int64_t)(k0 + i) * n + col] = acc;
      }
    }
  }
}

__global__ void set_identity_kernel(int n, double2* __restrict__ X) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x)
    X[idx] = make_double2((idx / n) == (idx % n) ? 1.0 : 0.0, 0.0);
}

}  // namespace

int64_t trtri_workspace_size(int n) {
  carc_contract_desc d = DescBuilder().m(NB, n, n).n(n, 1, 1).k(n, 1, n).d;
  return std::max<int64_t>(gett_workspace_size(d, 1), 0) + 256;
}

int trtri_lower(int n, const void* Lv, void* Xv, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  const double2* Lm = static_cast<const double2*>(Lv);
  double2* X = static_cast<double2*>(Xv);
  set_identity_kernel<<<(int)std::min<int64_t>(ceil_div((int64_t)n * n, 256), 1216), 256, 0, stream>>>(n, X);
  CARC_CHECK_LAUNCH();
  for (int k0 = 0; k0 < n; k0 += NB) {
    int nb = std::min(NB, n - k0);
    if (k0 > 0) {
      // X[k0:k0+nb, 0:k0] -= L[k0:k0+nb, 0:k0] X[0:k0, 0:k0]   (columns >= k0 of the block are still I)
      carc_contract_desc d = DescBuilder().m(nb, n, n).n(k0, 1, 1).k(k0, 1, n).d;
      const void* pa[1] = {Lm + (int64_t)k0 * n};
      const void* pb[1] = {X};
      void* pc[1] = {X + (int64_t)k0 * n};
      int32_t e[3] = {0, 0, 0};
      CARC_RETURN_IF(gett_launch(d, pa, 1, pb, 1, pc, 1, e, 1, make_double2(-1.0, 0.0), 1, ws, ws_bytes, stream));
    }
    int cols = k0 + nb;
    trsm_diag_kernel<<<(int)std::max<int64_t>(1, ceil_div(cols, TRSM_COLS)), TRSM_COLS * TRSM_ROWG, 0, stream>>>(
        n, Lm, X, k0, nb);
    CARC_CHECK_LAUNCH();
  }
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// normalizeAxis epilogue (data/__init__.py:282-301): from S (n) and Vh (n x n)
//   normalizer   N[i][j] = sum_k Vh[k][i] conj(Vh[k][j]) SI[k]
//   denormalizer D[i][j] = sum_k conj(Vh[k][i]) Vh[k][j] S[k]
// or, with sqrt_svals, A[k][j] = conj(Vh[k][j]) sqrt(SI[k]), B[k][j] = Vh[k][j] sqrt(S[k]);
// SI[k] = 1/S[k] where |S[k]| > thresh (thresh <= 0: always), else S[k].
// ---------------------------------------------------------------------------
namespace {

__global__ void normalize_axis_finish_kernel(int n, const double* __restrict__ S, const double2* __restrict__ Vh,
                                             double thresh, int sqrt_svals, double2* __restrict__ out_a,
                                             double2* __restrict__ out_b) {
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx / n, j = idx % n;
    if (sqrt_svals) {
      double s = S[i];
      double si = (thresh <= 0 || fabs(s) > thresh) ? 1.0 / s : s;
      out_a[idx] = cscale(cconj(Vh[i * n + j]), sqrt(si));
      out_b[idx] = cscale(Vh[i * n + j], sqrt(s));
    } else {
      double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
      for (int k = 0; k < n; ++k) {
        double s = S[k];
        double si = (thresh <= 0 || fabs(s) > thresh) ? 1.0 / s : s;
        a = cadd(a, cscale(cmul(Vh[k * n + i], cconj(Vh[k * n + j])), si));
        b = cadd(b, cscale(cmul(cconj(Vh[k * n + i]), Vh[k * n + j]), s));
      }
      out_a[idx] = a;
      out_b[idx] = b;
    }
  }
}

}  // namespace

int normalize_axis_finish(int n, const void* S, const void* Vh, double thresh, int sqrt_svals, void* out_a,
                          void* out_b, cudaStream_t stream) {
  normalize_axis_finish_kernel<<<1, 256, 0, stream>>>(n, static_cast<const double*>(S),
                                                       static_cast<const double2*>(Vh), thresh, sqrt_svals,
                                                       static_cast<double2*>(out_a), static_cast<double2*>(out_b));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// Economic QR of a small m x n matrix (m >= n), one CTA: modified
// Gram-Schmidt with a second orthogonalisation pass; R has a real,
// non-negative diagonal (LAPACK's Householder QR may flip column signs).
// Used by NDArrayData.qr / newEnlargener (data/__init__.py:43-50, :314-317).
// ---------------------------------------------------------------------------
namespace {

__global__ void qr_mgs_kernel(int m, int n, const double2* __restrict__ A, double2* __restrict__ Q,
                              double2* __restrict__ R) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ double2 part[32];
  __shared__ double2 hsh;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) R[idx] = make_double2(0.0, 0.0);
  for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) Q[idx] = A[idx];
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    for (int pass = 0; pass < 2; ++pass) {
      for (int c = 0; c < j; ++c) {
        double2 acc = make_double2(0.0, 0.0);
        for (int i = threadIdx.x; i < m; i += blockDim.x) acc = cadd(acc, cmulc(Q[(int64_t)i * n + c], Q[(int64_t)i * n + j]));
        acc = warp_sum2(acc);
        if (lane == 0) part[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
          double2 h = make_double2(0.0, 0.0);
          for (int w = 0; w < nw; ++w) h = cadd(h, part[w]);
          hsh = h;
          R[c * n + j] = cadd(R[c * n + j], h);
        }
        __syncthreads();
        const double2 h = hsh;
        for (int i = threadIdx.x; i < m; i += blockDim.x)
          Q[(int64_t)i * n + j] = csub(Q[(int64_t)i * n + j], cmul(h, Q[(int64_t)i * n + c]));
        __syncthreads();
      }
    }
    double a = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) a += cabs2(Q[(int64_t)i * n + j]);
    a = warp_sum(a);
    if (lane == 0) part[warp] = make_double2(a, 0.0);
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += part[w].x;
      hsh = make_double2(sqrt(t), 0.0);
      R[j * n + j] = hsh;
    }
    __syncthreads();
    const double inv = hsh.x > 0 ? 1.0 / hsh.x : 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) Q[(int64_t)i * n + j] = cscale(Q[(int64_t)i * n + j], inv);
    __syncthreads();
  }
}

}  // namespace

int qr_mgs(int m, int n, const void* A, void* Q, void* R, cudaStream_t stream) {
  if (m < 1 || n < 1 || m < n) return fail(CARC_BAD_SHAPE, "qr: needs m >= n >= 1 (got %d x %d)", m, n);
  qr_mgs_kernel<<<1, 256, 0, stream>>>(m, n, static_cast<const double2*>(A), static_cast<double2*>(Q),
                                      static_cast<double2*>(R));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace carc
