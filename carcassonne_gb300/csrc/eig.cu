// Lowest eigenpair of the generalized Hermitian-definite problem H x = l N x
// on the GPU (the center-site optimisation of System.minimizeExpectation,
// system/_2d.py:489-502):
//   N = L L^H (blocked Cholesky), C = L^{-1} H L^{-H},
//   Lanczos with full reorthogonalisation (two classical Gram-Schmidt passes
//   with warp-shuffle dot products) on C, restarted from the Ritz vector,
//   the small tridiagonal problem solved on the device by Sturm bisection and
//   inverse iteration, and x = L^{-H} u.
// The host loop syncs the stream only at convergence checkpoints.
#include "common.cuh"
#include "contract.cuh"
#include "linalg.cuh"
#include "umma_gemm.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace carc {

namespace {

inline int64_t a256(int64_t b) { return (b + 255) / 256 * 256; }

// y = A x, A n x n row-major; one warp per row
__global__ void gemv_kernel(int n, const double2* __restrict__ A, const double2* __restrict__ x, double2* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
    const double2* a = A + (int64_t)row * n;
    double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
    int j = lane;
    for (; j + 96 < n; j += 128) {  // four independent chains keep four loads in flight
      cfma(s0, a[j], x[j]);
      cfma(s1, a[j + 32], x[j + 32]);
      cfma(s2, a[j + 64], x[j + 64]);
      cfma(s3, a[j + 96], x[j + 96]);
    }
    for (; j < n; j += 32) cfma(s0, a[j], x[j]);
    double2 s = cadd(cadd(s0, s1), cadd(s2, s3));
    s = warp_sum2(s);
    if (lane == 0) y[row] = s;
  }
}

// h[r] = sum_i conj(Q[r][i]) w[i] for r < rows; one warp per row
__global__ void proj_kernel(int n, int rows, const double2* __restrict__ Q, const double2* __restrict__ w,
                            double2* __restrict__ h) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
    const double2* q = Q + (int64_t)r * n;
    double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
    int j = lane;
    for (; j + 96 < n; j += 128) {
      s0 = cadd(s0, cmulc(q[j], w[j]));
      s1 = cadd(s1, cmulc(q[j + 32], w[j + 32]));
      s2 = cadd(s2, cmulc(q[j + 64], w[j + 64]));
      s3 = cadd(s3, cmulc(q[j + 96], w[j + 96]));
    }
    for (; j < n; j += 32) s0 = cadd(s0, cmulc(q[j], w[j]));
    double2 s = cadd(cadd(s0, s1), cadd(s2, s3));
    s = warp_sum2(s);
    if (lane == 0) h[r] = s;
  }
}

// w[i] += sign * sum_r h[r] Q[r][i]: a block covers 32 consecutive i with its
// 8 warps splitting r, the 8 partial sums added in a fixed order
constexpr int COMB_I = 32, COMB_R = 8;
__global__ __launch_bounds__(COMB_I * COMB_R) void combine_kernel(int n, int rows, const double2* __restrict__ Q,
                                                                  const double2* __restrict__ h, double sign,
                                                                  double2* __restrict__ w, int overwrite) {
  __shared__ double2 part[COMB_R][COMB_I];
  const int li = threadIdx.x % COMB_I, lr = threadIdx.x / COMB_I;
  for (int i0 = blockIdx.x * COMB_I; i0 < n; i0 += gridDim.x * COMB_I) {
    const int i = i0 + li;
    double2 s0 = make_double2(0.0, 0.0), s1 = make_double2(0.0, 0.0);
    if (i < n) {
      int r = lr;
      for (; r + COMB_R < rows; r += 2 * COMB_R) {
        cfma(s0, h[r], Q[(int64_t)r * n + i]);
        cfma(s1, h[r + COMB_R], Q[(int64_t)(r + COMB_R) * n + i]);
      }
      if (r < rows) cfma(s0, h[r], Q[(int64_t)r * n + i]);
    }
    part[lr][li] = cadd(s0, s1);
    __syncthreads();
    if (lr == 0 && i < n) {
      double2 t = part[0][li];
      for (int q = 1; q < COMB_R; ++q) t = cadd(t, part[q][li]);
      w[i] = overwrite ? cscale(t, sign) : cadd(w[i], cscale(t, sign));
    }
    __syncthreads();
  }
}

// w -= alpha_j q_j + beta_{j-1} q_{j-1}; alpha_j = Re(dot) read from the device
__global__ void lanczos_axpy_kernel(int n, int j, const double2* __restrict__ dotv, double* __restrict__ alpha,
                                    const double* __restrict__ beta, const double2* __restrict__ qj,
                                    const double2* __restrict__ qjm1, double2* __restrict__ w) {
  const double a = dotv->x;
  const double b = j > 0 ? beta[j - 1] : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) alpha[j] = a;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 v = csub(w[i], cscale(qj[i], a));
    if (j > 0) v = csub(v, cscale(qjm1[i], b));
    w[i] = v;
  }
}

// beta_j = ||w||, q_{j+1} = w / beta_j  (breakdown flag when beta is negligible)
__global__ void lanczos_next_kernel(int n, int j, const double2* __restrict__ nrm2, double* __restrict__ beta,
                                    const double2* __restrict__ w, double2* __restrict__ qn, double scale_ref,
                                    int* __restrict__ breakdown) {
  const double b = sqrt(fmax(nrm2->x, 0.0));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    beta[j] = b;
    if (b <= 1e-13 * scale_ref) *breakdown = 1;
  }
  const double inv = b > 0 ? 1.0 / b : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) qn[i] = cscale(w[i], inv);
}

__global__ void scale_by_norm_kernel(int n, const double2* __restrict__ nrm2, double2* __restrict__ v) {
  const double b = sqrt(fmax(nrm2->x, 0.0));
  const double inv = b > 0 ? 1.0 / b : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = cscale(v[i], inv);
}

// Number of eigenvalues of the symmetric tridiagonal T = (alpha, beta) below
// x: sign changes of the characteristic-polynomial sequence
//   p_0 = 1, p_1 = alpha_0 - x, p_i = (alpha_{i-1} - x) p_{i-1} - beta_{i-2}^2 p_{i-2},
// rescaled as it grows (multiplications and additions only: no division in
// the recurrence).  A zero p_i takes the sign opposite to p_{i-1}.
template <typename T>
__device__ int sturm_count(int m, const double* alpha, const double* beta2, T x) {
  int c = 0;
  T p0 = 1, p1 = (T)alpha[0] - x;
  int s_prev = 1;
  int s1 = p1 > 0 ? 1 : (p1 < 0 ? -1 : -s_prev);
  if (s1 != s_prev) ++c;
  s_prev = s1;
  for (int i = 1; i < m; ++i) {
    T p2 = ((T)alpha[i] - x) * p1 - (T)beta2[i - 1] * p0;
    const int s2 = p2 > 0 ? 1 : (p2 < 0 ? -1 : -s_prev);
    if (s2 != s_prev) ++c;
    s_prev = s2;
    p0 = p1;
    p1 = p2;
    const T mag = fabs(p1) + fabs(p0);
    if (mag > (T)1e16 || (mag < (T)1e-16 && mag > 0)) {
      const T inv = (T)1 / mag;
      p0 *= inv;
      p1 *= inv;
    }
  }
  return c;
}

// Lowest eigenpair of the m x m tridiagonal matrix; out = (lambda, residual
// estimate |beta_{m-1} s_{m-1}|), s = unit eigenvector (m).  One block of
// TRI_THREADS threads: parallel multisection of the Gershgorin interval in
// FP32 (TRI_THREADS Sturm counts per round; GB300's FP64 rate makes FP64
// counts the expensive part), then, by one thread on shared-memory copies,
// inverse iteration in FP64 from the bracket's lower end (below the lowest
// eigenvalue, so the iteration converges to it) and the FP64 Rayleigh
// quotient of the iterate as the eigenvalue (quadratically accurate).
// m <= MAXM.
constexpr int MAXM = 512;
constexpr int TRI_THREADS = 256;

// Narrows [lo, hi] around the k-th lowest eigenvalue (k = 1, 2, ...).
template <typename T>
__device__ void multisect(int m, const double* a, const double* b2, double& lo, double& hi, double rel_stop,
                          int rounds, int* s_first, int k) {
  for (int r = 0; r < rounds; ++r) {
    const double w = hi - lo;
    if (!(w > rel_stop * fmax(fabs(lo), fabs(hi))) || w <= 0.0) break;
    if (threadIdx.x == 0) *s_first = TRI_THREADS;
    __syncthreads();
    const double xt = lo + w * (double)(threadIdx.x + 1) / (double)(TRI_THREADS + 1);
    if (sturm_count<T>(m, a, b2, (T)xt) >= k) atomicMin(s_first, (int)threadIdx.x);
    __syncthreads();
    const int f = *s_first;
    const double nlo = f == 0 ? lo : lo + w * (double)f / (double)(TRI_THREADS + 1);
    const double nhi = f == TRI_THREADS ? hi : lo + w * (double)(f + 1) / (double)(TRI_THREADS + 1);
    __syncthreads();
    lo = nlo;
    hi = nhi;
  }
}

__global__ __launch_bounds__(TRI_THREADS) void tridiag_lowest_kernel(int m, const double* __restrict__ alpha,
                                                                      const double* __restrict__ beta,
                                                                      double* __restrict__ out, double* __restrict__ s) {
  __shared__ double sa[MAXM], sb[MAXM], sb2[MAXM];
  __shared__ double dl[MAXM], dd[MAXM], du[MAXM], du2[MAXM], x[MAXM];
  __shared__ int piv[MAXM];
  __shared__ int s_first;
  __shared__ double s_lo, s_hi;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    sa[i] = alpha[i];
    sb[i] = i + 1 < m ? beta[i] : 0.0;
    sb2[i] = sb[i] * sb[i];
  }
  __syncthreads();
  if (m == 1) {
    if (threadIdx.x == 0) {
      s[0] = 1.0;
      out[0] = sa[0];
      out[1] = fabs(beta[0]);
      out[2] = nan("");
    }
    return;
  }
  if (threadIdx.x == 0) {
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < m; ++i) {
      const double r = (i > 0 ? fabs(sb[i - 1]) : 0.0) + (i + 1 < m ? fabs(sb[i]) : 0.0);
      lo = fmin(lo, sa[i] - r);
      hi = fmax(hi, sa[i] + r);
    }
    s_lo = lo;
    s_hi = hi;
  }
  __syncthreads();
  double lo = s_lo, hi = s_hi;
  const double span = fmax(hi - lo, 1e-300);
  multisect<float>(m, sa, sb2, lo, hi, 1e-6, 3, &s_first, 1);
  // the second-lowest eigenvalue to FP32 accuracy (a gap estimate for the caller)
  double lo2 = lo, hi2 = s_hi;
  multisect<float>(m, sa, sb2, lo2, hi2, 1e-6, 3, &s_first, 2);
  if (threadIdx.x != 0) return;
  out[2] = 0.5 * (lo2 + hi2);
  const double scale = fmax(fmax(fabs(s_lo), fabs(s_hi)), span);
  // FP32 counts can be off near the eigenvalue: shift below the bracket by a
  // margin larger than their error, so that T - shift is positive definite
  // and the iteration is drawn to the lowest eigenvector
  const double shift = lo - fmax(4.0 * (hi - lo), 1e-6 * scale);
  for (int i = 0; i < m; ++i) x[i] = 1.0 / sqrt((double)m) * (1.0 + 0.01 * (i % 7));
  double lam = 0.5 * (lo + hi);
  for (int iter = 0; iter < 4; ++iter) {
    for (int i = 0; i < m; ++i) {
      dd[i] = sa[i] - shift;
      dl[i] = sb[i];
      du[i] = sb[i];
      du2[i] = 0.0;
    }
    // LU with partial pivoting (the gttrf pattern)
    for (int i = 0; i + 1 < m; ++i) {
      if (fabs(dd[i]) >= fabs(dl[i])) {
        piv[i] = 0;
        double f = dd[i] != 0.0 ? dl[i] / dd[i] : 0.0;
        dl[i] = f;
        dd[i + 1] -= f * du[i];
      } else {
        piv[i] = 1;
        double f = dd[i] / dl[i];
        dd[i] = dl[i];
        dl[i] = f;
        double t = du[i];
        du[i] = dd[i + 1];
        dd[i + 1] = t - f * dd[i + 1];
        if (i + 2 < m) {
          du2[i] = du[i + 1];
          du[i + 1] = -f * du[i + 1];
        }
      }
    }
    for (int i = 0; i + 1 < m; ++i) {
      if (piv[i] == 0) {
        x[i + 1] -= dl[i] * x[i];
      } else {
        double t = x[i];
        x[i] = x[i + 1];
        x[i + 1] = t - dl[i] * x[i + 1];
      }
    }
    for (int i = m - 1; i >= 0; --i) {
      double v = x[i];
      if (i + 1 < m) v -= du[i] * x[i + 1];
      if (i + 2 < m) v -= du2[i] * x[i + 2];
      double d = dd[i] != 0.0 ? dd[i] : 1e-300 * scale;
      x[i] = v / d;
    }
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) nrm += x[i] * x[i];
    nrm = sqrt(nrm);
    if (!(nrm > 0.0) || isinf(nrm)) {
      for (int i = 0; i < m; ++i) x[i] = (i == 0) ? 1.0 : 0.0;
      nrm = 1.0;
    }
    const double inv = 1.0 / nrm;
    for (int i = 0; i < m; ++i) x[i] *= inv;
  }
  // Rayleigh quotient x^T T x
  double rq = 0.0;
  for (int i = 0; i < m; ++i) {
    double tx = sa[i] * x[i];
    if (i > 0) tx += sb[i - 1] * x[i - 1];
    if (i + 1 < m) tx += sb[i] * x[i + 1];
    rq += x[i] * tx;
  }
  lam = rq;
  for (int i = 0; i < m; ++i) s[i] = x[i];
  out[0] = lam;
  out[1] = fabs(beta[m - 1] * x[m - 1]);
}

// copy real s (m) into complex h (m)
__global__ void real_to_complex_kernel(int m, const double* __restrict__ s, double2* __restrict__ h) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) h[i] = make_double2(s[i], 0.0);
}

// u[i] += eps * max|u| * r_i with r_i a fixed hash sequence in [-1, 1]^2 (eps alone when u = 0).
// Launched as a single block so that every read of u precedes every write.
__global__ void perturb_start_kernel(int n, double2* __restrict__ u, double eps) {
  __shared__ double smax;
  if (threadIdx.x == 0) smax = 0.0;
  __syncthreads();
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, sqrt(cabs2(u[i])));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long*>(&smax), __double_as_longlong(m));
  __syncthreads();
  const double scale = eps * (smax > 0 ? smax : 1.0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    uint32_t h = 2654435761u * (uint32_t)(i + 1);
    h ^= h >> 16;
    h *= 2246822519u;
    h ^= h >> 13;
    uint32_t g = h * 3266489917u;
    g ^= g >> 16;
    const double rr = (double)(h & 0xffffff) / 8388608.0 - 1.0, ri = (double)(g & 0xffffff) / 8388608.0 - 1.0;
    u[i] = cadd(u[i], make_double2(scale * rr, scale * ri));
  }
}


// ---------------------------------------------------------------------------
// Lanczos iterations j0 .. j1-1 as one cooperative launch.  CTA c owns rows
// [c rpc, (c+1) rpc) of every vector: it forms its rows of w = C q_j (a warp
// per row), and every inner product is a fixed-order two-level sum (per-CTA
// partials, then one CTA per coefficient, or every CTA for a scalar)
// between bounded grid-wide barriers: 7 barriers per iteration (alpha, two
// reorthogonalisation passes of two, beta, q_{j+1} published) instead of
// about ten kernel launches.
// ---------------------------------------------------------------------------
constexpr int LZ_THREADS = 256;

struct LzParams {
  int n, j0, j1, rpc;
  const void* C;    // n x n, complex128 or complex64
  void* Q;          // (mk + 1) x n Krylov basis, same type
  double* alpha;
  double* beta;
  double2* pscal;   // [G] per-CTA partial of a scalar inner product
  double2* part;    // [(mk + 1) x G] per-CTA partials of the projections
  double2* h;       // (mk + 1) projections
  double scale_ref;
  double breakdown_tol;  // beta_j <= breakdown_tol * scale_ref ends the Krylov space
  int* breakdown;
  unsigned int* sync;  // barrier arrivals (zero at launch)
  int* abort;          // set by a CTA whose barrier wait ran out (zero at launch)
};

__device__ bool lz_grid_sync(unsigned int* ctr, unsigned int target, int* abort) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    int good = 0;
    for (uint32_t i = 0; i < (1u << 22); ++i) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
      if (v >= target) {
        good = 1;
        break;
      }
      if ((i & 255u) == 255u && *reinterpret_cast<volatile int*>(abort)) break;
      __nanosleep(32);
    }
    if (!good) atomicExch(abort, 1);
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <typename Z>
__device__ __forceinline__ Z from_d2(double2 a);
template <>
__device__ __forceinline__ double2 from_d2<double2>(double2 a) { return a; }
template <>
__device__ __forceinline__ float2 from_d2<float2>(double2 a) { return make_float2((float)a.x, (float)a.y); }

// Z = double2 (complex128) or float2 (complex64: the basis, the products and
// the per-CTA partials in FP32; the cross-CTA sums, alpha and beta in FP64)
template <typename Z>
__global__ __launch_bounds__(LZ_THREADS) void lanczos_chunk_kernel(const __grid_constant__ LzParams p) {
  using R = decltype(Z{}.x);
  extern __shared__ __align__(16) unsigned char lz_raw[];
  Z* lz_w = reinterpret_cast<Z*>(lz_raw);  // this CTA's rows of w
  __shared__ double s_alpha, s_bprev, s_beta;
  const Z* C = static_cast<const Z*>(p.C);
  Z* Q = static_cast<Z*>(p.Q);
  const int G = (int)gridDim.x, c = (int)blockIdx.x, n = p.n;
  const int r0 = c * p.rpc, r1 = min(n, r0 + p.rpc), nr = max(0, r1 - r0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  unsigned int bar = 0;
  auto gsync = [&]() { return lz_grid_sync(p.sync, ++bar * (unsigned)G, p.abort); };
  for (int j = p.j0; j < p.j1; ++j) {
    const Z* qj = Q + (int64_t)j * n;
    // w = C q_j on this CTA's rows (the four-chain row dot of gemv_kernel)
    for (int rl = warp; rl < nr; rl += nw) {
      const Z* a = C + (int64_t)(r0 + rl) * n;
      Z s0 = czero<Z>(), s1 = s0, s2 = s0, s3 = s0;
      int k = lane;
      for (; k + 96 < n; k += 128) {
        cfma(s0, a[k], qj[k]);
        cfma(s1, a[k + 32], qj[k + 32]);
        cfma(s2, a[k + 64], qj[k + 64]);
        cfma(s3, a[k + 96], qj[k + 96]);
      }
      for (; k < n; k += 32) cfma(s0, a[k], qj[k]);
      Z sum = warp_sum2(cadd(cadd(s0, s1), cadd(s2, s3)));
      if (lane == 0) lz_w[rl] = sum;
    }
    __syncthreads();
    // alpha_j = Re(q_j^H w)
    if (warp == 0) {
      double2 acc = make_double2(0.0, 0.0);
      for (int rl = lane; rl < nr; rl += 32) acc = cadd(acc, to_d2(cmulc(qj[r0 + rl], lz_w[rl])));
      acc = warp_sum2(acc);
      if (lane == 0) p.pscal[c] = acc;
    }
    if (!gsync()) return;
    if (warp == 0) {
      // the G partials in lane order, then a fixed shuffle tree: the same sum in every CTA
      double a = 0.0;
      for (int q = lane; q < G; q += 32) a += p.pscal[q].x;
      a = warp_sum(a);
      if (lane == 0) {
        s_alpha = a;
        s_bprev = j > 0 ? p.beta[j - 1] : 0.0;
      }
    }
    __syncthreads();
    for (int rl = threadIdx.x; rl < nr; rl += blockDim.x) {
      Z v = csub(lz_w[rl], cscale(qj[r0 + rl], (R)s_alpha));
      if (j > 0) v = csub(v, cscale(Q[(int64_t)(j - 1) * n + r0 + rl], (R)s_bprev));
      lz_w[rl] = v;
    }
    __syncthreads();
    // two classical Gram-Schmidt passes against q_0 .. q_j
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        Z acc = czero<Z>();
        const Z* qi = Q + (int64_t)i * n + r0;
#pragma unroll 8
        for (int rl = 0; rl < nr; ++rl) acc = cadd(acc, cmulc(qi[rl], lz_w[rl]));
        p.part[(int64_t)i * G + c] = to_d2(acc);
      }
      if (!gsync()) return;
      // coefficient i by warp (i / G) % nw of CTA i % G: lane-strided partials, fixed shuffle tree
      for (int i = c + warp * G; i <= j; i += nw * G) {
        double2 acc = make_double2(0.0, 0.0);
        for (int q = lane; q < G; q += 32) acc = cadd(acc, p.part[(int64_t)i * G + q]);
        acc = warp_sum2(acc);
        if (lane == 0) p.h[i] = acc;
      }
      if (!gsync()) return;
      for (int rl = warp; rl < nr; rl += nw) {
        Z acc = czero<Z>();
#pragma unroll 4
        for (int i = lane; i <= j; i += 32) cfma(acc, from_d2<Z>(p.h[i]), Q[(int64_t)i * n + r0 + rl]);
        acc = warp_sum2(acc);
        if (lane == 0) lz_w[rl] = csub(lz_w[rl], acc);
      }
      __syncthreads();
    }
    // beta_j = ||w||, q_{j+1} = w / beta_j
    if (threadIdx.x == 0) {
      double acc = 0.0;
      for (int rl = 0; rl < nr; ++rl) acc += (double)cabs2(lz_w[rl]);
      p.pscal[c] = make_double2(acc, 0.0);
    }
    if (!gsync()) return;
    if (warp == 0) {
      double b2 = 0.0;
      for (int q = lane; q < G; q += 32) b2 += p.pscal[q].x;
      b2 = warp_sum(b2);
      s_beta = sqrt(fmax(b2, 0.0));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (c == 0) {
        p.alpha[j] = s_alpha;
        p.beta[j] = s_beta;
        if (s_beta <= p.breakdown_tol * p.scale_ref) *p.breakdown = 1;
      }
    }
    __syncthreads();
    const R inv = s_beta > 0 ? (R)(1.0 / s_beta) : (R)0;
    for (int rl = threadIdx.x; rl < nr; rl += blockDim.x) Q[(int64_t)(j + 1) * n + r0 + rl] = cscale(lz_w[rl], inv);
    if (j + 1 < p.j1 && !gsync()) return;  // q_{j+1} complete before the next product
  }
}

inline int comb_blocks(int n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, COMB_I), 4 * 152)); }

inline int blocks_for(int64_t n, int threads = 256) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), 4 * 152));
}

struct LanczosWs {
  double2* Q;
  double2* w;
  double2* h;
  double2* dotv;
  double2* nrm;
  double* alpha;
  double* beta;
  double* tri_out;
  double* s;
  int* breakdown;
  void* dot_ws;
  int64_t dot_ws_bytes;
  double2* pscal;     // cooperative path: [LZ_MAX_CTAS]
  double2* part;      // [(mk + 1) x LZ_MAX_CTAS]
  unsigned int* sync; // [0] barrier arrivals, [1] abort flag
};

constexpr int LZ_MAX_CTAS = 152;

int64_t lanczos_ws_layout(int n, int mk, LanczosWs* L, void* base) {
  char* p = static_cast<char*>(base);
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    void* r = p ? p + off : nullptr;
    off += a256(bytes);
    return r;
  };
  LanczosWs t;
  t.Q = (double2*)take((int64_t)(mk + 1) * n * 16);
  t.w = (double2*)take((int64_t)n * 16);
  t.h = (double2*)take((int64_t)(mk + 1) * 16);
  t.dotv = (double2*)take(16);
  t.nrm = (double2*)take(16);
  t.alpha = (double*)take((int64_t)(mk + 1) * 8);
  t.beta = (double*)take((int64_t)(mk + 1) * 8);
  t.tri_out = (double*)take(4 * 8);
  t.s = (double*)take((int64_t)MAXM * 8);
  t.breakdown = (int*)take(16);
  t.dot_ws_bytes = dot_workspace_size(n);
  t.dot_ws = take(t.dot_ws_bytes);
  t.pscal = (double2*)take((int64_t)LZ_MAX_CTAS * 16);
  t.part = (double2*)take((int64_t)(mk + 1) * LZ_MAX_CTAS * 16);
  t.sync = (unsigned int*)take(16);
  if (L) *L = t;
  return off;
}

}  // namespace

int64_t lanczos_workspace_size(int n, int max_krylov) {
  int mk = std::max(1, std::min(max_krylov, std::min(n, MAXM)));
  return lanczos_ws_layout(n, mk, nullptr, nullptr);
}

int lanczos_lowest(int n, const void* Cv, const void* u0, void* u, double* eigenvalues, int max_krylov,
                   int max_restarts, double tol, int* iterations, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  if (n < 1) return fail(CARC_BAD_SHAPE, "lanczos: n = %d", n);
  const int mk = std::max(1, std::min(max_krylov, std::min(n, MAXM)));
  if (ws_bytes < lanczos_workspace_size(n, max_krylov)) return fail(CARC_BAD_ARG, "lanczos: workspace too small");
  LanczosWs W;
  lanczos_ws_layout(n, mk, &W, ws);
  const double2* C = static_cast<const double2*>(Cv);
  const int gb = blocks_for((int64_t)n * 32);
  const int eb = blocks_for(n);
  // cooperative chunks: about 8 rows per CTA (a warp per row), at most one CTA per SM
  static int sm_count = 0;
  if (sm_count == 0) {
    int dev = 0;
    CARC_CHECK_CUDA(cudaGetDevice(&dev));
    CARC_CHECK_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
  }
  const int lz_ctas = (int)std::max<int64_t>(1, std::min<int64_t>({ceil_div(n, 8), (int64_t)sm_count, LZ_MAX_CTAS}));
  const int lz_rpc = (int)ceil_div(n, lz_ctas);
  bool coop = true;
  // start vector
  CARC_CHECK_CUDA(cudaMemcpyAsync(W.Q, u0, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_RETURN_IF(dot_launch(n, W.Q, W.Q, 1, W.nrm, W.dot_ws, W.dot_ws_bytes, stream));
  scale_by_norm_kernel<<<eb, 256, 0, stream>>>(n, W.nrm, W.Q);
  CARC_CHECK_LAUNCH();
  // scale reference for the breakdown test: |C|_max row sum estimate via |C q0|
  double lam = 0.0, res = 0.0, lam2 = nan("");
  int total = 0;
  bool converged = false;
  for (int restart = 0; restart <= max_restarts && !converged; ++restart) {
    CARC_CHECK_CUDA(cudaMemsetAsync(W.breakdown, 0, sizeof(int), stream));
    int m = 0;
    double scale_ref = 1.0;
    {
      // scale of C from |C q0|
      gemv_kernel<<<gb, 256, 0, stream>>>(n, C, W.Q, W.w);
      CARC_CHECK_LAUNCH();
      CARC_RETURN_IF(dot_launch(n, W.w, W.w, 1, W.nrm, W.dot_ws, W.dot_ws_bytes, stream));
      double2 hn;
      CARC_CHECK_CUDA(cudaMemcpyAsync(&hn, W.nrm, 16, cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
      scale_ref = std::max(sqrt(std::max(hn.x, 0.0)), 1e-300);
    }
    for (int j = 0; j < mk; ++j) {
      if (coop && j % 8 == 0) {
        // iterations j .. j1-1 in one cooperative launch (per-iteration kernels below otherwise)
        const int j1 = std::min(mk, j + 8);
        LzParams lp;
        lp.n = n;
        lp.j0 = j;
        lp.j1 = j1;
        lp.rpc = lz_rpc;
        lp.C = C;
        lp.Q = W.Q;
        lp.alpha = W.alpha;
        lp.beta = W.beta;
        lp.pscal = W.pscal;
        lp.part = W.part;
        lp.h = W.h;
        lp.scale_ref = scale_ref;
        lp.breakdown_tol = 1e-13;
        lp.breakdown = W.breakdown;
        lp.sync = W.sync;
        lp.abort = reinterpret_cast<int*>(W.sync + 1);
        CARC_CHECK_CUDA(cudaMemsetAsync(W.sync, 0, 8, stream));
        cudaLaunchConfig_t cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3((unsigned)lz_ctas);
        cfg.blockDim = dim3(LZ_THREADS);
        cfg.dynamicSmemBytes = (size_t)lz_rpc * 16;
        cfg.stream = stream;
        cudaLaunchAttribute la[1];
        la[0].id = cudaLaunchAttributeCooperative;
        la[0].val.cooperative = 1;
        cfg.attrs = la;
        cfg.numAttrs = 1;
        if (cudaLaunchKernelEx(&cfg, lanczos_chunk_kernel<double2>, lp) == cudaSuccess) {
          count_launch();
          total += j1 - j - 1;
          j = j1 - 1;
          m = j1;
          ++total;
          const bool last = (j + 1 == mk);
          if ((m % 8) == 0 || last || m == n) {
            tridiag_lowest_kernel<<<1, TRI_THREADS, 0, stream>>>(m, W.alpha, W.beta, W.tri_out, W.s);
            CARC_CHECK_LAUNCH();
            double hv[3];
            int bd[3] = {0, 0, 0};
            CARC_CHECK_CUDA(cudaMemcpyAsync(hv, W.tri_out, 24, cudaMemcpyDeviceToHost, stream));
            CARC_CHECK_CUDA(cudaMemcpyAsync(&bd[0], W.breakdown, sizeof(int), cudaMemcpyDeviceToHost, stream));
            CARC_CHECK_CUDA(cudaMemcpyAsync(&bd[1], W.sync + 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
            CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
            if (bd[1]) return fail(CARC_NOT_CONVERGED, "lanczos: a grid barrier wait timed out");
            lam = hv[0];
            res = hv[1];
            lam2 = hv[2];
            if (bd[0] || res <= tol * std::max(fabs(lam), 1e-300) || m == n) {
              converged = true;
              break;
            }
          }
          continue;
        }
        (void)cudaGetLastError();  // not co-resident here: per-iteration kernels from now on
        coop = false;
      }
      double2* qj = W.Q + (int64_t)j * n;
      double2* qn = W.Q + (int64_t)(j + 1) * n;
      gemv_kernel<<<gb, 256, 0, stream>>>(n, C, qj, W.w);
      CARC_CHECK_LAUNCH();
      CARC_RETURN_IF(dot_launch(n, qj, W.w, 1, W.dotv, W.dot_ws, W.dot_ws_bytes, stream));
      lanczos_axpy_kernel<<<eb, 256, 0, stream>>>(n, j, W.dotv, W.alpha, W.beta, qj,
                                                  j > 0 ? W.Q + (int64_t)(j - 1) * n : qj, W.w);
      CARC_CHECK_LAUNCH();
      for (int pass = 0; pass < 2; ++pass) {
        proj_kernel<<<blocks_for((int64_t)(j + 1) * 32), 256, 0, stream>>>(n, j + 1, W.Q, W.w, W.h);
        CARC_CHECK_LAUNCH();
        combine_kernel<<<comb_blocks(n), COMB_I * COMB_R, 0, stream>>>(n, j + 1, W.Q, W.h, -1.0, W.w, 0);
        CARC_CHECK_LAUNCH();
      }
      CARC_RETURN_IF(dot_launch(n, W.w, W.w, 1, W.nrm, W.dot_ws, W.dot_ws_bytes, stream));
      lanczos_next_kernel<<<eb, 256, 0, stream>>>(n, j, W.nrm, W.beta, W.w, qn, scale_ref, W.breakdown);
      CARC_CHECK_LAUNCH();
      m = j + 1;
      ++total;
      const bool last = (j + 1 == mk);
      if ((m % 8) == 0 || last || m == n) {
        tridiag_lowest_kernel<<<1, TRI_THREADS, 0, stream>>>(m, W.alpha, W.beta, W.tri_out, W.s);
        CARC_CHECK_LAUNCH();
        double hv[3];
        int bd = 0;
        CARC_CHECK_CUDA(cudaMemcpyAsync(hv, W.tri_out, 24, cudaMemcpyDeviceToHost, stream));
        CARC_CHECK_CUDA(cudaMemcpyAsync(&bd, W.breakdown, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
        lam = hv[0];
        res = hv[1];
        lam2 = hv[2];
        if (bd || res <= tol * std::max(fabs(lam), 1e-300) || m == n) {
          converged = true;
          break;
        }
      }
    }
    // Ritz vector u = Q^T s (becomes the restart vector)
    real_to_complex_kernel<<<1, 256, 0, stream>>>(m, W.s, W.h);
    CARC_CHECK_LAUNCH();
    combine_kernel<<<comb_blocks(n), COMB_I * COMB_R, 0, stream>>>(n, m, W.Q, W.h, 1.0, W.w, 1);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(dot_launch(n, W.w, W.w, 1, W.nrm, W.dot_ws, W.dot_ws_bytes, stream));
    scale_by_norm_kernel<<<eb, 256, 0, stream>>>(n, W.nrm, W.w);
    CARC_CHECK_LAUNCH();
    CARC_CHECK_CUDA(cudaMemcpyAsync(W.Q, W.w, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  }
  CARC_CHECK_CUDA(cudaMemcpyAsync(u, W.w, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  if (eigenvalues) {
    eigenvalues[0] = lam;
    eigenvalues[1] = lam2;
  }
  if (iterations) *iterations = total;
  if (!converged)
    return fail(CARC_NOT_CONVERGED, "lanczos: residual %.3e after %d iterations (tolerance %.1e)", res, total, tol);
  return CARC_OK;
}

namespace {

// C = Li H Li^H on the tensor cores: views of the two products
ZView hegv_view(const void* base, int n, int64_t rs, int64_t ks, int conj) {
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = 1;
  v.r_ext[0] = n;
  v.r_str[0] = rs;
  v.nk = 1;
  v.k_ext[0] = n;
  v.k_str[0] = ks;
  v.conj = conj;
  return v;
}

ZOut hegv_out(void* base, int n) {
  ZOut o;
  memset(&o, 0, sizeof(o));
  o.base = base;
  o.nm = 1;
  o.m_ext[0] = n;
  o.m_str[0] = n;
  o.nn = 1;
  o.n_ext[0] = n;
  o.n_str[0] = 1;
  return o;
}

constexpr int HEGV_TC_KSPLIT = 4;

}  // namespace

// ---------------------------------------------------------------------------
// Single-precision reduction and Lanczos (CARC_HEGV_SINGLE), for the pencils
// of the mixed-precision solve: they carry the tensor-core forming error
// (about 1e-5 relative) already, and GB300 issues FP32 some 30 times faster
// than FP64.  N = L L^H and L^-1 in complex64 (blocked, NB = 32: diagonal
// block in shared memory, panel by forward substitution, trailing updates by
// a tiled complex64 GEMM), C = L^-1 H L^-H on the tensor cores (as with
// CARC_HEGV_TENSOR_CORE), and the cooperative Lanczos in complex64 with
// FP64 cross-CTA sums, alpha and beta.  The caller's eigenvalue comes from
// the tridiagonal in FP64; the solve's Rayleigh quotient with exact H x, N x
// makes the energy error second order in this eigenvector's error.
// ---------------------------------------------------------------------------
namespace {

constexpr int NB32 = 32;
constexpr int TRSM32_COLS = 16, TRSM32_ROWG = 16;

__global__ void c128_to_c64_kernel(int64_t count, const double2* __restrict__ a, float2* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

__global__ void c64_to_c128_kernel(int64_t count, const float2* __restrict__ a, double2* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = make_double2(a[i].x, a[i].y);
}

__global__ void potrf32_diag_kernel(int n, float2* __restrict__ A, int k0, int nb, int* status, float scale) {
  __shared__ float2 T[NB32][NB32 + 1];
  __shared__ float djj;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 32
  if (tx < nb && ty < nb) T[ty][tx] = A[(int64_t)(k0 + ty) * n + k0 + tx];
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (tx == 0 && ty == 0) {
      float d = T[j][j].x;
      if (!(d > 1e-30f * scale) || isnan(d)) {
        atomicExch(status, CARC_NOT_POSDEF);
        d = 1.0f;
      }
      djj = sqrtf(d);
      T[j][j] = make_float2(djj, 0.0f);
    }
    __syncthreads();
    if (ty == 0 && tx > j && tx < nb) T[tx][j] = cscale(T[tx][j], 1.0f / djj);
    __syncthreads();
    if (ty > j && ty < nb && tx > j && tx <= ty) T[ty][tx] = csub(T[ty][tx], cmul(T[ty][j], cconj(T[tx][j])));
    __syncthreads();
  }
  if (tx < nb && ty < nb) A[(int64_t)(k0 + ty) * n + k0 + tx] = tx <= ty ? T[ty][tx] : make_float2(0.0f, 0.0f);
}

// L21 = A21 L11^{-H}: a warp per row, forward substitution with shuffles
__global__ void potrf32_panel_kernel(int n, float2* __restrict__ A, int k0, int nb) {
  __shared__ float2 L11[NB32][NB32 + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) L11[idx / nb][idx % nb] = A[(int64_t)(k0 + idx / nb) * n + k0 + idx % nb];
  __syncthreads();
  for (int row = k0 + nb + blockIdx.x * nwarps + warp; row < n; row += gridDim.x * nwarps) {
    float2* a = A + (int64_t)row * n + k0;
    float2 x = lane < nb ? a[lane] : make_float2(0.0f, 0.0f);
    for (int j = 0; j < nb; ++j) {
      float2 xj = make_float2(__shfl_sync(0xffffffffu, x.x, j), __shfl_sync(0xffffffffu, x.y, j));
      xj = cscale(xj, 1.0f / L11[j][j].x);
      if (lane == j) x = xj;
      if (lane > j && lane < nb) x = csub(x, cmul(xj, cconj(L11[lane][j])));
    }
    if (lane < nb) a[lane] = x;
  }
}

// C[i][j] += alpha sum_k A[i][k] op(B)[k][j] over an M x N block, complex64
// row-major with leading dimensions: op(B)[k][j] = conj(B[j][k]) (BH) or
// B[k][j].  32 x 32 output tile per block of 256 threads (4 outputs each),
// K in steps of 16 through shared memory.
template <bool BH>
__global__ __launch_bounds__(256) void cgemm32_kernel(int M, int N, int K, float alpha, const float2* __restrict__ A,
                                                      int lda, const float2* __restrict__ B, int ldb,
                                                      float2* __restrict__ C, int ldc) {
  __shared__ float2 As[32][17], Bs[16][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // ty 0..7 -> rows ty, ty+8, ty+16, ty+24
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  float2 acc[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int idx = threadIdx.x; idx < 32 * 16; idx += 256) {
      const int r = idx / 16, kk = idx % 16;
      As[r][kk] = (i0 + r < M && k0 + kk < K) ? A[(int64_t)(i0 + r) * lda + k0 + kk] : make_float2(0.f, 0.f);
      const int kb = idx / 32, cc = idx % 32;
      float2 bv = make_float2(0.f, 0.f);
      if (k0 + kb < K && j0 + cc < N)
        bv = BH ? cconj(B[(int64_t)(j0 + cc) * ldb + k0 + kb]) : B[(int64_t)(k0 + kb) * ldb + j0 + cc];
      Bs[kb][cc] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const float2 b = Bs[kk][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) cfma(acc[q], As[ty + 8 * q][kk], b);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + ty + 8 * q, j = j0 + tx;
    if (i < M && j < N) C[(int64_t)i * ldc + j] = cadd(C[(int64_t)i * ldc + j], cscale(acc[q], alpha));
  }
}

template <bool BH>
int cgemm32(int M, int N, int K, float alpha, const float2* A, int lda, const float2* B, int ldb, float2* C, int ldc,
            cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0) return CARC_OK;
  cgemm32_kernel<BH><<<dim3((unsigned)ceil_div(N, 32), (unsigned)ceil_div(M, 32)), 256, 0, stream>>>(
      M, N, K, alpha, A, lda, B, ldb, C, ldc);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

__global__ void zero_upper32_kernel(int n, float2* __restrict__ A) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x)
    if ((int)(idx % n) > (int)(idx / n)) A[idx] = make_float2(0.f, 0.f);
}

int potrf32(int n, float2* A, int* status, cudaStream_t stream) {
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), stream));
  for (int k0 = 0; k0 < n; k0 += NB32) {
    const int nb = std::min(NB32, n - k0);
    potrf32_diag_kernel<<<1, dim3(32, 32), 0, stream>>>(n, A, k0, nb, status, 1.0f);
    CARC_CHECK_LAUNCH();
    const int rest = n - k0 - nb;
    if (rest <= 0) break;
    potrf32_panel_kernel<<<(int)std::min<int64_t>(ceil_div(rest, 8), 4 * 152), 256, 0, stream>>>(n, A, k0, nb);
    CARC_CHECK_LAUNCH();
    // A22 -= L21 L21^H (the full square; the strict upper part is zeroed at the end)
    float2* L21 = A + (int64_t)(k0 + nb) * n + k0;
    CARC_RETURN_IF(cgemm32<true>(rest, rest, nb, -1.0f, L21, n, L21, n, A + (int64_t)(k0 + nb) * n + k0 + nb, n, stream));
  }
  zero_upper32_kernel<<<(int)std::min<int64_t>(ceil_div((int64_t)n * n, 256), 1216), 256, 0, stream>>>(n, A);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// X[k0:k0+nb, 0:k0+nb] = L_kk^{-1} X[k0:k0+nb, 0:k0+nb] (the FP64 trsm_diag_kernel in complex64)
__global__ __launch_bounds__(TRSM32_COLS * TRSM32_ROWG) void trsm32_diag_kernel(int n, const float2* __restrict__ Lm,
                                                                                float2* __restrict__ X, int k0, int nb) {
  __shared__ float2 Lk[NB32][NB32 + 1];
  __shared__ float2 Li[NB32][NB32 + 1];
  __shared__ float2 dinv[NB32];
  __shared__ float2 Xs[NB32][TRSM32_COLS + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) Lk[idx / nb][idx % nb] = Lm[(int64_t)(k0 + idx / nb) * n + k0 + idx % nb];
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const float2 d = Lk[i][i];
    const float den = cabs2(d);
    dinv[i] = make_float2(d.x / den, -d.y / den);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    for (int i = 0; i < c; ++i) Li[i][c] = make_float2(0.f, 0.f);
    Li[c][c] = dinv[c];
    for (int i = c + 1; i < nb; ++i) {
      float2 acc = make_float2(0.f, 0.f);
      for (int j = c; j < i; ++j) acc = cadd(acc, cmul(Lk[i][j], Li[j][c]));
      Li[i][c] = cmul(dinv[i], make_float2(-acc.x, -acc.y));
    }
  }
  const int tc = threadIdx.x % TRSM32_COLS, tr = threadIdx.x / TRSM32_COLS;
  const int cols = k0 + nb;
  for (int c0 = blockIdx.x * TRSM32_COLS; c0 < cols; c0 += gridDim.x * TRSM32_COLS) {
    const int col = c0 + tc;
    __syncthreads();
    for (int i = tr; i < nb; i += TRSM32_ROWG) Xs[i][tc] = col < cols ? X[(int64_t)(k0 + i) * n + col] : make_float2(0.f, 0.f);
    __syncthreads();
    if (col < cols)
      for (int i = tr; i < nb; i += TRSM32_ROWG) {
        float2 acc = make_float2(0.f, 0.f);
        for (int j = 0; j <= i; ++j) cfma(acc, Li[i][j], Xs[j][tc]);
        X[(int64_t)(k0 + i) * n + col] = acc;
      }
  }
}

__global__ void set_identity32_kernel(int n, float2* __restrict__ X) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x)
    X[idx] = make_float2((idx / n) == (idx % n) ? 1.f : 0.f, 0.f);
}

int trtri32(int n, const float2* Lm, float2* X, cudaStream_t stream) {
  set_identity32_kernel<<<(int)std::min<int64_t>(ceil_div((int64_t)n * n, 256), 1216), 256, 0, stream>>>(n, X);
  CARC_CHECK_LAUNCH();
  for (int k0 = 0; k0 < n; k0 += NB32) {
    const int nb = std::min(NB32, n - k0);
    // X[k0:k0+nb, 0:k0] -= L[k0:k0+nb, 0:k0] X[0:k0, 0:k0]
    if (k0 > 0) CARC_RETURN_IF(cgemm32<false>(nb, k0, k0, -1.0f, Lm + (int64_t)k0 * n, n, X, n, X + (int64_t)k0 * n, n, stream));
    const int cols = k0 + nb;
    trsm32_diag_kernel<<<(int)std::max<int64_t>(1, ceil_div(cols, TRSM32_COLS)), TRSM32_COLS * TRSM32_ROWG, 0, stream>>>(
        n, Lm, X, k0, nb);
    CARC_CHECK_LAUNCH();
  }
  return CARC_OK;
}

// out[j] = sum_i conj(M[i][j]) v[i] (M n x n complex64, v complex128 or complex64), FP64 accumulation
template <typename V>
__global__ void mhv32_kernel(int n, const float2* __restrict__ M, const V* __restrict__ v, double2* __restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int i = 0; i < n; ++i) acc = cadd(acc, cmulc(to_d2(M[(int64_t)i * n + j]), to_d2(v[i])));
    out[j] = acc;
  }
}

// One block: v (complex64) scaled to unit norm (FP64 sum); *norm_out = |v| when given.
__global__ void normalize32_kernel(int n, float2* __restrict__ v, double* norm_out) {
  __shared__ double part[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += (double)cabs2(v[i]);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    part[0] = t;
    if (norm_out) *norm_out = sqrt(t);
  }
  __syncthreads();
  const float inv = part[0] > 0 ? (float)(1.0 / sqrt(part[0])) : 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = cscale(v[i], inv);
}

// out[i] = sum_r s[r] Q[r][i] (the Ritz vector), complex64
__global__ void ritz32_kernel(int n, int m, const float2* __restrict__ Q, const double* __restrict__ s,
                              float2* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int r = 0; r < m; ++r) acc = cadd(acc, cscale(Q[(int64_t)r * n + i], (float)s[r]));
    out[i] = acc;
  }
}

// ||C q|| for the breakdown scale (one block; C, q complex64)
__global__ void cq_norm32_kernel(int n, const float2* __restrict__ C, const float2* __restrict__ q, double* out) {
  __shared__ double part[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double acc = 0.0;
  for (int r = warp; r < n; r += nw) {
    float2 s = make_float2(0.f, 0.f);
    for (int k = lane; k < n; k += 32) cfma(s, C[(int64_t)r * n + k], q[k]);
    s = warp_sum2(s);
    if (lane == 0) acc += (double)cabs2(s);
  }
  if (lane == 0) part[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += part[w];
    *out = sqrt(t);
  }
}

struct Hegv32Ws {
  float2 *A, *Li, *C32, *Q;
  double2 *Li64, *T1, *C64, *u0, *u;
  double *alpha, *beta, *tri_out, *s, *scal;
  double2 *pscal, *part, *h;
  int *status, *breakdown;
  unsigned int* sync;
  void* tc;
  int64_t tc_bytes;
};

int64_t hegv32_layout(int n, int mk, Hegv32Ws* W, void* base) {
  char* p = static_cast<char*>(base);
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    void* r = p ? p + off : nullptr;
    off += a256(bytes);
    return r;
  };
  const int64_t nn = (int64_t)n * n;
  Hegv32Ws t;
  t.A = (float2*)take(nn * 8);
  t.Li = (float2*)take(nn * 8);
  t.C32 = (float2*)take(nn * 8);
  t.Q = (float2*)take((int64_t)(mk + 1) * n * 8);
  t.Li64 = (double2*)take(nn * 16);
  t.T1 = (double2*)take(nn * 16);
  t.C64 = (double2*)take(nn * 16);
  t.u0 = (double2*)take((int64_t)n * 16);
  t.u = (double2*)take((int64_t)n * 16);
  t.alpha = (double*)take((int64_t)(mk + 1) * 8);
  t.beta = (double*)take((int64_t)(mk + 1) * 8);
  t.tri_out = (double*)take(4 * 8);
  t.s = (double*)take((int64_t)MAXM * 8);
  t.scal = (double*)take(2 * 8);
  t.pscal = (double2*)take((int64_t)LZ_MAX_CTAS * 16);
  t.part = (double2*)take((int64_t)(mk + 1) * LZ_MAX_CTAS * 16);
  t.h = (double2*)take((int64_t)(mk + 1) * 16);
  t.status = (int*)take(16);
  t.breakdown = (int*)take(16);
  t.sync = (unsigned int*)take(16);
  const ZView a = hegv_view(nullptr, n, n, 1, 0), b = hegv_view(nullptr, n, 1, n, 0);
  t.tc_bytes = zgemm_tc_workspace(a, b, HEGV_TC_KSPLIT);
  t.tc = take(t.tc_bytes);
  if (W) *W = t;
  return off;
}

inline int cast_blocks(int64_t count) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(count, 256), 1216)); }

constexpr int HEGV32_UNAVAILABLE = -1;  // cooperative launch refused: the caller takes the FP64 path

int hegv_lowest_single(int n, const void* H, const void* Nm, const void* x0, void* x, double* eigenvalues,
                       int max_krylov, int max_restarts, double tol, int* iterations, void* factors, void* ws,
                       cudaStream_t stream) {
  const int mk = std::max(1, std::min(max_krylov, std::min(n, MAXM)));
  Hegv32Ws W;
  hegv32_layout(n, mk, &W, ws);
  const int64_t nn = (int64_t)n * n;
  {
    PhaseScope ph(PH_HEGV_POTRF, stream);
    c128_to_c64_kernel<<<cast_blocks(nn), 256, 0, stream>>>(nn, static_cast<const double2*>(Nm), W.A);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(potrf32(n, W.A, W.status, stream));
  }
  int hstat = 0;
  CARC_CHECK_CUDA(cudaMemcpyAsync(&hstat, W.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
  if (hstat != CARC_OK) return fail(CARC_NOT_POSDEF, "hegv: the normalization matrix is not positive definite");
  {
    PhaseScope ph(PH_HEGV_TRTRI, stream);
    CARC_RETURN_IF(trtri32(n, W.A, W.Li, stream));
  }
  {
    PhaseScope ph(PH_HEGV_REDUCE, stream);
    c64_to_c128_kernel<<<cast_blocks(nn), 256, 0, stream>>>(nn, W.Li, W.Li64);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(zgemm_tc(hegv_view(W.Li64, n, n, 1, 0), hegv_view(H, n, 1, n, 0), hegv_out(W.T1, n),
                            make_double2(1, 0), 0, HEGV_TC_KSPLIT, W.tc, W.tc_bytes, W.status, stream));
    CARC_RETURN_IF(zgemm_tc(hegv_view(W.T1, n, n, 1, 0), hegv_view(W.Li64, n, n, 1, 1), hegv_out(W.C64, n),
                            make_double2(1, 0), 0, HEGV_TC_KSPLIT, W.tc, W.tc_bytes, W.status, stream));
    c128_to_c64_kernel<<<cast_blocks(nn), 256, 0, stream>>>(nn, W.C64, W.C32);
    CARC_CHECK_LAUNCH();
  }
  // start vector u0 = L^H x0 (or a fixed vector), perturbed as in the FP64 path
  if (x0) {
    mhv32_kernel<double2><<<(int)ceil_div(n, 128), 128, 0, stream>>>(n, W.A, static_cast<const double2*>(x0), W.u0);
    CARC_CHECK_LAUNCH();
  } else {
    CARC_RETURN_IF(fill_launch(n, make_double2(0.0, 0.0), W.u0, stream));
  }
  perturb_start_kernel<<<1, 256, 0, stream>>>(n, W.u0, x0 ? 1e-3 : 1.0);
  CARC_CHECK_LAUNCH();
  c128_to_c64_kernel<<<cast_blocks(n), 256, 0, stream>>>(n, W.u0, W.Q);
  CARC_CHECK_LAUNCH();
  normalize32_kernel<<<1, 1024, 0, stream>>>(n, W.Q, nullptr);
  CARC_CHECK_LAUNCH();
  // Lanczos in complex64 (cooperative chunks of eight iterations)
  static int sm_count = 0;
  if (sm_count == 0) {
    int dev = 0;
    CARC_CHECK_CUDA(cudaGetDevice(&dev));
    CARC_CHECK_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
  }
  const int lz_ctas = (int)std::max<int64_t>(1, std::min<int64_t>({ceil_div(n, 8), (int64_t)sm_count, LZ_MAX_CTAS}));
  const int lz_rpc = (int)ceil_div(n, lz_ctas);
  // FP32 arithmetic: the residual estimate is trusted to about 1e-6
  tol = std::max(tol, 2e-6);
  double lam = 0.0, res = 0.0, lam2 = nan("");
  int total = 0, m = 0;
  bool converged = false;
  {
  PhaseScope ph_lz(PH_HEGV_LANCZOS, stream);
  for (int restart = 0; restart <= max_restarts && !converged; ++restart) {
    CARC_CHECK_CUDA(cudaMemsetAsync(W.breakdown, 0, sizeof(int), stream));
    cq_norm32_kernel<<<1, 1024, 0, stream>>>(n, W.C32, W.Q, W.scal);
    CARC_CHECK_LAUNCH();
    double scale_ref = 1.0;
    CARC_CHECK_CUDA(cudaMemcpyAsync(&scale_ref, W.scal, 8, cudaMemcpyDeviceToHost, stream));
    CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
    scale_ref = std::max(scale_ref, 1e-300);
    m = 0;
    for (int j = 0; j < mk; j += 8) {
      const int j1 = std::min(mk, j + 8);
      LzParams lp;
      lp.n = n;
      lp.j0 = j;
      lp.j1 = j1;
      lp.rpc = lz_rpc;
      lp.C = W.C32;
      lp.Q = W.Q;
      lp.alpha = W.alpha;
      lp.beta = W.beta;
      lp.pscal = W.pscal;
      lp.part = W.part;
      lp.h = W.h;
      lp.scale_ref = scale_ref;
      lp.breakdown_tol = 1e-6;
      lp.breakdown = W.breakdown;
      lp.sync = W.sync;
      lp.abort = reinterpret_cast<int*>(W.sync + 1);
      CARC_CHECK_CUDA(cudaMemsetAsync(W.sync, 0, 8, stream));
      cudaLaunchConfig_t cfg;
      memset(&cfg, 0, sizeof(cfg));
      cfg.gridDim = dim3((unsigned)lz_ctas);
      cfg.blockDim = dim3(LZ_THREADS);
      cfg.dynamicSmemBytes = (size_t)lz_rpc * 8;
      cfg.stream = stream;
      cudaLaunchAttribute la[1];
      la[0].id = cudaLaunchAttributeCooperative;
      la[0].val.cooperative = 1;
      cfg.attrs = la;
      cfg.numAttrs = 1;
      if (cudaLaunchKernelEx(&cfg, lanczos_chunk_kernel<float2>, lp) != cudaSuccess) {
        (void)cudaGetLastError();
        return HEGV32_UNAVAILABLE;
      }
      count_launch();
      total += j1 - j;
      m = j1;
      tridiag_lowest_kernel<<<1, TRI_THREADS, 0, stream>>>(m, W.alpha, W.beta, W.tri_out, W.s);
      CARC_CHECK_LAUNCH();
      double hv[3];
      int bd[2] = {0, 0};
      CARC_CHECK_CUDA(cudaMemcpyAsync(hv, W.tri_out, 24, cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaMemcpyAsync(&bd[0], W.breakdown, sizeof(int), cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaMemcpyAsync(&bd[1], W.sync + 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
      if (bd[1]) return fail(CARC_NOT_CONVERGED, "lanczos: a grid barrier wait timed out");
      lam = hv[0];
      res = hv[1];
      lam2 = hv[2];
      if (bd[0] || res <= tol * std::max(fabs(lam), 1e-300) || m == n) {
        converged = true;
        break;
      }
    }
    // Ritz vector (the restart vector, or the result)
    ritz32_kernel<<<(int)ceil_div(n, 256), 256, 0, stream>>>(n, m, W.Q, W.s, W.Q + (int64_t)mk * n);
    CARC_CHECK_LAUNCH();
    normalize32_kernel<<<1, 1024, 0, stream>>>(n, W.Q + (int64_t)mk * n, nullptr);
    CARC_CHECK_LAUNCH();
    CARC_CHECK_CUDA(cudaMemcpyAsync(W.Q, W.Q + (int64_t)mk * n, (int64_t)n * 8, cudaMemcpyDeviceToDevice, stream));
  }
  }
  c64_to_c128_kernel<<<cast_blocks(n), 256, 0, stream>>>(n, W.Q, W.u);
  CARC_CHECK_LAUNCH();
  // x = L^-H u
  mhv32_kernel<double2><<<(int)ceil_div(n, 128), 128, 0, stream>>>(n, W.Li, W.u, static_cast<double2*>(x));
  CARC_CHECK_LAUNCH();
  if (factors) {
    double2* f = static_cast<double2*>(factors);
    CARC_CHECK_CUDA(cudaMemcpyAsync(f, W.C64, nn * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_CHECK_CUDA(cudaMemcpyAsync(f + nn, W.Li64, nn * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_CHECK_CUDA(cudaMemcpyAsync(f + 2 * nn, W.u, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  }
  int tcstat = 0;
  CARC_CHECK_CUDA(cudaMemcpyAsync(&tcstat, W.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
  if (tcstat != CARC_OK) return fail(CARC_NOT_CONVERGED, "hegv: a tensor-core pipeline wait timed out");
  if (eigenvalues) {
    eigenvalues[0] = lam;
    eigenvalues[1] = lam2;
  }
  if (iterations) *iterations = total;
  if (!converged)
    return fail(CARC_NOT_CONVERGED, "lanczos: residual %.3e after %d iterations (tolerance %.1e)", res, total, tol);
  return CARC_OK;
}

}  // namespace

int64_t hegv_workspace_size(int n, int max_krylov, int flags) {
  int64_t mat = a256((int64_t)n * n * 16);
  carc_contract_desc d = DescBuilder().m(n, n, n).n(n, 1, 1).k(n, 1, n).d;
  int64_t g = std::max<int64_t>(gett_workspace_size(d, 1), 0);
  int64_t tc = 0;
  if (flags & CARC_HEGV_TENSOR_CORE) {
    const ZView a = hegv_view(nullptr, n, n, 1, 0), b = hegv_view(nullptr, n, 1, n, 0);
    tc = zgemm_tc_workspace(a, b, HEGV_TC_KSPLIT);
  }
  int64_t sub = std::max({potrf_workspace_size(n), trtri_workspace_size(n), a256(g), a256(tc),
                          lanczos_workspace_size(n, max_krylov)});
  const int64_t fp64 = 4 * mat + 2 * a256((int64_t)n * 16) + a256(64) + sub;
  if (flags & CARC_HEGV_SINGLE)
    return std::max(fp64, hegv32_layout(n, std::max(1, std::min(max_krylov, std::min(n, MAXM))), nullptr, nullptr));
  return fp64;
}

int hegv_lowest(int n, const void* H, const void* Nm, const void* x0, void* x, double* eigenvalues, int max_krylov,
                int max_restarts, double tol, int flags, int* iterations, void* factors, void* ws, int64_t ws_bytes,
                cudaStream_t stream) {
  if (n < 1) return fail(CARC_BAD_SHAPE, "hegv: n = %d", n);
  if (ws_bytes < hegv_workspace_size(n, max_krylov, flags)) return fail(CARC_BAD_ARG, "hegv: workspace too small");
  if (flags & CARC_HEGV_SINGLE) {
    const int st = hegv_lowest_single(n, H, Nm, x0, x, eigenvalues, max_krylov, max_restarts, tol, iterations, factors,
                                      ws, stream);
    if (st != HEGV32_UNAVAILABLE) return st;
    flags |= CARC_HEGV_TENSOR_CORE;  // not co-resident here: the FP64 path on the same tensor-core pencil
  }
  char* p = static_cast<char*>(ws);
  int64_t mat = a256((int64_t)n * n * 16);
  double2* Lm = (double2*)p;
  double2* Li = (double2*)(p + mat);
  double2* T1 = (double2*)(p + 2 * mat);
  double2* Cm = (double2*)(p + 3 * mat);
  double2* u0 = (double2*)(p + 4 * mat);
  double2* u = (double2*)(p + 4 * mat + a256((int64_t)n * 16));
  int* status = (int*)(p + 4 * mat + 2 * a256((int64_t)n * 16));
  void* sub = p + 4 * mat + 2 * a256((int64_t)n * 16) + a256(64);
  int64_t sub_bytes = ws_bytes - (4 * mat + 2 * a256((int64_t)n * 16) + a256(64));

  {
    PhaseScope ph(PH_HEGV_POTRF, stream);
    CARC_CHECK_CUDA(cudaMemcpyAsync(Lm, Nm, (int64_t)n * n * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_RETURN_IF(potrf(n, Lm, status, sub, sub_bytes, stream));
  }
  int hstat = 0;
  CARC_CHECK_CUDA(cudaMemcpyAsync(&hstat, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
  if (hstat != CARC_OK) return fail(CARC_NOT_POSDEF, "hegv: the normalization matrix is not positive definite");
  {
    PhaseScope ph(PH_HEGV_TRTRI, stream);
    CARC_RETURN_IF(trtri_lower(n, Lm, Li, sub, sub_bytes, stream));
  }
  // T1 = Linv H ; C = T1 Linv^H
  {
    PhaseScope ph(PH_HEGV_REDUCE, stream);
    if (flags & CARC_HEGV_TENSOR_CORE) {
      // T1[m][n] = sum_k Li[m][k] H[k][n];  C[m][n] = sum_k T1[m][k] conj(Li[n][k])
      CARC_RETURN_IF(zgemm_tc(hegv_view(Li, n, n, 1, 0), hegv_view(H, n, 1, n, 0), hegv_out(T1, n), make_double2(1, 0),
                              0, HEGV_TC_KSPLIT, sub, sub_bytes, status, stream));
      CARC_RETURN_IF(zgemm_tc(hegv_view(T1, n, n, 1, 0), hegv_view(Li, n, n, 1, 1), hegv_out(Cm, n),
                              make_double2(1, 0), 0, HEGV_TC_KSPLIT, sub, sub_bytes, status, stream));
    } else {
      carc_contract_desc d = DescBuilder().m(n, n, n).n(n, 1, 1).k(n, 1, n).d;
      const void* pa[1] = {Li};
      const void* pb[1] = {H};
      void* pc[1] = {T1};
      int32_t e[3] = {0, 0, 0};
      CARC_RETURN_IF(gett_launch(d, pa, 1, pb, 1, pc, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
      carc_contract_desc d2 = DescBuilder().m(n, n, n).n(n, n, 1).k(n, 1, 1).d;
      d2.conj_b = 1;
      const void* pa2[1] = {T1};
      const void* pb2[1] = {Li};
      void* pc2[1] = {Cm};
      CARC_RETURN_IF(gett_launch(d2, pa2, 1, pb2, 1, pc2, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
    }
  }
  // start vector u0 = L^H x0 (or a fixed vector)
  if (x0) {
    carc_contract_desc d = DescBuilder().m(n, 1, 1).k(n, n, 1).d;  // u0[j] = sum_i conj(L[i][j]) x0[i]
    d.conj_a = 1;
    const void* pa[1] = {Lm};
    const void* pb[1] = {x0};
    void* pc[1] = {u0};
    int32_t e[3] = {0, 0, 0};
    CARC_RETURN_IF(gett_launch(d, pa, 1, pb, 1, pc, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
  } else {
    CARC_RETURN_IF(fill_launch(n, make_double2(0.0, 0.0), u0, stream));
  }
  // Mix a fixed pseudo-random direction into the start vector: a start that is
  // exactly orthogonal to the ground state (e.g. by a symmetry of the
  // previous center) would otherwise keep Lanczos out of its sector.
  perturb_start_kernel<<<1, 256, 0, stream>>>(n, u0, x0 ? 1e-3 : 1.0);  // one block: reads finish before writes
  CARC_CHECK_LAUNCH();
  int st;
  {
    PhaseScope ph(PH_HEGV_LANCZOS, stream);
    st = lanczos_lowest(n, Cm, u0, u, eigenvalues, max_krylov, max_restarts, tol, iterations, sub, sub_bytes, stream);
  }
  if (st != CARC_OK && st != CARC_NOT_CONVERGED) return st;
  if (flags & CARC_HEGV_TENSOR_CORE) {
    CARC_CHECK_CUDA(cudaMemcpyAsync(&hstat, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
    if (hstat != CARC_OK) return fail(CARC_NOT_CONVERGED, "hegv: a tensor-core pipeline wait timed out");
  }
  // x = Linv^H u : x[j] = sum_i conj(Li[i][j]) u[i]
  {
    carc_contract_desc d = DescBuilder().m(n, 1, 1).k(n, n, 1).d;
    d.conj_a = 1;
    const void* pa[1] = {Li};
    const void* pb[1] = {u};
    void* pc[1] = {x};
    int32_t e[3] = {0, 0, 0};
    CARC_RETURN_IF(gett_launch(d, pa, 1, pb, 1, pc, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
  }
  if (factors) {
    // [C = L^-1 H L^-H | L^-1 | u], for corrections against the same reduced pencil
    double2* f = static_cast<double2*>(factors);
    const int64_t nn = (int64_t)n * n;
    CARC_CHECK_CUDA(cudaMemcpyAsync(f, Cm, nn * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_CHECK_CUDA(cudaMemcpyAsync(f + nn, Li, nn * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_CHECK_CUDA(cudaMemcpyAsync(f + 2 * nn, u, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  }
  return st;
}

// ---------------------------------------------------------------------------
// relaxOver (utils.py:805-878) on the GPU: restarted Krylov / Rayleigh-Ritz on
// M = N^{-1} H with single-pass classical Gram-Schmidt, the k x k projected
// (non-Hermitian) eigenproblem solved on the device, and the reference's
// stopping rule (|change of the lowest Ritz value| <= tol, complete space, or
// the multiplication budget).  M is formed once: M = L^{-H} L^{-1} H.
// ---------------------------------------------------------------------------
namespace {

constexpr int SMALLK = 8;

__device__ double2 cdiv(double2 a, double2 b) {
  double den = cabs2(b);
  return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

__device__ double2 csqrt_d(double2 z) {
  double r = sqrt(sqrt(cabs2(z)));
  double th = 0.5 * atan2(z.y, z.x);
  return make_double2(r * cos(th), r * sin(th));
}

// Eigenvalues of a small complex matrix by shifted QR iterations (full
// matrix, Gram-Schmidt QR, Wilkinson shifts, deflation from the bottom);
// picks the eigenvalue of minimum real part and its eigenvector of the
// original matrix by pivoted elimination.  Single thread.
__global__ void small_eig_min_real_kernel(int k, const double2* __restrict__ A0, double2* __restrict__ lam_out,
                                          double2* __restrict__ vec_out, int* __restrict__ status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double2 A[SMALLK][SMALLK], Q[SMALLK][SMALLK], R[SMALLK][SMALLK];
  double2 ev[SMALLK];
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) A[i][j] = A0[i * k + j];
  double scale = 0.0;
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) scale = fmax(scale, sqrt(cabs2(A[i][j])));
  if (scale == 0.0) scale = 1.0;
  int m = k;
  int guard = 0;
  while (m > 0 && guard < 500 * SMALLK) {
    ++guard;
    if (m == 1) {
      ev[0] = A[0][0];
      m = 0;
      break;
    }
    // deflation test on the last row
    double off = 0.0;
    for (int j = 0; j < m - 1; ++j) off = fmax(off, sqrt(cabs2(A[m - 1][j])));
    const double local = sqrt(cabs2(A[m - 1][m - 1])) + sqrt(cabs2(A[m - 2][m - 2]));
    if (off <= 1e-15 * scale || off <= 2e-15 * local) {
      ev[m - 1] = A[m - 1][m - 1];
      --m;
      continue;
    }
    // Wilkinson shift from the trailing 2x2 block
    double2 a = A[m - 2][m - 2], b = A[m - 2][m - 1], c = A[m - 1][m - 2], d = A[m - 1][m - 1];
    double2 tr = cadd(a, d), det = csub(cmul(a, d), cmul(b, c));
    double2 disc = csqrt_d(csub(cscale(cmul(tr, tr), 0.25), det));
    double2 h = cscale(tr, 0.5);
    double2 l1 = cadd(h, disc), l2 = csub(h, disc);
    double2 mu = cabs2(csub(l1, d)) < cabs2(csub(l2, d)) ? l1 : l2;
    if (guard % 37 == 0) mu = cadd(mu, make_double2(1e-3 * scale, 0.0));  // exceptional shift
    for (int i = 0; i < m; ++i) A[i][i] = csub(A[i][i], mu);
    // QR by modified Gram-Schmidt on the columns of the active block
    for (int j = 0; j < m; ++j) {
      for (int i = 0; i < m; ++i) Q[i][j] = A[i][j];
      for (int p = 0; p < j; ++p) {
        double2 r = make_double2(0.0, 0.0);
        for (int i = 0; i < m; ++i) r = cadd(r, cmulc(Q[i][p], Q[i][j]));
        R[p][j] = r;
        for (int i = 0; i < m; ++i) Q[i][j] = csub(Q[i][j], cmul(r, Q[i][p]));
      }
      double nr = 0.0;
      for (int i = 0; i < m; ++i) nr += cabs2(Q[i][j]);
      nr = sqrt(nr);
      R[j][j] = make_double2(nr, 0.0);
      for (int i = 0; i < m; ++i) Q[i][j] = nr > 0 ? cscale(Q[i][j], 1.0 / nr) : make_double2(i == j ? 1.0 : 0.0, 0.0);
      for (int p = j + 1; p < m; ++p) R[p][j] = make_double2(0.0, 0.0);
    }
    // A = R Q + mu I (the rest of the matrix keeps its already-deflated rows)
    double2 RQ[SMALLK][SMALLK];
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double2 s = make_double2(0.0, 0.0);
        for (int p = i; p < m; ++p) s = cadd(s, cmul(R[i][p], Q[p][j]));
        RQ[i][j] = s;
      }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) A[i][j] = i == j ? cadd(RQ[i][j], mu) : RQ[i][j];
  }
  if (m > 0) {
    // not deflated to rounding level: accept the diagonal when the remaining
    // coupling is small (the Ritz values are then accurate to it), else fail
    double off = 0.0;
    for (int i = 1; i < m; ++i)
      for (int j = 0; j < i; ++j) off = fmax(off, sqrt(cabs2(A[i][j])));
    if (off > 1e-10 * scale) *status = CARC_NOT_CONVERGED;
    for (int i = 0; i < m; ++i) ev[i] = A[i][i];
  }
  int best = 0;
  for (int i = 1; i < k; ++i)
    if (ev[i].x < ev[best].x) best = i;
  const double2 lam = ev[best];
  // eigenvector by inverse iteration on (A0 - mu I), mu = lam + tiny, with
  // partial pivoting: small residual even when Ritz values cluster
  const double2 mu = cadd(lam, make_double2(1e-13 * scale, 1e-13 * scale));
  double2 y[SMALLK];
  for (int i = 0; i < k; ++i) y[i] = make_double2(1.0 / sqrt((double)k), 0.01 * i);
  for (int iter = 0; iter < 4; ++iter) {
    double2 B[SMALLK][SMALLK];
    double2 rhs[SMALLK];
    for (int i = 0; i < k; ++i) {
      rhs[i] = y[i];
      for (int j = 0; j < k; ++j) B[i][j] = i == j ? csub(A0[i * k + j], mu) : A0[i * k + j];
    }
    for (int p = 0; p < k; ++p) {
      int piv = p;
      for (int i = p + 1; i < k; ++i)
        if (cabs2(B[i][p]) > cabs2(B[piv][p])) piv = i;
      if (piv != p) {
        for (int j = 0; j < k; ++j) {
          double2 t = B[p][j];
          B[p][j] = B[piv][j];
          B[piv][j] = t;
        }
        double2 t = rhs[p];
        rhs[p] = rhs[piv];
        rhs[piv] = t;
      }
      if (cabs2(B[p][p]) < 1e-60 * scale * scale) B[p][p] = make_double2(1e-30 * scale, 0.0);
      for (int i = p + 1; i < k; ++i) {
        double2 f = cdiv(B[i][p], B[p][p]);
        for (int j = p; j < k; ++j) B[i][j] = csub(B[i][j], cmul(f, B[p][j]));
        rhs[i] = csub(rhs[i], cmul(f, rhs[p]));
      }
    }
    for (int i = k - 1; i >= 0; --i) {
      double2 s2 = rhs[i];
      for (int j = i + 1; j < k; ++j) s2 = csub(s2, cmul(B[i][j], y[j]));
      y[i] = cdiv(s2, B[i][i]);
    }
    double mx = 0.0;
    for (int i = 0; i < k; ++i) mx = fmax(mx, sqrt(cabs2(y[i])));
    if (!(mx > 0.0) || isinf(mx) || isnan(mx)) {
      for (int i = 0; i < k; ++i) y[i] = make_double2(i == best ? 1.0 : 0.0, 0.0);
      break;
    }
    double nr = 0.0;
    for (int i = 0; i < k; ++i) {
      y[i] = cscale(y[i], 1.0 / mx);
      nr += cabs2(y[i]);
    }
    nr = sqrt(nr);
    for (int i = 0; i < k; ++i) y[i] = cscale(y[i], 1.0 / nr);
  }
  // LAPACK's convention for eigenvectors of a general matrix (unit norm, the
  // first component of largest modulus real and positive), which the
  // reference's projected solve inherits: the Ritz vector's phase then
  // follows the current iterate, so repeated solves of a converged state
  // return the same vector
  {
    int imax = 0;
    double amax = -1.0;
    for (int i = 0; i < k; ++i) {
      const double a = cabs2(y[i]);
      if (a > amax) {
        amax = a;
        imax = i;
      }
    }
    if (amax > 0.0) {
      const double m = sqrt(amax);
      const double2 ph = make_double2(y[imax].x / m, -y[imax].y / m);  // conj(y_max) / |y_max|
      for (int i = 0; i < k; ++i) y[i] = cmul(y[i], ph);
      y[imax].y = 0.0;
    }
  }
  for (int i = 0; i < k; ++i) vec_out[i] = y[i];
  *lam_out = lam;
}

struct RelaxWs {
  double2 *M, *K, *MK, *h, *small, *lam, *vec, *x, *tmp, *scal;
  int* status;
  void* dot_ws;
  int64_t dot_ws_bytes;
};

int64_t relax_layout(int n, int k, RelaxWs* R, void* base) {
  char* p = static_cast<char*>(base);
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    void* r = p ? p + off : nullptr;
    off += a256(bytes);
    return r;
  };
  RelaxWs t;
  t.M = (double2*)take((int64_t)n * n * 16);
  t.K = (double2*)take((int64_t)k * n * 16);
  t.MK = (double2*)take((int64_t)k * n * 16);
  t.h = (double2*)take((int64_t)k * 16);
  t.small = (double2*)take((int64_t)k * k * 16);
  t.lam = (double2*)take(16);
  t.vec = (double2*)take((int64_t)k * 16);
  t.x = (double2*)take((int64_t)n * 16);
  t.tmp = (double2*)take((int64_t)n * 16);
  t.scal = (double2*)take(4 * 16);
  t.status = (int*)take(16);
  t.dot_ws_bytes = dot_workspace_size(n);
  t.dot_ws = take(t.dot_ws_bytes);
  if (R) *R = t;
  return off;
}

__global__ void copy_column_kernel(int k, const double2* __restrict__ h, double2* __restrict__ small, int col) {
  for (int i = threadIdx.x; i < k; i += blockDim.x) small[i * k + col] = h[i];
}

}  // namespace

int64_t relax_workspace_size(int n, int k) {
  int64_t mat = a256((int64_t)n * n * 16);
  carc_contract_desc d = DescBuilder().m(n, n, n).n(n, 1, 1).k(n, 1, n).d;
  int64_t g = std::max<int64_t>(gett_workspace_size(d, 1), 0);
  return relax_layout(n, k, nullptr, nullptr) + 3 * mat + a256(64) +
         std::max({potrf_workspace_size(n), trtri_workspace_size(n), a256(g)});
}

int relax_over(int n, const void* Hv, const void* Nv, const void* x0, void* x_out, int k, int max_mults, double tol,
               double2* eigenvalue, int* mults_out, double2* values_out, void* ws, int64_t ws_bytes,
               cudaStream_t stream) {
  if (n < 1 || k < 1 || k > SMALLK) return fail(CARC_BAD_ARG, "relaxOver: n=%d, krylov dimension %d (1..%d)", n, k, SMALLK);
  if (ws_bytes < relax_workspace_size(n, k)) return fail(CARC_BAD_ARG, "relaxOver: workspace too small");
  RelaxWs W;
  int64_t used = relax_layout(n, k, &W, ws);
  char* p = static_cast<char*>(ws) + used;
  int64_t mat = a256((int64_t)n * n * 16);
  double2* Lm = (double2*)p;
  double2* Li = (double2*)(p + mat);
  double2* T1 = (double2*)(p + 2 * mat);
  int* st = (int*)(p + 3 * mat);
  void* sub = p + 3 * mat + a256(64);
  int64_t sub_bytes = ws_bytes - used - 3 * mat - a256(64);
  const int eb = blocks_for(n);
  const int gb = blocks_for((int64_t)n * 32);
  int32_t e[3] = {0, 0, 0};
  // M = N^{-1} H  (or H when N is absent)
  if (Nv) {
    CARC_CHECK_CUDA(cudaMemcpyAsync(Lm, Nv, (int64_t)n * n * 16, cudaMemcpyDeviceToDevice, stream));
    CARC_RETURN_IF(potrf(n, Lm, st, sub, sub_bytes, stream));
    int hs = 0;
    CARC_CHECK_CUDA(cudaMemcpyAsync(&hs, st, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
    if (hs != CARC_OK) return fail(CARC_NOT_POSDEF, "relaxOver: the normalization matrix is not positive definite");
    CARC_RETURN_IF(trtri_lower(n, Lm, Li, sub, sub_bytes, stream));
    carc_contract_desc d1 = DescBuilder().m(n, n, n).n(n, 1, 1).k(n, 1, n).d;  // T1 = Li H
    const void* a1[1] = {Li};
    const void* b1[1] = {Hv};
    void* c1[1] = {T1};
    CARC_RETURN_IF(gett_launch(d1, a1, 1, b1, 1, c1, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
    carc_contract_desc d2 = DescBuilder().m(n, 1, n).n(n, 1, 1).k(n, n, n).d;  // M[i][j] = sum_r conj(Li[r][i]) T1[r][j]
    d2.conj_a = 1;
    const void* a2[1] = {Li};
    const void* b2[1] = {T1};
    void* c2[1] = {W.M};
    CARC_RETURN_IF(gett_launch(d2, a2, 1, b2, 1, c2, 1, e, 1, make_double2(1, 0), 0, sub, sub_bytes, stream));
  } else {
    CARC_CHECK_CUDA(cudaMemcpyAsync(W.M, Hv, (int64_t)n * n * 16, cudaMemcpyDeviceToDevice, stream));
  }
  CARC_CHECK_CUDA(cudaMemsetAsync(W.status, 0, sizeof(int), stream));
  // x = x0 / |x0| ; initial value x^H M x
  CARC_CHECK_CUDA(cudaMemcpyAsync(W.x, x0, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_RETURN_IF(dot_launch(n, W.x, W.x, 1, W.scal, W.dot_ws, W.dot_ws_bytes, stream));
  scale_by_norm_kernel<<<eb, 256, 0, stream>>>(n, W.scal, W.x);
  CARC_CHECK_LAUNCH();
  gemv_kernel<<<gb, 256, 0, stream>>>(n, W.M, W.x, W.tmp);
  CARC_CHECK_LAUNCH();
  CARC_RETURN_IF(dot_launch(n, W.x, W.tmp, 1, W.scal + 1, W.dot_ws, W.dot_ws_bytes, stream));
  double2 initial_value;
  CARC_CHECK_CUDA(cudaMemcpyAsync(&initial_value, W.scal + 1, 16, cudaMemcpyDeviceToHost, stream));
  int mults = 0;
  bool have_last = false;
  double2 last = make_double2(0, 0);
  bool complete = (k == n);
  const int max_restarts = 100000;
  for (int restart = 0; restart < max_restarts; ++restart) {
    int kk = k;
    CARC_CHECK_CUDA(cudaMemcpyAsync(W.K, W.x, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
    for (int i = 0; i < k; ++i) {
      gemv_kernel<<<gb, 256, 0, stream>>>(n, W.M, W.K + (int64_t)i * n, W.MK + (int64_t)i * n);
      CARC_CHECK_LAUNCH();
      if (i < k - 1) {
        // K[i+1] = MK[i] - (K[:i+1]^H MK[i]) K[:i+1]   (single classical Gram-Schmidt pass, utils.py:852)
        proj_kernel<<<blocks_for((int64_t)(i + 1) * 32), 256, 0, stream>>>(n, i + 1, W.K, W.MK + (int64_t)i * n, W.h);
        CARC_CHECK_LAUNCH();
        CARC_CHECK_CUDA(cudaMemcpyAsync(W.K + (int64_t)(i + 1) * n, W.MK + (int64_t)i * n, (int64_t)n * 16,
                                        cudaMemcpyDeviceToDevice, stream));
        combine_kernel<<<comb_blocks(n), COMB_I * COMB_R, 0, stream>>>(n, i + 1, W.K, W.h, -1.0, W.K + (int64_t)(i + 1) * n, 0);
        CARC_CHECK_LAUNCH();
        double2* kn = W.K + (int64_t)(i + 1) * n;
        CARC_RETURN_IF(dot_launch(n, kn, kn, 1, W.scal + 2, W.dot_ws, W.dot_ws_bytes, stream));
        CARC_RETURN_IF(dot_launch(n, W.MK + (int64_t)i * n, W.MK + (int64_t)i * n, 1, W.scal + 3, W.dot_ws,
                                  W.dot_ws_bytes, stream));
        double2 nr2[2];
        CARC_CHECK_CUDA(cudaMemcpyAsync(nr2, W.scal + 2, 32, cudaMemcpyDeviceToHost, stream));
        CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
        if (nr2[0].x < 0.5 * nr2[1].x) {
          // The subtraction cancelled more than half of M K[i] (the reference's own
          // comment at utils.py:847-850 names the instability near an
          // eigenvector): a second Gram-Schmidt pass restores orthogonality, so
          // the projected matrix stays a Rayleigh-Ritz matrix.
          proj_kernel<<<blocks_for((int64_t)(i + 1) * 32), 256, 0, stream>>>(n, i + 1, W.K, kn, W.h);
          CARC_CHECK_LAUNCH();
          combine_kernel<<<comb_blocks(n), COMB_I * COMB_R, 0, stream>>>(n, i + 1, W.K, W.h, -1.0, kn, 0);
          CARC_CHECK_LAUNCH();
          CARC_RETURN_IF(dot_launch(n, kn, kn, 1, W.scal + 2, W.dot_ws, W.dot_ws_bytes, stream));
          CARC_CHECK_CUDA(cudaMemcpyAsync(nr2, W.scal + 2, 16, cudaMemcpyDeviceToHost, stream));
          CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
        }
        if (sqrt(std::max(nr2[0].x, 0.0)) <= 1e-14) {
          complete = true;
          kk = i + 1;
          break;
        }
        scale_by_norm_kernel<<<eb, 256, 0, stream>>>(n, W.scal + 2, W.K + (int64_t)(i + 1) * n);
        CARC_CHECK_LAUNCH();
      }
    }
    mults += k;
    // small[a][b] = K[a]^H MK[b]
    for (int b = 0; b < kk; ++b) {
      proj_kernel<<<blocks_for((int64_t)kk * 32), 256, 0, stream>>>(n, kk, W.K, W.MK + (int64_t)b * n, W.h);
      CARC_CHECK_LAUNCH();
      copy_column_kernel<<<1, 32, 0, stream>>>(kk, W.h, W.small, b);
      CARC_CHECK_LAUNCH();
    }
    small_eig_min_real_kernel<<<1, 1, 0, stream>>>(kk, W.small, W.lam, W.vec, W.status);
    CARC_CHECK_LAUNCH();
    double2 lam;
    int sst = 0;
    CARC_CHECK_CUDA(cudaMemcpyAsync(&lam, W.lam, 16, cudaMemcpyDeviceToHost, stream));
    CARC_CHECK_CUDA(cudaMemcpyAsync(&sst, W.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
    if (sst != 0) return fail(CARC_NOT_CONVERGED, "relaxOver: projected eigenproblem did not converge");
    // x = vec . K, normalized
    combine_kernel<<<comb_blocks(n), COMB_I * COMB_R, 0, stream>>>(n, kk, W.K, W.vec, 1.0, W.x, 1);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(dot_launch(n, W.x, W.x, 1, W.scal, W.dot_ws, W.dot_ws_bytes, stream));
    scale_by_norm_kernel<<<eb, 256, 0, stream>>>(n, W.scal, W.x);
    CARC_CHECK_LAUNCH();
    const bool changed_little = have_last && sqrt(cabs2(csub(last, lam))) <= tol;
    if (complete || changed_little || (max_mults > 0 && mults >= max_mults)) {
      gemv_kernel<<<gb, 256, 0, stream>>>(n, W.M, W.x, W.tmp);
      CARC_CHECK_LAUNCH();
      CARC_RETURN_IF(dot_launch(n, W.x, W.tmp, 1, W.scal + 1, W.dot_ws, W.dot_ws_bytes, stream));
      double2 final_value;
      CARC_CHECK_CUDA(cudaMemcpyAsync(&final_value, W.scal + 1, 16, cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaMemcpyAsync(x_out, W.x, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
      CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
      if (eigenvalue) *eigenvalue = lam;
      if (mults_out) *mults_out = mults;
      if (values_out) {
        values_out[0] = initial_value;
        values_out[1] = final_value;
      }
      // RelaxFailed test of utils.py:871-872 (real part of the complex ratio, as numpy compares)
      double2 diff = csub(final_value, initial_value);
      double den = sqrt(cabs2(final_value)) + sqrt(cabs2(initial_value));
      if (den > 0 && diff.x / den > 1 + 1e-7) return fail(CARC_RELAX_FAILED, "relaxOver: value rose");
      return CARC_OK;
    }
    last = lam;
    have_last = true;
  }
  return fail(CARC_NOT_CONVERGED, "relaxOver: restart budget spent");
}


// ---------------------------------------------------------------------------
// MINRES for the projected shifted system  P (C - shift) P z = P b,
// P = I - u u^H (u unit), C dense Hermitian n x n: the correction equation of
// a Newton step on an approximate pencil (mixed-precision center solve).
// The Paige-Saunders recurrence scalars stay on the device (double-buffered
// state, recomputed by every thread of the update kernel); the host checks
// convergence every MINRES_CHECK iterations.
// ---------------------------------------------------------------------------
namespace {

struct MinresState {
  double beta, oldb, dbar, epsln, phibar, cs, sn;
  double rtol_abs;  // stop when phibar <= rtol_abs
  int done;
  int pad;
};

constexpr int MINRES_CHECK = 8;

__global__ void minres_scale_kernel(int n, const MinresState* __restrict__ st, const double2* __restrict__ y,
                                    double2* __restrict__ v) {
  if (st->done) return;
  const double inv = 1.0 / st->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = cscale(y[i], inv);
}

// y = t - shift v - (u^H t) u - [itn > 0] (beta / oldb) r1
__global__ void minres_combo1_kernel(int n, int itn, const MinresState* __restrict__ st, double shift,
                                     const double2* __restrict__ t, const double2* __restrict__ v,
                                     const double2* __restrict__ u, const double2* __restrict__ ut,
                                     const double2* __restrict__ r1, double2* __restrict__ y) {
  if (st->done) return;
  const double2 c = *ut;
  const double f = itn > 0 ? st->beta / st->oldb : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 a = csub(csub(t[i], cscale(v[i], shift)), cmul(c, u[i]));
    if (itn > 0) a = csub(a, cscale(r1[i], f));
    y[i] = a;
  }
}

// out = y - (alfa / beta) r2
__global__ void minres_combo2_kernel(int n, const MinresState* __restrict__ st, const double2* __restrict__ alfa,
                                     const double2* __restrict__ y, const double2* __restrict__ r2,
                                     double2* __restrict__ out) {
  if (st->done) return;
  const double f = alfa->x / st->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = csub(y[i], cscale(r2[i], f));
}

// recurrence step; w_new = (v - oldeps wa - delta wb) / gamma written over wa
// (wa: direction of two iterations ago, wb: of the last one); x += phi w_new
__global__ void minres_update_kernel(int n, const MinresState* __restrict__ sin, MinresState* __restrict__ sout,
                                     const double2* __restrict__ alfa_c, const double2* __restrict__ beta2_c,
                                     const double2* __restrict__ v, double2* __restrict__ wa,
                                     const double2* __restrict__ wb, double2* __restrict__ x) {
  MinresState s = *sin;
  if (s.done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *sout = s;
    return;
  }
  const double alfa = alfa_c->x;
  const double beta = sqrt(fmax(beta2_c->x, 0.0));
  const double oldeps = s.epsln;
  const double delta = s.cs * s.dbar + s.sn * alfa;
  const double gbar = s.sn * s.dbar - s.cs * alfa;
  const double epsln = s.sn * beta;
  const double dbar = -s.cs * beta;
  const double gamma = fmax(hypot(gbar, beta), 1e-300);
  const double cs = gbar / gamma, sn = beta / gamma;
  const double phi = cs * s.phibar;
  const double phibar = sn * s.phibar;
  const double ig = 1.0 / gamma;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 wn = cscale(csub(csub(v[i], cscale(wa[i], oldeps)), cscale(wb[i], delta)), ig);
    wa[i] = wn;
    x[i] = cadd(x[i], cscale(wn, phi));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    MinresState o = s;
    o.oldb = s.beta;
    o.beta = beta;
    o.epsln = epsln;
    o.dbar = dbar;
    o.cs = cs;
    o.sn = sn;
    o.phibar = phibar;
    o.done = (beta == 0.0 || phibar <= s.rtol_abs) ? 1 : 0;
    *sout = o;
  }
}

__global__ void minres_init_kernel(MinresState* st, const double2* __restrict__ b2, double rtol) {
  const double beta1 = sqrt(fmax(b2->x, 0.0));
  MinresState s;
  s.beta = beta1;
  s.oldb = 0.0;
  s.dbar = 0.0;
  s.epsln = 0.0;
  s.phibar = beta1;
  s.cs = -1.0;
  s.sn = 0.0;
  s.rtol_abs = rtol * beta1;
  s.done = beta1 == 0.0 ? 1 : 0;
  s.pad = 0;
  st[0] = s;
  st[1] = s;
}

// b -= (u^H b) u
__global__ void project_out_kernel(int n, const double2* __restrict__ u, const double2* __restrict__ ub,
                                   double2* __restrict__ b) {
  const double2 c = *ub;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = csub(b[i], cmul(c, u[i]));
}

int64_t minres_ws_layout(int n, double2** vecs, MinresState** st, double2** scal, void** dot_ws, int64_t* dot_bytes,
                         void* base) {
  char* p = static_cast<char*>(base);
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    void* r = p ? p + off : nullptr;
    off += a256(bytes);
    return r;
  };
  for (int i = 0; i < 8; ++i) {
    void* q = take((int64_t)n * 16);
    if (vecs) vecs[i] = static_cast<double2*>(q);
  }
  void* s = take(2 * sizeof(MinresState));
  void* c = take(4 * 16);
  const int64_t db = dot_workspace_size(n);
  void* d = take(db);
  if (st) *st = static_cast<MinresState*>(s);
  if (scal) *scal = static_cast<double2*>(c);
  if (dot_ws) *dot_ws = d;
  if (dot_bytes) *dot_bytes = db;
  return off;
}

}  // namespace

int64_t minres_workspace_size(int n) { return minres_ws_layout(n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr); }

int minres_projected(int n, const void* Cv, const void* uv, double shift, const void* bv, void* zv, int maxit,
                     double rtol, int* iterations, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  if (n < 1) return fail(CARC_BAD_SHAPE, "minres: n = %d", n);
  if (ws_bytes < minres_workspace_size(n)) return fail(CARC_BAD_ARG, "minres: workspace too small");
  double2* V[8];
  MinresState* st;
  double2* scal;
  void* dws;
  int64_t dbytes;
  minres_ws_layout(n, V, &st, &scal, &dws, &dbytes, ws);
  const double2* C = static_cast<const double2*>(Cv);
  const double2* u = static_cast<const double2*>(uv);
  double2* z = static_cast<double2*>(zv);
  // y: scratch; r1, r2: the two latest Lanczos residuals; wa, wb: the
  // search directions of two iterations ago and of the last one
  double2 *y = V[0], *r1 = V[1], *r2 = V[2], *v = V[3], *t = V[4], *wa = V[5], *wb = V[6];
  const int eb = blocks_for(n);
  const int gb = blocks_for((int64_t)n * 32);
  // r1 = r2 = P b; z = wa = wb = 0
  CARC_CHECK_CUDA(cudaMemcpyAsync(r2, bv, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_RETURN_IF(dot_launch(n, u, r2, 1, scal, dws, dbytes, stream));
  project_out_kernel<<<eb, 256, 0, stream>>>(n, u, scal, r2);
  CARC_CHECK_LAUNCH();
  CARC_CHECK_CUDA(cudaMemcpyAsync(r1, r2, (int64_t)n * 16, cudaMemcpyDeviceToDevice, stream));
  CARC_RETURN_IF(fill_launch(n, make_double2(0, 0), z, stream));
  CARC_RETURN_IF(fill_launch(n, make_double2(0, 0), wa, stream));
  CARC_RETURN_IF(fill_launch(n, make_double2(0, 0), wb, stream));
  CARC_RETURN_IF(dot_launch(n, r2, r2, 1, scal + 1, dws, dbytes, stream));
  minres_init_kernel<<<1, 1, 0, stream>>>(st, scal + 1, rtol);
  CARC_CHECK_LAUNCH();
  int itn = 0;
  for (; itn < maxit; ++itn) {
    MinresState* sin = st + (itn & 1);
    MinresState* sout = st + ((itn + 1) & 1);
    minres_scale_kernel<<<eb, 256, 0, stream>>>(n, sin, r2, v);
    CARC_CHECK_LAUNCH();
    gemv_kernel<<<gb, 256, 0, stream>>>(n, C, v, t);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(dot_launch(n, u, t, 1, scal + 2, dws, dbytes, stream));
    minres_combo1_kernel<<<eb, 256, 0, stream>>>(n, itn, sin, shift, t, v, u, scal + 2, r1, y);
    CARC_CHECK_LAUNCH();
    CARC_RETURN_IF(dot_launch(n, v, y, 1, scal + 3, dws, dbytes, stream));
    // new residual y - (alfa/beta) r2 into r1's buffer, then r1 <- r2, r2 <- new
    minres_combo2_kernel<<<eb, 256, 0, stream>>>(n, sin, scal + 3, y, r2, r1);
    CARC_CHECK_LAUNCH();
    std::swap(r1, r2);
    CARC_RETURN_IF(dot_launch(n, r2, r2, 1, scal + 1, dws, dbytes, stream));
    // new direction (v - oldeps wa - delta wb) / gamma into wa's buffer, then swap
    minres_update_kernel<<<eb, 256, 0, stream>>>(n, sin, sout, scal + 3, scal + 1, v, wa, wb, z);
    CARC_CHECK_LAUNCH();
    std::swap(wa, wb);
    if ((itn + 1) % MINRES_CHECK == 0 || itn + 1 == maxit) {
      MinresState h;
      CARC_CHECK_CUDA(cudaMemcpyAsync(&h, sout, sizeof(h), cudaMemcpyDeviceToHost, stream));
      CARC_CHECK_CUDA(cudaStreamSynchronize(stream));
      if (h.done) {
        ++itn;
        break;
      }
    }
  }
  if (iterations) *iterations = itn;
  return CARC_OK;
}

}  // namespace carc
