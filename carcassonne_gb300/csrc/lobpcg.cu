// Batched block eigensolver over many independent center-site problems.
//
// Each problem b is a Hermitian-definite pencil H x = l N x of dimension n_b
// (the center's entries) whose lowest eigenpair is wanted, the unit of work
// of minimizeExpectation / relaxOver (system/_2d.py:489-497,
// utils.py:805-878).  The solver is LOBPCG with a block of m vectors and the
// search space S = [X; R; P] of k = 3m rows (X the Ritz block, R its
// residuals, P the previous update direction); it needs only H S and N S
// products, which the caller computes with the tensor-core matvec, so N is
// never inverted or formed.  One iteration over the whole batch is:
//
//   gram     GH = conj(S) HS^T, GN = conj(S) NS^T (k x k, FP64), ragged work
//            items of ITEM entries, partial sums reduced per problem in item
//            order (deterministic, independent of the batch's composition);
//   rr       GN -> unit-diagonal GN' = D GN D, GN' = V diag(w) V^H (batched
//            Jacobi), T = D V diag(s) with s_j = w_j^-1/2 on the kept
//            directions (w_j > drop max w) and 0 on the others,
//            G = T^H GH T (dropped directions moved far above the spectrum),
//            G = Y diag(theta) Y^H (batched Jacobi), C = T Y[:, :m];
//   update   X' = S^T C, P' = [R; P]^T C[m:], the same for HS and NS, and
//            R' = HX' - NX' diag(theta) with the relative residual norms
//            |R'_j| / (|HX'_j| + |theta_j| |NX'_j|).
//
// Layout: problem b's k x n_b blocks S, HS, NS are row-major at element
// offset off[b] of three pools (rows 0..m-1 X, m..2m-1 R, 2m..3m-1 P).  Work
// item w covers entries [item_start[w], item_start[w] + ITEM) of problem
// item_problem[w]; problem b owns items first[b] .. first[b+1]-1.  Problems
// with active[b] == 0 are left untouched by every kernel.
#include "common.cuh"

namespace carc {

namespace {

constexpr int LB_THREADS = 256;
constexpr int LB_ITEM = CARC_LOBPCG_ITEM;
constexpr int LB_SUB = 32;                      // entries per shared-memory stage of the Gram kernel
constexpr int LB_MAXM = CARC_LOBPCG_MAX_M;
constexpr int LB_MAXK = 3 * LB_MAXM;
constexpr int LB_OUT_PER_THREAD = (2 * LB_MAXK * LB_MAXK + LB_THREADS - 1) / LB_THREADS;

static_assert(LB_ITEM == LB_THREADS, "the update kernel maps one entry to one thread");

__device__ __forceinline__ double2 d2zero() { return make_double2(0.0, 0.0); }

// -- block inner products ---------------------------------------------------------
// out1 = conj(A rows a0..a0+ka-1) . (B1 rows b0..b0+kb-1)^T and out2 likewise
// with B2 (when given), per problem; partial sums per work item, reduced per
// problem in item order.
__global__ void __launch_bounds__(LB_THREADS) lobpcg_inner_kernel(int a0, int ka, int b0, int kb,
                                                                  const int32_t* __restrict__ ip,
                                                                  const int32_t* __restrict__ is,
                                                                  const int64_t* __restrict__ off,
                                                                  const int32_t* __restrict__ n,
                                                                  const int32_t* __restrict__ active,
                                                                  const double2* __restrict__ A,
                                                                  const double2* __restrict__ B1,
                                                                  const double2* __restrict__ B2,
                                                                  double2* __restrict__ part) {
  __shared__ double2 sA[LB_SUB][LB_MAXK];
  __shared__ double2 sB1[LB_SUB][LB_MAXK];
  __shared__ double2 sB2[LB_SUB][LB_MAXK];
  const int w = blockIdx.x, b = ip[w];
  if (!active[b]) return;
  const int nb = n[b], one = ka * kb, outs = (B2 ? 2 : 1) * one;
  const int e_begin = is[w], e_end = min(nb, e_begin + LB_ITEM);
  const int64_t base = off[b];
  double2 acc[LB_OUT_PER_THREAD];
#pragma unroll
  for (int r = 0; r < LB_OUT_PER_THREAD; ++r) acc[r] = d2zero();
  for (int e0 = e_begin; e0 < e_end; e0 += LB_SUB) {
    const int cnt = min(LB_SUB, e_end - e0);
    __syncthreads();
    for (int t = threadIdx.x; t < ka * LB_SUB; t += LB_THREADS) {
      const int i = t / LB_SUB, e = t - i * LB_SUB;
      sA[e][i] = e < cnt ? A[base + (int64_t)(a0 + i) * nb + e0 + e] : d2zero();
    }
    for (int t = threadIdx.x; t < kb * LB_SUB; t += LB_THREADS) {
      const int i = t / LB_SUB, e = t - i * LB_SUB;
      const int64_t idx = base + (int64_t)(b0 + i) * nb + e0 + e;
      sB1[e][i] = e < cnt ? B1[idx] : d2zero();
      if (B2) sB2[e][i] = e < cnt ? B2[idx] : d2zero();
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < LB_OUT_PER_THREAD; ++r) {
      const int o = threadIdx.x + r * LB_THREADS;
      if (o < outs) {
        const bool second = o >= one;
        const int q = second ? o - one : o, i = q / kb, j = q - i * kb;
        double2 s = acc[r];
        if (second) {
          for (int e = 0; e < LB_SUB; ++e) s = cadd(s, cmulc(sA[e][i], sB2[e][j]));
        } else {
          for (int e = 0; e < LB_SUB; ++e) s = cadd(s, cmulc(sA[e][i], sB1[e][j]));
        }
        acc[r] = s;
      }
    }
  }
  double2* P = part + (int64_t)w * outs;
#pragma unroll
  for (int r = 0; r < LB_OUT_PER_THREAD; ++r) {
    const int o = threadIdx.x + r * LB_THREADS;
    if (o < outs) P[o] = acc[r];
  }
}

__global__ void __launch_bounds__(LB_THREADS) lobpcg_inner_reduce_kernel(int one, int nout,
                                                                         const int32_t* __restrict__ first,
                                                                         const int32_t* __restrict__ active,
                                                                         const double2* __restrict__ part,
                                                                         double2* __restrict__ out1,
                                                                         double2* __restrict__ out2) {
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int outs = nout * one;
  for (int o = threadIdx.x; o < outs; o += LB_THREADS) {
    double2 s = d2zero();
    for (int w = first[b]; w < first[b + 1]; ++w) s = cadd(s, part[(int64_t)w * outs + o]);
    if (o < one)
      out1[(int64_t)b * one + o] = s;
    else
      out2[(int64_t)b * one + o - one] = s;
  }
}

// -- orthonormalisation of the residual and direction blocks ------------------------
// Q (3m x 2m) = [X; R; P]^H N [R, P] per problem.  With X N-orthonormal, the
// block Z (R or P) minus X A_Z (A_Z = X^H N Z) has the N-Gram matrix
// B_Z - A_Z^H A_Z (B_Z = Z^H N Z).  Ms receives the unit-diagonal Hermitian
// matrices D_Z (B_Z - A_Z^H A_Z) D_Z for Z = R, P (two m x m per problem) for
// the batched eigensolver; a column whose remaining N-norm^2 is at most floor
// times its original gets D = 0.
__global__ void lobpcg_orth_prepare_kernel(int m, double floor_, const int32_t* __restrict__ active,
                                           const double2* __restrict__ Q_all, double2* __restrict__ Ms_all,
                                           double* __restrict__ d_all) {
  __shared__ double2 Bp[2][LB_MAXM * LB_MAXM];
  __shared__ double d[2][LB_MAXM];
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int mm = m * m, ld = 2 * m;
  const double2* Q = Q_all + (int64_t)b * 3 * m * ld;
  for (int t = threadIdx.x; t < 2 * mm; t += blockDim.x) {
    const int z = t / mm, q = t - z * mm, i = q / m, j = q - i * m;
    // A_Z[l][j] = Q[l][z m + j], B_Z[i][j] = Q[(z + 1) m + i][z m + j]
    double2 acc = Q[((z + 1) * m + i) * ld + z * m + j];
    for (int l = 0; l < m; ++l) acc = csub(acc, cmulc(Q[l * ld + z * m + i], Q[l * ld + z * m + j]));
    Bp[z][q] = acc;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * m; t += blockDim.x) {
    const int z = t / m, j = t - z * m;
    const double r = Bp[z][j * m + j].x, r0 = Q[((z + 1) * m + j) * ld + z * m + j].x;
    d[z][j] = (r0 > 0.0 && r > floor_ * r0) ? 1.0 / sqrt(r) : 0.0;
    d_all[(int64_t)b * 2 * m + t] = d[z][j];
  }
  __syncthreads();
  double2* Ms = Ms_all + (int64_t)b * 2 * mm;
  for (int t = threadIdx.x; t < 2 * mm; t += blockDim.x) {
    const int z = t / mm, q = t - z * mm, i = q / m, j = q - i * m;
    const double2 u = Bp[z][i * m + j], v = Bp[z][j * m + i];
    double2 h = make_double2(0.5 * (u.x + v.x), 0.5 * (u.y - v.y));
    if (i == j) h.y = 0.0;
    Ms[t] = cscale(h, d[z][i] * d[z][j]);
  }
}

// From the eigenpairs (W, V) of the two matrices: for Z = R, P,
// M_Z1 = D_Z V_Z diag(s_Z), M_Z2 = -A_Z M_Z1, s = W^-1/2 on the kept
// directions (W_j > drop max W) and 0 on the others (all of P's when
// restart_p: P restarts from zero); M (4 m x m per problem: M_R1, M_R2, M_P1,
// M_P2).
__global__ void lobpcg_orth_finish_kernel(int m, double drop, int restart_p, const int32_t* __restrict__ active,
                                          const double2* __restrict__ Q_all, const double* __restrict__ d_all,
                                          const double* __restrict__ W_all, const double2* __restrict__ V_all,
                                          double2* __restrict__ M_all) {
  __shared__ double s[2][LB_MAXM];
  __shared__ double2 M1[2][LB_MAXM * LB_MAXM];
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int mm = m * m, ld = 2 * m;
  const double* W = W_all + (int64_t)b * 2 * m;
  const double2* V = V_all + (int64_t)b * 2 * mm;
  const double* d = d_all + (int64_t)b * 2 * m;
  if (threadIdx.x < 2) {
    const int z = threadIdx.x;
    double wmax = 0.0;
    for (int j = 0; j < m; ++j) wmax = fmax(wmax, W[z * m + j]);
    for (int j = 0; j < m; ++j) {
      const double wj = W[z * m + j];
      s[z][j] = (wj > drop * wmax && wj > 0.0 && !(z == 1 && restart_p)) ? 1.0 / sqrt(wj) : 0.0;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * mm; t += blockDim.x) {
    const int z = t / mm, q = t - z * mm, l = q / m, j = q - l * m;
    M1[z][q] = cscale(V[t], d[z * m + l] * s[z][j]);
  }
  __syncthreads();
  const double2* Q = Q_all + (int64_t)b * 3 * m * ld;
  double2* M = M_all + (int64_t)b * 4 * mm;
  for (int t = threadIdx.x; t < 2 * mm; t += blockDim.x) {
    const int z = t / mm, q = t - z * mm, l = q / m, j = q - l * m;
    double2 acc = d2zero();
    for (int r = 0; r < m; ++r) cfma(acc, Q[l * ld + z * m + r], M1[z][r * m + j]);
    M[2 * z * mm + q] = M1[z][q];
    M[(2 * z + 1) * mm + q] = make_double2(-acc.x, -acc.y);
  }
}

// In place, per entry: R <- R M_R1 + X M_R2 in S; P <- P M_P1 + X M_P2 in S,
// HS and NS (the caller recomputes H R and N R from the new R).
template <int M>
__global__ void __launch_bounds__(LB_THREADS) lobpcg_orth_apply_kernel(
    const int32_t* __restrict__ ip, const int32_t* __restrict__ is, const int64_t* __restrict__ off,
    const int32_t* __restrict__ n, const int32_t* __restrict__ active, const double2* __restrict__ M_all,
    double2* __restrict__ S, double2* __restrict__ HS, double2* __restrict__ NS) {
  __shared__ double2 Ms[4][LB_MAXM][LB_MAXM];
  const int w = blockIdx.x, b = ip[w];
  if (!active[b]) return;
  const int nb = n[b];
  const int e = is[w] + threadIdx.x;
  for (int t = threadIdx.x; t < 4 * M * M; t += LB_THREADS) {
    const int which = t / (M * M), q = t - which * M * M;
    Ms[which][q / M][q % M] = M_all[(int64_t)b * 4 * M * M + t];
  }
  __syncthreads();
  if (e >= nb) return;
  const int64_t base = off[b] + e;
  double2 r[M];
  double2* pools[3] = {S, HS, NS};
#pragma unroll
  for (int pi = 0; pi < 3; ++pi) {
    double2* Q = pools[pi];
#pragma unroll
    for (int z = 0; z < 2; ++z) {
      if (z == 0 && pi > 0) continue;  // R rows only in S
#pragma unroll
      for (int j = 0; j < M; ++j) r[j] = d2zero();
#pragma unroll 2
      for (int l = 0; l < M; ++l) {
        const double2 xv = Q[base + (int64_t)l * nb], zv = Q[base + (int64_t)((z + 1) * M + l) * nb];
#pragma unroll
        for (int j = 0; j < M; ++j) {
          cfma(r[j], Ms[2 * z][l][j], zv);
          cfma(r[j], Ms[2 * z + 1][l][j], xv);
        }
      }
#pragma unroll
      for (int j = 0; j < M; ++j) Q[base + (int64_t)((z + 1) * M + j) * nb] = r[j];
    }
  }
}

// -- Rayleigh-Ritz on the k x k pencils ------------------------------------------
__global__ void __launch_bounds__(LB_THREADS) lobpcg_rr_scale_kernel(int k, const int32_t* __restrict__ active,
                                                                     const double2* __restrict__ GN,
                                                                     double2* __restrict__ GNs,
                                                                     double* __restrict__ dscale) {
  __shared__ double d[LB_MAXK];
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int kk = k * k;
  const double2* g = GN + (int64_t)b * kk;
  for (int j = threadIdx.x; j < k; j += LB_THREADS) {
    const double a = g[j * k + j].x;
    d[j] = a > 0.0 ? 1.0 / sqrt(a) : 0.0;
    dscale[(int64_t)b * k + j] = d[j];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kk; t += LB_THREADS) {
    const int i = t / k, j = t - i * k;
    const double2 a = g[i * k + j], c = g[j * k + i];
    double2 h = make_double2(0.5 * (a.x + c.x), 0.5 * (a.y - c.y));
    if (i == j) h.y = 0.0;
    GNs[(int64_t)b * kk + t] = cscale(h, d[i] * d[j]);
  }
}

__global__ void __launch_bounds__(LB_THREADS) lobpcg_rr_reduce_kernel(int k, const int32_t* __restrict__ active,
                                                                      const double2* __restrict__ GH_all,
                                                                      const double* __restrict__ d_all,
                                                                      const double* __restrict__ W_all,
                                                                      const double2* __restrict__ V_all, double drop,
                                                                      double2* __restrict__ T_all,
                                                                      double2* __restrict__ G_all,
                                                                      int32_t* __restrict__ rank) {
  __shared__ double2 GH[LB_MAXK * LB_MAXK];
  __shared__ double2 T[LB_MAXK * LB_MAXK];
  __shared__ double2 U[LB_MAXK * LB_MAXK];
  __shared__ double s[LB_MAXK];
  __shared__ double d[LB_MAXK];
  __shared__ double big;
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int kk = k * k;
  const double2* GHb = GH_all + (int64_t)b * kk;
  const double2* Vb = V_all + (int64_t)b * kk;
  const double* Wb = W_all + (int64_t)b * k;
  for (int j = threadIdx.x; j < k; j += LB_THREADS) d[j] = d_all[(int64_t)b * k + j];
  if (threadIdx.x == 0) {
    double wmax = 0.0;
    for (int j = 0; j < k; ++j) wmax = fmax(wmax, Wb[j]);
    int r = 0;
    for (int j = 0; j < k; ++j) {
      const bool keep = Wb[j] > drop * wmax && Wb[j] > 0.0;
      s[j] = keep ? 1.0 / sqrt(Wb[j]) : 0.0;
      r += keep;
    }
    rank[b] = r;
  }
  __syncthreads();
  // Hermitian part of D GH D (rounding and the split-precision products break
  // the symmetry of S^H H S), and T' = V diag(s) in the scaled basis
  for (int t = threadIdx.x; t < kk; t += LB_THREADS) {
    const int i = t / k, j = t - i * k;
    const double2 a = GHb[i * k + j], c = GHb[j * k + i];
    double2 h = make_double2(0.5 * (a.x + c.x), 0.5 * (a.y - c.y));
    if (i == j) h.y = 0.0;
    GH[t] = cscale(h, d[i] * d[j]);
    T[t] = cscale(Vb[t], s[j]);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kk; t += LB_THREADS) {  // U = GH' T'
    const int i = t / k, j = t - i * k;
    double2 acc = d2zero();
    for (int l = 0; l < k; ++l) cfma(acc, GH[i * k + l], T[l * k + j]);
    U[t] = acc;
  }
  __syncthreads();
  double2* Gb = G_all + (int64_t)b * kk;
  for (int t = threadIdx.x; t < kk; t += LB_THREADS) {  // G = T'^H U, upper triangle mirrored
    const int i = t / k, j = t - i * k;
    if (i > j) continue;
    double2 acc = d2zero();
    for (int l = 0; l < k; ++l) acc = cadd(acc, cmulc(T[l * k + i], U[l * k + j]));
    if (i == j) acc.y = 0.0;
    Gb[i * k + j] = acc;
    Gb[j * k + i] = cconj(acc);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double f = 0.0;
    for (int t = 0; t < kk; ++t) f += cabs2(Gb[t]);
    big = 10.0 * sqrt(f) + 1.0;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += LB_THREADS)
    if (s[j] == 0.0) Gb[j * k + j] = make_double2(big, 0.0);
  double2* Tb = T_all + (int64_t)b * kk;  // coefficients in the unscaled basis: T = D T'
  for (int t = threadIdx.x; t < kk; t += LB_THREADS) Tb[t] = cscale(T[t], d[t / k]);
}

__global__ void __launch_bounds__(LB_THREADS) lobpcg_rr_combine_kernel(int k, int m,
                                                                       const int32_t* __restrict__ active,
                                                                       const double2* __restrict__ T_all,
                                                                       const double2* __restrict__ Y_all,
                                                                       double2* __restrict__ C_all) {
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int kk = k * k;
  const double2* T = T_all + (int64_t)b * kk;
  const double2* Y = Y_all + (int64_t)b * kk;
  double2* C = C_all + (int64_t)b * k * m;
  for (int t = threadIdx.x; t < k * m; t += LB_THREADS) {
    const int i = t / m, j = t - i * m;
    double2 acc = d2zero();
    for (int l = 0; l < k; ++l) cfma(acc, T[i * k + l], Y[l * k + j]);
    C[t] = acc;
  }
}

// -- block update and residuals -------------------------------------------------
template <int M>
__device__ __forceinline__ void combine_entry(const double2* __restrict__ Q, double2* __restrict__ Qn, int64_t base,
                                              int nb, bool valid, const double2 (*Cs)[LB_MAXM], double2* x) {
  constexpr int K = 3 * M;
  double2 p[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    x[j] = d2zero();
    p[j] = d2zero();
  }
  // the coefficients stream from shared memory (the l loops are not fully
  // unrolled, so C is not held in registers across the three pools)
#pragma unroll 2
  for (int l = 0; l < M; ++l) {
    const double2 q = valid ? Q[base + (int64_t)l * nb] : d2zero();
#pragma unroll
    for (int j = 0; j < M; ++j) cfma(x[j], Cs[l][j], q);
  }
#pragma unroll 2
  for (int l = M; l < K; ++l) {
    const double2 q = valid ? Q[base + (int64_t)l * nb] : d2zero();
#pragma unroll
    for (int j = 0; j < M; ++j) cfma(p[j], Cs[l][j], q);
  }
#pragma unroll
  for (int j = 0; j < M; ++j) {
    x[j] = cadd(x[j], p[j]);
    if (valid) {
      Qn[base + (int64_t)j * nb] = x[j];
      Qn[base + (int64_t)(2 * M + j) * nb] = p[j];
    }
  }
}

template <int M>
__global__ void __launch_bounds__(LB_THREADS) lobpcg_update_kernel(
    const int32_t* __restrict__ ip, const int32_t* __restrict__ is, const int64_t* __restrict__ off,
    const int32_t* __restrict__ n, const int32_t* __restrict__ active, const double2* __restrict__ C_all,
    const double* __restrict__ theta_all, const double2* __restrict__ S, const double2* __restrict__ HS,
    const double2* __restrict__ NS, double2* __restrict__ S2, double2* __restrict__ HS2, double2* __restrict__ NS2,
    double* __restrict__ part) {
  constexpr int K = 3 * M;
  __shared__ double2 Cs[LB_MAXK][LB_MAXM];
  __shared__ double th[LB_MAXM];
  __shared__ double red[LB_THREADS / 32][3 * LB_MAXM];
  const int w = blockIdx.x, b = ip[w];
  if (!active[b]) return;
  const int nb = n[b];
  const int e = is[w] + threadIdx.x;
  const bool valid = e < nb;
  for (int t = threadIdx.x; t < K * M; t += LB_THREADS) Cs[t / M][t % M] = C_all[(int64_t)b * K * M + t];
  if (threadIdx.x < M) th[threadIdx.x] = theta_all[(int64_t)b * K + threadIdx.x];
  __syncthreads();
  const int64_t base = off[b] + e;
  {
    double2 t[M];
    combine_entry<M>(S, S2, base, nb, valid, Cs, t);
    combine_entry<M>(HS, HS2, base, nb, valid, Cs, t);
  }
  double2 nx[M];
  combine_entry<M>(NS, NS2, base, nb, valid, Cs, nx);
  // residuals from this thread's own H X' entries, and their block sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    const double2 hx = valid ? HS2[base + (int64_t)j * nb] : d2zero();
    const double2 r = csub(hx, cscale(nx[j], th[j]));
    if (valid) S2[base + (int64_t)(M + j) * nb] = r;
    const double r2 = warp_sum(valid ? cabs2(r) : 0.0);
    const double h2 = warp_sum(valid ? cabs2(hx) : 0.0);
    const double n2 = warp_sum(valid ? cabs2(nx[j]) : 0.0);
    if (lane == 0) {
      red[warp][j] = r2;
      red[warp][M + j] = h2;
      red[warp][2 * M + j] = n2;
    }
  }
  __syncthreads();
  if (threadIdx.x < 3 * M) {
    double s = 0.0;
    for (int wp = 0; wp < LB_THREADS / 32; ++wp) s += red[wp][threadIdx.x];
    part[(int64_t)w * 3 * M + threadIdx.x] = s;
  }
}

__global__ void lobpcg_residual_kernel(int batch, int m, const int32_t* __restrict__ first,
                                       const int32_t* __restrict__ active, const double* __restrict__ part,
                                       const double* __restrict__ theta_all, double* __restrict__ res) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= batch * m) return;
  const int b = t / m, j = t - b * m;
  if (!active[b]) return;
  double r2 = 0.0, h2 = 0.0, n2 = 0.0;
  for (int w = first[b]; w < first[b + 1]; ++w) {
    r2 += part[(int64_t)w * 3 * m + j];
    h2 += part[(int64_t)w * 3 * m + m + j];
    n2 += part[(int64_t)w * 3 * m + 2 * m + j];
  }
  const double th = theta_all[(int64_t)b * 3 * m + j];
  const double den = sqrt(h2) + fabs(th) * sqrt(n2);
  res[t] = den > 0.0 ? sqrt(r2) / den : (r2 > 0.0 ? 1.0 : 0.0);
}

inline int64_t a256(int64_t v) { return (v + 255) / 256 * 256; }

int check_common(int32_t batch, int32_t m) {
  if (batch < 1) return fail(CARC_BAD_ARG, "lobpcg: batch %d", batch);
  if (m != 1 && m != 2 && m != 4 && m != 8) return fail(CARC_BAD_ARG, "lobpcg: block size %d (1, 2, 4 or 8)", m);
  return CARC_OK;
}

}  // namespace

}  // namespace carc

using namespace carc;

extern "C" int64_t carc_lobpcg_workspace_size(int32_t items, int32_t m) {
  if (items < 1 || m < 1 || m > CARC_LOBPCG_MAX_M) return -1;
  const int64_t k = 3 * m;
  return a256(items * 2 * k * k * (int64_t)sizeof(double2)) + a256(items * 3 * m * (int64_t)sizeof(double));
}

extern "C" int carc_lobpcg_inner(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem,
                                 const int32_t* item_start, const int32_t* first, const int64_t* off,
                                 const int32_t* n, const int32_t* active, const void* A, int32_t a0, int32_t ka,
                                 const void* B1, const void* B2, int32_t b0, int32_t kb, void* out1, void* out2,
                                 void* workspace, int64_t workspace_bytes, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!item_problem || !item_start || !first || !off || !n || !active || !A || !B1 || !out1 || !workspace ||
      (B2 && !out2))
    return fail(CARC_BAD_ARG, "carc_lobpcg_inner: NULL argument");
  const int k = 3 * m;
  if (ka < 1 || kb < 1 || a0 < 0 || b0 < 0 || a0 + ka > k || b0 + kb > k)
    return fail(CARC_BAD_ARG, "carc_lobpcg_inner: rows [%d, %d) x [%d, %d) outside the %d rows of a problem", a0,
                a0 + ka, b0, b0 + kb, k);
  const int64_t need = carc_lobpcg_workspace_size(items, m);
  if (need < 0 || workspace_bytes < need)
    return fail(CARC_BAD_ARG, "carc_lobpcg_inner: workspace %lld bytes, need %lld", (long long)workspace_bytes,
                (long long)need);
  cudaStream_t s = as_stream(stream);
  double2* part = static_cast<double2*>(workspace);
  lobpcg_inner_kernel<<<items, LB_THREADS, 0, s>>>(a0, ka, b0, kb, item_problem, item_start, off, n, active,
                                                    static_cast<const double2*>(A), static_cast<const double2*>(B1),
                                                    static_cast<const double2*>(B2), part);
  CARC_CHECK_LAUNCH();
  lobpcg_inner_reduce_kernel<<<batch, LB_THREADS, 0, s>>>(ka * kb, B2 ? 2 : 1, first, active, part,
                                                           static_cast<double2*>(out1), static_cast<double2*>(out2));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_orth_prepare(int32_t batch, int32_t m, const int32_t* active, const void* Q,
                                        double floor_, void* Ms, void* dscale, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!active || !Q || !Ms || !dscale) return fail(CARC_BAD_ARG, "carc_lobpcg_orth_prepare: NULL argument");
  if (!(floor_ >= 0.0 && floor_ < 1.0)) return fail(CARC_BAD_ARG, "carc_lobpcg_orth_prepare: floor %g", floor_);
  lobpcg_orth_prepare_kernel<<<batch, 128, 0, as_stream(stream)>>>(m, floor_, active, static_cast<const double2*>(Q),
                                                                    static_cast<double2*>(Ms),
                                                                    static_cast<double*>(dscale));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_orth_finish(int32_t batch, int32_t m, const int32_t* active, const void* Q,
                                       const void* dscale, const void* W, const void* V, double drop,
                                       int32_t restart_p, void* M, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!active || !Q || !dscale || !W || !V || !M) return fail(CARC_BAD_ARG, "carc_lobpcg_orth_finish: NULL argument");
  if (!(drop >= 0.0 && drop < 1.0)) return fail(CARC_BAD_ARG, "carc_lobpcg_orth_finish: drop %g", drop);
  lobpcg_orth_finish_kernel<<<batch, 128, 0, as_stream(stream)>>>(
      m, drop, restart_p, active, static_cast<const double2*>(Q), static_cast<const double*>(dscale),
      static_cast<const double*>(W), static_cast<const double2*>(V), static_cast<double2*>(M));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_orth_apply(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem,
                                      const int32_t* item_start, const int32_t* first, const int64_t* off,
                                      const int32_t* n, const int32_t* active, const void* M, void* S, void* HS,
                                      void* NS, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!item_problem || !item_start || !first || !off || !n || !active || !M || !S || !HS || !NS)
    return fail(CARC_BAD_ARG, "carc_lobpcg_orth_apply: NULL argument");
  if (items < 1) return fail(CARC_BAD_ARG, "carc_lobpcg_orth_apply: %d work items", items);
  cudaStream_t s = as_stream(stream);
  const double2* Mc = static_cast<const double2*>(M);
  double2 *Sc = static_cast<double2*>(S), *Hc = static_cast<double2*>(HS), *Nc = static_cast<double2*>(NS);
  switch (m) {
    case 1:
      lobpcg_orth_apply_kernel<1><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Mc, Sc, Hc, Nc);
      break;
    case 2:
      lobpcg_orth_apply_kernel<2><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Mc, Sc, Hc, Nc);
      break;
    case 4:
      lobpcg_orth_apply_kernel<4><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Mc, Sc, Hc, Nc);
      break;
    default:
      lobpcg_orth_apply_kernel<8><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Mc, Sc, Hc, Nc);
      break;
  }
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_rr_scale(int32_t batch, int32_t m, const int32_t* active, const void* GN, void* GNs,
                                    void* dscale, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!active || !GN || !GNs || !dscale) return fail(CARC_BAD_ARG, "carc_lobpcg_rr_scale: NULL argument");
  lobpcg_rr_scale_kernel<<<batch, LB_THREADS, 0, as_stream(stream)>>>(
      3 * m, active, static_cast<const double2*>(GN), static_cast<double2*>(GNs), static_cast<double*>(dscale));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_rr_reduce(int32_t batch, int32_t m, const int32_t* active, const void* GH,
                                     const void* dscale, const void* W, const void* V, double drop, void* T, void* G,
                                     int32_t* rank, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!active || !GH || !dscale || !W || !V || !T || !G || !rank)
    return fail(CARC_BAD_ARG, "carc_lobpcg_rr_reduce: NULL argument");
  if (!(drop >= 0.0 && drop < 1.0)) return fail(CARC_BAD_ARG, "carc_lobpcg_rr_reduce: drop %g", drop);
  lobpcg_rr_reduce_kernel<<<batch, LB_THREADS, 0, as_stream(stream)>>>(
      3 * m, active, static_cast<const double2*>(GH), static_cast<const double*>(dscale),
      static_cast<const double*>(W), static_cast<const double2*>(V), drop, static_cast<double2*>(T),
      static_cast<double2*>(G), rank);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_rr_combine(int32_t batch, int32_t m, const int32_t* active, const void* T, const void* Y,
                                      void* C, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!active || !T || !Y || !C) return fail(CARC_BAD_ARG, "carc_lobpcg_rr_combine: NULL argument");
  lobpcg_rr_combine_kernel<<<batch, LB_THREADS, 0, as_stream(stream)>>>(
      3 * m, m, active, static_cast<const double2*>(T), static_cast<const double2*>(Y), static_cast<double2*>(C));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

extern "C" int carc_lobpcg_update(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem,
                                  const int32_t* item_start, const int32_t* first, const int64_t* off,
                                  const int32_t* n, const int32_t* active, const void* C, const void* theta,
                                  const void* S, const void* HS, const void* NS, void* S2, void* HS2, void* NS2,
                                  void* res, void* workspace, int64_t workspace_bytes, void* stream) {
  CARC_RETURN_IF(check_common(batch, m));
  if (!item_problem || !item_start || !first || !off || !n || !active || !C || !theta || !S || !HS || !NS || !S2 ||
      !HS2 || !NS2 || !res || !workspace)
    return fail(CARC_BAD_ARG, "carc_lobpcg_update: NULL argument");
  const int64_t need = carc_lobpcg_workspace_size(items, m);
  if (need < 0 || workspace_bytes < need)
    return fail(CARC_BAD_ARG, "carc_lobpcg_update: workspace %lld bytes, need %lld", (long long)workspace_bytes,
                (long long)need);
  const int k = 3 * m;
  double* part = reinterpret_cast<double*>(static_cast<char*>(workspace) +
                                           a256(items * 2 * (int64_t)k * k * (int64_t)sizeof(double2)));
  cudaStream_t s = as_stream(stream);
  const double2* Cc = static_cast<const double2*>(C);
  const double* th = static_cast<const double*>(theta);
  const double2 *Sc = static_cast<const double2*>(S), *Hc = static_cast<const double2*>(HS),
                *Nc = static_cast<const double2*>(NS);
  double2 *S2c = static_cast<double2*>(S2), *H2c = static_cast<double2*>(HS2), *N2c = static_cast<double2*>(NS2);
  switch (m) {
    case 1:
      lobpcg_update_kernel<1><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Cc, th, Sc, Hc,
                                                            Nc, S2c, H2c, N2c, part);
      break;
    case 2:
      lobpcg_update_kernel<2><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Cc, th, Sc, Hc,
                                                            Nc, S2c, H2c, N2c, part);
      break;
    case 4:
      lobpcg_update_kernel<4><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Cc, th, Sc, Hc,
                                                            Nc, S2c, H2c, N2c, part);
      break;
    default:
      lobpcg_update_kernel<8><<<items, LB_THREADS, 0, s>>>(item_problem, item_start, off, n, active, Cc, th, Sc, Hc,
                                                            Nc, S2c, H2c, N2c, part);
      break;
  }
  CARC_CHECK_LAUNCH();
  lobpcg_residual_kernel<<<(batch * m + 127) / 128, 128, 0, s>>>(batch, m, first, active, part, th,
                                                                  static_cast<double*>(res));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}
