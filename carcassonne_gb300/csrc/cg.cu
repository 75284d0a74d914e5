// Conjugate gradients on a small Hermitian positive semi-definite system
// G x = c, the whole iteration in ONE thread block (no host round trip per
// iteration).
//
// Used by the product compressor (compression.py:26-46 of the reference
// solves the same normal equations A^H A x = A^H b by GMRES): G is at most
// CARC_CG_MAX_N square, read from global memory (it stays in L2) once per
// iteration; x, r, p and G p live in shared memory.  Inner products are
// summed in a fixed order (per-thread strided partial sums, then warp
// shuffles, then the warps in index order), so results are deterministic.
// The iteration stops when |r|^2 <= tol^2 |c|^2, when p^H G p <= 0 (a
// consistent PSD system has converged in the range of G), or after max_iter
// iterations; status[0] receives the iteration count, status[1] 1 if the
// iteration stopped by the residual test, by p^H G p <= 0 or because c = 0,
// and 0 if it ran out of iterations, and res[0] the final relative residual.
// Every loop is bounded.
#include "common.cuh"

namespace carc {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

// fixed-order block sum of a per-thread double2 partial; every thread
// returns the total
__device__ double2 block_sum2(double2 v, double2* red) {
  v = warp_sum2(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double2 t = make_double2(0.0, 0.0);
#pragma unroll
  for (int w = 0; w < kWarps; ++w) t = cadd(t, red[w]);
  return t;
}

__global__ void __launch_bounds__(kThreads) zcg_kernel(int n, const double2* __restrict__ G,
                                                        const double2* __restrict__ c, double2* __restrict__ x_out,
                                                        double tol, int max_iter, int32_t* status, double* res) {
  extern __shared__ double2 sm[];
  double2* x = sm;
  double2* r = sm + n;
  double2* p = sm + 2 * n;
  double2* gp = sm + 3 * n;
  __shared__ double2 red[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  double2 part = make_double2(0.0, 0.0);
  for (int i = tid; i < n; i += kThreads) {
    const double2 ci = c[i];
    x[i] = make_double2(0.0, 0.0);
    r[i] = ci;
    p[i] = ci;
    part.x += cabs2(ci);
  }
  const double c2 = block_sum2(part, red).x;
  double rr = c2;
  int it = 0, converged = 0;
  if (c2 == 0.0) converged = 1;
  const double thresh = tol * tol * c2;
  while (!converged && it < max_iter) {
    __syncthreads();
    // G p: one warp per row, lanes striding the row (coalesced)
    for (int i = warp; i < n; i += kWarps) {
      const double2* gi = G + (int64_t)i * n;
      double2 s = make_double2(0.0, 0.0);
      for (int j = lane; j < n; j += 32) cfma(s, gi[j], p[j]);
      s = warp_sum2(s);
      if (lane == 0) gp[i] = s;
    }
    __syncthreads();
    part = make_double2(0.0, 0.0);
    for (int i = tid; i < n; i += kThreads) {
      const double2 t = cmulc(p[i], gp[i]);
      part.x += t.x;
    }
    const double pgp = block_sum2(part, red).x;
    if (!(pgp > 0.0)) {  // no descent direction left: x solves the consistent system on the range of G
      converged = 1;
      break;
    }
    const double alpha = rr / pgp;
    part = make_double2(0.0, 0.0);
    for (int i = tid; i < n; i += kThreads) {
      x[i] = cadd(x[i], cscale(p[i], alpha));
      const double2 ri = csub(r[i], cscale(gp[i], alpha));
      r[i] = ri;
      part.x += cabs2(ri);
    }
    const double rr_new = block_sum2(part, red).x;
    ++it;
    if (rr_new <= thresh) {
      rr = rr_new;
      converged = 1;
      break;
    }
    const double beta = rr_new / rr;
    for (int i = tid; i < n; i += kThreads) p[i] = cadd(r[i], cscale(p[i], beta));
    rr = rr_new;
  }
  __syncthreads();
  for (int i = tid; i < n; i += kThreads) x_out[i] = x[i];
  if (tid == 0) {
    status[0] = it;
    status[1] = converged;
    res[0] = c2 > 0.0 ? sqrt(rr / c2) : 0.0;
  }
}

}  // namespace

int zcg_hpsd(int n, const void* G, const void* c, void* x, double tol, int max_iter, int32_t* status, double* res,
             cudaStream_t stream) {
  if (n < 1 || n > CARC_CG_MAX_N) return fail(CARC_TOO_LARGE, "carc_zcg_hpsd: n = %d outside [1, %d]", n, CARC_CG_MAX_N);
  if (max_iter < 0) return fail(CARC_BAD_ARG, "carc_zcg_hpsd: max_iter %d", max_iter);
  const size_t smem = (size_t)4 * n * sizeof(double2);
  CARC_CHECK_CUDA(cudaFuncSetAttribute(zcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)((size_t)4 * CARC_CG_MAX_N * sizeof(double2))));
  zcg_kernel<<<1, kThreads, smem, stream>>>(n, static_cast<const double2*>(G), static_cast<const double2*>(c),
                                            static_cast<double2*>(x), tol, max_iter, status, res);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace carc

using namespace carc;

extern "C" int carc_zcg_hpsd(int32_t n, const void* G, const void* c, void* x, double tol, int32_t max_iter,
                             void* status, void* residual, void* stream) {
  if (!G || !c || !x || !status || !residual) return fail(CARC_BAD_ARG, "carc_zcg_hpsd: NULL argument");
  return zcg_hpsd(n, G, c, x, tol, max_iter, static_cast<int32_t*>(status), static_cast<double*>(residual),
                  as_stream(stream));
}
