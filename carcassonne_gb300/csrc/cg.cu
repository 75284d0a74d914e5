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

#include <algorithm>
#include <cstring>

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

// ---------------------------------------------------------------------------
// The same iteration spread over a cooperative grid: CTA b owns rows
// [b rpc, (b + 1) rpc) of x, r, p and G p (in shared memory); the direction p
// is published in global memory for every CTA's rows of G p.  Per iteration
// three grid barriers: after the partial sums of p^H G p, after those of
// |r|^2, and after the new p.  Every CTA adds the per-CTA partials in CTA
// order, so all take the same decisions and the result is deterministic.
// FP64 on one SM is the single-block kernel's limit (its G p is n^2 complex
// multiply-adds per iteration); this form divides it by the grid size.
// ---------------------------------------------------------------------------
constexpr int kGridThreads = 256;
constexpr int kGridWarps = kGridThreads / 32;

struct CgGridParams {
  int n, rpc, max_iter;
  const double2* G;
  const double2* c;
  double2* x_out;
  double2* p_glob;      // n
  double* part;         // [2][gridDim.x]
  unsigned int* sync;   // [0] arrivals; [1] abort word
  double tol;
  int32_t* status;
  double* res;
};

__device__ bool cg_grid_sync(unsigned int* ctr, unsigned int target, int* abort) {
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

// fixed-order block sum of one double per thread; every thread returns it
__device__ double block_sum_d(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < kGridWarps; ++w) t += red[w];
  return t;
}

// the per-CTA partials of one slot, added in CTA order by thread 0 (which
// acquired them at the grid barrier) and broadcast: every CTA the same value
__device__ double grid_total(const double* part, double* red) {
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) t += *reinterpret_cast<const volatile double*>(part + b);
    red[kGridWarps] = t;
  }
  __syncthreads();
  return red[kGridWarps];
}

__global__ void __launch_bounds__(kGridThreads) zcg_grid_kernel(const __grid_constant__ CgGridParams p) {
  extern __shared__ double2 gsm[];
  const int rpc = p.rpc, n = p.n;
  double2* x = gsm;
  double2* r = gsm + rpc;
  double2* pl = gsm + 2 * rpc;
  double2* gp = gsm + 3 * rpc;
  double2* xb = gsm + 4 * rpc;  // the iterate with the smallest residual so far
  __shared__ double red[kGridWarps + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = (int)gridDim.x, b = (int)blockIdx.x;
  const int r0 = b * rpc, nr = max(0, min(rpc, n - r0));
  double* part0 = p.part;
  double* part1 = p.part + G;
  int* abort = reinterpret_cast<int*>(p.sync + 1);
  unsigned int bar = 0;
  auto gsync = [&]() { return cg_grid_sync(p.sync, ++bar * (unsigned)G, abort); };

  double v = 0.0;
  for (int i = tid; i < nr; i += kGridThreads) {
    const double2 ci = p.c[r0 + i];
    x[i] = make_double2(0.0, 0.0);
    xb[i] = make_double2(0.0, 0.0);
    r[i] = ci;
    pl[i] = ci;
    p.p_glob[r0 + i] = ci;
    v += cabs2(ci);
  }
  v = block_sum_d(v, red);
  if (tid == 0) part1[b] = v;
  bool ok = gsync();
  const double c2 = ok ? grid_total(part1, red) : 0.0;
  double rr = c2, best = c2, last = c2;  // last: the recursive |r|^2 of the current x
  int it = 0, converged = (c2 == 0.0) ? 1 : 0;
  const double thresh = p.tol * p.tol * c2;
  while (ok && !converged && it < p.max_iter) {
    // G p on this CTA's rows: one warp per row, lanes striding the row
    for (int i = warp; i < nr; i += kGridWarps) {
      const double2* gi = p.G + (int64_t)(r0 + i) * n;
      double2 s = make_double2(0.0, 0.0);
      for (int j = lane; j < n; j += 32) cfma(s, gi[j], __ldcg(p.p_glob + j));
      s = warp_sum2(s);
      if (lane == 0) gp[i] = s;
    }
    __syncthreads();
    v = 0.0;
    for (int i = tid; i < nr; i += kGridThreads) v += cmulc(pl[i], gp[i]).x;
    v = block_sum_d(v, red);
    if (tid == 0) part0[b] = v;
    if (!(ok = gsync())) break;
    const double pgp = grid_total(part0, red);
    if (!(pgp > 0.0)) {  // no descent direction left: x solves the consistent system on the range of G
      converged = 1;
      break;
    }
    const double alpha = rr / pgp;
    v = 0.0;
    for (int i = tid; i < nr; i += kGridThreads) {
      x[i] = cadd(x[i], cscale(pl[i], alpha));
      const double2 ri = csub(r[i], cscale(gp[i], alpha));
      r[i] = ri;
      v += cabs2(ri);
    }
    v = block_sum_d(v, red);
    if (tid == 0) part1[b] = v;
    if (!(ok = gsync())) break;
    const double rr_new = grid_total(part1, red);
    ++it;
    last = rr_new;
    if (rr_new < best) {
      best = rr_new;
      for (int i = tid; i < nr; i += kGridThreads) xb[i] = x[i];
    }
    if (rr_new <= thresh) {
      rr = rr_new;
      converged = 1;
      break;
    }
    // a right-hand side with a rounding-level part outside the range of a
    // singular G: the steps along G's near-null directions grow without
    // bound, so the iteration stops once the residual is far above its best
    if (rr_new > 1e8 * best) break;
    const double beta = rr_new / rr;
    for (int i = tid; i < nr; i += kGridThreads) {
      pl[i] = cadd(r[i], cscale(pl[i], beta));
      p.p_glob[r0 + i] = pl[i];
    }
    rr = rr_new;
    if (!(ok = gsync())) break;
  }
  __syncthreads();
  // the returned x is the iterate with the smallest recursive residual (the
  // current one unless the residual rose after its best), and the reported
  // residual is the true |c - G x| / |c| of that x
  const bool use_best = best < last;
  for (int i = tid; i < nr; i += kGridThreads) p.x_out[r0 + i] = use_best ? xb[i] : x[i];
  double true_rr = 0.0;
  if (ok && c2 > 0.0 && (ok = gsync())) {
    v = 0.0;
    for (int i = warp; i < nr; i += kGridWarps) {
      const double2* gi = p.G + (int64_t)(r0 + i) * n;
      double2 s = make_double2(0.0, 0.0);
      for (int j = lane; j < n; j += 32) cfma(s, gi[j], __ldcg(p.x_out + j));
      s = warp_sum2(s);
      if (lane == 0) v += cabs2(csub(p.c[r0 + i], s));
    }
    v = block_sum_d(v, red);
    if (tid == 0) part0[b] = v;
    if ((ok = gsync())) true_rr = grid_total(part0, red);
  }
  if (b == 0 && tid == 0) {
    p.status[0] = ok ? it : -1;
    p.status[1] = ok ? converged : 0;
    p.res[0] = !ok ? 1.0e300 : (c2 > 0.0 ? sqrt(true_rr / c2) : 0.0);
  }
}

int cg_grid_ctas(int n) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, std::min(sms, (n + 3) / 4));  // at least 4 rows per CTA
}

}  // namespace

int64_t zcg_hpsd_grid_workspace(int n) {
  const int64_t G = 1024;  // any grid this entry point launches
  return 256 + ((int64_t)n * 16 + 255) / 256 * 256 + (2 * G * 8 + 255) / 256 * 256;
}

int zcg_hpsd_grid(int n, const void* Gm, const void* c, void* x, double tol, int max_iter, int32_t* status,
                  double* res, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  if (n < 1 || n > (1 << 20)) return fail(CARC_TOO_LARGE, "carc_zcg_hpsd_grid: n = %d", n);
  if (max_iter < 0) return fail(CARC_BAD_ARG, "carc_zcg_hpsd_grid: max_iter %d", max_iter);
  if (!ws || ws_bytes < zcg_hpsd_grid_workspace(n)) return fail(CARC_BAD_ARG, "carc_zcg_hpsd_grid: workspace too small");
  const int G = cg_grid_ctas(n);
  const int rpc = (n + G - 1) / G;
  const size_t smem = (size_t)5 * rpc * sizeof(double2);
  if (smem > 48 * 1024) return fail(CARC_TOO_LARGE, "carc_zcg_hpsd_grid: %d rows per CTA", rpc);
  char* w = static_cast<char*>(ws);
  CgGridParams p;
  p.n = n;
  p.rpc = rpc;
  p.max_iter = max_iter;
  p.G = static_cast<const double2*>(Gm);
  p.c = static_cast<const double2*>(c);
  p.x_out = static_cast<double2*>(x);
  p.sync = reinterpret_cast<unsigned int*>(w);
  p.p_glob = reinterpret_cast<double2*>(w + 256);
  p.part = reinterpret_cast<double*>(w + 256 + ((int64_t)n * 16 + 255) / 256 * 256);
  p.tol = tol;
  p.status = status;
  p.res = res;
  CARC_CHECK_CUDA(cudaMemsetAsync(p.sync, 0, 16, stream));
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)G);
  cfg.blockDim = dim3(kGridThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute la[1];
  la[0].id = cudaLaunchAttributeCooperative;
  la[0].val.cooperative = 1;
  cfg.attrs = la;
  cfg.numAttrs = 1;
  CARC_CHECK_CUDA(cudaLaunchKernelEx(&cfg, zcg_grid_kernel, p));
  count_launch();
  return CARC_OK;
}

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

extern "C" int carc_zcg_hpsd_grid(int32_t n, const void* G, const void* c, void* x, double tol, int32_t max_iter,
                                  void* status, void* residual, void* workspace, int64_t workspace_bytes,
                                  void* stream) {
  if (!G || !c || !x || !status || !residual) return fail(CARC_BAD_ARG, "carc_zcg_hpsd_grid: NULL argument");
  return zcg_hpsd_grid(n, G, c, x, tol, max_iter, static_cast<int32_t*>(status), static_cast<double*>(residual),
                       workspace, workspace_bytes, as_stream(stream));
}

extern "C" int64_t carc_zcg_hpsd_grid_workspace_size(int32_t n) { return n < 1 ? -1 : zcg_hpsd_grid_workspace(n); }
