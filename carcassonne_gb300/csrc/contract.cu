// FP64 complex contraction engine: a grouped, strided, split-K "GETT"
// (general tensor-times-tensor) kernel, plus permute / elementwise / reduction
// kernels.  These carry every dense contraction of the center-site path at
// FP64 precision on the CUDA cores; the tensor-core path lives elsewhere.
#include "common.cuh"
#include "contract.cuh"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace carc {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---- per-phase timing ----------------------------------------------------------
static std::atomic<bool> g_phase_on{false};
static std::mutex g_phase_mu;
struct PhaseRec {
  int phase;
  cudaEvent_t start, stop;
};
static std::vector<PhaseRec> g_phase_recs;

bool phase_timing_on() { return g_phase_on.load(std::memory_order_relaxed); }

void phase_record(int phase, cudaStream_t stream, bool start) {
  std::lock_guard<std::mutex> lk(g_phase_mu);
  if (start) {
    PhaseRec r{phase, nullptr, nullptr};
    if (cudaEventCreate(&r.start) != cudaSuccess || cudaEventCreate(&r.stop) != cudaSuccess) return;
    cudaEventRecord(r.start, stream);
    g_phase_recs.push_back(r);
  } else {
    for (auto it = g_phase_recs.rbegin(); it != g_phase_recs.rend(); ++it)
      if (it->phase == phase) {
        cudaEventRecord(it->stop, stream);
        break;
      }
  }
}

int phase_timing_enable(int on) {
  g_phase_on.store(on != 0, std::memory_order_relaxed);
  return CARC_OK;
}

int phase_timing_read(int phase, double* total_ms, int64_t* count) {
  std::lock_guard<std::mutex> lk(g_phase_mu);
  double t = 0.0;
  int64_t n = 0;
  std::vector<PhaseRec> keep;
  for (auto& r : g_phase_recs) {
    if (r.phase != phase) {
      keep.push_back(r);
      continue;
    }
    float ms = 0.f;
    cudaError_t e = cudaEventElapsedTime(&ms, r.start, r.stop);
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
    if (e != cudaSuccess) {
      g_phase_recs.swap(keep);
      return fail(CARC_CUDA_ERROR, "phase timing: %s (synchronize the stream first)", cudaGetErrorString(e));
    }
    t += ms;
    ++n;
  }
  g_phase_recs.swap(keep);
  if (total_ms) *total_ms = t;
  if (count) *count = n;
  return CARC_OK;
}

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

const char* last_error() { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// GETT kernel
// ---------------------------------------------------------------------------
namespace {

constexpr int NT = 256;

__device__ __forceinline__ int64_t decompose(int64_t idx, int n, const int64_t* ext, const int64_t* str) {
  int64_t off = 0;
  for (int j = n - 1; j >= 0; --j) {
    int64_t e = ext[j];
    int64_t q = idx % e;
    idx /= e;
    off += q * str[j];
  }
  return off;
}

// Output tile TBM x TBN, a 4 x 4 register tile per thread; when the tile needs
// fewer than 256 threads the block splits K into KS slices (each thread group
// takes TBK consecutive k of every KSTEP) and sums the slices in shared memory.
template <int TBM, int TBN>
struct GettCfg {
  static constexpr int TX = TBN / 4, TY = TBM / 4, TPS = TX * TY;
  static constexpr int KS = NT / TPS;
  static constexpr int TBK = KS >= 4 ? 4 : 8;
  static constexpr int KSTEP = KS * TBK;
  static constexpr int STAGE = KSTEP * (TBM + TBN);
  static constexpr int SMEM_ELEMS = (KS > 1 && TBM * TBN > STAGE) ? TBM * TBN : STAGE;
};

template <int TBM, int TBN>
__global__ __launch_bounds__(NT) void gett_kernel(const __grid_constant__ GettParams p) {
  using Cfg = GettCfg<TBM, TBN>;
  static_assert(Cfg::TPS * Cfg::KS == NT, "tile must divide the block");
  const int out = blockIdx.z;
  const int ks = blockIdx.y;
  const int64_t tiles_n = (p.N + TBN - 1) / TBN;
  const int64_t tm = blockIdx.x / tiles_n, tn = blockIdx.x % tiles_n;
  const int tid = threadIdx.x;
  const int slice = tid / Cfg::TPS, lt = tid % Cfg::TPS;
  const int tx = lt % Cfg::TX, ty = lt / Cfg::TX;

  __shared__ int64_t s_arow[TBM], s_crow[TBM], s_bcol[TBN], s_ccol[TBN];
  __shared__ int64_t s_ak[Cfg::KSTEP], s_bk[Cfg::KSTEP];
  __shared__ double2 sbuf[Cfg::SMEM_ELEMS];  // operand stage, then the slice reduction
  double2(*As)[TBM] = reinterpret_cast<double2(*)[TBM]>(sbuf);
  double2(*Bs)[TBN] = reinterpret_cast<double2(*)[TBN]>(sbuf + Cfg::KSTEP * TBM);

  for (int i = tid; i < TBM; i += NT) {
    int64_t m = tm * TBM + i;
    if (m < p.M) {
      s_arow[i] = decompose(m, p.nm, p.m_ext, p.a_m);
      s_crow[i] = decompose(m, p.nm, p.m_ext, p.c_m);
    } else {
      s_arow[i] = -1;
      s_crow[i] = -1;
    }
  }
  for (int i = tid; i < TBN; i += NT) {
    int64_t n = tn * TBN + i;
    if (n < p.N) {
      s_bcol[i] = decompose(n, p.nn, p.n_ext, p.b_n);
      s_ccol[i] = decompose(n, p.nn, p.n_ext, p.c_n);
    } else {
      s_bcol[i] = -1;
      s_ccol[i] = -1;
    }
  }

  const int64_t k_begin = (int64_t)ks * p.kchunk;
  const int64_t k_end = min(p.K, k_begin + p.kchunk);

  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);

  const int e_begin = p.ob[out], e_end = p.ob[out + 1];
  for (int e = e_begin; e < e_end; ++e) {
    const double2* __restrict__ A = p.a[p.ea[e]];
    const double2* __restrict__ B = p.b[p.eb[e]];
    for (int64_t k0 = k_begin; k0 < k_end; k0 += Cfg::KSTEP) {
      __syncthreads();
      for (int i = tid; i < 2 * Cfg::KSTEP; i += NT) {
        const int kk = i % Cfg::KSTEP;
        const int64_t k = k0 + kk;
        if (i < Cfg::KSTEP)
          s_ak[kk] = k < k_end ? decompose(k, p.nk, p.k_ext, p.a_k) : -1;
        else
          s_bk[kk] = k < k_end ? decompose(k, p.nk, p.k_ext, p.b_k) : -1;
      }
      __syncthreads();
      for (int idx = tid; idx < Cfg::KSTEP * TBM; idx += NT) {
        int kk = idx / TBM, mm = idx % TBM;
        double2 v = make_double2(0.0, 0.0);
        int64_t ro = s_arow[mm], ko = s_ak[kk];
        if (ro >= 0 && ko >= 0) {
          v = A[ro + ko];
          if (p.conj_a) v.y = -v.y;
        }
        As[kk][mm] = v;
      }
      for (int idx = tid; idx < Cfg::KSTEP * TBN; idx += NT) {
        int kk = idx / TBN, nn = idx % TBN;
        double2 v = make_double2(0.0, 0.0);
        int64_t co = s_bcol[nn], ko = s_bk[kk];
        if (co >= 0 && ko >= 0) {
          v = B[co + ko];
          if (p.conj_b) v.y = -v.y;
        }
        Bs[kk][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < Cfg::TBK; ++kk) {
        const int kq = slice * Cfg::TBK + kk;
        double2 a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kq][ty * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kq][tx * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
      }
    }
  }

  if (Cfg::KS > 1) {
    // sum the K slices into slice 0 (in slice order: deterministic)
    double2* red = sbuf;
    for (int r = 0; r < Cfg::KS; ++r) {
      __syncthreads();
      if (slice == r) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            double2* q = &red[(ty * 4 + i) * TBN + tx * 4 + j];
            *q = r == 0 ? acc[i][j] : cadd(*q, acc[i][j]);
          }
      }
    }
    __syncthreads();
    if (slice != 0) return;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = red[(ty * 4 + i) * TBN + tx * 4 + j];
  }

  if (p.ksplit == 1) {
    double2* __restrict__ C = p.c[out];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t ro = s_crow[ty * 4 + i];
      if (ro < 0) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int64_t co = s_ccol[tx * 4 + j];
        if (co < 0) continue;
        double2 v = cmul(p.alpha, acc[i][j]);
        if (p.accumulate) v = cadd(v, C[ro + co]);
        C[ro + co] = v;
      }
    }
  } else {
    double2* __restrict__ P = p.partial + ((int64_t)ks * p.n_out + out) * p.M * p.N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t m = tm * TBM + ty * 4 + i;
      if (m >= p.M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int64_t n = tn * TBN + tx * 4 + j;
        if (n >= p.N) continue;
        P[m * p.N + n] = acc[i][j];
      }
    }
  }
}

__global__ void gett_reduce_kernel(const __grid_constant__ GettParams p) {
  const int64_t total = (int64_t)p.n_out * p.M * p.N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t n = i % p.N;
    int64_t t = i / p.N;
    int64_t m = t % p.M;
    int out = (int)(t / p.M);
    // eight partials in flight, added in split order
    const double2* src = p.partial + (int64_t)out * p.M * p.N + m * p.N + n;
    const int64_t stride = (int64_t)p.n_out * p.M * p.N;
    double2 s = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < p.ksplit; k0 += 8) {
      double2 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = k0 + u < p.ksplit ? src[(k0 + u) * stride] : make_double2(0.0, 0.0);
#pragma unroll
      for (int u = 0; u < 8; ++u) s = cadd(s, v[u]);
    }
    int64_t off = decompose(m, p.nm, p.m_ext, p.c_m) + decompose(n, p.nn, p.n_ext, p.c_n);
    double2* C = p.c[out];
    double2 v = cmul(p.alpha, s);
    if (p.accumulate) v = cadd(v, C[off]);
    C[off] = v;
  }
}

}  // namespace

static int64_t prod_ext(int n, const int64_t* e) {
  int64_t r = 1;
  for (int i = 0; i < n; ++i) r *= e[i];
  return r;
}

// Output tile shapes of the GETT kernel; the launcher takes the one that pads
// the output least (larger tiles on ties: more reuse per loaded element).
struct TileShape {
  int bm, bn, kstep;
};
constexpr TileShape kTiles[] = {
    {64, 64, GettCfg<64, 64>::KSTEP}, {64, 32, GettCfg<64, 32>::KSTEP}, {32, 64, GettCfg<32, 64>::KSTEP},
    {32, 32, GettCfg<32, 32>::KSTEP}, {32, 16, GettCfg<32, 16>::KSTEP}, {16, 32, GettCfg<16, 32>::KSTEP},
    {16, 16, GettCfg<16, 16>::KSTEP}};

static int choose_tile(int64_t M, int64_t N) {
  int best = 0;
  int64_t best_area = -1;
  for (int i = 0; i < (int)(sizeof(kTiles) / sizeof(kTiles[0])); ++i) {
    const int64_t area = ceil_div(M, kTiles[i].bm) * kTiles[i].bm * ceil_div(N, kTiles[i].bn) * kTiles[i].bn;
    if (best_area < 0 || area < best_area) {
      best = i;
      best_area = area;
    }
  }
  return best;
}

static int choose_ksplit(int64_t M, int64_t N, int64_t K, int n_out, int64_t* kchunk) {
  const TileShape& t = kTiles[choose_tile(M, N)];
  int64_t tiles = ceil_div(M, t.bm) * ceil_div(N, t.bn) * (int64_t)n_out;
  int ks = 1;
  const int64_t target = 2 * 152;
  if (tiles < target && K >= 256) {
    int64_t want = ceil_div(target, tiles);
    int64_t maxk = K / 128;
    ks = (int)std::max<int64_t>(1, std::min<int64_t>({want, maxk, (int64_t)512}));
  }
  int64_t chunk = ceil_div(K, ks);
  chunk = ceil_div(chunk, t.kstep) * t.kstep;
  ks = (int)ceil_div(K, chunk);
  if (ks < 1) ks = 1;
  *kchunk = chunk;
  return ks;
}

int validate_desc(const carc_contract_desc& d) {
  if (d.nm < 0 || d.nn < 0 || d.nk < 0 || d.nm > CARC_MAX_SUBDIMS || d.nn > CARC_MAX_SUBDIMS ||
      d.nk > CARC_MAX_SUBDIMS)
    return fail(CARC_BAD_ARG, "contraction descriptor: sub-dimension counts out of range (%d,%d,%d)", d.nm, d.nn, d.nk);
  for (int i = 0; i < d.nm; ++i)
    if (d.m_ext[i] < 1) return fail(CARC_BAD_SHAPE, "contraction descriptor: m extent %d is %lld", i, (long long)d.m_ext[i]);
  for (int i = 0; i < d.nn; ++i)
    if (d.n_ext[i] < 1) return fail(CARC_BAD_SHAPE, "contraction descriptor: n extent %d is %lld", i, (long long)d.n_ext[i]);
  for (int i = 0; i < d.nk; ++i)
    if (d.k_ext[i] < 1) return fail(CARC_BAD_SHAPE, "contraction descriptor: k extent %d is %lld", i, (long long)d.k_ext[i]);
  return CARC_OK;
}

int64_t gett_workspace_size(const carc_contract_desc& d, int n_out) {
  if (validate_desc(d) != CARC_OK) return -1;
  int64_t M = prod_ext(d.nm, d.m_ext), N = prod_ext(d.nn, d.n_ext), K = prod_ext(d.nk, d.k_ext);
  int64_t chunk;
  int ks = choose_ksplit(M, N, K, n_out, &chunk);
  if (ks <= 1) return 0;
  return (int64_t)ks * n_out * M * N * (int64_t)sizeof(double2);
}

int gett_launch(const carc_contract_desc& d, const void* const* a_ptrs, int n_a, const void* const* b_ptrs, int n_b,
                void* const* c_ptrs, int n_c, const int32_t* entries, int n_entries, double2 alpha, int accumulate,
                void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
  CARC_RETURN_IF(validate_desc(d));
  if (n_a < 1 || n_b < 1 || n_c < 1 || n_a > CARC_MAX_SLOTS || n_b > CARC_MAX_SLOTS || n_c > CARC_MAX_SLOTS)
    return fail(CARC_TOO_LARGE, "grouped contraction: slot counts (%d,%d,%d) outside 1..%d", n_a, n_b, n_c, CARC_MAX_SLOTS);
  if (n_entries < 0 || n_entries > CARC_MAX_ENTRIES)
    return fail(CARC_TOO_LARGE, "grouped contraction: %d entries exceeds %d", n_entries, CARC_MAX_ENTRIES);
  GettParams p;
  std::memset(&p, 0, sizeof(p));
  p.nm = d.nm;
  p.nn = d.nn;
  p.nk = d.nk;
  p.conj_a = d.conj_a;
  p.conj_b = d.conj_b;
  for (int i = 0; i < CARC_MAX_SUBDIMS; ++i) {
    p.m_ext[i] = d.m_ext[i];
    p.n_ext[i] = d.n_ext[i];
    p.k_ext[i] = d.k_ext[i];
    p.a_m[i] = d.a_m[i];
    p.a_k[i] = d.a_k[i];
    p.b_n[i] = d.b_n[i];
    p.b_k[i] = d.b_k[i];
    p.c_m[i] = d.c_m[i];
    p.c_n[i] = d.c_n[i];
  }
  p.M = prod_ext(d.nm, d.m_ext);
  p.N = prod_ext(d.nn, d.n_ext);
  p.K = prod_ext(d.nk, d.k_ext);
  p.alpha = alpha;
  p.accumulate = accumulate;
  p.n_out = n_c;
  for (int i = 0; i < n_a; ++i) p.a[i] = static_cast<const double2*>(a_ptrs[i]);
  for (int i = 0; i < n_b; ++i) p.b[i] = static_cast<const double2*>(b_ptrs[i]);
  for (int i = 0; i < n_c; ++i) {
    p.c[i] = static_cast<double2*>(c_ptrs[i]);
    if (!p.c[i]) return fail(CARC_BAD_ARG, "grouped contraction: output slot %d is NULL", i);
  }
  // stable grouping of the entries by output slot
  int count[CARC_MAX_SLOTS + 1] = {0};
  for (int e = 0; e < n_entries; ++e) {
    int a = entries[3 * e], b = entries[3 * e + 1], c = entries[3 * e + 2];
    if (a < 0 || a >= n_a || b < 0 || b >= n_b || c < 0 || c >= n_c)
      return fail(CARC_BAD_ARG, "grouped contraction: entry %d = (%d,%d,%d) out of range", e, a, b, c);
    if (!p.a[a] || !p.b[b]) return fail(CARC_BAD_ARG, "grouped contraction: entry %d uses a NULL operand", e);
    count[c + 1]++;
  }
  for (int c = 0; c < n_c; ++c) count[c + 1] += count[c];
  for (int c = 0; c <= n_c; ++c) p.ob[c] = (int16_t)count[c];
  int fill[CARC_MAX_SLOTS];
  for (int c = 0; c < n_c; ++c) fill[c] = count[c];
  for (int e = 0; e < n_entries; ++e) {
    int c = entries[3 * e + 2];
    int pos = fill[c]++;
    p.ea[pos] = (int16_t)entries[3 * e];
    p.eb[pos] = (int16_t)entries[3 * e + 1];
  }
  int64_t chunk;
  p.ksplit = choose_ksplit(p.M, p.N, p.K, n_c, &chunk);
  p.kchunk = chunk;
  if (p.ksplit > 1) {
    int64_t need = (int64_t)p.ksplit * n_c * p.M * p.N * (int64_t)sizeof(double2);
    if (!workspace || workspace_bytes < need)
      return fail(CARC_BAD_ARG, "grouped contraction: workspace of %lld bytes needed, %lld given", (long long)need,
                  (long long)workspace_bytes);
    p.partial = static_cast<double2*>(workspace);
  }
  const int tile = choose_tile(p.M, p.N);
  int64_t tiles = ceil_div(p.M, kTiles[tile].bm) * ceil_div(p.N, kTiles[tile].bn);
  if (tiles > 0x7fffffff || n_c > 65535 || p.ksplit > 65535)
    return fail(CARC_TOO_LARGE, "grouped contraction: grid too large");
  dim3 grid((unsigned)tiles, (unsigned)p.ksplit, (unsigned)n_c);
  switch (tile) {
    case 0: gett_kernel<64, 64><<<grid, NT, 0, stream>>>(p); break;
    case 1: gett_kernel<64, 32><<<grid, NT, 0, stream>>>(p); break;
    case 2: gett_kernel<32, 64><<<grid, NT, 0, stream>>>(p); break;
    case 3: gett_kernel<32, 32><<<grid, NT, 0, stream>>>(p); break;
    case 4: gett_kernel<32, 16><<<grid, NT, 0, stream>>>(p); break;
    case 5: gett_kernel<16, 32><<<grid, NT, 0, stream>>>(p); break;
    default: gett_kernel<16, 16><<<grid, NT, 0, stream>>>(p); break;
  }
  CARC_CHECK_LAUNCH();
  if (p.ksplit > 1) {
    int64_t total = (int64_t)n_c * p.M * p.N;
    int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 4 * 152);
    gett_reduce_kernel<<<blocks, 256, 0, stream>>>(p);
    CARC_CHECK_LAUNCH();
  }
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// permute / elementwise / reductions
// ---------------------------------------------------------------------------
namespace {

struct PermuteParams {
  int ndim;
  int conj;
  int64_t shape[CARC_MAX_PERMUTE_DIMS];
  int64_t istr[CARC_MAX_PERMUTE_DIMS];
  int64_t total;
};

__global__ void permute_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                               const __grid_constant__ PermuteParams p) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t idx = i, off = 0;
    for (int j = p.ndim - 1; j >= 0; --j) {
      int64_t q = idx % p.shape[j];
      idx /= p.shape[j];
      off += q * p.istr[j];
    }
    double2 v = in[off];
    if (p.conj) v.y = -v.y;
    out[i] = v;
  }
}

__global__ void axpby_kernel(int64_t n, double2 a, const double2* __restrict__ x, double2 b,
                             const double2* __restrict__ y, double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 r = make_double2(0.0, 0.0);
    if (x) r = cmul(a, x[i]);
    if (y) r = cadd(r, cmul(b, y[i]));
    out[i] = r;
  }
}

__global__ void mul_kernel(int64_t n, const double2* __restrict__ x, const double2* __restrict__ y,
                           double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = cmul(x[i], y[i]);
}

__global__ void fill_kernel(int64_t n, double2 v, double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v;
}

constexpr int DOT_THREADS = 256;

__device__ double2 block_sum2(double2 v) {
  __shared__ double2 warps[DOT_THREADS / 32];
  v = warp_sum2(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warps[w] = v;
  __syncthreads();
  double2 r = make_double2(0.0, 0.0);
  if (w == 0) {
    r = lane < DOT_THREADS / 32 ? warps[lane] : make_double2(0.0, 0.0);
    r = warp_sum2(r);
  }
  __syncthreads();
  return r;
}

__global__ __launch_bounds__(DOT_THREADS) void dot_partial_kernel(int64_t n, const double2* __restrict__ x,
                                                                   const double2* __restrict__ y, int conj_x,
                                                                   double2* __restrict__ partial) {
  double2 s = make_double2(0.0, 0.0);
  for (int64_t i = blockIdx.x * (int64_t)DOT_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * DOT_THREADS) {
    double2 a = x[i];
    if (conj_x) a.y = -a.y;
    cfma(s, a, y[i]);
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ __launch_bounds__(DOT_THREADS) void dot_final_kernel(int nblocks, const double2* __restrict__ partial,
                                                                 double2* __restrict__ out) {
  double2 s = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < nblocks; i += DOT_THREADS) s = cadd(s, partial[i]);
  s = block_sum2(s);
  if (threadIdx.x == 0) *out = s;
}

__global__ void hasnan_kernel(int64_t n, const double2* __restrict__ x, int* flag) {
  int local = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 v = x[i];
    if (isnan(v.x) || isnan(v.y)) local = 1;
  }
  if (__any_sync(0xffffffffu, local) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

inline int grid_for(int64_t n, int threads = 256) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), 8 * 152));
}

}  // namespace

int permute_launch(const void* in, void* out, int ndim, const int64_t* shape, const int64_t* istr, int conj,
                   cudaStream_t stream) {
  if (ndim < 0 || ndim > CARC_MAX_PERMUTE_DIMS) return fail(CARC_BAD_ARG, "permute: ndim %d out of range", ndim);
  PermuteParams p;
  std::memset(&p, 0, sizeof(p));
  p.ndim = ndim;
  p.conj = conj;
  p.total = 1;
  for (int i = 0; i < ndim; ++i) {
    if (shape[i] < 0) return fail(CARC_BAD_SHAPE, "permute: negative extent");
    p.shape[i] = shape[i];
    p.istr[i] = istr[i];
    p.total *= shape[i];
  }
  if (p.total == 0) return CARC_OK;
  permute_kernel<<<grid_for(p.total), 256, 0, stream>>>(static_cast<const double2*>(in), static_cast<double2*>(out), p);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int axpby_launch(int64_t n, double2 a, const void* x, double2 b, const void* y, void* out, cudaStream_t stream) {
  if (n <= 0) return CARC_OK;
  axpby_kernel<<<grid_for(n), 256, 0, stream>>>(n, a, static_cast<const double2*>(x), b,
                                                 static_cast<const double2*>(y), static_cast<double2*>(out));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int mul_launch(int64_t n, const void* x, const void* y, void* out, cudaStream_t stream) {
  if (n <= 0) return CARC_OK;
  mul_kernel<<<grid_for(n), 256, 0, stream>>>(n, static_cast<const double2*>(x), static_cast<const double2*>(y),
                                               static_cast<double2*>(out));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int fill_launch(int64_t n, double2 v, void* out, cudaStream_t stream) {
  if (n <= 0) return CARC_OK;
  fill_kernel<<<grid_for(n), 256, 0, stream>>>(n, v, static_cast<double2*>(out));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

static int dot_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, DOT_THREADS * 4), 2 * 152));
}

int64_t dot_workspace_size(int64_t n) { return (int64_t)dot_blocks(n) * (int64_t)sizeof(double2); }

int dot_launch(int64_t n, const void* x, const void* y, int conj_x, void* out, void* ws, int64_t ws_bytes,
               cudaStream_t stream) {
  int nb = dot_blocks(n);
  if (!ws || ws_bytes < (int64_t)nb * (int64_t)sizeof(double2))
    return fail(CARC_BAD_ARG, "dot: workspace too small");
  dot_partial_kernel<<<nb, DOT_THREADS, 0, stream>>>(n, static_cast<const double2*>(x), static_cast<const double2*>(y),
                                                     conj_x, static_cast<double2*>(ws));
  CARC_CHECK_LAUNCH();
  dot_final_kernel<<<1, DOT_THREADS, 0, stream>>>(nb, static_cast<const double2*>(ws), static_cast<double2*>(out));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int hasnan_launch(int64_t n, const void* x, void* flag, cudaStream_t stream) {
  CARC_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), stream));
  if (n <= 0) return CARC_OK;
  hasnan_kernel<<<grid_for(n), 256, 0, stream>>>(n, static_cast<const double2*>(x), static_cast<int*>(flag));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace carc
