// Complex FP64 contractions on the 5th-generation tensor cores.
//
// A complex product C = A B^T (A: M x K, B: N x K, complex128) is carried out
// as ONE real BF16 GEMM with FP32 accumulation in TMEM:
//   * real embedding: row (m,re) of A is [a_r, -a_i] per k, row (m,im) is
//     [a_i, a_r]; row n of B is [b_r, b_i] per k; so (A_emb B_col^T) holds
//     C_re / C_im in rows (m,re) / (m,im);
//   * split precision: every real value v = hi + lo with hi = bf16(v) and
//     lo = bf16(v - hi) (about 16 significant bits); A is stacked along M as
//     (hi, lo) rows and B is concatenated along K as [hi | lo], so one GEMM
//     forms hi.hi + hi.lo (rows s=hi) and lo.hi + lo.lo (rows s=lo), which the
//     epilogue sums in FP64.
// Operand A_op is 4M x 4K (rows (m, re/im, hi/lo)), B_op is N x 4K, both
// BF16 K-major; the GEMM kernel is a TMA + tcgen05 pipeline (BM=128 rows,
// BN<=256 columns, 64-wide K blocks in 128-byte swizzled shared memory,
// 4 stages), with optional split-K into FP32 partial planes.
#include "common.cuh"
#include "umma.cuh"
#include "umma_gemm.cuh"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

namespace carc {

namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // bf16 elements per K block (128 bytes)
constexpr int THREADS = 192;
constexpr int A_STAGE_BYTES = BM * BK * 2;

__host__ __device__ constexpr int tmem_cols_for(int bn) { return bn <= 32 ? 32 : (bn <= 64 ? 64 : (bn <= 128 ? 128 : 256)); }

// Pipeline depth: the plain GEMM streams long K ranges (4 stages, one CTA
// per SM); the folding GEMM has short K and a long epilogue, so it keeps two
// stages and fits two CTAs per SM, one CTA's epilogue overlapping the other's
// loads and MMAs.
__host__ __device__ constexpr int stages_for(int epi) { return epi ? 2 : 4; }

template <int BN, int EPI>
constexpr int smem_bytes() {
  return 1024 + stages_for(EPI) * (A_STAGE_BYTES + BN * BK * 2) + 256;
}

// ---- folding epilogue --------------------------------------------------------
// The tile's accumulator is 128 rows (4m + 2c + s: complex row m, re/im c,
// hi/lo s) x BN columns n.  It is staged HC columns at a time as FP32 with a
// row pitch of HC + 4 floats (conflict-free float4 stores).  After the staged
// block come two index tables: per complex row m of the tile {row part, k part}
// of the destination (or -1), and per slot q {n_local, row part, k part,
// valid}, slots in p-major order so that consecutive slots walk (vec, k2, k3),
// i.e. consecutive destination k.
template <int BN>
__host__ __device__ constexpr int FOLD_HC() { return BN == 256 ? 128 : (BN == 128 ? 64 : BN); }

template <int BN>
__host__ __device__ constexpr int FOLD_PITCH() { return FOLD_HC<BN>() + 4; }

template <int BN>
__host__ __device__ constexpr int fold_smem_bytes() { return 128 * FOLD_PITCH<BN>() * 4 + 32 * 8 + FOLD_HC<BN>() * 16; }

template <int BN>
__device__ __forceinline__ void fold_tables(float* sP, const FoldEpi& fe, int m0, int nb, int tid, int nthreads) {
  constexpr int HC = FOLD_HC<BN>();
  int2* tabM = reinterpret_cast<int2*>(sP + 128 * FOLD_PITCH<BN>());
  int4* tabN = reinterpret_cast<int4*>(tabM + 32);
  const int L0 = (int)fe.l0, L1 = (int)fe.l1, X1 = (int)fe.x1, K2 = (int)fe.k2, K3 = (int)fe.k3, Dp = (int)fe.d;
  for (int i = tid; i < 32; i += nthreads) {
    const int64_t m = (int64_t)(m0 >> 2) + i;
    int2 t = make_int2(-1, 0);
    if (m < fe.M) {
      int r = (int)m;
      const int ll1 = r % L1; r /= L1;
      const int ll0 = r % L0; r /= L0;
      const int xx1 = r % X1; r /= X1;
      t = make_int2((ll0 * L1 + ll1) * Dp, (r * X1 + xx1) * K2 * K3);
    }
    tabM[i] = t;
  }
  const bool pmajor = (HC % Dp) == 0 && (nb % Dp) == 0;
  for (int q = tid; q < HC; q += nthreads) {
    const int nl = pmajor ? (q % (HC / Dp)) * Dp + q / (HC / Dp) : q;
    const int64_t n = (int64_t)nb + nl;
    int4 t = make_int4(nl, 0, 0, 0);
    if (n < fe.N) {
      int r = (int)n;
      const int p = r % Dp; r /= Dp;
      const int k3 = r % K3; r /= K3;
      const int k2 = r % K2; r /= K2;
      t = make_int4(nl, r * L0 * L1 * Dp + p, k2 * K3 + k3, 1);
    }
    tabN[q] = t;
  }
}

// W[m, n] = (P[4m] + P[4m+1]) + i (P[4m+2] + P[4m+3]), split into bf16 hi/lo
// pairs; consecutive threads store consecutive k of one destination row.
template <int BN>
__device__ __forceinline__ void fold_write(const float* sP, const FoldEpi& fe) {
  constexpr int HC = FOLD_HC<BN>();
  const int2* tabM = reinterpret_cast<const int2*>(sP + 128 * FOLD_PITCH<BN>());
  const int4* tabN = reinterpret_cast<const int4*>(tabM + 32);
  uint32_t* W = static_cast<uint32_t*>(fe.dst);  // bf16 pairs; pitch, col_off and kc are even
  const int64_t pitch2 = fe.pitch >> 1, off2 = fe.col_off >> 1;
  const int kc = (int)fe.kc;
#pragma unroll 4
  for (int e = threadIdx.x; e < 32 * HC; e += blockDim.x) {
    const int ml = e / HC;
    const int2 tm = tabM[ml];
    const int4 tn = tabN[e % HC];
    if (tm.x < 0 || tn.w == 0) continue;
    const float* col = sP + 4 * ml * FOLD_PITCH<BN>() + tn.x;
    const float re = col[0] + col[FOLD_PITCH<BN>()];
    const float im = col[2 * FOLD_PITCH<BN>()] + col[3 * FOLD_PITCH<BN>()];
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(re, im);
    const float2 hf = __bfloat1622float2(h2);
    const __nv_bfloat162 l2 = __floats2bfloat162_rn(re - hf.x, im - hf.y);
    uint32_t* rowp = W + (int64_t)(tn.y + tm.x) * pitch2 + off2 + (tm.y + tn.z);
    rowp[0] = *reinterpret_cast<const uint32_t*>(&h2);
    rowp[kc] = *reinterpret_cast<const uint32_t*>(&l2);
  }
}

template <int BN, int EPI>
__global__ __launch_bounds__(THREADS, EPI ? 2 : 1) void gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                   const __grid_constant__ CUtensorMap tmB,
                                                                   float* __restrict__ out, int64_t ld_out,
                                                                   int64_t split_stride, int kb_per_split,
                                                                   int kb_total, int a_rows, int* __restrict__ err,
                                                                   const __grid_constant__ FoldEpi fe) {
  using namespace umma;
  constexpr int B_STAGE_BYTES = BN * BK * 2;
  constexpr uint32_t TMEM_COLS = tmem_cols_for(BN);
  constexpr int STAGES = stages_for(EPI);
  static_assert(EPI == 0 || fold_smem_bytes<BN>() <= STAGES * (A_STAGE_BYTES + B_STAGE_BYTES),
                "the staged tile must fit in the pipeline stages");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_STAGE_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + STAGES * B_STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kb0 = blockIdx.z * kb_per_split;
  const int kb1 = min(kb_total, kb0 + kb_per_split);
  const int nkb = max(0, kb1 - kb0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (a_rows < BM) {
    // the TMA fills only rows [0, a_rows) of each A stage: the rest is zero
    // (the operand's padding rows), so they need not be read from memory
    for (int s = 0; s < STAGES; ++s) {
      uint4* z = reinterpret_cast<uint4*>(sA + s * A_STAGE_BYTES + a_rows * BK * 2);
      for (int i = threadIdx.x; i < (BM - a_rows) * BK * 2 / 16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async();
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)((i / STAGES) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag)) break;
        mbar_arrive_expect_tx(&full[s], (uint32_t)(a_rows * BK * 2 + B_STAGE_BYTES));
        const int kx = (kb0 + i) * BK;
        tma_load_2d(sA + s * A_STAGE_BYTES, &tmA, kx, m0, &full[s]);
        tma_load_2d(sB + s * B_STAGE_BYTES, &tmB, kx, n0, &full[s]);
        ++issued;
      }
      if (*abort_flag) {
        // let copies already in flight land before the CTA exits (bounded)
        for (int i = max(0, issued - STAGES); i < issued; ++i) {
          const int s = i % STAGES;
          for (uint32_t t = 0; t < (1u << 20); ++t)
            if (mbar_try_wait(&full[s], (uint32_t)((i / STAGES) & 1))) break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // single-thread MMA issuer
      const uint32_t idesc = idesc_bf16_f32(BM, BN);
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)((i / STAGES) & 1);
        if (!mbar_wait(&full[s], ph, abort_flag)) break;
        tc_fence_after();
        const uint32_t a_base = smem_u32(sA + s * A_STAGE_BYTES);
        const uint32_t b_base = smem_u32(sB + s * B_STAGE_BYTES);
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const uint64_t ad = smem_desc_sw128(a_base + kk * 32);
          const uint64_t bd = smem_desc_sw128(b_base + kk * 32);
          mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit(&empty[s]);
      }
      mma_commit(done);
    }
  } else {
    // epilogue: warps 2..5 own TMEM lane quadrants (warp % 4)
    const int quad = warp & 3;
    const bool ok = mbar_wait(done, 0, abort_flag);
    tc_fence_after();
    if (EPI == 1) {
      // the folding epilogue runs below, after the CTA-wide barrier
    } else if (ok) {
      const int row = m0 + quad * 32 + lane;
      float* dst = out + (int64_t)blockIdx.z * split_stride + (int64_t)row * ld_out + n0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
        tmem_ld_wait();
        // BN = 16 tiles read 32 allocated columns but own only the first 16
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          if (c0 + j >= BN) break;
          *reinterpret_cast<float4*>(dst + c0 + j) =
              nkb > 0 ? make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                                    __uint_as_float(r[j + 3]))
                      : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (EPI == 1) {
    // Folding epilogue, HC columns at a time: warps 2..5 move the raw FP32
    // accumulator rows of their TMEM lane quadrant to shared memory (reusing
    // the pipeline stages: once `done` has fired every load has landed and
    // every MMA has read its operands), then all threads fold and write them.
    constexpr int HC = FOLD_HC<BN>();
    float* sP = reinterpret_cast<float*>(smem);
    const bool ok = !*abort_flag;
    tc_fence_after();
#pragma unroll 1
    for (int h0 = 0; h0 < BN; h0 += HC) {
      if (ok && warp >= 2) {
        const int quad = warp & 3;
#pragma unroll 1
        for (int c0 = 0; c0 < HC; c0 += 32) {
          uint32_t r[32];
          tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(h0 + c0), r);
          tmem_ld_wait();
          float4* dst = reinterpret_cast<float4*>(sP + (quad * 32 + lane) * FOLD_PITCH<BN>() + c0);
#pragma unroll
          for (int j = 0; j < 32; j += 4) {
            if (c0 + j >= HC) break;
            dst[j / 4] = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                                     __uint_as_float(r[j + 3]));
          }
        }
      }
      tc_fence_before();
      fold_tables<BN>(sP, fe, m0, n0 + h0, threadIdx.x, blockDim.x);
      __syncthreads();
      if (ok) fold_write<BN>(sP, fe);
      __syncthreads();
      tc_fence_after();
    }
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, CARC_NOT_CONVERGED);
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---- tensor maps ------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int make_map(CUtensorMap* map, const void* base, uint64_t inner, uint64_t rows, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(CARC_CUDA_ERROR, "tensor core GEMM: cuTensorMapEncodeTiled is unavailable");
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(CARC_BAD_ARG, "tensor core GEMM: operand not 16-byte aligned");
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {inner * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(CARC_CUDA_ERROR, "tensor core GEMM: cuTensorMapEncodeTiled failed (%d)", (int)r);
  return CARC_OK;
}

template <int BN, int EPI>
int launch_bn(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int a_rows, float* out, int64_t ld_out,
              int64_t split_stride, int ksplit, int kb_per, int kb_total, int* err, const FoldEpi& fe,
              cudaStream_t stream) {
  constexpr int SMEM = smem_bytes<BN, EPI>();
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(gemm_bf16_tn_kernel<BN, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
  });
  if (attr_err != cudaSuccess) return fail(CARC_CUDA_ERROR, "tensor core GEMM: %s", cudaGetErrorString(attr_err));
  dim3 grid(M / BM, N / BN, ksplit);
  gemm_bf16_tn_kernel<BN, EPI><<<grid, THREADS, SMEM, stream>>>(ma, mb, out, ld_out, split_stride, kb_per, kb_total, a_rows,
                                                                 err, fe);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

template <int EPI>
int launch_any(int bn, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int a_rows, float* out,
               int64_t ld_out,
               int64_t split_stride, int ksplit, int kb_per, int kb_total, int* err, const FoldEpi& fe,
               cudaStream_t stream) {
  switch (bn) {
    case 256: return launch_bn<256, EPI>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, fe, stream);
    case 128: return launch_bn<128, EPI>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, fe, stream);
    case 64: return launch_bn<64, EPI>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, fe, stream);
    case 32: return launch_bn<32, EPI>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, fe, stream);
    default: return launch_bn<16, EPI>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, fe, stream);
  }
}

}  // namespace

int gemm_bf16_tn(const void* A, int M, const void* B, int N, int K, float* out, int64_t ld_out, int ksplit, int* err,
                 cudaStream_t stream, int m_live) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM != 0 || K % BK != 0 || N % 16 != 0)
    return fail(CARC_BAD_SHAPE, "tensor core GEMM: shape %d x %d x %d not tileable (M%%128, K%%64, N%%16)", M, N, K);
  if (ld_out < N || ld_out % 4 != 0) return fail(CARC_BAD_ARG, "tensor core GEMM: ld_out %lld", (long long)ld_out);
  const int kb_total = K / BK;
  ksplit = std::max(1, std::min(ksplit, kb_total));
  const int kb_per = (kb_total + ksplit - 1) / ksplit;
  ksplit = (kb_total + kb_per - 1) / kb_per;
  int bn = N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : N % 64 == 0 ? 64 : N % 32 == 0 ? 32 : 16;
  // one 128-row tile whose rows >= 64 are zero padding: load only the live half
  const int a_rows = (M == BM && m_live > 0 && m_live <= 64) ? 64 : BM;
  CUtensorMap ma, mb;
  CARC_RETURN_IF(make_map(&ma, A, (uint64_t)K, (uint64_t)M, (uint32_t)a_rows));
  CARC_RETURN_IF(make_map(&mb, B, (uint64_t)K, (uint64_t)N, (uint32_t)bn));
  const int64_t split_stride = (int64_t)M * ld_out;
  FoldEpi none;
  memset(&none, 0, sizeof(none));
  return launch_any<0>(bn, ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, none,
                       stream);
}

int gemm_bf16_tn_fold(const void* A, int M, const void* B, int N, int K, const FoldEpi& fe, int* err,
                      cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM != 0 || K % BK != 0 || N % 16 != 0)
    return fail(CARC_BAD_SHAPE, "tensor core GEMM: shape %d x %d x %d not tileable (M%%128, K%%64, N%%16)", M, N, K);
  if (fe.M * 4 > M || fe.N > N || (fe.pitch & 1) || (fe.col_off & 1))
    return fail(CARC_BAD_ARG, "tensor core GEMM: folding epilogue does not fit the tile grid");
  const int kb_total = K / BK;
  int bn = N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : N % 64 == 0 ? 64 : N % 32 == 0 ? 32 : 16;
  CUtensorMap ma, mb;
  CARC_RETURN_IF(make_map(&ma, A, (uint64_t)K, (uint64_t)M, BM));
  CARC_RETURN_IF(make_map(&mb, B, (uint64_t)K, (uint64_t)N, (uint32_t)bn));
  return launch_any<1>(bn, ma, mb, M, N, BM, nullptr, N, 0, 1, kb_total, kb_total, err, fe, stream);
}

int tma_map_bf16(CUtensorMap* map, const void* base, uint64_t inner, uint64_t rows, uint32_t box_rows) {
  return make_map(map, base, inner, rows, box_rows);
}

int gemm_effective_ksplit(int K, int ksplit) {
  const int kb_total = K / BK;
  ksplit = std::max(1, std::min(ksplit, kb_total));
  const int kb_per = (kb_total + ksplit - 1) / ksplit;
  return (kb_total + kb_per - 1) / kb_per;
}

// ---------------------------------------------------------------------------
// packing of complex128 operands into split-BF16 K-major form
// ---------------------------------------------------------------------------
namespace {

struct PackParams {
  int nr, nk;                 // row / k sub-dimension counts
  int64_t r_ext[CARC_MAX_SUBDIMS], r_str[CARC_MAX_SUBDIMS];
  int64_t k_ext[CARC_MAX_SUBDIMS], k_str[CARC_MAX_SUBDIMS];
  int64_t R, Kc;              // logical complex rows / k
  int64_t rows_out, kp_out;   // padded output rows and row pitch (bf16 columns)
  int64_t col_off;            // first column of this operand's K region
  int conj;
};

__device__ __forceinline__ int64_t pdecomp(int64_t idx, int n, const int64_t* ext, const int64_t* str) {
  int64_t off = 0;
  for (int j = n - 1; j >= 0; --j) {
    int64_t q = idx % ext[j];
    idx /= ext[j];
    off += q * str[j];
  }
  return off;
}

__device__ __forceinline__ void split_bf16(double v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  float f = (float)v;
  hi = __float2bfloat16_rn(f);
  lo = __float2bfloat16_rn(f - __bfloat162float(hi));
}

// A role: out row (m, c, s) (4 per complex row), column (h, k, c') for h in {0,1}
__global__ void pack_a_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                              const __grid_constant__ PackParams p) {
  const int64_t total = p.rows_out / 4 * p.Kc;  // one thread per (m, k) complex element, padded rows included
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / p.Kc, k = t % p.Kc;
    double2 a = make_double2(0.0, 0.0);
    if (m < p.R) {
      a = X[pdecomp(m, p.nr, p.r_ext, p.r_str) + pdecomp(k, p.nk, p.k_ext, p.k_str)];
      if (p.conj) a.y = -a.y;
    }
    // (c, c') entries of the real embedding: [[a_r, -a_i], [a_i, a_r]]
    const double e[2][2] = {{a.x, -a.y}, {a.y, a.x}};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) {
        __nv_bfloat16 hi, lo;
        split_bf16(e[c][cp], hi, lo);
        const int64_t col0 = p.col_off + 2 * k + cp, col1 = p.col_off + 2 * p.Kc + 2 * k + cp;
        __nv_bfloat16* r_hi = out + (4 * m + 2 * c + 0) * p.kp_out;
        __nv_bfloat16* r_lo = out + (4 * m + 2 * c + 1) * p.kp_out;
        r_hi[col0] = hi;
        r_hi[col1] = hi;
        r_lo[col0] = lo;
        r_lo[col1] = lo;
      }
    }
  }
}

// B role: out row n, column (h, k, c'): part h of [b_r, b_i]
__global__ void pack_b_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                              const __grid_constant__ PackParams p) {
  const int64_t total = p.rows_out * p.Kc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = t / p.Kc, k = t % p.Kc;
    double2 b = make_double2(0.0, 0.0);
    if (n < p.R) {
      b = X[pdecomp(n, p.nr, p.r_ext, p.r_str) + pdecomp(k, p.nk, p.k_ext, p.k_str)];
      if (p.conj) b.y = -b.y;
    }
    __nv_bfloat16 hr, lr, hi_, li_;
    split_bf16(b.x, hr, lr);
    split_bf16(b.y, hi_, li_);
    __nv_bfloat16* row = out + n * p.kp_out + p.col_off;
    row[2 * k] = hr;
    row[2 * k + 1] = hi_;
    row[2 * p.Kc + 2 * k] = lr;
    row[2 * p.Kc + 2 * k + 1] = li_;
  }
}

// zero columns [c0, c1) of every row (row pitch kp)
__global__ void pack_pad_kernel(__nv_bfloat16* __restrict__ out, int64_t rows, int64_t c0, int64_t c1, int64_t kp) {
  const int64_t w = c1 - c0;
  const int64_t total = rows * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    out[(t / w) * kp + c0 + t % w] = __float2bfloat16_rn(0.f);
}

struct ReduceParams {
  int nm, nn;
  int64_t m_ext[CARC_MAX_SUBDIMS], m_str[CARC_MAX_SUBDIMS];
  int64_t n_ext[CARC_MAX_SUBDIMS], n_str[CARC_MAX_SUBDIMS];
  int64_t Mc, Nc;       // logical complex output extents
  int64_t ld, split_stride;
  int ksplit;
  int accumulate;
  double2 alpha;
};

// C[m,n] (+)= alpha * sum_z sum_s (P[z][4m+s][n] + i P[z][4m+2+s][n])
__global__ void reduce_kernel(const float* __restrict__ P, double2* __restrict__ C, const __grid_constant__ ReduceParams p) {
  const int64_t total = p.Mc * p.Nc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / p.Nc, n = t % p.Nc;
    Kahan re, im;
    for (int z = 0; z < p.ksplit; ++z) {
      const float* b = P + z * p.split_stride + (4 * m) * p.ld + n;
      re.add(b[0]);
      re.add(b[p.ld]);
      im.add(b[2 * p.ld]);
      im.add(b[3 * p.ld]);
    }
    double2 v = cmul(p.alpha, make_double2(re.value(), im.value()));
    const int64_t off = pdecomp(m, p.nm, p.m_ext, p.m_str) + pdecomp(n, p.nn, p.n_ext, p.n_str);
    if (p.accumulate) v = cadd(v, C[off]);
    C[off] = v;
  }
}

// C[m,n] (+)= alpha * sum_z (P[z][4m..4m+1][n] + i P[z][4m+2..4m+3][n]), in
// FP64 and in a fixed order: a block covers one complex row m and 32
// consecutive n (lanes: coalesced 128-byte rows), its 8 warps take the planes
// z = w, w+8, ... and the 8 partial sums are added in warp order.
constexpr int RP_WARPS = 8;

// Row-major planes P[z][r][n] (r = 4m + 2c + s): a block covers 32 columns of
// one complex row m, its 8 warps take planes z = w, w+8, ...; the warps'
// compensated partial sums are added in FP64 in warp order.
__global__ __launch_bounds__(32 * RP_WARPS) void reduce_planes_kernel(const float* __restrict__ P,
                                                                       double2* __restrict__ C,
                                                                       const __grid_constant__ ReduceParams p) {
  __shared__ double2 part[RP_WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t m = blockIdx.y;
  const int64_t n = (int64_t)blockIdx.x * 32 + lane;
  Kahan re, im;
  if (n < p.Nc) {
    // four planes (16 loads) in flight per thread before they are summed (in plane order)
    const float* base = P + (4 * m) * p.ld + n;
    for (int z0 = w; z0 < p.ksplit; z0 += 4 * RP_WARPS) {
      float v[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int z = z0 + u * RP_WARPS;
        const float* b = base + z * p.split_stride;
#pragma unroll
        for (int q = 0; q < 4; ++q) v[u][q] = z < p.ksplit ? __ldcg(b + q * p.ld) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        re.add(v[u][0]);
        re.add(v[u][1]);
        im.add(v[u][2]);
        im.add(v[u][3]);
      }
    }
  }
  part[w][lane] = make_double2(re.value(), im.value());
  __syncthreads();
  if (w == 0 && n < p.Nc) {
    double2 v = part[0][lane];
    for (int q = 1; q < RP_WARPS; ++q) v = cadd(v, part[q][lane]);
    v = cmul(p.alpha, v);
    const int64_t off = pdecomp(m, p.nm, p.m_ext, p.m_str) + pdecomp(n, p.nn, p.n_ext, p.n_str);
    if (p.accumulate) v = cadd(v, C[off]);
    C[off] = v;
  }
}

// Column-major planes P[z][n][r] (r = 4m + 2c + s over `rows` rows): a block
// covers one column n and 32 consecutive rows (8 complex m), its 8 warps take
// planes z = w, w+8, ... (coalesced 128-byte loads) with compensated FP32
// sums, the partials are added in FP64 in warp order, then each quad of lanes
// folds its 4 rows into C[m, n].
__global__ __launch_bounds__(32 * RP_WARPS) void reduce_planes_cm_kernel(const float* __restrict__ P,
                                                                          double2* __restrict__ C, int64_t rows,
                                                                          const __grid_constant__ ReduceParams p) {
  __shared__ double part[RP_WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t n = blockIdx.x;
  const int64_t r = (int64_t)blockIdx.y * 32 + lane;
  Kahan acc;
  if (r < rows) {
    // up to 24 plane loads in flight per thread (one round trip for 192
    // planes) before they are summed in plane order
    const float* src = P + n * rows + r;
    for (int z0 = w; z0 < p.ksplit; z0 += 24 * RP_WARPS) {
      float v[24];
#pragma unroll
      for (int u = 0; u < 24; ++u) {
        const int z = z0 + u * RP_WARPS;
        v[u] = z < p.ksplit ? __ldcg(src + z * p.split_stride) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 24; ++u) acc.add(v[u]);
    }
  }
  part[w][lane] = acc.value();
  __syncthreads();
  if (w == 0) {
    double v = part[0][lane];
    for (int q = 1; q < RP_WARPS; ++q) v += part[q][lane];
    v += __shfl_xor_sync(0xffffffffu, v, 1);            // hi + lo
    const double o = __shfl_xor_sync(0xffffffffu, v, 2);  // the other of re / im
    const int64_t m = r >> 2;
    if ((lane & 3) == 0 && m < p.Mc) {
      double2 val = cmul(p.alpha, make_double2(v, o));
      const int64_t off = pdecomp(m, p.nm, p.m_ext, p.m_str) + pdecomp(n, p.nn, p.n_ext, p.n_str);
      if (p.accumulate) val = cadd(val, C[off]);
      C[off] = val;
    }
  }
}

inline int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * 152)); }

PackParams pack_params(const ZView& v, int64_t rows_out, int64_t kp_out, int64_t col_off) {
  PackParams p;
  std::memset(&p, 0, sizeof(p));
  p.nr = v.nr;
  p.nk = v.nk;
  p.R = 1;
  p.Kc = 1;
  for (int i = 0; i < v.nr; ++i) {
    p.r_ext[i] = v.r_ext[i];
    p.r_str[i] = v.r_str[i];
    p.R *= v.r_ext[i];
  }
  for (int i = 0; i < v.nk; ++i) {
    p.k_ext[i] = v.k_ext[i];
    p.k_str[i] = v.k_str[i];
    p.Kc *= v.k_ext[i];
  }
  p.rows_out = rows_out;
  p.kp_out = kp_out;
  p.col_off = col_off;
  p.conj = v.conj;
  return p;
}

}  // namespace

int64_t zview_rows(const ZView& v) {
  int64_t r = 1;
  for (int i = 0; i < v.nr; ++i) r *= v.r_ext[i];
  return r;
}

int64_t zview_k(const ZView& v) {
  int64_t r = 1;
  for (int i = 0; i < v.nk; ++i) r *= v.k_ext[i];
  return r;
}

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

int pack_operand_region(const ZView& v, int role, void* out, int64_t rows_out, int64_t kp_out, int64_t col_off,
                        int64_t region, cudaStream_t stream) {
  PackParams p = pack_params(v, rows_out, kp_out, col_off);
  const int64_t kc4 = 4 * p.Kc;
  if (region < kc4 || col_off + region > kp_out)
    return fail(CARC_BAD_ARG, "pack: region [%lld, +%lld) cannot hold 4K = %lld in a row of %lld", (long long)col_off,
                (long long)region, (long long)kc4, (long long)kp_out);
  auto* o = static_cast<__nv_bfloat16*>(out);
  if (role == 0) {
    if (rows_out % 4 != 0 || rows_out / 4 < p.R) return fail(CARC_BAD_ARG, "pack A: rows_out %lld", (long long)rows_out);
    pack_a_kernel<<<grid_of(rows_out / 4 * p.Kc), 256, 0, stream>>>(static_cast<const double2*>(v.base), o, p);
  } else {
    if (rows_out < p.R) return fail(CARC_BAD_ARG, "pack B: rows_out %lld", (long long)rows_out);
    pack_b_kernel<<<grid_of(rows_out * p.Kc), 256, 0, stream>>>(static_cast<const double2*>(v.base), o, p);
  }
  CARC_CHECK_LAUNCH();
  if (region > kc4) {
    pack_pad_kernel<<<grid_of(rows_out * (region - kc4)), 256, 0, stream>>>(o, rows_out, col_off + kc4,
                                                                             col_off + region, kp_out);
    CARC_CHECK_LAUNCH();
  }
  return CARC_OK;
}

int pack_operand(const ZView& v, int role, void* out, int64_t rows_out, int64_t kp_out, cudaStream_t stream) {
  return pack_operand_region(v, role, out, rows_out, kp_out, 0, kp_out, stream);
}

int reduce_partials(const float* P, int64_t ld, int64_t split_stride, int ksplit, const ZOut& o, double2 alpha,
                    int accumulate, cudaStream_t stream) {
  ReduceParams p;
  std::memset(&p, 0, sizeof(p));
  p.nm = o.nm;
  p.nn = o.nn;
  p.Mc = 1;
  p.Nc = 1;
  for (int i = 0; i < o.nm; ++i) {
    p.m_ext[i] = o.m_ext[i];
    p.m_str[i] = o.m_str[i];
    p.Mc *= o.m_ext[i];
  }
  for (int i = 0; i < o.nn; ++i) {
    p.n_ext[i] = o.n_ext[i];
    p.n_str[i] = o.n_str[i];
    p.Nc *= o.n_ext[i];
  }
  p.ld = ld;
  p.split_stride = split_stride;
  p.ksplit = ksplit;
  p.accumulate = accumulate;
  p.alpha = alpha;
  reduce_kernel<<<grid_of(p.Mc * p.Nc), 256, 0, stream>>>(P, static_cast<double2*>(o.base), p);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}


int64_t reduce_partials2_workspace(int64_t Mc, int64_t Nc, int ksplit) {
  (void)Mc;
  (void)Nc;
  (void)ksplit;
  return 256;
}

int reduce_partials2(const float* P, int64_t ld, int64_t split_stride, int ksplit, const ZOut& o, double2 alpha,
                     int accumulate, void* ws, int64_t ws_bytes, cudaStream_t stream) {
  ReduceParams p;
  std::memset(&p, 0, sizeof(p));
  p.nm = o.nm;
  p.nn = o.nn;
  p.Mc = 1;
  p.Nc = 1;
  for (int i = 0; i < o.nm; ++i) {
    p.m_ext[i] = o.m_ext[i];
    p.m_str[i] = o.m_str[i];
    p.Mc *= o.m_ext[i];
  }
  for (int i = 0; i < o.nn; ++i) {
    p.n_ext[i] = o.n_ext[i];
    p.n_str[i] = o.n_str[i];
    p.Nc *= o.n_ext[i];
  }
  p.ld = ld;
  p.split_stride = split_stride;
  p.ksplit = ksplit;
  p.accumulate = accumulate;
  p.alpha = alpha;
  (void)ws;
  (void)ws_bytes;
  if (p.Mc > 65535) return fail(CARC_TOO_LARGE, "reduce: %lld output rows", (long long)p.Mc);
  dim3 grid((unsigned)((p.Nc + 31) / 32), (unsigned)p.Mc);
  reduce_planes_kernel<<<grid, 32 * RP_WARPS, 0, stream>>>(P, static_cast<double2*>(o.base), p);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int reduce_planes_colmajor(const float* P, int64_t rows, int64_t split_stride, int ksplit, const ZOut& o,
                           double2 alpha, int accumulate, cudaStream_t stream) {
  ReduceParams p;
  std::memset(&p, 0, sizeof(p));
  p.nm = o.nm;
  p.nn = o.nn;
  p.Mc = 1;
  p.Nc = 1;
  for (int i = 0; i < o.nm; ++i) {
    p.m_ext[i] = o.m_ext[i];
    p.m_str[i] = o.m_str[i];
    p.Mc *= o.m_ext[i];
  }
  for (int i = 0; i < o.nn; ++i) {
    p.n_ext[i] = o.n_ext[i];
    p.n_str[i] = o.n_str[i];
    p.Nc *= o.n_ext[i];
  }
  p.split_stride = split_stride;
  p.ksplit = ksplit;
  p.accumulate = accumulate;
  p.alpha = alpha;
  if (4 * p.Mc > rows || rows % 32 != 0) return fail(CARC_BAD_ARG, "reduce: %lld plane rows", (long long)rows);
  if (p.Nc > 0x7fffffff) return fail(CARC_TOO_LARGE, "reduce: %lld output columns", (long long)p.Nc);
  dim3 grid((unsigned)p.Nc, (unsigned)(rows / 32));
  reduce_planes_cm_kernel<<<grid, 32 * RP_WARPS, 0, stream>>>(P, static_cast<double2*>(o.base), rows, p);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// C = alpha A B^T (+ C): the whole split-BF16 complex product
// ---------------------------------------------------------------------------
int64_t zgemm_tc_workspace(const ZView& a, const ZView& b, int ksplit) {
  const int64_t M = zview_rows(a), N = zview_rows(b), Kc = zview_k(a);
  const int64_t rows_a = round_up(4 * M, BM), rows_b = round_up(N, 16), kp = round_up(4 * Kc, BK);
  const int64_t ld = rows_b;
  const int ks = gemm_effective_ksplit((int)kp, ksplit);
  auto al = [](int64_t x) { return (x + 255) / 256 * 256; };
  return al(rows_a * kp * 2) + al(rows_b * kp * 2) + al((int64_t)ks * rows_a * ld * 4) + 256;
}

int zgemm_tc(const ZView& a, const ZView& b, const ZOut& c, double2 alpha, int accumulate, int ksplit, void* ws,
             int64_t ws_bytes, int* err, cudaStream_t stream) {
  const int64_t M = zview_rows(a), N = zview_rows(b), Kc = zview_k(a);
  if (zview_k(b) != Kc) return fail(CARC_BAD_SHAPE, "tensor core GEMM: K mismatch");
  const int64_t rows_a = round_up(4 * M, BM), rows_b = round_up(N, 16), kp = round_up(4 * Kc, BK);
  if (rows_a > (1ll << 30) || rows_b > (1ll << 30) || kp > (1ll << 30)) return fail(CARC_TOO_LARGE, "tensor core GEMM: too large");
  if (ws_bytes < zgemm_tc_workspace(a, b, ksplit)) return fail(CARC_BAD_ARG, "tensor core GEMM: workspace too small");
  auto al = [](int64_t x) { return (x + 255) / 256 * 256; };
  char* p = static_cast<char*>(ws);
  void* A_op = p;
  void* B_op = p + al(rows_a * kp * 2);
  float* P = reinterpret_cast<float*>(p + al(rows_a * kp * 2) + al(rows_b * kp * 2));
  CARC_RETURN_IF(pack_operand(a, 0, A_op, rows_a, kp, stream));
  CARC_RETURN_IF(pack_operand(b, 1, B_op, rows_b, kp, stream));
  const int ks = gemm_effective_ksplit((int)kp, ksplit);
  const int64_t ld = rows_b;
  CARC_RETURN_IF(gemm_bf16_tn(A_op, (int)rows_a, B_op, (int)rows_b, (int)kp, P, ld, ks, err, stream));
  return reduce_partials(P, ld, (int64_t)rows_a * ld, ks, c, alpha, accumulate, stream);
}

ZView zview_a(const carc_contract_desc& d, const void* base) {
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = d.nm;
  v.nk = d.nk;
  for (int i = 0; i < d.nm; ++i) {
    v.r_ext[i] = d.m_ext[i];
    v.r_str[i] = d.a_m[i];
  }
  for (int i = 0; i < d.nk; ++i) {
    v.k_ext[i] = d.k_ext[i];
    v.k_str[i] = d.a_k[i];
  }
  v.conj = d.conj_a;
  return v;
}

ZView zview_b(const carc_contract_desc& d, const void* base) {
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = d.nn;
  v.nk = d.nk;
  for (int i = 0; i < d.nn; ++i) {
    v.r_ext[i] = d.n_ext[i];
    v.r_str[i] = d.b_n[i];
  }
  for (int i = 0; i < d.nk; ++i) {
    v.k_ext[i] = d.k_ext[i];
    v.k_str[i] = d.b_k[i];
  }
  v.conj = d.conj_b;
  return v;
}

ZOut zout_c(const carc_contract_desc& d, void* base) {
  ZOut o;
  memset(&o, 0, sizeof(o));
  o.base = base;
  o.nm = d.nm;
  o.nn = d.nn;
  for (int i = 0; i < d.nm; ++i) {
    o.m_ext[i] = d.m_ext[i];
    o.m_str[i] = d.c_m[i];
  }
  for (int i = 0; i < d.nn; ++i) {
    o.n_ext[i] = d.n_ext[i];
    o.n_str[i] = d.c_n[i];
  }
  return o;
}

}  // namespace carc
