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
#include <vector>

namespace carc {

namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // bf16 elements per K block (128 bytes)
constexpr int THREADS = 192;
constexpr int A_STAGE_BYTES = BM * BK * 2;

__host__ __device__ constexpr int tmem_cols_for(int bn) { return bn <= 32 ? 32 : (bn <= 64 ? 64 : (bn <= 128 ? 128 : 256)); }

// The plain GEMM streams long K ranges: 4 pipeline stages, one CTA per SM.
constexpr int STAGES = 4;

template <int BN>
constexpr int smem_bytes() {
  return 1024 + STAGES * (A_STAGE_BYTES + BN * BK * 2) + 256;
}

// ---- folding epilogue --------------------------------------------------------
// The tile's accumulator is 128 rows (4m + 2c + s: complex row m, re/im c,
// hi/lo s) x BN columns n.  It is staged HC columns at a time as FP32 with a
// row pitch of HC + 4 floats (conflict-free float4 stores), the columns in
// slot order: when the physical dimension d is 2, 4 or 8 (and HC >= 32),
// p-major (slot (n % d) HC/d + n / d), so that consecutive slots walk (vec,
// k2, k3), i.e. consecutive destination k, and consecutive lanes read
// consecutive words; otherwise in column order.  After the staged block come
// two index tables: per complex row m of the tile {row part, k part} of the
// destination (row part -1: past M), and per slot {row part, k part} (row
// part -1: past N).  Destination row = sum of the row parts, complex k = sum
// of the k parts.
template <int BN>
__host__ __device__ constexpr int FOLD_HC() { return BN == 256 ? 128 : (BN == 128 ? 64 : BN); }

template <int BN>
__host__ __device__ constexpr int FOLD_PITCH() { return FOLD_HC<BN>() + 4; }

template <int BN>
__host__ __device__ constexpr int fold_smem_bytes() { return 128 * FOLD_PITCH<BN>() * 4 + 32 * 8 + FOLD_HC<BN>() * 8; }

// slot-order stride: d when the staged columns are p-major, 1 otherwise
template <int BN>
__device__ __forceinline__ int fold_ds(int64_t d) {
  constexpr int HC = FOLD_HC<BN>();
  return (HC >= 32 && (d == 2 || d == 4 || d == 8)) ? (int)d : 1;
}

// one lane's 32 accumulator columns [c0, c0 + 32) of its row into slot order
template <int BN, int DS>
__device__ __forceinline__ void fold_stage(float* row, int c0, const uint32_t* r) {
  constexpr int HC = FOLD_HC<BN>();
  if constexpr (HC < 32 || DS == 1) {
#pragma unroll
    for (int j = 0; j < 32; j += 4) {
      if (c0 + j >= HC) break;
      *reinterpret_cast<float4*>(row + c0 + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                             __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
    }
  } else {
    // column c0 + p + DS i goes to slot p HC/DS + c0/DS + i
#pragma unroll
    for (int p = 0; p < DS; ++p) {
#pragma unroll
      for (int i = 0; i < 32 / DS; i += 4) {
        *reinterpret_cast<float4*>(row + p * (HC / DS) + c0 / DS + i) =
            make_float4(__uint_as_float(r[p + DS * i]), __uint_as_float(r[p + DS * (i + 1)]),
                        __uint_as_float(r[p + DS * (i + 2)]), __uint_as_float(r[p + DS * (i + 3)]));
      }
    }
  }
}

template <int BN>
__device__ __forceinline__ void fold_tables(float* sP, const FoldEpi& fe, int m0, int nb, int ds, int tid,
                                            int nthreads) {
  constexpr int HC = FOLD_HC<BN>();
  int2* tabM = reinterpret_cast<int2*>(sP + 128 * FOLD_PITCH<BN>());
  int2* tabN = tabM + 32;
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
  const int per = HC / ds;
  for (int q = tid; q < HC; q += nthreads) {
    const int nl = (q % per) * ds + q / per;
    const int64_t n = (int64_t)nb + nl;
    int2 t = make_int2(-1, 0);
    if (n < fe.N) {
      int r = (int)n;
      const int p = r % Dp; r /= Dp;
      const int k3 = r % K3; r /= K3;
      const int k2 = r % K2; r /= K2;
      t = make_int2(r * L0 * L1 * Dp + p, k2 * K3 + k3);
    }
    tabN[q] = t;
  }
}

// W[m, n] = (P[4m] + P[4m+1]) + i (P[4m+2] + P[4m+3]), split into bf16 hi/lo
// pairs.  Warp w of nw (nw a multiple of the HC/32 slot groups) takes slot
// group w % (HC/32) and every (nw / (HC/32))-th complex row: each lane keeps
// its slot's destination parts in registers, reads one consecutive staged
// word per row and stores consecutive k of one destination row with its
// neighbours (one 128-byte run of a K block).
template <int BN>
__device__ __forceinline__ void fold_write(const float* sP, const FoldEpi& fe, int warp, int nw) {
  constexpr int HC = FOLD_HC<BN>();
  constexpr int PITCH = FOLD_PITCH<BN>();
  constexpr int JQ = (HC + 31) / 32;  // 32-slot groups per row
  const int2* tabM = reinterpret_cast<const int2*>(sP + 128 * PITCH);
  const int2* tabN = tabM + 32;
  const int lane = threadIdx.x & 31;
  const int q = (warp % JQ) * 32 + lane;
  const int rstep = nw / JQ;
  if (q >= HC) return;
  const int2 tn = tabN[q];
  if (tn.x < 0) return;
  // bf16 (re, im) pairs in K blocks of 32 pairs x rows (col_off is even)
  uint32_t* W = static_cast<uint32_t*>(fe.dst);
  const int rows32 = (int)fe.rows * 32;
  const int cp_lane = (int)(fe.col_off >> 1) + tn.y;
  const int kc = (int)fe.kc;
  const float* col = sP + q;
#pragma unroll 4
  for (int ml = warp / JQ; ml < 32; ml += rstep) {
    const int2 tm = tabM[ml];
    if (tm.x < 0) continue;
    const float* c = col + 4 * ml * PITCH;
    const float re = c[0] + c[PITCH];
    const float im = c[2 * PITCH] + c[3 * PITCH];
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(re, im);
    const float2 hf = __bfloat1622float2(h2);
    const __nv_bfloat162 l2 = __floats2bfloat162_rn(re - hf.x, im - hf.y);
    const int row32 = (tn.x + tm.x) * 32;
    const int cp = cp_lane + tm.y, cl = cp + kc;
    W[(int64_t)(cp >> 5) * rows32 + row32 + (cp & 31)] = *reinterpret_cast<const uint32_t*>(&h2);
    W[(int64_t)(cl >> 5) * rows32 + row32 + (cl & 31)] = *reinterpret_cast<const uint32_t*>(&l2);
  }
}

// Plain GEMM: out[z][m][n] = sum over split z's K blocks of A[m,:] . B[n,:].
// The N tile is bn: BN, or (on the BN = 256 instance) any multiple of 16 up
// to 256 chosen at run time; shared-memory stages and TMEM are sized for BN.
// One tile: A rows [a_y, a_y + 128) and B rows [b_y, b_y + bn) over the K
// blocks [kb0, kb0 + nkb), accumulated in TMEM and stored as FP32 at
// out_tile (row pitch ld_out).
template <int BN>
__device__ __forceinline__ void gemm_tile(const CUtensorMap* tmA, const CUtensorMap* tmB, float* __restrict__ out_tile,
                                          int64_t ld_out, int a_y, int b_y, int kb0, int nkb, int a_rows,
                                          int* __restrict__ err, int bn, int b_blk) {
  using namespace umma;
  constexpr int B_STAGE_BYTES = BN * BK * 2;
  constexpr uint32_t TMEM_COLS = tmem_cols_for(BN);
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
      prefetch_tensormap(tmA);
      prefetch_tensormap(tmB);
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)((i / STAGES) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag)) break;
        mbar_arrive_expect_tx(&full[s], (uint32_t)(a_rows * BK * 2 + bn * BK * 2));
        const int kx = (kb0 + i) * BK;
        tma_load_2d(sA + s * A_STAGE_BYTES, tmA, kx, a_y, &full[s]);
        if (b_blk)
          tma_load_3d(sB + s * B_STAGE_BYTES, tmB, 0, b_y, kb0 + i, &full[s]);
        else
          tma_load_2d(sB + s * B_STAGE_BYTES, tmB, kx, b_y, &full[s]);
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
      const uint32_t idesc = idesc_bf16_f32(BM, bn);
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
    // epilogue: warps 2..5 own TMEM lane quadrants (warp % 4); they wait for
    // the whole main loop, suspended in hardware so that they take no issue
    // slots from the producer and the MMA issuer
    const int quad = warp & 3;
    const bool ok = mbar_wait_sleep(done, 0, abort_flag);
    tc_fence_after();
    if (ok) {
      float* dst = out_tile + (int64_t)(quad * 32 + lane) * ld_out;
#pragma unroll 1
      for (int c0 = 0; c0 < bn; c0 += 32) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
        tmem_ld_wait();
        // a tile whose width is not a multiple of 32 reads allocated columns
        // past it but stores only its own
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          if (c0 + j >= bn) break;
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
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, CARC_NOT_CONVERGED);
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

template <int BN>
__global__ __launch_bounds__(THREADS, 1) void gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                  const __grid_constant__ CUtensorMap tmB,
                                                                  float* __restrict__ out, int64_t ld_out,
                                                                  int64_t split_stride, int kb_per_split,
                                                                  int kb_total, int a_rows, int* __restrict__ err,
                                                                  int bn, int b_blk) {
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * bn;
  const int kb0 = blockIdx.z * kb_per_split;
  const int nkb = max(0, min(kb_total, kb0 + kb_per_split) - kb0);
  gemm_tile<BN>(&tmA, &tmB, out + (int64_t)blockIdx.z * split_stride + (int64_t)m0 * ld_out + n0, ld_out, m0, n0,
                kb0, nkb, a_rows, err, bn, b_blk);
}

// Grouped GEMM over a table of (A block, B block) pairs of one shape feeding
// a set of outputs: the A operands are stacked in one buffer (a_rows_per rows
// each), the B operands in another (b_rows_per rows each), so one tensor map
// covers each.  CTA (m tile, n tile, o ks + z) chains the K blocks of split z
// of every entry of output o (entries e_first[o] .. e_first[o+1]-1, in table
// order) through one TMEM accumulator.  With one split the epilogue writes
// the complex FP64 result straight into output o; with several it writes an
// FP32 plane (o ks + z) for the grouped reduction.
struct GemmGroup {
  int n_out, ks, a_rows_per, b_rows_per, kb_total, kb_per;
  int e_first[CARC_MAX_SLOTS + 1];
  int2 ij[CARC_MAX_ENTRIES];
};

struct GroupEpi {
  int nm, nn, accumulate, alpha_one;
  int64_t m_ext[CARC_MAX_SUBDIMS], m_str[CARC_MAX_SUBDIMS];
  int64_t n_ext[CARC_MAX_SUBDIMS], n_str[CARC_MAX_SUBDIMS];
  int64_t Mc, Nc;
  double2 alpha;
  double2* dst[CARC_MAX_SLOTS];
};

// float -> double by its bit fields (IEEE 754: exponent rebased by 1023 - 127,
// mantissa moved up 29 bits), on the integer pipe: the conversion instruction
// issues on the FP64 pipe, whose rate is low on this part.  Infinities and
// NaNs map to their double counterparts; float subnormals (below 1.2e-38,
// far under the 1e-5 scale of the split-precision result's error) to zero.
__device__ __forceinline__ double f32_to_f64_int(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint32_t hi, lo;
  if (e == 0u) {
    hi = sign;
    lo = 0u;
  } else {
    const uint32_t ed = e == 0xffu ? 0x7ffu : e + (1023u - 127u);
    hi = sign | (ed << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ int64_t epi_decomp(int64_t idx, int n, const int64_t* ext, const int64_t* str) {
  int64_t off = 0;
  for (int j = n - 1; j >= 0; --j) {
    const int64_t q = idx % ext[j];
    idx /= ext[j];
    off += q * str[j];
  }
  return off;
}

template <int BN, int NST>
__global__ __launch_bounds__(THREADS, 1) void gemm_bf16_tn_grouped_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                          const __grid_constant__ CUtensorMap tmB,
                                                                          float* __restrict__ planes, int64_t ld,
                                                                          int64_t plane_stride, int* __restrict__ err,
                                                                          int bn, const __grid_constant__ GemmGroup grp,
                                                                          const __grid_constant__ GroupEpi epi) {
  using namespace umma;
  constexpr int B_STAGE_BYTES = BN * BK * 2;
  constexpr uint32_t TMEM_COLS = tmem_cols_for(BN);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + NST * A_STAGE_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + NST * B_STAGE_BYTES);
  uint64_t* empty = full + NST;
  uint64_t* done = empty + NST;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = blockIdx.z / grp.ks, z = blockIdx.z - o * grp.ks;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * bn;
  const int kb0 = z * grp.kb_per;
  const int nkb = max(0, min(grp.kb_total, kb0 + grp.kb_per) - kb0);
  const int e0 = grp.e_first[o];
  const int n_iter = (grp.e_first[o + 1] - e0) * nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer: the K blocks of split z of each entry, entry after entry
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      int issued = 0;
      for (int i = 0; i < n_iter; ++i) {
        const int s = i % NST;
        const uint32_t ph = (uint32_t)((i / NST) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag)) break;
        const int q = i / nkb, e = e0 + q;
        const int kx = (kb0 + i - q * nkb) * BK;
        mbar_arrive_expect_tx(&full[s], (uint32_t)(BM * BK * 2 + bn * BK * 2));
        tma_load_2d(sA + s * A_STAGE_BYTES, &tmA, kx, grp.ij[e].x * grp.a_rows_per + m0, &full[s]);
        tma_load_2d(sB + s * B_STAGE_BYTES, &tmB, kx, grp.ij[e].y * grp.b_rows_per + n0, &full[s]);
        ++issued;
      }
      if (*abort_flag) {
        // let copies already in flight land before the CTA exits (bounded)
        for (int i = max(0, issued - NST); i < issued; ++i) {
          const int s = i % NST;
          for (uint32_t t = 0; t < (1u << 20); ++t)
            if (mbar_try_wait(&full[s], (uint32_t)((i / NST) & 1))) break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(BM, bn);
      for (int i = 0; i < n_iter; ++i) {
        const int s = i % NST;
        const uint32_t ph = (uint32_t)((i / NST) & 1);
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
    // epilogue: warps 2..5 (TMEM lane quadrant warp % 4)
    const int quad = warp & 3;
    const int et = threadIdx.x - 64;  // 0..127
    int64_t* ntab = reinterpret_cast<int64_t*>(reinterpret_cast<uint8_t*>(full) + 256);  // bn column offsets
    int64_t* mtab = ntab + 256;                                                          // 32 row offsets
    if (grp.ks == 1) {
      // output offsets of the tile's columns and complex rows, while the main loop runs
      for (int q = et; q < bn; q += 128) {
        const int64_t n = (int64_t)n0 + q;
        ntab[q] = n < epi.Nc ? epi_decomp(n, epi.nn, epi.n_ext, epi.n_str) : -1;
      }
      if (et < 32) {
        const int64_t m = (int64_t)(m0 >> 2) + et;
        mtab[et] = m < epi.Mc ? epi_decomp(m, epi.nm, epi.m_ext, epi.m_str) : -1;
      }
    }
    const bool waited = mbar_wait_sleep(done, 0, abort_flag);
    // one decision for the four epilogue warps (named barrier 1), which also
    // publishes the offset tables
    uint32_t all_ok;
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 q, %1, 0;\n"
        "bar.red.and.pred p, 1, 128, q;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(all_ok)
        : "r"((uint32_t)waited)
        : "memory");
    tc_fence_after();
    if (all_ok) {
      const int row = m0 + quad * 32 + lane;
      if (grp.ks > 1) {
        float* dst = planes + (int64_t)blockIdx.z * plane_stride + (int64_t)row * ld + n0;
#pragma unroll 1
        for (int c0 = 0; c0 < bn; c0 += 32) {
          uint32_t r[32];
          tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 32; j += 4) {
            if (c0 + j >= bn) break;
            *reinterpret_cast<float4*>(dst + c0 + j) =
                n_iter > 0 ? make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                                         __uint_as_float(r[j + 3]))
                           : make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      } else {
        // 32 columns at a time through shared memory (the A stages, free once
        // every MMA has completed): rows 4m + 2c + s staged with a pitch of 33
        // floats, then each thread forms C[m, n] = (hi + lo) + i (hi + lo) in
        // FP64 for one column n of several complex rows m, consecutive n on
        // consecutive lanes (coalesced stores into the output)
        float* stage = reinterpret_cast<float*>(sA);
        double2* C = epi.dst[o];
        const int nl = et & 31;
#pragma unroll 1
        for (int c0 = 0; c0 < bn; c0 += 32) {
          uint32_t r[32];
          tmem_ld_32x32b_x32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
          tmem_ld_wait();
          float* srow = stage + (quad * 32 + lane) * 33;
#pragma unroll
          for (int j = 0; j < 32; ++j) srow[j] = n_iter > 0 ? __uint_as_float(r[j]) : 0.f;
          asm volatile("bar.sync 1, 128;" ::: "memory");
          const int64_t no = c0 + nl < bn ? ntab[c0 + nl] : -1;
#pragma unroll 2
          for (int i = et >> 5; i < 32; i += 4) {
            const int64_t mo = mtab[i];
            if (mo >= 0 && no >= 0) {
              // hi + lo in FP32 (6e-8 relative, far below the split's 1e-5) and
              // converted on the integer pipe: no FP64 instruction, whose issue
              // rate is low on this part, unless alpha != 1 or C is added
              const float* sv = stage + (4 * i) * 33 + nl;
              double2 val = make_double2(f32_to_f64_int(__fadd_rn(sv[0], sv[33])),
                                         f32_to_f64_int(__fadd_rn(sv[66], sv[99])));
              if (!epi.alpha_one) val = cmul(epi.alpha, val);
              if (epi.accumulate) val = cadd(val, C[mo + no]);
              C[mo + no] = val;
            }
          }
          asm volatile("bar.sync 1, 128;" ::: "memory");
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, CARC_NOT_CONVERGED);
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---- persistent folding GEMM --------------------------------------------------
// W = A . B^T folded into the step-B operand (the epilogue above), as a
// persistent warp-specialised kernel: one CTA per SM walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... N-tile-fastest (the N tiles of one M tile run
// on neighbouring SMs at the same time, so the A tile is read from HBM once).
//   warp 0        TMA producer: A and B K-blocks through fg_stages<BN>()
//                 stages (3 at BN = 256, else 4), running ahead into the
//                 next tiles
//   warp 1        MMA issuer: tile i into TMEM accumulator i % 2
//   warps 2..17   epilogue: accumulator -> staged FP32 block (four warps
//                 per TMEM lane quadrant) -> fold -> W; they release the
//                 accumulator as soon as its last columns are staged, so
//                 the MMAs of tile i + 2 overlap the fold of tile i.
// Every wait is bounded; on expiry the CTA raises its abort flag, stops,
// lets its copies and MMAs land, frees TMEM and reports CARC_NOT_CONVERGED.
constexpr int FG_EPI_WARPS = 16;
constexpr int FG_THREADS = 32 * (2 + FG_EPI_WARPS);
// the second configuration: two CTAs per SM, each with 8 fold warps, two
// stages and 128-column tiles (about 100 KB of shared memory and 256 TMEM
// columns per CTA), so that one CTA's fold overlaps the other's loads and MMAs
constexpr int FG2_EPI_WARPS = 8;
constexpr int FG2_STAGES = 2;

template <int BN>
__host__ __device__ constexpr int fg_stage_bytes() { return A_STAGE_BYTES + BN * BK * 2; }

template <int BN>
__host__ __device__ constexpr int fg_stages() {
  // up to 4 stages next to the staged block, within the 227 KB opt-in limit
  return (227 * 1024 - 1024 - fold_smem_bytes<BN>() - 256) / fg_stage_bytes<BN>() >= 4
             ? 4
             : (227 * 1024 - 1024 - fold_smem_bytes<BN>() - 256) / fg_stage_bytes<BN>();
}

template <int BN>
__host__ __device__ constexpr int fg_smem_bytes() {
  return 1024 + fg_stages<BN>() * fg_stage_bytes<BN>() + fold_smem_bytes<BN>() + 256;
}

template <int BN, int NST>
__host__ __device__ constexpr int fg_smem_bytes_st() {
  return 1024 + NST * fg_stage_bytes<BN>() + fold_smem_bytes<BN>() + 256;
}

// OR of a predicate over the epilogue warps (named barrier 1): every one of
// them takes the same branch after a wait that may have given up.
template <int EPIW>
__device__ __forceinline__ bool fg_epilogue_any(bool v) {
  uint32_t r;
  asm volatile(
      "{\n"
      ".reg .pred p, q;\n"
      "setp.ne.u32 q, %1, 0;\n"
      "bar.red.or.pred p, 1, %2, q;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(32 * EPIW)
      : "memory");
  return r != 0;
}

template <int BN, int EPIW, int NST>
__global__ __launch_bounds__(32 * (2 + EPIW), EPIW == EPIW ? 1 : 2) void fold_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                  const __grid_constant__ CUtensorMap tmB,
                                                                  int n_tiles, int tiles, int nkb, int* __restrict__ err,
                                                                  const __grid_constant__ FoldEpi fe) {
  using namespace umma;
  constexpr int STAGES = NST;
  static_assert(STAGES >= 2, "the folding GEMM needs at least two pipeline stages");
  static_assert(EPIW % ((FOLD_HC<BN>() + 31) / 32) == 0, "epilogue warps per slot group");
  constexpr int B_STAGE_BYTES = BN * BK * 2;
  constexpr uint32_t ACC_COLS = tmem_cols_for(BN);
  constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  constexpr int HC = FOLD_HC<BN>();
  constexpr int EPI_THREADS = 32 * EPIW;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_STAGE_BYTES;
  float* sP = reinterpret_cast<float*>(sB + STAGES * B_STAGE_BYTES);
  uint64_t* full = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(sP) + fold_smem_bytes<BN>());
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;   // [2] MMAs of the buffer's tile done
  uint64_t* acc_empty = acc_full + 2;    // [2] the buffer's columns staged (one arrival per epilogue warp)
  uint64_t* done = acc_empty + 2;        // every MMA issued has completed (abort path)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int my_tiles = blockIdx.x < tiles ? (tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], EPIW);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      int c = 0;  // K-blocks issued by this CTA
      for (int i = 0; i < my_tiles && !*abort_flag; ++i) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        const int m0 = (t / n_tiles) * BM, n0 = (t % n_tiles) * BN;
        for (int kb = 0; kb < nkb; ++kb, ++c) {
          const int s = c % STAGES;
          if (!mbar_wait(&empty[s], (uint32_t)(((c / STAGES) & 1) ^ 1), abort_flag)) break;
          mbar_arrive_expect_tx(&full[s], (uint32_t)(A_STAGE_BYTES + B_STAGE_BYTES));
          tma_load_2d(sA + s * A_STAGE_BYTES, &tmA, kb * BK, m0, &full[s]);
          tma_load_2d(sB + s * B_STAGE_BYTES, &tmB, kb * BK, n0, &full[s]);
        }
      }
      if (*abort_flag) {
        // let the copies in flight land before the CTA exits (bounded)
        for (int j = max(0, c - STAGES); j < c; ++j) {
          const int s = j % STAGES;
          for (uint32_t k = 0; k < (1u << 20); ++k)
            if (mbar_try_wait(&full[s], (uint32_t)((j / STAGES) & 1))) break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(BM, BN);
      int c = 0;
      for (int i = 0; i < my_tiles && !*abort_flag; ++i) {
        const int b = i & 1;
        // the epilogue has staged this buffer's previous tile (i - 2)
        if (!mbar_wait(&acc_empty[b], (uint32_t)(((i >> 1) & 1) ^ 1), abort_flag)) break;
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)b * ACC_COLS;
        bool ok = true;
        for (int kb = 0; kb < nkb; ++kb, ++c) {
          const int s = c % STAGES;
          if (!mbar_wait(&full[s], (uint32_t)((c / STAGES) & 1), abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_base = smem_u32(sA + s * A_STAGE_BYTES);
          const uint32_t b_base = smem_u32(sB + s * B_STAGE_BYTES);
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(acc, smem_desc_sw128(a_base + kk * 32), smem_desc_sw128(b_base + kk * 32), idesc,
                     (kb > 0 || kk > 0) ? 1u : 0u);
          mma_commit(&empty[s]);
        }
        if (!ok) break;
        mma_commit(&acc_full[b]);
      }
      // every MMA issued has landed before TMEM is freed (bounded)
      mma_commit(done);
      for (uint32_t k = 0; k < (1u << 22); ++k)
        if (mbar_try_wait(done, 0)) break;
    }
  } else {
    // epilogue warps: e = 0..15, TMEM lane quadrant warp % 4, column block
    // phase h (each 32-column block of a quadrant goes to one of its warps)
    constexpr int PER_QUAD = EPIW / 4;
    const int e = warp - 2, quad = warp & 3, h = e >> 2;
    const int ds = fold_ds<BN>(fe.d);
    for (int i = 0; i < my_tiles; ++i) {
      const int b = i & 1;
      const int t = (int)blockIdx.x + i * (int)gridDim.x;
      const int m0 = (t / n_tiles) * BM, n0 = (t % n_tiles) * BN;
      const bool got = mbar_wait_sleep(&acc_full[b], (uint32_t)((i >> 1) & 1), abort_flag);
      if (fg_epilogue_any<EPIW>(!got)) break;  // all epilogue warps leave together
      tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)b * ACC_COLS + ((uint32_t)(quad * 32) << 16);
      for (int h0 = 0; h0 < BN; h0 += HC) {
        // the previous block's fold has read the staged block and the tables
        asm volatile("bar.sync 1, %0;" ::"n"(EPI_THREADS) : "memory");
        float* row = sP + (quad * 32 + lane) * FOLD_PITCH<BN>();
#pragma unroll 1
        for (int c0 = 32 * h; c0 < HC; c0 += 32 * PER_QUAD) {
          uint32_t r[32];
          tmem_ld_32x32b_x32(acc + (uint32_t)(h0 + c0), r);
          tmem_ld_wait();
          switch (ds) {
            case 2: fold_stage<BN, 2>(row, c0, r); break;
            case 4: fold_stage<BN, 4>(row, c0, r); break;
            case 8: fold_stage<BN, 8>(row, c0, r); break;
            default: fold_stage<BN, 1>(row, c0, r); break;
          }
        }
        if (h0 + HC >= BN) {
          // the accumulator is staged: the MMAs of tile i + 2 may overwrite it
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
        fold_tables<BN>(sP, fe, m0, n0 + h0, ds, threadIdx.x - 64, EPI_THREADS);
        asm volatile("bar.sync 1, %0;" ::"n"(EPI_THREADS) : "memory");
        fold_write<BN>(sP, fe, e, EPIW);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
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

// 3D tensor map of a K-block-major BF16 operand ([K / 64][rows][64]): box of
// 64 columns x box_rows rows of one K block, 128-byte swizzle; the shared
// memory tile is the same as make_map's.
int make_map_kblocked(CUtensorMap* map, const void* base, uint64_t inner, uint64_t rows, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(CARC_CUDA_ERROR, "tensor core GEMM: cuTensorMapEncodeTiled is unavailable");
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || inner % BK != 0)
    return fail(CARC_BAD_ARG, "tensor core GEMM: K-blocked operand not 16-byte aligned or K not a multiple of 64");
  cuuint64_t dims[3] = {(cuuint64_t)BK, rows, inner / BK};
  cuuint64_t strides[2] = {(cuuint64_t)BK * 2, rows * BK * 2};
  cuuint32_t box[3] = {(cuuint32_t)BK, box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(CARC_CUDA_ERROR, "tensor core GEMM: cuTensorMapEncodeTiled failed (%d)", (int)r);
  return CARC_OK;
}

template <int BN>
int launch_bn(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int a_rows, float* out, int64_t ld_out,
              int64_t split_stride, int ksplit, int kb_per, int kb_total, int* err, cudaStream_t stream, int bn,
              int b_blk) {
  constexpr int SMEM = smem_bytes<BN>();
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(gemm_bf16_tn_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
  });
  if (attr_err != cudaSuccess) return fail(CARC_CUDA_ERROR, "tensor core GEMM: %s", cudaGetErrorString(attr_err));
  const dim3 grid(M / BM, N / bn, ksplit);
  gemm_bf16_tn_kernel<BN><<<grid, THREADS, SMEM, stream>>>(ma, mb, out, ld_out, split_stride, kb_per, kb_total, a_rows,
                                                            err, bn, b_blk);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// shared memory of the grouped GEMM: NST pipeline stages, the barriers and
// the epilogue's offset tables (the staged block reuses the A stages)
template <int BN, int NST>
constexpr int grouped_smem_bytes() {
  return 1024 + NST * (A_STAGE_BYTES + BN * BK * 2) + 256 + (256 + 32) * 8;
}

template <int BN, int NST>
int launch_grouped_bn(const CUtensorMap& ma, const CUtensorMap& mb, int mt, int nt, float* planes, int64_t ld,
                      int64_t plane_stride, int* err, int bn, const GemmGroup& grp, const GroupEpi& epi,
                      cudaStream_t stream) {
  constexpr int SMEM = grouped_smem_bytes<BN, NST>();
  static_assert(SMEM <= 227 * 1024, "grouped GEMM shared memory");
  static_assert(NST * A_STAGE_BYTES >= 128 * 33 * 4, "the staged epilogue block fits in the A stages");
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(gemm_bf16_tn_grouped_kernel<BN, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    SMEM);
  });
  if (attr_err != cudaSuccess) return fail(CARC_CUDA_ERROR, "grouped tensor core GEMM: %s", cudaGetErrorString(attr_err));
  const dim3 grid(mt, nt, grp.n_out * grp.ks);
  gemm_bf16_tn_grouped_kernel<BN, NST><<<grid, THREADS, SMEM, stream>>>(ma, mb, planes, ld, plane_stride, err, bn, grp,
                                                                         epi);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// two pipeline stages (two CTAs per SM) when every output's chain of K
// blocks is short, so the epilogue of one CTA overlaps the other's work
template <int BN>
int launch_grouped_st(bool short_k, const CUtensorMap& ma, const CUtensorMap& mb, int mt, int nt, float* planes,
                      int64_t ld, int64_t plane_stride, int* err, int bn, const GemmGroup& grp, const GroupEpi& epi,
                      cudaStream_t stream) {
  if (short_k) return launch_grouped_bn<BN, 2>(ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
  return launch_grouped_bn<BN, 4>(ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
}

int launch_grouped(int bn, bool short_k, const CUtensorMap& ma, const CUtensorMap& mb, int mt, int nt, float* planes,
                   int64_t ld, int64_t plane_stride, int* err, const GemmGroup& grp, const GroupEpi& epi,
                   cudaStream_t stream) {
  switch (bn) {
    case 128: return launch_grouped_st<128>(short_k, ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
    case 64: return launch_grouped_st<64>(short_k, ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
    case 32: return launch_grouped_st<32>(short_k, ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
    case 16: return launch_grouped_st<16>(short_k, ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
    default:
      if (bn % 16 != 0 || bn < 16 || bn > 256) return fail(CARC_BAD_ARG, "grouped tensor core GEMM: N tile %d", bn);
      return launch_grouped_st<256>(short_k, ma, mb, mt, nt, planes, ld, plane_stride, err, bn, grp, epi, stream);
  }
}

int launch_any(int bn, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int a_rows, float* out,
               int64_t ld_out, int64_t split_stride, int ksplit, int kb_per, int kb_total, int* err,
               cudaStream_t stream, int b_blk) {
  switch (bn) {
    case 256: return launch_bn<256>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
    case 128: return launch_bn<128>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
    case 64: return launch_bn<64>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
    case 32: return launch_bn<32>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
    case 16: return launch_bn<16>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
    default:
      // other widths (multiples of 16 below 256) run on the 256-wide instance
      if (bn % 16 != 0 || bn < 16 || bn > 256) return fail(CARC_BAD_ARG, "tensor core GEMM: N tile %d", bn);
      return launch_bn<256>(ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream, bn, b_blk);
  }
}

}  // namespace

int gemm_tile_n(int N) {
  const int nt = (N + 255) / 256;
  if (N > 0 && N % nt == 0 && (N / nt) % 16 == 0) return N / nt;
  return N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : N % 64 == 0 ? 64 : N % 32 == 0 ? 32 : 16;
}

int64_t gemm_pad_n(int64_t n) {
  if (n <= 0) return 0;
  const int64_t nt = (n + 255) / 256;
  return nt * round_up((n + nt - 1) / nt, 16);
}

int gemm_bf16_tn(const void* A, int M, const void* B, int N, int K, float* out, int64_t ld_out, int ksplit, int* err,
                 cudaStream_t stream, int m_live, int b_blocked) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM != 0 || K % BK != 0 || N % 16 != 0)
    return fail(CARC_BAD_SHAPE, "tensor core GEMM: shape %d x %d x %d not tileable (M%%128, K%%64, N%%16)", M, N, K);
  if (ld_out < N || ld_out % 4 != 0) return fail(CARC_BAD_ARG, "tensor core GEMM: ld_out %lld", (long long)ld_out);
  const int kb_total = K / BK;
  ksplit = std::max(1, std::min(ksplit, kb_total));
  const int kb_per = (kb_total + ksplit - 1) / ksplit;
  ksplit = (kb_total + kb_per - 1) / kb_per;
  const int bn = gemm_tile_n(N);
  // one 128-row tile whose rows >= 64 are zero padding: load only the live half
  const int a_rows = (M == BM && m_live > 0 && m_live <= 64) ? 64 : BM;
  CUtensorMap ma, mb;
  CARC_RETURN_IF(make_map(&ma, A, (uint64_t)K, (uint64_t)M, (uint32_t)a_rows));
  if (b_blocked)
    CARC_RETURN_IF(make_map_kblocked(&mb, B, (uint64_t)K, (uint64_t)N, (uint32_t)bn));
  else
    CARC_RETURN_IF(make_map(&mb, B, (uint64_t)K, (uint64_t)N, (uint32_t)bn));
  const int64_t split_stride = (int64_t)M * ld_out;
  return launch_any(bn, ma, mb, M, N, a_rows, out, ld_out, split_stride, ksplit, kb_per, kb_total, err, stream,
                    b_blocked ? 1 : 0);
}

namespace {

template <int BN, int EPIW, int NST>
int launch_fold(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int nkb, int* err, const FoldEpi& fe,
                cudaStream_t stream) {
  constexpr int SMEM = fg_smem_bytes_st<BN, NST>();
  constexpr int CTAS_PER_SM = EPIW == FG_EPI_WARPS ? 1 : 2;
  static_assert(SMEM <= 227 * 1024, "folding GEMM shared memory");
  static_assert(CTAS_PER_SM * SMEM <= 228 * 1024, "folding GEMM shared memory per SM");
  static_assert(CTAS_PER_SM * 2 * (int)tmem_cols_for(BN) <= 512, "folding GEMM TMEM per SM");
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(fold_gemm_kernel<BN, EPIW, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    SMEM);
  });
  if (attr_err != cudaSuccess) return fail(CARC_CUDA_ERROR, "folding GEMM: %s", cudaGetErrorString(attr_err));
  int dev = 0, sms = 0;
  CARC_CHECK_CUDA(cudaGetDevice(&dev));
  CARC_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int n_tiles = N / BN;
  const int64_t tiles = (int64_t)(M / BM) * n_tiles;
  if (tiles >= (int64_t(1) << 31)) return fail(CARC_TOO_LARGE, "folding GEMM: %lld tiles", (long long)tiles);
  const int grid = (int)std::min<int64_t>(tiles, (int64_t)std::max(1, sms) * CTAS_PER_SM);
  fold_gemm_kernel<BN, EPIW, NST><<<grid, 32 * (2 + EPIW), SMEM, stream>>>(ma, mb, n_tiles, (int)tiles, nkb, err, fe);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace

int gemm_bf16_tn_fold(const void* A, int M, const void* B, int N, int K, const FoldEpi& fe, int* err,
                      cudaStream_t stream, int variant) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM != 0 || K % BK != 0 || N % 16 != 0)
    return fail(CARC_BAD_SHAPE, "tensor core GEMM: shape %d x %d x %d not tileable (M%%128, K%%64, N%%16)", M, N, K);
  if (fe.M * 4 > M || fe.N > N || (fe.col_off & 1) || fe.rows < fe.l0 * fe.l1 * fe.d * fe.nvec ||
      fe.rows * 32 >= (int64_t(1) << 31) || fe.col_off / 2 + 2 * fe.kc >= (int64_t(1) << 31))
    return fail(CARC_BAD_ARG, "tensor core GEMM: folding epilogue does not fit the tile grid");
  const int kb_total = K / BK;
  int bn = N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : N % 64 == 0 ? 64 : N % 32 == 0 ? 32 : 16;
  CUtensorMap ma, mb;
  CARC_RETURN_IF(make_map(&ma, A, (uint64_t)K, (uint64_t)M, BM));
  CARC_RETURN_IF(make_map(&mb, B, (uint64_t)K, (uint64_t)N, (uint32_t)bn));
  if (variant == 1 && N % 128 == 0) {
    // two CTAs per SM: 128-column tiles, 8 fold warps, 2 stages each
    CUtensorMap mb2;
    CARC_RETURN_IF(make_map(&mb2, B, (uint64_t)K, (uint64_t)N, 128u));
    return launch_fold<128, FG2_EPI_WARPS, FG2_STAGES>(ma, mb2, M, N, kb_total, err, fe, stream);
  }
  switch (bn) {
    case 256: return launch_fold<256, FG_EPI_WARPS, fg_stages<256>()>(ma, mb, M, N, kb_total, err, fe, stream);
    case 128: return launch_fold<128, FG_EPI_WARPS, fg_stages<128>()>(ma, mb, M, N, kb_total, err, fe, stream);
    case 64: return launch_fold<64, FG_EPI_WARPS, fg_stages<64>()>(ma, mb, M, N, kb_total, err, fe, stream);
    case 32: return launch_fold<32, FG_EPI_WARPS, fg_stages<32>()>(ma, mb, M, N, kb_total, err, fe, stream);
    default: return launch_fold<16, FG_EPI_WARPS, fg_stages<16>()>(ma, mb, M, N, kb_total, err, fe, stream);
  }
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
__device__ __forceinline__ void pack_a_body(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                                            const PackParams& p) {
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

__global__ void pack_a_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                              const __grid_constant__ PackParams p) {
  pack_a_body(X, out, p);
}

// B role: out row n, column (h, k, c'): part h of [b_r, b_i]
__device__ __forceinline__ void pack_b_body(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                                            const PackParams& p) {
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

__global__ void pack_b_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                              const __grid_constant__ PackParams p) {
  pack_b_body(X, out, p);
}

// Grouped packing: operand blockIdx.y of the table into block blockIdx.y of
// the stacked output (block_elems bf16 each).
struct PtrTable {
  const double2* p[CARC_MAX_SLOTS];
};

__global__ void pack_grouped_kernel(const __grid_constant__ PtrTable src, __nv_bfloat16* __restrict__ out,
                                    int64_t block_elems, int role, const __grid_constant__ PackParams p) {
  __nv_bfloat16* o = out + (int64_t)blockIdx.y * block_elems;
  if (role == 0)
    pack_a_body(src.p[blockIdx.y], o, p);
  else
    pack_b_body(src.p[blockIdx.y], o, p);
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
__device__ __forceinline__ void reduce_planes_body(const float* __restrict__ P, double2* __restrict__ C,
                                                   const ReduceParams& p, int ksplit) {
  __shared__ double2 part[RP_WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t m = blockIdx.y;
  const int64_t n = (int64_t)blockIdx.x * 32 + lane;
  Kahan re, im;
  if (n < p.Nc) {
    // four planes (16 loads) in flight per thread before they are summed (in plane order)
    const float* base = P + (4 * m) * p.ld + n;
    for (int z0 = w; z0 < ksplit; z0 += 4 * RP_WARPS) {
      float v[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int z = z0 + u * RP_WARPS;
        const float* b = base + z * p.split_stride;
#pragma unroll
        for (int q = 0; q < 4; ++q) v[u][q] = z < ksplit ? __ldcg(b + q * p.ld) : 0.f;
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

__global__ __launch_bounds__(32 * RP_WARPS) void reduce_planes_kernel(const float* __restrict__ P,
                                                                       double2* __restrict__ C,
                                                                       const __grid_constant__ ReduceParams p) {
  reduce_planes_body(P, C, p, p.ksplit);
}

// Grouped reduction: output blockIdx.z sums planes [first, first + count)
// (its entries' split planes, in entry order) into its own C.
struct GroupOut {
  int first[CARC_MAX_SLOTS], count[CARC_MAX_SLOTS];
  double2* dst[CARC_MAX_SLOTS];
};

__global__ __launch_bounds__(32 * RP_WARPS) void reduce_planes_grouped_kernel(const float* __restrict__ P,
                                                                               const __grid_constant__ ReduceParams p,
                                                                               const __grid_constant__ GroupOut go) {
  const int c = blockIdx.z;
  reduce_planes_body(P + (int64_t)go.first[c] * p.split_stride, go.dst[c], p, go.count[c]);
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

// ---------------------------------------------------------------------------
// C[c] = alpha sum over entries (i, j, c) of A[i] B[j]^T (+ C[c]), all entries
// of one shape in four launches: the distinct A and B operands packed once
// each into stacked buffers, one grouped GEMM over (entry, tile, split), one
// grouped reduction per referenced output (entries summed in table order).
// ---------------------------------------------------------------------------
namespace {

struct GroupedGeo {
  int64_t rows_a, rows_b, kp, ld;
  int bn, ks, mt, nt;
};

GroupedGeo grouped_geo(const ZView& a, const ZView& b, int n_out) {
  GroupedGeo g;
  const int64_t M = zview_rows(a), N = zview_rows(b), Kc = zview_k(a);
  g.rows_a = round_up(4 * M, BM);
  g.rows_b = round_up(N, 16);
  g.kp = round_up(4 * Kc, BK);
  g.ld = g.rows_b;
  g.bn = gemm_tile_n((int)g.rows_b);
  g.mt = (int)(g.rows_a / BM);
  g.nt = (int)(g.rows_b / g.bn);
  // K splits only when the outputs' tiles do not fill the 152 SMs
  const int64_t tiles = (int64_t)std::max(1, n_out) * g.mt * g.nt;
  const int want = tiles >= 152 ? 1 : (int)((152 + tiles - 1) / tiles);
  g.ks = gemm_effective_ksplit((int)g.kp, std::max(1, std::min(want, 65535 / std::max(1, n_out))));
  return g;
}

int64_t al256(int64_t x) { return (x + 255) / 256 * 256; }

int64_t grouped_plane_bytes(const GroupedGeo& g, int n_out) {
  return g.ks > 1 ? (int64_t)n_out * g.ks * g.rows_a * g.ld * 4 : 0;
}

}  // namespace

int64_t zgemm_tc_grouped_workspace(const ZView& a, const ZView& b, int n_a, int n_b, int n_e) {
  const GroupedGeo g = grouped_geo(a, b, 1);
  int64_t planes = 0;
  for (int n = 1; n <= std::min(n_e, CARC_MAX_SLOTS); ++n) planes = std::max(planes, grouped_plane_bytes(grouped_geo(a, b, n), n));
  return al256((int64_t)n_a * g.rows_a * g.kp * 2) + al256((int64_t)n_b * g.rows_b * g.kp * 2) + al256(planes) + 256;
}

int zgemm_tc_grouped(const ZView& a, const ZView& b, const ZOut& c, const void* const* a_ptrs, int n_a,
                     const void* const* b_ptrs, int n_b, void* const* c_ptrs, int n_c, const int32_t* entries,
                     int n_e, double2 alpha, int accumulate, void* ws, int64_t ws_bytes, int* err,
                     cudaStream_t stream) {
  const int64_t M = zview_rows(a), Kc = zview_k(a);
  if (zview_k(b) != Kc) return fail(CARC_BAD_SHAPE, "grouped tensor core GEMM: K mismatch");
  if (n_a < 1 || n_b < 1 || n_c < 1 || n_e < 1 || n_a > CARC_MAX_SLOTS || n_b > CARC_MAX_SLOTS ||
      n_c > CARC_MAX_SLOTS || n_e > CARC_MAX_ENTRIES)
    return fail(CARC_BAD_ARG, "grouped tensor core GEMM: %d A, %d B, %d C, %d entries (at most %d operands, %d entries)",
                n_a, n_b, n_c, n_e, CARC_MAX_SLOTS, CARC_MAX_ENTRIES);
  for (int e = 0; e < n_e; ++e) {
    const int i = entries[3 * e], j = entries[3 * e + 1], k = entries[3 * e + 2];
    if (i < 0 || i >= n_a || j < 0 || j >= n_b || k < 0 || k >= n_c || !a_ptrs[i] || !b_ptrs[j] || !c_ptrs[k])
      return fail(CARC_BAD_ARG, "grouped tensor core GEMM: entry %d (%d, %d, %d) out of range", e, i, j, k);
  }
  // entries ordered by output (stable: table order within an output)
  std::vector<int> order(n_e);
  for (int e = 0; e < n_e; ++e) order[e] = e;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return entries[3 * x + 2] < entries[3 * y + 2]; });
  GemmGroup grp;
  std::memset(&grp, 0, sizeof(grp));
  GroupEpi epi;
  std::memset(&epi, 0, sizeof(epi));
  int n_out = 0;
  for (int q = 0; q < n_e; ++q) {
    const int e = order[q], k = entries[3 * e + 2];
    grp.ij[q] = make_int2(entries[3 * e], entries[3 * e + 1]);
    if (q == 0 || entries[3 * order[q - 1] + 2] != k) {
      grp.e_first[n_out] = q;
      epi.dst[n_out] = static_cast<double2*>(c_ptrs[k]);
      ++n_out;
    }
  }
  grp.e_first[n_out] = n_e;
  const GroupedGeo g = grouped_geo(a, b, n_out);
  if ((int64_t)n_a * g.rows_a > (1ll << 30) || (int64_t)n_b * g.rows_b > (1ll << 30) || g.kp > (1ll << 30))
    return fail(CARC_TOO_LARGE, "grouped tensor core GEMM: too large");
  if (g.ks > 1 && M > 65535) return fail(CARC_TOO_LARGE, "grouped tensor core GEMM: %lld output rows", (long long)M);
  if (ws_bytes < zgemm_tc_grouped_workspace(a, b, n_a, n_b, n_e))
    return fail(CARC_BAD_ARG, "grouped tensor core GEMM: workspace too small");
  grp.n_out = n_out;
  grp.ks = g.ks;
  grp.a_rows_per = (int)g.rows_a;
  grp.b_rows_per = (int)g.rows_b;
  grp.kb_total = (int)(g.kp / BK);
  grp.kb_per = (grp.kb_total + g.ks - 1) / g.ks;
  epi.nm = c.nm;
  epi.nn = c.nn;
  epi.Mc = 1;
  epi.Nc = 1;
  for (int i = 0; i < c.nm; ++i) {
    epi.m_ext[i] = c.m_ext[i];
    epi.m_str[i] = c.m_str[i];
    epi.Mc *= c.m_ext[i];
  }
  for (int i = 0; i < c.nn; ++i) {
    epi.n_ext[i] = c.n_ext[i];
    epi.n_str[i] = c.n_str[i];
    epi.Nc *= c.n_ext[i];
  }
  epi.alpha = alpha;
  epi.alpha_one = alpha.x == 1.0 && alpha.y == 0.0;
  epi.accumulate = accumulate;
  char* p = static_cast<char*>(ws);
  auto* A_all = reinterpret_cast<__nv_bfloat16*>(p);
  auto* B_all = reinterpret_cast<__nv_bfloat16*>(p + al256((int64_t)n_a * g.rows_a * g.kp * 2));
  float* P = reinterpret_cast<float*>(p + al256((int64_t)n_a * g.rows_a * g.kp * 2) +
                                      al256((int64_t)n_b * g.rows_b * g.kp * 2));
  // pack every distinct operand once
  PtrTable ta, tb;
  std::memset(&ta, 0, sizeof(ta));
  std::memset(&tb, 0, sizeof(tb));
  for (int i = 0; i < n_a; ++i) ta.p[i] = static_cast<const double2*>(a_ptrs[i]);
  for (int j = 0; j < n_b; ++j) tb.p[j] = static_cast<const double2*>(b_ptrs[j]);
  const PackParams pa = pack_params(a, g.rows_a, g.kp, 0), pb = pack_params(b, g.rows_b, g.kp, 0);
  pack_grouped_kernel<<<dim3(grid_of(g.rows_a / 4 * Kc), n_a), 256, 0, stream>>>(ta, A_all, g.rows_a * g.kp, 0, pa);
  CARC_CHECK_LAUNCH();
  pack_grouped_kernel<<<dim3(grid_of(g.rows_b * Kc), n_b), 256, 0, stream>>>(tb, B_all, g.rows_b * g.kp, 1, pb);
  CARC_CHECK_LAUNCH();
  if (g.kp > 4 * Kc) {
    pack_pad_kernel<<<grid_of((int64_t)n_a * g.rows_a * (g.kp - 4 * Kc)), 256, 0, stream>>>(
        A_all, (int64_t)n_a * g.rows_a, 4 * Kc, g.kp, g.kp);
    CARC_CHECK_LAUNCH();
    pack_pad_kernel<<<grid_of((int64_t)n_b * g.rows_b * (g.kp - 4 * Kc)), 256, 0, stream>>>(
        B_all, (int64_t)n_b * g.rows_b, 4 * Kc, g.kp, g.kp);
    CARC_CHECK_LAUNCH();
  }
  // one grouped GEMM (its epilogue writes the outputs when there is one split)
  CUtensorMap ma, mb;
  CARC_RETURN_IF(make_map(&ma, A_all, (uint64_t)g.kp, (uint64_t)(n_a * g.rows_a), BM));
  CARC_RETURN_IF(make_map(&mb, B_all, (uint64_t)g.kp, (uint64_t)(n_b * g.rows_b), (uint32_t)g.bn));
  const int64_t plane_stride = g.rows_a * g.ld;
  int max_chain = 0;  // longest chain of K blocks of one output (entries x split K blocks)
  for (int q = 0; q < n_out; ++q) max_chain = std::max(max_chain, (grp.e_first[q + 1] - grp.e_first[q]) * grp.kb_per);
  CARC_RETURN_IF(launch_grouped(g.bn, max_chain <= 4, ma, mb, g.mt, g.nt, P, g.ld, plane_stride, err, grp, epi,
                                stream));
  if (g.ks == 1) return CARC_OK;
  // several splits: one grouped reduction of each output's planes
  ReduceParams rp;
  std::memset(&rp, 0, sizeof(rp));
  rp.nm = epi.nm;
  rp.nn = epi.nn;
  for (int i = 0; i < CARC_MAX_SUBDIMS; ++i) {
    rp.m_ext[i] = epi.m_ext[i];
    rp.m_str[i] = epi.m_str[i];
    rp.n_ext[i] = epi.n_ext[i];
    rp.n_str[i] = epi.n_str[i];
  }
  rp.Mc = epi.Mc;
  rp.Nc = epi.Nc;
  rp.ld = g.ld;
  rp.split_stride = plane_stride;
  rp.accumulate = accumulate;
  rp.alpha = alpha;
  GroupOut go;
  std::memset(&go, 0, sizeof(go));
  for (int q = 0; q < n_out; ++q) {
    go.first[q] = q * g.ks;
    go.count[q] = g.ks;
    go.dst[q] = epi.dst[q];
  }
  dim3 grid((unsigned)((rp.Nc + 31) / 32), (unsigned)rp.Mc, (unsigned)n_out);
  reduce_planes_grouped_kernel<<<grid, 32 * RP_WARPS, 0, stream>>>(P, rp, go);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
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
