// Host-side interface of the split-BF16 tensor-core complex GEMM (umma_gemm.cu).
#pragma once
#include "common.cuh"
#include <cuda.h>

namespace carc {

// Compensated FP32 accumulation (Knuth's TwoSum): s + c carries the running
// sum of FP32 terms with an error of order n u^2 sum |x| (u = 2^-24), as
// accurate as an FP64 sum of the same terms for n in the hundreds, without
// FP64 arithmetic in the loop (FP64 issue rate is low on this part).
// __fadd_rn keeps the compiler from reassociating or contracting the terms.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    s = t;
    c = __fadd_rn(c, err);
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// A complex128 operand seen as a (rows x k) matrix through strided index groups.
struct ZView {
  const void* base;
  int nr, nk;
  int64_t r_ext[CARC_MAX_SUBDIMS], r_str[CARC_MAX_SUBDIMS];
  int64_t k_ext[CARC_MAX_SUBDIMS], k_str[CARC_MAX_SUBDIMS];
  int conj;
};

// A complex128 output seen as (m x n) through strided index groups.
struct ZOut {
  void* base;
  int nm, nn;
  int64_t m_ext[CARC_MAX_SUBDIMS], m_str[CARC_MAX_SUBDIMS];
  int64_t n_ext[CARC_MAX_SUBDIMS], n_str[CARC_MAX_SUBDIMS];
};

// Epilogue that folds the GEMM rows (4m + 2c + s) into complex W[m, n] and
// writes it split (hi | lo) into a region of a packed operand:
//   m -> (x0,x1,l0,l1), n -> (vec,k2,k3,p);  row (vec,l0,l1,p), k (x0,x1,k2,k3).
// The operand is K-block-major: element (row, column c) of a `rows`-row
// operand sits at (c / 64) rows 64 + row 64 + c % 64, so that one 64-column K
// block of all its rows is one contiguous run (one TMA box of the step-B GEMM
// reads whole DRAM pages, not 128 bytes from each of its rows).
struct FoldEpi {
  int64_t x0, x1, l0, l1;
  int64_t nvec, k2, k3, d;
  int64_t M, N;      // valid complex rows / columns
  int64_t kc;        // complex K of the destination region
  int64_t col_off;   // first bf16 column of the region (even)
  int64_t rows;      // rows of the destination operand
  void* dst;
};

int64_t zview_rows(const ZView& v);
int64_t zview_k(const ZView& v);
int64_t round_up(int64_t a, int64_t b);

// Raw GEMM: out[z][m][n] (fp32, ld_out) = sum over split z's K range of A[m,:] . B[n,:]
// (A: M x K, B: N x K, BF16 K-major; M % 128 == 0, K % 64 == 0, N % 16 == 0).
// m_live (optional): when M == 128 and only rows [0, m_live <= 64) of A can be
// nonzero, the zero rows are not read from memory.
// b_blocked: B is K-block-major ([K / 64][N][64], as the folding epilogue
// writes W) instead of row-major N x K.
int gemm_bf16_tn(const void* A, int M, const void* B, int N, int K, float* out, int64_t ld_out, int ksplit, int* err,
                 cudaStream_t stream, int m_live = 0, int b_blocked = 0);
int gemm_effective_ksplit(int K, int ksplit);
// C[c] (+)= alpha sum over entries (i, j, c) of A[i] B[j]^T for operands of one
// shape (a, b, c give the geometry; their bases are ignored): the distinct
// operands packed once each, one grouped GEMM launch over (entry, tile,
// split), one grouped reduction; entries (HOST int32 [n_e][3]).
int64_t zgemm_tc_grouped_workspace(const ZView& a, const ZView& b, int n_a, int n_b, int n_e);
int zgemm_tc_grouped(const ZView& a, const ZView& b, const ZOut& c, const void* const* a_ptrs, int n_a,
                     const void* const* b_ptrs, int n_b, void* const* c_ptrs, int n_c, const int32_t* entries,
                     int n_e, double2 alpha, int accumulate, void* ws, int64_t ws_bytes, int* err,
                     cudaStream_t stream);
// N tile of gemm_bf16_tn: N in ceil(N / 256) equal tiles when those are
// multiples of 16 (each N tile streams the whole A operand once), else the
// largest of 256/128/64/32/16 dividing N.
int gemm_tile_n(int N);
// Rows to pad a B operand of n rows to so that gemm_bf16_tn tiles it in
// ceil(n / 256) equal tiles of a multiple of 16 (the least padding).
int64_t gemm_pad_n(int64_t n);
// 2D tensor map of a BF16 K-major matrix (inner = K columns, rows), box of
// 64 columns x box_rows rows, 128-byte swizzle (the GEMM operand layout).
int tma_map_bf16(CUtensorMap* map, const void* base, uint64_t inner, uint64_t rows, uint32_t box_rows);
// The same GEMM (no K split) with the folding epilogue instead of FP32 planes:
// a persistent warp-specialised kernel (one CTA per SM, two TMEM accumulators)
// writing W K-block-major (FoldEpi).
int gemm_bf16_tn_fold(const void* A, int M, const void* B, int N, int K, const FoldEpi& fe, int* err,
                      cudaStream_t stream, int variant = 0);
// Deterministic FP64 reduction of split-K planes into a complex output in one
// launch (coalesced over columns, planes spread over 8 warps per block); the
// workspace arguments are kept for the callers' layouts and need 256 bytes.
int64_t reduce_partials2_workspace(int64_t Mc, int64_t Nc, int ksplit);
// The same for column-major planes P[z][n][r] with `rows` rows (a multiple of 32).
int reduce_planes_colmajor(const float* P, int64_t rows, int64_t split_stride, int ksplit, const ZOut& o,
                           double2 alpha, int accumulate, cudaStream_t stream);
int reduce_partials2(const float* P, int64_t ld, int64_t split_stride, int ksplit, const ZOut& o, double2 alpha,
                     int accumulate, void* ws, int64_t ws_bytes, cudaStream_t stream);
// role 0: A operand (rows (m, re/im, hi/lo)); role 1: B operand (row n, K = [hi | lo]).
int pack_operand(const ZView& v, int role, void* out, int64_t rows_out, int64_t kp_out, cudaStream_t stream);
// Pack into the K-column region [col_off, col_off + region) of rows of pitch kp_out (region >= 4K, rest zeroed).
int pack_operand_region(const ZView& v, int role, void* out, int64_t rows_out, int64_t kp_out, int64_t col_off,
                        int64_t region, cudaStream_t stream);
int reduce_partials(const float* P, int64_t ld, int64_t split_stride, int ksplit, const ZOut& o, double2 alpha,
                    int accumulate, cudaStream_t stream);

ZView zview_a(const carc_contract_desc& d, const void* base);
ZView zview_b(const carc_contract_desc& d, const void* base);
ZOut zout_c(const carc_contract_desc& d, void* base);

// C (+)= alpha A B^T, complex, on the tensor cores with split-BF16 operands.
int64_t zgemm_tc_workspace(const ZView& a, const ZView& b, int ksplit);
int zgemm_tc(const ZView& a, const ZView& b, const ZOut& c, double2 alpha, int accumulate, int ksplit, void* ws,
             int64_t ws_bytes, int* err, cudaStream_t stream);

}  // namespace carc
