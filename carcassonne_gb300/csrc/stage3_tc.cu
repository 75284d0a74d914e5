// The stage-3 operator on the tensor cores (split-BF16 operands, FP32
// accumulation in TMEM, FP64 reductions):
//
//  matvec  y[v] = sum_t S2_0[i0_t] (x) S2_1[i1_t] (x) O[io_t] . x[v]
//    terms are grouped by their S2_1 tag g;
//    step A (one persistent tcgen05 folding GEMM per group, terms
//    concatenated along K):
//      W_g[(x0,x1,l0,l1),(v,k2,k3,p)] = sum_{t in g} sum_{k0,k1} S2_0[i0_t] . Vin_t
//      whose epilogue folds the (hi,lo) and (re,im) rows and writes W_g split
//      straight into region g of step B's packed, K-block-major operand;
//    step B (one split-K tcgen05 GEMM over all groups, concatenated along K):
//      y^T[(l2,l3),(v,l0,l1,p)] = sum_g sum_{x0,x1,k2,k3} S2_1[g] . W_g,
//      split planes summed by a coalesced reduction (compensated FP32 per
//      plane sequence, FP64 combination);
//    or, for eligible shapes, both steps in one fused kernel with W on chip
//    (below).
//  matrix  H = sum_o G_o (x) O_o,  G_o = sum_{t in o} S2_0[i0_t] . S2_1[i1_t] over x,
//          terms of one operator group concatenated along K in one GEMM.
//
// The S2 tensors are packed once per operator ("plan", in term-group order):
// the many matvecs of a solve reuse them.  Index convention as in stage3.cu
// (tensors/_2d/dense.py:114-195).
#include "common.cuh"
#include "contract.cuh"
#include "stage3.cuh"
#include "stage3_tc.cuh"
#include "umma.cuh"
#include "umma_gemm.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace carc {

namespace {

inline int64_t a256(int64_t b) { return (b + 255) / 256 * 256; }

struct S3 {
  int64_t x0, x1, k0, k1, l0, l1, k2, k3, l2, l3, d;
  int64_t s0[6], s1[6];
};

int s3_shapes(const int64_t* a, const int64_t* b, int64_t d, S3* s) {
  for (int i = 0; i < 6; ++i)
    if (a[i] < 1 || b[i] < 1) return fail(CARC_BAD_SHAPE, "stage3 tc: non-positive extent");
  if (a[0] != b[1] || a[1] != b[0]) return fail(CARC_BAD_SHAPE, "stage3 tc: S2 halves do not glue");
  s->x0 = a[0];
  s->x1 = a[1];
  s->k0 = a[2];
  s->k1 = a[3];
  s->l0 = a[4];
  s->l1 = a[5];
  s->k2 = b[2];
  s->k3 = b[3];
  s->l2 = b[4];
  s->l3 = b[5];
  s->d = d;
  int64_t st = 1;
  for (int i = 5; i >= 0; --i) {
    s->s0[i] = st;
    st *= a[i];
  }
  st = 1;
  for (int i = 5; i >= 0; --i) {
    s->s1[i] = st;
    st *= b[i];
  }
  return CARC_OK;
}

// The matvec's term structure: terms sharing their S2_1 tag (i1) form one
// group; a group's step-A GEMM concatenates its terms along K, so it yields
// sum_t S2_0[i0_t] . Vin_t directly, and the single step-B GEMM concatenates
// the groups along K.
struct TermGroups {
  std::vector<int> i1;                  // S2_1 tag of each group
  std::vector<std::vector<int>> terms;  // term indices of each group
  int max_terms = 0;
};

TermGroups group_terms(const int32_t* terms, int n_terms) {
  TermGroups g;
  for (int t = 0; t < n_terms; ++t) {
    const int i1 = terms[3 * t + 1];
    int k = -1;
    for (size_t q = 0; q < g.i1.size(); ++q)
      if (g.i1[q] == i1) k = (int)q;
    if (k < 0) {
      k = (int)g.i1.size();
      g.i1.push_back(i1);
      g.terms.emplace_back();
    }
    g.terms[k].push_back(t);
  }
  for (auto& v : g.terms) g.max_terms = std::max(g.max_terms, (int)v.size());
  return g;
}

struct Geo {
  int64_t MA, NA;         // step A: complex rows (x0 x1 l0 l1) / columns (nvec k2 k3 d)
  int64_t rowsA_a, regA;  // packed rows of S2_0 (4 MA), K region per term (4 k0 k1)
  int64_t rowsA_b;        // packed rows of Vin
  int64_t rowsB_a, regB;  // step B: packed rows of S2_1 (4 l2 l3), K region per group (4 x0 x1 k2 k3)
  int64_t rowsB_b;        // packed rows of W (nvec l0 l1 d)
  int64_t kcB;
};

// Padded row count of step A's B operand (Vin): the folding GEMM tiles N by
// the largest of 256/128/64/32/16 dividing it, and every N tile streams the
// whole A operand again, so pad to one power-of-two tile up to 256 and to
// whole 256-row tiles above (NA = 400 at D = 5 would otherwise run 25 tiles
// of 16).  W, step B's B operand, is padded by gemm_pad_n instead: the plain
// GEMM takes any tile width that is a multiple of 16, so 400 rows become two
// tiles of 208 (not 512 rows) and 576 three of 192 (not 768), and step B,
// which streams W from HBM, reads that much less.
int64_t pad_b_rows(int64_t n) {
  if (n > 256) return round_up(n, 256);
  int64_t t = 16;
  while (t < n) t *= 2;
  return t;
}

Geo geometry(const S3& s, int nvec) {
  Geo g;
  g.MA = s.x0 * s.x1 * s.l0 * s.l1;
  g.NA = (int64_t)nvec * s.k2 * s.k3 * s.d;
  g.rowsA_a = round_up(4 * g.MA, 128);
  g.regA = round_up(4 * s.k0 * s.k1, 64);
  g.rowsA_b = pad_b_rows(g.NA);
  g.kcB = s.x0 * s.x1 * s.k2 * s.k3;
  g.rowsB_a = round_up(4 * s.l2 * s.l3, 128);
  g.regB = round_up(4 * g.kcB, 64);
  g.rowsB_b = gemm_pad_n((int64_t)nvec * s.l0 * s.l1 * s.d);
  return g;
}

ZView view_s2_0_stepA(const S3& s, const void* base) {
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = 4;
  v.r_ext[0] = s.x0; v.r_str[0] = s.s0[0];
  v.r_ext[1] = s.x1; v.r_str[1] = s.s0[1];
  v.r_ext[2] = s.l0; v.r_str[2] = s.s0[4];
  v.r_ext[3] = s.l1; v.r_str[3] = s.s0[5];
  v.nk = 2;
  v.k_ext[0] = s.k0; v.k_str[0] = s.s0[2];
  v.k_ext[1] = s.k1; v.k_str[1] = s.s0[3];
  return v;
}

ZView view_s2_1_stepB(const S3& s, const void* base) {
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = 2;
  v.r_ext[0] = s.l2; v.r_str[0] = s.s1[4];
  v.r_ext[1] = s.l3; v.r_str[1] = s.s1[5];
  v.nk = 4;  // (x0, x1, k2, k3): x0 is S2_1's axis 1, x1 its axis 0
  v.k_ext[0] = s.x0; v.k_str[0] = s.s1[1];
  v.k_ext[1] = s.x1; v.k_str[1] = s.s1[0];
  v.k_ext[2] = s.k2; v.k_str[2] = s.s1[2];
  v.k_ext[3] = s.k3; v.k_str[3] = s.s1[3];
  return v;
}

// zero the K padding of the valid rows of the packed W, per region the
// columns [4 kc, reg) (the folding epilogue writes only the valid entries);
// W is K-block-major with `rows` rows: column c of row r at
// (c / 64) rows 64 + r 64 + c % 64
__global__ void clear_w_padding_kernel(__nv_bfloat16* __restrict__ W, int64_t rows_valid, int64_t rows, int64_t kc4,
                                       int64_t reg, int64_t n_reg) {
  const int64_t pad = reg - kc4;
  const int64_t t1 = rows_valid * n_reg * pad;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < t1; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / (n_reg * pad), rem = t % (n_reg * pad);
    const int64_t c = (rem / pad) * reg + kc4 + rem % pad;
    W[(c >> 6) * rows * 64 + row * 64 + (c & 63)] = __float2bfloat16_rn(0.f);
  }
}

inline int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * 152)); }

// Autotune cache: the step-B split-K count per problem shape, written by the
// host-side autotuner (carc_tc_autotune_set) after timing candidates; shapes
// without an entry use the one-wave heuristic below.  The only mutable global
// of the library, guarded by a mutex.
struct TuneKey {
  int64_t v[15];
  bool operator<(const TuneKey& o) const { return std::lexicographical_compare(v, v + 15, o.v, o.v + 15); }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
std::map<TuneKey, int> g_tune_fold;  // step A's folding-GEMM configuration (0 or 1)

TuneKey tune_key(const int64_t* s0, const int64_t* s1, int64_t d, int nvec, int groups) {
  TuneKey k;
  for (int i = 0; i < 6; ++i) {
    k.v[i] = s0[i];
    k.v[6 + i] = s1[i];
  }
  k.v[12] = d;
  k.v[13] = nvec;
  k.v[14] = groups;
  return k;
}

int tuned_ksplit(const int64_t* s0, const int64_t* s1, int64_t d, int nvec, int groups) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(s0, s1, d, nvec, groups));
  return it == g_tune.end() ? 0 : it->second;
}

int tuned_fold(const int64_t* s0, const int64_t* s1, int64_t d, int nvec, int groups) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune_fold.find(tune_key(s0, s1, d, nvec, groups));
  return it == g_tune_fold.end() ? 0 : it->second;
}

// split-K count that fills the 152 SMs (one CTA each) in a single wave
int choose_ksplit(int64_t tiles, int64_t kp) {
  const int64_t kb = kp / 64;
  int64_t ks = tiles >= 152 ? 1 : 152 / tiles;
  ks = std::max<int64_t>(1, std::min<int64_t>(ks, kb));
  return (int)ks;
}

// N tile the plain GEMM uses for a B operand of n rows
int bn_for(int64_t n) { return gemm_tile_n((int)n); }

// ---- compact operands of the fused matvec (F2 kernel, below) -----------------
// S2_0, step A's A operand: rows (m, c) for the MA complex rows m = (x0,x1,l0,l1)
// and c = re / im output row of the real embedding [[a_r, -a_i], [a_i, a_r]];
// per term a 64-column region [hi plane | lo plane] of the row's (k0 k1, c')
// entries, the lo plane starting at column Wp = round_up(2 k0 k1, 16).
// S2_1, step B's B operand: rows (j, c) for j = (l2,l3) (padded to NBB, a
// multiple of 16) and c = re / im of the output, row (j,0) = [s_r, -s_i] and
// row (j,1) = [s_i, s_r] over the complex K index kB = (x0,x1,k2,k3); per
// group a region of 4 KcB columns [hi plane (2 KcB) | lo plane (2 KcB)].
// 8 bytes per complex entry and plane pair in both, against 32 (S2_0) in the
// first layout.
constexpr int F2_XT = 64;    // complex step-A rows per x-tile
constexpr int F2_MAXG = 8;   // S2_1 tags with terms

struct Geo2 {
  bool ok;
  int64_t MA, kc, Wp, KcB, NBB, rowsA;
};

Geo2 geometry2(const S3& s, const TermGroups& tg) {
  Geo2 g;
  memset(&g, 0, sizeof(g));
  const int64_t L = s.l0 * s.l1, K23 = s.k2 * s.k3;
  g.MA = s.x0 * s.x1 * L;
  g.kc = s.k0 * s.k1;
  g.Wp = round_up(2 * g.kc, 16);
  g.KcB = s.x0 * s.x1 * K23;
  g.NBB = round_up(2 * s.l2 * s.l3, 16);
  g.rowsA = 2 * g.MA;
  g.ok = K23 == L && L % 4 == 0 && F2_XT % L == 0 && g.MA % F2_XT == 0 && 2 * g.Wp <= 64 && g.NBB <= 128 &&
         !tg.i1.empty() && (int)tg.i1.size() <= F2_MAXG && (s.d == 1 || s.d == 2 || s.d == 4 || s.d == 8);
  return g;
}

int64_t plan2_bytes(const Geo2& g, const TermGroups& tg) {
  if (!g.ok) return 0;
  int64_t b = 0;
  for (auto& v : tg.terms) b += a256(g.rowsA * 64 * (int64_t)v.size() * 2);
  b += a256(g.NBB * 4 * g.KcB * (int64_t)tg.i1.size() * 2);
  return b;
}

__device__ __forceinline__ void split_d(double v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __double2bfloat16(v);
  lo = __double2bfloat16(v - (double)__bfloat162float(hi));
}

struct Pack2 {
  int64_t e[6], st[6];  // the S2 tensor's extents and strides in its own axis order
  int64_t pitch;        // bf16 per packed row
  int64_t col0;         // first column of the region
  int64_t lo_off;       // column offset of the lo plane inside the region
  int64_t n;            // complex rows (S2_0) / K entries (S2_1)
  int64_t kc;           // complex K entries per row (S2_0) / rows j (S2_1)
};

// S2_0 (x0,x1,k0,k1,l0,l1): one thread per (m, k), m = (x0,x1,l0,l1), k = (k0,k1)
__global__ void pack2_s2_0_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                                  const __grid_constant__ Pack2 p) {
  const int64_t total = p.n * p.kc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / p.kc, k = t % p.kc;
    int64_t r = m;
    const int64_t l1 = r % p.e[5]; r /= p.e[5];
    const int64_t l0 = r % p.e[4]; r /= p.e[4];
    const int64_t x1 = r % p.e[1], x0 = r / p.e[1];
    const int64_t k1 = k % p.e[3], k0 = k / p.e[3];
    const double2 a = X[x0 * p.st[0] + x1 * p.st[1] + k0 * p.st[2] + k1 * p.st[3] + l0 * p.st[4] + l1 * p.st[5]];
    const double e[2][2] = {{a.x, -a.y}, {a.y, a.x}};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      __nv_bfloat16* row = out + (2 * m + c) * p.pitch + p.col0;
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) {
        __nv_bfloat16 hi, lo;
        split_d(e[c][cp], hi, lo);
        row[2 * k + cp] = hi;
        row[p.lo_off + 2 * k + cp] = lo;
      }
    }
  }
}

// S2_1 (x1,x0,k2,k3,l2,l3): one thread per (j, kB), j = (l2,l3), kB = (x0,x1,k2,k3)
__global__ void pack2_s2_1_kernel(const double2* __restrict__ X, __nv_bfloat16* __restrict__ out,
                                  const __grid_constant__ Pack2 p) {
  const int64_t total = p.n * p.kc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / p.n, kb = t % p.n;
    int64_t r = kb;
    const int64_t k3 = r % p.e[3]; r /= p.e[3];
    const int64_t k2 = r % p.e[2]; r /= p.e[2];
    const int64_t x1 = r % p.e[0], x0 = r / p.e[0];
    const int64_t l3 = j % p.e[5], l2 = j / p.e[5];
    const double2 a = X[x1 * p.st[0] + x0 * p.st[1] + k2 * p.st[2] + k3 * p.st[3] + l2 * p.st[4] + l3 * p.st[5]];
    const double e[2][2] = {{a.x, -a.y}, {a.y, a.x}};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      __nv_bfloat16* row = out + (2 * j + c) * p.pitch + p.col0;
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) {
        __nv_bfloat16 hi, lo;
        split_d(e[c][cp], hi, lo);
        row[2 * kb + cp] = hi;
        row[p.lo_off + 2 * kb + cp] = lo;
      }
    }
  }
}

Pack2 pack2_params(const S3& s, const int64_t* ext, const int64_t* st, int64_t pitch, int64_t col0, int64_t lo_off,
                   int64_t n, int64_t kc) {
  Pack2 p;
  memset(&p, 0, sizeof(p));
  for (int i = 0; i < 6; ++i) {
    p.e[i] = ext[i];
    p.st[i] = st[i];
  }
  p.pitch = pitch;
  p.col0 = col0;
  p.lo_off = lo_off;
  p.n = n;
  p.kc = kc;
  return p;
}

// plan layout: [per group g: S2_0 step-A operand, rowsA_a x (regA * |T_g|)] [S2_1 step-B operand, rowsB_a x (regB * G)]
// then, for shapes the F2 kernel takes, [per group g: compact S2_0, rowsA x 64 |T_g|] [compact S2_1, NBB x 4 KcB G]
int64_t plan_bytes_for(const Geo& g1, const TermGroups& tg) {
  int64_t b = 0;
  for (auto& v : tg.terms) b += a256(g1.rowsA_a * g1.regA * (int64_t)v.size() * 2);
  b += a256(g1.rowsB_a * g1.regB * (int64_t)tg.i1.size() * 2);
  return b;
}

}  // namespace

int tc_autotune_set(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int nvec, int groups, int ksplit) {
  if (ksplit < -2 || nvec < 1 || groups < 1) return fail(CARC_BAD_ARG, "tc autotune: bad entry");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const TuneKey k = tune_key(s0_shape, s1_shape, d, nvec, groups);
  if (ksplit == 0)
    g_tune.erase(k);
  else
    g_tune[k] = ksplit;
  return CARC_OK;
}

int tc_autotune_set_fold(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int nvec, int groups,
                         int variant) {
  if (variant < 0 || variant > 1 || nvec < 1 || groups < 1) return fail(CARC_BAD_ARG, "tc autotune: bad fold entry");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const TuneKey k = tune_key(s0_shape, s1_shape, d, nvec, groups);
  if (variant == 0)
    g_tune_fold.erase(k);
  else
    g_tune_fold[k] = variant;
  return CARC_OK;
}

int tc_autotune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  g_tune_fold.clear();
  return CARC_OK;
}

int64_t stage3_tc_plan_size(const int64_t* s0_shape, const int64_t* s1_shape, const int32_t* terms, int n_terms) {
  S3 s;
  if (s3_shapes(s0_shape, s1_shape, 1, &s) != CARC_OK) return -1;
  if (n_terms < 1) return 256;
  const TermGroups tg = group_terms(terms, n_terms);
  return plan_bytes_for(geometry(s, 1), tg) + plan2_bytes(geometry2(s, tg), tg);
}

int stage3_tc_prepare(const int64_t* s0_shape, const int64_t* s1_shape, const void* const* s0_ptrs, int n0,
                      const void* const* s1_ptrs, int n1, const int32_t* terms, int n_terms, void* plan,
                      int64_t plan_bytes, cudaStream_t stream) {
  S3 s;
  CARC_RETURN_IF(s3_shapes(s0_shape, s1_shape, 1, &s));
  if (n_terms < 1) return CARC_OK;
  for (int t = 0; t < n_terms; ++t)
    if (terms[3 * t] < 0 || terms[3 * t] >= n0 || terms[3 * t + 1] < 0 || terms[3 * t + 1] >= n1)
      return fail(CARC_BAD_ARG, "stage3 tc: term %d out of range", t);
  const TermGroups tg = group_terms(terms, n_terms);
  const Geo g = geometry(s, 1);
  if (plan_bytes < plan_bytes_for(g, tg) + plan2_bytes(geometry2(s, tg), tg))
    return fail(CARC_BAD_ARG, "stage3 tc: plan too small");
  char* p = static_cast<char*>(plan);
  for (size_t q = 0; q < tg.terms.size(); ++q) {
    const int64_t kp = g.regA * (int64_t)tg.terms[q].size();
    for (size_t j = 0; j < tg.terms[q].size(); ++j)
      CARC_RETURN_IF(pack_operand_region(view_s2_0_stepA(s, s0_ptrs[terms[3 * tg.terms[q][j]]]), 0, p, g.rowsA_a, kp,
                                         (int64_t)j * g.regA, g.regA, stream));
    p += a256(g.rowsA_a * kp * 2);
  }
  const int64_t kpB = g.regB * (int64_t)tg.i1.size();
  for (size_t q = 0; q < tg.i1.size(); ++q)
    CARC_RETURN_IF(pack_operand_region(view_s2_1_stepB(s, s1_ptrs[tg.i1[q]]), 0, p, g.rowsB_a, kpB,
                                       (int64_t)q * g.regB, g.regB, stream));
  p += a256(g.rowsB_a * kpB * 2);
  // the compact operands of the F2 kernel
  const Geo2 g2 = geometry2(s, tg);
  if (!g2.ok) return CARC_OK;
  const int64_t ext0[6] = {s.x0, s.x1, s.k0, s.k1, s.l0, s.l1};
  const int64_t ext1[6] = {s.x1, s.x0, s.k2, s.k3, s.l2, s.l3};
  for (size_t q = 0; q < tg.terms.size(); ++q) {
    const int64_t pitch = 64 * (int64_t)tg.terms[q].size();
    CARC_CHECK_CUDA(cudaMemsetAsync(p, 0, g2.rowsA * pitch * 2, stream));
    for (size_t j = 0; j < tg.terms[q].size(); ++j) {
      const Pack2 pk = pack2_params(s, ext0, s.s0, pitch, 64 * (int64_t)j, g2.Wp, g2.MA, g2.kc);
      pack2_s2_0_kernel<<<grid_of(g2.MA * g2.kc), 256, 0, stream>>>(
          static_cast<const double2*>(s0_ptrs[terms[3 * tg.terms[q][j]]]), reinterpret_cast<__nv_bfloat16*>(p), pk);
      CARC_CHECK_LAUNCH();
    }
    p += a256(g2.rowsA * pitch * 2);
  }
  const int64_t pitchB = 4 * g2.KcB * (int64_t)tg.i1.size();
  CARC_CHECK_CUDA(cudaMemsetAsync(p, 0, g2.NBB * pitchB * 2, stream));
  for (size_t q = 0; q < tg.i1.size(); ++q) {
    const Pack2 pk = pack2_params(s, ext1, s.s1, pitchB, 4 * g2.KcB * (int64_t)q, 2 * g2.KcB, g2.KcB, s.l2 * s.l3);
    pack2_s2_1_kernel<<<grid_of(g2.KcB * s.l2 * s.l3), 256, 0, stream>>>(
        static_cast<const double2*>(s1_ptrs[tg.i1[q]]), reinterpret_cast<__nv_bfloat16*>(p), pk);
    CARC_CHECK_LAUNCH();
  }
  return CARC_OK;
}

namespace {

struct MvWs {
  char* vin;     // packed Vin operands of all groups (step-A B operands)
  char* w_pk;    // packed W of all groups (step-B operand); unused when fused
  float* pB;     // step-B split planes
  char* red;     // reduction partial sums
  int ksB;
  bool fused;    // step A and step B in one kernel, W on chip
  std::vector<int64_t> vin_off;  // byte offset of each group's Vin operand
};

bool fused_eligible(const S3& s, int nvec, const TermGroups& tg);
int fused_grid(const S3& s, const TermGroups& tg);

int64_t mv_layout(const S3& s, const int64_t* s0_shape, const int64_t* s1_shape, int nvec, const TermGroups& tg,
                  MvWs* w, void* base) {
  const Geo g = geometry(s, nvec);
  const int64_t kpB = g.regB * (int64_t)tg.i1.size();
  const int64_t tilesB = (g.rowsB_a / 128) * (g.rowsB_b / bn_for(g.rowsB_b));
  // autotune entry: > 0 the unfused path with that step-B split, -1 (or none) the fused kernel where eligible
  const int tuned = tuned_ksplit(s0_shape, s1_shape, s.d, nvec, (int)tg.i1.size());
  const bool fused = tuned <= 0 && fused_eligible(s, nvec, tg);
  const int ksB = fused ? fused_grid(s, tg)
                        : gemm_effective_ksplit((int)kpB, tuned > 0 ? tuned : choose_ksplit(tilesB, kpB));
  std::vector<int64_t> vin_off;
  int64_t vin_bytes = 0;
  for (auto& v : tg.terms) {
    vin_off.push_back(vin_bytes);
    vin_bytes += a256(g.rowsA_b * g.regA * (int64_t)v.size() * 2);
  }
  const int64_t nb = (int64_t)nvec * s.l0 * s.l1 * s.d;
  const int64_t sizes[4] = {vin_bytes, fused ? 0 : g.rowsB_b * kpB * 2,
                            fused ? (int64_t)ksB * round_up(4 * s.l2 * s.l3, 32) * nb * 4
                                  : (int64_t)ksB * g.rowsB_a * g.rowsB_b * 4,
                            reduce_partials2_workspace(s.l2 * s.l3, nb, ksB)};
  char* p = static_cast<char*>(base);
  int64_t off = 0;
  char* ptrs[4];
  for (int i = 0; i < 4; ++i) {
    ptrs[i] = p ? p + off : nullptr;
    off += a256(sizes[i]);
  }
  if (w) {
    w->vin = ptrs[0];
    w->w_pk = ptrs[1];
    w->pB = reinterpret_cast<float*>(ptrs[2]);
    w->red = ptrs[3];
    w->ksB = ksB;
    w->fused = fused;
    w->vin_off = vin_off;
  }
  return off;
}

// Step A's B operands for every term in one launch: Vin_t = O[io_t] applied
// to the physical index of x (x itself for identity terms), split into BF16
// hi/lo and packed K-major as rows (vec,k2,k3,p) x [hi | lo] of (k0,k1, re/im)
// into the term's K region of its group's operand; padding rows and columns
// are written as zeros.
constexpr int kVinTermsPerLaunch = 64;

struct VinTerms {
  int n;
  int64_t rows_out, rows_valid, kc, reg4, k23, d;
  const double2* op[kVinTermsPerLaunch];
  int64_t dst[kVinTermsPerLaunch];    // uint32 (bf16 pair) offset of the term's region in row 0
  int64_t pitch[kVinTermsPerLaunch];  // row pitch in bf16 pairs
};

// One packed Vin slot: slot `t` of term `term` (row n = t / reg4, column
// slot = t % reg4), the site operator applied to x and the result split into
// (hi | lo) bf16 pairs.  32-bit index arithmetic (the host checks that a
// term's slot count fits).
__device__ __forceinline__ void pack_vin_slot(const double2* __restrict__ x, uint32_t* __restrict__ out,
                                              const VinTerms& p, int term, int t) {
  const int reg4 = (int)p.reg4, kc = (int)p.kc, k23 = (int)p.k23, d = (int)p.d;
  const double2* O = p.op[term];
  const int n = t / reg4, slot = t - n * reg4;
  uint32_t* row = out + p.dst[term] + (int64_t)n * p.pitch[term];
  if (slot >= kc) {  // padding columns [4 kc, reg)
    row[2 * slot] = 0u;
    row[2 * slot + 1] = 0u;
    return;
  }
  uint32_t hi = 0u, lo = 0u;
  if (n < p.rows_valid) {
    const int q = n / d, pp = n - q * d;
    const int vec = q / k23, kk = q - vec * k23;
    const double2* xv = x + (((int64_t)vec * kc + slot) * k23 + kk) * d;
    // the operator application in FP32: its rounding (2^-24) is far below
    // the hi + lo split that follows (2^-17)
    float fr, fi;
    if (O == nullptr) {
      const double2 v = xv[pp];
      fr = (float)v.x;
      fi = (float)v.y;
    } else {
      fr = 0.f;
      fi = 0.f;
      for (int qq = 0; qq < d; ++qq) {
        const double2 o = O[pp * d + qq], v = xv[qq];
        const float orr = (float)o.x, oi = (float)o.y, vr = (float)v.x, vi = (float)v.y;
        fr = fmaf(orr, vr, fmaf(-oi, vi, fr));
        fi = fmaf(orr, vi, fmaf(oi, vr, fi));
      }
    }
    const __nv_bfloat16 hr = __float2bfloat16_rn(fr), hm = __float2bfloat16_rn(fi);
    const __nv_bfloat16 lr = __float2bfloat16_rn(fr - __bfloat162float(hr));
    const __nv_bfloat16 lm = __float2bfloat16_rn(fi - __bfloat162float(hm));
    const __nv_bfloat162 h2 = __halves2bfloat162(hr, hm), l2 = __halves2bfloat162(lr, lm);
    hi = *reinterpret_cast<const uint32_t*>(&h2);
    lo = *reinterpret_cast<const uint32_t*>(&l2);
  }
  row[slot] = hi;
  row[kc + slot] = lo;
}

// grid (blocks over one term's rows_out x reg4 slots, terms)
__global__ void pack_vin_kernel(const double2* __restrict__ x, uint32_t* __restrict__ out,
                                const __grid_constant__ VinTerms p) {
  const int per_term = (int)(p.rows_out * p.reg4);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < per_term; t += gridDim.x * blockDim.x)
    pack_vin_slot(x, out, p, (int)blockIdx.y, t);
}

}  // namespace

// ---------------------------------------------------------------------------
// Fused matvec: step A and step B in one persistent kernel, W kept on chip.
//
// A pair is (x-tile t, S2_1 tag g): 32 complex rows of step A (XP x values x
// all L = l0 l1 rows) against the tag's Vin; a unit is one vector part of a
// pair (VH = 2 parts when the halves stay MMA-shaped).  Per unit:
//   MMA-A   TMEM_A[u % nbuf][128 x NA/VH] = packed S2_0 tile . Vin part
//           (TMA-fed, up to 4 stages)
//   fold    epilogue warps read TMEM_A, fold (hi+lo, re/im) and write the
//           unit's W slice straight into shared memory as step B's K-major
//           128B-swizzled operand B_B (rows (vec,l0,l1,p), 32 complex k)
//   MMA-B   TMEM_B[128 x NB/VH] += S2_1[g] K-slice (TMA) . B_B part
// TMEM_B accumulates over all units of the CTA and becomes one split-K plane.
// Roles: warp 0 issues the step-A TMA loads, warp 18 the step-B slice loads,
// warp 1 the MMA-A and warp 19 the MMA-B instructions (one elected lane
// each), warps 2..17 run the fold, four per TMEM lane quadrant, in two teams
// when TMEM_A is double-buffered.  In single-launch (cooperative) mode the
// grid also packs Vin before the units and sums the planes into y after
// them, between bounded grid barriers.  Every wait is bounded; on expiry the
// CTA aborts, lets its copies land, frees TMEM and flags the caller's status
// word.
// Shapes: L divides 32 and is a multiple of 4, k2 k3 == l0 l1 (a unit's K
// slice is 128 bf16 columns: two swizzle atoms), d in {1, 2, 4, 8}, NA = nvec
// k2 k3 d and NB = nvec l0 l1 d multiples of 16 up to 256, at most 8 S2_1
// tags with terms.
// ---------------------------------------------------------------------------
namespace {

constexpr int FU_THREADS = 640;  // warps: 0 A loads, 1 MMA-A, 2..17 fold, 18 B loads, 19 MMA-B
constexpr int FU_MAXG = 8;
constexpr int FU_STAGES = 4;
constexpr int FU_STAGE_A = 128 * 128;        // A tile: 128 rows x 64 bf16
constexpr int FU_STAGE_V = 256 * 128;        // Vin tile: up to 256 rows x 64 bf16
constexpr int FU_BB_ATOM = 256 * 128;        // B_B atom: up to 256 rows x 128 B
constexpr int FU_AB_ATOM = 128 * 128;        // A_B atom: 128 rows x 128 B
constexpr int FU_SMEM_MAX = 227 * 1024;      // dynamic shared memory opt-in limit per CTA
constexpr int FU_FIXED = 1024 + 2 * FU_BB_ATOM + 2 * FU_AB_ATOM + 256;  // alignment, B_B, A_B, barriers
constexpr int FU_PF_PAIRS = 2;                // L2 prefetch distance of the S2_0 tiles, in pairs

struct FusedMaps {
  CUtensorMap a[FU_MAXG];    // packed S2_0 tags of group g: rows (x0,x1,l0,l1, re/im, hi/lo), K (terms, k0 k1)
  CUtensorMap vin[FU_MAXG];  // packed Vin of group g: rows (vec,k2,k3,p), box NA / VH rows
  CUtensorMap b;             // packed S2_1 tags: rows (l2,l3, re/im, hi/lo), K regions per group
};

struct FusedParams {
  int n_pairs, x_tiles, G;
  int nkb[FU_MAXG];
  int NA, NB, a_rows;
  int VH;                 // vector parts per (x-tile, tag) pair: units are (pair, part)
  int NAh, NBh;           // step-A / step-B columns of one part
  int nbuf;               // TMEM_A buffers (2 when 2 NAh <= 256)
  int stages;             // step-A pipeline depth
  int stage_bytes;        // bytes of one stage (A tile + Vin part)
  int L, K23, d, XP;
  int64_t regB, kcB;
  int live_rows;  // rows of TMEM_B that carry data (4 l2 l3, rounded to 32)
  float* planes;  // [grid][NB][live_rows], column-major per CTA
  int* err;
  // single-launch mode (cooperative launch, all CTAs resident): the kernel
  // also packs Vin before step A and reduces the planes into y after step B,
  // the phases separated by grid-wide barriers on `sync` (zero at launch)
  int coop;
  VinTerms vt;
  const double2* x;
  uint32_t* vin;
  double2* y;
  int accumulate;
  int nvec, l0, l1, l2, l3;
  int64_t yv, yl0, yl1, yl2, yl3;
  unsigned int* sync;
};

// Pair pr = blockIdx.x + pc * gridDim.x of a CTA, tag-major (g = pr / x_tiles,
// t = pr % x_tiles), so that every CTA takes about the same share of each
// S2_1 tag; advanced incrementally, without divisions.
struct PairWalk {
  int t, g, t_inc, g_inc, x_tiles;
  __device__ PairWalk(int pr0, int step, int xt)
      : t(pr0 % xt), g(pr0 / xt), t_inc(step % xt), g_inc(step / xt), x_tiles(xt) {}
  __device__ void next() {
    t += t_inc;
    g += g_inc;
    if (t >= x_tiles) {
      t -= x_tiles;
      ++g;
    }
  }
};

// Grid-wide barrier of a cooperative launch: every CTA adds one arrival, then
// thread 0 polls (bounded) until all gridDim.x have arrived.  Release/acquire
// at GPU scope order the phases' global-memory writes before the reads.  A
// CTA whose wait runs out raises the launch's global abort word; every other
// CTA polls it (every 256 polls) and stops waiting too, raising its own
// abort flag, so the launch ends early instead of each CTA using up its bound.
__device__ bool grid_barrier(unsigned int* ctr, int* abort_word, volatile int* abort) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    uint32_t i = 0;
    for (; i < (1u << 22); ++i) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
      if (v >= gridDim.x) break;
      if ((i & 255u) == 255u && *reinterpret_cast<volatile int*>(abort_word)) break;
      __nanosleep(64);
    }
    if (i == (1u << 22)) atomicExch(abort_word, 1);
    if (*reinterpret_cast<volatile int*>(abort_word)) *abort = 1;
  }
  __syncthreads();
  return *abort == 0;
}

// Unit uc of a CTA (local counter) is part (uc % VH) of its pair (uc / VH);
// the CTA takes pairs blockIdx.x, blockIdx.x + gridDim.x, ... so that both
// parts of a pair run back to back (they share the pair's S2_1 slice).
// DD = d, the physical dimension (1, 2, 4 or 8): a compile-time constant so
// that the fold's register indexing is static.
template <int DD>
__global__ __launch_bounds__(FU_THREADS, 1) void stage3_fused_kernel(const __grid_constant__ FusedMaps maps,
                                                                     const __grid_constant__ FusedParams p) {
  using namespace umma;
  extern __shared__ uint8_t fsm_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(fsm_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* stage = sm;                                   // stages x (A tile, Vin part)
  uint8_t* bB = sm + p.stages * p.stage_bytes;           // 2 atoms (hi, lo), rows of part h at h NBh
  uint8_t* aB = bB + 2 * FU_BB_ATOM;                     // 2 atoms (hi, lo)
  // the fold's setup tables live in B_B until the fold warps have read them
  int2* tabN = reinterpret_cast<int2*>(bB);
  int2* tabM = tabN + 256;
  uint64_t* bars = reinterpret_cast<uint64_t*>(aB + 2 * FU_AB_ATOM);
  uint64_t* full = bars;             // [FU_STAGES]
  uint64_t* empty = bars + 4;        // [FU_STAGES]
  uint64_t* accA_full = bars + 8;    // [2] per TMEM_A buffer
  uint64_t* bB_ready = bars + 10;    // [2] per TMEM_A buffer: fold done (buffer free, B_B part written)
  uint64_t* bB_free = bars + 12;     // [2] per part: MMA-B of the part done (its B_B rows free)
  uint64_t* aB_full = bars + 14;
  uint64_t* aB_empty = bars + 15;
  uint64_t* doneB = bars + 16;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 17);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < FU_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accA_full[b], 1);
      mbar_init(&bB_ready[b], (p.VH == 2 && p.nbuf == 2) ? 8 : 16);  // the fold warps of the buffer's team
      mbar_init(&bB_free[b], 1);
    }
    mbar_init(aB_full, 1);
    mbar_init(aB_empty, 1);
    mbar_init(doneB, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (p.a_rows < 128) {
    // rows [a_rows, 128) of both A_B atoms stay zero (the operand's padding rows)
    for (int h = 0; h < 2; ++h) {
      uint4* z = reinterpret_cast<uint4*>(aB + h * FU_AB_ATOM + p.a_rows * 128);
      for (int i = threadIdx.x; i < (128 - p.a_rows) * 128 / 16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async();
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tB = tmem + 256;

  // Loads that do not depend on Vin start before phase 0: the S2_0 tiles of
  // the first `pre` step-A stages (their Vin parts follow after the barrier,
  // on the same full barrier) and the first pair's S2_1 slice.
  const int my_pairs0 = blockIdx.x < p.n_pairs ? (p.n_pairs - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  int pre = 0;
  PairWalk cwB((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
  int issuedB = 0, pcB0 = 0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < p.G; ++q) {
      prefetch_tensormap(&maps.a[q]);
      prefetch_tensormap(&maps.vin[q]);
    }
    prefetch_tensormap(&maps.b);
    PairWalk w((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
    for (int uc = 0, part = 0, kb = 0; pre < p.stages && uc < my_pairs0 * p.VH; ++pre) {
      mbar_arrive_expect_tx(&full[pre], (uint32_t)(FU_STAGE_A + p.NAh * 128));
      tma_load_2d(stage + pre * p.stage_bytes, &maps.a[w.g], kb * 64, w.t * 128, &full[pre]);
      if (++kb == p.nkb[w.g]) {
        kb = 0;
        ++uc;
        if (++part == p.VH) {
          part = 0;
          w.next();
        }
      }
    }
  } else if (threadIdx.x == 18 * 32 && my_pairs0 > 0) {
    mbar_arrive_expect_tx(aB_full, (uint32_t)(2 * p.a_rows * 128));
    const int64_t kk0 = (int64_t)cwB.t * p.XP * p.K23;
    tma_load_2d(aB, &maps.b, (int)(cwB.g * p.regB + 2 * kk0), 0, aB_full);
    tma_load_2d(aB + FU_AB_ATOM, &maps.b, (int)(cwB.g * p.regB + 2 * p.kcB + 2 * kk0), 0, aB_full);
    issuedB = 1;
    pcB0 = 1;
    cwB.next();
    if (my_pairs0 > 1) {
      const int64_t kn = (int64_t)cwB.t * p.XP * p.K23;
      tma_prefetch_2d(&maps.b, (int)(cwB.g * p.regB + 2 * kn), 0);
      tma_prefetch_2d(&maps.b, (int)(cwB.g * p.regB + 2 * p.kcB + 2 * kn), 0);
    }
  }
  if (p.coop) {
    // ---- phase 0: Vin of every term packed by the whole grid; the async
    // proxy (TMA) of every CTA reads it after the barrier
    const int per_term = (int)(p.vt.rows_out * p.vt.reg4), total = per_term * p.vt.n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
      const int term = e / per_term;
      pack_vin_slot(p.x, p.vin, p.vt, term, e - term * per_term);
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    grid_barrier(p.sync, reinterpret_cast<int*>(p.sync + 2), abort_flag);
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  // a CTA whose phase 0 failed takes no units (the status word reports it)
  const int my_pairs =
      (blockIdx.x < p.n_pairs && *abort_flag == 0) ? (p.n_pairs - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int n_units = my_pairs * p.VH;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer of step A: the unit's S2_0 tile and its Vin part
      int issued = 0, s = 0, part = 0;
      uint32_t ph = 0;
      bool ok = true;
      PairWalk cw((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
      // L2 prefetch of the S2_0 tiles FU_PF_PAIRS pairs ahead (pairs 1 ..
      // FU_PF_PAIRS - 1 up front; pair 0 was prefetched before phase 0)
      int pf = 1;
      PairWalk pw = cw;
      pw.next();
      auto prefetch_pair = [&]() {
        if (pf < my_pairs)
          for (int kb = 0; kb < p.nkb[pw.g]; ++kb) tma_prefetch_2d(&maps.a[pw.g], kb * 64, pw.t * 128);
        ++pf;
        pw.next();
      };
      for (int k = 1; k < FU_PF_PAIRS; ++k) prefetch_pair();
      for (int uc = 0; ok && uc < n_units; ++uc) {
        if (part == 0) prefetch_pair();
        const int g = cw.g, t = cw.t, nkb = p.nkb[g];
        for (int kb = 0; kb < nkb; ++kb) {
          uint8_t* st = stage + s * p.stage_bytes;
          if (issued >= pre) {  // (the first `pre` stages have their S2_0 tile requested)
            if (!(ok = mbar_wait_sleep(&empty[s], ph ^ 1u, abort_flag))) break;
            mbar_arrive_expect_tx(&full[s], (uint32_t)(FU_STAGE_A + p.NAh * 128));
            tma_load_2d(st, &maps.a[g], kb * 64, t * 128, &full[s]);
          }
          tma_load_2d(st + FU_STAGE_A, &maps.vin[g], kb * 64, part * p.NAh, &full[s]);
          ++issued;
          if (++s == p.stages) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (++part == p.VH) {
          part = 0;
          cw.next();
        }
      }
      if (*abort_flag) {
        // complete the early stages whose Vin part was never requested (any
        // in-bounds box), then let copies in flight land (bounded)
        for (; issued < pre; ++issued)
          tma_load_2d(stage + issued * p.stage_bytes + FU_STAGE_A, &maps.vin[0], 0, 0, &full[issued]);
        for (int i = max(0, issued - p.stages); i < issued; ++i)
          for (uint32_t q = 0; q < (1u << 20); ++q)
            if (mbar_try_wait(&full[i % p.stages], (uint32_t)((i / p.stages) & 1))) break;
      }
    }
  } else if (warp == 18) {
    if (lane == 0) {
      // ---- TMA producer of step B's S2_1 slice, one per pair (pair 0's was
      // requested before phase 0)
      int issued = issuedB;
      PairWalk cw = cwB;
      for (int pc = pcB0; pc < my_pairs; ++pc) {
        if (!mbar_wait_sleep(aB_empty, (uint32_t)((pc & 1) ^ 1), abort_flag)) break;
        mbar_arrive_expect_tx(aB_full, (uint32_t)(2 * p.a_rows * 128));
        const int64_t kk0 = (int64_t)cw.t * p.XP * p.K23;
        tma_load_2d(aB, &maps.b, (int)(cw.g * p.regB + 2 * kk0), 0, aB_full);
        tma_load_2d(aB + FU_AB_ATOM, &maps.b, (int)(cw.g * p.regB + 2 * p.kcB + 2 * kk0), 0, aB_full);
        ++issued;
        cw.next();
        if (pc + 1 < my_pairs) {  // the next pair's slice into L2 while this one is used
          const int64_t kn = (int64_t)cw.t * p.XP * p.K23;
          tma_prefetch_2d(&maps.b, (int)(cw.g * p.regB + 2 * kn), 0);
          tma_prefetch_2d(&maps.b, (int)(cw.g * p.regB + 2 * p.kcB + 2 * kn), 0);
        }
      }
      if (*abort_flag && issued > 0)
        for (uint32_t q = 0; q < (1u << 20); ++q)
          if (mbar_try_wait(aB_full, (uint32_t)((issued - 1) & 1))) break;
    }
  } else if (warp == 1 || warp == 19) {
    // ---- MMA issuers: warp 1 issues every unit's MMA-A into TMEM_A buffer
    // u % nbuf, warp 19 every unit's MMA-B once its fold is done, so that
    // neither's waits hold up the other's MMAs.  Each warp runs its loop
    // converged (its values stay warp-uniform) and one elected lane issues
    // each MMA and commit; per MMA the descriptors only advance their
    // start-address field (bytes >> 4).
    const bool leader = elect_one();
    struct Unit {
      int b, part, pc;
      uint32_t bph;  // phase parity of the unit's use of TMEM_A buffer b
    };
    auto advance = [&](Unit& u) {
      if (++u.part == p.VH) {
        u.part = 0;
        ++u.pc;
      }
      if (++u.b == p.nbuf) {
        u.b = 0;
        u.bph ^= 1u;
      }
    };
    bool ok = true;
    Unit u{0, 0, 0, 0u};
    if (warp == 1) {
      const uint32_t idA = idesc_bf16_f32(128, p.NAh);
      const uint64_t dStage = smem_desc_sw128(smem_u32(stage));
      const uint32_t dStageStep = (uint32_t)p.stage_bytes >> 4;
      constexpr uint32_t dV = FU_STAGE_A >> 4;
      int s = 0;
      PairWalk cw((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
      uint32_t ph = 0;
      for (int uc = 0; ok && uc < n_units; ++uc) {
        // TMEM_A buffer u.b was last read by the fold of unit uc - nbuf
        if (uc >= p.nbuf && !(ok = mbar_wait_sleep(&bB_ready[u.b], u.bph ^ 1u, abort_flag))) break;
        const uint32_t tA = tmem + (uint32_t)(u.b * p.NAh);
        const int nkb = p.nkb[cw.g];
        for (int kb = 0; kb < nkb; ++kb) {
          if (!(ok = mbar_wait_sleep(&full[s], ph, abort_flag))) break;
          tc_fence_after();
          if (leader) {
            const uint64_t da = dStage + s * dStageStep;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              mma_bf16(tA, da + kk * 2, da + (dV + kk * 2), idA, (kb > 0 || kk > 0) ? 1u : 0u);
            mma_commit(&empty[s]);
          }
          __syncwarp();
          if (++s == p.stages) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (!ok) break;
        if (leader) mma_commit(&accA_full[u.b]);
        __syncwarp();
        advance(u);
        if (u.part == 0) cw.next();
      }
    } else {
      const uint32_t idB = idesc_bf16_f32(128, p.NBh);
      const uint64_t dAB = smem_desc_sw128(smem_u32(aB)), dBB = smem_desc_sw128(smem_u32(bB));
      const uint32_t dPartB = (uint32_t)(p.NBh * 128) >> 4;
      constexpr uint32_t dAtomAB = FU_AB_ATOM >> 4, dAtomBB = FU_BB_ATOM >> 4;
      for (int uc = 0; ok && uc < n_units; ++uc) {
        // MMA-B of unit uc: its fold wrote B_B part u.part; the pair's S2_1 slice is loaded
        if (!(ok = mbar_wait_sleep(&bB_ready[u.b], u.bph, abort_flag))) break;
        if (u.part == 0 && !(ok = mbar_wait_sleep(aB_full, (uint32_t)(u.pc & 1), abort_flag))) break;
        tc_fence_after();
        if (leader) {
          const uint32_t d = tB + (uint32_t)(u.part * p.NBh);
          const uint64_t bb = dBB + u.part * dPartB;
#pragma unroll
          for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              mma_bf16(d, dAB + (h * dAtomAB + kk * 2), bb + (h * dAtomBB + kk * 2), idB,
                       (u.pc > 0 || h > 0 || kk > 0) ? 1u : 0u);
          mma_commit(&bB_free[u.part]);
          if (u.part == p.VH - 1) mma_commit(aB_empty);
        }
        __syncwarp();
        advance(u);
      }
      if (leader) mma_commit(doneB);
      __syncwarp();
    }
  } else if (warp >= 2 && warp <= 17) {
    // ---- fold epilogue: warps 2..17; quadrant = warp % 4.  With two vector
    // parts and two TMEM_A buffers the warps form two teams of 8 (team =
    // part = buffer) that fold alternate units concurrently; otherwise one
    // team of 16.  A warp takes the 32-column chunks cgi, cgi + ncg, ...
    const int quad = warp & 3, quarter = (warp - 2) >> 2;
    const int nteams = (p.VH == 2 && p.nbuf == 2) ? 2 : 1, ncg = 4 / nteams;
    const int team = nteams == 2 ? (quarter & 1) : 0, cgi = nteams == 2 ? (quarter >> 1) : quarter;
    const int et = threadIdx.x - 64;  // 0..511
    // tables over the columns of part 0 (part h shifts the B_B rows by h NBh):
    // per step-A column n = (vec, k23, p): {B_B row part, k part}; per tile row m = (xp, l)
    for (int n = et; n < p.NAh; n += 512) {
      const int pp = n % DD, q = n / DD;
      const int k23 = q % p.K23, vec = q / p.K23;
      tabN[n] = make_int2(vec * p.L * DD + pp, k23);
    }
    if (et < 32) tabM[et] = make_int2((et % p.L) * DD, (et / p.L) * p.K23);
    asm volatile("bar.sync 1, 512;" ::: "memory");
    const int m = quad * 8 + (lane >> 2);  // complex row of this lane's quad within the tile
    const int2 tm = tabM[m];
    const uint32_t sh_hi = smem_u32(bB), sh_lo = smem_u32(bB + FU_BB_ATOM);
    // Ownership after the two exchange stages.  The 32 columns of a chunk form
    // 8 sets of 4 columns with one (vec, p) and 4 consecutive k23 (column
    // stride d): the 4 complex values of a set are 16 contiguous bytes of one
    // B_B row, written with one 16-byte store per half (hi, lo).  Lane
    // (c, h) = ((lane >> 1) & 1, lane & 1) of a quad ends with sets
    // 4h + 2c + s2, s2 = 0, 1.  Set S holds chunk columns (S / d) 4d + e d + S % d.
    const int hsel = lane & 1, csel = (lane >> 1) & 1;
    const int nchunks = (p.NAh + 31) / 32;
    const int nch = (nchunks - cgi + ncg - 1) / ncg;  // at most 2 (NAh <= 128 with two teams)
    // This lane's B_B byte offsets are the same in every unit (plus the part's
    // row shift): computed once, so no shared-memory load sits between stores.
    uint32_t offs[4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int S = 4 * hsel + 2 * csel + s2;
        const int col = (cgi + ncg * i) * 32 + (S / DD) * 4 * DD + S % DD;
        uint32_t off = 0xffffffffu;
        if (i < nch && col < p.NAh) {
          const int2 tn = tabN[col];
          const int row = tn.x + tm.x, kk = tn.y + tm.y;  // kk % 4 == 0
          off = (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + (((kk >> 2) ^ (row & 7)) << 4));
        }
        offs[i * 2 + s2] = off;
      }
    asm volatile("bar.sync 1, 512;" ::: "memory");  // tables read: B_B may be written
    // chunk column of element e of set S: (S / d) 4d + e d + S % d
    auto setcol = [](int S, int e) { return (S / DD) * 4 * DD + e * DD + S % DD; };
    bool ok = true;
    int b = 0, part = 0, pc = 0;
    uint32_t bph = 0;
    auto step_unit = [&]() {
      if (++b == p.nbuf) {
        b = 0;
        bph ^= 1u;
      }
      if (++part == p.VH) {
        part = 0;
        ++pc;
      }
    };
    if (team == 1) step_unit();
    for (int uc = team; uc < n_units; uc += nteams) {
      if (!(ok = mbar_wait_sleep(&accA_full[b], bph, abort_flag))) break;
      // B_B part `part` was last read by the MMA-B of unit uc - VH (pair pc - 1)
      if (pc > 0 && !(ok = mbar_wait_sleep(&bB_free[part], (uint32_t)((pc & 1) ^ 1), abort_flag))) break;
      tc_fence_after();
      const uint32_t tA = tmem + (uint32_t)(b * p.NAh);
      const uint32_t lanes = (uint32_t)(quad * 32) << 16;
      const uint32_t shift = (uint32_t)(part * p.NBh * 128);
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (i >= nch) break;
        uint32_t r[32];
        tmem_ld_32x32b_x32(tA + lanes + (uint32_t)((cgi + ncg * i) * 32), r);
        tmem_ld_wait();
        // stage 1 (lane ^ 1): sum the hi/lo rows; lane h keeps sets 4h..4h+3
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const float a = __uint_as_float(r[setcol(k >> 2, k & 3)]);
          const float z = __uint_as_float(r[setcol(4 + (k >> 2), k & 3)]);
          const float keep = hsel ? z : a, send = hsel ? a : z;
          v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
        }
        // stage 2 (lane ^ 2): exchange re/im; lane c keeps sets 4h + 2c + s2
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
          uint32_t hi[4], lo[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float a = v[s2 * 4 + e], z = v[(2 + s2) * 4 + e];
            const float keep = csel ? z : a, send = csel ? a : z;
            const float recv = __shfl_xor_sync(0xffffffffu, send, 2);
            const float re = csel ? recv : keep, im = csel ? keep : recv;
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(re, im);
            const float2 hf = __bfloat1622float2(h2);
            const __nv_bfloat162 l2 = __floats2bfloat162_rn(re - hf.x, im - hf.y);
            hi[e] = *reinterpret_cast<const uint32_t*>(&h2);
            lo[e] = *reinterpret_cast<const uint32_t*>(&l2);
          }
          const uint32_t off = offs[i * 2 + s2];
          if (off != 0xffffffffu) {
            // explicit shared-space stores (the aligned base pointer is generic)
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(sh_hi + shift + off), "r"(hi[0]),
                         "r"(hi[1]), "r"(hi[2]), "r"(hi[3])
                         : "memory");
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(sh_lo + shift + off), "r"(lo[0]),
                         "r"(lo[1]), "r"(lo[2]), "r"(lo[3])
                         : "memory");
          }
        }
      }
      fence_proxy_async();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bB_ready[b]);
      for (int k = 0; k < nteams; ++k) step_unit();
    }
    // ---- TMEM_B -> this CTA's split-K plane (zeros when the CTA had no unit)
    const bool done = ok && mbar_wait_sleep(doneB, 0, abort_flag);
    tc_fence_after();
    if (done && quad * 32 < p.live_rows) {
      // column-major plane [NB][live_rows]: a warp's 32 lanes (rows) store 128
      // consecutive bytes per column
      float* plane = p.planes + (int64_t)blockIdx.x * p.live_rows * p.NB;
      const int row = quad * 32 + lane;
      for (int c0 = quarter * 32; c0 < p.NB; c0 += 128) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tB + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (c0 + j < p.NB && row < p.live_rows)
            plane[(int64_t)(c0 + j) * p.live_rows + row] = n_units > 0 ? __uint_as_float(r[j]) : 0.f;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
  if (p.coop && grid_barrier(p.sync + 1, reinterpret_cast<int*>(p.sync + 2), abort_flag) && warp >= 2 &&
      warp <= 17) {
    // ---- phase 2: the planes of all CTAs summed into y, the same arithmetic
    // as reduce_planes_cm_kernel: a unit is (column n, 32 rows); two groups
    // of 8 warps, warp w of a group takes planes w, w + 8, ... (compensated
    // FP32), partials added in FP64 in warp order, quads fold their 4 rows
    const int grp = (warp - 2) >> 3, wq = (warp - 2) & 7;
    double* part = reinterpret_cast<double*>(stage) + grp * 256;
    const int rgs = p.live_rows / 32, n_red = p.NB * rgs, L = p.live_rows;
    const int64_t pstride = (int64_t)L * p.NB;
    for (int ur = blockIdx.x * 2 + grp; ur < n_red; ur += 2 * gridDim.x) {
      const int n = ur / rgs, r = (ur - n * rgs) * 32 + lane;
      const float* src = p.planes + (int64_t)n * L + r;
      Kahan acc;
      for (int z0 = wq; z0 < (int)gridDim.x; z0 += 24 * 8) {
        float v[24];
#pragma unroll
        for (int u = 0; u < 24; ++u) {
          const int z = z0 + u * 8;
          v[u] = z < (int)gridDim.x ? __ldcg(src + z * pstride) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 24; ++u) acc.add(v[u]);
      }
      part[wq * 32 + lane] = acc.value();
      asm volatile("bar.sync %0, 256;" ::"r"(2 + grp) : "memory");
      if (wq == 0) {
        double v = part[lane];
        for (int q = 1; q < 8; ++q) v += part[q * 32 + lane];
        v += __shfl_xor_sync(0xffffffffu, v, 1);            // hi + lo
        const double o = __shfl_xor_sync(0xffffffffu, v, 2);  // the other of re / im
        const int m = r >> 2;
        if ((lane & 3) == 0 && m < p.l2 * p.l3) {
          int nn = n;
          const int pi = nn % DD;
          nn /= DD;
          const int l1i = nn % p.l1;
          nn /= p.l1;
          const int l0i = nn % p.l0, vec = nn / p.l0;
          const int64_t off = (m / p.l3) * p.yl2 + (m % p.l3) * p.yl3 + vec * p.yv + l0i * p.yl0 + l1i * p.yl1 + pi;
          double2 val = make_double2(v, o);
          if (p.accumulate) val = cadd(val, p.y[off]);
          p.y[off] = val;
        }
      }
      asm volatile("bar.sync %0, 256;" ::"r"(2 + grp) : "memory");
    }
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(p.err, CARC_NOT_CONVERGED);
}

int fused_grid(const S3& s, const TermGroups& tg) {
  const int64_t pairs = (s.x0 * s.x1 * s.l0 * s.l1 / 32) * (int64_t)tg.i1.size();
  return (int)std::max<int64_t>(1, std::min<int64_t>(152, pairs));
}

bool fused_eligible(const S3& s, int nvec, const TermGroups& tg) {
  const int64_t L = s.l0 * s.l1, K23 = s.k2 * s.k3;
  const int64_t NA = (int64_t)nvec * K23 * s.d, NB = (int64_t)nvec * L * s.d;
  return L <= 32 && 32 % L == 0 && K23 == L && NA % 16 == 0 && NA <= 256 && NB % 16 == 0 && NB <= 256 &&
         (int)tg.i1.size() <= FU_MAXG && 4 * s.l2 * s.l3 <= 128 && (s.x0 * s.x1 * L) % 32 == 0 &&
         L % 4 == 0 && 8 % s.d == 0;
}

// ---------------------------------------------------------------------------
// Fused matvec on compact operands (F2): step A and step B in one persistent
// cooperative kernel, W kept on chip, hi and lo parts of the split summed in
// the accumulator and the lo x lo product left out.
//
// A pair is (x-tile t of 64 complex step-A rows = XP x values x all L rows,
// S2_1 tag g); a unit is one vector part of a pair (VH parts of NAh complex
// columns).  Per unit:
//   MMA-A  TMEM_A[u % 2][(m, re/im) x NAh] = S2_0 tile . Vin part, per term
//          and K step three products hi.hi + hi.lo + lo.hi (TMA-fed, up to
//          4 stages of one term each)
//   fold   TMEM_A -> W^T[u % 2] as step B's A operand in shared memory: row
//          n_B = (vec, l0, l1, p) of the part, K = the pair's 64 complex
//          (x, k2, k3), [hi plane | lo plane] of (re, im), 128-byte swizzled
//   MMA-B  TMEM_B[part][n_B x (j, re/im)] += W^T . S2_1 slice (TMA), three
//          products per K step, accumulated over all units of the CTA
// TMEM_B becomes one split-K plane per CTA; after a grid barrier the grid sums
// the planes into y (compensated FP32 per warp in plane order, FP64 across
// warps in warp order).  Vin is packed by the whole grid before a first grid
// barrier.  Roles: warp 0 step-A TMA, warp 1 MMA-A, warps 2..17 fold, warp 18
// S2_1 TMA, warp 19 MMA-B.  Every wait is bounded; on expiry the CTA aborts,
// lets its copies land, frees TMEM and flags the caller's status word.
// Shapes (geometry2 and f2_eligible): k2 k3 == l0 l1 = L, L % 4 == 0, L
// divides 64, x0 x1 L a multiple of 64, 2 round_up(2 k0 k1, 16) <= 64,
// 2 l2 l3 <= 128, d in {1, 2, 4, 8}, NAh = nvec L d / VH a multiple of 16
// up to 128, at most 8 S2_1 tags with terms.
// ---------------------------------------------------------------------------
constexpr int F2_THREADS = 640;
constexpr int F2_STAGES = 4;
constexpr int F2_STAGE_A = 128 * 128;   // A tile: 128 rows x 64 bf16
constexpr int F2_AB_ATOM = 128 * 128;   // W^T: 128 rows x 64 bf16 per atom
constexpr int F2_AB = 4 * F2_AB_ATOM;   // W^T: [hi 128 | lo 128] columns
constexpr int F2_SMEM_MAX = 227 * 1024;
constexpr int F2_PF_PAIRS = 2;          // L2 prefetch distance, in pairs

struct Vin2 {
  int n;
  int64_t rows, kc, k23, d, wp2;          // wp2: u32 column of the lo plane
  const double2* op[kVinTermsPerLaunch];
  int64_t dst[kVinTermsPerLaunch];        // u32 offset of the term's region in row 0
  int64_t pitch[kVinTermsPerLaunch];      // u32 per row
};

// one u32 (bf16 pair) of a packed Vin region: row n = (vec, k2, k3, p),
// column col in [0, 32): hi (re, im) of k = col below wp2, lo of k = col - wp2
// in [wp2, 2 wp2), zero elsewhere and for k >= kc
__device__ __forceinline__ void pack_vin2_slot(const double2* __restrict__ x, uint32_t* __restrict__ out,
                                               const Vin2& p, int term, int t) {
  const int n = t >> 5, col = t & 31;
  const int kc = (int)p.kc, k23 = (int)p.k23, d = (int)p.d, wp2 = (int)p.wp2;
  int k = col;
  bool lo = false;
  if (col >= wp2) {
    k = col - wp2;
    lo = true;
  }
  uint32_t word = 0u;
  if (k < kc && col < 2 * wp2) {
    const double2* O = p.op[term];
    const int q = n / d, pp = n - q * d;
    const int vec = q / k23, kk = q - vec * k23;
    const double2* xv = x + (((int64_t)vec * kc + k) * k23 + kk) * d;
    float fr, fi;
    if (O == nullptr) {
      const double2 v = xv[pp];
      fr = (float)v.x;
      fi = (float)v.y;
    } else {
      fr = 0.f;
      fi = 0.f;
      for (int qq = 0; qq < d; ++qq) {
        const double2 o = O[pp * d + qq], v = xv[qq];
        const float orr = (float)o.x, oi = (float)o.y, vr = (float)v.x, vi = (float)v.y;
        fr = fmaf(orr, vr, fmaf(-oi, vi, fr));
        fi = fmaf(orr, vi, fmaf(oi, vr, fi));
      }
    }
    const __nv_bfloat16 hr = __float2bfloat16_rn(fr), hm = __float2bfloat16_rn(fi);
    __nv_bfloat162 w2;
    if (lo)
      w2 = __halves2bfloat162(__float2bfloat16_rn(fr - __bfloat162float(hr)),
                              __float2bfloat16_rn(fi - __bfloat162float(hm)));
    else
      w2 = __halves2bfloat162(hr, hm);
    word = *reinterpret_cast<const uint32_t*>(&w2);
  }
  out[p.dst[term] + (int64_t)n * p.pitch[term] + col] = word;
}

struct F2Maps {
  CUtensorMap a[F2_MAXG];    // compact S2_0 of group g: rows (m, re/im), one 64-column region per term
  CUtensorMap vin[F2_MAXG];  // Vin of group g: rows (vec, k2, k3, p), box NAh rows
  CUtensorMap b;             // compact S2_1: rows (j, re/im), regions of 4 KcB per group
};

struct F2Params {
  int n_pairs, x_tiles, G;
  int nterm[F2_MAXG];
  int VH, NAh, NBh, NBB, nksA;
  int stages, stage_bytes;
  int L, K23, XP;
  int64_t kcB4, kcB2;
  float* planes;  // [grid][VH][NBB][128] (column-major per part)
  int* err;
  Vin2 vt;
  const double2* x;
  uint32_t* vin;
  double2* y;
  int accumulate;
  int nvec, l0, l1, l2, l3;
  int64_t yv, yl0, yl1, yl2, yl3;
  unsigned int* sync;
  int* abort_word;  // raised by a CTA whose grid barrier timed out
};

__device__ bool f2_grid_barrier(unsigned int* ctr, int* abort_word, volatile int* abort) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    uint32_t i = 0;
    for (; i < (1u << 22); ++i) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
      if (v >= gridDim.x) break;
      if ((i & 255u) == 255u && *reinterpret_cast<volatile int*>(abort_word)) break;
      __nanosleep(64);
    }
    if (i == (1u << 22)) atomicExch(abort_word, 1);
    if (*reinterpret_cast<volatile int*>(abort_word)) *abort = 1;
  }
  __syncthreads();
  return *abort == 0;
}

template <int DD>
__global__ __launch_bounds__(F2_THREADS, 1) void stage3_fused2_kernel(const __grid_constant__ F2Maps maps,
                                                                      const __grid_constant__ F2Params p) {
  using namespace umma;
  extern __shared__ uint8_t f2sm_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(f2sm_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* stage = sm;                                      // stages x (A tile, Vin part)
  uint8_t* aB = sm + p.stages * p.stage_bytes;              // W^T: 2 buffers x 4 atoms of 128 rows
  const int bb_atom = p.NBB * 128;
  uint8_t* bB = aB + 2 * F2_AB;                             // 2 buffers x 4 atoms of NBB rows
  uint64_t* bars = reinterpret_cast<uint64_t*>(bB + 8 * bb_atom);
  uint64_t* full = bars;           // [4]
  uint64_t* empty = bars + 4;      // [4]
  uint64_t* accA_full = bars + 8;  // [2] MMA-A of the unit committed into TMEM_A[u % 2]
  uint64_t* fold_done = bars + 10; // [2] fold of unit u finished (TMEM_A[u % 2] read, W^T[u % 2] written)
  uint64_t* aB_free = bars + 12;   // [2] MMA-B of unit u done reading W^T[u % 2]
  uint64_t* bB_full = bars + 14;   // [2] per pair parity
  uint64_t* bB_empty = bars + 16;  // [2]
  uint64_t* doneB = bars + 18;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 19);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < F2_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accA_full[b], 1);
      mbar_init(&fold_done[b], 16);
      mbar_init(&aB_free[b], 1);
      mbar_init(&bB_full[b], 1);
      mbar_init(&bB_empty[b], 1);
    }
    mbar_init(doneB, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  // rows [NBh, 128) of W^T feed only discarded output rows; zero them once
  if (p.NBh < 128) {
    for (int a = 0; a < 8; ++a) {
      uint4* z = reinterpret_cast<uint4*>(aB + a * F2_AB_ATOM + p.NBh * 128);
      for (int i = threadIdx.x; i < (128 - p.NBh) * 8; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async();
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tB = tmem + 256;
  const uint32_t stepA_bytes = (uint32_t)(F2_STAGE_A + p.NAh * 128);

  // S2_0 tiles of the first stages and the first pair's S2_1 slice do not
  // depend on Vin: requested before the packing phase
  const int my_pairs0 = blockIdx.x < p.n_pairs ? (p.n_pairs - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  int pre = 0;
  PairWalk cwB((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
  int pcB0 = 0;
  auto load_bB = [&](int pc, const PairWalk& w) {
    const int sb = pc & 1;
    uint8_t* dst = bB + sb * 4 * bb_atom;
    mbar_arrive_expect_tx(&bB_full[sb], (uint32_t)(4 * bb_atom));
    const int x0 = (int)(w.g * p.kcB4 + 2 * (int64_t)w.t * F2_XT);
    tma_load_2d(dst, &maps.b, x0, 0, &bB_full[sb]);
    tma_load_2d(dst + bb_atom, &maps.b, x0 + 64, 0, &bB_full[sb]);
    tma_load_2d(dst + 2 * bb_atom, &maps.b, (int)(x0 + p.kcB2), 0, &bB_full[sb]);
    tma_load_2d(dst + 3 * bb_atom, &maps.b, (int)(x0 + p.kcB2 + 64), 0, &bB_full[sb]);
  };
  // L2 prefetch of a pair's S2_0 tiles / S2_1 slice
  auto prefetch_a = [&](const PairWalk& w) {
    for (int j = 0; j < p.nterm[w.g]; ++j) tma_prefetch_2d(&maps.a[w.g], j * 64, w.t * 128);
  };
  auto prefetch_b = [&](const PairWalk& w) {
    const int x0 = (int)(w.g * p.kcB4 + 2 * (int64_t)w.t * F2_XT);
    tma_prefetch_2d(&maps.b, x0, 0);
    tma_prefetch_2d(&maps.b, x0 + 64, 0);
    tma_prefetch_2d(&maps.b, (int)(x0 + p.kcB2), 0);
    tma_prefetch_2d(&maps.b, (int)(x0 + p.kcB2 + 64), 0);
  };
  if (threadIdx.x == 0) {
    for (int q = 0; q < p.G; ++q) {
      prefetch_tensormap(&maps.a[q]);
      prefetch_tensormap(&maps.vin[q]);
    }
    prefetch_tensormap(&maps.b);
    PairWalk w((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
    {  // pairs 0 .. F2_PF_PAIRS into L2 while Vin is packed
      PairWalk w2 = w;
      for (int k = 0; k <= F2_PF_PAIRS && k < my_pairs0; ++k, w2.next()) prefetch_a(w2);
    }
    for (int uc = 0, part = 0, j = 0; pre < p.stages && uc < my_pairs0 * p.VH; ++pre) {
      mbar_arrive_expect_tx(&full[pre], stepA_bytes);
      tma_load_2d(stage + pre * p.stage_bytes, &maps.a[w.g], j * 64, w.t * 128, &full[pre]);
      if (++j == p.nterm[w.g]) {
        j = 0;
        ++uc;
        if (++part == p.VH) {
          part = 0;
          w.next();
        }
      }
    }
  } else if (threadIdx.x == 18 * 32 && my_pairs0 > 0) {
    load_bB(0, cwB);
    cwB.next();
    pcB0 = 1;
    PairWalk w2 = cwB;
    for (int k = 1; k <= F2_PF_PAIRS && k < my_pairs0; ++k, w2.next()) prefetch_b(w2);
  }
  // ---- phase 0: Vin of every term packed by the whole grid
  {
    const int per_term = (int)(p.vt.rows * 32), total = per_term * p.vt.n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
      const int term = e / per_term;
      pack_vin2_slot(p.x, p.vin, p.vt, term, e - term * per_term);
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    f2_grid_barrier(p.sync, p.abort_word, abort_flag);
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  const int my_pairs = (my_pairs0 > 0 && *abort_flag == 0) ? my_pairs0 : 0;
  const int n_units = my_pairs * p.VH;

  if (warp == 0) {
    if (lane == 0) {
      // ---- step-A producer: per unit and term, the S2_0 tile and the Vin part
      int issued = 0, s = 0, part = 0;
      uint32_t ph = 0;
      bool ok = true;
      PairWalk cw((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
      PairWalk pw = cw;  // L2 prefetch of the S2_0 tiles F2_PF_PAIRS pairs ahead
      for (int k = 0; k < F2_PF_PAIRS; ++k) pw.next();
      for (int uc = 0; ok && uc < n_units; ++uc) {
        if (part == 0 && uc / p.VH + F2_PF_PAIRS < my_pairs) prefetch_a(pw);
        const int g = cw.g, t = cw.t;
        for (int j = 0; j < p.nterm[g]; ++j) {
          uint8_t* st = stage + s * p.stage_bytes;
          if (issued >= pre) {
            if (!(ok = mbar_wait_sleep(&empty[s], ph ^ 1u, abort_flag))) break;
            mbar_arrive_expect_tx(&full[s], stepA_bytes);
            tma_load_2d(st, &maps.a[g], j * 64, t * 128, &full[s]);
          }
          tma_load_2d(st + F2_STAGE_A, &maps.vin[g], j * 64, part * p.NAh, &full[s]);
          ++issued;
          if (++s == p.stages) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (++part == p.VH) {
          part = 0;
          cw.next();
          pw.next();
        }
      }
      if (*abort_flag) {
        // stages whose S2_0 tile was requested but not their Vin part get an
        // in-bounds Vin box, then every copy in flight is let land (bounded)
        for (; issued < pre; ++issued)
          tma_load_2d(stage + issued * p.stage_bytes + F2_STAGE_A, &maps.vin[0], 0, 0, &full[issued]);
        for (int i = max(0, issued - p.stages); i < issued; ++i)
          for (uint32_t q = 0; q < (1u << 20); ++q)
            if (mbar_try_wait(&full[i % p.stages], (uint32_t)((i / p.stages) & 1))) break;
      }
    }
  } else if (warp == 18) {
    if (lane == 0) {
      // ---- step-B producer: the pair's S2_1 slice (4 atoms), double-buffered
      int issued = pcB0;
      PairWalk cw = cwB;
      for (int pc = pcB0; pc < my_pairs; ++pc) {
        if (pc >= 2 && !mbar_wait_sleep(&bB_empty[pc & 1], (uint32_t)(((pc >> 1) & 1) ^ 1), abort_flag)) break;
        load_bB(pc, cw);
        ++issued;
        cw.next();
        if (pc + F2_PF_PAIRS < my_pairs) {
          PairWalk w2 = cw;
          for (int k = 1; k < F2_PF_PAIRS; ++k) w2.next();
          prefetch_b(w2);
        }
      }
      if (*abort_flag)
        for (int i = max(0, issued - 2); i < issued; ++i)
          for (uint32_t q = 0; q < (1u << 20); ++q)
            if (mbar_try_wait(&bB_full[i & 1], (uint32_t)((i >> 1) & 1))) break;
    }
  } else if (warp == 1) {
    // ---- MMA-A issuer (converged warp, one elected lane issues)
    const bool leader = elect_one();
    const uint32_t idA = idesc_bf16_f32(128, p.NAh);
    const uint64_t dStage = smem_desc_sw128(smem_u32(stage));
    const uint32_t dStageStep = (uint32_t)p.stage_bytes >> 4;
    constexpr uint32_t dV = F2_STAGE_A >> 4;
    const int nks = p.nksA;
    int s = 0, part = 0;
    uint32_t ph = 0;
    bool ok = true;
    PairWalk cw((int)blockIdx.x, (int)gridDim.x, p.x_tiles);
    for (int uc = 0; ok && uc < n_units; ++uc) {
      const int b = uc & 1;
      // TMEM_A[b] was last read by the fold of unit uc - 2
      if (uc >= 2 && !(ok = mbar_wait_sleep(&fold_done[b], (uint32_t)(((uc >> 1) & 1) ^ 1), abort_flag))) break;
      const uint32_t tA = tmem + (uint32_t)(b * 128);
      const int nt = p.nterm[cw.g];
      for (int j = 0; j < nt; ++j) {
        if (!(ok = mbar_wait_sleep(&full[s], ph, abort_flag))) break;
        tc_fence_after();
        if (leader) {
          const uint64_t da = dStage + s * dStageStep, dv = da + dV;
          for (int kk = 0; kk < nks; ++kk) {
            mma_bf16(tA, da + kk * 2, dv + kk * 2, idA, (j > 0 || kk > 0) ? 1u : 0u);  // hi . hi
            mma_bf16(tA, da + kk * 2, dv + (nks + kk) * 2, idA, 1u);                     // hi . lo
            mma_bf16(tA, da + (nks + kk) * 2, dv + kk * 2, idA, 1u);                     // lo . hi
          }
          mma_commit(&empty[s]);
        }
        __syncwarp();
        if (++s == p.stages) {
          s = 0;
          ph ^= 1u;
        }
      }
      if (!ok) break;
      if (leader) mma_commit(&accA_full[b]);
      __syncwarp();
      if (++part == p.VH) {
        part = 0;
        cw.next();
      }
    }
  } else if (warp == 19) {
    // ---- MMA-B issuer
    const bool leader = elect_one();
    const uint32_t idB = idesc_bf16_f32(128, p.NBB);
    const uint64_t dAB = smem_desc_sw128(smem_u32(aB)), dBB = smem_desc_sw128(smem_u32(bB));
    constexpr uint32_t dAtomA = F2_AB_ATOM >> 4;
    const uint32_t dAtomB = (uint32_t)bb_atom >> 4;
    bool ok = true;
    int part = 0, pc = 0;
    for (int uc = 0; ok && uc < n_units; ++uc) {
      if (!(ok = mbar_wait_sleep(&fold_done[uc & 1], (uint32_t)((uc >> 1) & 1), abort_flag))) break;
      if (part == 0 && !(ok = mbar_wait_sleep(&bB_full[pc & 1], (uint32_t)((pc >> 1) & 1), abort_flag))) break;
      tc_fence_after();
      if (leader) {
        const uint32_t d = tB + (uint32_t)(part * p.NBB);
        const uint64_t bb = dBB + (uint32_t)((pc & 1) * 4) * dAtomB;
        const uint64_t da = dAB + (uint32_t)((uc & 1) * 4) * dAtomA;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const uint32_t oa = (uint32_t)(kk >> 2) * dAtomA + (uint32_t)(kk & 3) * 2;
          const uint32_t ob = (uint32_t)(kk >> 2) * dAtomB + (uint32_t)(kk & 3) * 2;
          mma_bf16(d, da + oa, bb + ob, idB, (pc > 0 || kk > 0) ? 1u : 0u);  // hi . hi
          mma_bf16(d, da + oa, bb + 2 * dAtomB + ob, idB, 1u);                // hi . lo
          mma_bf16(d, da + 2 * dAtomA + oa, bb + ob, idB, 1u);                // lo . hi
        }
        mma_commit(&aB_free[uc & 1]);
        if (part == p.VH - 1) mma_commit(&bB_empty[pc & 1]);
      }
      __syncwarp();
      if (++part == p.VH) {
        part = 0;
        ++pc;
      }
    }
    if (leader) mma_commit(doneB);
    __syncwarp();
  } else if (warp >= 2 && warp <= 17) {
    // ---- fold: TMEM_A (lanes (m, re/im), columns n of the part) -> W^T.
    // The quadrant's 4 warps take the 32-column chunks ci = 0..3 (NAh / 32
    // of them carry columns).  Lane pair (m, re), (m, im) exchanges halves
    // so that each lane ends with 4 sets of 4 complex values, a set being 4
    // consecutive k2 k3 of one (vec, p): 16 contiguous bytes of a W^T row
    // per plane.  Set S holds chunk columns (S / d) 4d + e d + S % d.
    const int quad = warp & 3, ci = (warp - 2) >> 2;
    const int csel = lane & 1;
    const int m = quad * 16 + (lane >> 1);  // complex step-A row within the x-tile
    const int xp = m / p.L, l = m - xp * p.L;
    const bool has_chunk = ci * 32 < p.NAh;
    uint32_t offs[4];
#pragma unroll
    for (int s2 = 0; s2 < 4; ++s2) {
      const int S = 2 * s2 + csel;
      const int n = ci * 32 + (S / DD) * 4 * DD + S % DD;  // part column of element 0 of set S
      const int pp = n % DD, q = n / DD;
      const int k23 = q % p.K23, vec = q / p.K23;
      const int row = (vec * p.L + l) * DD + pp;            // W^T row n_B
      const int kb = xp * p.K23 + k23;                      // complex K column (multiple of 4)
      offs[s2] = (uint32_t)((kb >> 5) * F2_AB_ATOM + (row >> 3) * 1024 + (row & 7) * 128 +
                            ((((kb & 31) >> 2) ^ (row & 7)) << 4));
    }
    auto setcol = [](int S, int e) { return (S / DD) * 4 * DD + e * DD + S % DD; };
    const uint32_t sh0 = smem_u32(aB);
    bool ok = true;
    for (int uc = 0; uc < n_units; ++uc) {
      const int b = uc & 1;
      if (!(ok = mbar_wait_sleep(&accA_full[b], (uint32_t)((uc >> 1) & 1), abort_flag))) break;
      // W^T[b] was last read by the MMA-B of unit uc - 2
      if (uc >= 2 && !(ok = mbar_wait_sleep(&aB_free[b], (uint32_t)(((uc >> 1) & 1) ^ 1), abort_flag))) break;
      tc_fence_after();
      if (has_chunk) {
        const uint32_t sh = sh0 + (uint32_t)(b * F2_AB);
        uint32_t r[32];
        tmem_ld_32x32b_x32(tmem + (uint32_t)(b * 128) + ((uint32_t)(quad * 32) << 16) + (uint32_t)(ci * 32), r);
        tmem_ld_wait();
#pragma unroll
        for (int s2 = 0; s2 < 4; ++s2) {
          uint32_t hi[4], lo[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            // this lane keeps set 2 s2 + csel, the partner set 2 s2 + (1 - csel)
            const float a = __uint_as_float(r[setcol(2 * s2, e)]);
            const float z = __uint_as_float(r[setcol(2 * s2 + 1, e)]);
            const float keep = csel ? z : a, send = csel ? a : z;
            const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
            const float re = csel ? recv : keep, im = csel ? keep : recv;
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(re, im);
            const float2 hf = __bfloat1622float2(h2);
            const __nv_bfloat162 l2 = __floats2bfloat162_rn(re - hf.x, im - hf.y);
            hi[e] = *reinterpret_cast<const uint32_t*>(&h2);
            lo[e] = *reinterpret_cast<const uint32_t*>(&l2);
          }
          const uint32_t off = offs[s2];
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(sh + off), "r"(hi[0]), "r"(hi[1]),
                       "r"(hi[2]), "r"(hi[3])
                       : "memory");
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(sh + 2 * F2_AB_ATOM + off), "r"(lo[0]),
                       "r"(lo[1]), "r"(lo[2]), "r"(lo[3])
                       : "memory");
        }
      }
      fence_proxy_async();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&fold_done[b]);
    }
    // ---- TMEM_B -> this CTA's planes [VH][NBB][128]
    const bool done = ok && mbar_wait_sleep(doneB, 0, abort_flag);
    tc_fence_after();
    const int nchunk = (p.VH * p.NBB + 31) / 32;
    if (done && ci < nchunk) {
      float* plane = p.planes + (int64_t)blockIdx.x * p.VH * p.NBB * 128;
      const int row = quad * 32 + lane;
      for (int c0 = ci * 32; c0 < p.VH * p.NBB; c0 += 4 * 32) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tB + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, r);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (c0 + j < p.VH * p.NBB) plane[(int64_t)(c0 + j) * 128 + row] = n_units > 0 ? __uint_as_float(r[j]) : 0.f;
      }
    } else if (!done && ci < nchunk) {
      // an aborted CTA leaves zeros (the status word reports the abort)
      float* plane = p.planes + (int64_t)blockIdx.x * p.VH * p.NBB * 128;
      const int row = quad * 32 + lane;
      for (int c0 = ci * 32; c0 < p.VH * p.NBB; c0 += 4 * 32)
        for (int j = 0; j < 32 && c0 + j < p.VH * p.NBB; ++j) plane[(int64_t)(c0 + j) * 128 + row] = 0.f;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
  if (f2_grid_barrier(p.sync + 1, p.abort_word, abort_flag) && warp >= 2 && warp <= 17) {
    // ---- phase 2: planes of all CTAs summed into y.  Item = (part, j, 32
    // rows n_B), one per CTA at a time; its 16 warps take planes w, w + 16,
    // ... (compensated FP32, re and im, one batch of loads for up to 160
    // planes), the partials are added in FP64 in warp order.
    const int wq = warp - 2;
    double* part_sum = reinterpret_cast<double*>(stage);
    const int l23 = p.l2 * p.l3, rgs = (p.NBh + 31) / 32;
    const int n_items = p.VH * l23 * rgs;
    const int64_t pstride = (int64_t)p.VH * p.NBB * 128;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
      const int rg = it % rgs, rest = it / rgs;
      const int j = rest % l23, pt = rest / l23;
      const int r = rg * 32 + lane;
      const float* src = p.planes + (int64_t)(pt * p.NBB + 2 * j) * 128 + r;
      Kahan are, aim;
      for (int z0 = wq; z0 < (int)gridDim.x; z0 += 10 * 16) {
        float vr[10], vi[10];
#pragma unroll
        for (int u = 0; u < 10; ++u) {
          const int z = z0 + u * 16;
          vr[u] = z < (int)gridDim.x ? __ldcg(src + z * pstride) : 0.f;
          vi[u] = z < (int)gridDim.x ? __ldcg(src + z * pstride + 128) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 10; ++u) {
          are.add(vr[u]);
          aim.add(vi[u]);
        }
      }
      part_sum[wq * 64 + lane] = are.value();
      part_sum[wq * 64 + 32 + lane] = aim.value();
      asm volatile("bar.sync 2, 512;" ::: "memory");
      if (wq == 0 && r < p.NBh) {
        double vre = part_sum[lane], vim = part_sum[32 + lane];
        for (int q = 1; q < 16; ++q) {
          vre += part_sum[q * 64 + lane];
          vim += part_sum[q * 64 + 32 + lane];
        }
        // n_B = (vec_local, l0, l1, p) of part pt; j = (l2, l3)
        int nn = r;
        const int pi = nn % DD;
        nn /= DD;
        const int l1i = nn % p.l1;
        nn /= p.l1;
        const int l0i = nn % p.l0, vec = pt * (p.nvec / p.VH) + nn / p.l0;
        const int64_t off = (j / p.l3) * p.yl2 + (j % p.l3) * p.yl3 + vec * p.yv + l0i * p.yl0 + l1i * p.yl1 + pi;
        double2 val = make_double2(vre, vim);
        if (p.accumulate) val = cadd(val, p.y[off]);
        p.y[off] = val;
      }
      asm volatile("bar.sync 2, 512;" ::: "memory");
    }
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(p.err, CARC_NOT_CONVERGED);
}

// F2 launch geometry for nvec centers, or VH = 0 when the kernel does not take them
struct F2Geo {
  int VH, NAh, NBh;
};

F2Geo f2_geo(const S3& s, const Geo2& g2, int nvec) {
  F2Geo f{0, 0, 0};
  if (!g2.ok) return f;
  const int64_t NA = (int64_t)nvec * s.k2 * s.k3 * s.d;
  int VH = NA <= 128 ? 1 : 2;
  if (VH == 2 && nvec % 2 != 0) return f;
  const int64_t NAh = NA / VH;
  if (NAh % 16 != 0 || NAh > 128 || NAh < 16) return f;
  f.VH = VH;
  f.NAh = (int)NAh;
  f.NBh = (int)NAh;  // k2 k3 == l0 l1
  return f;
}

int f2_grid(const S3& s, const Geo2& g2, const TermGroups& tg) {
  const int64_t pairs = (g2.MA / F2_XT) * (int64_t)tg.i1.size();
  return (int)std::max<int64_t>(1, std::min<int64_t>(152, pairs));
}

int64_t f2_ws_bytes(const S3& s, const Geo2& g2, const TermGroups& tg, int nvec) {
  const F2Geo f = f2_geo(s, g2, nvec);
  if (!f.VH) return 0;
  int64_t vin = 0;
  for (auto& v : tg.terms) vin += a256((int64_t)f.NAh * f.VH * 64 * (int64_t)v.size() * 2);
  const int64_t planes = (int64_t)f2_grid(s, g2, tg) * f.VH * g2.NBB * 128 * 4;
  return vin + a256(planes) + 256;
}

// Enqueues the cooperative F2 launch; *done tells whether it was accepted (a
// grid that cannot be co-resident is refused before anything runs).
int launch_fused2(const S3& s, int nvec, const TermGroups& tg, const Geo2& g2, const void* plan2, void* ws,
                  const double2* x, double2* y, const void* const* op_ptrs, const int32_t* terms, int accumulate,
                  bool* done, int* status, cudaStream_t stream) {
  *done = false;
  const F2Geo f = f2_geo(s, g2, nvec);
  if (!f.VH) return CARC_OK;
  const int G = (int)tg.i1.size();
  int n_terms_all = 0;
  for (auto& v : tg.terms) n_terms_all += (int)v.size();
  if (n_terms_all > kVinTermsPerLaunch) return CARC_OK;
  F2Maps maps;
  memset(&maps, 0, sizeof(maps));
  F2Params fp;
  memset(&fp, 0, sizeof(fp));
  fp.VH = f.VH;
  fp.NAh = f.NAh;
  fp.NBh = f.NBh;
  fp.NBB = (int)g2.NBB;
  fp.nksA = (int)(g2.Wp / 16);
  fp.L = (int)(s.l0 * s.l1);
  fp.K23 = (int)(s.k2 * s.k3);
  fp.XP = F2_XT / fp.L;
  fp.x_tiles = (int)(g2.MA / F2_XT);
  fp.G = G;
  fp.n_pairs = fp.x_tiles * G;
  fp.kcB4 = 4 * g2.KcB;
  fp.kcB2 = 2 * g2.KcB;
  // workspace: [Vin per group][planes][sync, abort word]
  char* w = static_cast<char*>(ws);
  std::vector<int64_t> vin_off;
  int64_t vin_bytes = 0;
  for (auto& v : tg.terms) {
    vin_off.push_back(vin_bytes);
    vin_bytes += a256((int64_t)f.NAh * f.VH * 64 * (int64_t)v.size() * 2);
  }
  const int grid = f2_grid(s, g2, tg);
  float* planes = reinterpret_cast<float*>(w + vin_bytes);
  char* sync = w + vin_bytes + a256((int64_t)grid * f.VH * g2.NBB * 128 * 4);
  const char* pA = static_cast<const char*>(plan2);
  const int64_t NA = (int64_t)f.NAh * f.VH;
  Vin2 vt;
  memset(&vt, 0, sizeof(vt));
  vt.rows = NA;
  vt.kc = s.k0 * s.k1;
  vt.k23 = s.k2 * s.k3;
  vt.d = s.d;
  vt.wp2 = g2.Wp / 2;
  for (int q = 0; q < G; ++q) {
    const int nt = (int)tg.terms[q].size();
    fp.nterm[q] = nt;
    CARC_RETURN_IF(tma_map_bf16(&maps.a[q], pA, (uint64_t)(64 * nt), (uint64_t)g2.rowsA, 128));
    CARC_RETURN_IF(tma_map_bf16(&maps.vin[q], w + vin_off[q], (uint64_t)(64 * nt), (uint64_t)NA, (uint32_t)f.NAh));
    pA += a256(g2.rowsA * 64 * (int64_t)nt * 2);
    for (int j = 0; j < nt; ++j) {
      const int io = terms[3 * tg.terms[q][j] + 2];
      vt.op[vt.n] = io < 0 ? nullptr : static_cast<const double2*>(op_ptrs[io]);
      vt.dst[vt.n] = vin_off[q] / 4 + (int64_t)j * 32;
      vt.pitch[vt.n] = 32 * (int64_t)nt;
      ++vt.n;
    }
  }
  CARC_RETURN_IF(tma_map_bf16(&maps.b, pA, (uint64_t)(4 * g2.KcB * G), (uint64_t)g2.NBB, (uint32_t)g2.NBB));
  fp.stage_bytes = F2_STAGE_A + f.NAh * 128;
  const int fixed = 1024 + 2 * F2_AB + 8 * (int)g2.NBB * 128 + 256;
  fp.stages = std::min(F2_STAGES, (F2_SMEM_MAX - fixed) / fp.stage_bytes);
  if (fp.stages < 2) return CARC_OK;
  const int smem = fixed + fp.stages * fp.stage_bytes;
  fp.planes = planes;
  fp.err = status;
  fp.vt = vt;
  fp.x = x;
  fp.vin = reinterpret_cast<uint32_t*>(w);
  fp.y = y;
  fp.accumulate = accumulate;
  fp.nvec = nvec;
  fp.l0 = (int)s.l0;
  fp.l1 = (int)s.l1;
  fp.l2 = (int)s.l2;
  fp.l3 = (int)s.l3;
  fp.yl3 = s.d;
  fp.yl2 = s.l3 * fp.yl3;
  fp.yl1 = s.l2 * fp.yl2;
  fp.yl0 = s.l1 * fp.yl1;
  fp.yv = s.l0 * fp.yl0;
  fp.sync = reinterpret_cast<unsigned int*>(sync);
  fp.abort_word = reinterpret_cast<int*>(sync + 8);
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    for (auto k : {stage3_fused2_kernel<1>, stage3_fused2_kernel<2>, stage3_fused2_kernel<4>, stage3_fused2_kernel<8>}) {
      const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, F2_SMEM_MAX);
      if (e != cudaSuccess) attr = e;
    }
  });
  if (attr != cudaSuccess) return fail(CARC_CUDA_ERROR, "fused matvec (compact): %s", cudaGetErrorString(attr));
  CARC_CHECK_CUDA(cudaMemsetAsync(sync, 0, 16, stream));
  PhaseScope ph(PH_TC_STEP_A, stream);
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(F2_THREADS);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = stream;
  cudaLaunchAttribute la[1];
  la[0].id = cudaLaunchAttributeCooperative;
  la[0].val.cooperative = 1;
  cfg.attrs = la;
  cfg.numAttrs = 1;
  cudaError_t e = cudaErrorInvalidValue;
  switch (s.d) {
    case 1: e = cudaLaunchKernelEx(&cfg, stage3_fused2_kernel<1>, maps, fp); break;
    case 2: e = cudaLaunchKernelEx(&cfg, stage3_fused2_kernel<2>, maps, fp); break;
    case 4: e = cudaLaunchKernelEx(&cfg, stage3_fused2_kernel<4>, maps, fp); break;
    case 8: e = cudaLaunchKernelEx(&cfg, stage3_fused2_kernel<8>, maps, fp); break;
  }
  if (e == cudaSuccess) {
    ::carc::count_launch();
    *done = true;
    return CARC_OK;
  }
  (void)cudaGetLastError();  // not co-resident: the caller takes another path
  return CARC_OK;
}

}  // namespace

int64_t stage3_matvec_tc_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const int32_t* terms,
                            int n_terms, int nvec) {
  S3 s;
  if (s3_shapes(s0_shape, s1_shape, d, &s) != CARC_OK) return -1;
  if (n_terms < 1 || nvec < 1) return 0;
  const TermGroups tg = group_terms(terms, n_terms);
  return std::max(mv_layout(s, s0_shape, s1_shape, nvec, tg, nullptr, nullptr),
                  f2_ws_bytes(s, geometry2(s, tg), tg, nvec));
}

namespace {

// step A (one folding GEMM per S2_1 tag, W to HBM) and step B (one split-K GEMM)
int unfused_steps(const S3& s, int nvec, const TermGroups& tg, const Geo& g1, const Geo& g, const void* plan,
                  const MvWs& w, int* status, cudaStream_t stream, int fold_variant) {
  const int G = (int)tg.i1.size();
  const int64_t kpB = g.regB * G;
  const int64_t rows_valid_w = (int64_t)nvec * s.l0 * s.l1 * s.d;
  // only the K padding of the valid rows needs zeros: a padding row of W
  // (rows past nvec l0 l1 d, there to fill the N tile) feeds only its own
  // output column, which the reduction never reads
  const int64_t pad_w = rows_valid_w * G * (g.regB - 4 * g.kcB);
  if (pad_w > 0) {
    clear_w_padding_kernel<<<grid_of(pad_w), 256, 0, stream>>>(reinterpret_cast<__nv_bfloat16*>(w.w_pk), rows_valid_w,
                                                              g.rowsB_b, 4 * g.kcB, g.regB, G);
    CARC_CHECK_LAUNCH();
  }
  // step A per group: W_g = sum_{t in g} S2_0[i0_t] . Vin_t, folded straight into region g of the step-B operand
  const char* planA = static_cast<const char*>(plan);
  {
    PhaseScope ph(PH_TC_STEP_A, stream);
    for (int q = 0; q < G; ++q) {
      const int64_t kpA = g.regA * (int64_t)tg.terms[q].size();
      FoldEpi fe;
      fe.x0 = s.x0;
      fe.x1 = s.x1;
      fe.l0 = s.l0;
      fe.l1 = s.l1;
      fe.nvec = nvec;
      fe.k2 = s.k2;
      fe.k3 = s.k3;
      fe.d = s.d;
      fe.M = g.MA;
      fe.N = g.NA;
      fe.kc = g.kcB;
      fe.col_off = (int64_t)q * g.regB;
      fe.rows = g.rowsB_b;
      fe.dst = w.w_pk;
      CARC_RETURN_IF(gemm_bf16_tn_fold(planA, (int)g1.rowsA_a, w.vin + w.vin_off[q], (int)g.rowsA_b, (int)kpA, fe,
                                       status, stream, fold_variant));
      planA += a256(g1.rowsA_a * kpA * 2);
    }
  }
  // step B: y^T[(l2,l3),(vec,l0,l1,p)] = sum_g S2_1[i1_g] . W_g in one split-K GEMM
  const char* planB = planA;
  {
    PhaseScope ph(PH_TC_STEP_B, stream);
    CARC_RETURN_IF(gemm_bf16_tn(planB, (int)g1.rowsB_a, w.w_pk, (int)g.rowsB_b, (int)kpB, w.pB, g.rowsB_b, w.ksB,
                                status, stream, (int)(4 * s.l2 * s.l3), /*b_blocked=*/1));
  }
  return CARC_OK;
}

// With vt (single-launch mode) the kernel is launched cooperatively and also
// packs Vin and reduces into y; *coop_done tells whether that launch was
// accepted (when not, nothing was enqueued but a memset and the caller runs
// the three-kernel sequence).
int launch_fused(const S3& s, int nvec, const TermGroups& tg, const Geo& g1, const Geo& g, const void* plan,
                 const MvWs& w, const VinTerms* vt, const void* x, void* y, int accumulate, bool* coop_done,
                 int* status, cudaStream_t stream) {
  if (coop_done) *coop_done = false;
  const int G = (int)tg.i1.size();
  FusedMaps maps;
  memset(&maps, 0, sizeof(maps));
  FusedParams fp;
  memset(&fp, 0, sizeof(fp));
  fp.NA = (int)g.NA;
  fp.NB = (int)(nvec * s.l0 * s.l1 * s.d);
  // two vector parts per pair when the halves stay MMA-shaped: TMEM_A is then
  // double-buffered and one part's fold overlaps the next part's MMAs
  fp.VH = (nvec % 2 == 0 && (fp.NA / 2) % 16 == 0 && (fp.NB / 2) % 16 == 0) ? 2 : 1;
  fp.NAh = fp.NA / fp.VH;
  fp.NBh = fp.NB / fp.VH;
  const char* planA = static_cast<const char*>(plan);
  for (int q = 0; q < G; ++q) {
    const int64_t kpA = g.regA * (int64_t)tg.terms[q].size();
    CARC_RETURN_IF(tma_map_bf16(&maps.a[q], planA, (uint64_t)kpA, (uint64_t)g1.rowsA_a, 128));
    CARC_RETURN_IF(tma_map_bf16(&maps.vin[q], w.vin + w.vin_off[q], (uint64_t)kpA, (uint64_t)g.rowsA_b,
                                (uint32_t)fp.NAh));
    fp.nkb[q] = (int)(kpA / 64);
    planA += a256(g1.rowsA_a * kpA * 2);
  }
  const int live_b = (int)(4 * s.l2 * s.l3);
  fp.a_rows = live_b <= 64 ? 64 : 128;
  CARC_RETURN_IF(tma_map_bf16(&maps.b, planA, (uint64_t)(g.regB * G), (uint64_t)g1.rowsB_a, (uint32_t)fp.a_rows));
  fp.L = (int)(s.l0 * s.l1);
  fp.K23 = (int)(s.k2 * s.k3);
  fp.d = (int)s.d;
  fp.XP = 32 / fp.L;
  fp.x_tiles = (int)(s.x0 * s.x1 * s.l0 * s.l1 / 32);
  fp.G = G;
  fp.n_pairs = fp.x_tiles * G;
  fp.nbuf = 2 * fp.NAh <= 256 ? 2 : 1;
  fp.stage_bytes = FU_STAGE_A + fp.NAh * 128;
  fp.stages = std::min(FU_STAGES, (FU_SMEM_MAX - FU_FIXED) / fp.stage_bytes);
  const int smem = FU_FIXED + fp.stages * fp.stage_bytes;
  fp.regB = g.regB;
  fp.kcB = g.kcB;
  fp.live_rows = (int)round_up(4 * s.l2 * s.l3, 32);
  fp.planes = w.pB;
  fp.err = status;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    for (auto k : {stage3_fused_kernel<1>, stage3_fused_kernel<2>, stage3_fused_kernel<4>, stage3_fused_kernel<8>}) {
      const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, FU_SMEM_MAX);
      if (e != cudaSuccess) attr = e;
    }
  });
  if (attr != cudaSuccess) return fail(CARC_CUDA_ERROR, "fused matvec: %s", cudaGetErrorString(attr));
  PhaseScope ph(PH_TC_STEP_A, stream);
  if (vt) {
    if (fp.d != 1 && fp.d != 2 && fp.d != 4 && fp.d != 8) return CARC_OK;
    fp.coop = 1;
    fp.vt = *vt;
    fp.x = static_cast<const double2*>(x);
    fp.vin = reinterpret_cast<uint32_t*>(w.vin);
    fp.y = static_cast<double2*>(y);
    fp.accumulate = accumulate;
    fp.nvec = nvec;
    fp.l0 = (int)s.l0;
    fp.l1 = (int)s.l1;
    fp.l2 = (int)s.l2;
    fp.l3 = (int)s.l3;
    fp.yl3 = s.d;
    fp.yl2 = s.l3 * fp.yl3;
    fp.yl1 = s.l2 * fp.yl2;
    fp.yl0 = s.l1 * fp.yl1;
    fp.yv = s.l0 * fp.yl0;
    fp.sync = reinterpret_cast<unsigned int*>(w.red);  // [arrivals phase 0, arrivals phase 2, abort word]
    CARC_CHECK_CUDA(cudaMemsetAsync(w.red, 0, 16, stream));
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3((unsigned)w.ksB);
    cfg.blockDim = dim3(FU_THREADS);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = stream;
    cudaLaunchAttribute la[1];
    la[0].id = cudaLaunchAttributeCooperative;
    la[0].val.cooperative = 1;
    cfg.attrs = la;
    cfg.numAttrs = 1;
    cudaError_t e = cudaErrorInvalidValue;
    switch (fp.d) {
      case 1: e = cudaLaunchKernelEx(&cfg, stage3_fused_kernel<1>, maps, fp); break;
      case 2: e = cudaLaunchKernelEx(&cfg, stage3_fused_kernel<2>, maps, fp); break;
      case 4: e = cudaLaunchKernelEx(&cfg, stage3_fused_kernel<4>, maps, fp); break;
      case 8: e = cudaLaunchKernelEx(&cfg, stage3_fused_kernel<8>, maps, fp); break;
    }
    if (e == cudaSuccess) {
      ::carc::count_launch();
      *coop_done = true;
      return CARC_OK;
    }
    (void)cudaGetLastError();  // not co-resident here: the caller runs the three kernels
    return CARC_OK;
  }
  switch (fp.d) {
    case 1: stage3_fused_kernel<1><<<w.ksB, FU_THREADS, smem, stream>>>(maps, fp); break;
    case 2: stage3_fused_kernel<2><<<w.ksB, FU_THREADS, smem, stream>>>(maps, fp); break;
    case 4: stage3_fused_kernel<4><<<w.ksB, FU_THREADS, smem, stream>>>(maps, fp); break;
    case 8: stage3_fused_kernel<8><<<w.ksB, FU_THREADS, smem, stream>>>(maps, fp); break;
    default: return fail(CARC_BAD_ARG, "fused matvec: d = %d is not 1, 2, 4 or 8", fp.d);
  }
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace

int stage3_matvec_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* plan, int n0, int n1,
                     const void* const* op_ptrs, int nop, const int32_t* terms, int n_terms, const void* x, void* y,
                     int nvec, int accumulate, void* ws, int64_t ws_bytes, int* status, cudaStream_t stream) {
  S3 s;
  CARC_RETURN_IF(s3_shapes(s0_shape, s1_shape, d, &s));
  const int64_t nl4 = s.l0 * s.l1 * s.l2 * s.l3;
  if (n_terms == 0) {
    if (!accumulate) return fill_launch((int64_t)nvec * nl4 * d, make_double2(0, 0), y, stream);
    return CARC_OK;
  }
  for (int t = 0; t < n_terms; ++t) {
    int i0 = terms[3 * t], i1 = terms[3 * t + 1], io = terms[3 * t + 2];
    if (i0 < 0 || i0 >= n0 || i1 < 0 || i1 >= n1 || io >= nop)
      return fail(CARC_BAD_ARG, "stage3 tc matvec: term %d out of range", t);
  }
  const TermGroups tg = group_terms(terms, n_terms);
  const Geo g1 = geometry(s, 1);
  // the compact-operand fused kernel (autotune entry -2 or none) where it
  // takes the shape; -1 selects the first fused kernel, > 0 the two-kernel path
  {
    const Geo2 g2 = geometry2(s, tg);
    const int tuned = tuned_ksplit(s0_shape, s1_shape, s.d, nvec, (int)tg.i1.size());
    if (g2.ok && (tuned == 0 || tuned == -2) && f2_geo(s, g2, nvec).VH) {
      if (ws_bytes < f2_ws_bytes(s, g2, tg, nvec)) return fail(CARC_BAD_ARG, "stage3 tc matvec: workspace too small");
      bool done = false;
      const char* plan2 = static_cast<const char*>(plan) + plan_bytes_for(g1, tg);
      CARC_RETURN_IF(launch_fused2(s, nvec, tg, g2, plan2, ws, static_cast<const double2*>(x),
                                   static_cast<double2*>(y), op_ptrs, terms, accumulate, &done, status, stream));
      if (done) return CARC_OK;
    }
  }
  if (ws_bytes < mv_layout(s, s0_shape, s1_shape, nvec, tg, nullptr, nullptr))
    return fail(CARC_BAD_ARG, "stage3 tc matvec: workspace too small");
  const Geo g = geometry(s, nvec);
  MvWs w;
  mv_layout(s, s0_shape, s1_shape, nvec, tg, &w, ws);
  const int G = (int)tg.i1.size();
  // Vin of every term, operator applied and packed: up to 64 terms per launch
  std::vector<VinTerms> chunks;
  {
    VinTerms vt;
    memset(&vt, 0, sizeof(vt));
    vt.rows_out = g.rowsA_b;
    vt.rows_valid = g.NA;
    vt.kc = s.k0 * s.k1;
    vt.reg4 = g.regA / 4;
    vt.k23 = s.k2 * s.k3;
    vt.d = s.d;
    if (vt.rows_out * vt.reg4 * kVinTermsPerLaunch >= (1ll << 31))
      return fail(CARC_TOO_LARGE, "tensor-core matvec: Vin operand too large");
    for (int q = 0; q < G; ++q) {
      const int nt = (int)tg.terms[q].size();
      for (int j = 0; j < nt; ++j) {
        const int io = terms[3 * tg.terms[q][j] + 2];
        vt.op[vt.n] = io < 0 ? nullptr : static_cast<const double2*>(op_ptrs[io]);
        vt.dst[vt.n] = w.vin_off[q] / 4 + (int64_t)j * g.regA / 2;
        vt.pitch[vt.n] = g.regA * nt / 2;
        if (++vt.n == kVinTermsPerLaunch) {
          chunks.push_back(vt);
          vt.n = 0;
        }
      }
    }
    if (vt.n > 0) chunks.push_back(vt);
  }
  // the fused kernel as one cooperative launch (pack, step A + B, reduce)
  if (w.fused && chunks.size() == 1) {
    bool done = false;
    CARC_RETURN_IF(launch_fused(s, nvec, tg, g1, g, plan, w, &chunks[0], x, y, accumulate, &done, status, stream));
    if (done) return CARC_OK;
  }
  {
    PhaseScope ph(PH_TC_PACK, stream);
    for (const VinTerms& vt : chunks) {
      const int64_t per_term = vt.rows_out * vt.reg4;
      const dim3 grid((unsigned)std::min<int64_t>((per_term + 255) / 256, 1024), (unsigned)vt.n);
      pack_vin_kernel<<<grid, 256, 0, stream>>>(static_cast<const double2*>(x), reinterpret_cast<uint32_t*>(w.vin),
                                                 vt);
      CARC_CHECK_LAUNCH();
    }
  }
  const int64_t rows_valid_w = (int64_t)nvec * s.l0 * s.l1 * s.d;
  int64_t plane_ld, plane_stride;
  if (w.fused) {
    CARC_RETURN_IF(launch_fused(s, nvec, tg, g1, g, plan, w, nullptr, nullptr, nullptr, 0, nullptr, status, stream));
    plane_ld = rows_valid_w;
    plane_stride = round_up(4 * s.l2 * s.l3, 32) * rows_valid_w;
  } else {
    CARC_RETURN_IF(unfused_steps(s, nvec, tg, g1, g, plan, w, status, stream,
                                 tuned_fold(s0_shape, s1_shape, s.d, nvec, (int)tg.i1.size())));
    plane_ld = g.rowsB_b;
    plane_stride = g.rowsB_a * g.rowsB_b;
  }
  ZOut o;
  memset(&o, 0, sizeof(o));
  o.base = y;
  const int64_t yl3 = s.d, yl2 = s.l3 * yl3, yl1 = s.l2 * yl2, yl0 = s.l1 * yl1, yv = s.l0 * yl0;
  o.nm = 2;
  o.m_ext[0] = s.l2; o.m_str[0] = yl2;
  o.m_ext[1] = s.l3; o.m_str[1] = yl3;
  o.nn = 4;
  o.n_ext[0] = nvec; o.n_str[0] = yv;
  o.n_ext[1] = s.l0; o.n_str[1] = yl0;
  o.n_ext[2] = s.l1; o.n_str[2] = yl1;
  o.n_ext[3] = s.d; o.n_str[3] = 1;
  PhaseScope ph(PH_TC_REDUCE, stream);
  if (w.fused)  // column-major planes [z][n][row]
    return reduce_planes_colmajor(w.pB, round_up(4 * s.l2 * s.l3, 32), plane_stride, w.ksB, o, make_double2(1, 0),
                                  accumulate, stream);
  return reduce_partials2(w.pB, plane_ld, plane_stride, w.ksB, o, make_double2(1, 0), accumulate, w.red,
                          reduce_partials2_workspace(s.l2 * s.l3, rows_valid_w, w.ksB), stream);
}

// ---------------------------------------------------------------------------
// H_eff on the tensor cores
// ---------------------------------------------------------------------------
namespace {

ZView view_s2_0_G(const S3& s, const void* base) {  // rows (l0,l1,k0,k1), k (x0,x1)
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = 4;
  v.r_ext[0] = s.l0; v.r_str[0] = s.s0[4];
  v.r_ext[1] = s.l1; v.r_str[1] = s.s0[5];
  v.r_ext[2] = s.k0; v.r_str[2] = s.s0[2];
  v.r_ext[3] = s.k1; v.r_str[3] = s.s0[3];
  v.nk = 2;
  v.k_ext[0] = s.x0; v.k_str[0] = s.s0[0];
  v.k_ext[1] = s.x1; v.k_str[1] = s.s0[1];
  return v;
}

ZView view_s2_1_G(const S3& s, const void* base) {  // rows (l2,l3,k2,k3), k (x0,x1)
  ZView v;
  memset(&v, 0, sizeof(v));
  v.base = base;
  v.nr = 4;
  v.r_ext[0] = s.l2; v.r_str[0] = s.s1[4];
  v.r_ext[1] = s.l3; v.r_str[1] = s.s1[5];
  v.r_ext[2] = s.k2; v.r_str[2] = s.s1[2];
  v.r_ext[3] = s.k3; v.r_str[3] = s.s1[3];
  v.nk = 2;
  v.k_ext[0] = s.x0; v.k_str[0] = s.s1[1];
  v.k_ext[1] = s.x1; v.k_str[1] = s.s1[0];
  return v;
}

struct FormGeo {
  int64_t M, N, rows_a, rows_b, region, kp_max;
  int max_terms, ks;
};

FormGeo form_geometry(const S3& s, int max_terms) {
  FormGeo f;
  f.M = s.l0 * s.l1 * s.k0 * s.k1;
  f.N = s.l2 * s.l3 * s.k2 * s.k3;
  f.rows_a = round_up(4 * f.M, 128);
  f.rows_b = gemm_pad_n(f.N);
  f.region = round_up(4 * s.x0 * s.x1, 64);
  f.max_terms = max_terms;
  f.kp_max = f.region * max_terms;
  const int64_t tiles = (f.rows_a / 128) * (f.rows_b / bn_for(f.rows_b));
  // the split count is not monotonic in K: size for the largest over all group sizes
  f.ks = 1;
  for (int nt = 1; nt <= max_terms; ++nt) {
    const int64_t kp = f.region * nt;
    f.ks = std::max(f.ks, gemm_effective_ksplit((int)kp, choose_ksplit(tiles, kp)));
  }
  return f;
}

}  // namespace

int64_t stage3_form_matrix_tc_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms) {
  S3 s;
  if (s3_shapes(s0_shape, s1_shape, d, &s) != CARC_OK) return -1;
  if (n_terms < 1) return 0;
  FormGeo f = form_geometry(s, n_terms);
  return a256(f.rows_a * f.kp_max * 2) + a256(f.rows_b * f.kp_max * 2) + a256((int64_t)f.ks * f.rows_a * f.rows_b * 4) +
         (int64_t)n_terms * a256(f.M * f.N * 16);
}

int stage3_form_matrix_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                          int n0, const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop,
                          const int32_t* terms, int n_terms, void* H, int accumulate, void* ws, int64_t ws_bytes,
                          int* status, cudaStream_t stream) {
  S3 s;
  CARC_RETURN_IF(s3_shapes(s0_shape, s1_shape, d, &s));
  const int64_t nrow = s.l0 * s.l1 * s.l2 * s.l3 * d, ncol = s.k0 * s.k1 * s.k2 * s.k3 * d;
  if (n_terms == 0) {
    if (!accumulate) return fill_launch(nrow * ncol, make_double2(0, 0), H, stream);
    return CARC_OK;
  }
  if (ws_bytes < stage3_form_matrix_tc_ws(s0_shape, s1_shape, d, n_terms))
    return fail(CARC_BAD_ARG, "stage3 tc matrix: workspace too small");
  // operator groups
  std::vector<int> group_op;
  std::vector<std::vector<int>> group_terms;
  for (int t = 0; t < n_terms; ++t) {
    int i0 = terms[3 * t], i1 = terms[3 * t + 1], io = terms[3 * t + 2];
    if (i0 < 0 || i0 >= n0 || i1 < 0 || i1 >= n1 || io >= nop)
      return fail(CARC_BAD_ARG, "stage3 tc matrix: term %d out of range", t);
    int key = io < 0 ? -1 : io;
    int g = -1;
    for (size_t q = 0; q < group_op.size(); ++q)
      if (group_op[q] == key) g = (int)q;
    if (g < 0) {
      g = (int)group_op.size();
      group_op.push_back(key);
      group_terms.emplace_back();
    }
    group_terms[g].push_back(t);
  }
  FormGeo f = form_geometry(s, n_terms);
  char* p = static_cast<char*>(ws);
  char* A_op = p;
  char* B_op = A_op + a256(f.rows_a * f.kp_max * 2);
  float* P = reinterpret_cast<float*>(B_op + a256(f.rows_b * f.kp_max * 2));
  char* Gbase = reinterpret_cast<char*>(P) + a256((int64_t)f.ks * f.rows_a * f.rows_b * 4);
  std::vector<const void*> gptr(group_op.size()), gops(group_op.size());
  for (size_t g = 0; g < group_op.size(); ++g) {
    const std::vector<int>& tl = group_terms[g];
    const int64_t kp = f.region * (int64_t)tl.size();
    for (size_t j = 0; j < tl.size(); ++j) {
      const int t = tl[j];
      CARC_RETURN_IF(pack_operand_region(view_s2_0_G(s, s0_ptrs[terms[3 * t]]), 0, A_op, f.rows_a, kp,
                                         (int64_t)j * f.region, f.region, stream));
      CARC_RETURN_IF(pack_operand_region(view_s2_1_G(s, s1_ptrs[terms[3 * t + 1]]), 1, B_op, f.rows_b, kp,
                                         (int64_t)j * f.region, f.region, stream));
    }
    const int64_t tiles = (f.rows_a / 128) * (f.rows_b / bn_for(f.rows_b));
    const int ks = gemm_effective_ksplit((int)kp, choose_ksplit(tiles, kp));
    CARC_RETURN_IF(gemm_bf16_tn(A_op, (int)f.rows_a, B_op, (int)f.rows_b, (int)kp, P, f.rows_b, ks, status, stream));
    void* G = Gbase + (int64_t)g * a256(f.M * f.N * 16);
    // G[(l0,l1,l2,l3),(k0,k1,k2,k3)] from rows (l0,l1,k0,k1) x cols (l2,l3,k2,k3)
    const int64_t gk3 = 1, gk2 = s.k3, gk1 = s.k2 * gk2, gk0 = s.k1 * gk1, gl3 = s.k0 * gk0, gl2 = s.l3 * gl3,
                  gl1 = s.l2 * gl2, gl0 = s.l1 * gl1;
    ZOut o;
    memset(&o, 0, sizeof(o));
    o.base = G;
    o.nm = 4;
    o.m_ext[0] = s.l0; o.m_str[0] = gl0;
    o.m_ext[1] = s.l1; o.m_str[1] = gl1;
    o.m_ext[2] = s.k0; o.m_str[2] = gk0;
    o.m_ext[3] = s.k1; o.m_str[3] = gk1;
    o.nn = 4;
    o.n_ext[0] = s.l2; o.n_str[0] = gl2;
    o.n_ext[1] = s.l3; o.n_str[1] = gl3;
    o.n_ext[2] = s.k2; o.n_str[2] = gk2;
    o.n_ext[3] = s.k3; o.n_str[3] = gk3;
    CARC_RETURN_IF(reduce_partials(P, f.rows_b, f.rows_a * f.rows_b, ks, o, make_double2(1, 0), 0, stream));
    gptr[g] = G;
    gops[g] = group_op[g] < 0 ? nullptr : op_ptrs[group_op[g]];
  }
  return kron_launch(H, gptr.data(), gops.data(), (int)group_op.size(), (int)s.d, s.l0 * s.l1 * s.l2 * s.l3,
                     s.k0 * s.k1 * s.k2 * s.k3, accumulate, stream);
}

}  // namespace carc
