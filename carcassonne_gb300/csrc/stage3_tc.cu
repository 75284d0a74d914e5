// The stage-3 operator on the tensor cores (split-BF16 operands, FP32
// accumulation in TMEM, FP64 reductions):
//
//  matvec  y[v] = sum_t S2_0[i0_t] (x) S2_1[i1_t] (x) O[io_t] . x[v]
//    terms are grouped by their S2_1 tag g;
//    step A (one tcgen05 GEMM per group, terms concatenated along K):
//      W_g[(x0,x1,l0,l1),(v,k2,k3,p)] = sum_{t in g} sum_{k0,k1} S2_0[i0_t] . Vin_t
//      whose epilogue folds the (hi,lo) and (re,im) rows and writes W_g split
//      straight into region g of step B's packed operand;
//    step B (one split-K tcgen05 GEMM over all groups, concatenated along K):
//      y^T[(l2,l3),(v,l0,l1,p)] = sum_g sum_{x0,x1,k2,k3} S2_1[g] . W_g,
//      split planes summed in FP64 by a two-level coalesced reduction.
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

Geo geometry(const S3& s, int nvec) {
  Geo g;
  g.MA = s.x0 * s.x1 * s.l0 * s.l1;
  g.NA = (int64_t)nvec * s.k2 * s.k3 * s.d;
  g.rowsA_a = round_up(4 * g.MA, 128);
  g.regA = round_up(4 * s.k0 * s.k1, 64);
  g.rowsA_b = round_up(g.NA, 16);
  g.kcB = s.x0 * s.x1 * s.k2 * s.k3;
  g.rowsB_a = round_up(4 * s.l2 * s.l3, 128);
  g.regB = round_up(4 * g.kcB, 64);
  g.rowsB_b = round_up((int64_t)nvec * s.l0 * s.l1 * s.d, 16);
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

// zero the padding of the packed W: rows >= rows_valid, and per region the
// columns [4 kc, reg) (the folding epilogue writes only the valid entries)
__global__ void clear_w_padding_kernel(__nv_bfloat16* __restrict__ W, int64_t rows_valid, int64_t rows_total,
                                       int64_t kc4, int64_t reg, int64_t n_reg) {
  const int64_t kp = reg * n_reg, pad = reg - kc4;
  const int64_t t1 = rows_valid * n_reg * pad, t2 = (rows_total - rows_valid) * kp;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < t1 + t2; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < t1) {
      const int64_t row = t / (n_reg * pad), rem = t % (n_reg * pad);
      W[row * kp + (rem / pad) * reg + kc4 + rem % pad] = __float2bfloat16_rn(0.f);
    } else {
      W[rows_valid * kp + (t - t1)] = __float2bfloat16_rn(0.f);
    }
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

// split-K count that fills the 152 SMs (one CTA each) in a single wave
int choose_ksplit(int64_t tiles, int64_t kp) {
  const int64_t kb = kp / 64;
  int64_t ks = tiles >= 152 ? 1 : 152 / tiles;
  ks = std::max<int64_t>(1, std::min<int64_t>(ks, kb));
  return (int)ks;
}

int bn_for(int64_t n) { return n % 256 == 0 ? 256 : n % 128 == 0 ? 128 : n % 64 == 0 ? 64 : n % 32 == 0 ? 32 : 16; }

// plan layout: [per group g: S2_0 step-A operand, rowsA_a x (regA * |T_g|)] [S2_1 step-B operand, rowsB_a x (regB * G)]
int64_t plan_bytes_for(const Geo& g1, const TermGroups& tg) {
  int64_t b = 0;
  for (auto& v : tg.terms) b += a256(g1.rowsA_a * g1.regA * (int64_t)v.size() * 2);
  b += a256(g1.rowsB_a * g1.regB * (int64_t)tg.i1.size() * 2);
  return b;
}

}  // namespace

int tc_autotune_set(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int nvec, int groups, int ksplit) {
  if (ksplit < 0 || nvec < 1 || groups < 1) return fail(CARC_BAD_ARG, "tc autotune: bad entry");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const TuneKey k = tune_key(s0_shape, s1_shape, d, nvec, groups);
  if (ksplit == 0)
    g_tune.erase(k);
  else
    g_tune[k] = ksplit;
  return CARC_OK;
}

int tc_autotune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return CARC_OK;
}

int64_t stage3_tc_plan_size(const int64_t* s0_shape, const int64_t* s1_shape, const int32_t* terms, int n_terms) {
  S3 s;
  if (s3_shapes(s0_shape, s1_shape, 1, &s) != CARC_OK) return -1;
  if (n_terms < 1) return 256;
  return plan_bytes_for(geometry(s, 1), group_terms(terms, n_terms));
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
  if (plan_bytes < plan_bytes_for(g, tg)) return fail(CARC_BAD_ARG, "stage3 tc: plan too small");
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
  return CARC_OK;
}

namespace {

struct MvWs {
  char* vin;     // packed Vin operands of all groups (step-A B operands)
  char* w_pk;    // packed W of all groups (step-B operand)
  float* pB;     // step-B split planes
  char* red;     // reduction partial sums
  int ksB;
  std::vector<int64_t> vin_off;  // byte offset of each group's Vin operand
};

int64_t mv_layout(const S3& s, const int64_t* s0_shape, const int64_t* s1_shape, int nvec, const TermGroups& tg,
                  MvWs* w, void* base) {
  const Geo g = geometry(s, nvec);
  const int64_t kpB = g.regB * (int64_t)tg.i1.size();
  const int64_t tilesB = (g.rowsB_a / 128) * (g.rowsB_b / bn_for(g.rowsB_b));
  const int tuned = tuned_ksplit(s0_shape, s1_shape, s.d, nvec, (int)tg.i1.size());
  const int ksB = gemm_effective_ksplit((int)kpB, tuned > 0 ? tuned : choose_ksplit(tilesB, kpB));
  std::vector<int64_t> vin_off;
  int64_t vin_bytes = 0;
  for (auto& v : tg.terms) {
    vin_off.push_back(vin_bytes);
    vin_bytes += a256(g.rowsA_b * g.regA * (int64_t)v.size() * 2);
  }
  const int64_t sizes[4] = {vin_bytes, g.rowsB_b * kpB * 2, (int64_t)ksB * g.rowsB_a * g.rowsB_b * 4,
                            reduce_partials2_workspace(s.l2 * s.l3, (int64_t)nvec * s.l0 * s.l1 * s.d, ksB)};
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

__global__ void pack_vin_kernel(const double2* __restrict__ x, uint32_t* __restrict__ out,
                                const __grid_constant__ VinTerms p) {
  const int64_t per_term = p.rows_out * p.reg4;
  const int64_t total = (int64_t)p.n * per_term;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int term = (int)(t / per_term);
    const int64_t rem = t % per_term;
    const int64_t n = rem / p.reg4, slot = rem % p.reg4;
    uint32_t* row = out + p.dst[term] + n * p.pitch[term];
    if (slot >= p.kc) {  // padding columns [4 kc, reg)
      row[2 * slot] = 0u;
      row[2 * slot + 1] = 0u;
      continue;
    }
    uint32_t hi = 0u, lo = 0u;
    if (n < p.rows_valid) {
      const int64_t pp = n % p.d, q = n / p.d;
      const int64_t k23 = q % p.k23, vec = q / p.k23;
      const double2* xv = x + ((vec * p.kc + slot) * p.k23 + k23) * p.d;
      double2 b;
      const double2* O = p.op[term];
      if (O == nullptr) {
        b = xv[pp];
      } else {
        b = make_double2(0.0, 0.0);
        for (int64_t qq = 0; qq < p.d; ++qq) b = cadd(b, cmul(O[pp * p.d + qq], xv[qq]));
      }
      const float fr = (float)b.x, fi = (float)b.y;
      const __nv_bfloat16 hr = __float2bfloat16_rn(fr), hm = __float2bfloat16_rn(fi);
      const __nv_bfloat16 lr = __float2bfloat16_rn(fr - __bfloat162float(hr));
      const __nv_bfloat16 lm = __float2bfloat16_rn(fi - __bfloat162float(hm));
      const __nv_bfloat162 h2 = __halves2bfloat162(hr, hm), l2 = __halves2bfloat162(lr, lm);
      hi = *reinterpret_cast<const uint32_t*>(&h2);
      lo = *reinterpret_cast<const uint32_t*>(&l2);
    }
    row[slot] = hi;
    row[p.kc + slot] = lo;
  }
}

}  // namespace

int64_t stage3_matvec_tc_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const int32_t* terms,
                            int n_terms, int nvec) {
  S3 s;
  if (s3_shapes(s0_shape, s1_shape, d, &s) != CARC_OK) return -1;
  if (n_terms < 1 || nvec < 1) return 0;
  return mv_layout(s, s0_shape, s1_shape, nvec, group_terms(terms, n_terms), nullptr, nullptr);
}

int stage3_matvec_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* plan, int n0, int n1,
                     const void* const* op_ptrs, int nop, const int32_t* terms, int n_terms, const void* x, void* y,
                     int nvec, int accumulate, void* ws, int64_t ws_bytes, int* status, cudaStream_t stream) {
  S3 s;
  CARC_RETURN_IF(s3_shapes(s0_shape, s1_shape, d, &s));
  const int64_t nl4 = s.l0 * s.l1 * s.l2 * s.l3, nk4 = s.k0 * s.k1 * s.k2 * s.k3;
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
  if (ws_bytes < mv_layout(s, s0_shape, s1_shape, nvec, tg, nullptr, nullptr))
    return fail(CARC_BAD_ARG, "stage3 tc matvec: workspace too small");
  const Geo g1 = geometry(s, 1);
  const Geo g = geometry(s, nvec);
  MvWs w;
  mv_layout(s, s0_shape, s1_shape, nvec, tg, &w, ws);
  const int G = (int)tg.i1.size();
  const int64_t kpB = g.regB * G;
  // Vin of every term, operator applied and packed, in launches of up to 64 terms
  {
    PhaseScope ph(PH_TC_PACK, stream);
    VinTerms vt;
    memset(&vt, 0, sizeof(vt));
    vt.rows_out = g.rowsA_b;
    vt.rows_valid = g.NA;
    vt.kc = s.k0 * s.k1;
    vt.reg4 = g.regA / 4;
    vt.k23 = s.k2 * s.k3;
    vt.d = s.d;
    auto flush = [&]() -> int {
      if (vt.n == 0) return CARC_OK;
      pack_vin_kernel<<<grid_of((int64_t)vt.n * vt.rows_out * vt.reg4), 256, 0, stream>>>(
          static_cast<const double2*>(x), reinterpret_cast<uint32_t*>(w.vin), vt);
      CARC_CHECK_LAUNCH();
      vt.n = 0;
      return CARC_OK;
    };
    for (int q = 0; q < G; ++q) {
      const int nt = (int)tg.terms[q].size();
      for (int j = 0; j < nt; ++j) {
        const int io = terms[3 * tg.terms[q][j] + 2];
        vt.op[vt.n] = io < 0 ? nullptr : static_cast<const double2*>(op_ptrs[io]);
        vt.dst[vt.n] = w.vin_off[q] / 4 + (int64_t)j * g.regA / 2;
        vt.pitch[vt.n] = g.regA * nt / 2;
        if (++vt.n == kVinTermsPerLaunch) CARC_RETURN_IF(flush());
      }
    }
    CARC_RETURN_IF(flush());
  }
  const int64_t rows_valid_w = (int64_t)nvec * s.l0 * s.l1 * s.d;
  const int64_t pad_w = rows_valid_w * G * (g.regB - 4 * g.kcB) + (g.rowsB_b - rows_valid_w) * kpB;
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
      fe.pitch = kpB;
      fe.dst = w.w_pk;
      CARC_RETURN_IF(gemm_bf16_tn_fold(planA, (int)g1.rowsA_a, w.vin + w.vin_off[q], (int)g.rowsA_b, (int)kpA, fe,
                                       status, stream));
      planA += a256(g1.rowsA_a * kpA * 2);
    }
  }
  // step B: y^T[(l2,l3),(vec,l0,l1,p)] = sum_g S2_1[i1_g] . W_g in one split-K GEMM
  const char* planB = planA;
  const int64_t planeB = g.rowsB_a * g.rowsB_b;
  {
    PhaseScope ph(PH_TC_STEP_B, stream);
    CARC_RETURN_IF(gemm_bf16_tn(planB, (int)g1.rowsB_a, w.w_pk, (int)g.rowsB_b, (int)kpB, w.pB, g.rowsB_b, w.ksB,
                                status, stream, (int)(4 * s.l2 * s.l3)));
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
  return reduce_partials2(w.pB, g.rowsB_b, planeB, w.ksB, o, make_double2(1, 0), accumulate, w.red,
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
  f.rows_b = round_up(f.N, 16);
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
