// Stage-3 of the center-site operator (FP64 path): the matvec
//   y = sum_t S2_0[i0_t] (x) S2_1[i1_t] (x) O[io_t] . x
// and the explicit matrix H = sum_t G_t (x) O_t, both as a short sequence of
// grouped contractions over the term table.
//
// Index convention (tensors/_2d/dense.py:114-195): S2_0 = (x0,x1,k0,k1,l0,l1),
// S2_1 = (x1,x0,k2,k3,l2,l3); ket axes k contract with the center, bra axes l
// index the result; the x axes of the two halves are glued crosswise.
#include "common.cuh"
#include "contract.cuh"
#include "stage3.cuh"

#include <algorithm>
#include <map>
#include <utility>
#include <vector>

namespace carc {

namespace {

struct Shapes {
  int64_t x0, x1, k0, k1, l0, l1, k2, k3, l2, l3, d;
  int64_t s0[6], s1[6];  // element strides of S2_0 / S2_1
  int64_t nk4, nl4;
};

int make_shapes(const int64_t* a, const int64_t* b, int64_t d, Shapes* s) {
  for (int i = 0; i < 6; ++i)
    if (a[i] < 1 || b[i] < 1) return fail(CARC_BAD_SHAPE, "stage3: non-positive extent in S2 shapes");
  if (a[0] != b[1] || a[1] != b[0])
    return fail(CARC_BAD_SHAPE, "stage3: S2_0 axes (0,1) = (%lld,%lld) do not glue to S2_1 axes (1,0) = (%lld,%lld)",
                (long long)a[0], (long long)a[1], (long long)b[1], (long long)b[0]);
  if (d < 1) return fail(CARC_BAD_SHAPE, "stage3: physical dimension %lld", (long long)d);
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
  s->nk4 = s->k0 * s->k1 * s->k2 * s->k3;
  s->nl4 = s->l0 * s->l1 * s->l2 * s->l3;
  return CARC_OK;
}

inline int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

// Largest split-K scratch the engine may ask for with 1..n_max output slots.
int64_t max_gett_ws(const carc_contract_desc& d, int n_max) {
  int64_t m = 0;
  for (int n = 1; n <= n_max; ++n) m = std::max(m, gett_workspace_size(d, n));
  return m;
}

struct Carver {
  char* base;
  int64_t used = 0, cap;
  Carver(void* p, int64_t c) : base(static_cast<char*>(p)), cap(c) {}
  void* take(int64_t bytes) {
    void* r = base ? base + used : nullptr;
    used += align256(bytes);
    return r;
  }
};

// Layout of one W intermediate: [vec][x0][x1][l0][l1][k2][k3][p]
struct WLayout {
  int64_t p, k3, k2, l1, l0, x1, x0, vec, size;
  explicit WLayout(const Shapes& s, int nvec) {
    p = 1;
    k3 = s.d;
    k2 = s.k3 * k3;
    l1 = s.k2 * k2;
    l0 = s.l1 * l1;
    x1 = s.l0 * l0;
    x0 = s.x1 * x1;
    vec = s.x0 * x0;
    size = vec * nvec;
  }
};

int64_t matvec_ws(const Shapes& s, int n_terms, int nvec, std::vector<int64_t>* parts) {
  WLayout w(s, nvec);
  int64_t vop = nvec * s.nk4 * s.d;
  // step 0: ops (M=d, N=nvec*nk4, K=d) -- never split (K small)
  // step A: M = x0 x1 l0 l1, N = nvec k2 k3 d, K = k0 k1
  carc_contract_desc a = DescBuilder()
                             .m(s.x0, 0, 0)
                             .m(s.x1, 0, 0)
                             .m(s.l0, 0, 0)
                             .m(s.l1, 0, 0)
                             .n(nvec, 0, 0)
                             .n(s.k2, 0, 0)
                             .n(s.k3, 0, 0)
                             .n(s.d, 0, 0)
                             .k(s.k0, 0, 0)
                             .k(s.k1, 0, 0)
                             .d;
  carc_contract_desc b = DescBuilder()
                             .m(nvec, 0, 0)
                             .m(s.l0, 0, 0)
                             .m(s.l1, 0, 0)
                             .m(s.d, 0, 0)
                             .n(s.l2, 0, 0)
                             .n(s.l3, 0, 0)
                             .k(s.x0, 0, 0)
                             .k(s.x1, 0, 0)
                             .k(s.k2, 0, 0)
                             .k(s.k3, 0, 0)
                             .d;
  int64_t ws_a = max_gett_ws(a, n_terms);
  int64_t ws_b = gett_workspace_size(b, 1);
  int64_t sizes[4] = {(int64_t)n_terms * vop * 16, (int64_t)n_terms * w.size * 16, ws_a, ws_b};
  int64_t total = 0;
  for (int i = 0; i < 4; ++i) {
    if (parts) parts->push_back(sizes[i]);
    total += align256(sizes[i]);
  }
  return total;
}

}  // namespace

int64_t stage3_matvec_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms, int nvec) {
  Shapes s;
  if (make_shapes(s0_shape, s1_shape, d, &s) != CARC_OK) return -1;
  if (n_terms < 1 || nvec < 1) return 0;
  return matvec_ws(s, n_terms, nvec, nullptr);
}

int stage3_matvec(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs, int n0,
                  const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop, const int32_t* terms,
                  int n_terms, const void* x, void* y, int nvec, int accumulate, void* ws, int64_t ws_bytes,
                  cudaStream_t stream) {
  Shapes s;
  CARC_RETURN_IF(make_shapes(s0_shape, s1_shape, d, &s));
  if (nvec < 1) return fail(CARC_BAD_ARG, "stage3 matvec: nvec %d", nvec);
  if (n_terms > CARC_MAX_ENTRIES || n0 > CARC_MAX_SLOTS || n1 > CARC_MAX_SLOTS || nop > CARC_MAX_SLOTS)
    return fail(CARC_TOO_LARGE, "stage3 matvec: too many terms or tags");
  const int64_t nout = nvec * s.nl4 * s.d;
  if (n_terms == 0) {
    if (!accumulate) return fill_launch(nout, make_double2(0, 0), y, stream);
    return CARC_OK;
  }
  for (int t = 0; t < n_terms; ++t) {
    int i0 = terms[3 * t], i1 = terms[3 * t + 1], io = terms[3 * t + 2];
    if (i0 < 0 || i0 >= n0 || i1 < 0 || i1 >= n1 || io >= nop)
      return fail(CARC_BAD_ARG, "stage3 matvec: term %d = (%d,%d,%d) out of range", t, i0, i1, io);
  }
  int64_t need = matvec_ws(s, n_terms, nvec, nullptr);
  if (!ws || ws_bytes < need)
    return fail(CARC_BAD_ARG, "stage3 matvec: workspace of %lld bytes needed, %lld given", (long long)need,
                (long long)ws_bytes);
  std::vector<int64_t> parts;
  matvec_ws(s, n_terms, nvec, &parts);
  Carver cv(ws, ws_bytes);
  char* vop_base = static_cast<char*>(cv.take(parts[0]));
  char* w_base = static_cast<char*>(cv.take(parts[1]));
  void* ws_a = cv.take(parts[2]);
  void* ws_b = cv.take(parts[3]);

  const int64_t vop_size = nvec * s.nk4 * s.d;
  WLayout wl(s, nvec);

  // step 0: the distinct operators applied to x  (Join(2,1,3,4) of dense.py:155)
  std::vector<int> op_slot_of(nop, -1);
  std::vector<const void*> op_a;
  std::vector<void*> op_c;
  std::vector<int32_t> op_entries;
  for (int t = 0; t < n_terms; ++t) {
    int io = terms[3 * t + 2];
    if (io >= 0 && op_slot_of[io] < 0) {
      op_slot_of[io] = (int)op_c.size();
      op_a.push_back(op_ptrs[io]);
      op_c.push_back(vop_base + (int64_t)op_c.size() * vop_size * 16);
    }
  }
  if (!op_c.empty()) {
    // Vop[vec][k4][p] = sum_q O[p,q] x[vec][k4][q]
    carc_contract_desc dop = DescBuilder()
                                 .m(s.d, s.d, 1)
                                 .n(nvec, s.nk4 * s.d, s.nk4 * s.d)
                                 .n(s.nk4, s.d, s.d)
                                 .k(s.d, 1, 1)
                                 .d;
    const void* bx[1] = {x};
    for (size_t i = 0; i < op_c.size(); ++i) {
      op_entries.push_back((int32_t)i);
      op_entries.push_back(0);
      op_entries.push_back((int32_t)i);
    }
    CARC_RETURN_IF(gett_launch(dop, op_a.data(), (int)op_a.size(), bx, 1, op_c.data(), (int)op_c.size(),
                               op_entries.data(), (int)op_c.size(), make_double2(1, 0), 0, nullptr, 0, stream));
  }

  // step A: W_g = sum_{t : i1_t = g} S2_0[i0_t] . Vin_t over (k0,k1), one W per S2_1 tag g (the
  // grouped launch accumulates all entries of one output slot), so that step B runs once per tag
  std::vector<const void*> vin;  // slot 0 = x, then the op results
  vin.push_back(x);
  for (void* p : op_c) vin.push_back(p);
  std::vector<int> group_of_i1(n1, -1), group_i1;
  std::vector<void*> w_c;
  std::vector<int32_t> a_entries, b_entries;
  for (int t = 0; t < n_terms; ++t) {
    const int i0 = terms[3 * t], i1 = terms[3 * t + 1], io = terms[3 * t + 2];
    const int vs = io < 0 ? 0 : 1 + op_slot_of[io];
    if (group_of_i1[i1] < 0) {
      group_of_i1[i1] = (int)w_c.size();
      group_i1.push_back(i1);
      w_c.push_back(w_base + (int64_t)w_c.size() * wl.size * 16);
    }
    a_entries.push_back(i0);
    a_entries.push_back(vs);
    a_entries.push_back(group_of_i1[i1]);
  }
  const int64_t vk0 = s.k1 * s.k2 * s.k3 * s.d, vk1 = s.k2 * s.k3 * s.d, vk2 = s.k3 * s.d, vk3 = s.d;
  const int64_t vvec = s.nk4 * s.d;
  carc_contract_desc da = DescBuilder()
                              .m(s.x0, s.s0[0], wl.x0)
                              .m(s.x1, s.s0[1], wl.x1)
                              .m(s.l0, s.s0[4], wl.l0)
                              .m(s.l1, s.s0[5], wl.l1)
                              .n(nvec, vvec, wl.vec)
                              .n(s.k2, vk2, wl.k2)
                              .n(s.k3, vk3, wl.k3)
                              .n(s.d, 1, 1)
                              .k(s.k0, s.s0[2], vk0)
                              .k(s.k1, s.s0[3], vk1)
                              .d;
  CARC_RETURN_IF(gett_launch(da, s0_ptrs, n0, vin.data(), (int)vin.size(), w_c.data(), (int)w_c.size(),
                             a_entries.data(), n_terms, make_double2(1, 0), 0, ws_a, parts[2], stream));

  // step B: y += sum_g W_g . S2_1[g] over (x0,x1,k2,k3)
  for (size_t g = 0; g < w_c.size(); ++g) {
    b_entries.push_back((int32_t)g);
    b_entries.push_back(group_i1[g]);
    b_entries.push_back(0);
  }
  const int64_t yl3 = s.d, yl2 = s.l3 * s.d, yl1 = s.l2 * yl2, yl0 = s.l1 * yl1, yvec = s.l0 * yl0;
  carc_contract_desc db = DescBuilder()
                              .m(nvec, wl.vec, yvec)
                              .m(s.l0, wl.l0, yl0)
                              .m(s.l1, wl.l1, yl1)
                              .m(s.d, 1, 1)
                              .n(s.l2, s.s1[4], yl2)
                              .n(s.l3, s.s1[5], yl3)
                              .k(s.x0, wl.x0, s.s1[1])
                              .k(s.x1, wl.x1, s.s1[0])
                              .k(s.k2, wl.k2, s.s1[2])
                              .k(s.k3, wl.k3, s.s1[3])
                              .d;
  void* yc[1] = {y};
  CARC_RETURN_IF(gett_launch(db, (const void* const*)w_c.data(), (int)w_c.size(), s1_ptrs, n1, yc, 1,
                             b_entries.data(), (int)w_c.size(), make_double2(1, 0), accumulate, ws_b, parts[3],
                             stream));
  return CARC_OK;
}

// ---------------------------------------------------------------------------
// explicit matrix
// ---------------------------------------------------------------------------
namespace {

constexpr int KRON_MAX_GROUPS = 64;
constexpr int KRON_MAX_D = 16;

struct KronParams {
  int n_groups;
  int d;
  int64_t nl4, nk4;
  int accumulate;
  const double2* g[KRON_MAX_GROUPS];
  const double2* op[KRON_MAX_GROUPS];  // NULL = identity
};

// H[(l,p),(k,q)] (+)= sum_o G_o[l,k] O_o[p,q]
__global__ void kron_kernel(double2* __restrict__ H, const __grid_constant__ KronParams p) {
  const int64_t total = p.nl4 * p.nk4;
  const int64_t ncol = p.nk4 * p.d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = i / p.nk4, k = i % p.nk4;
    double2 gv[KRON_MAX_GROUPS];
    for (int o = 0; o < p.n_groups; ++o) gv[o] = p.g[o][i];
    for (int pp = 0; pp < p.d; ++pp) {
      for (int qq = 0; qq < p.d; ++qq) {
        double2 s = make_double2(0.0, 0.0);
        for (int o = 0; o < p.n_groups; ++o) {
          if (p.op[o])
            cfma(s, gv[o], p.op[o][pp * p.d + qq]);
          else if (pp == qq)
            s = cadd(s, gv[o]);
        }
        int64_t off = (l * p.d + pp) * ncol + k * p.d + qq;
        if (p.accumulate) s = cadd(s, H[off]);
        H[off] = s;
      }
    }
  }
}

carc_contract_desc g_desc(const Shapes& s) {
  // G[l0,l1,l2,l3,k0,k1,k2,k3]
  const int64_t gk3 = 1, gk2 = s.k3, gk1 = s.k2 * gk2, gk0 = s.k1 * gk1, gl3 = s.k0 * gk0, gl2 = s.l3 * gl3,
                gl1 = s.l2 * gl2, gl0 = s.l1 * gl1;
  return DescBuilder()
      .m(s.l0, s.s0[4], gl0)
      .m(s.l1, s.s0[5], gl1)
      .m(s.k0, s.s0[2], gk0)
      .m(s.k1, s.s0[3], gk1)
      .n(s.l2, s.s1[4], gl2)
      .n(s.l3, s.s1[5], gl3)
      .n(s.k2, s.s1[2], gk2)
      .n(s.k3, s.s1[3], gk3)
      .k(s.x0, s.s0[0], s.s1[1])
      .k(s.x1, s.s0[1], s.s1[0])
      .d;
}

}  // namespace

int64_t stage3_form_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms) {
  Shapes s;
  if (make_shapes(s0_shape, s1_shape, d, &s) != CARC_OK) return -1;
  if (n_terms < 1) return 0;
  carc_contract_desc gd = g_desc(s);
  return align256((int64_t)n_terms * s.nl4 * s.nk4 * 16) + align256(max_gett_ws(gd, n_terms));
}

int stage3_form_matrix(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                       int n0, const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop,
                       const int32_t* terms, int n_terms, void* H, int accumulate, void* ws, int64_t ws_bytes,
                       cudaStream_t stream) {
  Shapes s;
  CARC_RETURN_IF(make_shapes(s0_shape, s1_shape, d, &s));
  if (d > KRON_MAX_D) return fail(CARC_TOO_LARGE, "stage3 matrix: physical dimension %lld > %d", (long long)d, KRON_MAX_D);
  if (n_terms > CARC_MAX_ENTRIES || n0 > CARC_MAX_SLOTS || n1 > CARC_MAX_SLOTS || nop > CARC_MAX_SLOTS)
    return fail(CARC_TOO_LARGE, "stage3 matrix: too many terms or tags");
  const int64_t nrow = s.nl4 * s.d, ncol = s.nk4 * s.d;
  if (n_terms == 0) {
    if (!accumulate) return fill_launch(nrow * ncol, make_double2(0, 0), H, stream);
    return CARC_OK;
  }
  int64_t need = stage3_form_ws(s0_shape, s1_shape, d, n_terms);
  if (!ws || ws_bytes < need)
    return fail(CARC_BAD_ARG, "stage3 matrix: workspace of %lld bytes needed, %lld given", (long long)need,
                (long long)ws_bytes);
  // group terms by operator (identity = -1)
  std::map<int, int> group_of;
  std::vector<int> group_op;
  std::vector<int32_t> entries;
  for (int t = 0; t < n_terms; ++t) {
    int i0 = terms[3 * t], i1 = terms[3 * t + 1], io = terms[3 * t + 2];
    if (i0 < 0 || i0 >= n0 || i1 < 0 || i1 >= n1 || io >= nop)
      return fail(CARC_BAD_ARG, "stage3 matrix: term %d = (%d,%d,%d) out of range", t, i0, i1, io);
    int key = io < 0 ? -1 : io;
    auto it = group_of.find(key);
    int g;
    if (it == group_of.end()) {
      g = (int)group_op.size();
      group_of[key] = g;
      group_op.push_back(key);
    } else {
      g = it->second;
    }
    entries.push_back(i0);
    entries.push_back(i1);
    entries.push_back(g);
  }
  const int n_groups = (int)group_op.size();
  if (n_groups > KRON_MAX_GROUPS) return fail(CARC_TOO_LARGE, "stage3 matrix: %d operator groups", n_groups);
  Carver cv(ws, ws_bytes);
  const int64_t gsize = s.nl4 * s.nk4;
  char* gbase = static_cast<char*>(cv.take((int64_t)n_terms * gsize * 16));
  carc_contract_desc gd = g_desc(s);
  int64_t gws = max_gett_ws(gd, n_terms);
  void* gw = cv.take(gws);
  std::vector<void*> gptr(n_groups);
  for (int g = 0; g < n_groups; ++g) gptr[g] = gbase + (int64_t)g * gsize * 16;
  CARC_RETURN_IF(gett_launch(gd, s0_ptrs, n0, s1_ptrs, n1, gptr.data(), n_groups, entries.data(), n_terms,
                             make_double2(1, 0), 0, gw, gws, stream));
  std::vector<const void*> gops(n_groups);
  for (int g = 0; g < n_groups; ++g) gops[g] = group_op[g] < 0 ? nullptr : op_ptrs[group_op[g]];
  return kron_launch(H, (const void* const*)gptr.data(), gops.data(), n_groups, (int)s.d, s.nl4, s.nk4, accumulate,
                     stream);
}

int kron_launch(void* H, const void* const* groups, const void* const* ops, int n_groups, int d, int64_t nl4,
                int64_t nk4, int accumulate, cudaStream_t stream) {
  if (n_groups > KRON_MAX_GROUPS || d > KRON_MAX_D) return fail(CARC_TOO_LARGE, "kron: %d groups, d = %d", n_groups, d);
  KronParams kp;
  memset(&kp, 0, sizeof(kp));
  kp.n_groups = n_groups;
  kp.d = d;
  kp.nl4 = nl4;
  kp.nk4 = nk4;
  kp.accumulate = accumulate;
  for (int g = 0; g < n_groups; ++g) {
    kp.g[g] = static_cast<const double2*>(groups[g]);
    kp.op[g] = static_cast<const double2*>(ops[g]);
  }
  const int64_t gsize = nl4 * nk4;
  int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(gsize, 128), 8 * 152));
  kron_kernel<<<blocks, 128, 0, stream>>>(static_cast<double2*>(H), kp);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace carc
