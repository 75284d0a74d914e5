// extern "C" entry points of libcarcgb300.so (declared in include/carcassonne_gb300.h).
#include "common.cuh"
#include "contract.cuh"
#include "stage3.cuh"
#include "linalg.cuh"
#include "umma_gemm.cuh"
#include "stage3_tc.cuh"

using namespace carc;

namespace carc {
// ---- learned start vector: MLP kernels (csrc/mlp.cu) ------------------------
int mlp_linear_forward(int B, int K, int N, const float* X, const float* W, const float* b, int relu, float* Y,
                       cudaStream_t stream);
int mlp_linear_backward(int B, int K, int N, const float* X, const float* W, const float* Y, const float* dY,
                        int relu, float* dZ, float* dX, float* dW, float* db, cudaStream_t stream);
int mlp_mse(int64_t n, int B, const float* Y, const float* T, float* dY, float* loss, cudaStream_t stream);
int mlp_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps, int step,
             cudaStream_t stream);
int mlp_to_bf16(int64_t n, const float* x, void* y, cudaStream_t stream);
int mlp_linear_bf16(int B, int K, int N, const void* X, const void* W, const float* b, int relu, void* Yb, float* Yf,
                    cudaStream_t stream);
}  // namespace carc

extern "C" {

const char* carc_last_error_string(void) { return last_error(); }

int carc_version(void) { return 100; }

int64_t carc_launch_counter(void) { return (int64_t)launch_count(); }

int carc_host_alloc_mapped(int64_t bytes, void** host_ptr, void** device_ptr) {
  if (!host_ptr || !device_ptr || bytes <= 0) return fail(CARC_BAD_ARG, "carc_host_alloc_mapped: bad argument");
  *host_ptr = nullptr;
  *device_ptr = nullptr;
  void* h = nullptr;
  CARC_CHECK_CUDA(cudaHostAlloc(&h, (size_t)bytes, cudaHostAllocMapped | cudaHostAllocPortable));
  void* d = nullptr;
  const cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
  if (e != cudaSuccess || !d) {
    cudaFreeHost(h);
    return fail(CARC_CUDA_ERROR, "carc_host_alloc_mapped: no device mapping (%s)", cudaGetErrorString(e));
  }
  *host_ptr = h;
  *device_ptr = d;
  return CARC_OK;
}

int carc_host_free(void* host_ptr) {
  if (!host_ptr) return CARC_OK;
  CARC_CHECK_CUDA(cudaFreeHost(host_ptr));
  return CARC_OK;
}

int carc_phase_timing_enable(int32_t on) { return phase_timing_enable(on); }

int carc_phase_timing_read(int32_t phase, double* total_ms, int64_t* count) {
  if (phase < 0 || phase >= PH_COUNT) return fail(CARC_BAD_ARG, "phase timing: phase %d", phase);
  return phase_timing_read(phase, total_ms, count);
}

int carc_zcontract_grouped(const carc_contract_desc* desc, const void* const* a_ptrs, int32_t n_a,
                           const void* const* b_ptrs, int32_t n_b, void* const* c_ptrs, int32_t n_c,
                           const int32_t* entries, int32_t n_entries, double alpha_re, double alpha_im,
                           int32_t accumulate, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!desc || !a_ptrs || !b_ptrs || !c_ptrs || (n_entries > 0 && !entries))
    return fail(CARC_BAD_ARG, "carc_zcontract_grouped: NULL argument");
  return gett_launch(*desc, a_ptrs, n_a, b_ptrs, n_b, c_ptrs, n_c, entries, n_entries, cmk(alpha_re, alpha_im),
                     accumulate, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_zcontract_workspace_size(const carc_contract_desc* desc, int32_t n_c) {
  if (!desc) return -1;
  return gett_workspace_size(*desc, n_c);
}

int carc_zpermute(const void* in, void* out, int32_t ndim, const int64_t* out_shape, const int64_t* in_strides,
                  int32_t conj, void* stream) {
  if ((ndim > 0 && (!out_shape || !in_strides)) || !in || !out) return fail(CARC_BAD_ARG, "carc_zpermute: NULL argument");
  return permute_launch(in, out, ndim, out_shape, in_strides, conj, as_stream(stream));
}

int carc_zaxpby(int64_t n, double a_re, double a_im, const void* x, double b_re, double b_im, const void* y,
                void* out, void* stream) {
  if (!out) return fail(CARC_BAD_ARG, "carc_zaxpby: NULL output");
  return axpby_launch(n, cmk(a_re, a_im), x, cmk(b_re, b_im), y, out, as_stream(stream));
}

int carc_zmul(int64_t n, const void* x, const void* y, void* out, void* stream) {
  if (!x || !y || !out) return fail(CARC_BAD_ARG, "carc_zmul: NULL argument");
  return mul_launch(n, x, y, out, as_stream(stream));
}

int carc_zfill(int64_t n, double re, double im, void* out, void* stream) {
  if (!out) return fail(CARC_BAD_ARG, "carc_zfill: NULL output");
  return fill_launch(n, cmk(re, im), out, as_stream(stream));
}

int carc_zdot(int64_t n, const void* x, const void* y, int32_t conj_x, void* out, void* workspace,
              int64_t workspace_bytes, void* stream) {
  if (!x || !y || !out) return fail(CARC_BAD_ARG, "carc_zdot: NULL argument");
  return dot_launch(n, x, y, conj_x, out, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_zdot_workspace_size(int64_t n) { return dot_workspace_size(n); }

int carc_zhasnan(int64_t n, const void* x, void* flag, void* stream) {
  if (!flag || (n > 0 && !x)) return fail(CARC_BAD_ARG, "carc_zhasnan: NULL argument");
  return hasnan_launch(n, x, flag, as_stream(stream));
}

int carc_stage3_matvec_f64(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                           int32_t n0, const void* const* s1_ptrs, int32_t n1, const void* const* op_ptrs,
                           int32_t nop, const int32_t* terms, int32_t n_terms, const void* x, void* y, int32_t nvec,
                           int32_t accumulate, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!s0_shape || !s1_shape || !s0_ptrs || !s1_ptrs || (nop > 0 && !op_ptrs) || (n_terms > 0 && !terms) || !x || !y)
    return fail(CARC_BAD_ARG, "carc_stage3_matvec_f64: NULL argument");
  return stage3_matvec(s0_shape, s1_shape, d, s0_ptrs, n0, s1_ptrs, n1, op_ptrs, nop, terms, n_terms, x, y, nvec,
                       accumulate, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_stage3_matvec_f64_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                              int32_t n_terms, int32_t nvec) {
  if (!s0_shape || !s1_shape) return -1;
  return stage3_matvec_ws(s0_shape, s1_shape, d, n_terms, nvec);
}

int carc_stage3_form_matrix_f64(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                const void* const* s0_ptrs, int32_t n0, const void* const* s1_ptrs, int32_t n1,
                                const void* const* op_ptrs, int32_t nop, const int32_t* terms, int32_t n_terms,
                                void* H, int32_t accumulate, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!s0_shape || !s1_shape || !s0_ptrs || !s1_ptrs || (nop > 0 && !op_ptrs) || (n_terms > 0 && !terms) || !H)
    return fail(CARC_BAD_ARG, "carc_stage3_form_matrix_f64: NULL argument");
  return stage3_form_matrix(s0_shape, s1_shape, d, s0_ptrs, n0, s1_ptrs, n1, op_ptrs, nop, terms, n_terms, H,
                            accumulate, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_stage3_form_matrix_f64_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                                   int32_t n_terms) {
  if (!s0_shape || !s1_shape) return -1;
  return stage3_form_ws(s0_shape, s1_shape, d, n_terms);
}

int carc_zgesvd_jacobi(int32_t m, int32_t n, int32_t batch, const void* A, void* U, void* S, void* Vh, void* status,
                       void* workspace, int64_t workspace_bytes, void* stream) {
  if (!A || !U || !S || !Vh || !status) return fail(CARC_BAD_ARG, "carc_zgesvd_jacobi: NULL argument");
  return svd_jacobi(m, n, batch, A, U, S, Vh, status, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_zgesvd_jacobi_workspace_size(int32_t m, int32_t n, int32_t batch) {
  return svd_workspace_size(m, n, batch);
}

int carc_normalize_axis_finish(int32_t n, const void* S, const void* Vh, double dont_recip_under, int32_t sqrt_svals,
                               void* out_a, void* out_b, void* stream) {
  if (!S || !Vh || !out_a || !out_b) return fail(CARC_BAD_ARG, "carc_normalize_axis_finish: NULL argument");
  return normalize_axis_finish(n, S, Vh, dont_recip_under, sqrt_svals, out_a, out_b, as_stream(stream));
}

int carc_zgeqr_economic(int32_t m, int32_t n, const void* A, void* Q, void* R, void* stream) {
  if (!A || !Q || !R) return fail(CARC_BAD_ARG, "carc_zgeqr_economic: NULL argument");
  return qr_mgs(m, n, A, Q, R, as_stream(stream));
}

int carc_zheev_jacobi(int32_t n, int32_t batch, const void* A, void* W, void* V, void* status, void* workspace,
                      int64_t workspace_bytes, void* stream) {
  if (!A || !W || !V || !status) return fail(CARC_BAD_ARG, "carc_zheev_jacobi: NULL argument");
  return heev_jacobi(n, batch, A, W, V, status, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_zheev_jacobi_workspace_size(int32_t n, int32_t batch) { return heev_workspace_size(n, batch); }

int carc_zpotrf(int32_t n, void* A, void* status, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!A || !status) return fail(CARC_BAD_ARG, "carc_zpotrf: NULL argument");
  return potrf(n, A, status, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_zpotrf_workspace_size(int32_t n) { return potrf_workspace_size(n); }

int carc_ztrtri_lower(int32_t n, const void* L, void* X, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!L || !X) return fail(CARC_BAD_ARG, "carc_ztrtri_lower: NULL argument");
  return trtri_lower(n, L, X, workspace, workspace_bytes, as_stream(stream));
}

int64_t carc_ztrtri_lower_workspace_size(int32_t n) { return trtri_workspace_size(n); }

int carc_zhegv_lowest(int32_t n, const void* H, const void* N, const void* x0, void* x, double* eigenvalues,
                      int32_t max_krylov, int32_t max_restarts, double tol, int32_t flags, int32_t* iterations,
                      void* factors, void* workspace, int64_t workspace_bytes, void* stream) {
  if (!H || !N || !x) return fail(CARC_BAD_ARG, "carc_zhegv_lowest: NULL argument");
  if (flags & ~(CARC_HEGV_TENSOR_CORE | CARC_HEGV_SINGLE)) return fail(CARC_BAD_ARG, "carc_zhegv_lowest: unknown flags 0x%x", flags);
  int it = 0;
  int st = hegv_lowest(n, H, N, x0, x, eigenvalues, max_krylov, max_restarts, tol, flags, &it, factors, workspace,
                       workspace_bytes, as_stream(stream));
  if (iterations) *iterations = it;
  return st;
}

int64_t carc_zhegv_lowest_workspace_size(int32_t n, int32_t max_krylov, int32_t flags) {
  return hegv_workspace_size(n, max_krylov, flags);
}

int carc_zheev_lowest_lanczos(int32_t n, const void* C, const void* u0, void* u, double* eigenvalues,
                              int32_t max_krylov, int32_t max_restarts, double tol, int32_t* iterations,
                              void* workspace, int64_t workspace_bytes, void* stream) {
  if (!C || !u0 || !u) return fail(CARC_BAD_ARG, "carc_zheev_lowest_lanczos: NULL argument");
  int it = 0;
  int st = lanczos_lowest(n, C, u0, u, eigenvalues, max_krylov, max_restarts, tol, &it, workspace, workspace_bytes,
                          as_stream(stream));
  if (iterations) *iterations = it;
  return st;
}

int carc_zminres_projected(int32_t n, const void* C, const void* u, double shift, const void* b, void* z,
                           int32_t maxit, double rtol, int32_t* iterations, void* workspace, int64_t workspace_bytes,
                           void* stream) {
  if (!C || !u || !b || !z) return fail(CARC_BAD_ARG, "carc_zminres_projected: NULL argument");
  int it = 0;
  int st = minres_projected(n, C, u, shift, b, z, maxit, rtol, &it, workspace, workspace_bytes, as_stream(stream));
  if (iterations) *iterations = it;
  return st;
}

int64_t carc_zminres_projected_workspace_size(int32_t n) { return minres_workspace_size(n); }

int64_t carc_zheev_lowest_lanczos_workspace_size(int32_t n, int32_t max_krylov) {
  return lanczos_workspace_size(n, max_krylov);
}

int carc_relax_over(int32_t n, const void* H, const void* N, const void* x0, void* x, int32_t k, int32_t max_mults,
                    double tol, double* eigenvalue, int32_t* mults, double* values, void* workspace,
                    int64_t workspace_bytes, void* stream) {
  if (!H || !x0 || !x) return fail(CARC_BAD_ARG, "carc_relax_over: NULL argument");
  double2 lam = make_double2(0, 0);
  double2 vals[2] = {make_double2(0, 0), make_double2(0, 0)};
  int m = 0;
  int st = relax_over(n, H, N, x0, x, k, max_mults, tol, &lam, &m, vals, workspace, workspace_bytes, as_stream(stream));
  if (eigenvalue) {
    eigenvalue[0] = lam.x;
    eigenvalue[1] = lam.y;
  }
  if (mults) *mults = m;
  if (values) {
    values[0] = vals[0].x;
    values[1] = vals[0].y;
    values[2] = vals[1].x;
    values[3] = vals[1].y;
  }
  return st;
}

int64_t carc_relax_over_workspace_size(int32_t n, int32_t k) { return relax_workspace_size(n, k); }

int carc_zcontract_tc(const carc_contract_desc* desc, const void* A, const void* B, void* C, double alpha_re,
                      double alpha_im, int32_t accumulate, int32_t ksplit, void* workspace, int64_t workspace_bytes,
                      void* status, void* stream) {
  if (!desc || !A || !B || !C || !status) return fail(CARC_BAD_ARG, "carc_zcontract_tc: NULL argument");
  CARC_RETURN_IF(validate_desc(*desc));
  ZView a = zview_a(*desc, A), b = zview_b(*desc, B);
  ZOut c = zout_c(*desc, C);
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), as_stream(stream)));
  return zgemm_tc(a, b, c, cmk(alpha_re, alpha_im), accumulate, ksplit, workspace, workspace_bytes,
                  static_cast<int*>(status), as_stream(stream));
}

int64_t carc_zcontract_tc_workspace_size(const carc_contract_desc* desc, int32_t ksplit) {
  if (!desc || validate_desc(*desc) != CARC_OK) return -1;
  return zgemm_tc_workspace(zview_a(*desc, nullptr), zview_b(*desc, nullptr), ksplit);
}

int carc_zcontract_tc_grouped(const carc_contract_desc* desc, const void* const* a_ptrs, int32_t n_a,
                              const void* const* b_ptrs, int32_t n_b, void* const* c_ptrs, int32_t n_c,
                              const int32_t* entries, int32_t n_entries, double alpha_re, double alpha_im,
                              int32_t accumulate, void* workspace, int64_t workspace_bytes, void* status,
                              void* stream) {
  if (!desc || !a_ptrs || !b_ptrs || !c_ptrs || !entries || !status)
    return fail(CARC_BAD_ARG, "carc_zcontract_tc_grouped: NULL argument");
  CARC_RETURN_IF(validate_desc(*desc));
  ZView a = zview_a(*desc, nullptr), b = zview_b(*desc, nullptr);
  ZOut c = zout_c(*desc, nullptr);
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), as_stream(stream)));
  return zgemm_tc_grouped(a, b, c, a_ptrs, n_a, b_ptrs, n_b, c_ptrs, n_c, entries, n_entries,
                          cmk(alpha_re, alpha_im), accumulate, workspace, workspace_bytes, static_cast<int*>(status),
                          as_stream(stream));
}

int64_t carc_zcontract_tc_grouped_workspace_size(const carc_contract_desc* desc, int32_t n_a, int32_t n_b,
                                                 int32_t n_entries) {
  if (!desc || validate_desc(*desc) != CARC_OK || n_a < 1 || n_b < 1 || n_entries < 1) return -1;
  return zgemm_tc_grouped_workspace(zview_a(*desc, nullptr), zview_b(*desc, nullptr), n_a, n_b, n_entries);
}

int carc_gemm_bf16_tn(const void* A, int32_t M, const void* B, int32_t N, int32_t K, float* out, int64_t ld_out,
                      int32_t ksplit, void* status, void* stream) {
  if (!A || !B || !out || !status) return fail(CARC_BAD_ARG, "carc_gemm_bf16_tn: NULL argument");
  CARC_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), as_stream(stream)));
  return gemm_bf16_tn(A, M, B, N, K, out, ld_out, ksplit, static_cast<int*>(status), as_stream(stream));
}

int64_t carc_stage3_tc_plan_size(const int64_t* s0_shape, const int64_t* s1_shape, const int32_t* terms,
                                 int32_t n_terms) {
  if (!s0_shape || !s1_shape || (n_terms > 0 && !terms)) return -1;
  return stage3_tc_plan_size(s0_shape, s1_shape, terms, n_terms);
}

int carc_stage3_tc_prepare(const int64_t* s0_shape, const int64_t* s1_shape, const void* const* s0_ptrs, int32_t n0,
                           const void* const* s1_ptrs, int32_t n1, const int32_t* terms, int32_t n_terms, void* plan,
                           int64_t plan_bytes, void* stream) {
  if (!s0_shape || !s1_shape || !s0_ptrs || !s1_ptrs || !plan || (n_terms > 0 && !terms))
    return fail(CARC_BAD_ARG, "carc_stage3_tc_prepare: NULL");
  return stage3_tc_prepare(s0_shape, s1_shape, s0_ptrs, n0, s1_ptrs, n1, terms, n_terms, plan, plan_bytes,
                           as_stream(stream));
}

int carc_stage3_matvec_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* plan, int32_t n0,
                          int32_t n1, const void* const* op_ptrs, int32_t nop, const int32_t* terms, int32_t n_terms,
                          const void* x, void* y, int32_t nvec, int32_t accumulate, void* workspace,
                          int64_t workspace_bytes, void* status, void* stream) {
  if (!s0_shape || !s1_shape || !plan || (nop > 0 && !op_ptrs) || (n_terms > 0 && !terms) || !x || !y || !status)
    return fail(CARC_BAD_ARG, "carc_stage3_matvec_tc: NULL argument");
  return stage3_matvec_tc(s0_shape, s1_shape, d, plan, n0, n1, op_ptrs, nop, terms, n_terms, x, y, nvec, accumulate,
                          workspace, workspace_bytes, static_cast<int*>(status), as_stream(stream));
}

int carc_tc_autotune_set(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int32_t nvec, int32_t groups,
                         int32_t ksplit) {
  if (!s0_shape || !s1_shape) return fail(CARC_BAD_ARG, "carc_tc_autotune_set: NULL shape");
  return tc_autotune_set(s0_shape, s1_shape, d, nvec, groups, ksplit);
}

int carc_tc_autotune_set_fold(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int32_t nvec,
                              int32_t groups, int32_t variant) {
  if (!s0_shape || !s1_shape) return fail(CARC_BAD_ARG, "carc_tc_autotune_set_fold: NULL shape");
  return tc_autotune_set_fold(s0_shape, s1_shape, d, nvec, groups, variant);
}

int carc_tc_autotune_clear(void) { return tc_autotune_clear(); }

int64_t carc_stage3_matvec_tc_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                             const int32_t* terms, int32_t n_terms, int32_t nvec) {
  if (!s0_shape || !s1_shape || (n_terms > 0 && !terms)) return -1;
  return stage3_matvec_tc_ws(s0_shape, s1_shape, d, terms, n_terms, nvec);
}

int carc_stage3_form_matrix_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                               int32_t n0, const void* const* s1_ptrs, int32_t n1, const void* const* op_ptrs,
                               int32_t nop, const int32_t* terms, int32_t n_terms, void* H, int32_t accumulate,
                               void* workspace, int64_t workspace_bytes, void* status, void* stream) {
  if (!s0_shape || !s1_shape || !s0_ptrs || !s1_ptrs || (nop > 0 && !op_ptrs) || (n_terms > 0 && !terms) || !H ||
      !status)
    return fail(CARC_BAD_ARG, "carc_stage3_form_matrix_tc: NULL argument");
  return stage3_form_matrix_tc(s0_shape, s1_shape, d, s0_ptrs, n0, s1_ptrs, n1, op_ptrs, nop, terms, n_terms, H,
                               accumulate, workspace, workspace_bytes, static_cast<int*>(status), as_stream(stream));
}

int64_t carc_stage3_form_matrix_tc_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                                  int32_t n_terms) {
  if (!s0_shape || !s1_shape) return -1;
  return stage3_form_matrix_tc_ws(s0_shape, s1_shape, d, n_terms);
}


int carc_mlp_linear_forward(int32_t B, int32_t K, int32_t N, const float* X, const float* W, const float* b,
                            int32_t relu, float* Y, void* stream) {
  if (!X || !W || !Y) return fail(CARC_BAD_ARG, "carc_mlp_linear_forward: NULL argument");
  return mlp_linear_forward(B, K, N, X, W, b, relu, Y, as_stream(stream));
}

int carc_mlp_linear_backward(int32_t B, int32_t K, int32_t N, const float* X, const float* W, const float* Y,
                             const float* dY, int32_t relu, float* dZ, float* dX, float* dW, float* db, void* stream) {
  if (!X || !W || !Y || !dY || !dW || !db || (relu && !dZ))
    return fail(CARC_BAD_ARG, "carc_mlp_linear_backward: NULL argument");
  return mlp_linear_backward(B, K, N, X, W, Y, dY, relu, dZ, dX, dW, db, as_stream(stream));
}

int carc_mlp_mse(int64_t n, int32_t B, const float* Y, const float* T, float* dY, float* loss, void* stream) {
  if (!Y || !T || !dY || !loss || B < 1) return fail(CARC_BAD_ARG, "carc_mlp_mse: bad argument");
  return mlp_mse(n, B, Y, T, dY, loss, as_stream(stream));
}

int carc_mlp_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                  float eps, int32_t step, void* stream) {
  if (!p || !g || !m || !v) return fail(CARC_BAD_ARG, "carc_mlp_adam: NULL argument");
  return mlp_adam(n, p, g, m, v, lr, beta1, beta2, eps, step, as_stream(stream));
}

int carc_mlp_to_bf16(int64_t n, const float* x, void* y, void* stream) {
  if (!x || !y) return fail(CARC_BAD_ARG, "carc_mlp_to_bf16: NULL argument");
  return mlp_to_bf16(n, x, y, as_stream(stream));
}

int carc_mlp_linear_bf16(int32_t B, int32_t K, int32_t N, const void* X, const void* W, const float* b, int32_t relu,
                         void* Yb, float* Yf, void* stream) {
  if (!X || !W || (!Yb && !Yf)) return fail(CARC_BAD_ARG, "carc_mlp_linear_bf16: bad argument");
  return mlp_linear_bf16(B, K, N, X, W, b, relu, Yb, Yf, as_stream(stream));
}

}  // extern "C"
