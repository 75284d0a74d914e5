// Host-side entry points of the tensor-core stage-3 operator (stage3_tc.cu).
#pragma once
#include "common.cuh"

namespace carc {
int64_t stage3_tc_plan_size(const int64_t* s0_shape, const int64_t* s1_shape, const int32_t* terms, int n_terms);
int stage3_tc_prepare(const int64_t* s0_shape, const int64_t* s1_shape, const void* const* s0_ptrs, int n0,
                      const void* const* s1_ptrs, int n1, const int32_t* terms, int n_terms, void* plan,
                      int64_t plan_bytes, cudaStream_t stream);
int tc_autotune_set(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int nvec, int groups, int ksplit);
int tc_autotune_set_fold(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int nvec, int groups,
                         int variant);
int tc_autotune_clear();
int64_t stage3_matvec_tc_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const int32_t* terms,
                            int n_terms, int nvec);
int stage3_matvec_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* plan, int n0, int n1,
                     const void* const* op_ptrs, int nop, const int32_t* terms, int n_terms, const void* x, void* y,
                     int nvec, int accumulate, void* ws, int64_t ws_bytes, int* status, cudaStream_t stream);
int64_t stage3_form_matrix_tc_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms);
int stage3_form_matrix_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                          int n0, const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop,
                          const int32_t* terms, int n_terms, void* H, int accumulate, void* ws, int64_t ws_bytes,
                          int* status, cudaStream_t stream);
}  // namespace carc
