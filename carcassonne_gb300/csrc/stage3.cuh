// Host-side entry points of the FP64 stage-3 operator (stage3.cu).
#pragma once
#include "common.cuh"

namespace carc {
int64_t stage3_matvec_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms, int nvec);
int stage3_matvec(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs, int n0,
                  const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop, const int32_t* terms,
                  int n_terms, const void* x, void* y, int nvec, int accumulate, void* ws, int64_t ws_bytes,
                  cudaStream_t stream);
int64_t stage3_form_ws(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int n_terms);
int stage3_form_matrix(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* const* s0_ptrs,
                       int n0, const void* const* s1_ptrs, int n1, const void* const* op_ptrs, int nop,
                       const int32_t* terms, int n_terms, void* H, int accumulate, void* ws, int64_t ws_bytes,
                       cudaStream_t stream);
// H[(l,p),(k,q)] (+)= sum_g G_g[l,k] O_g[p,q] (ops[g] == NULL: identity)
int kron_launch(void* H, const void* const* groups, const void* const* ops, int n_groups, int d, int64_t nl4,
                int64_t nk4, int accumulate, cudaStream_t stream);
}  // namespace carc
