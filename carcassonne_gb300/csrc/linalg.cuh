// Host-side entry points of the FP64 dense linear algebra (linalg.cu, eig.cu).
#pragma once
#include "common.cuh"

namespace carc {
int64_t svd_workspace_size(int m, int n, int batch);
int svd_jacobi(int m, int n, int batch, const void* A, void* U, void* S, void* Vh, void* status, void* ws,
               int64_t ws_bytes, cudaStream_t stream);
int64_t heev_workspace_size(int n, int batch);
int heev_jacobi(int n, int batch, const void* A, void* W, void* V, void* status, void* ws, int64_t ws_bytes,
                cudaStream_t stream);
int64_t potrf_workspace_size(int n);
int potrf(int n, void* A, void* status, void* ws, int64_t ws_bytes, cudaStream_t stream);
int64_t trtri_workspace_size(int n);
int trtri_lower(int n, const void* L, void* X, void* ws, int64_t ws_bytes, cudaStream_t stream);
int64_t hegv_workspace_size(int n, int max_krylov, int flags);
int hegv_lowest(int n, const void* H, const void* N, const void* x0, void* x, double* eigenvalues, int max_krylov,
                int max_restarts, double tol, int flags, int* iterations, void* factors, void* ws, int64_t ws_bytes,
                cudaStream_t stream);
int64_t minres_workspace_size(int n);
int minres_projected(int n, const void* C, const void* u, double shift, const void* b, void* z, int maxit,
                     double rtol, int* iterations, void* ws, int64_t ws_bytes, cudaStream_t stream);
int lanczos_lowest(int n, const void* C, const void* u0, void* u, double* eigenvalues, int max_krylov,
                   int max_restarts, double tol, int* iterations, void* ws, int64_t ws_bytes, cudaStream_t stream);
int64_t lanczos_workspace_size(int n, int max_krylov);
int64_t relax_workspace_size(int n, int k);
int relax_over(int n, const void* H, const void* N, const void* x0, void* x_out, int k, int max_mults, double tol,
               double2* eigenvalue, int* mults_out, double2* values_out, void* ws, int64_t ws_bytes,
               cudaStream_t stream);
int normalize_axis_finish(int n, const void* S, const void* Vh, double thresh, int sqrt_svals, void* out_a,
                          void* out_b, cudaStream_t stream);
int qr_mgs(int m, int n, const void* A, void* Q, void* R, cudaStream_t stream);
}  // namespace carc
