/*
 * carcassonne_gb300 -- C ABI of the GB300 (sm_103a) center-site path.
 *
 * Every entry point takes plain device pointers and sizes, returns an int
 * status (CARC_OK on success), never throws, and enqueues its work on the
 * given cudaStream_t (passed as void*).  Device buffers belong to the caller;
 * the library never frees them.  The message of the last failure on the
 * calling thread is returned by carc_last_error_string().
 *
 * Complex data is complex128 stored as interleaved (re, im) doubles, the
 * layout of numpy/torch complex128 tensors, in C (row-major) order.
 *
 * Each declaration names the reference interface (gcross/Carcassonne, path
 * within that project) whose arithmetic it carries out.
 */
#ifndef CARCASSONNE_GB300_H
#define CARCASSONNE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum carc_status_code {
  CARC_OK = 0,
  CARC_BAD_SHAPE = 1,      /* DimensionMismatchError / UnexpectedTensorRankError (utils.py:13-41) */
  CARC_BAD_ARG = 2,        /* ValueError */
  CARC_CUDA_ERROR = 3,
  CARC_NOT_CONVERGED = 4,  /* iteration budget spent (gmres info != 0 in compression.py:43) */
  CARC_NAN = 5,            /* checkForNaNsIn / assertHasNoNaNs (utils.py:250-253) */
  CARC_NOT_POSDEF = 6,     /* normalization matrix not positive definite */
  CARC_TOO_LARGE = 7,      /* request exceeds a documented fixed limit */
  CARC_RELAX_FAILED = 8    /* RelaxFailed: the Rayleigh value rose (utils.py:871-872) */
};

#define CARC_MAX_SUBDIMS 6   /* index groups per contraction operand side */
#define CARC_MAX_SLOTS 64    /* tags per sparse boundary in one grouped call */
#define CARC_MAX_ENTRIES 512 /* tag pairs in one grouped call */
#define CARC_NOALLOC_SCRATCH_BYTES (16u << 20) /* fixed scratch of carc_stage3_matvec_f64_noalloc */
#define CARC_CG_MAX_N 2048 /* largest system carc_zcg_hpsd takes (x, r, p, G p in shared memory) */
#define CARC_LOBPCG_MAX_M 8 /* block vectors per problem of the batched eigensolver */
#define CARC_LOBPCG_ITEM 256 /* center entries of one problem per work item of the batched eigensolver */

/* Message of the last failing call on this thread ("" if none). */
const char* carc_last_error_string(void);
/* Library version (major*10000 + minor*100 + patch). */
int carc_version(void);
/* Kernels launched by this library so far, over all threads (a monotone
 * counter for instrumentation; no counterpart in the reference). */
int64_t carc_launch_counter(void);
/* Per-phase device timing of the tensor-core stage-3 operator (no counterpart
 * in the reference; instrumentation for benchmarks).  While enabled, each
 * phase's launches are bracketed by a CUDA event pair on the launching stream.
 * Phases: 0 operand packing, 1 step-A GEMMs (folding epilogue; the fused
 * kernel), 2 step-B GEMM, 3 split-K reductions; of carc_zhegv_lowest: 4 the
 * Cholesky factorization, 5 the triangular inverse, 6 the pencil reduction,
 * 7 the Lanczos iteration.  carc_phase_timing_read, called after the
 * stream is synchronized, returns the summed milliseconds and the number of
 * bracketed intervals of one phase and drops its records. */
int carc_phase_timing_enable(int32_t on);
/* Page-locked host memory mapped into the device's address space
 * (cudaHostAllocMapped | cudaHostAllocPortable): *host_ptr for the host,
 * *device_ptr for kernels, which read and write it directly over the
 * host link (NVLink-C2C on Grace parts).  Passing *device_ptr as x or y of a
 * matvec entry point moves the block and the result inside that call, with
 * no separate copy.  Free with carc_host_free.  (No counterpart in the
 * reference; host plumbing for callers that keep their data on the host.) */
int carc_host_alloc_mapped(int64_t bytes, void** host_ptr, void** device_ptr);
int carc_host_free(void* host_ptr);
int carc_phase_timing_read(int32_t phase, double* total_ms, int64_t* count);

/*
 * A strided complex contraction  C[m; n] (+)= alpha * sum_k op(A)[m; k] op(B)[k; n]
 * where m, n and k are multi-indices (outermost first) with arbitrary
 * element strides into A, B and C.  nm/nn/nk may be 0 (then that extent is 1).
 * conj_a / conj_b conjugate the operand on load.
 */
typedef struct carc_contract_desc {
  int32_t nm, nn, nk;
  int32_t conj_a, conj_b;
  int64_t m_ext[CARC_MAX_SUBDIMS];
  int64_t n_ext[CARC_MAX_SUBDIMS];
  int64_t k_ext[CARC_MAX_SUBDIMS];
  int64_t a_m[CARC_MAX_SUBDIMS];
  int64_t a_k[CARC_MAX_SUBDIMS];
  int64_t b_n[CARC_MAX_SUBDIMS];
  int64_t b_k[CARC_MAX_SUBDIMS];
  int64_t c_m[CARC_MAX_SUBDIMS];
  int64_t c_n[CARC_MAX_SUBDIMS];
} carc_contract_desc;

/*
 * Grouped contraction over a tag-pair table: for every output slot c,
 * C[c] = alpha * sum over entries e with entries[3e+2]==c, in table order, of
 * A[entries[3e]] . B[entries[3e+1]]   (+ the old C[c] when accumulate != 0).
 * a_ptrs/b_ptrs/c_ptrs and entries are HOST arrays (device pointers inside).
 * Replaces: sparse.contractSparseTensors (sparse.py:223-240) driving the dense
 * contractors, and NDArrayData.contractWith (data/__init__.py:157-159).
 * workspace: device scratch of carc_zcontract_workspace_size() bytes (may be
 * NULL when that size is 0).
 */
int carc_zcontract_grouped(const carc_contract_desc* desc,
                           const void* const* a_ptrs, int32_t n_a,
                           const void* const* b_ptrs, int32_t n_b,
                           void* const* c_ptrs, int32_t n_c,
                           const int32_t* entries, int32_t n_entries,
                           double alpha_re, double alpha_im, int32_t accumulate,
                           void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zcontract_workspace_size(const carc_contract_desc* desc, int32_t n_c);

/*
 * out = permutation/reshape of in: out is C-contiguous with shape out_shape;
 * element out[i0..i_{n-1}] = in[sum_j i_j * in_strides[j]] (conjugated if conj).
 * Replaces NDArrayData.join / transpose / conj (data/__init__.py:247-256, :151-153).
 */
int carc_zpermute(const void* in, void* out, int32_t ndim, const int64_t* out_shape,
                  const int64_t* in_strides, int32_t conj, void* stream);

/* out = a*x + b*y over n complex elements (x or y may be NULL when its
 * coefficient is 0).  Replaces NDArrayData.__add__/__sub__/__iadd__/__mul__(scalar)
 * (data/__init__.py:91-140). */
int carc_zaxpby(int64_t n, double a_re, double a_im, const void* x,
                double b_re, double b_im, const void* y, void* out, void* stream);
/* out = x * y (elementwise).  Replaces NDArrayData.__mul__/__imul__ with data. */
int carc_zmul(int64_t n, const void* x, const void* y, void* out, void* stream);
/* out[i] = value. */
int carc_zfill(int64_t n, double re, double im, void* out, void* stream);
/* out (device complex128 scalar) = sum_i op(x_i) y_i, op = conj if conj_x.
 * Warp-shuffle tree reduction in a fixed order (deterministic).
 * Replaces contractWith over all axes (system/_2d.py:429-430) and norm(). */
int carc_zdot(int64_t n, const void* x, const void* y, int32_t conj_x, void* out,
              void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zdot_workspace_size(int64_t n);
/* *flag (device int32) = 1 if any element of x is NaN, else 0.  Replaces hasNaN
 * (data/__init__.py:209-211). */
int carc_zhasnan(int64_t n, const void* x, void* flag, void* stream);

/*
 * Stage-3 operator application (the center-site matvec) in FP64:
 *   y[v] = sum_t S2_0[i0_t] (x) S2_1[i1_t] (x) O[io_t] . x[v]     (+ y if accumulate)
 * S2_0 tags have shape s0_shape = (x0,x1,k0,k1,l0,l1), S2_1 tags have
 * s1_shape = (x1,x0,k2,k3,l2,l3); the operator tags are (d,d); io_t < 0 means
 * the identity (formNormalizationStage3).  x and y hold nvec centers of shape
 * (k0,k1,k2,k3,d) / (l0,l1,l2,l3,d), contiguous one after the other.
 * terms: HOST int32 [n_terms][3] = (i0, i1, io).
 * Replaces formDenseStage3 multiply (tensors/_2d/dense.py:145-174),
 * formNormalizationStage3 multiply (:114-144) and the term sum of
 * formExpectationStage3 (tensors/_2d/sparse.py:129-133).
 */
int carc_stage3_matvec_f64(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                           const void* const* s0_ptrs, int32_t n0,
                           const void* const* s1_ptrs, int32_t n1,
                           const void* const* op_ptrs, int32_t nop,
                           const int32_t* terms, int32_t n_terms,
                           const void* x, void* y, int32_t nvec, int32_t accumulate,
                           void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_stage3_matvec_f64_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape,
                                              int64_t d, int32_t n_terms, int32_t nvec);

/*
 * The strided complex contraction of carc_contract_desc (one pair, no
 * grouping) on the tensor cores: operands split into BF16 hi+lo parts
 * (~16 significant bits), one BF16 tcgen05 GEMM with FP32 accumulation in
 * TMEM (TMA-fed, 128-byte swizzled shared memory), partial products summed
 * in FP64.  Relative error ~1e-5 of the operands' scale.  ksplit splits K
 * across CTAs.  *status (device int32) is nonzero if a pipeline wait timed out.
 * Replaces NDArrayData.contractWith (data/__init__.py:157-159) where the
 * caller accepts split-BF16 accuracy.
 */
int carc_zcontract_tc(const carc_contract_desc* desc, const void* A, const void* B, void* C,
                      double alpha_re, double alpha_im, int32_t accumulate, int32_t ksplit,
                      void* workspace, int64_t workspace_bytes, void* status, void* stream);
int64_t carc_zcontract_tc_workspace_size(const carc_contract_desc* desc, int32_t ksplit);
/*
 * The grouped form of carc_zcontract_tc, with the arguments of
 * carc_zcontract_grouped: C[c] = alpha * sum over entries (i, j, c), in table
 * order, of A[i] . B[j] (+ the old C[c] when accumulate != 0), every pair of
 * one shape on the tensor cores in four launches for the whole table (each
 * distinct operand packed once into a stacked split-BF16 buffer, one grouped
 * GEMM over (entry, tile, split) work items, one grouped reduction).  HOST
 * pointer and entry arrays; at most CARC_MAX_SLOTS operands of each role and
 * CARC_MAX_ENTRIES entries.  *status (device int32) = CARC_NOT_CONVERGED if a
 * pipeline wait timed out.  Replaces the tag-pair loop of
 * contractSparseTensors (sparse.py:223-240) in the absorptions.
 */
int carc_zcontract_tc_grouped(const carc_contract_desc* desc, const void* const* a_ptrs, int32_t n_a,
                              const void* const* b_ptrs, int32_t n_b, void* const* c_ptrs, int32_t n_c,
                              const int32_t* entries, int32_t n_entries, double alpha_re, double alpha_im,
                              int32_t accumulate, void* workspace, int64_t workspace_bytes, void* status,
                              void* stream);
int64_t carc_zcontract_tc_grouped_workspace_size(const carc_contract_desc* desc, int32_t n_a, int32_t n_b,
                                                 int32_t n_entries);
/* The raw tensor-core GEMM: out[z][m][n] = sum over K-split z of A[m,:].B[n,:]
 * (BF16, K-major, M % 128 == 0, K % 64 == 0, N % 16 == 0, FP32 out with row
 * pitch ld_out, ksplit partial planes of M*ld_out floats). */
int carc_gemm_bf16_tn(const void* A, int32_t M, const void* B, int32_t N, int32_t K, float* out,
                      int64_t ld_out, int32_t ksplit, void* status, void* stream);

/*
 * The stage-3 operator on the tensor cores (split-BF16 operands, FP32
 * accumulation in TMEM, FP64 reductions; relative error ~1e-5).
 * carc_stage3_tc_prepare packs the S2 tags of a term table once into a
 * caller-provided plan buffer of carc_stage3_tc_plan_size bytes (the many
 * matvecs of a solve reuse it; the plan is valid for that term table only);
 * carc_stage3_matvec_tc then applies the operator exactly as
 * carc_stage3_matvec_f64 does (same terms, x, y layout), and
 * carc_stage3_form_matrix_tc forms H as carc_stage3_form_matrix_f64 does.
 * *status (device int32) is nonzero if a pipeline wait timed out.
 * Replaces formDenseStage3 / formNormalizationStage3 multiply and formMatrix
 * (tensors/_2d/dense.py:114-203) where split-BF16 accuracy is accepted.
 */
int64_t carc_stage3_tc_plan_size(const int64_t* s0_shape, const int64_t* s1_shape, const int32_t* terms,
                                 int32_t n_terms);
int carc_stage3_tc_prepare(const int64_t* s0_shape, const int64_t* s1_shape,
                           const void* const* s0_ptrs, int32_t n0, const void* const* s1_ptrs, int32_t n1,
                           const int32_t* terms, int32_t n_terms, void* plan, int64_t plan_bytes, void* stream);
int carc_stage3_matvec_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, const void* plan,
                          int32_t n0, int32_t n1, const void* const* op_ptrs, int32_t nop,
                          const int32_t* terms, int32_t n_terms, const void* x, void* y, int32_t nvec,
                          int32_t accumulate, void* workspace, int64_t workspace_bytes, void* status, void* stream);
/* Autotune cache of the tensor-core matvec (no counterpart in the reference):
 * the kernel choice for one problem shape (S2 shapes, d, block size, number
 * of S2_1 tags carrying terms): > 0 the two-kernel path with that step-B
 * split-K count, -1 the fused kernel on the first (re/im x hi/lo row)
 * operand layout, -2 the fused kernel on compact operands; 0 removes the
 * entry (the compact fused kernel where it takes the shape, else the first
 * fused kernel, else the two-kernel path with the one-wave heuristic).
 * Query workspace sizes after setting an entry. */
int carc_tc_autotune_set(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int32_t nvec, int32_t groups,
                         int32_t ksplit);
/* The folding-GEMM configuration of step A on the two-kernel path for one
 * shape: 0 (default) one CTA per SM with 16 fold warps, stages and N tiles
 * as the shape allows; 1 two CTAs per SM, each with 8 fold warps, 2 stages
 * and 128-column N tiles (used where step A's padded N is a multiple of 128).
 * Cleared with the rest of the cache by carc_tc_autotune_clear. */
int carc_tc_autotune_set_fold(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d, int32_t nvec,
                              int32_t groups, int32_t variant);
int carc_tc_autotune_clear(void);
int64_t carc_stage3_matvec_tc_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                             const int32_t* terms, int32_t n_terms, int32_t nvec);
int carc_stage3_form_matrix_tc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                               const void* const* s0_ptrs, int32_t n0, const void* const* s1_ptrs, int32_t n1,
                               const void* const* op_ptrs, int32_t nop, const int32_t* terms, int32_t n_terms,
                               void* H, int32_t accumulate, void* workspace, int64_t workspace_bytes,
                               void* status, void* stream);
int64_t carc_stage3_form_matrix_tc_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                                  int32_t n_terms);

/*
 * carc_stage3_matvec_f64 for callers that cannot allocate device memory while
 * they run (a host application that owns the whole GPU and forbids library
 * allocations, or a loop that cannot afford the synchronisation cudaMalloc
 * may cause) and cannot size a workspace in advance.  It allocates nothing:
 * its scratch is a fixed CARC_NOALLOC_SCRATCH_BYTES (16 MiB) device array
 * inside this library, held on every GPU that loads the library until the
 * process exits.  Problems needing more scratch than that (see
 * carc_stage3_matvec_f64_workspace_size) are rejected with CARC_TOO_LARGE.
 * The array's address is looked up on the first call made on each device
 * (with that device current); make that first call before any stream
 * capture.  The address is cached for the life of the process: after
 * cudaDeviceReset, or anything else that destroys the device's primary
 * context, it is stale, and the library must be unloaded and loaded again
 * before the next call.  All calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller.  No counterpart in the
 * reference (which never manages device memory).
 */
int carc_stage3_matvec_f64_noalloc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                   const void* const* s0_ptrs, int32_t n0,
                                   const void* const* s1_ptrs, int32_t n1,
                                   const void* const* op_ptrs, int32_t nop,
                                   const int32_t* terms, int32_t n_terms,
                                   const void* x, void* y, int32_t nvec, int32_t accumulate, void* stream);

/*
 * Dense stage-3 matrix H[(l,p),(k,q)] = sum_t G_t[l,k] O_t[p,q] with
 * G_t = sum_x S2_0[i0_t] S2_1[i1_t] (formDenseStage3_formMatrix,
 * tensors/_2d/dense.py:175-195; formNormalizationSubmatrix :204-225 when d=1
 * and all io_t < 0; formExpectationMatrix tensors/_2d/sparse.py:144-148).
 * H is (N,N) row-major, N = l0*l1*l2*l3*d, overwritten (or accumulated).
 */
int carc_stage3_form_matrix_f64(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                const void* const* s0_ptrs, int32_t n0,
                                const void* const* s1_ptrs, int32_t n1,
                                const void* const* op_ptrs, int32_t nop,
                                const int32_t* terms, int32_t n_terms,
                                void* H, int32_t accumulate,
                                void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_stage3_form_matrix_f64_workspace_size(const int64_t* s0_shape, const int64_t* s1_shape,
                                                   int64_t d, int32_t n_terms);

/*
 * Batched one-sided Jacobi SVD, FP64 complex: A (batch x m x n, m >= n,
 * row-major) = U diag(S) Vh with U (m x n), S (n, descending), Vh (n x n).
 * *status (device int32) = CARC_NOT_CONVERGED if a sweep budget ran out.
 * Replaces NDArrayData.svd (data/__init__.py:344-346, scipy.linalg.svd).
 */
int carc_zgesvd_jacobi(int32_t m, int32_t n, int32_t batch, const void* A, void* U, void* S, void* Vh,
                       void* status, void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zgesvd_jacobi_workspace_size(int32_t m, int32_t n, int32_t batch);

/*
 * The normalizer / denormalizer of NDArrayData.normalizeAxis
 * (data/__init__.py:282-301) from S (n) and Vh (n x n):
 *   sqrt_svals == 0: out_a = Vh^T (Vh * SI)^*,  out_b = Vh^H (Vh * S)
 *   sqrt_svals != 0: out_a = (Vh * sqrt(SI))^*, out_b = Vh * sqrt(S)
 * with SI = 1/S where |S| > dont_recip_under (always when it is <= 0).
 */
int carc_normalize_axis_finish(int32_t n, const void* S, const void* Vh, double dont_recip_under,
                               int32_t sqrt_svals, void* out_a, void* out_b, void* stream);

/* Economic QR A = Q R of a small m x n matrix (m >= n), row-major: modified
 * Gram-Schmidt with reorthogonalisation, R with a non-negative real diagonal.
 * Replaces NDArrayData.qr(mode='economic') (data/__init__.py:314-317) as used
 * by newEnlargener (:43-50). */
int carc_zgeqr_economic(int32_t m, int32_t n, const void* A, void* Q, void* R, void* stream);

/*
 * Batched Hermitian eigensolver (parallel cyclic Jacobi), n <= 512:
 * A = V diag(W) V^H, W ascending.  Replaces scipy.linalg.eigh in
 * computeCompressor (utils.py:268-302).
 */
int carc_zheev_jacobi(int32_t n, int32_t batch, const void* A, void* W, void* V, void* status,
                      void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zheev_jacobi_workspace_size(int32_t n, int32_t batch);

/* In-place blocked Cholesky A = L L^H (lower; strict upper zeroed);
 * *status = CARC_NOT_POSDEF when a pivot is not positive.  Replaces the LU
 * factorisation of the normalization matrix in relaxOver (utils.py:816-817). */
int carc_zpotrf(int32_t n, void* A, void* status, void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zpotrf_workspace_size(int32_t n);
/* X = L^{-1} for lower-triangular L (blocked forward substitution). */
int carc_ztrtri_lower(int32_t n, const void* L, void* X, void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_ztrtri_lower_workspace_size(int32_t n);

/*
 * Lowest eigenpair of H x = l N x (H Hermitian, N Hermitian positive
 * definite, both n x n): Cholesky of N, C = L^-1 H L^-H, restarted Lanczos
 * with full reorthogonalisation from u0 = L^H x0 (x0 may be NULL), stopping
 * when |beta_m s_m| <= tol |l|; x is N-normalized (x^H N x = 1).
 * eigenvalues (HOST, 2 doubles, may be NULL): [0] the lowest eigenvalue,
 * [1] the second-lowest Ritz value of the last Lanczos tridiagonal to about
 * 1e-6 relative (an estimate of the spectral gap; NaN after one step).
 * *iterations is a HOST pointer.  factors (device, may be NULL; 2 n^2 + n
 * complex128) receives [C | L^-1 | u], u the unit Lanczos eigenvector of C
 * (x = L^-H u / |..|): what a caller needs to solve correction equations
 * against the same reduced pencil.  The call synchronizes the
 * stream at its convergence checkpoints.  Replaces
 * minimizeExpectationUsingFullEigensolver (system/_2d.py:498-502) and the
 * solve of minimizeExpectation (:489-497).
 * flags: CARC_HEGV_TENSOR_CORE forms C = L^-1 H L^-H with the split-BF16
 * tensor-core GEMM (about 1e-5 relative) instead of FP64 -- for pencils that
 * are themselves tensor-core approximations (the mixed-precision solve).
 * CARC_HEGV_SINGLE also factors N and inverts L in complex64 and runs the
 * Lanczos iteration in complex64 (FP64 cross-block sums, alpha, beta and
 * tridiagonal); its residual test is clamped to tol >= 2e-6.  For the
 * same tensor-core pencils, whose energy the caller takes as the Rayleigh
 * quotient of exact H x and N x.
 */
#define CARC_HEGV_TENSOR_CORE 1
#define CARC_HEGV_SINGLE 2
int carc_zhegv_lowest(int32_t n, const void* H, const void* N, const void* x0, void* x, double* eigenvalues,
                      int32_t max_krylov, int32_t max_restarts, double tol, int32_t flags, int32_t* iterations,
                      void* factors, void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zhegv_lowest_workspace_size(int32_t n, int32_t max_krylov, int32_t flags);
/* The Lanczos part alone, for a dense Hermitian C (eigenvalues as above). */
int carc_zheev_lowest_lanczos(int32_t n, const void* C, const void* u0, void* u, double* eigenvalues,
                              int32_t max_krylov, int32_t max_restarts, double tol, int32_t* iterations,
                              void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zheev_lowest_lanczos_workspace_size(int32_t n, int32_t max_krylov);
/* MINRES for P (C - shift) P z = P b with P = I - u u^H (u unit, C dense
 * Hermitian n x n): the correction equation of a Newton step against the
 * reduced tensor-core pencil in the mixed-precision center solve (no
 * counterpart in the reference, whose solves are FP64 throughout).  Stops at
 * |residual| <= rtol |P b| or after maxit iterations; *iterations (HOST). */
int carc_zminres_projected(int32_t n, const void* C, const void* u, double shift, const void* b, void* z,
                           int32_t maxit, double rtol, int32_t* iterations, void* workspace, int64_t workspace_bytes,
                           void* stream);
int64_t carc_zminres_projected_workspace_size(int32_t n);

/*
 * Conjugate gradients on a Hermitian positive semi-definite G x = c (n x n
 * row-major complex128, n <= CARC_CG_MAX_N) from x = 0, the whole iteration
 * in one thread block with no host round trip: stops when
 * |r| <= tol |c|, when p^H G p <= 0, or after max_iter iterations.  status
 * (device int32[2]) receives the iteration count and 1 if the iteration
 * stopped by one of the first two tests (0: out of iterations); residual
 * (device double[1]) the final |r| / |c|.  Replaces the
 * GMRES solve of the normal equations in computeProductCompressor
 * (compression.py:38-43), whose non-convergence is its assert info == 0.
 */
int carc_zcg_hpsd(int32_t n, const void* G, const void* c, void* x, double tol, int32_t max_iter, void* status,
                  void* residual, void* stream);
/* The same iteration over a cooperative grid (rows of G spread over up to one
 * CTA per SM, three bounded grid barriers per iteration, per-CTA partial sums
 * added in CTA order: deterministic), for the FP64 rate of the whole GPU
 * rather than one SM.  It also keeps the iterate with the smallest residual
 * and stops once the residual is 1e8 above it (a c with a part outside the
 * range of a singular G makes the iterates grow without bound); x receives
 * that iterate and residual its true |c - G x| / |c| (one more pass over G).
 * status[0] = -1 and status[1] = 0 if a grid barrier timed out.  workspace:
 * device scratch of carc_zcg_hpsd_grid_workspace_size(n) bytes. */
int carc_zcg_hpsd_grid(int32_t n, const void* G, const void* c, void* x, double tol, int32_t max_iter, void* status,
                       void* residual, void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_zcg_hpsd_grid_workspace_size(int32_t n);

/*
 * relaxOver (utils.py:805-878): restarted Krylov / Rayleigh-Ritz on
 * M = N^{-1} H (N may be NULL for the standard problem) with dimension k
 * (1..8), stopping when the lowest Ritz value moves by <= tol, the space is
 * complete, or max_mults multiplications were spent (<= 0: no budget).
 * x0/x are device vectors of n; *eigenvalue (the last Ritz value),
 * *mults and values[2] = (initial, final Rayleigh values) are HOST outputs.
 * Returns CARC_RELAX_FAILED where the reference raises RelaxFailed.
 */
int carc_relax_over(int32_t n, const void* H, const void* N, const void* x0, void* x, int32_t k,
                    int32_t max_mults, double tol, double* eigenvalue, int32_t* mults, double* values,
                    void* workspace, int64_t workspace_bytes, void* stream);
int64_t carc_relax_over_workspace_size(int32_t n, int32_t k);

/*
 * Learned start vector (no counterpart in the reference, whose start is the
 * previous center, system/_2d.py:435-439 and :491-492): a fully connected
 * network from boundary features to the center, trained and run by these
 * kernels.  FP32 training, BF16 inference with FP32 accumulation.  Layouts:
 * activations row-major (batch, features); weights (out, in) row-major; a
 * layer computes Y = X W^T + b (ReLU when relu != 0).  All pointers device.
 */
int carc_mlp_linear_forward(int32_t B, int32_t K, int32_t N, const float* X, const float* W, const float* b,
                            int32_t relu, float* Y, void* stream);
/* dY (B, N): gradient w.r.t. the layer output Y; dZ (B, N) scratch when relu;
 * outputs dX (B, K, may be NULL), dW (N, K), db (N). */
int carc_mlp_linear_backward(int32_t B, int32_t K, int32_t N, const float* X, const float* W, const float* Y,
                             const float* dY, int32_t relu, float* dZ, float* dX, float* dW, float* db, void* stream);
/* loss (one float) = sum (Y - T)^2 / (2 B) over n = B * features; dY = (Y - T) / B */
int carc_mlp_mse(int64_t n, int32_t B, const float* Y, const float* T, float* dY, float* loss, void* stream);
/* Adam step (bias-corrected, step >= 1) on n parameters */
int carc_mlp_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                  float eps, int32_t step, void* stream);
int carc_mlp_to_bf16(int64_t n, const float* x, void* y, void* stream);
/* Y = X W^T + b with BF16 X, W; output BF16 (Yb) and/or FP32 (Yf) */
int carc_mlp_linear_bf16(int32_t B, int32_t K, int32_t N, const void* X, const void* W, const float* b, int32_t relu,
                         void* Yb, float* Yf, void* stream);

/*
 * Batched block eigensolver (LOBPCG) over many independent center-site
 * problems: the lowest eigenpairs of Hermitian-definite pencils H x = l N x,
 * the per-problem unit of minimizeExpectation / relaxOver
 * (system/_2d.py:489-497, utils.py:805-878), which the reference solves one
 * problem at a time.  Block of m in {1, 2, 4, 8} vectors; search space
 * S = [X; R; P] of k = 3m rows with H S and N S supplied by the caller's
 * matvecs.  Per iteration over the whole batch (orthonormalising form): the
 * caller applies N to R; carc_lobpcg_inner gives [X; R; P]^H N [R, P];
 * carc_lobpcg_orth_prepare, carc_zheev_jacobi (n = m, 2 batch matrices) and
 * carc_lobpcg_orth_finish give the coefficients with which
 * carc_lobpcg_orth_apply makes R and P each N-orthonormal and N-orthogonal
 * to X; the caller applies H and N to the new R (every few iterations it
 * also applies them to X afresh and restarts P, which bounds the drift of the
 * implicitly updated images under the split-precision rounding); carc_lobpcg_inner
 * gives S^H H S and S^H N S; carc_lobpcg_rr_scale, carc_zheev_jacobi (n = k),
 * carc_lobpcg_rr_reduce, carc_zheev_jacobi and carc_lobpcg_rr_combine the
 * Rayleigh-Ritz coefficients; carc_lobpcg_update the next X, P, R and the
 * residuals.  Layout: problem b's k x n[b] blocks of S, HS, NS row-major at
 * element offset off[b] of three complex128 pools; work item w covers entries
 * [item_start[w], item_start[w] + CARC_LOBPCG_ITEM) of problem
 * item_problem[w], and problem b owns items first[b] .. first[b+1]-1.
 * Problems with active[b] == 0 are skipped.  Small matrices are row-major per
 * problem.  All pointers device.
 */
int64_t carc_lobpcg_workspace_size(int32_t items, int32_t m);
/* out1 (batch x ka x kb) = conj(A rows a0..) . (B1 rows b0..)^T per problem; out2 likewise from B2 (may be NULL) */
int carc_lobpcg_inner(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem, const int32_t* item_start,
                      const int32_t* first, const int64_t* off, const int32_t* n, const int32_t* active,
                      const void* A, int32_t a0, int32_t ka, const void* B1, const void* B2, int32_t b0, int32_t kb,
                      void* out1, void* out2, void* workspace, int64_t workspace_bytes, void* stream);
/* Q (batch x 3m x 2m) = [X; R; P]^H N [R, P] -> Ms (batch x 2 x m x m): for Z = R, P the unit-diagonal
 * N-Gram matrix of Z - X (X^H N Z); dscale (batch x 2 x m) their diagonal scalings (0 for a column whose
 * remaining N-norm^2 is at most floor times its original) */
int carc_lobpcg_orth_prepare(int32_t batch, int32_t m, const int32_t* active, const void* Q, double floor_, void* Ms,
                             void* dscale, void* stream);
/* W (batch x 2 x m), V: eigenpairs of Ms -> M (batch x 4 x m x m) = [M_R1; M_R2; M_P1; M_P2] with
 * Z <- Z M_Z1 + X M_Z2; directions with W_j <= drop max W are dropped, and all of P's when restart_p != 0
 * (P restarts from zero, as after a refresh of X's images) */
int carc_lobpcg_orth_finish(int32_t batch, int32_t m, const int32_t* active, const void* Q, const void* dscale,
                            const void* W, const void* V, double drop, int32_t restart_p, void* M, void* stream);
/* in place: R rows of S <- R M_R1 + X M_R2; P rows of S, HS, NS <- P M_P1 + X M_P2 */
int carc_lobpcg_orth_apply(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem,
                           const int32_t* item_start, const int32_t* first, const int64_t* off, const int32_t* n,
                           const int32_t* active, const void* M, void* S, void* HS, void* NS, void* stream);
/* GNs = D herm(GN) D with D = diag(GN)^-1/2 (0 where the diagonal is 0); dscale (batch x k) = D */
int carc_lobpcg_rr_scale(int32_t batch, int32_t m, const int32_t* active, const void* GN, void* GNs, void* dscale,
                         void* stream);
/* W, V: eigenpairs of GNs; keeps directions with W_j > drop max W (rank per problem);
 * T = D V diag(W^-1/2 on kept, 0 else), G = T^H herm(GH) T with dropped diagonals raised above the spectrum */
int carc_lobpcg_rr_reduce(int32_t batch, int32_t m, const int32_t* active, const void* GH, const void* dscale,
                          const void* W, const void* V, double drop, void* T, void* G, int32_t* rank, void* stream);
/* C (batch x k x m) = T Y[:, :m], Y the eigenvectors of G */
int carc_lobpcg_rr_combine(int32_t batch, int32_t m, const int32_t* active, const void* T, const void* Y, void* C,
                           void* stream);
/* into the second pools: X' = S^T C, P' = [R; P]^T C[m:] (and likewise from HS, NS), R' = H X' - N X' diag(theta)
 * (theta: the eigenvalues of G, batch x k ascending); res (batch x m) = |R'_j| / (|H X'_j| + |theta_j| |N X'_j|) */
int carc_lobpcg_update(int32_t batch, int32_t items, int32_t m, const int32_t* item_problem, const int32_t* item_start,
                       const int32_t* first, const int64_t* off, const int32_t* n, const int32_t* active, const void* C,
                       const void* theta, const void* S, const void* HS, const void* NS, void* S2, void* HS2,
                       void* NS2, void* res, void* workspace, int64_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CARCASSONNE_GB300_H */
