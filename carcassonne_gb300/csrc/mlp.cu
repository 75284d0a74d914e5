// The learned start vector's network: a fully connected MLP trained and run
// by these kernels alone.
//
//   training (FP32): strided tiled SGEMM for every forward and backward
//   product, fused bias + ReLU epilogue, bias-gradient column sums, masked
//   ReLU backward, mean-squared-error loss and gradient, Adam update;
//   inference (BF16 weights and activations, FP32 accumulation): one warp per
//   output with a shuffle reduction.
//
// Layouts: activations row-major (batch, features); a weight matrix W is
// (out, in) row-major, a layer computes Y = X W^T + b.
#include "common.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace carc {

namespace {

constexpr int SG_BM = 64, SG_BN = 64, SG_BK = 16, SG_T = 256;

// C[m][n] = alpha * sum_k A(m,k) B(n,k) + beta * C[m][n] (+ bias[n], ReLU)
// with A(m,k) = A[m*sam + k*sak], B(n,k) = B[n*sbn + k*sbk].
struct SgemmArgs {
  const float* A;
  const float* B;
  float* C;
  const float* bias;
  int M, N, K;
  int64_t sam, sak, sbn, sbk, ldc;
  float alpha, beta;
  int relu;
};

__global__ __launch_bounds__(SG_T) void sgemm_kernel(const SgemmArgs a) {
  __shared__ float As[SG_BK][SG_BM + 1];
  __shared__ float Bs[SG_BK][SG_BN + 1];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * SG_BM, n0 = blockIdx.x * SG_BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < a.K; k0 += SG_BK) {
    for (int i = tid; i < SG_BK * SG_BM; i += SG_T) {
      const int kk = i / SG_BM, mm = i % SG_BM;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < a.M && k < a.K) ? a.A[m * a.sam + k * a.sak] : 0.f;
    }
    for (int i = tid; i < SG_BK * SG_BN; i += SG_T) {
      const int kk = i / SG_BN, nn = i % SG_BN;
      const int n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < a.N && k < a.K) ? a.B[n * a.sbn + k * a.sbk] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < SG_BK; ++kk) {
      float av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= a.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= a.N) continue;
      float v = a.alpha * acc[i][j];
      float* c = a.C + (int64_t)m * a.ldc + n;
      if (a.beta != 0.f) v += a.beta * *c;
      if (a.bias) v += a.bias[n];
      if (a.relu) v = fmaxf(v, 0.f);
      *c = v;
    }
  }
}

int sgemm(const SgemmArgs& a, cudaStream_t stream) {
  if (a.M < 1 || a.N < 1 || a.K < 1) return fail(CARC_BAD_SHAPE, "mlp sgemm: %d x %d x %d", a.M, a.N, a.K);
  dim3 grid((a.N + SG_BN - 1) / SG_BN, (a.M + SG_BM - 1) / SG_BM);
  sgemm_kernel<<<grid, SG_T, 0, stream>>>(a);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

// db[n] = sum_b dY[b][n]
__global__ void colsum_kernel(const float* __restrict__ dY, float* __restrict__ db, int B, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += dY[(int64_t)b * N + n];
  db[n] = s;
}

// dZ = dY * (Y > 0)
__global__ void relu_bwd_kernel(int64_t n, const float* __restrict__ Y, const float* __restrict__ dY,
                                float* __restrict__ dZ) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dZ[i] = Y[i] > 0.f ? dY[i] : 0.f;
}

// loss = sum (Y - T)^2 / (2 B); dY = (Y - T) / B.  Block partial sums, then one atomic per block.
__global__ void mse_kernel(int64_t n, int B, const float* __restrict__ Y, const float* __restrict__ T,
                           float* __restrict__ dY, float* __restrict__ loss) {
  __shared__ float red[32];
  float s = 0.f;
  const float inv = 1.f / (float)B;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    dY[i] = d * inv;
    s += 0.5f * d * d * inv;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(loss, s);
  }
}

__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void to_bf16_kernel(int64_t n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

// Y[b][o] = act(sum_k X[b][k] W[o][k] + bias[o]), BF16 operands, FP32 accumulation; one warp per (b, o).
__global__ void linear_bf16_kernel(int B, int K, int N, const __nv_bfloat16* __restrict__ X,
                                   const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias, int relu,
                                   __nv_bfloat16* __restrict__ Yb, float* __restrict__ Yf) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (warp >= (int64_t)B * N) return;
  const int b = (int)(warp / N), o = (int)(warp % N);
  const __nv_bfloat16* x = X + (int64_t)b * K;
  const __nv_bfloat16* w = W + (int64_t)o * K;
  // element-wise (2-byte) loads: rows of odd length K start at odd element
  // offsets, where a paired bf16x2 load would be misaligned
  float s = 0.f;
  for (int k = lane; k < K; k += 32) s = fmaf(__bfloat162float(x[k]), __bfloat162float(w[k]), s);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) {
    float v = s + (bias ? bias[o] : 0.f);
    if (relu) v = fmaxf(v, 0.f);
    if (Yb) Yb[(int64_t)b * N + o] = __float2bfloat16_rn(v);
    if (Yf) Yf[(int64_t)b * N + o] = v;
  }
}

inline int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4 * 152)); }

}  // namespace

// Y = relu?(X W^T + b): X (B, K), W (N, K), Y (B, N), FP32
int mlp_linear_forward(int B, int K, int N, const float* X, const float* W, const float* b, int relu, float* Y,
                       cudaStream_t stream) {
  SgemmArgs a{X, W, Y, b, B, N, K, K, 1, K, 1, N, 1.f, 0.f, relu};
  return sgemm(a, stream);
}

// Given dY (B, N) (gradient after the activation), the layer's input X (B, K),
// output Y (B, N) and weights W (N, K): dX (B, K) (may be NULL), dW (N, K), db (N).
int mlp_linear_backward(int B, int K, int N, const float* X, const float* W, const float* Y, const float* dY,
                        int relu, float* dZ, float* dX, float* dW, float* db, cudaStream_t stream) {
  const float* g = dY;
  if (relu) {
    relu_bwd_kernel<<<grid1((int64_t)B * N), 256, 0, stream>>>((int64_t)B * N, Y, dY, dZ);
    CARC_CHECK_LAUNCH();
    g = dZ;
  }
  // dW[n][k] = sum_b g[b][n] X[b][k]
  SgemmArgs aw{g, X, dW, nullptr, N, K, B, 1, N, 1, K, K, 1.f, 0.f, 0};
  CARC_RETURN_IF(sgemm(aw, stream));
  colsum_kernel<<<(N + 255) / 256, 256, 0, stream>>>(g, db, B, N);
  CARC_CHECK_LAUNCH();
  if (dX) {
    // dX[b][k] = sum_n g[b][n] W[n][k]
    SgemmArgs ax{g, W, dX, nullptr, B, K, N, N, 1, 1, K, K, 1.f, 0.f, 0};
    CARC_RETURN_IF(sgemm(ax, stream));
  }
  return CARC_OK;
}

int mlp_mse(int64_t n, int B, const float* Y, const float* T, float* dY, float* loss, cudaStream_t stream) {
  CARC_CHECK_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), stream));
  mse_kernel<<<grid1(n), 256, 0, stream>>>(n, B, Y, T, dY, loss);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int mlp_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps, int step,
             cudaStream_t stream) {
  if (step < 1) return fail(CARC_BAD_ARG, "adam: step %d", step);
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<grid1(n), 256, 0, stream>>>(n, p, g, m, v, lr, b1, b2, eps, c1, c2);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int mlp_to_bf16(int64_t n, const float* x, void* y, cudaStream_t stream) {
  to_bf16_kernel<<<grid1(n), 256, 0, stream>>>(n, x, static_cast<__nv_bfloat16*>(y));
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

int mlp_linear_bf16(int B, int K, int N, const void* X, const void* W, const float* b, int relu, void* Yb, float* Yf,
                    cudaStream_t stream) {
  const int64_t warps = (int64_t)B * N;
  linear_bf16_kernel<<<(int)((warps * 32 + 255) / 256), 256, 0, stream>>>(
      B, K, N, static_cast<const __nv_bfloat16*>(X), static_cast<const __nv_bfloat16*>(W), b, relu,
      static_cast<__nv_bfloat16*>(Yb), Yf);
  CARC_CHECK_LAUNCH();
  return CARC_OK;
}

}  // namespace carc
