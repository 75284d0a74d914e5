// Shared definitions of the carcassonne_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include "../../include/carcassonne_gb300.h"

namespace carc {

// Thread-local last error message, readable through carc_last_error_string().
void set_error(const char* fmt, ...);
int fail(int status, const char* fmt, ...);

#define CARC_CHECK_CUDA(expr)                                                     \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess)                                                        \
      return ::carc::fail(CARC_CUDA_ERROR, "%s: %s (%s:%d)", #expr,              \
                          cudaGetErrorString(_e), __FILE__, __LINE__);            \
  } while (0)

// Number of kernels this library has launched (all threads), read through
// carc_launch_counter(); every launch site goes through CARC_CHECK_LAUNCH.
void count_launch();

#define CARC_CHECK_LAUNCH()                                                       \
  do {                                                                            \
    ::carc::count_launch();                                                       \
    cudaError_t _e = cudaGetLastError();                                          \
    if (_e != cudaSuccess)                                                        \
      return ::carc::fail(CARC_CUDA_ERROR, "kernel launch: %s (%s:%d)",           \
                          cudaGetErrorString(_e), __FILE__, __LINE__);            \
  } while (0)

// Optional per-phase device timing: when enabled (carc_phase_timing_enable),
// a PhaseScope records a CUDA event pair on the launching stream around the
// launches of one phase; carc_phase_timing_read sums the elapsed times.
enum Phase {
  PH_TC_PACK = 0, PH_TC_STEP_A = 1, PH_TC_STEP_B = 2, PH_TC_REDUCE = 3,  // tensor-core matvec
  PH_HEGV_POTRF = 4, PH_HEGV_TRTRI = 5, PH_HEGV_REDUCE = 6, PH_HEGV_LANCZOS = 7,  // hegv_lowest
  PH_COUNT = 8
};
bool phase_timing_on();
void phase_record(int phase, cudaStream_t stream, bool start);

struct PhaseScope {
  int phase;
  cudaStream_t stream;
  bool on;
  PhaseScope(int ph, cudaStream_t s) : phase(ph), stream(s), on(phase_timing_on()) {
    if (on) phase_record(phase, stream, true);
  }
  ~PhaseScope() {
    if (on) phase_record(phase, stream, false);
  }
};

#define CARC_RETURN_IF(status_expr)                                               \
  do {                                                                            \
    int _s = (status_expr);                                                       \
    if (_s != CARC_OK) return _s;                                                 \
  } while (0)

// ---- complex double helpers ------------------------------------------------
__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a += b * c
__device__ __forceinline__ void cfma(double2& a, double2 b, double2 c) {
  a.x = fma(b.x, c.x, a.x);
  a.x = fma(-b.y, c.y, a.x);
  a.y = fma(b.x, c.y, a.y);
  a.y = fma(b.y, c.x, a.y);
}
// conj(b) * c
__host__ __device__ __forceinline__ double2 cmulc(double2 b, double2 c) {
  return make_double2(b.x * c.x + b.y * c.y, b.x * c.y - b.y * c.x);
}
__host__ __device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}

// ---- complex float (complex64) overloads ------------------------------------
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ void cfma(float2& a, float2 b, float2 c) {
  a.x = fmaf(b.x, c.x, a.x);
  a.x = fmaf(-b.y, c.y, a.x);
  a.y = fmaf(b.x, c.y, a.y);
  a.y = fmaf(b.y, c.x, a.y);
}
__host__ __device__ __forceinline__ float2 cmulc(float2 b, float2 c) {
  return make_float2(b.x * c.x + b.y * c.y, b.x * c.y - b.y * c.x);
}
__host__ __device__ __forceinline__ float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float2 warp_sum2(float2 v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}
// zero of a complex type; widening to complex128
template <typename Z>
__host__ __device__ __forceinline__ Z czero() {
  Z z;
  z.x = 0;
  z.y = 0;
  return z;
}
__host__ __device__ __forceinline__ double2 to_d2(double2 a) { return a; }
__host__ __device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(a.x, a.y); }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace carc
