// Allocation-free variant of the FP64 stage-3 matvec.
//
// Some callers cannot allocate device memory while they run: a host
// application that reserves the whole GPU up front and forbids libraries to
// call cudaMalloc afterwards, or a latency-bound loop that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may cause.  They also cannot
// be asked for a workspace buffer of a size they do not know in advance.  For
// them, carc_stage3_matvec_f64_noalloc takes the matvec's scratch from a fixed
// array compiled into this library instead of from the caller.
//
// The array is CARC_NOALLOC_SCRATCH_BYTES (16 MiB) of device memory that every
// GPU which loads this library holds until the process exits.  Its device
// address is looked up once per device, on the first call made with that
// device current; make that first call before any stream capture.  The
// cached address belongs to the device's primary context: after
// cudaDeviceReset (or any other destruction of that context) it is stale, and
// the library has to be unloaded and loaded again.  All calls
// share the one array, so calls that overlap on the GPU (on different streams,
// or from different host threads) race on it and must be serialised by the
// caller.  No byte of the array needs to start at zero: every byte a call
// reads was written earlier in the same call.
#include "common.cuh"
#include "stage3.cuh"

#include <mutex>

namespace carc {

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_stage3_scratch[CARC_NOALLOC_SCRATCH_BYTES];

std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_stage3_scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = -1;
  CARC_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(CARC_BAD_ARG, "noalloc: device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_stage3_scratch);
    if (e != cudaSuccess || !p)
      return fail(CARC_CUDA_ERROR, "noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                  cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return CARC_OK;
}

}  // namespace

}  // namespace carc

using namespace carc;

extern "C" int carc_stage3_matvec_f64_noalloc(const int64_t* s0_shape, const int64_t* s1_shape, int64_t d,
                                              const void* const* s0_ptrs, int32_t n0, const void* const* s1_ptrs,
                                              int32_t n1, const void* const* op_ptrs, int32_t nop,
                                              const int32_t* terms, int32_t n_terms, const void* x, void* y,
                                              int32_t nvec, int32_t accumulate, void* stream) {
  if (!s0_shape || !s1_shape || !s0_ptrs || !s1_ptrs || (nop > 0 && !op_ptrs) || (n_terms > 0 && !terms) || !x || !y)
    return fail(CARC_BAD_ARG, "carc_stage3_matvec_f64_noalloc: NULL argument");
  const int64_t need = stage3_matvec_ws(s0_shape, s1_shape, d, n_terms, nvec);
  if (need < 0) return CARC_BAD_SHAPE;
  if (need > (int64_t)CARC_NOALLOC_SCRATCH_BYTES)
    return fail(CARC_TOO_LARGE,
                "carc_stage3_matvec_f64_noalloc: this problem needs %lld bytes of scratch, more than the fixed "
                "%lld-byte array; use carc_stage3_matvec_f64 with a caller-provided workspace",
                (long long)need, (long long)CARC_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  CARC_RETURN_IF(scratch_address(&scratch));
  return stage3_matvec(s0_shape, s1_shape, d, s0_ptrs, n0, s1_ptrs, n1, op_ptrs, nop, terms, n_terms, x, y, nvec,
                       accumulate, scratch, (int64_t)CARC_NOALLOC_SCRATCH_BYTES, as_stream(stream));
}
