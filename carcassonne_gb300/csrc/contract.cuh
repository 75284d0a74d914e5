// Host-side launchers of the FP64 contraction engine (contract.cu).
#pragma once
#include "common.cuh"
#include <cstring>

#define CARC_MAX_PERMUTE_DIMS 16

namespace carc {

// Kernel parameters of the grouped GETT, passed by value (fits the 32 KB
// kernel-parameter space of sm_90+).
struct GettParams {
  int nm, nn, nk;
  int conj_a, conj_b;
  int accumulate;
  int n_out;
  int ksplit;
  int64_t m_ext[CARC_MAX_SUBDIMS], n_ext[CARC_MAX_SUBDIMS], k_ext[CARC_MAX_SUBDIMS];
  int64_t a_m[CARC_MAX_SUBDIMS], a_k[CARC_MAX_SUBDIMS];
  int64_t b_n[CARC_MAX_SUBDIMS], b_k[CARC_MAX_SUBDIMS];
  int64_t c_m[CARC_MAX_SUBDIMS], c_n[CARC_MAX_SUBDIMS];
  int64_t M, N, K;
  int64_t kchunk;
  double2 alpha;
  double2* partial;
  const double2* a[CARC_MAX_SLOTS];
  const double2* b[CARC_MAX_SLOTS];
  double2* c[CARC_MAX_SLOTS];
  int16_t ea[CARC_MAX_ENTRIES];
  int16_t eb[CARC_MAX_ENTRIES];
  int16_t ob[CARC_MAX_SLOTS + 1];
};

const char* last_error();
long long launch_count();
int phase_timing_enable(int on);
int phase_timing_read(int phase, double* total_ms, int64_t* count);
int validate_desc(const carc_contract_desc& d);
int64_t gett_workspace_size(const carc_contract_desc& d, int n_out);
int gett_launch(const carc_contract_desc& d, const void* const* a_ptrs, int n_a, const void* const* b_ptrs, int n_b,
                void* const* c_ptrs, int n_c, const int32_t* entries, int n_entries, double2 alpha, int accumulate,
                void* workspace, int64_t workspace_bytes, cudaStream_t stream);
int permute_launch(const void* in, void* out, int ndim, const int64_t* shape, const int64_t* istr, int conj,
                   cudaStream_t stream);
int axpby_launch(int64_t n, double2 a, const void* x, double2 b, const void* y, void* out, cudaStream_t stream);
int mul_launch(int64_t n, const void* x, const void* y, void* out, cudaStream_t stream);
int fill_launch(int64_t n, double2 v, void* out, cudaStream_t stream);
int64_t dot_workspace_size(int64_t n);
int dot_launch(int64_t n, const void* x, const void* y, int conj_x, void* out, void* ws, int64_t ws_bytes,
               cudaStream_t stream);
int hasnan_launch(int64_t n, const void* x, void* flag, cudaStream_t stream);

// A small helper to build contraction descriptors on the host.
struct DescBuilder {
  carc_contract_desc d;
  DescBuilder() { memset(&d, 0, sizeof(d)); }
  DescBuilder& m(int64_t ext, int64_t a_str, int64_t c_str) {
    d.m_ext[d.nm] = ext;
    d.a_m[d.nm] = a_str;
    d.c_m[d.nm] = c_str;
    d.nm++;
    return *this;
  }
  DescBuilder& n(int64_t ext, int64_t b_str, int64_t c_str) {
    d.n_ext[d.nn] = ext;
    d.b_n[d.nn] = b_str;
    d.c_n[d.nn] = c_str;
    d.nn++;
    return *this;
  }
  DescBuilder& k(int64_t ext, int64_t a_str, int64_t b_str) {
    d.k_ext[d.nk] = ext;
    d.a_k[d.nk] = a_str;
    d.b_k[d.nk] = b_str;
    d.nk++;
    return *this;
  }
};

}  // namespace carc
