// Shared definitions for the KPM CUDA kernels and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/kwant_gb300.h"

namespace kpm {

// --- error reporting -------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

#define KPM_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t err__ = (call);                                             \
    if (err__ != cudaSuccess) {                                             \
      ::kpm::set_error("%s:%d: %s failed: %s", __FILE__, __LINE__, #call,   \
                       cudaGetErrorString(err__));                          \
      return KPM_ECUDA;                                                     \
    }                                                                       \
  } while (0)

#define KPM_CHECK_LAUNCH() KPM_CUDA(cudaGetLastError())

#define KPM_REQUIRE(cond, ...)                                              \
  do {                                                                      \
    if (!(cond)) {                                                          \
      ::kpm::set_error(__VA_ARGS__);                                        \
      return KPM_EINVAL;                                                    \
    }                                                                       \
  } while (0)

#define KPM_TRY(expr)                                                       \
  do {                                                                      \
    int st__ = (expr);                                                      \
    if (st__ != KPM_OK) return st__;                                        \
  } while (0)

// NVTX range over an API call (named in Nsight Systems / Compute
// timelines; a no-op unless a tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// --- launch geometry -------------------------------------------------------
// A "slot" is LANES consecutive threads that together own one matrix row for
// one group of vectors; each lane holds 16 bytes of vector data
// (1 complex128 or 2 complex64).
constexpr int LANES = 16;
constexpr int STEP_THREADS = 256;
constexpr int SLOTS = STEP_THREADS / LANES;
// Vectors per group: 16 (complex128) or 32 (complex64).
constexpr int GROUP_FP64 = LANES;
constexpr int GROUP_FP32 = 2 * LANES;
// Upper bound on the number of row partitions ("x items") of a step, per
// SM.  The partition count depends only on the number of rows and the
// device's SM count, never on the number of vectors or on the launch
// shape, so the reduction order of every dot product is fixed for a given
// GPU model.  4 is the resident blocks per SM of the complex64 ELL step
// kernel: its persistent grid then gets exactly one long run of rows per
// vector group and block (the per-item pipeline start and block reduction
// are amortised over many rows, and no block idles in a last round).
#ifndef KPM_XITEMS_PER_SM
#define KPM_XITEMS_PER_SM 4
#endif
constexpr int XITEMS_PER_SM = KPM_XITEMS_PER_SM;

inline int group_size(int precision) {
  return precision == KPM_PREC_MIXED ? GROUP_FP32 : GROUP_FP64;
}
// Vector group of a block of R vectors: complex64 blocks of at most 16
// vectors use 16-vector groups (one complex64 per lane), so that R <= 16
// (Kwant's default is 10) does not move padding vectors.
inline int group_size(int precision, int64_t R) {
  return precision == KPM_PREC_MIXED && R > GROUP_FP64 ? GROUP_FP32
                                                       : GROUP_FP64;
}
__host__ __device__ inline int64_t round_up(int64_t x, int64_t m) {
  return (x + m - 1) / m * m;
}
__host__ __device__ inline int64_t ceil_div(int64_t x, int64_t m) {
  return (x + m - 1) / m;
}

// SplitMix64 finaliser (Steele, Lea & Flood 2014; Vigna's constants): the
// counter-based generator of the device-side random-phase vectors.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// 16-byte asynchronous global -> shared copy (L2 only), grouped per thread
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// wait until at most the most recent group is still in flight
__device__ __forceinline__ void cp_async_wait_prev() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
}

inline int xitems_for_rows(int64_t rows, int num_sms,
                           int per_sm = XITEMS_PER_SM) {
  int64_t x = ceil_div(rows, (int64_t)SLOTS);
  const int64_t cap = (int64_t)per_sm * (num_sms > 0 ? num_sms : 1);
  if (x > cap) x = cap;
  if (x < 1) x = 1;
  return (int)x;
}

// --- handle / block state ---------------------------------------------------
struct Matrix {
  int64_t rows = 0, nnz = 0;
  int32_t* indptr = nullptr;   // rows + 1
  int32_t* indices = nullptr;  // nnz
  void* data = nullptr;        // nnz complex (double2 raw H | float2 2H/a)
  // ELL copy for the complex64 step kernel: ell_k entries per row (the row's
  // CSR entries in order, then padding with column = row, value = 0)
  int ell_k = 0;
  int32_t* ell_idx = nullptr;  // [rows][ell_k]
  float2* ell_val = nullptr;   // [rows][ell_k]
};

}  // namespace kpm

struct kpm_handle {
  int precision = KPM_PREC_FP64;
  // mixed precision: DOS blocks keep a bfloat16 lo part next to every
  // complex64 element and step with the compensated kernel (cleared by
  // KPM_FLAG_PLAIN_C64; needs the complex64 ELL copy)
  bool compensated = false;
  // bounds-checked builds (-DKPM_CHECK): first out-of-range column index a
  // step kernel met, plus one (0: none)
  unsigned long long* check = nullptr;
  // compensated DOS: ELL copy with every row's diagonal entry first and the
  // diagonal shift -2b/a folded into it (rebuilt on the device by each DOS
  // call); dg_ok: every row had a real diagonal entry (else the general
  // compensated kernel runs)
  int32_t* dg_idx = nullptr;
  float4* dg_val = nullptr;   // (hr, hr, hi, hi) per entry
  int* dg_flag = nullptr;
  bool dg_ok = false;
  int device = 0;
  int num_sms = 0;
  double a = 1.0, b = 0.0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  kpm::Matrix H;
  // dot-product partials: [group][vector*3 + component][xitems] doubles
  double* partials = nullptr;
  size_t partials_cap = 0;
  // host vectors already copied to the device ([R][N] complex128, in flight
  // on the handle's stream order): the next upload of exactly that host
  // array uses and frees it instead of copying again
  void* vec_staging = nullptr;
  const void* vec_staging_src = nullptr;
  size_t vec_staging_bytes = 0;
  int resident_step_blocks = 0;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  bool timed = false;
  // device time of the last tensor-core contraction and its MMA flops
  cudaEvent_t ev_gemm0 = nullptr, ev_gemm1 = nullptr;
  double last_gemm_ms = 0.0, last_gemm_flops = 0.0;
  // K elements per pipeline stage of the tensor-core contraction: 32 (two
  // stages, 64-byte rows; measured 3.09 ms on the 200x200x2 / R=16 / M=256
  // workload) or 16 (four stages, 32-byte rows; 6.13 ms)
  int tc_kc = 32;
  // optional locality reordering: device row p holds original row perm[p]
  int32_t* perm = nullptr;            // device, new -> old (null: identity)
  std::vector<int32_t> h_iperm;       // host, old -> new
  // per-launch profiling of step kernels (pairs of events)
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;
  size_t prof_used = 0;
  // parametric family: CSR-ordered complex128 B, Theta (real part), D1, D2
  // in the handle's row order (null: no family set)
  double2* fam_base = nullptr;
  double2* fam_theta = nullptr;
  double2* fam_d1 = nullptr;
  double2* fam_d2 = nullptr;
};

struct kpm_block {
  kpm_handle* h = nullptr;
  int64_t R = 0;        // real vectors
  int64_t Rpad = 0;     // padded to the group size
  int G = 0;            // vectors per group (16, or 32 for complex64 R > 16)
  int groups = 0;
  int64_t N = 0;
  bool keep_a0 = false;
  void* a0 = nullptr;    // [N][Rpad]
  void* buf[2] = {nullptr, nullptr};
  // compensated blocks: bfloat16 lo parts of a0 / buf, [N][Rpad] words
  // (null otherwise); valid for a0 always, for buf while mode is DOS
  uint32_t* lo_a0 = nullptr;
  uint32_t* lo_buf[2] = {nullptr, nullptr};
  void* p_cur = nullptr;   // alpha_n (a0 or one of buf)
  void* p_prev = nullptr;  // alpha_{n-1}
  double* mu01 = nullptr;   // [Rpad][2] complex: mu0, mu1 per vector
  int64_t steps_done = 0;   // number of matvecs applied (n of alpha_n)
  int mode = -1;            // 0 = DOS, 1 = operator/vectors
  void* op_coef = nullptr;  // [terms][Rpad] complex128 bra factors
  const void* op_tag = nullptr;  // operator the factors belong to
};
