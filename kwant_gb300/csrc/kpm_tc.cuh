// tcgen05 / TMA / mbarrier building blocks shared by the tensor-core
// kernels (kpm_gemm_tc.cu: correlator moments matrix; kpm_mlp.cu: surrogate
// network matmuls).  Inline PTX written for sm_103a.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "kpm_common.cuh"

namespace kpm {
namespace tc {

constexpr int TM = 128;          // output rows per CTA (MMA M)
constexpr int THREADS = 128;

// Limit of every bounded mbarrier wait (ns of GPU time, default 2 s) and
// the test-only producer stall, set by kpm_debug_set (host side).
struct WaitCfg {
  uint64_t ns;
  int stall;
};
WaitCfg wait_cfg();

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; returns false (and records err) when the deadline passes
// or another thread has recorded an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          int* err, int code,
                                          uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*(volatile int*)err) return false;
    if (global_ns() - t0 > limit_ns) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

// Bounded wait that does not give up on another thread's error (for
// copies and MMAs already in flight, which complete regardless).
__device__ __forceinline__ bool mbar_wait_all(uint64_t* bar, uint32_t parity,
                                              uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// The producer's last `issued` TMA loads (at most one pending phase per
// stage) have landed in shared memory: called before the CTA releases its
// resources, also after an error stopped the pipeline.
__device__ __forceinline__ void drain_loads(uint64_t* full, int stages,
                                            int64_t issued, int* err,
                                            uint64_t limit_ns) {
  for (int64_t i = issued > stages ? issued - stages : 0; i < issued; ++i) {
    const int s = (int)(i % stages);
    if (!mbar_wait_all(&full[s], (uint32_t)((i / stages) & 1), limit_ns))
      atomicCAS(err, 0, 4);
  }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map,
                                            uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0),
      "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map,
                                            uint64_t* bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0),
      "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

// Per-stage K width: rows of KC bf16 = 2*KC bytes, swizzled over that width
// (64 B -> 2 stages, 32 B -> 4 stages in the same shared memory).
template <int KC> struct Stage;
template <> struct Stage<32> {
  static constexpr int STAGES = 2;
  static constexpr uint64_t LAYOUT = 4;   // descriptor: 64-byte swizzle
  static constexpr uint32_t SBO = 512;    // 8 rows x 64 B
};
template <> struct Stage<16> {
  static constexpr int STAGES = 4;
  static constexpr uint64_t LAYOUT = 6;   // descriptor: 32-byte swizzle
  static constexpr uint32_t SBO = 256;    // 8 rows x 32 B
};

// Shared-memory matrix descriptor: K-major, swizzled rows of 2*KC bytes,
// 8-row groups SBO bytes apart (stride byte offset), version 1.
template <int KC>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);      // start address
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused)
  d |= (uint64_t)(Stage<KC>::SBO >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;                       // descriptor version
  d |= Stage<KC>::LAYOUT << 61;                 // swizzle mode
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16 (or both FP16
// when f16), both K-major, M = 128, N = n; optional negation of A.
__host__ __device__ constexpr uint32_t instr_desc(int n, bool neg_a,
                                                  bool f16 = false) {
  return (1u << 4)                    // D format F32
         | ((f16 ? 0u : 1u) << 7)     // A format: 0 FP16, 1 BF16
         | ((f16 ? 0u : 1u) << 10)    // B format (the same as A)
         | ((neg_a ? 1u : 0u) << 13)  // negate A
         | ((uint32_t)(n >> 3) << 17) // N / 8
         | ((uint32_t)(TM >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc,
                                         uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];" ::"r"(smem_u32(bar))
      : "memory");
}


// TMA 2D tile load (coordinates: {inner, outer}) completing on an mbarrier
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map,
                                            uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx"
      "::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0),
      "r"(c1)
      : "memory");
}

inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  }
  return fn;
}

}  // namespace tc
}  // namespace kpm
