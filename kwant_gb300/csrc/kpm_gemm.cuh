// K-major vector stores and the moments-matrix contraction of the correlator.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kpm_common.cuh"

namespace kpm {

enum { STORE_C128 = 0, STORE_BF16X3 = 1 };

// K padding of the BF16x3 planes: a multiple of the tensor-core K tile.
constexpr int64_t STORE_KPAD = 128;
// BF16x3 planes are K-blocked: [K / KB][plane][row][K % KB].  A tensor-core
// pipeline stage (KB or KB/2 K-elements of 128 rows and 4 planes) is then
// four contiguous runs of 128 x 64 bytes, instead of 512 pieces of 64 bytes
// one row stride (the whole K extent, 2.5 MB on the Kubo workload) apart.
constexpr int64_t STORE_KB = 32;

__host__ __device__ inline int64_t store_index(int64_t M, int q, int64_t n,
                                               int64_t k) {
  return ((k / STORE_KB) * 4 * M + q * M + n) * STORE_KB + (k % STORE_KB);
}

// STORE_BF16X3 planes hold 16-bit splits hi = t(x), lo = t(x - hi) with
// t = bfloat16 (the default) or, when f16 is set, IEEE half: the same
// layout and MMA count, 11 instead of 8 significant bits per part (FP16
// overflows above 65504, far beyond the entries of normalised Chebyshev
// vectors).
struct StoreRow {
  double2* c128;            // STORE_C128 row
  __nv_bfloat16* planes;    // STORE_BF16X3: the store's planes (re_hi,
  int64_t M, n;             //   re_lo, im_hi, im_lo) and the row n
  int f16;                  // planes are FP16 (else bfloat16)
};

struct Store {
  int kind = STORE_C128;
  int64_t M = 0, K = 0, Kp = 0;  // rows, logical K, padded K
  double2* c128 = nullptr;
  __nv_bfloat16* planes = nullptr;  // 4 K-blocked planes of M x Kp
  int f16 = 0;                      // FP16 planes (else bfloat16)
  StoreRow row(int64_t n) const {
    StoreRow r{};
    if (kind == STORE_C128) {
      r.c128 = c128 + n * K;
    } else {
      r.planes = planes;
      r.M = M;
      r.n = n;
      r.f16 = f16;
    }
    return r;
  }
};

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi,
                                           __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

__device__ __forceinline__ void split_f16(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}

template <int STORE, typename S>
__device__ __forceinline__ void store_put(const StoreRow& r, int64_t k, S re,
                                          S im) {
  if constexpr (STORE == STORE_C128) {
    r.c128[k] = make_double2((double)re, (double)im);
  } else {
    const int64_t i = store_index(r.M, 0, r.n, k);
    const int64_t ps = r.M * STORE_KB;    // plane step within a K block
    if (r.f16) {
      __half* p = reinterpret_cast<__half*>(r.planes) + i;
      __half h, l;
      split_f16((float)re, h, l);
      p[0] = h;
      p[ps] = l;
      split_f16((float)im, h, l);
      p[2 * ps] = h;
      p[3 * ps] = l;
      return;
    }
    __nv_bfloat16 h, l;
    split_bf16((float)re, h, l);
    r.planes[i] = h;
    r.planes[i + ps] = l;
    split_bf16((float)im, h, l);
    r.planes[i + 2 * ps] = h;
    r.planes[i + 3 * ps] = l;
  }
}

// Two K-adjacent complex values (k even) into a BF16x3 store row: each
// plane gets one 4-byte bf16x2 (or half2) write; the same roundings as
// store_put.
__device__ __forceinline__ void store_put2_bf16x3(const StoreRow& r, int64_t k,
                                                  float re0, float im0,
                                                  float re1, float im1) {
  const int64_t i = store_index(r.M, 0, r.n, k);
  const int64_t ps = r.M * STORE_KB;
  const int64_t ps2 = ps / 2;
  if (r.f16) {
    __half2* q = reinterpret_cast<__half2*>(r.planes + i);
    const __half2 hr = __floats2half2_rn(re0, re1);
    const __half2 hi = __floats2half2_rn(im0, im1);
    q[0] = hr;
    q[ps2] = __floats2half2_rn(re0 - __low2float(hr), re1 - __high2float(hr));
    q[2 * ps2] = hi;
    q[3 * ps2] =
        __floats2half2_rn(im0 - __low2float(hi), im1 - __high2float(hi));
    return;
  }
  __nv_bfloat162* p = reinterpret_cast<__nv_bfloat162*>(r.planes + i);
  const __nv_bfloat162 hr = __floats2bfloat162_rn(re0, re1);
  const __nv_bfloat162 hi = __floats2bfloat162_rn(im0, im1);
  p[0] = hr;
  p[ps2] = __floats2bfloat162_rn(re0 - __low2float(hr), re1 - __high2float(hr));
  p[2 * ps2] = hi;
  p[3 * ps2] =
      __floats2bfloat162_rn(im0 - __low2float(hi), im1 - __high2float(hi));
}

int store_alloc(Store* s, int kind, int64_t M, int64_t K, cudaStream_t st);
void store_free(Store* s, cudaStream_t st);

// mu = Omega^* Psi^T / R  (M x M complex128 to the host); FP64 CUDA cores.
int gemm_fp64(kpm_handle* h, const Store* omega, const Store* psi, int64_t M,
              int64_t K, int64_t R, int per_vector, double* mu_host);
// Same contraction on BF16x3 stores (bfloat16 or FP16 planes): tensor cores
// (tcgen05), FP32 accumulation.
int gemm_bf16x3(kpm_handle* h, const Store* omega, const Store* psi,
                int64_t M, int64_t K, int64_t R, double* mu_host);
// CUDA-core evaluation of exactly the BF16x3 products (hi*hi + hi*lo +
// lo*hi, FP32 per-tile accumulation): the check for the tensor-core kernel.
int gemm_bf16x3_simt(kpm_handle* h, const Store* omega, const Store* psi,
                     int64_t M, int64_t K, int64_t R, double* mu_host);

}  // namespace kpm
