// Kubo-Bastin correlator moments on the device.
//
// Correlator.__init__ (kwant/kpm.py:557-606) runs two Chebyshev recursions
// and contracts their stored vectors:
//   Psi_n   = v_beta T_n(H~) |r>            (kwant/kpm.py:708-718)
//   Omega_m = T_m(H~') v_alpha |r>          (kwant/kpm.py:697-706, :603)
//   mu_mn   = mean_r <Omega_m | Psi_n>      (kwant/kpm.py:685-695)
// Here both recursions run batched over all R vectors; every step writes its
// vectors straight into a K-major store (row n = one Chebyshev order,
// K = orbital * R + vector), so the contraction is one "NT" GEMM over
// K = N R:  mu = Omega^* Psi^T / R.
//
// Stores and contractions:
//   FP64  : complex128 rows, FP64 CUDA-core GEMM (split-K, fixed-order
//           reduction).
//   BF16x3: each real component x stored as hi = bf16(x), lo = bf16(x - hi)
//           in four planes (re_hi, re_lo, im_hi, im_lo); the tensor-core GEMM
//           (kpm_gemm_tc.cu) forms hi*hi + hi*lo + lo*hi with FP32
//           accumulation.  FP16x3: the same with IEEE half parts (11
//           significant bits each instead of 8).

#include <cuda_bf16.h>

#include <cmath>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_gemm.cuh"

namespace kpm {

// Complex arithmetic in the recursion's precision: complex64 values, vectors
// and FP32 math in mixed mode (GB300's FP64 pipe is narrow), complex128 in
// FP64 mode.
template <bool MIXED> struct CT;
template <> struct CT<true> {
  using S = float;
  using V2 = float2;
  static __device__ __forceinline__ V2 make(S a, S b) {
    return make_float2(a, b);
  }
};
template <> struct CT<false> {
  using S = double;
  using V2 = double2;
  static __device__ __forceinline__ V2 make(S a, S b) {
    return make_double2(a, b);
  }
};

// y[i][r] = sum_j V_ij x[j][r], written to the K-major store row
// (K index i * R + r).  One thread per (row, vector); vectors fastest.
// V == nullptr copies x (the Omega side has no operator).
template <bool MIXED, int STORE>
__global__ void spmm_to_store_kernel(int64_t rows, int64_t R, int64_t Rpad,
                                     const int32_t* __restrict__ ip,
                                     const int32_t* __restrict__ ix,
                                     const void* __restrict__ vals,
                                     const void* __restrict__ x,
                                     StoreRow dst) {
  using S = typename CT<MIXED>::S;
  using V2 = typename CT<MIXED>::V2;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows * R) return;
  const int64_t i = idx / R, r = idx % R;
  const V2* __restrict__ X = reinterpret_cast<const V2*>(x);
  const V2* __restrict__ V = reinterpret_cast<const V2*>(vals);
  S yr = 0, yi = 0;
  if (V == nullptr) {
    const V2 a = X[i * Rpad + r];
    yr = a.x;
    yi = a.y;
  } else {
    for (int jj = ip[i]; jj < ip[i + 1]; ++jj) {
      const V2 h = V[jj];
      const V2 a = X[(int64_t)ix[jj] * Rpad + r];
      yr = fma(h.x, a.x, fma(-h.y, a.y, yr));
      yi = fma(h.x, a.y, fma(h.y, a.x, yi));
    }
  }
  store_put<STORE>(dst, idx, yr, yi);
}

// y[i][r] = sum_j V_ij x[j][r] in block layout (used for v_alpha |r>).
template <bool MIXED>
__global__ void spmm_block_kernel(int64_t rows, int64_t Rpad,
                                  const int32_t* __restrict__ ip,
                                  const int32_t* __restrict__ ix,
                                  const void* __restrict__ vals,
                                  const void* __restrict__ x, void* y) {
  using S = typename CT<MIXED>::S;
  using V2 = typename CT<MIXED>::V2;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows * Rpad) return;
  const int64_t i = idx / Rpad, r = idx % Rpad;
  const V2* __restrict__ X = reinterpret_cast<const V2*>(x);
  const V2* __restrict__ V = reinterpret_cast<const V2*>(vals);
  S yr = 0, yi = 0;
  for (int jj = ip[i]; jj < ip[i + 1]; ++jj) {
    const V2 h = V[jj];
    const V2 a = X[(int64_t)ix[jj] * Rpad + r];
    yr = fma(h.x, a.x, fma(-h.y, a.y, yr));
    yi = fma(h.x, a.y, fma(h.y, a.x, yi));
  }
  reinterpret_cast<V2*>(y)[idx] = CT<MIXED>::make(yr, yi);
}

template <int STORE>
static int put_row(kpm_handle* h, const Matrix* V, const void* x, int64_t N,
                   int64_t R, int64_t Rpad, StoreRow dst) {
  const int64_t n = N * R;
  const unsigned grid = (unsigned)ceil_div(n, 256);
  const bool mixed = h->precision == KPM_PREC_MIXED;
  const int32_t* ip = V ? V->indptr : nullptr;
  const int32_t* ix = V ? V->indices : nullptr;
  const void* vv = V ? V->data : nullptr;
  if (mixed)
    spmm_to_store_kernel<true, STORE><<<grid, 256, 0, h->stream>>>(
        N, R, Rpad, ip, ix, vv, x, dst);
  else
    spmm_to_store_kernel<false, STORE><<<grid, 256, 0, h->stream>>>(
        N, R, Rpad, ip, ix, vv, x, dst);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// Build a block whose starting vectors are already on the device.
static int block_from_device(kpm_handle* h, int64_t R, void* a0_owned,
                             kpm_block** out) {
  auto* b = new kpm_block();
  b->h = h;
  b->R = R;
  b->N = h->H.rows;
  const int G = group_size(h->precision, R);
  b->G = G;
  b->Rpad = round_up(R, G);
  b->groups = (int)(b->Rpad / G);
  b->keep_a0 = true;
  b->a0 = a0_owned;
  const size_t csz = h->precision == KPM_PREC_MIXED ? 8 : 16;
  const size_t vbytes = (size_t)b->N * b->Rpad * csz;
  int st = dev_alloc(&b->buf[0], vbytes, h->stream);
  if (st == KPM_OK) st = dev_alloc(&b->buf[1], vbytes, h->stream);
  if (st == KPM_OK)
    st = dev_alloc((void**)&b->mu01, (size_t)b->Rpad * 2 * 16, h->stream);
  if (st != KPM_OK) {
    kpm_block_destroy(b);
    return st;
  }
  b->p_cur = b->a0;
  *out = b;
  return KPM_OK;
}

// One order n of a stored recursion: alpha_n (advancing from alpha_{n-1}
// for n > 0) and its store row, launched on `stream` with the scale (a, b)
// of this recursion (the correlator's second recursion uses (a2, b2)).
template <int STORE>
static int recursion_order(kpm_block* b, const Matrix* V, int64_t n,
                           Store* store, double a, double bshift,
                           cudaStream_t stream) {
  kpm_handle* h = b->h;
  const double a_save = h->a, b_save = h->b;
  const cudaStream_t s_save = h->stream;
  h->a = a;
  h->b = bshift;
  h->stream = stream;
  int st = KPM_OK;
  if (n > 0) st = block_advance(b, false);
  if (st == KPM_OK)
    st = put_row<STORE>(h, V, b->p_cur, b->N, b->R, b->Rpad, store->row(n));
  h->a = a_save;
  h->b = b_save;
  h->stream = s_save;
  return st;
}

// Order n of a recursion with the store row of alpha_n written by the step
// that computes alpha_{n+1} (complex64 ELL handles, BF16x3 stores): V's
// product shares H's gathered rows, and no separate store launch is needed.
static int fused_order(kpm_block* b, const Matrix* V, int64_t n, Store* store,
                       double a, double bshift, cudaStream_t stream) {
  kpm_handle* h = b->h;
  const double a_save = h->a, b_save = h->b;
  const cudaStream_t s_save = h->stream;
  h->a = a;
  h->b = bshift;
  h->stream = stream;
  int st = block_advance_store(b, V ? 2 : 1, V ? V->ell_val : nullptr,
                               store->row(n), b->R);
  h->a = a_save;
  h->b = b_save;
  h->stream = s_save;
  return st;
}

// Both recursions of the correlator, interleaved order by order on two
// streams: each is a chain of small dependent launches (latency-bound at
// the sizes of the Kubo workload), and they are independent of each other.
// With `fused`, orders 0 .. M-2 store from inside the step kernels and only
// the last order uses the separate store kernel.
template <int STORE>
static int run_recursions(kpm_block* bR, const Matrix* Vb, Store* psi,
                          double a, double b, kpm_block* bL, Store* omega,
                          double a2, double b2, int64_t M,
                          cudaStream_t s2, bool fused) {
  int st = KPM_OK;
  if (fused) {
    for (int64_t n = 0; st == KPM_OK && n + 1 < M; ++n) {
      st = fused_order(bR, Vb, n, psi, a, b, bR->h->stream);
      if (st == KPM_OK) st = fused_order(bL, nullptr, n, omega, a2, b2, s2);
    }
    // last order: alpha_{M-1} is already computed; store it separately
    if (st == KPM_OK) {
      kpm_handle* h = bR->h;
      st = put_row<STORE>(h, Vb, bR->p_cur, bR->N, bR->R, bR->Rpad,
                          psi->row(M - 1));
      const cudaStream_t s_save = h->stream;
      h->stream = s2;
      if (st == KPM_OK)
        st = put_row<STORE>(h, nullptr, bL->p_cur, bL->N, bL->R, bL->Rpad,
                            omega->row(M - 1));
      h->stream = s_save;
    }
    return st;
  }
  for (int64_t n = 0; st == KPM_OK && n < M; ++n) {
    st = recursion_order<STORE>(bR, Vb, n, psi, a, b, bR->h->stream);
    if (st == KPM_OK)
      st = recursion_order<STORE>(bL, nullptr, n, omega, a2, b2, s2);
  }
  return st;
}

__global__ void ell_index_diff_kernel(const int32_t* __restrict__ a,
                                      const int32_t* __restrict__ b,
                                      int64_t n, int* __restrict__ diff) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && a[i] != b[i]) atomicExch(diff, 1);
}

// Does V's ELL copy line up entry for entry with H's (same widths, same
// column indices)?  Then V can share H's gathers.
static int ell_aligned(kpm_handle* h, const Matrix* V, bool* aligned) {
  *aligned = false;
  if (h->H.ell_k == 0 || V->ell_k != h->H.ell_k || !V->ell_val) return KPM_OK;
  int* diff = nullptr;
  KPM_TRY(dev_alloc((void**)&diff, sizeof(int), h->stream));
  const int64_t n = h->H.rows * (int64_t)h->H.ell_k;
  int hd = 1;
  cudaError_t e = cudaMemsetAsync(diff, 0, sizeof(int), h->stream);
  if (e == cudaSuccess) {
    ell_index_diff_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, h->stream>>>(
        h->H.ell_idx, V->ell_idx, n, diff);
    count_launch(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&hd, diff, sizeof(int), cudaMemcpyDeviceToHost,
                        h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dev_free(diff, h->stream);
  KPM_CUDA(e);
  *aligned = hd == 0;
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_correlator_moments(kpm_handle* h, double a2, double b2,
                           const kpm_csr_desc* v_alpha,
                           const kpm_csr_desc* v_beta, const double* vecs,
                           int64_t R, int64_t M, int gemm, int per_vector,
                           double* mu_out) {
  NvtxRange nvtx("kpm_correlator_moments");
  KPM_REQUIRE(h && v_alpha && v_beta && vecs && mu_out,
              "kpm_correlator_moments: null argument");
  KPM_REQUIRE(R > 0 && M >= 2, "kpm_correlator_moments: need R > 0, M >= 2");
  KPM_REQUIRE(v_alpha->rows == h->H.rows && v_beta->rows == h->H.rows,
              "kpm_correlator_moments: operator shape mismatch");
  KPM_REQUIRE(a2 > 0, "kpm_correlator_moments: a2 must be positive");
  if (gemm == 2) gemm = h->precision == KPM_PREC_MIXED ? 1 : 0;
  KPM_REQUIRE(gemm >= 0 && gemm <= 5 && gemm != 2,
              "kpm_correlator_moments: bad gemm");
  const bool simt = gemm == 3 || gemm == 5;   // CUDA-core split products
  const int f16 = gemm >= 4;                  // FP16 planes
  if (gemm != 0 && per_vector) {
    set_error("kpm_correlator_moments: per-vector moments need gemm=0");
    return KPM_EUNSUPPORTED;
  }
  const int64_t N = h->H.rows;
  const int64_t K = N * R;
  cudaStream_t s = h->stream;
  Matrix Va, Vb;
  kpm_block *bR = nullptr, *bL = nullptr;
  Store psi, omega;
  // operators in the recursion's precision (complex64 values in mixed mode)
  const double vscale = h->precision == KPM_PREC_MIXED ? 1.0 : 0.0;
  int st = upload_matrix_for(h, v_alpha, vscale, &Va, false);
  const int kind = gemm == 0 ? STORE_C128 : STORE_BF16X3;
  // complex64 + BF16x3: V_beta also as ELL, to share the step's gathers
  const bool want_fuse = h->precision == KPM_PREC_MIXED &&
                         kind == STORE_BF16X3 && h->H.ell_k > 0 &&
                         getenv("KPM_CORRELATOR_UNFUSED") == nullptr;
  if (st == KPM_OK)
    st = upload_matrix_for(h, v_beta, vscale, &Vb, want_fuse);
  bool fused = false;
  if (st == KPM_OK && want_fuse) st = ell_aligned(h, &Vb, &fused);
  if (st == KPM_OK) st = store_alloc(&psi, kind, M, K, s);
  if (st == KPM_OK) st = store_alloc(&omega, kind, M, K, s);
  psi.f16 = omega.f16 = f16;
  if (st == KPM_OK) st = kpm_block_create(h, vecs, R, 1, &bR);
  if (st == KPM_OK) st = timed_begin(h);
  // Omega's starting vectors v_alpha|r>
  if (st == KPM_OK) {
    const size_t csz = h->precision == KPM_PREC_MIXED ? 8 : 16;
    void* a0L = nullptr;
    st = dev_alloc(&a0L, (size_t)N * bR->Rpad * csz, s);
    if (st == KPM_OK) {
      const int64_t n = N * bR->Rpad;
      if (h->precision == KPM_PREC_MIXED)
        spmm_block_kernel<true><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(
            N, bR->Rpad, Va.indptr, Va.indices, Va.data, bR->a0, a0L);
      else
        spmm_block_kernel<false><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(
            N, bR->Rpad, Va.indptr, Va.indices, Va.data, bR->a0, a0L);
      count_launch(1);
      if (cudaGetLastError() != cudaSuccess) {
        set_error("kpm_correlator_moments: spmm launch failed");
        st = KPM_ECUDA;
      }
    }
    if (st == KPM_OK) st = block_from_device(h, R, a0L, &bL);
    else dev_free(a0L, s);
  }
  // Psi_n = v_beta T_n(H~)|r> on the handle's stream and Omega_m =
  // T_m(H~') v_alpha|r> on a second stream, interleaved
  cudaStream_t s2 = nullptr;
  cudaEvent_t ready = nullptr, done = nullptr;
  if (st == KPM_OK &&
      (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) !=
           cudaSuccess ||
       cudaEventCreateWithFlags(&done, cudaEventDisableTiming) !=
           cudaSuccess)) {
    set_error("kpm_correlator_moments: stream creation failed");
    st = KPM_ECUDA;
  }
  if (st == KPM_OK && (cudaEventRecord(ready, s) != cudaSuccess ||
                       cudaStreamWaitEvent(s2, ready, 0) != cudaSuccess)) {
    set_error("kpm_correlator_moments: stream ordering failed");
    st = KPM_ECUDA;
  }
  if (st == KPM_OK) {
    // complex64 values are pre-scaled by 2/a; a2 equals a up to rounding
    // (kwant/kpm.py:576-579), so in mixed mode only the diagonal shift of
    // the second recursion is re-derived.
    const double aL = h->precision == KPM_PREC_MIXED ? h->a : a2;
    st = kind == STORE_C128
             ? run_recursions<STORE_C128>(bR, &Vb, &psi, h->a, h->b, bL,
                                          &omega, aL, b2, M, s2, false)
             : run_recursions<STORE_BF16X3>(bR, &Vb, &psi, h->a, h->b, bL,
                                            &omega, aL, b2, M, s2, fused);
  }
  if (s2) {
    // the contraction (on the handle's stream) needs both stores
    if (cudaEventRecord(done, s2) != cudaSuccess ||
        cudaStreamWaitEvent(s, done, 0) != cudaSuccess) {
      if (st == KPM_OK) {
        set_error("kpm_correlator_moments: stream ordering failed");
        st = KPM_ECUDA;
      }
      cudaStreamSynchronize(s2);
    }
  }
  if (bL) {
    kpm_block_destroy(bL);   // frees on its handle's stream (after s2's work)
    bL = nullptr;
  }
  if (bR) {
    kpm_block_destroy(bR);
    bR = nullptr;
  }
  if (st == KPM_OK) {
    if (gemm == 0)
      st = gemm_fp64(h, &omega, &psi, M, K, R, per_vector, mu_out);
    else if (simt)
      st = gemm_bf16x3_simt(h, &omega, &psi, M, K, R, mu_out);
    else
      st = gemm_bf16x3(h, &omega, &psi, M, K, R, mu_out);
  }
  if (st == KPM_OK) st = timed_end(h);
  if (st == KPM_OK && f16) {
    // an FP16 part above 65504 becomes infinite: report it, with mu written
    for (int64_t i = 0; i < 2 * M * M; ++i)
      if (!std::isfinite(mu_out[i])) {
        set_error("kpm_correlator_moments: non-finite moments with FP16 "
                  "planes (a vector entry above the FP16 range); use the "
                  "bfloat16 or FP64 contraction");
        st = KPM_EDIVERGED;
        break;
      }
  }
  if (bR) kpm_block_destroy(bR);
  store_free(&psi, s);
  store_free(&omega, s);
  free_matrix(&Va, s);
  free_matrix(&Vb, s);
  cudaStreamSynchronize(s);
  if (s2) {
    cudaStreamSynchronize(s2);
    cudaStreamDestroy(s2);
  }
  if (ready) cudaEventDestroy(ready);
  if (done) cudaEventDestroy(done);
  if (st == KPM_OK) st = check_bounds(h, "kpm_correlator_moments");
  return st;
}

}  // extern "C"
