// Complex64 Chebyshev step on an ELL copy of the Hamiltonian.
//
// Same arithmetic as the complex64 branch of cheb_step_kernel (kpm_core.cu),
// entry for entry and in the same order (ELL padding adds 0 * x exactly, and
// the FP32 -> FP64 flush points and the reduction order are unchanged), so
// results are bit-identical; it differs only in how it feeds the memory
// system.  A row's column indices and values are fetched with 16-byte loads
// that do not depend on a row-pointer load, and the row's own vector entry
// and its alpha_{n-1} entry are requested together with them: every row
// costs two dependent memory round trips instead of four.  RPI rows per
// iteration overlap those round trips across rows; the FP64 dot-product
// accumulators live in shared memory to keep registers (and so occupancy)
// low.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// Blocks per SM the register budget is sized for (narrow rows need few
// registers; 6 x 256 threads leaves 40 registers per thread).
#ifndef KPM_ELL_MIN_BLOCKS
#define KPM_ELL_MIN_BLOCKS 5
#endif
template <int K, int RPI>
constexpr int ell_min_blocks() {
  return (K <= 4 && RPI == 1) ? KPM_ELL_MIN_BLOCKS : 1;
}

template <int K, int MODE, bool DOTS, int RPI>
__global__ void __launch_bounds__(STEP_THREADS, ell_min_blocks<K, RPI>())
cheb_step_ell_kernel(StepArgs p, const int32_t* __restrict__ eidx,
                     const float2* __restrict__ eval) {
  constexpr int G = GROUP_FP32;
  constexpr int KQ = K / 4;
  const int lane = threadIdx.x & (LANES - 1);
  const int slot = threadIdx.x / LANES;
  // FP64 accumulators of this slot's lanes, then the in-block reduction
  __shared__ double red[DOTS ? SLOTS : 1][DOTS ? G * 3 : 1];

  const float4* __restrict__ x = reinterpret_cast<const float4*>(p.x);
  const float4* prev = reinterpret_cast<const float4*>(p.prev);
  float4* out = reinterpret_cast<float4*>(p.out);
  const int64_t work = (int64_t)p.xitems * p.groups;
  const int64_t stride = (int64_t)p.xitems * SLOTS;
  const float shift = p.shift;
  constexpr int FLUSH = 32;

  for (int64_t w = blockIdx.x; w < work; w += gridDim.x) {
    const int xi = (int)(w / p.groups);
    const int g = (int)(w - (int64_t)xi * p.groups);
    const int64_t col = (int64_t)g * LANES + lane;
    double* my = DOTS ? &red[slot][lane * 2 * 3] : nullptr;
    if constexpr (DOTS) {
#pragma unroll
      for (int e = 0; e < 6; ++e) my[e] = 0.0;
    }
    float fn0 = 0.f, fn1 = 0.f, fr0 = 0.f, fr1 = 0.f, fi0 = 0.f, fi1 = 0.f;
    int pending = 0;

    for (int64_t i0 = (int64_t)xi * SLOTS + slot; i0 < p.rows;
         i0 += RPI * stride) {
      int64_t row[RPI];
      bool ok[RPI];
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        row[u] = i0 + u * stride;
        ok[u] = row[u] < p.rows;
      }
      float4 xv[RPI], pv[RPI];
      int4 c4[RPI][KQ];
      float4 hv[RPI][2 * KQ];
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        if (!ok[u]) continue;
        const int64_t r = row[u];
        xv[u] = x[r * p.rp + col];
        if constexpr (MODE == STEP_RECUR) pv[u] = prev[r * p.rp + col];
        const int4* ri = reinterpret_cast<const int4*>(eidx + r * K);
        const float4* rv = reinterpret_cast<const float4*>(eval + r * K);
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
          c4[u][q] = __ldg(ri + q);
          hv[u][2 * q] = __ldg(rv + 2 * q);
          hv[u][2 * q + 1] = __ldg(rv + 2 * q + 1);
        }
      }
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        if (!ok[u]) continue;
        float a0r = shift * xv[u].x, a0i = shift * xv[u].y;
        float a1r = shift * xv[u].z, a1i = shift * xv[u].w;
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
          const int cc[4] = {c4[u][q].x, c4[u][q].y, c4[u][q].z, c4[u][q].w};
          float4 xx[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) xx[t] = x[(int64_t)cc[t] * p.rp + col];
          const float hr[4] = {hv[u][2 * q].x, hv[u][2 * q].z,
                               hv[u][2 * q + 1].x, hv[u][2 * q + 1].z};
          const float hi[4] = {hv[u][2 * q].y, hv[u][2 * q].w,
                               hv[u][2 * q + 1].y, hv[u][2 * q + 1].w};
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            a0r = fmaf(hr[t], xx[t].x, a0r);
            a0r = fmaf(-hi[t], xx[t].y, a0r);
            a0i = fmaf(hr[t], xx[t].y, a0i);
            a0i = fmaf(hi[t], xx[t].x, a0i);
            a1r = fmaf(hr[t], xx[t].z, a1r);
            a1r = fmaf(-hi[t], xx[t].w, a1r);
            a1i = fmaf(hr[t], xx[t].w, a1i);
            a1i = fmaf(hi[t], xx[t].z, a1i);
          }
        }
        float4 o;
        if constexpr (MODE == STEP_FIRST) {
          o = make_float4(0.5f * a0r, 0.5f * a0i, 0.5f * a1r, 0.5f * a1i);
        } else {
          o = make_float4(a0r - pv[u].x, a0i - pv[u].y, a1r - pv[u].z,
                          a1i - pv[u].w);
        }
        out[row[u] * p.rp + col] = o;
        if constexpr (DOTS) {
          const float4 v = xv[u];
          fn0 = fmaf(v.x, v.x, fmaf(v.y, v.y, fn0));
          fn1 = fmaf(v.z, v.z, fmaf(v.w, v.w, fn1));
          fr0 = fmaf(o.x, v.x, fmaf(o.y, v.y, fr0));
          fr1 = fmaf(o.z, v.z, fmaf(o.w, v.w, fr1));
          fi0 = fmaf(o.x, v.y, fmaf(-o.y, v.x, fi0));
          fi1 = fmaf(o.z, v.w, fmaf(-o.w, v.z, fi1));
          if (++pending == FLUSH) {
            my[0] += (double)fn0;
            my[1] += (double)fr0;
            my[2] += (double)fi0;
            my[3] += (double)fn1;
            my[4] += (double)fr1;
            my[5] += (double)fi1;
            fn0 = fn1 = fr0 = fr1 = fi0 = fi1 = 0.f;
            pending = 0;
          }
        }
      }
    }
    if constexpr (DOTS) {
      my[0] += (double)fn0;
      my[1] += (double)fr0;
      my[2] += (double)fi0;
      my[3] += (double)fn1;
      my[4] += (double)fr1;
      my[5] += (double)fi1;
      __syncthreads();
      // layout [group][vector*3 + component][partition]: the finalize
      // kernel reads each vector's partitions contiguously
      double* dst = p.partials + (int64_t)g * (G * 3) * p.xitems + xi;
      for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < SLOTS; ++q) s += red[q][e];
        dst[(int64_t)e * p.xitems] = s;
      }
      __syncthreads();
    }
  }
}

template <int K, int MODE, bool DOTS, int RPI>
static int launch_ell_t(kpm_handle* h, const StepArgs& a) {
  static int occ = -1;
  if (occ < 0) {
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, cheb_step_ell_kernel<K, MODE, DOTS, RPI>, STEP_THREADS, 0));
    occ = blocks > 0 ? blocks : 1;
  }
  const int64_t work = (int64_t)a.xitems * a.groups;
  int64_t grid = (int64_t)occ * h->num_sms;
  if (grid > work) grid = work;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->profiling) {
    while (h->prof_events.size() < h->prof_used + 2) {
      cudaEvent_t e;
      KPM_CUDA(cudaEventCreate(&e));
      h->prof_events.push_back(e);
    }
    e0 = h->prof_events[h->prof_used];
    e1 = h->prof_events[h->prof_used + 1];
    h->prof_used += 2;
    KPM_CUDA(cudaEventRecord(e0, h->stream));
  }
  cheb_step_ell_kernel<K, MODE, DOTS, RPI>
      <<<(unsigned)grid, STEP_THREADS, 0, h->stream>>>(a, h->H.ell_idx,
                                                        h->H.ell_val);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (e1) KPM_CUDA(cudaEventRecord(e1, h->stream));
  return KPM_OK;
}

template <int K, int RPI>
static int dispatch_mode(kpm_handle* h, int mode, bool dots,
                         const StepArgs& a) {
  if (mode == STEP_FIRST)
    return dots ? launch_ell_t<K, STEP_FIRST, true, RPI>(h, a)
                : launch_ell_t<K, STEP_FIRST, false, RPI>(h, a);
  return dots ? launch_ell_t<K, STEP_RECUR, true, RPI>(h, a)
              : launch_ell_t<K, STEP_RECUR, false, RPI>(h, a);
}

template <int RPI>
static int dispatch_k(kpm_handle* h, int mode, bool dots, const StepArgs& a) {
  switch (h->H.ell_k) {
    case 4: return dispatch_mode<4, RPI>(h, mode, dots, a);
    case 8: return dispatch_mode<8, RPI>(h, mode, dots, a);
    case 12: return dispatch_mode<12, RPI>(h, mode, dots, a);
    case 16: return dispatch_mode<16, RPI>(h, mode, dots, a);
  }
  set_error("ELL width %d not supported", h->H.ell_k);
  return KPM_EUNSUPPORTED;
}

int launch_step_ell(kpm_handle* h, int mode, bool dots, const StepArgs& a) {
  if (h->step_rpi == 2) return dispatch_k<2>(h, mode, dots, a);
  return dispatch_k<1>(h, mode, dots, a);
}

}  // namespace kpm
