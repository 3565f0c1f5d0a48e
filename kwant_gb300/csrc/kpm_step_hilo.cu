// Compensated complex64 Chebyshev step of the DOS recursion (mixed
// precision, ELL copy of the Hamiltonian).
//
// Why: the DOS path computes two moments per matvec with the doubling
// identities mu_2n = 2<a_n|a_n> - mu_0 and mu_2n+1 = 2<a_n+1|a_n> - mu_1
// (kwant/kpm.py:464-473).  An error r_k injected into a_k propagates as
// U_{n-k}(H) r_k, and T_n U_{n-k} = (U_{2n-k} - U_{k-2}) / 2 has a part that
// does not depend on n: every rounding of a stored vector shifts ALL later
// even moments by the same amount.  With plain complex64 vectors those
// shifts random-walk in n, and the DCT reconstruction sums them coherently
// where 1/sqrt(1 - x^2) is largest (the outermost Chebyshev nodes): the
// per-orbital DOS there was off by ~2e-4 on the 2e6-orbital graphene
// workload.  The same holds for any error common to all moments: mu_0 and
// mu_1 themselves, and a bias of FP32 sums of |a_i|^2 (~1e-9 relative).
//
// What: every vector element is stored as a complex64 "hi" part plus a
// bfloat16 "lo" correction (4 more bytes per complex element, in a separate
// [row][vector] array), and each step computes a_{n+1} = 2H~ a_n - a_{n-1}
// to ~2^-38 relative with error-free FP32 transformations before splitting
// it again:
//   * the hi products h * x_hi are accumulated from an anchor C = 32: every
//     partial sum stays within a factor two of the previous one, so
//     s1 = fma(h, x, s), m = s - s1 (exact, Sterbenz) and e = fma(h, x, m)
//     give the rounding error of each fused multiply-add exactly; the errors
//     are summed in FP32 (they are ~2^-19 each);
//   * the lo products h * x_lo (and the lo part of a_{n-1}) are one FP32
//     sum: a 2^-24 error on a 2^-24-relative quantity;
//   * hi = RN(v), lo = RZ_bf16(RZ(v - hi)): round toward zero keeps |lo| at
//     most half an ulp of hi, so the split is unique and a vector downloaded
//     as complex128 (hi + lo, exact) uploads to the same hi and lo.
// The fused dot products use the hi parts: mu_0 and mu_1 in FP64 from hi+lo
// (once), then <a_n|a_n> and Re <a_n+1|a_n> with Ogita-Rump-Oishi Dot2
// (TwoProd + TwoSum, flushed to FP64 every 32 rows) and Im <a_n+1|a_n> as a
// plain FP32 sum.  Leaving out lo in these dots is a zero-mean error of
// each moment alone, not a shift of all of them.
//
// The H values themselves stay complex64 (2H/a): rounding them perturbs the
// Hamiltonian, whose moments are still those of a Hermitian operator, and
// leaves the reconstruction consistent (a ~1e-7 relative shift of the
// spectrum, not noise).

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// anchor of the compensated row sums (partial sums within C/2 of it keep
// the captured rounding errors exact; larger ones lose the compensation
// gracefully, not the hi part)
constexpr float HILO_ANCHOR = 32.0f;

__device__ __forceinline__ float bf_re(uint32_t w) {
  return __uint_as_float(w << 16);
}
__device__ __forceinline__ float bf_im(uint32_t w) {
  return __uint_as_float(w & 0xffff0000u);
}
// truncate two floats to bfloat16 (round toward zero): re in the low half
__device__ __forceinline__ uint32_t bf_pack_rz(float re, float im) {
  return __byte_perm(__float_as_uint(re), __float_as_uint(im), 0x7632);
}

// s + a*b with its rounding error added to c (exact while s stays within a
// factor two of the anchor).  Intrinsics: nothing may be contracted or
// reassociated here.
__device__ __forceinline__ void acc_fma(float& s, float& c, float a, float b) {
  const float s1 = __fmaf_rn(a, b, s);
  const float m = __fsub_rn(s, s1);
  c = __fadd_rn(c, __fmaf_rn(a, b, m));
  s = s1;
}
// s - b with its rounding error added to c
__device__ __forceinline__ void acc_sub(float& s, float& c, float b) {
  const float s1 = __fsub_rn(s, b);
  const float m = __fsub_rn(s, s1);
  c = __fadd_rn(c, __fsub_rn(m, b));
  s = s1;
}
// Dot2 accumulation (TwoProd + TwoSum) of a*b into (s, c)
__device__ __forceinline__ void dot2(float& s, float& c, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float pe = __fmaf_rn(a, b, -p);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c = __fadd_rn(c, __fadd_rn(e, pe));
}

// The step over 16-vector sub-groups in 8-lane slots whose lanes hold two
// complex64 vectors each (a float4 of hi parts, a uint2 of lo parts).
// MODE STEP_FIRST: a_1 = H~ a_0 with the FP64 dots mu_0 = <a_0|a_0> and
// <a_1|a_0>; STEP_RECUR: a_{n+1} = 2 H~ a_n - a_{n-1} with the compensated
// dots <a_n|a_n>, <a_n+1|a_n>.
template <int K, int MODE>
__global__ void __launch_bounds__(STEP_THREADS)
cheb_step_hilo_kernel(StepArgs p, HiloArgs q,
                      const int32_t* __restrict__ eidx,
                      const float2* __restrict__ eval) {
  constexpr int SW = 8;
  constexpr int VPL = 2;
  constexpr int G = SW * VPL;
  constexpr int KQ = K / 4;
  constexpr int SPW = 32 / SW;
  constexpr int NSLOT = STEP_THREADS / SW;
  constexpr int FLUSH = 32;
  const int lane = threadIdx.x & (SW - 1);
  const int slot = threadIdx.x / SW;
  const int wq = slot / SPW, half = slot % SPW, wl = threadIdx.x & 31;
  __shared__ double red[NSLOT][G * 3];
  __shared__ __align__(16) int32_t sidx[STEP_THREADS / 32][2][SPW * K];
  __shared__ __align__(16) float2 sval[STEP_THREADS / 32][2][SPW * K];

  const float4* __restrict__ x = reinterpret_cast<const float4*>(p.x);
  const float4* prev = reinterpret_cast<const float4*>(p.prev);
  float4* out = reinterpret_cast<float4*>(p.out);
  const uint2* __restrict__ xl = reinterpret_cast<const uint2*>(q.xlo);
  const uint2* pl = reinterpret_cast<const uint2*>(q.plo);
  uint2* ol = reinterpret_cast<uint2*>(q.olo);
  const int work = p.xitems * p.groups;
  const int rows = (int)p.rows;
  const int stride = p.xitems * NSLOT;
  const float shift = p.shift;
  const float C = HILO_ANCHOR;

  auto stage = [&](int r0, int b) {
    constexpr int IC = SPW * K / 4, VC = SPW * K / 2;
    for (int c = wl; c < IC + VC; c += 32) {
      if (c < IC) {
        if (r0 + (4 * c) / K < rows)
          cp_async16(&sidx[wq][b][4 * c], eidx + (int64_t)r0 * K + 4 * c);
      } else {
        const int e = c - IC;
        if (r0 + (2 * e) / K < rows)
          cp_async16(&sval[wq][b][2 * e], eval + (int64_t)r0 * K + 2 * e);
      }
    }
  };

  for (int w = blockIdx.x; w < work; w += gridDim.x) {
    const int xi = w / p.groups;
    const int g = w - xi * p.groups;
    const int col = g * SW + lane;
    double* my = &red[slot][lane * VPL * 3];
#pragma unroll
    for (int e = 0; e < VPL * 3; ++e) my[e] = 0.0;
    // compensated FP32 dot accumulators (STEP_RECUR)
    float sn[VPL], cn[VPL], sr[VPL], cr[VPL], fi[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) sn[k] = cn[k] = sr[k] = cr[k] = fi[k] = 0.f;
    int pending = 0;

    const int wb0 = xi * NSLOT + SPW * wq;
    if (wb0 < rows) stage(wb0, 0);
    cp_async_commit();
    int sb = 0;
    for (int wb = wb0; wb < rows; wb += stride) {
      if (wb + stride < rows) stage(wb + stride, sb ^ 1);
      cp_async_commit();
      cp_async_wait_prev();
      __syncwarp();
      const int64_t r = wb + half;
      if (r < rows) {
        const float4 xv = x[r * p.rp + col];
        const uint2 xlv = xl[r * q.lrp + col];
        float4 pv = make_float4(0.f, 0.f, 0.f, 0.f);
        uint2 plv = make_uint2(0u, 0u);
        if constexpr (MODE == STEP_RECUR) {
          pv = prev[r * p.rp + col];
          plv = pl[r * q.lrp + col];
        }
        const int4* ri =
            reinterpret_cast<const int4*>(&sidx[wq][sb][half * K]);
        const float4* rv =
            reinterpret_cast<const float4*>(&sval[wq][sb][half * K]);
        const float xr[2] = {xv.x, xv.z}, xim[2] = {xv.y, xv.w};
        const uint32_t xw[2] = {xlv.x, xlv.y};
        float s_r[2], c_r[2], s_i[2], c_i[2], l_r[2], l_i[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          s_r[k] = s_i[k] = C;
          c_r[k] = c_i[k] = 0.f;
          acc_fma(s_r[k], c_r[k], shift, xr[k]);
          acc_fma(s_i[k], c_i[k], shift, xim[k]);
          l_r[k] = __fmul_rn(shift, bf_re(xw[k]));
          l_i[k] = __fmul_rn(shift, bf_im(xw[k]));
        }
#pragma unroll
        for (int qq = 0; qq < KQ; ++qq) {
          const int4 c4 = ri[qq];
          const float4 h01 = rv[2 * qq], h23 = rv[2 * qq + 1];
          const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
          const float hr[4] = {h01.x, h01.z, h23.x, h23.z};
          const float hi[4] = {h01.y, h01.w, h23.y, h23.w};
          float4 xx[4];
          uint2 xxl[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            xx[t] = x[(int64_t)cc[t] * p.rp + col];
            xxl[t] = xl[(int64_t)cc[t] * q.lrp + col];
          }
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const float gr[2] = {xx[t].x, xx[t].z};
            const float gi[2] = {xx[t].y, xx[t].w};
            const uint32_t gw[2] = {xxl[t].x, xxl[t].y};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              acc_fma(s_r[k], c_r[k], hr[t], gr[k]);
              acc_fma(s_r[k], c_r[k], -hi[t], gi[k]);
              acc_fma(s_i[k], c_i[k], hr[t], gi[k]);
              acc_fma(s_i[k], c_i[k], hi[t], gr[k]);
              const float lr = bf_re(gw[k]), li = bf_im(gw[k]);
              l_r[k] = __fmaf_rn(hr[t], lr, __fmaf_rn(-hi[t], li, l_r[k]));
              l_i[k] = __fmaf_rn(hr[t], li, __fmaf_rn(hi[t], lr, l_i[k]));
            }
          }
        }
        float orr[2], oii[2], olr[2], oli[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if constexpr (MODE == STEP_RECUR) {
            const float pr[2] = {pv.x, pv.z}, pim[2] = {pv.y, pv.w};
            const uint32_t pw[2] = {plv.x, plv.y};
            acc_sub(s_r[k], c_r[k], pr[k]);
            acc_sub(s_i[k], c_i[k], pim[k]);
            l_r[k] = __fsub_rn(l_r[k], bf_re(pw[k]));
            l_i[k] = __fsub_rn(l_i[k], bf_im(pw[k]));
          }
          // v = (s - C) + (c + l): hi = RN(v), lo = RZ(v - hi)
          const float v0r = __fsub_rn(s_r[k], C), v0i = __fsub_rn(s_i[k], C);
          const float tr = __fadd_rn(c_r[k], l_r[k]);
          const float ti = __fadd_rn(c_i[k], l_i[k]);
          float hr_ = __fadd_rn(v0r, tr), hi_ = __fadd_rn(v0i, ti);
          float lr_ = __fadd_rz(__fsub_rn(v0r, hr_), tr);
          float li_ = __fadd_rz(__fsub_rn(v0i, hi_), ti);
          if constexpr (MODE == STEP_FIRST) {  // a_1 = (2 H~ a_0) / 2
            hr_ *= 0.5f;
            hi_ *= 0.5f;
            lr_ *= 0.5f;
            li_ *= 0.5f;
          }
          orr[k] = hr_;
          oii[k] = hi_;
          olr[k] = lr_;
          oli[k] = li_;
        }
        const uint32_t ow[2] = {bf_pack_rz(olr[0], oli[0]),
                                bf_pack_rz(olr[1], oli[1])};
        out[r * p.rp + col] = make_float4(orr[0], oii[0], orr[1], oii[1]);
        ol[r * q.lrp + col] = make_uint2(ow[0], ow[1]);
        if constexpr (MODE == STEP_FIRST) {
          // mu_0 and <a_1|a_0> in FP64 from hi + lo
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const double ar = (double)xr[k] + (double)bf_re(xw[k]);
            const double ai = (double)xim[k] + (double)bf_im(xw[k]);
            const double br = (double)orr[k] + (double)bf_re(ow[k]);
            const double bi = (double)oii[k] + (double)bf_im(ow[k]);
            my[k * 3 + 0] += ar * ar + ai * ai;
            my[k * 3 + 1] += br * ar + bi * ai;
            my[k * 3 + 2] += br * ai - bi * ar;
          }
        } else {
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            dot2(sn[k], cn[k], xr[k], xr[k]);
            dot2(sn[k], cn[k], xim[k], xim[k]);
            dot2(sr[k], cr[k], orr[k], xr[k]);
            dot2(sr[k], cr[k], oii[k], xim[k]);
            fi[k] = fmaf(orr[k], xim[k], fmaf(-oii[k], xr[k], fi[k]));
          }
          if (++pending == FLUSH) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              my[k * 3 + 0] += (double)sn[k] + (double)cn[k];
              my[k * 3 + 1] += (double)sr[k] + (double)cr[k];
              my[k * 3 + 2] += (double)fi[k];
              sn[k] = cn[k] = sr[k] = cr[k] = fi[k] = 0.f;
            }
            pending = 0;
          }
        }
      }
      __syncwarp();
      sb ^= 1;
    }
    if constexpr (MODE == STEP_RECUR) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        my[k * 3 + 0] += (double)sn[k] + (double)cn[k];
        my[k * 3 + 1] += (double)sr[k] + (double)cr[k];
        my[k * 3 + 2] += (double)fi[k];
      }
    }
    __syncthreads();
    // partials are addressed by vector: [vector*3 + component][xitems]
    double* dst = p.partials + (int64_t)g * (G * 3) * p.xitems + xi;
    for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int sl = 0; sl < NSLOT; ++sl) s += red[sl][e];
      dst[(int64_t)e * p.xitems] = s;
    }
    __syncthreads();
  }
}

template <int K, int MODE>
static int launch_hilo_t(kpm_handle* h, const StepArgs& a,
                         const HiloArgs& q) {
  static int occ = -1;
  if (occ < 0) {
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, cheb_step_hilo_kernel<K, MODE>, STEP_THREADS, 0));
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
  cheb_step_hilo_kernel<K, MODE>
      <<<(unsigned)grid, STEP_THREADS, 0, h->stream>>>(a, q, h->H.ell_idx,
                                                        h->H.ell_val);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (e1) KPM_CUDA(cudaEventRecord(e1, h->stream));
  return KPM_OK;
}

template <int K>
static int dispatch_hilo_k(kpm_handle* h, int mode, const StepArgs& a,
                           const HiloArgs& q) {
  return mode == STEP_FIRST ? launch_hilo_t<K, STEP_FIRST>(h, a, q)
                            : launch_hilo_t<K, STEP_RECUR>(h, a, q);
}

// Every block runs as 16-vector sub-groups in 8-lane slots with two
// vectors per lane (a 32-vector group is two sub-groups: the partials are
// addressed by vector, [vector*3 + component][xitems], so the sub-groups
// write exactly the group's entries).  Each vector thus sees the same row
// partition, slot and flush points whatever its block's group size, and
// add_vectors stays bit-identical to a fresh run.
int launch_step_hilo(kpm_handle* h, int mode, const StepArgs& a,
                     const HiloArgs& q) {
  if (mode != STEP_FIRST && mode != STEP_RECUR) {
    set_error("compensated step: unsupported mode %d", mode);
    return KPM_EINVAL;
  }
  const int64_t rpad = a.vpl == 2 ? 2 * a.rp : a.rp;  // complex64 per row
  StepArgs w = a;
  w.vpl = 2;
  w.rp = rpad / 2;
  w.groups = (int)(rpad / 16);
  HiloArgs wq = q;
  wq.lrp = rpad / 2;
  switch (h->H.ell_k) {
    case 4: return dispatch_hilo_k<4>(h, mode, w, wq);
    case 8: return dispatch_hilo_k<8>(h, mode, w, wq);
    case 12: return dispatch_hilo_k<12>(h, mode, w, wq);
    case 16: return dispatch_hilo_k<16>(h, mode, w, wq);
  }
  set_error("ELL width %d not supported", h->H.ell_k);
  return KPM_EUNSUPPORTED;
}

}  // namespace kpm
