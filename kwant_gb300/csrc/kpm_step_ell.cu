// Complex64 Chebyshev step on an ELL copy of the Hamiltonian.
//
// Every row gets the products of the complex64 branch of cheb_step_kernel
// (kpm_core.cu), entry for entry and in the same order (ELL padding adds
// 0 * x exactly), so the Chebyshev vectors are bit-identical to it; the
// fused DOS dot products are accumulated per 8-lane slot, which groups the
// rows of each FP32 partial differently from the CSR kernel (a fixed order,
// the same for every vector whatever its group size).
//
// A slot is 8 lanes with two (16-vector groups) or four (32-vector groups)
// complex64 vectors per lane: 128 or 256 bytes per row, and four rows in
// flight per warp (the correlator's store steps on 16-vector blocks: 4
// lanes of four vectors, eight rows per warp).  The column indices and
// values of a warp's next rows are copied into shared memory with cp.async
// (16-byte chunks, no row-pointer load) while the current ones compute, so
// a row's gathers go out together with its own vector entry and its
// alpha_{n-1} entry: one dependent memory round trip per row (a CSR row
// costs four).  The FP64
// dot-product accumulators live in shared memory to keep registers (and so
// occupancy) low.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// Blocks per SM the register budget is sized for: 4 x 256 threads leaves
// 64 registers per thread, which the variants in use fit without spilling
// (at 5 blocks, 48 registers, the fused-dots step spills and runs 1.6x
// slower).
#ifndef KPM_ELL_MIN_BLOCKS
#define KPM_ELL_MIN_BLOCKS 4
#endif
// Lanes per row of the store steps of 16-vector blocks: 4 (four vectors
// per lane, eight rows per warp) or 8 (two vectors per lane, four rows).
// Measured on the Kubo workload (Rashba square 200 x 200 x 2 orbitals,
// R = 16, M = 256): 9.19 ms per conductivity with 4, 9.62 ms with 8; a
// grid of one block per row group instead of resident blocks looping over
// them: 9.37 and 10.59 ms.
#ifndef KPM_STORE_SW
#define KPM_STORE_SW 4
#endif

template <int K, int RPI>
constexpr int ell_min_blocks() {
  return RPI != 1 ? 1 : KPM_ELL_MIN_BLOCKS;
}

template <int VPL> struct EllPay;
template <> struct EllPay<2> {
  using T = float4;
  __device__ static float re(const float4& v, int k) { return k ? v.z : v.x; }
  __device__ static float im(const float4& v, int k) { return k ? v.w : v.y; }
  __device__ static float4 make(const float (&r)[2], const float (&i)[2]) {
    return make_float4(r[0], i[0], r[1], i[1]);
  }
};
struct alignas(32) F8 {
  float4 a, b;
};
template <> struct EllPay<4> {
  using T = F8;
  __device__ static float re(const F8& v, int k) {
    const float4& h = k < 2 ? v.a : v.b;
    return (k & 1) ? h.z : h.x;
  }
  __device__ static float im(const F8& v, int k) {
    const float4& h = k < 2 ? v.a : v.b;
    return (k & 1) ? h.w : h.y;
  }
  __device__ static F8 make(const float (&r)[4], const float (&i)[4]) {
    return F8{make_float4(r[0], i[0], r[1], i[1]),
              make_float4(r[2], i[2], r[3], i[3])};
  }
};

// VPL complex64 vectors per lane of an SW-lane slot: 2 (groups of 16
// vectors) or 4 (groups of 32); every vector gets the same FMA sequence
// either way.
// SM (store mode, the correlator's recursions): 1 also writes alpha_n (the
// input x) into the BF16x3 store row, 2 writes V alpha_n, with V's entries
// in an ELL copy aligned with H's, so that V shares H's gathered rows; the
// products follow the separate store kernel's operation order.
// RPI (rows per slot iteration) is 1 in every launch.  The per-row arrays
// stay: rewriting them as scalars changed the compiler's load schedule and
// made the fused-dots step 25 % slower (0.563 -> 0.702 ms on the 2e6-orbital
// graphene workload) at the same register count.
template <int K, int MODE, bool DOTS, int RPI, int VPL, int SM = 0,
          int SW = 8>
__global__ void __launch_bounds__(STEP_THREADS, ell_min_blocks<K, RPI>())
cheb_step_ell_kernel(StepArgs p, const int32_t* __restrict__ eidx,
                     const float2* __restrict__ eval, StoreArgs sa) {
  static_assert(SM == 0 || (!DOTS && RPI == 1), "store fusion: no dots");
  static_assert(SW == 4 || SW == 8 || SW == 16, "4-, 8- or 16-lane slots");
  using Pay = EllPay<VPL>;
  using PT = typename Pay::T;
  constexpr int G = SW * VPL;
  constexpr int KQ = K / 4;
  constexpr int SPW = 32 / SW;                // slots per warp
  constexpr int NSLOT = STEP_THREADS / SW;    // slots per block
  const int lane = threadIdx.x & (SW - 1);
  const int slot = threadIdx.x / SW;
  const int wq = slot / SPW, half = slot % SPW, wl = threadIdx.x & 31;
  // FP64 accumulators of this slot's lanes, then the in-block reduction
  __shared__ double red[DOTS ? NSLOT : 1][DOTS ? G * 3 : 1];
  // ELL entries of each warp's next SPW rows (per row-per-iteration u),
  // double-buffered
  __shared__ __align__(16) int32_t sidx[STEP_THREADS / 32][2][RPI][SPW * K];
  __shared__ __align__(16) float2 sval[STEP_THREADS / 32][2][RPI][SPW * K];

  const PT* __restrict__ x = reinterpret_cast<const PT*>(p.x);
  const PT* prev = reinterpret_cast<const PT*>(p.prev);
  PT* out = reinterpret_cast<PT*>(p.out);
  const int work = p.xitems * p.groups;
  // the next store step may launch now: its blocks take the SM slots this
  // grid frees and stage their first rows while this grid finishes
  if constexpr (SM != 0)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // row counters in 32 bits (CSR indices are int32); addresses in 64
  const int rows = (int)p.rows;
  const int stride = p.xitems * NSLOT;
  const float shift = p.shift;
  constexpr int FLUSH = 32;

  // Copy the entries of rows r0 + h + u * stride (h < SPW, u < RPI) into
  // stage buffer b: 16-byte chunks, the rows' indices then their values.
  auto stage = [&](int r0, int b) {
    constexpr int IC = SPW * K / 4, VC = SPW * K / 2;
    for (int c = wl; c < RPI * (IC + VC); c += 32) {
      const int u = c / (IC + VC), d = c % (IC + VC);
      const int base = r0 + u * stride;
      if (d < IC) {
        if (base + (4 * d) / K < rows)
          cp_async16(&sidx[wq][b][u][4 * d],
                     eidx + (int64_t)base * K + 4 * d);
      } else {
        const int e = d - IC;
        if (base + (2 * e) / K < rows)
          cp_async16(&sval[wq][b][u][2 * e],
                     eval + (int64_t)base * K + 2 * e);
      }
    }
  };

  for (int w = blockIdx.x; w < work; w += gridDim.x) {
    const int xi = w / p.groups;
    const int g = w - xi * p.groups;
    const int col = g * SW + lane;
    double* my = DOTS ? &red[slot][lane * VPL * 3] : nullptr;
    if constexpr (DOTS) {
#pragma unroll
      for (int e = 0; e < VPL * 3; ++e) my[e] = 0.0;
    }
    float fn[VPL], fr[VPL], fi[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) fn[k] = fr[k] = fi[k] = 0.f;
    int pending = 0;

    // the warp's slots walk adjacent rows; the entries of its next rows
    // are in flight while the current ones compute, so a row's gathers go
    // out together with its own vector loads
    const int wb0 = xi * NSLOT + SPW * wq;
    if (wb0 < rows) stage(wb0, 0);
    cp_async_commit();
    // store steps run as programmatic dependent launches: H's entries above
    // are constant, everything below reads or overwrites the vectors of
    // the previous step, which this wait sees completed
    if constexpr (SM != 0) asm volatile("griddepcontrol.wait;" ::: "memory");
    int sb = 0;
    for (int wb = wb0; wb < rows; wb += RPI * stride) {
      if (wb + RPI * stride < rows) stage(wb + RPI * stride, sb ^ 1);
      cp_async_commit();
      cp_async_wait_prev();
      __syncwarp();
      const int i0 = wb + half;
      int64_t row[RPI];
      bool ok[RPI];
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        row[u] = i0 + u * stride;
        ok[u] = row[u] < rows;
      }
      PT xv[RPI], pv[RPI];
      int4 c4[RPI][KQ];
      float4 hv[RPI][2 * KQ];
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        if (!ok[u]) continue;
        const int64_t r = row[u];
        xv[u] = x[r * p.rp + col];
        if constexpr (MODE == STEP_RECUR) pv[u] = prev[r * p.rp + col];
        const int4* ri = reinterpret_cast<const int4*>(&sidx[wq][sb][u][half * K]);
        const float4* rv =
            reinterpret_cast<const float4*>(&sval[wq][sb][u][half * K]);
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
          c4[u][q] = ri[q];
          hv[u][2 * q] = rv[2 * q];
          hv[u][2 * q + 1] = rv[2 * q + 1];
        }
      }
#pragma unroll
      for (int u = 0; u < RPI; ++u) {
        if (!ok[u]) continue;
        float ar[VPL], ai[VPL];
        float sr[VPL], si[VPL];        // store values (SM == 2: V alpha_n)
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          ar[k] = shift * Pay::re(xv[u], k);
          ai[k] = shift * Pay::im(xv[u], k);
          sr[k] = si[k] = 0.f;
        }
        const float4* vv = SM == 2
            ? reinterpret_cast<const float4*>(sa.vell + (int64_t)row[u] * K)
            : nullptr;
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
          const int cc[4] = {col_index(p, c4[u][q].x), col_index(p, c4[u][q].y),
                             col_index(p, c4[u][q].z), col_index(p, c4[u][q].w)};
          PT xx[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) xx[t] = x[(int64_t)cc[t] * p.rp + col];
          const float hr[4] = {hv[u][2 * q].x, hv[u][2 * q].z,
                               hv[u][2 * q + 1].x, hv[u][2 * q + 1].z};
          const float hi[4] = {hv[u][2 * q].y, hv[u][2 * q].w,
                               hv[u][2 * q + 1].y, hv[u][2 * q + 1].w};
#pragma unroll
          for (int t = 0; t < 4; ++t) {
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
              ar[k] = fmaf(hr[t], Pay::re(xx[t], k), ar[k]);
              ar[k] = fmaf(-hi[t], Pay::im(xx[t], k), ar[k]);
              ai[k] = fmaf(hr[t], Pay::im(xx[t], k), ai[k]);
              ai[k] = fmaf(hi[t], Pay::re(xx[t], k), ai[k]);
            }
          }
          if constexpr (SM == 2) {
            const float4 v01 = __ldg(vv + 2 * q), v23 = __ldg(vv + 2 * q + 1);
            const float wr[4] = {v01.x, v01.z, v23.x, v23.z};
            const float wi[4] = {v01.y, v01.w, v23.y, v23.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
#pragma unroll
              for (int k = 0; k < VPL; ++k) {
                const float xr = Pay::re(xx[t], k), xi = Pay::im(xx[t], k);
                sr[k] = fmaf(wr[t], xr, fmaf(-wi[t], xi, sr[k]));
                si[k] = fmaf(wr[t], xi, fmaf(wi[t], xr, si[k]));
              }
            }
          }
        }
        if constexpr (SM != 0) {
          // store row of alpha_n: K index row * R + vector, real vectors
          // only; pairs of K-adjacent vectors as bf16x2 writes when R is even
#pragma unroll
          for (int k = 0; k < VPL; k += 2) {
            const int64_t vec = (int64_t)g * G + (int64_t)lane * VPL + k;
            const int64_t kk = (int64_t)row[u] * sa.R + vec;
            const float re0 = SM == 2 ? sr[k] : Pay::re(xv[u], k);
            const float im0 = SM == 2 ? si[k] : Pay::im(xv[u], k);
            const float re1 = SM == 2 ? sr[k + 1] : Pay::re(xv[u], k + 1);
            const float im1 = SM == 2 ? si[k + 1] : Pay::im(xv[u], k + 1);
            if ((sa.R & 1) == 0) {
              if (vec < sa.R)
                store_put2_bf16x3(sa.store, kk, re0, im0, re1, im1);
            } else {
              if (vec < sa.R) store_put<STORE_BF16X3>(sa.store, kk, re0, im0);
              if (vec + 1 < sa.R)
                store_put<STORE_BF16X3>(sa.store, kk + 1, re1, im1);
            }
          }
        }
        float orr[VPL], oii[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          if constexpr (MODE == STEP_FIRST) {
            orr[k] = 0.5f * ar[k];
            oii[k] = 0.5f * ai[k];
          } else {
            orr[k] = ar[k] - Pay::re(pv[u], k);
            oii[k] = ai[k] - Pay::im(pv[u], k);
          }
        }
        out[(int64_t)row[u] * p.rp + col] = Pay::make(orr, oii);
        if constexpr (DOTS) {
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            const float vr = Pay::re(xv[u], k), vi = Pay::im(xv[u], k);
            fn[k] = fmaf(vr, vr, fmaf(vi, vi, fn[k]));
            fr[k] = fmaf(orr[k], vr, fmaf(oii[k], vi, fr[k]));
            fi[k] = fmaf(orr[k], vi, fmaf(-oii[k], vr, fi[k]));
          }
          if (++pending == FLUSH) {
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
              my[k * 3 + 0] += (double)fn[k];
              my[k * 3 + 1] += (double)fr[k];
              my[k * 3 + 2] += (double)fi[k];
              fn[k] = fr[k] = fi[k] = 0.f;
            }
            pending = 0;
          }
        }
      }
      __syncwarp();   // stage buffer sb is refilled two iterations on
      sb ^= 1;
    }
    if constexpr (DOTS) {
#pragma unroll
      for (int k = 0; k < VPL; ++k) {
        my[k * 3 + 0] += (double)fn[k];
        my[k * 3 + 1] += (double)fr[k];
        my[k * 3 + 2] += (double)fi[k];
      }
      __syncthreads();
      // layout [group][vector*3 + component][partition]: the finalize
      // kernel reads each vector's partitions contiguously
      double* dst = p.partials + (int64_t)g * (G * 3) * p.xitems + xi;
      for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NSLOT; ++q) s += red[q][e];
        dst[(int64_t)e * p.xitems] = s;
      }
      __syncthreads();
    }
  }
}

template <int K, int MODE, bool DOTS, int RPI, int VPL, int SM = 0,
          int SW = 8>
static int launch_ell_t(kpm_handle* h, const StepArgs& a,
                        const StoreArgs& sa = StoreArgs{}) {
  static int occ = -1;
  if (occ < 0) {
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, cheb_step_ell_kernel<K, MODE, DOTS, RPI, VPL, SM, SW>,
        STEP_THREADS, 0));
    occ = blocks > 0 ? blocks : 1;
  }
  const int64_t work = (int64_t)a.xitems * a.groups;
  int64_t grid = (int64_t)occ * h->num_sms;
  if (grid > work) grid = work;
  cudaEvent_t e1 = nullptr;
  KPM_TRY(prof_begin(h, &e1));
  if constexpr (SM != 0) {
    // programmatic dependent launch (the kernel waits for its predecessor
    // in griddepcontrol.wait)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(STEP_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    KPM_CUDA(cudaLaunchKernelEx(
        &cfg, cheb_step_ell_kernel<K, MODE, DOTS, RPI, VPL, SM, SW>, a,
        h->H.ell_idx, h->H.ell_val, sa));
  } else {
    cheb_step_ell_kernel<K, MODE, DOTS, RPI, VPL, SM, SW>
        <<<(unsigned)grid, STEP_THREADS, 0, h->stream>>>(a, h->H.ell_idx,
                                                          h->H.ell_val, sa);
  }
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (e1) KPM_CUDA(cudaEventRecord(e1, h->stream));
  return KPM_OK;
}

// Store steps (no dot products).  Blocks of 16 vectors (one complex64
// vector per lane in 16-lane slots) run as KPM_STORE_SW-lane slots of
// 16 / KPM_STORE_SW vectors per lane: the same 128 bytes per row, more rows
// in flight per warp, and each vector's arithmetic unchanged.
template <int K, int VPL, int SM, int SW = 8>
static int dispatch_store_mode(kpm_handle* h, int mode, const StepArgs& a,
                               const StoreArgs& sa) {
  return mode == STEP_FIRST
             ? launch_ell_t<K, STEP_FIRST, false, 1, VPL, SM, SW>(h, a, sa)
             : launch_ell_t<K, STEP_RECUR, false, 1, VPL, SM, SW>(h, a, sa);
}

template <int SW>
static int dispatch_store_16(kpm_handle* h, int mode, const StepArgs& a,
                             const StoreArgs& sa) {
  constexpr int VPL = 16 / SW;
  switch (h->H.ell_k) {
#define KPM_STORE_CASE(KK)                                                 \
  case KK:                                                                 \
    return sa.smode == 2 ? dispatch_store_mode<KK, VPL, 2, SW>(h, mode, a, sa) \
                         : dispatch_store_mode<KK, VPL, 1, SW>(h, mode, a, sa);
    KPM_STORE_CASE(4)
    KPM_STORE_CASE(8)
    KPM_STORE_CASE(12)
    KPM_STORE_CASE(16)
#undef KPM_STORE_CASE
  }
  set_error("ELL width %d not supported", h->H.ell_k);
  return KPM_EUNSUPPORTED;
}

template <int K, int VPL>
static int dispatch_mode(kpm_handle* h, int mode, bool dots,
                         const StepArgs& a, const StoreArgs* sa) {
  if (sa && sa->smode)
    return sa->smode == 2 ? dispatch_store_mode<K, VPL, 2>(h, mode, a, *sa)
                          : dispatch_store_mode<K, VPL, 1>(h, mode, a, *sa);
  if (mode == STEP_FIRST)
    return dots ? launch_ell_t<K, STEP_FIRST, true, 1, VPL>(h, a)
                : launch_ell_t<K, STEP_FIRST, false, 1, VPL>(h, a);
  return dots ? launch_ell_t<K, STEP_RECUR, true, 1, VPL>(h, a)
              : launch_ell_t<K, STEP_RECUR, false, 1, VPL>(h, a);
}

template <int VPL>
static int dispatch_k(kpm_handle* h, int mode, bool dots, const StepArgs& a,
                      const StoreArgs* sa) {
  switch (h->H.ell_k) {
    case 4: return dispatch_mode<4, VPL>(h, mode, dots, a, sa);
    case 8: return dispatch_mode<8, VPL>(h, mode, dots, a, sa);
    case 12: return dispatch_mode<12, VPL>(h, mode, dots, a, sa);
    case 16: return dispatch_mode<16, VPL>(h, mode, dots, a, sa);
  }
  set_error("ELL width %d not supported", h->H.ell_k);
  return KPM_EUNSUPPORTED;
}

// The block layout holds one (16-vector groups) or two (32-vector groups)
// complex64 vectors per 16-byte lane of a 16-lane row; the ELL step runs
// both as 8-lane slots with twice as many vectors per lane: the same bytes
// per row, twice the rows in flight per warp, and the same slot of every
// row and the same flush points for every vector whatever its group size.
int launch_step_ell(kpm_handle* h, int mode, bool dots, const StepArgs& a,
                    const StoreArgs* sa) {
  StepArgs w = a;
  // steps without dot partials: every resident block gets a partition
  if (!dots) w.xitems = xitems_for_rows(a.rows, h->num_sms);
  if (sa && sa->smode && a.vpl == 1 && KPM_STORE_SW != 8) {
    constexpr int SW = KPM_STORE_SW;
    w.vpl = 16 / SW;
    w.rp = a.rp / w.vpl;
    return dispatch_store_16<SW>(h, mode, w, *sa);
  }
  w.vpl = 2 * a.vpl;
  w.rp = a.rp / 2;
  return a.vpl == 1 ? dispatch_k<2>(h, mode, dots, w, sa)
                    : dispatch_k<4>(h, mode, dots, w, sa);
}

}  // namespace kpm
