// Batched multi-system KPM DOS on block-sparse (4 x 4) Hamiltonians.
//
// Many disorder realisations / lattices of different size are advanced
// together: one launch per Chebyshev step covers every system (the work
// items of all systems form one index space, found by binary search over a
// prefix array), and the step loop of a run is captured once into a CUDA
// graph and replayed.  Replaces one SpectralDensity per realisation
// (kwant/kpm.py:163-252) for the batched-realisation workload.
//
// BSR4 step: a 16-lane slot owns one block row (4 orbitals) for a group of
// 16 * VPL vectors; each lane holds VPL vectors (8 or 16 bytes) of all four
// orbital rows.  Blocks are stored ELL-style, KB = 8 per block row, the
// diagonal block first with the -2b/a shift folded in (so the first
// neighbour rows loaded are the row's own entries, reused for the DOS dot
// products), padding blocks are zero and point at the row itself.
// Arithmetic per vector is independent of VPL (same FMA order, same flush
// points, same reduction order), so the autotuner's choice of VPL never
// changes results.
//
// Sparse blocks: when every orbital row of every system has at most 16
// non-zero entries (the Wilson-Dirac blocks are 8/16 (hopping) and 4/16
// (onsite) filled: 13 per row instead of the dense 28), the blocks are
// converted on the device to an orbital-row ELL (entries in block, column
// order, zeros dropped, width rounded up to 4) and the ELL step kernel runs
// instead: 2.2x fewer FMAs for one more gathered row per entry, the
// products of each row in the same order as the BSR kernel.
//
// Random-phase vectors: counter-based SplitMix64 (Steele, Lea & Flood 2014;
// Vigna's constants) of (seed, system, vector) then orbital; the top 24 bits
// give u in [0, 1) and the entry is exp(2 pi i u).

#include <algorithm>
#include <vector>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {
namespace bt {

constexpr int KB = 8;            // blocks per block row
constexpr int BS = 4;            // block size

struct SysDev {
  int64_t nb;            // block rows
  int xitems;            // row partitions (depends only on the row count)
  const int32_t* bidx;   // [nb][KB]
  const float2* bval;    // [nb][KB][16], 2 (H - b) / a
  int ell_k;             // ELL width (0: BSR kernel)
  const int32_t* eidx;   // [4 nb][ell_k]
  const float2* eval;    // [4 nb][ell_k]
  const int32_t* spidx;  // [4 nb][16]: panel slot q * 4 + cc of each entry
  const float2* spval;   // [4 nb][16]: its value (sparse-block kernel)
  void* v[3];            // a0, b0, b1: [4 nb][Rpad] complex64
  double* partials;      // [Rpad * 3][xitems]
  double2* mu01;         // [Rpad][2]
  double2* mom;          // [M][Rpad]
};

template <int VPL> struct Pay;
template <> struct Pay<1> { using T = float2; };
template <> struct Pay<2> { using T = float4; };

// complex MAC of block entry h (float2) into acc (re, im) for one vector
__device__ __forceinline__ void cmac(float& ar, float& ai, float hr, float hi,
                                     float xr, float xi) {
  ar = fmaf(hr, xr, ar);
  ar = fmaf(-hi, xi, ar);
  ai = fmaf(hr, xi, ai);
  ai = fmaf(hi, xr, ai);
}

// Block rows per CTA tile: one per 16-lane slot.
constexpr int TILE = SLOTS;
// 16-byte chunks of one tile's block values and indices
constexpr int VAL_CHUNKS = TILE * KB * 16 * 8 / 16;   // 1024
constexpr int IDX_CHUNKS = TILE * KB * 4 / 16;        // 32

// Stage the block values and block-column indices of block rows
// [base, base + TILE) (those below nb) into shared memory, asynchronously.
__device__ __forceinline__ void stage_tile(const SysDev& S, int64_t base,
                                           float2* sval, int32_t* sidx) {
  const float4* gv = reinterpret_cast<const float4*>(S.bval + base * KB * 16);
  float4* dv = reinterpret_cast<float4*>(sval);
  for (int c = threadIdx.x; c < VAL_CHUNKS; c += STEP_THREADS)
    if (base + c / (KB * 16 * 8 / 16) < S.nb) cp_async16(dv + c, gv + c);
  if (threadIdx.x < IDX_CHUNKS && base + threadIdx.x / (KB * 4 / 16) < S.nb)
    cp_async16(reinterpret_cast<int4*>(sidx) + threadIdx.x,
               reinterpret_cast<const int4*>(S.bidx + base * KB) +
                   threadIdx.x);
}

// Per-warp variant: the two block rows [base, base + 2) of one warp's two
// slots (2 x 1 KB of values: 4 chunks per lane; 2 x 32 B of indices: lanes
// 0-3), so that warps advance without CTA-wide barriers.
constexpr int WROWS = 2;                                 // slots per warp
constexpr int WVAL = WROWS * KB * 16;                    // float2 per stage
constexpr int WIDX = WROWS * KB;                         // int32 per stage
__device__ __forceinline__ void stage_warp(const SysDev& S, int64_t base,
                                           int lane, float2* sval,
                                           int32_t* sidx) {
  const float4* gv = reinterpret_cast<const float4*>(S.bval + base * KB * 16);
  float4* dv = reinterpret_cast<float4*>(sval);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = lane + 32 * k;                 // 128 chunks, 64 per row
    if (base + c / 64 < S.nb) cp_async16(dv + c, gv + c);
  }
  if (lane < 4 && base + lane / 2 < S.nb)
    cp_async16(reinterpret_cast<int4*>(sidx) + lane,
               reinterpret_cast<const int4*>(S.bidx + base * KB) + lane);
}

// PHASE 0: x = a0 -> b0 (first step); 1: x = b0, prev = a0 -> b1;
// 2: x = b1, prev = b0 -> b0; 3: x = b0, prev = b1 -> b1.
//
// The CTA walks its partition in tiles of TILE consecutive block rows (one
// per slot).  The block values and indices of tile t + 1 are copied into
// shared memory with cp.async while tile t computes, so the only global
// loads on a row's critical path are the gathered vector rows; those are
// double-buffered one block ahead in registers.  Padding blocks (column ==
// the row itself after the diagonal block) skip their products: adding
// 0 * x would not change the sums.
template <int VPL, int PHASE, int OCC>
__global__ void __launch_bounds__(STEP_THREADS, OCC)
bsr_step_kernel(const SysDev* __restrict__ sys,
                const int64_t* __restrict__ prefix, int nsys, int64_t total,
                int64_t Rpad, int gmajor) {
  using PT = typename Pay<VPL>::T;
  constexpr int G = 16 * VPL;
  constexpr int FLUSH = 8;       // block rows (32 orbital rows)
  const int lane = threadIdx.x & 15;
  const int slot = threadIdx.x >> 4;
  __shared__ double red[SLOTS][G * 3];
  __shared__ __align__(16) float2 sval[STEP_THREADS / 32][2][WVAL];
  __shared__ __align__(16) int32_t sidx[STEP_THREADS / 32][2][WIDX];
  const int64_t groups = Rpad / G;
  const int64_t rp = Rpad / VPL;
  const int wid = threadIdx.x >> 5, wl = threadIdx.x & 31;
  const int half = slot & 1;                     // this slot's row in the warp

  for (int64_t w = blockIdx.x; w < total; w += gridDim.x) {
    int lo = 0, hi = nsys;   // largest s with prefix[s] <= w
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= w) lo = mid; else hi = mid;
    }
    const SysDev& S = sys[lo];
    const int64_t local = w - prefix[lo];
    // work order within a system: partition-major (the vector groups of a
    // row partition side by side, sharing its block rows in L2) or
    // group-major (all partitions of one vector group side by side, so the
    // resident blocks cover a wider band of rows and the gathered rows of
    // distant neighbours are still in L2); the results do not depend on it
    int xi, g;
    if (gmajor) {
      g = (int)(local / S.xitems);
      xi = (int)(local - (int64_t)g * S.xitems);
    } else {
      xi = (int)(local / groups);
      g = (int)(local - (int64_t)xi * groups);
    }
    const int64_t col = (int64_t)g * 16 + lane;
    const PT* __restrict__ X;
    const PT* P = nullptr;
    PT* O;
    if constexpr (PHASE == 0) {
      X = (const PT*)S.v[0]; O = (PT*)S.v[1];
    } else if constexpr (PHASE == 1) {
      X = (const PT*)S.v[1]; P = (const PT*)S.v[0]; O = (PT*)S.v[2];
    } else if constexpr (PHASE == 2) {
      X = (const PT*)S.v[2]; P = (const PT*)S.v[1]; O = (PT*)S.v[1];
    } else {
      X = (const PT*)S.v[1]; P = (const PT*)S.v[2]; O = (PT*)S.v[2];
    }
    double* my = &red[slot][lane * VPL * 3];
#pragma unroll
    for (int e = 0; e < VPL * 3; ++e) my[e] = 0.0;
    float fn[VPL], fr[VPL], fi[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) fn[k] = fr[k] = fi[k] = 0.f;
    int pending = 0;
    const int64_t stride = (int64_t)S.xitems * SLOTS;
    const int64_t first = (int64_t)xi * SLOTS;
    const int64_t tiles = first < S.nb ? (S.nb - first + stride - 1) / stride
                                       : 0;
    const int64_t wfirst = first + 2 * wid;      // this warp's rows
    if (tiles > 0) stage_warp(S, wfirst, wl, sval[wid][0], sidx[wid][0]);
    cp_async_commit();

    for (int64_t t = 0; t < tiles; ++t) {
      const int buf = (int)(t & 1);
      if (t + 1 < tiles)
        stage_warp(S, wfirst + (t + 1) * stride, wl, sval[wid][buf ^ 1],
                   sidx[wid][buf ^ 1]);
      cp_async_commit();
      cp_async_wait_prev();
      __syncwarp();
      const int64_t i = first + t * stride + slot;
      if (i < S.nb) {
        const float4* bvs =
            reinterpret_cast<const float4*>(sval[wid][buf] + half * KB * 16);
        const int4* ip =
            reinterpret_cast<const int4*>(sidx[wid][buf] + half * KB);
        const int4 i0 = ip[0], i1 = ip[1];
        const int cidx[KB] = {i0.x, i0.y, i0.z, i0.w,
                              i1.x, i1.y, i1.z, i1.w};
        float acc[BS][VPL][2];
#pragma unroll
        for (int rr = 0; rr < BS; ++rr)
#pragma unroll
          for (int k = 0; k < VPL; ++k) acc[rr][k][0] = acc[rr][k][1] = 0.f;
        PT xbuf[2][BS];
#pragma unroll
        for (int cc = 0; cc < BS; ++cc)
          xbuf[0][cc] = X[((int64_t)cidx[0] * BS + cc) * rp + col];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
          PT* xn = xbuf[q & 1];
          if (q + 1 < KB && cidx[q + 1] != (int)i) {
#pragma unroll
            for (int cc = 0; cc < BS; ++cc)
              xbuf[(q + 1) & 1][cc] =
                  X[((int64_t)cidx[q + 1] * BS + cc) * rp + col];
          }
          if (q > 0 && cidx[q] == (int)i) continue;   // padding block
          const float4* bv = bvs + q * 8;
#pragma unroll
          for (int rr = 0; rr < BS; ++rr) {
            const float4 b01 = bv[2 * rr], b23 = bv[2 * rr + 1];
            const float hr[4] = {b01.x, b01.z, b23.x, b23.z};
            const float hi[4] = {b01.y, b01.w, b23.y, b23.w};
#pragma unroll
            for (int cc = 0; cc < BS; ++cc) {
              if constexpr (VPL == 1) {
                cmac(acc[rr][0][0], acc[rr][0][1], hr[cc], hi[cc], xn[cc].x,
                     xn[cc].y);
              } else {
                cmac(acc[rr][0][0], acc[rr][0][1], hr[cc], hi[cc], xn[cc].x,
                     xn[cc].y);
                cmac(acc[rr][1][0], acc[rr][1][1], hr[cc], hi[cc], xn[cc].z,
                     xn[cc].w);
              }
            }
          }
        }
#pragma unroll
        for (int rr = 0; rr < BS; ++rr) {
          const int64_t orow = (i * BS + rr) * rp + col;
          float o[VPL][2];
          if constexpr (PHASE == 0) {
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
              o[k][0] = 0.5f * acc[rr][k][0];
              o[k][1] = 0.5f * acc[rr][k][1];
            }
          } else {
            const PT pv = P[orow];
            if constexpr (VPL == 1) {
              o[0][0] = acc[rr][0][0] - pv.x;
              o[0][1] = acc[rr][0][1] - pv.y;
            } else {
              o[0][0] = acc[rr][0][0] - pv.x;
              o[0][1] = acc[rr][0][1] - pv.y;
              o[1][0] = acc[rr][1][0] - pv.z;
              o[1][1] = acc[rr][1][1] - pv.w;
            }
          }
          PT ov;
          if constexpr (VPL == 1) {
            ov = make_float2(o[0][0], o[0][1]);
          } else {
            ov = make_float4(o[0][0], o[0][1], o[1][0], o[1][1]);
          }
          O[orow] = ov;
          // DOS dots of this vector: <x|x>, <o|x> (x = the row's own
          // entries, read again: they were loaded as block 0, the diagonal
          // block)
          const PT xo = X[orow];
          float xr[VPL], xim[VPL];
          if constexpr (VPL == 1) {
            xr[0] = xo.x; xim[0] = xo.y;
          } else {
            xr[0] = xo.x; xim[0] = xo.y;
            xr[1] = xo.z; xim[1] = xo.w;
          }
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            fn[k] = fmaf(xr[k], xr[k], fmaf(xim[k], xim[k], fn[k]));
            fr[k] = fmaf(o[k][0], xr[k], fmaf(o[k][1], xim[k], fr[k]));
            fi[k] = fmaf(o[k][0], xim[k], fmaf(-o[k][1], xr[k], fi[k]));
          }
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
      __syncwarp();   // buffer buf is restaged at t + 2
    }
#pragma unroll
    for (int k = 0; k < VPL; ++k) {
      my[k * 3 + 0] += (double)fn[k];
      my[k * 3 + 1] += (double)fr[k];
      my[k * 3 + 2] += (double)fi[k];
    }
    __syncthreads();
    // partials [vector * 3 + component][partition]
    double* dst = S.partials + (int64_t)g * G * 3 * S.xitems + xi;
    for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < SLOTS; ++q) s += red[q][e];
      dst[(int64_t)e * S.xitems] = s;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- ELL
constexpr int EK = 16;   // widest ELL row of the batched ELL kernel

// non-zero entries of orbital row r (padding blocks and zeros skipped);
// the maximum over rows goes to *kmax
__global__ void ell_count_kernel(int64_t nb, const int32_t* __restrict__ bidx,
                                 const float2* __restrict__ bval,
                                 int* __restrict__ kmax) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb * BS) return;
  const int64_t i = r / BS;
  const int rr = (int)(r % BS);
  int cnt = 0;
  for (int q = 0; q < KB; ++q) {
    if (q > 0 && bidx[i * KB + q] == (int32_t)i) continue;
    for (int cc = 0; cc < BS; ++cc) {
      const float2 v = bval[(i * KB + q) * 16 + rr * BS + cc];
      cnt += (v.x != 0.f || v.y != 0.f) ? 1 : 0;
    }
  }
  atomicMax(kmax, cnt);
}

// ELL rows: entries in (block, column) order, then (r, 0) padding
__global__ void ell_fill_kernel(int64_t nb, int K,
                                const int32_t* __restrict__ bidx,
                                const float2* __restrict__ bval,
                                int32_t* __restrict__ eidx,
                                float2* __restrict__ eval) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb * BS) return;
  const int64_t i = r / BS;
  const int rr = (int)(r % BS);
  int e = 0;
  for (int q = 0; q < KB; ++q) {
    const int32_t c = bidx[i * KB + q];
    if (q > 0 && c == (int32_t)i) continue;
    for (int cc = 0; cc < BS; ++cc) {
      const float2 v = bval[(i * KB + q) * 16 + rr * BS + cc];
      if ((v.x != 0.f || v.y != 0.f) && e < K) {
        eidx[r * K + e] = c * BS + cc;
        eval[r * K + e] = v;
        ++e;
      }
    }
  }
  for (; e < K; ++e) {
    eidx[r * K + e] = (int32_t)r;
    eval[r * K + e] = make_float2(0.f, 0.f);
  }
}

// Stage the ELL entries of rows [base, base + TILE) (those below rows):
// TILE * K entries of 4 + 8 bytes, contiguous in both arrays.
__device__ __forceinline__ void stage_ell(const SysDev& S, int64_t rows,
                                          int64_t base, float2* sval,
                                          int32_t* sidx) {
  const int K = S.ell_k;
  const int vchunks = TILE * K / 2, ichunks = TILE * K / 4;
  const int vper = K / 2, iper = K / 4;   // chunks per row
  const float4* gv = reinterpret_cast<const float4*>(S.eval + base * K);
  const int4* gi = reinterpret_cast<const int4*>(S.eidx + base * K);
  for (int c = threadIdx.x; c < vchunks + ichunks; c += STEP_THREADS) {
    if (c < vchunks) {
      if (base + c / vper < rows)
        cp_async16(reinterpret_cast<float4*>(sval) + c, gv + c);
    } else {
      const int d = c - vchunks;
      if (base + d / iper < rows)
        cp_async16(reinterpret_cast<int4*>(sidx) + d, gi + d);
    }
  }
}

// One Chebyshev step of every ELL system: a slot owns one orbital row for a
// group of 16 * VPL vectors; the row's entries come from shared memory
// (staged one tile ahead with cp.async), the gathered vector rows are
// loaded four entries ahead.
template <int VPL, int PHASE>
__global__ void __launch_bounds__(STEP_THREADS, VPL == 1 ? 6 : 4)
ell_batch_step_kernel(const SysDev* __restrict__ sys,
                      const int64_t* __restrict__ prefix, int nsys,
                      int64_t total, int64_t Rpad, int gmajor) {
  using PT = typename Pay<VPL>::T;
  constexpr int G = 16 * VPL;
  constexpr int FLUSH = 32;      // orbital rows
  const int lane = threadIdx.x & 15;
  const int slot = threadIdx.x >> 4;
  __shared__ double red[SLOTS][G * 3];
  __shared__ __align__(16) float2 sval[2][TILE * EK];
  __shared__ __align__(16) int32_t sidx[2][TILE * EK];
  const int64_t groups = Rpad / G;
  const int64_t rp = Rpad / VPL;

  for (int64_t w = blockIdx.x; w < total; w += gridDim.x) {
    int lo = 0, hi = nsys;   // largest s with prefix[s] <= w
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= w) lo = mid; else hi = mid;
    }
    const SysDev& S = sys[lo];
    const int K = S.ell_k;
    const int KQ = K / 4;
    const int64_t rows = S.nb * BS;
    const int64_t local = w - prefix[lo];
    int xi, g;                 // work order as in bsr_step_kernel
    if (gmajor) {
      g = (int)(local / S.xitems);
      xi = (int)(local - (int64_t)g * S.xitems);
    } else {
      xi = (int)(local / groups);
      g = (int)(local - (int64_t)xi * groups);
    }
    const int64_t col = (int64_t)g * 16 + lane;
    const PT* __restrict__ X;
    const PT* P = nullptr;
    PT* O;
    if constexpr (PHASE == 0) {
      X = (const PT*)S.v[0]; O = (PT*)S.v[1];
    } else if constexpr (PHASE == 1) {
      X = (const PT*)S.v[1]; P = (const PT*)S.v[0]; O = (PT*)S.v[2];
    } else if constexpr (PHASE == 2) {
      X = (const PT*)S.v[2]; P = (const PT*)S.v[1]; O = (PT*)S.v[1];
    } else {
      X = (const PT*)S.v[1]; P = (const PT*)S.v[2]; O = (PT*)S.v[2];
    }
    double* my = &red[slot][lane * VPL * 3];
#pragma unroll
    for (int e = 0; e < VPL * 3; ++e) my[e] = 0.0;
    float fn[VPL], fr[VPL], fi[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) fn[k] = fr[k] = fi[k] = 0.f;
    int pending = 0;
    const int64_t stride = (int64_t)S.xitems * SLOTS;
    const int64_t first = (int64_t)xi * SLOTS;
    const int64_t tiles = first < rows ? (rows - first + stride - 1) / stride
                                       : 0;
    if (tiles > 0) stage_ell(S, rows, first, sval[0], sidx[0]);
    cp_async_commit();

    for (int64_t t = 0; t < tiles; ++t) {
      const int buf = (int)(t & 1);
      if (t + 1 < tiles)
        stage_ell(S, rows, first + (t + 1) * stride, sval[buf ^ 1],
                  sidx[buf ^ 1]);
      cp_async_commit();
      cp_async_wait_prev();
      __syncthreads();
      const int64_t r = first + t * stride + slot;
      if (r < rows) {
        const int4* ci = reinterpret_cast<const int4*>(sidx[buf] + slot * K);
        const float4* cv = reinterpret_cast<const float4*>(sval[buf] + slot * K);
        float acc[VPL][2];
#pragma unroll
        for (int k = 0; k < VPL; ++k) acc[k][0] = acc[k][1] = 0.f;
        PT xb[2][4];
        {
          const int4 c0 = ci[0];
          const int cc[4] = {c0.x, c0.y, c0.z, c0.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) xb[0][u] = X[(int64_t)cc[u] * rp + col];
        }
#pragma unroll
        for (int qc = 0; qc < EK / 4; ++qc) {
          if (qc < KQ) {
            if (qc + 1 < KQ) {
              const int4 c1 = ci[qc + 1];
              const int cc[4] = {c1.x, c1.y, c1.z, c1.w};
#pragma unroll
              for (int u = 0; u < 4; ++u)
                xb[(qc + 1) & 1][u] = X[(int64_t)cc[u] * rp + col];
            }
            const float4 v01 = cv[2 * qc], v23 = cv[2 * qc + 1];
            const float hr[4] = {v01.x, v01.z, v23.x, v23.z};
            const float hi[4] = {v01.y, v01.w, v23.y, v23.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const PT xv = xb[qc & 1][u];
              if constexpr (VPL == 1) {
                cmac(acc[0][0], acc[0][1], hr[u], hi[u], xv.x, xv.y);
              } else {
                cmac(acc[0][0], acc[0][1], hr[u], hi[u], xv.x, xv.y);
                cmac(acc[1][0], acc[1][1], hr[u], hi[u], xv.z, xv.w);
              }
            }
          }
        }
        const int64_t orow = r * rp + col;
        float o[VPL][2];
        if constexpr (PHASE == 0) {
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            o[k][0] = 0.5f * acc[k][0];
            o[k][1] = 0.5f * acc[k][1];
          }
        } else {
          const PT pv = P[orow];
          if constexpr (VPL == 1) {
            o[0][0] = acc[0][0] - pv.x;
            o[0][1] = acc[0][1] - pv.y;
          } else {
            o[0][0] = acc[0][0] - pv.x;
            o[0][1] = acc[0][1] - pv.y;
            o[1][0] = acc[1][0] - pv.z;
            o[1][1] = acc[1][1] - pv.w;
          }
        }
        PT ov;
        if constexpr (VPL == 1) {
          ov = make_float2(o[0][0], o[0][1]);
        } else {
          ov = make_float4(o[0][0], o[0][1], o[1][0], o[1][1]);
        }
        O[orow] = ov;
        const PT xo = X[orow];
        float xr[VPL], xim[VPL];
        if constexpr (VPL == 1) {
          xr[0] = xo.x; xim[0] = xo.y;
        } else {
          xr[0] = xo.x; xim[0] = xo.y;
          xr[1] = xo.z; xim[1] = xo.w;
        }
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          fn[k] = fmaf(xr[k], xr[k], fmaf(xim[k], xim[k], fn[k]));
          fr[k] = fmaf(o[k][0], xr[k], fmaf(o[k][1], xim[k], fr[k]));
          fi[k] = fmaf(o[k][0], xim[k], fmaf(-o[k][1], xr[k], fi[k]));
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
      __syncthreads();   // buffer buf is restaged at t + 2
    }
#pragma unroll
    for (int k = 0; k < VPL; ++k) {
      my[k * 3 + 0] += (double)fn[k];
      my[k * 3 + 1] += (double)fr[k];
      my[k * 3 + 2] += (double)fi[k];
    }
    __syncthreads();
    double* dst = S.partials + (int64_t)g * G * 3 * S.xitems + xi;
    for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < SLOTS; ++q) s += red[q][e];
      dst[(int64_t)e * S.xitems] = s;
    }
    __syncthreads();
  }
}

// Sparse-block entries of orbital row r: the non-zero entries of its block
// row in (block, column) order as (panel slot q * 4 + cc, value); padding
// (slot rr of the diagonal block, value 0) up to EK.
__global__ void sb_fill_kernel(int64_t nb, const int32_t* __restrict__ bidx,
                               const float2* __restrict__ bval,
                               int32_t* __restrict__ spidx,
                               float2* __restrict__ spval) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb * BS) return;
  const int64_t i = r / BS;
  const int rr = (int)(r % BS);
  int e = 0;
  for (int q = 0; q < KB; ++q) {
    if (q > 0 && bidx[i * KB + q] == (int32_t)i) continue;
    for (int cc = 0; cc < BS; ++cc) {
      const float2 v = bval[(i * KB + q) * 16 + rr * BS + cc];
      if ((v.x != 0.f || v.y != 0.f) && e < EK) {
        spidx[r * EK + e] = q * BS + cc;
        spval[r * EK + e] = v;
        ++e;
      }
    }
  }
  for (; e < EK; ++e) {
    spidx[r * EK + e] = rr;
    spval[r * EK + e] = make_float2(0.f, 0.f);
  }
}

// Sparse-block step.  A warp owns two consecutive block rows (one per
// 16-lane half) for a group of 16 vectors (one complex64 per lane).  The
// vector rows of every non-padding block of the next row pair (4 rows x 16
// vectors per block), its alpha_{n-1} rows and its entries are copied into
// shared memory with cp.async while the current pair computes, so every
// gather is asynchronous; the products then run over the non-zero entries
// only (zeros of the 4 x 4 blocks skipped), reading the staged rows by
// panel slot.  No CTA-wide barrier inside the row loop.
constexpr int SB_WARPS = 4;
constexpr int SB_THREADS = SB_WARPS * 32;
constexpr int SB_SLOTS = SB_WARPS * 2;
struct SbStage {
  float2 x[2][KB * BS][16];    // 2 rows x 8 blocks x 4 rows x 16 vectors
  float2 p[2][BS][16];         // alpha_{n-1}
  float2 val[2][BS][EK];
  int32_t pidx[2][BS][EK];
};
struct SbWarp {
  SbStage st[2];
  int32_t bidx[3][2][KB];      // block columns, staged two pairs ahead
};
constexpr size_t SB_SMEM = SB_WARPS * sizeof(SbWarp) +
                           SB_SLOTS * 16 * 3 * sizeof(double);

template <int PHASE>
__device__ __forceinline__ void sb_stage_idx(const SysDev& S, int64_t base,
                                             int lane, int32_t (*dst)[KB]) {
  // 2 rows x 8 int32 = 4 chunks of 16 bytes
  if (lane < 4 && base + lane / 2 < S.nb)
    cp_async16(&dst[lane / 2][(lane % 2) * 4],
               S.bidx + (base + lane / 2) * KB + (lane % 2) * 4);
}

template <int PHASE>
__device__ __forceinline__ void sb_stage_data(const SysDev& S, int64_t base,
                                              int lane, int64_t gcol,
                                              int64_t Rpad,
                                              const float2* X, const float2* P,
                                              const int32_t (*bidx)[KB],
                                              SbStage& st) {
  // vector rows of the blocks: chunk lane of each (row, block): 4 rows x
  // 128 bytes = 32 chunks
  const int cc = lane >> 3, part = lane & 7;
#pragma unroll
  for (int s2 = 0; s2 < 2; ++s2) {
    const int64_t i = base + s2;
    if (i >= S.nb) continue;
#pragma unroll
    for (int q = 0; q < KB; ++q) {
      const int32_t c = bidx[s2][q];
      if (q > 0 && c == (int32_t)i) continue;     // padding block
      cp_async16(&st.x[s2][q * BS + cc][part * 2],
                 X + ((int64_t)c * BS + cc) * Rpad + gcol + part * 2);
    }
    if constexpr (PHASE != 0)
      cp_async16(&st.p[s2][cc][part * 2],
                 P + (i * BS + cc) * Rpad + gcol + part * 2);
    // entries: 4 rows x 16 x 8 bytes = 32 chunks; indices 16 chunks
    cp_async16(reinterpret_cast<float4*>(&st.val[s2][0][0]) + lane,
               reinterpret_cast<const float4*>(S.spval + i * BS * EK) + lane);
    if (lane < 16)
      cp_async16(reinterpret_cast<int4*>(&st.pidx[s2][0][0]) + lane,
                 reinterpret_cast<const int4*>(S.spidx + i * BS * EK) + lane);
  }
}

template <int PHASE>
__global__ void __launch_bounds__(SB_THREADS)
sb_step_kernel(const SysDev* __restrict__ sys,
               const int64_t* __restrict__ prefix, int nsys, int64_t total,
               int64_t Rpad) {
  extern __shared__ __align__(16) uint8_t sb_smem[];
  SbWarp* wsm = reinterpret_cast<SbWarp*>(sb_smem);
  double (*red)[16 * 3] = reinterpret_cast<double (*)[16 * 3]>(
      sb_smem + SB_WARPS * sizeof(SbWarp));
  constexpr int G = 16;
  constexpr int FLUSH = 32;                  // orbital rows
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4, v = lane & 15;
  const int slot = wid * 2 + half;
  SbWarp& W = wsm[wid];
  const int64_t groups = Rpad / G;

  for (int64_t w = blockIdx.x; w < total; w += gridDim.x) {
    int lo = 0, hi = nsys;   // largest s with prefix[s] <= w
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= w) lo = mid; else hi = mid;
    }
    const SysDev& S = sys[lo];
    const int64_t local = w - prefix[lo];
    const int xi = (int)(local / groups);
    const int g = (int)(local - (int64_t)xi * groups);
    const int64_t gcol = (int64_t)g * G;
    const float2* X;
    const float2* P = nullptr;
    float2* O;
    if constexpr (PHASE == 0) {
      X = (const float2*)S.v[0]; O = (float2*)S.v[1];
    } else if constexpr (PHASE == 1) {
      X = (const float2*)S.v[1]; P = (const float2*)S.v[0];
      O = (float2*)S.v[2];
    } else if constexpr (PHASE == 2) {
      X = (const float2*)S.v[2]; P = (const float2*)S.v[1];
      O = (float2*)S.v[1];
    } else {
      X = (const float2*)S.v[1]; P = (const float2*)S.v[2];
      O = (float2*)S.v[2];
    }
    double dn = 0.0, dr = 0.0, di = 0.0;
    float fn = 0.f, fr = 0.f, fi = 0.f;
    int pending = 0;
    const int64_t stride = (int64_t)S.xitems * SB_SLOTS;
    const int64_t wfirst = (int64_t)xi * SB_SLOTS + 2 * wid;
    const int64_t pairs = wfirst < S.nb ? (S.nb - wfirst + stride - 1) / stride
                                        : 0;
    // prologue: indices of pairs 0 and 1, then the data of pair 0
    if (pairs > 0) sb_stage_idx<PHASE>(S, wfirst, lane, W.bidx[0]);
    if (pairs > 1) sb_stage_idx<PHASE>(S, wfirst + stride, lane, W.bidx[1]);
    cp_async_commit();
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();
    if (pairs > 0)
      sb_stage_data<PHASE>(S, wfirst, lane, gcol, Rpad, X, P, W.bidx[0],
                           W.st[0]);
    cp_async_commit();

    for (int64_t t = 0; t < pairs; ++t) {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncwarp();
      const int64_t base = wfirst + t * stride;
      if (t + 2 < pairs)
        sb_stage_idx<PHASE>(S, base + 2 * stride, lane,
                            W.bidx[(int)((t + 2) % 3)]);
      if (t + 1 < pairs)
        sb_stage_data<PHASE>(S, base + stride, lane, gcol, Rpad, X, P,
                             W.bidx[(int)((t + 1) % 3)], W.st[(t + 1) & 1]);
      cp_async_commit();
      const SbStage& st = W.st[t & 1];
      const int64_t i = base + half;
      if (i < S.nb) {
#pragma unroll
        for (int rr = 0; rr < BS; ++rr) {
          float ar = 0.f, ai = 0.f;
#pragma unroll
          for (int e4 = 0; e4 < EK / 4; ++e4) {
            const int4 p4 = reinterpret_cast<const int4*>(st.pidx[half][rr])[e4];
            const float4 v01 = reinterpret_cast<const float4*>(st.val[half][rr])[2 * e4];
            const float4 v23 = reinterpret_cast<const float4*>(st.val[half][rr])[2 * e4 + 1];
            const float2 x0 = st.x[half][p4.x][v], x1 = st.x[half][p4.y][v];
            const float2 x2 = st.x[half][p4.z][v], x3 = st.x[half][p4.w][v];
            cmac(ar, ai, v01.x, v01.y, x0.x, x0.y);
            cmac(ar, ai, v01.z, v01.w, x1.x, x1.y);
            cmac(ar, ai, v23.x, v23.y, x2.x, x2.y);
            cmac(ar, ai, v23.z, v23.w, x3.x, x3.y);
          }
          float2 o;
          if constexpr (PHASE == 0) {
            o = make_float2(0.5f * ar, 0.5f * ai);
          } else {
            const float2 pv = st.p[half][rr][v];
            o = make_float2(ar - pv.x, ai - pv.y);
          }
          O[(i * BS + rr) * Rpad + gcol + v] = o;
          const float2 xo = st.x[half][rr][v];     // diagonal block, row rr
          fn = fmaf(xo.x, xo.x, fmaf(xo.y, xo.y, fn));
          fr = fmaf(o.x, xo.x, fmaf(o.y, xo.y, fr));
          fi = fmaf(o.x, xo.y, fmaf(-o.y, xo.x, fi));
          if (++pending == FLUSH) {
            dn += (double)fn;
            dr += (double)fr;
            di += (double)fi;
            fn = fr = fi = 0.f;
            pending = 0;
          }
        }
      }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    dn += (double)fn;
    dr += (double)fr;
    di += (double)fi;
    red[slot][v * 3 + 0] = dn;
    red[slot][v * 3 + 1] = dr;
    red[slot][v * 3 + 2] = di;
    __syncthreads();
    double* dst = S.partials + (int64_t)g * G * 3 * S.xitems + xi;
    for (int e = threadIdx.x; e < G * 3; e += blockDim.x) {
      double sum = 0.0;
#pragma unroll
      for (int q = 0; q < SB_SLOTS; ++q) sum += red[q][e];
      dst[(int64_t)e * S.xitems] = sum;
    }
    __syncthreads();
  }
}

// grid (Rpad, nsys): fixed-order sums of the partials into DOS moments
__global__ void bsr_finalize_kernel(const SysDev* __restrict__ sys,
                                    int64_t Rpad, int mode, int64_t m_even,
                                    int64_t m_odd) {
  const int64_t v = blockIdx.x;
  const SysDev& S = sys[blockIdx.y];
  __shared__ double sh[3][128];
  double acc[3] = {0.0, 0.0, 0.0};
  const double* src = S.partials + v * 3 * (int64_t)S.xitems;
  for (int xi = threadIdx.x; xi < S.xitems; xi += blockDim.x) {
    acc[0] += src[xi];
    acc[1] += src[S.xitems + xi];
    acc[2] += src[2 * (int64_t)S.xitems + xi];
  }
  for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double nrm = sh[0][0], cre = sh[1][0], cim = sh[2][0];
  if (mode == 0) {
    const double2 m0 = make_double2(nrm, 0.0), m1 = make_double2(cre, -cim);
    S.mu01[2 * v] = m0;
    S.mu01[2 * v + 1] = m1;
    S.mom[0 * Rpad + v] = m0;
    S.mom[1 * Rpad + v] = m1;
  } else {
    const double2 m0 = S.mu01[2 * v], m1 = S.mu01[2 * v + 1];
    S.mom[m_even * Rpad + v] = make_double2(2.0 * nrm - m0.x, 0.0 - m0.y);
    S.mom[m_odd * Rpad + v] = make_double2(2.0 * cre - m1.x, 2.0 * cim - m1.y);
  }
}

// out[s][m] = mean over the R real vectors (fixed order), grid (M, nsys)
__global__ void bsr_mean_kernel(const SysDev* __restrict__ sys, int64_t R,
                                int64_t Rpad, int64_t M, double2* out) {
  const int64_t m = blockIdx.x;
  const SysDev& S = sys[blockIdx.y];
  __shared__ double sr[128], si[128];
  double r = 0.0, im = 0.0;
  for (int64_t v = threadIdx.x; v < R; v += blockDim.x) {
    const double2 x = S.mom[m * Rpad + v];
    r += x.x;
    im += x.y;
  }
  sr[threadIdx.x] = r;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double inv = 1.0 / (double)R;
    out[blockIdx.y * M + m] = make_double2(sr[0] * inv, si[0] * inv);
  }
}

// random-phase starting vectors, complex64, zero padding vectors
__global__ void rng_vectors_kernel(float2* __restrict__ a0, int64_t N,
                                   int64_t R, int64_t Rpad, uint64_t key) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * Rpad) return;
  const int64_t n = idx / Rpad, r = idx % Rpad;
  float2 v = make_float2(0.f, 0.f);
  if (r < R) {
    const uint64_t h = mix64(mix64(key ^ (uint64_t)r) + (uint64_t)n);
    const float u = (float)(h >> 40) * 0x1.0p-24f;
    float s, c;
    sincospif(2.0f * u, &s, &c);
    v = make_float2(c, s);
  }
  a0[idx] = v;
}

struct WdBlocks {
  float2 diag[16];          // (m - 3) G0 (before disorder, shift, scale)
  float2 fwd[3][16];        // H[s, s + e_j] = T_j^dagger
  float2 bwd[3][16];        // H[s, s - e_j] = T_j
};

// Wilson-Dirac BSR rows, scaled: 2 (H - b) / a
__global__ void wd_generate_kernel(int64_t L, WdBlocks blk, double W,
                                   uint64_t key, double scale, double shift,
                                   int32_t* __restrict__ bidx,
                                   float2* __restrict__ bval) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nb = L * L * L;
  if (s >= nb) return;
  const int64_t x = s / (L * L), y = (s / L) % L, z = s % L;
  const uint64_t h = mix64(mix64(key ^ 0xD15C0ull) + (uint64_t)s);
  const double w = W * ((double)(h >> 11) * 0x1.0p-53 - 0.5);
  int q = 0;
  auto put = [&](int64_t col, const float2* b, bool diag) {
    bidx[s * KB + q] = (int32_t)col;
    for (int e = 0; e < 16; ++e) {
      double re = b ? b[e].x : 0.0, im = b ? b[e].y : 0.0;
      if (diag && (e % 5 == 0)) re += w - shift;
      bval[(s * KB + q) * 16 + e] =
          make_float2((float)(re * scale), (float)(im * scale));
    }
    ++q;
  };
  put(s, blk.diag, true);
  const int64_t coord[3] = {x, y, z};
  const int64_t strides[3] = {L * L, L, 1};
  for (int j = 0; j < 3; ++j) {
    if (coord[j] + 1 < L) put(s + strides[j], blk.fwd[j], false);
    if (coord[j] - 1 >= 0) put(s - strides[j], blk.bwd[j], false);
  }
  while (q < KB) put(s, nullptr, false);
}

}  // namespace bt
}  // namespace kpm

using namespace kpm;
using namespace kpm::bt;

struct kpm_batch {
  int64_t R = 0, Rpad = 0, M = 0;
  uint64_t seed = 0;
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  struct Sys {
    int64_t nb = 0;
    double a = 1, b = 0;
    int32_t* bidx = nullptr;
    float2* bval = nullptr;
    int ell_k = 0;
    int32_t* eidx = nullptr;
    float2* eval = nullptr;
    int32_t* spidx = nullptr;
    float2* spval = nullptr;
    void* v[3] = {nullptr, nullptr, nullptr};
    double* partials = nullptr;
    double2* mu01 = nullptr;
    double2* mom = nullptr;
  };
  std::vector<Sys> sys;
  // per step format (0 = BSR, 1 = ELL): system table, work-item prefix
  // sums and totals per VPL (1, 2)
  SysDev* d_sys[2] = {nullptr, nullptr};
  int64_t* d_prefix[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  int64_t total[2][2] = {{0, 0}, {0, 0}};
  double2* d_out = nullptr;
  int vpl = 0;
  int ell = 0;               // step format: 0 BSR, 1 orbital-row ELL,
                             // 2 sparse-block (staged BSR, zeros skipped)
  int occ2 = 0;              // 1: BSR VPL-2 kernel budgeted for 2 blocks/SM
  int gmajor = 0;            // 1: BSR work items in vector-group-major order
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t nodes = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
  bool ready = false;
};

namespace {

int batch_free(kpm_batch* bt) {
  if (!bt) return KPM_OK;
  cudaStream_t s = bt->stream;
  if (bt->exec) cudaGraphExecDestroy(bt->exec);
  if (bt->graph) cudaGraphDestroy(bt->graph);
  for (auto& y : bt->sys) {
    dev_free(y.bidx, s);
    dev_free(y.bval, s);
    dev_free(y.eidx, s);
    dev_free(y.eval, s);
    dev_free(y.spidx, s);
    dev_free(y.spval, s);
    for (int k = 0; k < 3; ++k) dev_free(y.v[k], s);
    dev_free(y.partials, s);
    dev_free(y.mu01, s);
    dev_free(y.mom, s);
  }
  for (int f = 0; f < 2; ++f) {
    dev_free(bt->d_sys[f], s);
    dev_free(bt->d_prefix[f][0], s);
    dev_free(bt->d_prefix[f][1], s);
  }
  dev_free(bt->d_out, s);
  if (s) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  if (bt->e0) cudaEventDestroy(bt->e0);
  if (bt->e1) cudaEventDestroy(bt->e1);
  cudaGetLastError();
  delete bt;
  return KPM_OK;
}

template <int PHASE>
int launch_sb(kpm_batch* bt) {
  static int occ = -1;
  if (occ < 0) {
    KPM_CUDA(cudaFuncSetAttribute(sb_step_kernel<PHASE>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)SB_SMEM));
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, sb_step_kernel<PHASE>, SB_THREADS, SB_SMEM));
    occ = blocks > 0 ? blocks : 1;
  }
  const int64_t total = bt->total[0][0];          // BSR partitions, VPL 1
  int64_t grid = (int64_t)occ * bt->num_sms;
  if (grid > total) grid = total;
  sb_step_kernel<PHASE><<<(unsigned)grid, SB_THREADS, SB_SMEM, bt->stream>>>(
      bt->d_sys[0], bt->d_prefix[0][0], (int)bt->sys.size(), total,
      bt->Rpad);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

template <int VPL, int PHASE>
int launch_bsr(kpm_batch* bt) {
  if (bt->ell == 2) return launch_sb<PHASE>(bt);
  // kernel variants: ELL, or BSR with registers budgeted for 2 or 3 (VPL 2)
  // / 4 (VPL 1) resident blocks per SM
  static int occ[3] = {-1, -1, -1};
  const int var = bt->ell ? 2 : (VPL == 2 && bt->occ2 ? 1 : 0);
  auto kern = var == 2 ? ell_batch_step_kernel<VPL, PHASE>
              : var == 1 ? bsr_step_kernel<VPL, PHASE, 2>
                         : bsr_step_kernel<VPL, PHASE, VPL == 1 ? 4 : 3>;
  int& o = occ[var];
  if (o < 0) {
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, kern, STEP_THREADS, 0));
    o = blocks > 0 ? blocks : 1;
  }
  const int64_t total = bt->total[bt->ell][VPL - 1];
  int64_t grid = (int64_t)o * bt->num_sms;
  if (grid > total) grid = total;
  kern<<<(unsigned)grid, STEP_THREADS, 0, bt->stream>>>(
      bt->d_sys[bt->ell], bt->d_prefix[bt->ell][VPL - 1],
      (int)bt->sys.size(), total, bt->Rpad, bt->gmajor);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// If every row of every system fits the ELL kernel, build the ELL copies
// on the device (the autotuner then times both formats).
int choose_format(kpm_batch* bt) {
  cudaStream_t s = bt->stream;
  const char* env = getenv("KPM_BATCH_FORMAT");
  if (env && strcmp(env, "bsr") == 0) return KPM_OK;
  int* dmax = nullptr;
  KPM_TRY(dev_alloc((void**)&dmax, sizeof(int) * bt->sys.size(), s));
  KPM_CUDA(cudaMemsetAsync(dmax, 0, sizeof(int) * bt->sys.size(), s));
  for (size_t i = 0; i < bt->sys.size(); ++i) {
    auto& y = bt->sys[i];
    ell_count_kernel<<<(unsigned)ceil_div(y.nb * BS, 256), 256, 0, s>>>(
        y.nb, y.bidx, y.bval, dmax + i);
    count_launch(1);
  }
  std::vector<int> kmax(bt->sys.size());
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(kmax.data(), dmax, sizeof(int) * kmax.size(),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  dev_free(dmax, s);
  KPM_CUDA(e);
  for (int k : kmax)
    if (round_up(k > 0 ? k : 1, 4) > EK) return KPM_OK;   // stay BSR
  for (size_t i = 0; i < bt->sys.size(); ++i) {
    auto& y = bt->sys[i];
    const int K = (int)round_up(kmax[i] > 0 ? kmax[i] : 1, 4);
    const size_t n = (size_t)y.nb * BS * K;
    KPM_TRY(dev_alloc((void**)&y.eidx, n * sizeof(int32_t), s));
    KPM_TRY(dev_alloc((void**)&y.eval, n * sizeof(float2), s));
    ell_fill_kernel<<<(unsigned)ceil_div(y.nb * BS, 256), 256, 0, s>>>(
        y.nb, K, y.bidx, y.bval, y.eidx, y.eval);
    count_launch(1);
    KPM_CHECK_LAUNCH();
    y.ell_k = K;
    const size_t ns = (size_t)y.nb * BS * EK;
    KPM_TRY(dev_alloc((void**)&y.spidx, ns * sizeof(int32_t), s));
    KPM_TRY(dev_alloc((void**)&y.spval, ns * sizeof(float2), s));
    sb_fill_kernel<<<(unsigned)ceil_div(y.nb * BS, 256), 256, 0, s>>>(
        y.nb, y.bidx, y.bval, y.spidx, y.spval);
    count_launch(1);
    KPM_CHECK_LAUNCH();
  }
  KPM_CUDA(cudaStreamSynchronize(s));
  return KPM_OK;
}

template <int VPL>
int launch_phase(kpm_batch* bt, int phase) {
  switch (phase) {
    case 0: return launch_bsr<VPL, 0>(bt);
    case 1: return launch_bsr<VPL, 1>(bt);
    case 2: return launch_bsr<VPL, 2>(bt);
    default: return launch_bsr<VPL, 3>(bt);
  }
}

int launch_step_phase(kpm_batch* bt, int vpl, int phase) {
  return vpl == 1 ? launch_phase<1>(bt, phase) : launch_phase<2>(bt, phase);
}

int finalize_all(kpm_batch* bt, int mode, int64_t me, int64_t mo) {
  dim3 grid((unsigned)bt->Rpad, (unsigned)bt->sys.size());
  bsr_finalize_kernel<<<grid, 128, 0, bt->stream>>>(bt->d_sys[bt->ell == 1],
                                                    bt->Rpad, mode,
                                                    me, mo);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// Enqueue one complete DOS run (steps + finalizes + means) on the stream.
int enqueue_run(kpm_batch* bt, int vpl) {
  KPM_TRY(launch_step_phase(bt, vpl, 0));
  KPM_TRY(finalize_all(bt, 0, 0, 1));
  for (int64_t n = 1; n < bt->M / 2; ++n) {
    const int phase = n == 1 ? 1 : (n % 2 == 0 ? 2 : 3);
    KPM_TRY(launch_step_phase(bt, vpl, phase));
    KPM_TRY(finalize_all(bt, 1, 2 * n, 2 * n + 1));
  }
  dim3 grid((unsigned)bt->M, (unsigned)bt->sys.size());
  bsr_mean_kernel<<<grid, 128, 0, bt->stream>>>(bt->d_sys[bt->ell == 1], bt->R,
                                                bt->Rpad,
                                                bt->M, bt->d_out);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

int prepare(kpm_batch* bt) {
  cudaStream_t s = bt->stream;
  const int S = (int)bt->sys.size();
  KPM_REQUIRE(S > 0, "kpm_batch_run: no systems added");
  KPM_TRY(choose_format(bt));
  const bool have_ell = bt->sys[0].ell_k > 0;
  std::vector<SysDev> hs[2] = {std::vector<SysDev>(S), std::vector<SysDev>(S)};
  std::vector<int64_t> pre[2][2];
  for (int f = 0; f < 2; ++f)
    for (int v = 0; v < 2; ++v) pre[f][v].assign(S + 1, 0);
  for (int i = 0; i < S; ++i) {
    auto& y = bt->sys[i];
    const int64_t N = y.nb * BS;
    const size_t vb = (size_t)N * bt->Rpad * sizeof(float2);
    for (int k = 0; k < 3; ++k) KPM_TRY(dev_alloc(&y.v[k], vb, s));
    // row partitions: of block rows (BSR) or orbital rows (ELL)
    const int xit[2] = {xitems_for_rows(y.nb, bt->num_sms),
                          xitems_for_rows(N, bt->num_sms)};
    const int xmax = std::max(xit[0], have_ell ? xit[1] : 0);
    KPM_TRY(dev_alloc((void**)&y.partials,
                      (size_t)bt->Rpad * 3 * xmax * sizeof(double), s));
    KPM_TRY(dev_alloc((void**)&y.mu01, (size_t)bt->Rpad * 2 * 16, s));
    KPM_TRY(dev_alloc((void**)&y.mom, (size_t)bt->M * bt->Rpad * 16, s));
    // starting vectors: (seed, system) key
    const uint64_t key = mix64(bt->seed ^ ((uint64_t)i << 32));
    rng_vectors_kernel<<<(unsigned)ceil_div(N * bt->Rpad, 256), 256, 0, s>>>(
        (float2*)y.v[0], N, bt->R, bt->Rpad, key);
    count_launch(1);
    KPM_CHECK_LAUNCH();
    for (int f = 0; f < 2; ++f) {
      hs[f][i] = SysDev{y.nb,     xit[f],  y.bidx,  y.bval, f ? y.ell_k : 0,
                        y.eidx,   y.eval,  y.spidx, y.spval,
                        {y.v[0], y.v[1], y.v[2]}, y.partials, y.mu01,
                        y.mom};
      for (int v = 0; v < 2; ++v)
        pre[f][v][i + 1] =
            pre[f][v][i] + (int64_t)xit[f] * (bt->Rpad / (16 * (v + 1)));
    }
  }
  for (int f = 0; f < (have_ell ? 2 : 1); ++f) {
    KPM_TRY(dev_alloc((void**)&bt->d_sys[f], S * sizeof(SysDev), s));
    KPM_CUDA(cudaMemcpyAsync(bt->d_sys[f], hs[f].data(), S * sizeof(SysDev),
                             cudaMemcpyHostToDevice, s));
    for (int v = 0; v < 2; ++v) {
      KPM_TRY(dev_alloc((void**)&bt->d_prefix[f][v],
                        (S + 1) * sizeof(int64_t), s));
      KPM_CUDA(cudaMemcpyAsync(bt->d_prefix[f][v], pre[f][v].data(),
                               (S + 1) * sizeof(int64_t),
                               cudaMemcpyHostToDevice, s));
      bt->total[f][v] = pre[f][v][S];
    }
  }
  KPM_TRY(dev_alloc((void**)&bt->d_out, (size_t)S * bt->M * 16, s));
  KPM_CUDA(cudaEventCreate(&bt->e0));
  KPM_CUDA(cudaEventCreate(&bt->e1));
  KPM_CUDA(cudaStreamSynchronize(s));

  // autotuner: time three steps of each (format, register budget, work
  // order, VPL) variant; within a format the arithmetic is identical across
  // VPL, budgets and work orders, and the two formats differ only in the
  // order of the dot-product partial sums
  float best = 1e30f;
  int best_fmt = 0, best_occ2 = 0, best_gm = 0;
  const char* force = getenv("KPM_BATCH_FORMAT");
  int f_lo = 0, f_hi = have_ell ? 2 : 0;
  if (have_ell && force && strcmp(force, "ell") == 0) f_lo = f_hi = 1;
  if (have_ell && force && strcmp(force, "sparse") == 0) f_lo = f_hi = 2;
  // work orders: both (BSR, ELL), or the one KPM_BATCH_ORDER names
  const char* ord = getenv("KPM_BATCH_ORDER");
  const int gm_only = ord && strcmp(ord, "partition") == 0 ? 0
                      : ord && strcmp(ord, "group") == 0 ? 1 : -1;
  for (int f = f_lo; f <= f_hi; ++f)
  for (int o2 = 0; o2 < (f ? 1 : 2); ++o2)
  for (int gm = 0; gm < (f == 2 ? 1 : 2); ++gm) {
    if (f != 2 && gm_only >= 0 && gm != gm_only) continue;
    bt->ell = f;
    bt->occ2 = o2;
    bt->gmajor = gm;
    for (int vpl = 1; vpl <= 2; ++vpl) {
      if (bt->Rpad % (16 * vpl)) continue;
      if (o2 && vpl == 1) continue;
      if (f == 2 && vpl == 2) continue;          // sparse-block: 16 vectors
      KPM_TRY(launch_step_phase(bt, vpl, 0));  // warm-up
      KPM_CUDA(cudaEventRecord(bt->e0, s));
      KPM_TRY(launch_step_phase(bt, vpl, 0));
      KPM_TRY(launch_step_phase(bt, vpl, 1));
      KPM_TRY(launch_step_phase(bt, vpl, 2));
      KPM_CUDA(cudaEventRecord(bt->e1, s));
      KPM_TRY(launch_step_phase(bt, vpl, 3));  // (occupancy query before capture)
      KPM_CUDA(cudaEventSynchronize(bt->e1));
      float ms = 0.f;
      KPM_CUDA(cudaEventElapsedTime(&ms, bt->e0, bt->e1));
      if (ms < best) {
        best = ms;
        bt->vpl = vpl;
        best_fmt = f;
        best_occ2 = o2;
        best_gm = gm;
      }
    }
  }
  bt->ell = best_fmt;
  bt->occ2 = best_occ2;
  bt->gmajor = best_gm;
  // keep only the chosen format's matrices (the sparse-block kernel reads
  // the BSR block columns and its own entries)
  for (auto& y : bt->sys) {
    if (bt->ell == 1) {
      dev_free(y.bidx, s);
      dev_free(y.bval, s);
      y.bidx = nullptr;
      y.bval = nullptr;
    }
    if (bt->ell != 1) {
      dev_free(y.eidx, s);
      dev_free(y.eval, s);
      y.eidx = nullptr;
      y.eval = nullptr;
    }
    if (bt->ell != 2) {
      dev_free(y.spidx, s);
      dev_free(y.spval, s);
      y.spidx = nullptr;
      y.spval = nullptr;
    }
  }
  // capture the whole run in a CUDA graph
  KPM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int st = enqueue_run(bt, bt->vpl);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (st != KPM_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  KPM_CUDA(e);
  bt->graph = g;
  KPM_CUDA(cudaGraphInstantiate(&bt->exec, g, 0));
  size_t nn = 0;
  KPM_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
  bt->nodes = (int64_t)nn;
  bt->ready = true;
  return KPM_OK;
}

// Host BSR -> ELL-BSR (diagonal block first, KB blocks per row), scaled.
int upload_bsr(kpm_batch* bt, const kpm_bsr_desc* m, double a, double b,
               kpm_batch::Sys* y) {
  const int64_t nb = m->block_rows;
  KPM_REQUIRE(m->indptr[0] == 0 && m->indptr[nb] == m->nnzb,
              "BSR indptr must start at 0 and end at nnzb");
  std::vector<int32_t> idx((size_t)nb * KB);
  std::vector<float2> val((size_t)nb * KB * 16, make_float2(0.f, 0.f));
  const double sc = 2.0 / a;
  for (int64_t i = 0; i < nb; ++i) {
    KPM_REQUIRE(m->indptr[i] <= m->indptr[i + 1], "BSR indptr not monotone");
    const int64_t cnt = m->indptr[i + 1] - m->indptr[i];
    int64_t diag = -1;
    for (int32_t k = m->indptr[i]; k < m->indptr[i + 1]; ++k) {
      KPM_REQUIRE(m->indices[k] >= 0 && m->indices[k] < nb,
                  "BSR column out of range");
      if (m->indices[k] == i) diag = k;
    }
    KPM_REQUIRE(cnt + (diag < 0 ? 1 : 0) <= KB,
                "BSR row %lld has more than %d blocks", (long long)i, KB);
    int q = 0;
    auto put = [&](int32_t col, const double* blk, bool is_diag) {
      idx[i * KB + q] = col;
      for (int e = 0; e < 16; ++e) {
        double re = blk ? blk[2 * e] : 0.0, im = blk ? blk[2 * e + 1] : 0.0;
        if (is_diag && e % 5 == 0) re -= b;
        val[(i * KB + q) * 16 + e] =
            make_float2((float)(re * sc), (float)(im * sc));
      }
      ++q;
    };
    put((int32_t)i, diag >= 0 ? m->data + 32 * diag : nullptr, true);
    for (int32_t k = m->indptr[i]; k < m->indptr[i + 1]; ++k)
      if (k != diag) put(m->indices[k], m->data + 32 * k, false);
    while (q < KB) put((int32_t)i, nullptr, false);
  }
  KPM_TRY(dev_alloc((void**)&y->bidx, idx.size() * 4, bt->stream));
  KPM_TRY(dev_alloc((void**)&y->bval, val.size() * 8, bt->stream));
  KPM_CUDA(cudaMemcpyAsync(y->bidx, idx.data(), idx.size() * 4,
                           cudaMemcpyHostToDevice, bt->stream));
  KPM_CUDA(cudaMemcpyAsync(y->bval, val.data(), val.size() * 8,
                           cudaMemcpyHostToDevice, bt->stream));
  KPM_CUDA(cudaStreamSynchronize(bt->stream));
  return KPM_OK;
}

}  // namespace

extern "C" {

int kpm_batch_create(int64_t num_vectors, int64_t num_moments, uint64_t seed,
                     kpm_batch** out) {
  KPM_REQUIRE(out && num_vectors > 0 && num_moments >= 2 &&
                  num_moments % 2 == 0,
              "kpm_batch_create: need num_vectors > 0 and an even "
              "num_moments >= 2");
  auto* bt = new kpm_batch();
  bt->R = num_vectors;
  bt->Rpad = round_up(num_vectors, 32);
  bt->M = num_moments;
  bt->seed = seed;
  int st = init_device(&bt->device, &bt->num_sms);
  if (st == KPM_OK &&
      cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) !=
          cudaSuccess) {
    set_error("kpm_batch_create: stream creation failed");
    st = KPM_ECUDA;
  }
  if (st != KPM_OK) {
    batch_free(bt);
    return st;
  }
  *out = bt;
  return KPM_OK;
}

int kpm_batch_add_bsr(kpm_batch* bt, const kpm_bsr_desc* ham, double a,
                      double b) {
  KPM_REQUIRE(bt && ham && ham->indptr && ham->indices && ham->data,
              "kpm_batch_add_bsr: null argument");
  KPM_REQUIRE(!bt->ready, "kpm_batch_add_bsr: batch already run");
  KPM_REQUIRE(ham->block_rows > 0 && ham->block_rows * BS < INT32_MAX,
              "kpm_batch_add_bsr: invalid size");
  KPM_REQUIRE(a > 0 && std::isfinite(a) && std::isfinite(b),
              "kpm_batch_add_bsr: scale a must be positive");
  kpm_batch::Sys y;
  y.nb = ham->block_rows;
  y.a = a;
  y.b = b;
  int st = upload_bsr(bt, ham, a, b, &y);
  bt->sys.push_back(y);  // freed with the batch even on failure
  return st;
}

int kpm_batch_add_wilson_dirac(kpm_batch* bt, int64_t L, double m, double W,
                               uint64_t seed, double a, double b) {
  KPM_REQUIRE(bt, "kpm_batch_add_wilson_dirac: null batch");
  KPM_REQUIRE(!bt->ready, "kpm_batch_add_wilson_dirac: batch already run");
  KPM_REQUIRE(L >= 2 && L * L * L * BS < INT32_MAX,
              "kpm_batch_add_wilson_dirac: invalid L");
  KPM_REQUIRE(a > 0 && std::isfinite(a), "scale a must be positive");
  // Gamma matrices: G0 = tau_z (x) s0, Gj = tau_x (x) sj
  auto kron = [](const double t[2][2][2], const double s[2][2][2],
                 double out[4][4][2]) {
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k)
          for (int l = 0; l < 2; ++l) {
            const double ar = t[i][j][0], ai = t[i][j][1];
            const double br = s[k][l][0], bi = s[k][l][1];
            out[2 * i + k][2 * j + l][0] = ar * br - ai * bi;
            out[2 * i + k][2 * j + l][1] = ar * bi + ai * br;
          }
  };
  const double s0[2][2][2] = {{{1, 0}, {0, 0}}, {{0, 0}, {1, 0}}};
  const double sx[2][2][2] = {{{0, 0}, {1, 0}}, {{1, 0}, {0, 0}}};
  const double sy[2][2][2] = {{{0, 0}, {0, -1}}, {{0, 1}, {0, 0}}};
  const double sz[2][2][2] = {{{1, 0}, {0, 0}}, {{0, 0}, {-1, 0}}};
  double G0[4][4][2], Gj[3][4][4][2];
  kron(sz, s0, G0);
  kron(sx, sx, Gj[0]);
  kron(sx, sy, Gj[1]);
  kron(sx, sz, Gj[2]);
  WdBlocks blk;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      blk.diag[4 * r + c] =
          make_float2((float)((m - 3) * G0[r][c][0]), 0.f);
      for (int j = 0; j < 3; ++j) {
        // T = (G0 - i Gj) / 2 ;  T[r][c]
        const double tr = (G0[r][c][0] + Gj[j][r][c][1]) / 2;
        const double ti = (G0[r][c][1] - Gj[j][r][c][0]) / 2;
        blk.bwd[j][4 * r + c] = make_float2((float)tr, (float)ti);
        // T^dagger[r][c] = conj(T[c][r])
        const double ur = (G0[c][r][0] + Gj[j][c][r][1]) / 2;
        const double ui = (G0[c][r][1] - Gj[j][c][r][0]) / 2;
        blk.fwd[j][4 * r + c] = make_float2((float)ur, (float)(-ui));
      }
    }
  kpm_batch::Sys y;
  y.nb = L * L * L;
  y.a = a;
  y.b = b;
  int st = dev_alloc((void**)&y.bidx, (size_t)y.nb * KB * 4, bt->stream);
  if (st == KPM_OK)
    st = dev_alloc((void**)&y.bval, (size_t)y.nb * KB * 16 * 8, bt->stream);
  if (st == KPM_OK) {
    wd_generate_kernel<<<(unsigned)ceil_div(y.nb, 256), 256, 0, bt->stream>>>(
        L, blk, W, mix64(seed), 2.0 / a, b, y.bidx, y.bval);
    count_launch(1);
    if (cudaGetLastError() != cudaSuccess ||
        cudaStreamSynchronize(bt->stream) != cudaSuccess) {
      set_error("kpm_batch_add_wilson_dirac: generation failed");
      st = KPM_ECUDA;
    }
  }
  bt->sys.push_back(y);
  return st;
}

int kpm_batch_run(kpm_batch* bt, double* out) {
  NvtxRange nvtx("kpm_batch_run");
  KPM_REQUIRE(bt && out, "kpm_batch_run: null argument");
  if (!bt->ready) KPM_TRY(prepare(bt));
  KPM_CUDA(cudaEventRecord(bt->e0, bt->stream));
  KPM_CUDA(cudaGraphLaunch(bt->exec, bt->stream));
  KPM_CUDA(cudaEventRecord(bt->e1, bt->stream));
  KPM_CUDA(cudaMemcpyAsync(out, bt->d_out, bt->sys.size() * bt->M * 16,
                           cudaMemcpyDeviceToHost, bt->stream));
  KPM_CUDA(cudaStreamSynchronize(bt->stream));
  float ms = 0.f;
  KPM_CUDA(cudaEventElapsedTime(&ms, bt->e0, bt->e1));
  bt->last_ms = ms;
  return KPM_OK;
}

int kpm_batch_stats(kpm_batch* bt, double* ms, int64_t* nodes,
                    int* vectors_per_lane) {
  KPM_REQUIRE(bt && ms && nodes && vectors_per_lane,
              "kpm_batch_stats: null argument");
  *ms = bt->last_ms;
  *nodes = bt->nodes;
  *vectors_per_lane = bt->vpl;
  return KPM_OK;
}

int kpm_batch_format(kpm_batch* bt, int* format, int* ell_width) {
  KPM_REQUIRE(bt && format && ell_width, "kpm_batch_format: null argument");
  *format = bt->ell;
  *ell_width = 0;
  if (bt->ell == 1)
    for (auto& y : bt->sys) *ell_width = std::max(*ell_width, y.ell_k);
  return KPM_OK;
}

int kpm_batch_order(kpm_batch* bt, int* group_major) {
  KPM_REQUIRE(bt && group_major, "kpm_batch_order: null argument");
  *group_major = bt->gmajor;
  return KPM_OK;
}

int kpm_batch_destroy(kpm_batch* bt) { return batch_free(bt); }

}  // extern "C"
