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
// to ~2^-38 (relative to the anchor below) with error-free FP32
// transformations before splitting it again:
//   * the hi products h * x_hi are accumulated from an anchor C = 32: every
//     partial sum stays within a factor two of the previous one, so
//     s1 = fma(h, x, s), m = s - s1 (exact, Sterbenz) and e = fma(h, x, m)
//     give the rounding error of each fused multiply-add exactly; the errors
//     are summed in FP32 (they are ~2^-19 each).  Components far below the
//     anchor (|x| < ~1e-5, the decaying tails of a localised vector) keep
//     only FP32 precision; their share of every moment is as small;
//   * the lo products h * x_lo (and the lo part of a_{n-1}) are one FP32
//     sum: a 2^-24 error on a 2^-24-relative quantity;
//   * hi = RN(v), lo = RZ_bf16(RZ(v - hi)): round toward zero keeps |lo| at
//     most half an ulp of hi, so the split is unique and a vector downloaded
//     as complex128 (hi + lo, exact) uploads to the same hi and lo.
// The fused dot products use the hi parts.  mu_0 and mu_1 come from hi + lo
// once, as compensated sums (FP64 products per row took 4.6x a recursion
// step on GB300's narrow FP64 pipe).  Then <a_n|a_n> is summed with
// Ogita-Rump-Oishi Dot2 (TwoProd + TwoSum), Re and Im <a_n+1|a_n> as plain
// FP32 sums, all flushed to FP64 every 128 rows.  Leaving out lo in these
// dots is a zero-mean error of each moment alone, not a shift of all of
// them.  The sums of |a_i|^2 need the compensation: their terms are all
// positive, and plain FP32 partials (flushed every 128 or 32 rows) took the
// per-orbital DOS error at the outermost node of the 2e6-orbital workload
// to 1.0e-4 or 1.0e-5 (2.6e-7 with Dot2).  The terms of <a_n+1|a_n> change
// sign; a plain sum there left the error at 2.6e-7 and saved 0.7 % of the
// step.  (An anchored sum with a per-vector anchor >= 4 mu_0, which bounds
// every partial sum, was measured too: the anchor is then far above a
// row's terms, their fractional parts land in the FP32 residual sum, and
// its bias took the outer-node error from 2.6e-7 to 1.7e-5.)
//
// The H values themselves stay complex64 (2H/a): rounding them perturbs the
// Hamiltonian, whose moments are still those of a Hermitian operator, and
// leaves the reconstruction consistent (a ~1e-7 relative shift of the
// spectrum, not noise).

#include <type_traits>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// anchor of the compensated row sums (partial sums within C/2 of it keep
// the captured rounding errors exact; larger ones lose the compensation
// gracefully, not the hi part)
constexpr float HILO_ANCHOR = 32.0f;

// Packed (re, im) pairs: every operation below runs on a float2 with one
// FFMA2 / FADD2 / FMUL2 instruction.  Intrinsics only: nothing may be
// contracted or reassociated in the error-free transformations.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);   // a - b, one rounding
}
// s + a*b with its rounding error added to c (exact while s stays within a
// factor two of the anchor)
__device__ __forceinline__ void acc_fma(float2& s, float2& c, float2 a,
                                        float2 b) {
  const float2 s1 = __ffma2_rn(a, b, s);
  const float2 m = sub2(s, s1);
  c = __fadd2_rn(c, __ffma2_rn(a, b, m));
  s = s1;
}
// s - b with its rounding error added to c
__device__ __forceinline__ void acc_sub(float2& s, float2& c, float2 b) {
  const float2 s1 = sub2(s, b);
  const float2 m = sub2(s, s1);
  c = __fadd2_rn(c, sub2(m, b));
  s = s1;
}
// Dot2 accumulation of a*b into (s, c) (Ogita, Rump & Oishi 2005: TwoProd
// by FMA, Knuth's TwoSum; scale-invariant)
__device__ __forceinline__ void dot2(float2& s, float2& c, float2 a,
                                     float2 b) {
  const float2 p = __fmul2_rn(a, b);
  const float2 pe =
      __ffma2_rn(a, b, __fmul2_rn(p, make_float2(-1.f, -1.f)));
  const float2 t = __fadd2_rn(s, p);
  const float2 z = sub2(t, s);
  const float2 e = __fadd2_rn(sub2(s, sub2(t, z)), sub2(p, z));
  s = t;
  c = __fadd2_rn(c, __fadd2_rn(e, pe));
}
// value of a compensated pair in FP64, both halves
__device__ __forceinline__ double pair_sum(float2 s, float2 c) {
  return ((double)s.x + (double)s.y) + ((double)c.x + (double)c.y);
}
// bfloat16 pair word (re in the low half) -> (re, im)
__device__ __forceinline__ float2 lo_pair(uint32_t w) {
  return make_float2(__uint_as_float(w << 16),
                     __uint_as_float(w & 0xffff0000u));
}
// truncate (re, im) to bfloat16 (round toward zero): re in the low half
__device__ __forceinline__ uint32_t lo_pack_rz(float2 v) {
  return __byte_perm(__float_as_uint(v.x), __float_as_uint(v.y), 0x7632);
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Block shape: each thread stages, per chunk of four ELL entries of a row,
// the four gathered rows (24 bytes each, hi and lo), plus alpha_{n-1} with
// the last chunk and the row's own x with the first (unless it is the
// first gathered row, D0), double-buffered.  The staging does not grow with
// the ELL width, so every width runs two blocks of 256 threads per SM
// (16 warps).  When every slice of a row was staged at once, an ELL width
// of 16 left room for 6 warps per SM and the step took 2.8x the time per
// orbital and vector of the 4-wide graphene rows.
template <int K, bool D0> struct HiloCfg {
  static constexpr int THREADS = 256;
  static constexpr int MIN_BLOCKS = 2;
  static constexpr int CHUNKS = K / 4;          // ELL entries in groups of 4
  static constexpr int ITEMS = 4 + (D0 ? 1 : 2);
  // staged item indices: the row's own x, alpha_{n-1}, first gathered row
  static constexpr int OWN = D0 ? 1 : 0;
  static constexpr int PREV = D0 ? 0 : 1;
  static constexpr int GATH = D0 ? 1 : 2;
  static constexpr int NW = THREADS / 32;
  static constexpr int NSLOT = THREADS / 8;
  // ELL values: D0 copies hold them pre-broadcast, (hr, hr, hi, hi), so
  // that the packed products need no register moves
  using VT = typename std::conditional<D0, float4, float2>::type;
  static constexpr size_t SMEM =
      2 * ITEMS * THREADS * (sizeof(float4) + sizeof(uint2)) +
      NW * 3 * 4 * K * (sizeof(int32_t) + sizeof(VT)) +
      NSLOT * 48 * sizeof(double);
};

// The step over 16-vector sub-groups in 8-lane slots whose lanes hold two
// complex64 vectors each (a float4 of hi parts, a uint2 of lo parts).  A
// warp's four slots walk adjacent rows.  A row is computed in chunks of
// four ELL entries; while a thread computes one chunk it copies the slices
// of its next chunk (the next row's first chunk after the last) into shared
// memory with cp.async, and the warp's ELL entries are staged two rows
// ahead (their column indices address those copies), so the memory latency
// of a chunk overlaps the previous chunk's arithmetic.  The entries of a row
// are summed in ELL order whatever the chunking.  MODE STEP_FIRST:
// a_1 = H~ a_0 with the dots mu_0 = <a_0|a_0> and <a_1|a_0> of hi + lo;
// STEP_RECUR: a_{n+1} = 2 H~ a_n - a_{n-1} with the compensated dots
// <a_n|a_n>, <a_n+1|a_n>.
//
// Per vector, P = sum hr (xr, xi) and Q = sum hi (xr, xi) (the diagonal
// shift and -a_{n-1} go into P) are anchored compensated sums, so
// re = P.x - Q.y and im = P.y + Q.x recombine exactly: both anchored sums
// lie in the anchor's binade, their difference is exact (Sterbenz) and the
// sum of their offsets from the anchor fits in 24 bits.
//
// D0: the ELL rows hold the diagonal entry first, with the shift folded in
// and a zero imaginary part (prepare_hilo); the own x is then the first
// gathered row, and the diagonal contributes to P only.
template <int K, int MODE, bool D0>
__global__ void __launch_bounds__(HiloCfg<K, D0>::THREADS,
                                  HiloCfg<K, D0>::MIN_BLOCKS)
cheb_step_hilo_kernel(StepArgs p, HiloArgs q,
                      const int32_t* __restrict__ eidx,
                      const typename HiloCfg<K, D0>::VT* __restrict__ eval) {
  using Cfg = HiloCfg<K, D0>;
  using VT = typename Cfg::VT;
  constexpr int OWN = Cfg::OWN, PREV = Cfg::PREV, GATH = Cfg::GATH;
  constexpr int CHUNKS = Cfg::CHUNKS;
  constexpr int T = Cfg::THREADS, ITEMS = Cfg::ITEMS, NSLOT = Cfg::NSLOT;
  constexpr int SW = 8, G = 16, SPW = 4, FLUSH = 128;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* vhi = reinterpret_cast<float4*>(smem);              // [2][ITEMS][T]
  uint2* vlo = reinterpret_cast<uint2*>(vhi + 2 * ITEMS * T);  // [2][ITEMS][T]
  int32_t* sidx = reinterpret_cast<int32_t*>(vlo + 2 * ITEMS * T);
  VT* sval = reinterpret_cast<VT*>(sidx + Cfg::NW * 3 * 4 * K);
  double* red = reinterpret_cast<double*>(sval + Cfg::NW * 3 * 4 * K);

  const int tid = threadIdx.x;
  const int lane = tid & (SW - 1);
  const int slot = tid / SW;
  const int wq = slot / SPW, half = slot % SPW, wl = tid & 31;
  int32_t* widx = sidx + wq * 3 * 4 * K;   // this warp's ring: [3][SPW * K]
  VT* wval = sval + wq * 3 * 4 * K;

  const float4* __restrict__ x = reinterpret_cast<const float4*>(p.x);
  const float4* prev = reinterpret_cast<const float4*>(p.prev);
  float4* out = reinterpret_cast<float4*>(p.out);
  const uint2* __restrict__ xl = reinterpret_cast<const uint2*>(q.xlo);
  const uint2* pl = reinterpret_cast<const uint2*>(q.plo);
  uint2* ol = reinterpret_cast<uint2*>(q.olo);
  const int work = p.xitems * p.groups;
  const int rows = (int)p.rows;
  const int stride = p.xitems * NSLOT;
  const float2 shift = f2(p.shift);
  // lane payloads per row, the same for the hi (float4) and lo (uint2)
  // arrays: element offsets are one 32 x 32 -> 64-bit multiply per row
  const uint32_t rp = (uint32_t)p.rp;
  auto off = [rp](int row, int col) -> int64_t {
    return (int64_t)((uint64_t)(uint32_t)row * rp) + col;
  };
  const float C = HILO_ANCHOR;

  // ELL entries of the warp's rows r0 .. r0 + 3 into ring buffer b
  auto stage_ell = [&](int r0, int b) {
    constexpr int EPC = 16 / (int)sizeof(VT);   // values per 16-byte chunk
    constexpr int IC = SPW * K / 4, VC = SPW * K / EPC;
    for (int c = wl; c < IC + VC; c += 32) {
      if (c < IC) {
        if (r0 + (4 * c) / K < rows)
          cp_async16(widx + b * 4 * K + 4 * c, eidx + (int64_t)r0 * K + 4 * c);
      } else {
        const int e = c - IC;
        if (r0 + (EPC * e) / K < rows)
          cp_async16(wval + b * 4 * K + EPC * e,
                     eval + (int64_t)r0 * K + EPC * e);
      }
    }
  };
  // this thread's slices of chunk c of row r (ELL entries in ring buffer
  // eb) into vector buffer vb: the four gathered rows, the own x with the
  // first chunk (unless D0) and alpha_{n-1} with the last
  auto stage_vec = [&](int r, int vb, int eb, int col, int c) {
    if (r >= rows) return;
    float4* dh = vhi + vb * ITEMS * T + tid;
    uint2* dl = vlo + vb * ITEMS * T + tid;
    const int64_t o = off(r, col);
    if constexpr (!D0) {
      if (c == 0) {
        cp_async16(dh + OWN * T, x + o);
        cp_async8(dl + OWN * T, xl + o);
      }
    }
    if constexpr (MODE == STEP_RECUR) {
      if (c == CHUNKS - 1) {
        cp_async16(dh + PREV * T, prev + o);
        cp_async8(dl + PREV * T, pl + o);
      }
    }
    const int32_t* ci = widx + eb * 4 * K + half * K + 4 * c;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t oc = off(col_index(p, ci[t]), col);
      cp_async16(dh + (GATH + t) * T, x + oc);
      cp_async8(dl + (GATH + t) * T, xl + oc);
    }
  };

  // work order: pairs of sub-groups, partition by partition (the two
  // sub-groups of a partition run side by side and share its ELL rows in
  // L2), the next pair after all partitions.  Against all sub-groups of a
  // partition side by side, the resident blocks then cover twice as many
  // consecutive rows, so more of the gathered neighbours are still in L2,
  // for one more read of the ELL rows per pair.  Measured on the 2e6-orbital
  // graphene workload: R = 64 0.973 ms per step against 0.987 (0.713 /
  // 0.703 of HBM), R = 128 1.961 against 2.135 ms; one sub-group at a time
  // took 1.029 ms (R = 64).  The Wilson-Dirac systems (R = 256, width 16):
  // 7.05 s against 7.14 s per run of four.  Results are identical in every
  // order.  Blocks of 192 or 160 threads (3 or 4 per SM) were slower
  // (1.15-1.22 ms at the time), and so were blocks of 128 threads at 4 or 5
  // per SM (1.03 and 1.33 ms against 1.01 ms).  The gathered hi slices are
  // copied through L2 only (cp.async.cg): 1.026 -> 1.010 ms against copies
  // that also allocate in L1 (15 % L1 hit rate)
  const int pair = p.groups < 2 ? p.groups : 2;
  for (int w = blockIdx.x; w < work; w += gridDim.x) {
    const int g0 = (w / (p.xitems * pair)) * pair;   // first of this pair
    const int npair = p.groups - g0 < pair ? p.groups - g0 : pair;
    const int rem = w - g0 * p.xitems;               // < xitems * npair
    const int xi = rem / npair;
    const int g = g0 + (rem - xi * npair);
    const int col = g * SW + lane;
    double* my = red + slot * (G * 3) + lane * 6;   // vectors 2 lane, +1
#pragma unroll
    for (int e = 0; e < 6; ++e) my[e] = 0.0;
    // FP32 dots (STEP_RECUR): <a_n|a_n> as compensated (xr^2, xi^2) sums,
    // Re <a_n+1|a_n> as plain (or xr, oi xi) sums, Im plain
    // (STEP_FIRST: all three compensated, the products with lo parts added
    // to the compensation terms)
    float2 dns[2], dnc[2], drs[2], drc[2], dis[2], dic[2];
    float fim[2];
    auto clear_dots = [&]() {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        dns[k] = dnc[k] = drs[k] = drc[k] = dis[k] = dic[k] =
            make_float2(0.f, 0.f);
        fim[k] = 0.f;
      }
    };
    // add the FP32 partials to the slot's FP64 accumulators
    auto flush_dots = [&]() {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        my[k * 3 + 0] += pair_sum(dns[k], dnc[k]);
        if constexpr (MODE == STEP_FIRST) {
          my[k * 3 + 1] += pair_sum(drs[k], drc[k]);
          my[k * 3 + 2] += pair_sum(dis[k], dic[k]);
        } else {
          my[k * 3 + 1] += (double)drs[k].x + (double)drs[k].y;
          my[k * 3 + 2] += (double)fim[k];
        }
      }
      clear_dots();
    };
    clear_dots();
    int pending = 0;

    const int wb0 = xi * NSLOT + SPW * wq;
    stage_ell(wb0, 0);
    cp_async_commit();
    stage_ell(wb0 + stride, 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    stage_vec(wb0 + half, 0, 0, col, 0);
    cp_async_commit();
    int e0 = 0, e1 = 1, e2 = 2, vb = 0;   // ring positions of rows it, +1, +2
    for (int wb = wb0; wb < rows; wb += stride) {
      const int r = wb + half;
      // the row's state across its chunks
      float2 xk[2], Ps[2], Pc[2], Qs[2], Qc[2], LP[2], LQ[2];
      uint32_t xlw[2];
#pragma unroll
      for (int c = 0; c < CHUNKS; ++c) {
        if (c == 0) {
          stage_ell(wb + 2 * stride, e2);
          cp_async_commit();
          // pending groups: ELL(it + 1), vectors(it, 0), ELL(it + 2)
          cp_async_wait<1>();
        } else {
          cp_async_wait<0>();          // vectors(it, c), ELL(it + 2)
        }
        __syncwarp();
        if (c + 1 < CHUNKS)
          stage_vec(r, vb ^ 1, e0, col, c + 1);
        else
          stage_vec(wb + stride + half, vb ^ 1, e1, col, 0);
        cp_async_commit();
        if (r < rows) {
          const float4* sh = vhi + vb * ITEMS * T + tid;
          const uint2* sl = vlo + vb * ITEMS * T + tid;
          if (c == 0) {
            const float4 xo = sh[OWN * T];
            const uint2 xol = sl[OWN * T];
            xk[0] = make_float2(xo.x, xo.y);
            xk[1] = make_float2(xo.z, xo.w);
            xlw[0] = xol.x;
            xlw[1] = xol.y;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              Ps[k] = Qs[k] = f2(C);
              Pc[k] = Qc[k] = LQ[k] = make_float2(0.f, 0.f);
              if constexpr (D0) {
                LP[k] = make_float2(0.f, 0.f);
              } else {
                acc_fma(Ps[k], Pc[k], shift, xk[k]);
                LP[k] = __fmul2_rn(shift, lo_pair(xlw[k]));
              }
            }
          }
          const VT* hv = wval + e0 * 4 * K + half * K + 4 * c;
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            float2 hr, hi;
            if constexpr (D0) {
              const float4 h = hv[t];
              hr = make_float2(h.x, h.y);
              hi = make_float2(h.z, h.w);
            } else {
              const float2 h = hv[t];
              hr = f2(h.x);
              hi = f2(h.y);
            }
            const float4 gx = sh[(GATH + t) * T];
            const uint2 gl = sl[(GATH + t) * T];
            const float2 gk[2] = {make_float2(gx.x, gx.y),
                                  make_float2(gx.z, gx.w)};
            const uint32_t glw[2] = {gl.x, gl.y};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              acc_fma(Ps[k], Pc[k], hr, gk[k]);
              const float2 l = lo_pair(glw[k]);
              LP[k] = __ffma2_rn(hr, l, LP[k]);
              if (!D0 || c > 0 || t > 0) {   // a D0 row's first entry is real
                acc_fma(Qs[k], Qc[k], hi, gk[k]);
                LQ[k] = __ffma2_rn(hi, l, LQ[k]);
              }
            }
          }
          if (c == CHUNKS - 1) {
            if constexpr (MODE == STEP_RECUR) {
              const float4 pv = sh[PREV * T];
              const uint2 plv = sl[PREV * T];
              const float2 pk[2] = {make_float2(pv.x, pv.y),
                                    make_float2(pv.z, pv.w)};
              const uint32_t plw[2] = {plv.x, plv.y};
#pragma unroll
              for (int k = 0; k < 2; ++k) {
                acc_sub(Ps[k], Pc[k], pk[k]);
                LP[k] = sub2(LP[k], lo_pair(plw[k]));
              }
            }
            float2 ohi[2];
            uint32_t olw[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              // v = (re, im) of the anchored sums (exact), cc = their
              // compensation plus the lo bracket
              const float2 v = make_float2(
                  __fsub_rn(Ps[k].x, Qs[k].y),
                  __fadd_rn(__fsub_rn(Ps[k].y, C), __fsub_rn(Qs[k].x, C)));
              const float2 cc = make_float2(
                  __fadd_rn(__fsub_rn(Pc[k].x, Qc[k].y),
                            __fsub_rn(LP[k].x, LQ[k].y)),
                  __fadd_rn(__fadd_rn(Pc[k].y, Qc[k].x),
                            __fadd_rn(LP[k].y, LQ[k].x)));
              float2 h = __fadd2_rn(v, cc);                 // hi = RN(v)
              float2 l = __fadd2_rz(sub2(v, h), cc);        // lo = RZ(v - hi)
              if constexpr (MODE == STEP_FIRST) {   // a_1 = (2 H~ a_0) / 2
                h = __fmul2_rn(h, f2(0.5f));
                l = __fmul2_rn(l, f2(0.5f));
              }
              ohi[k] = h;
              olw[k] = lo_pack_rz(l);
            }
            const int64_t o = off(r, col);
            out[o] = make_float4(ohi[0].x, ohi[0].y, ohi[1].x, ohi[1].y);
            ol[o] = make_uint2(olw[0], olw[1]);
            if constexpr (MODE == STEP_FIRST) {
              // mu_0 and <a_1|a_0> of a = hi + lo: Dot2 on the hi products, the
              // products with a lo part (2^-8 of them, relative) as FP32 sums
              // into the compensation terms
#pragma unroll
              for (int k = 0; k < 2; ++k) {
                const float2 al = lo_pair(xlw[k]), bl = lo_pair(olw[k]);
                dot2(dns[k], dnc[k], xk[k], xk[k]);
                dnc[k] = __ffma2_rn(__fmul2_rn(f2(2.f), xk[k]), al, dnc[k]);
                dnc[k] = __ffma2_rn(al, al, dnc[k]);
                // Re <a_1|a_0> = br ar + bi ai
                dot2(drs[k], drc[k], ohi[k], xk[k]);
                drc[k] = __ffma2_rn(ohi[k], al, drc[k]);
                drc[k] = __ffma2_rn(bl, __fadd2_rn(xk[k], al), drc[k]);
                // Im <a_1|a_0> = br ai - bi ar
                const float2 u = make_float2(ohi[k].x, -ohi[k].y);
                const float2 ul = make_float2(bl.x, -bl.y);
                const float2 v = make_float2(xk[k].y, xk[k].x);
                const float2 vl = make_float2(al.y, al.x);
                dot2(dis[k], dic[k], u, v);
                dic[k] = __ffma2_rn(u, vl, dic[k]);
                dic[k] = __ffma2_rn(ul, __fadd2_rn(v, vl), dic[k]);
              }
            } else {
#pragma unroll
              for (int k = 0; k < 2; ++k) {
                dot2(dns[k], dnc[k], xk[k], xk[k]);
                drs[k] = __ffma2_rn(ohi[k], xk[k], drs[k]);
                fim[k] = fmaf(ohi[k].x, xk[k].y,
                              fmaf(-ohi[k].y, xk[k].x, fim[k]));
              }
            }
            if (++pending == FLUSH) {
              flush_dots();
              pending = 0;
            }
          }
        }
        __syncwarp();
        vb ^= 1;
      }
      const int e_old = e0;
      e0 = e1;
      e1 = e2;
      e2 = e_old;
    }
    cp_async_wait<0>();
    flush_dots();
    __syncthreads();
    // partials are addressed by vector: [vector*3 + component][xitems]
    double* dst = p.partials + (int64_t)g * (G * 3) * p.xitems + xi;
    for (int e = tid; e < G * 3; e += T) {
      double s = 0.0;
#pragma unroll
      for (int sl = 0; sl < NSLOT; ++sl) s += red[sl * (G * 3) + e];
      dst[(int64_t)e * p.xitems] = s;
    }
    __syncthreads();
  }
}

template <int K, int MODE, bool D0>
static int launch_hilo_t(kpm_handle* h, const StepArgs& a,
                         const HiloArgs& q) {
  using Cfg = HiloCfg<K, D0>;
  static int occ = -1;
  if (occ < 0) {
    KPM_CUDA(cudaFuncSetAttribute(cheb_step_hilo_kernel<K, MODE, D0>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)Cfg::SMEM));
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, cheb_step_hilo_kernel<K, MODE, D0>, Cfg::THREADS,
        Cfg::SMEM));
    occ = blocks > 0 ? blocks : 1;
  }
  const int64_t work = (int64_t)a.xitems * a.groups;
  int64_t grid = (int64_t)occ * h->num_sms;
  if (grid > work) grid = work;
  cudaEvent_t e1 = nullptr;
  KPM_TRY(prof_begin(h, &e1));
  cheb_step_hilo_kernel<K, MODE, D0>
      <<<(unsigned)grid, Cfg::THREADS, Cfg::SMEM, h->stream>>>(
          a, q, D0 ? h->dg_idx : h->H.ell_idx,
          reinterpret_cast<const typename Cfg::VT*>(
              D0 ? (const void*)h->dg_val : (const void*)h->H.ell_val));
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (e1) KPM_CUDA(cudaEventRecord(e1, h->stream));
  return KPM_OK;
}

template <int K>
static int dispatch_hilo_k(kpm_handle* h, int mode, const StepArgs& a,
                           const HiloArgs& q) {
  if (h->dg_ok)
    return mode == STEP_FIRST ? launch_hilo_t<K, STEP_FIRST, true>(h, a, q)
                              : launch_hilo_t<K, STEP_RECUR, true>(h, a, q);
  return mode == STEP_FIRST ? launch_hilo_t<K, STEP_FIRST, false>(h, a, q)
                            : launch_hilo_t<K, STEP_RECUR, false>(h, a, q);
}

// Diagonal-first copy of the ELL rows: the first entry whose column is the
// row (a CSR diagonal, or else the zero padding entry) moves to slot 0 with
// the shift added to its value; the other entries keep their order.  *bad
// is set when a row has no such entry or a diagonal with a nonzero
// imaginary part.
__global__ void diag_first_kernel(int64_t n, int K,
                                  const int32_t* __restrict__ eidx,
                                  const float2* __restrict__ eval,
                                  float shift, int32_t* __restrict__ oidx,
                                  float4* __restrict__ oval, int* bad) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t* ri = eidx + r * K;
  const float2* rv = eval + r * K;
  int d = -1;
  for (int t = 0; t < K; ++t)
    if (ri[t] == (int32_t)r) {
      d = t;
      break;
    }
  if (d < 0 || rv[d].y != 0.f) {
    atomicOr(bad, 1);
    d = -1;
  }
  int o = 0;
  if (d >= 0) {
    oidx[r * K] = (int32_t)r;
    const float dv = __fadd_rn(rv[d].x, shift);
    oval[r * K] = make_float4(dv, dv, 0.f, 0.f);
    o = 1;
  }
  for (int t = 0; t < K; ++t) {
    if (t == d) continue;
    oidx[r * K + o] = ri[t];
    oval[r * K + o] = make_float4(rv[t].x, rv[t].x, rv[t].y, rv[t].y);
    ++o;
  }
}

int prepare_hilo(kpm_handle* h) {
  const int K = h->H.ell_k;
  if (K == 0) return KPM_OK;
  const int64_t n = h->H.rows;
  const size_t cnt = (size_t)n * K;
  if (!h->dg_idx) {
    KPM_TRY(dev_alloc((void**)&h->dg_idx, cnt * sizeof(int32_t), h->stream));
    KPM_TRY(dev_alloc((void**)&h->dg_val, cnt * sizeof(float4), h->stream));
    KPM_TRY(dev_alloc((void**)&h->dg_flag, sizeof(int), h->stream));
  }
  KPM_CUDA(cudaMemsetAsync(h->dg_flag, 0, sizeof(int), h->stream));
  diag_first_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, h->stream>>>(
      n, K, h->H.ell_idx, h->H.ell_val, (float)(-2.0 * h->b / h->a),
      h->dg_idx, h->dg_val, h->dg_flag);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  int bad = 0;
  KPM_CUDA(cudaMemcpyAsync(&bad, h->dg_flag, sizeof(int),
                           cudaMemcpyDeviceToHost, h->stream));
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  h->dg_ok = bad == 0;
  return KPM_OK;
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
  wq.lrp = rpad / 2;   // the kernel addresses lo with the hi stride
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
