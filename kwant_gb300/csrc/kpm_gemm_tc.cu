// Tensor-core (tcgen05) contraction of the correlator moments matrix.
//
//   mu_mn = (1/R) sum_K conj(Omega[m][K]) Psi[n][K]
//
// (Correlator._calculate_moments_matrix, kwant/kpm.py:685-695) on BF16x3
// stores: every real component x is held as hi = bf16(x), lo = bf16(x - hi),
// in four K-major planes (re_hi, re_lo, im_hi, im_lo); FP16 stores hold
// hi = half(x), lo = half(x - hi) in the same layout and run the same MMAs
// with both operand formats set to FP16 (~2^-22 instead of ~2^-16 relative
// per product, for the same time).  With A = Omega,
// B = Psi:
//   Re mu = Ar Br^T + Ai Bi^T,   Im mu = Ar Bi^T - Ai Br^T,
// and every real product X Y^T is formed as Xh Yh^T + Xh Yl^T + Xl Yh^T
// (the lo*lo term, ~2^-16 relative, is dropped): 12 BF16 MMAs per K step,
// FP32 accumulation in tensor memory, the minus sign through the MMA's
// negate-A bit.
//
// One CTA computes a 128 x NT output tile of both Re and Im over one K range
// (split-K); 6 warps: warp 0 allocates TMEM and issues the TMA loads (one 4D
// box per operand = its four planes of one K block of the K-blocked store),
// warp 1 issues the MMAs from one thread, warps 2-5 (one per quarter of the
// TMEM lanes) drain the accumulators.  Pipeline stages of 32 K-elements
// (64-byte swizzle), as many as the shared memory holds.
//
// Accumulation runs: the MMAs accumulate `promote` K chunks (1024 K
// elements by default) into TMEM columns [0, 2 NT), then the MMA thread
// commits to `promo` and waits on `resume`; the drain warps add the run's
// sums into a master copy in columns [2 NT, 4 NT) (FP32, round to nearest;
// the first run is copied) and arrive on `resume`, and the next run's first
// MMA overwrites the accumulators.  After the last run the drain warps write
// accumulators + master to this split's FP32 partials, which are summed in
// FP64 in a fixed order.  The tensor cores' FP32 accumulation error grows
// with the products summed into one accumulator; the runs bound that count.
// 256-wide tiles (2 NT = 512 columns) leave no room for the master copy and
// run one accumulation per split.
//
// Every wait on an mbarrier is bounded (2 s of GPU time by default,
// KPM_DEBUG_WAIT_NS); on expiry the kernel records an error code and stops
// issuing work: the producer waits for the loads it already issued, each
// drain warp decides from one lane whether it reads tensor memory (its
// warp-collective accesses never diverge), the MMA thread always commits
// `done`, which thread 0 awaits before the CTA releases its tensor memory,
// and the host reports KPM_ETIMEOUT.

#include <cuda.h>
#include <cudaTypedefs.h>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_gemm.cuh"
#include "kpm_tc.cuh"

namespace kpm {

namespace tc {

struct TcArgs {
  int64_t M;        // rows of the output (num_moments)
  int64_t kchunks;  // K / KC (padded K)
  int splits;
  int nt;           // output columns per CTA (multiple of 16, <= 256)
  int ntiles_n;
  int tmem_cols;    // power of two >= 2 * nt (4 * nt when promoting)
  float2* part;     // [split][M][M] (re, im) partials
  int* err;
  uint64_t wait_ns; // bound of every mbarrier wait
  int stall;        // test only: the producer issues no loads
  int f16;          // FP16 planes (else bfloat16); A and B alike
  int64_t promote;  // K chunks per FP32 accumulation run (0: the split)
};

// warps: 0 allocates tensor memory and runs the TMA producer (one lane),
// 1 issues the MMAs (one lane), 2-5 drain the accumulators; warp w reaches
// the tensor-memory lanes 32 (w % 4) .. 32 (w % 4) + 31, so warps 2-5 cover
// all 128 rows of the tile.
constexpr int GEMM_THREADS = 192;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
        "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
        "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
        "=r"(v[15])
      : "r"(addr));
}

__device__ __forceinline__ void tmem_st16(uint32_t addr,
                                          const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(addr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]),
      "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]),
      "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
}

template <int KC, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
bf16x3_tc_kernel(const __grid_constant__ CUtensorMap map_a,
                 const __grid_constant__ CUtensorMap map_b, TcArgs args) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // align the dynamic shared memory to 1024 bytes (swizzle atoms)
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nt = args.nt;
  const uint32_t a_bytes = 4 * TM * KC * 2;   // 4 planes x 128 rows
  const uint32_t b_bytes = 4 * nt * KC * 2;   // 4 planes x nt rows
  uint8_t* sa = smem;                          // STAGES x a_bytes
  uint8_t* sb = smem + STAGES * a_bytes;       // STAGES x b_bytes
  uint64_t* full = reinterpret_cast<uint64_t*>(sb + STAGES * b_bytes);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;   // every MMA of the CTA completed
  uint64_t* promo = done + 1;        // a run's MMAs completed
  uint64_t* resume = promo + 1;      // its accumulators were drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(resume + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // tile / split of this CTA
  const int tiles = (int)(ceil_div(args.M, TM) * args.ntiles_n);
  const int tile = blockIdx.x % tiles;
  const int split = blockIdx.x / tiles;
  const int tm = tile / args.ntiles_n, tn = tile % args.ntiles_n;
  const int64_t c_per = ceil_div(args.kchunks, args.splits);
  const int64_t kc0 = split * c_per;
  const int64_t kc1 = kc0 + c_per < args.kchunks ? kc0 + c_per : args.kchunks;
  const int64_t nk = kc1 > kc0 ? kc1 - kc0 : 0;
  // FP32 accumulation runs of `run` K chunks; each run's sums are added
  // into a master copy in tensor memory (FP32, round to nearest)
  const int64_t run = args.promote > 0 ? args.promote : (nk > 0 ? nk : 1);
  const int64_t runs = ceil_div(nk, run);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    mbar_init(promo, 1);
    mbar_init(resume, 4);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
            "r"(smem_u32(tmem_slot)),
        "r"(args.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    int64_t issued = 0;
    for (int64_t i = 0; i < nk && !args.stall; ++i) {
      const int s = (int)(i % STAGES);
      const uint32_t ph = (uint32_t)((i / STAGES) & 1);
      if (!mbar_wait(&empty[s], ph ^ 1, args.err, 1, args.wait_ns)) break;
      mbar_expect_tx(&full[s], a_bytes + b_bytes);
      // K-blocked planes: element kx is (kx % KB) of block kx / KB
      const int kx = (int)((kc0 + i) * KC);
      const int kb = kx / (int)STORE_KB, ki = kx % (int)STORE_KB;
      tma_load_4d(sa + s * a_bytes, &map_a, &full[s], ki, tm * TM, 0, kb);
      tma_load_4d(sb + s * b_bytes, &map_b, &full[s], ki, tn * nt, 0, kb);
      ++issued;
    }
    drain_loads(full, STAGES, issued, args.err, args.wait_ns);
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    const uint32_t id_pos = instr_desc(nt, false, args.f16 != 0);
    const uint32_t id_neg = instr_desc(nt, true, args.f16 != 0);
    const uint32_t d_re = tmem, d_im = tmem + (uint32_t)nt;
    const uint32_t plane_a = TM * KC * 2, plane_b = (uint32_t)nt * KC * 2;
    bool ok = true;
    for (int64_t i = 0; i < nk && ok; ++i) {
      const int64_t in_run = i % run;
      if (in_run == 0 && i > 0) {
        // the previous run's accumulators must be drained first
        if (!mbar_wait(resume, (uint32_t)((i / run - 1) & 1), args.err, 5,
                       args.wait_ns)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
      }
      const int s = (int)(i % STAGES);
      const uint32_t ph = (uint32_t)((i / STAGES) & 1);
      if (!mbar_wait(&full[s], ph, args.err, 2, args.wait_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(sa + s * a_bytes);
      const uint32_t b0 = smem_u32(sb + s * b_bytes);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ++ks) {
        const uint32_t ko = ks * 32;  // bytes along K inside a row
        // planes: 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo
        const uint64_t Arh = smem_desc<KC>(a0 + 0 * plane_a + ko);
        const uint64_t Arl = smem_desc<KC>(a0 + 1 * plane_a + ko);
        const uint64_t Aih = smem_desc<KC>(a0 + 2 * plane_a + ko);
        const uint64_t Ail = smem_desc<KC>(a0 + 3 * plane_a + ko);
        const uint64_t Brh = smem_desc<KC>(b0 + 0 * plane_b + ko);
        const uint64_t Brl = smem_desc<KC>(b0 + 1 * plane_b + ko);
        const uint64_t Bih = smem_desc<KC>(b0 + 2 * plane_b + ko);
        const uint64_t Bil = smem_desc<KC>(b0 + 3 * plane_b + ko);
        // the first MMA of a run overwrites the accumulators
        const uint32_t acc0 = (in_run > 0 || ks > 0) ? 1u : 0u;
        // Re += Ar Br + Ai Bi
        mma_bf16(d_re, Arh, Brh, id_pos, acc0);
        mma_bf16(d_re, Arh, Brl, id_pos, 1u);
        mma_bf16(d_re, Arl, Brh, id_pos, 1u);
        mma_bf16(d_re, Aih, Bih, id_pos, 1u);
        mma_bf16(d_re, Aih, Bil, id_pos, 1u);
        mma_bf16(d_re, Ail, Bih, id_pos, 1u);
        // Im += Ar Bi - Ai Br
        mma_bf16(d_im, Arh, Bih, id_pos, acc0);
        mma_bf16(d_im, Arh, Bil, id_pos, 1u);
        mma_bf16(d_im, Arl, Bih, id_pos, 1u);
        mma_bf16(d_im, Aih, Brh, id_neg, 1u);
        mma_bf16(d_im, Aih, Brl, id_neg, 1u);
        mma_bf16(d_im, Ail, Brh, id_neg, 1u);
      }
      mma_commit(&empty[s]);  // frees the stage when these MMAs complete
      if (in_run == run - 1 || i == nk - 1) mma_commit(promo);  // run done
    }
    mma_commit(done);  // all MMAs of this thread
  } else if (warp >= 2) {
    // ---- drain: after every run, add its accumulators into the master
    // copy (tensor-memory columns 2 nt .. 4 nt); after the last, write the
    // sums to this split's partials.  Each warp decides from one lane, so
    // that its warp-collective tensor-memory accesses are never divergent.
    const int q = warp % 4;
    const int row = tm * TM + q * 32 + lane;
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const uint32_t acc = tmem + lane_base, mst = acc + 2 * (uint32_t)nt;
    float2* dst = args.part + ((int64_t)split * args.M + row) * args.M;
    for (int64_t g = 0; g < runs; ++g) {
      int ok = 1;
      if (lane == 0)
        ok = mbar_wait(promo, (uint32_t)(g & 1), args.err, 3, args.wait_ns);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const bool last = g == runs - 1;
      for (int c = 0; c < 2 * nt; c += 16) {
        // columns c .. c + 15 of [re (nt) | im (nt)]
        uint32_t v[16], m[16];
        tmem_ld16(acc + (uint32_t)c, v);
        if (g > 0) tmem_ld16(mst + (uint32_t)c, m);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (g > 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            v[j] = __float_as_uint(__uint_as_float(v[j]) +
                                   __uint_as_float(m[j]));
        }
        if (!last) {
          tmem_st16(mst + (uint32_t)c, v);
        } else if (row < args.M) {
          const bool im = c >= nt;
          const int64_t col0 = (int64_t)tn * nt + (im ? c - nt : c);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int64_t col = col0 + j;
            if (col < args.M) {
              if (im) dst[col].y = __uint_as_float(v[j]);
              else dst[col].x = __uint_as_float(v[j]);
            }
          }
        }
      }
      if (!last) {
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(resume);
      }
    }
  }

  // ---- release: no MMA may still be running when the tensor memory is
  // freed (the MMA thread always commits `done`)
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_all(done, 0, args.wait_ns))
    atomicCAS(args.err, 0, 3);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0) {
    asm volatile(
        "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
        "r"(args.tmem_cols));
  }
}

// sum the split partials in fixed order (FP64), scale, complex128 out
__global__ void tc_reduce_kernel(const float2* __restrict__ part, int splits,
                                 int64_t MM, double scale,
                                 double2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MM) return;
  double r = 0.0, im = 0.0;
  for (int s = 0; s < splits; ++s) {
    const float2 p = part[(int64_t)s * MM + i];
    r += (double)p.x;
    im += (double)p.y;
  }
  out[i] = make_double2(r * scale, im * scale);
}

// 4D map over the four K-blocked planes of a store: dims {KB, M, 4,
// Kp / KB}, box {KC, rows, 4, 1}, swizzled over the 2*KC-byte rows (the box
// lands in shared memory as [plane][row][KC], as a 3D box over row-major
// planes would).
template <int KC>
static int make_map(CUtensorMap* map, const Store* s, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled unavailable");
    return KPM_ECUDA;
  }
  cuuint64_t dims[4] = {(cuuint64_t)STORE_KB, (cuuint64_t)s->M, 4,
                        (cuuint64_t)(s->Kp / STORE_KB)};
  cuuint64_t strides[3] = {(cuuint64_t)STORE_KB * 2,
                           (cuuint64_t)s->M * STORE_KB * 2,
                           (cuuint64_t)4 * s->M * STORE_KB * 2};
  cuuint32_t box[4] = {(cuuint32_t)KC, (cuuint32_t)box_rows, 4, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(map,
                  s->f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                         : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                  4, s->planes, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  KC == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                           : CU_TENSOR_MAP_SWIZZLE_32B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return KPM_ECUDA;
  }
  return KPM_OK;
}

}  // namespace tc

template <int KC, int STAGES>
static int gemm_bf16x3_tc_kc(kpm_handle* h, const Store* omega,
                             const Store* psi, int64_t M, int64_t R, int nt,
                             int64_t run_k, double* mu_host) {
  using namespace tc;
  KPM_REQUIRE(omega->kind == STORE_BF16X3 && psi->kind == STORE_BF16X3,
              "tensor-core contraction needs BF16x3 stores");
  // one MMA kind::f16 takes A and B of the same type
  KPM_REQUIRE(omega->f16 == psi->f16,
              "tensor-core contraction: plane types differ");
  KPM_REQUIRE(omega->Kp % KC == 0 && omega->Kp == psi->Kp,
              "store K padding mismatch");
  KPM_REQUIRE(M < (1 << 20), "too many moments");
  const int ntiles_n = (int)ceil_div(M, nt);
  // runs of run_k K elements need a master copy of the accumulators in
  // tensor memory: 4 nt <= 512 columns
  const int64_t promote = run_k > 0 && 4 * nt <= 512 ? ceil_div(run_k, KC) : 0;
  int tmem_cols = 32;
  while (tmem_cols < (promote ? 4 : 2) * nt) tmem_cols *= 2;
  const int64_t kchunks = omega->Kp / KC;
  const int tiles = (int)(ceil_div(M, TM) * ntiles_n);
  // one CTA per SM in total, split K among the tiles
  int splits = (int)(h->num_sms / tiles);
  if (splits < 1) splits = 1;
  if (splits > kchunks) splits = (int)kchunks;
  // every split gets at least one K chunk (all partials are written)
  const int64_t c_per = ceil_div(kchunks, splits);
  splits = (int)ceil_div(kchunks, c_per);

  CUtensorMap map_a, map_b;
  KPM_TRY(make_map<KC>(&map_a, omega, TM));
  KPM_TRY(make_map<KC>(&map_b, psi, nt));

  const size_t a_bytes = 4 * TM * KC * 2, b_bytes = (size_t)4 * nt * KC * 2;
  const size_t smem = 1024 + STAGES * (a_bytes + b_bytes) +
                      (2 * STAGES + 3) * 8 + 16;
  KPM_CUDA(cudaFuncSetAttribute(bf16x3_tc_kernel<KC, STAGES>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  float2* part = nullptr;
  int* err = nullptr;
  KPM_TRY(dev_alloc((void**)&part, (size_t)splits * M * M * sizeof(float2),
                    h->stream));
  int st = dev_alloc((void**)&err, sizeof(int), h->stream);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) e = cudaMemsetAsync(err, 0, sizeof(int), h->stream);
  if (st == KPM_OK && e == cudaSuccess && !h->ev_gemm0) {
    e = cudaEventCreate(&h->ev_gemm0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev_gemm1);
  }
  if (st == KPM_OK && e == cudaSuccess) {
    const WaitCfg wc = wait_cfg();
    TcArgs args{M,    kchunks, splits, nt,      ntiles_n,
                tmem_cols, part, err,  wc.ns,   wc.stall, omega->f16,
                promote};
    cudaEventRecord(h->ev_gemm0, h->stream);
    bf16x3_tc_kernel<KC, STAGES><<<(unsigned)(tiles * splits), GEMM_THREADS,
                                   smem,
                           h->stream>>>(map_a, map_b, args);
    count_launch(1);
    e = cudaGetLastError();
    cudaEventRecord(h->ev_gemm1, h->stream);
  }
  int herr = 0;
  if (st == KPM_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost,
                        h->stream);
  if (st == KPM_OK && e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (st == KPM_OK && e == cudaSuccess) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev_gemm0, h->ev_gemm1) == cudaSuccess)
      h->last_gemm_ms = ms;
    h->last_gemm_flops = 3.0 * 4.0 * 2.0 * (double)M * (double)M *
                         (double)omega->Kp;
  }
  double2* mu = nullptr;
  if (st == KPM_OK && e == cudaSuccess && herr == 0) {
    st = dev_alloc((void**)&mu, (size_t)M * M * sizeof(double2), h->stream);
    if (st == KPM_OK) {
      tc_reduce_kernel<<<(unsigned)ceil_div(M * M, 256), 256, 0, h->stream>>>(
          part, splits, M * M, 1.0 / (double)R, mu);
      count_launch(1);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(mu_host, mu, (size_t)M * M * sizeof(double2),
                            cudaMemcpyDeviceToHost, h->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
  }
  dev_free(mu, h->stream);
  dev_free(part, h->stream);
  dev_free(err, h->stream);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  if (herr != 0) {
    set_error("tensor-core contraction: a bounded wait expired (code %d)",
              herr);
    return KPM_ETIMEOUT;
  }
  return KPM_OK;
}

// Output tile width nt (MMA N) and as many pipeline stages as the shared
// memory holds (at most 4): a 128 x 128 tile has 64 KB stages (3), a
// 128 x 256 tile 96 KB (2).  Measured on the Kubo workload (M = 256,
// K = 1.28e6, K-blocked stores) both take 1.11 ms (0.95 of the measured
// BF16 peak); before the stores were K-blocked the same kernel took 3.09 ms
// (row-major planes: a stage gathered 512 pieces of 64 bytes, each a 2.5 MB
// row stride apart).
//
// The tensor cores' FP32 accumulation error grows with the number of
// products summed into one accumulator: with one accumulation run per
// split (K / 76 = 16,800 products per CTA on that workload) the moments
// matrix was 1.0e-4 off the FP64 contraction, with 4,096 / 1,024 / 256
// K elements per run 2.5e-5 / 5.8e-6 / 1.5e-6.  So 128-wide tiles (the
// default) add every run of RUN_K = 1024 K elements into a master copy
// in tensor memory (FP32, round to nearest) and restart the MMA
// accumulation.  KPM_TC_NT=256 selects 256-wide tiles (no room for the
// master copy: one run per split); KPM_TC_RUN sets the run length in K
// elements (0: one run per split).
constexpr int64_t RUN_K = 1024;

int gemm_bf16x3(kpm_handle* h, const Store* omega, const Store* psi,
                int64_t M, int64_t K, int64_t R, double* mu_host) {
  (void)K;
  int nt_max = 128;
  if (const char* e = getenv("KPM_TC_NT")) nt_max = atoi(e) >= 256 ? 256 : 128;
  int64_t run_k = RUN_K;
  if (const char* e = getenv("KPM_TC_RUN")) run_k = atoll(e);
  const int nt = (int)round_up(M < nt_max ? M : nt_max, 16);
  if (h->tc_kc != 32)
    return gemm_bf16x3_tc_kc<16, tc::Stage<16>::STAGES>(h, omega, psi, M, R,
                                                        nt, run_k, mu_host);
  const size_t stage = (size_t)4 * (tc::TM + nt) * 32 * 2;
  const size_t budget = 227 * 1024 - 2048;
  const size_t stages = budget / stage;
  if (stages >= 4)
    return gemm_bf16x3_tc_kc<32, 4>(h, omega, psi, M, R, nt, run_k, mu_host);
  if (stages == 3)
    return gemm_bf16x3_tc_kc<32, 3>(h, omega, psi, M, R, nt, run_k, mu_host);
  return gemm_bf16x3_tc_kc<32, 2>(h, omega, psi, M, R, nt, run_k, mu_host);
}

}  // namespace kpm
