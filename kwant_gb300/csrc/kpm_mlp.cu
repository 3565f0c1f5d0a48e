// Learned moment surrogate: a small MLP trained and evaluated on the GPU
// with hand-written kernels (no reference counterpart; the plain KPM is its
// error check and fallback).
//
//   x (model parameters) -> [Linear -> GELU] x (L-1) -> Linear -> moments
//
// FP32 master weights; every matmul in BF16 on the tensor cores with FP32
// accumulation: a TN tcgen05 GEMM  C[M][N] = A[M][K] B[N][K]^T  with both
// operands K-major, loaded by TMA (64-byte swizzle, 4 stages).  Forward:
// Z = H W^T.  Backward keeps transposed BF16 copies so that both gradient
// products are TN GEMMs too: dH = dZ (W^T)^T  and  dW = dZ^T (H^T)^T.
// GELU is the exact erf form; the loss is the mean squared error; the
// optimiser is Adam (Kingma & Ba 2015) on the flat FP32 parameter vector.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_tc.cuh"

namespace kpm {
namespace mlp {

using bf16 = __nv_bfloat16;
constexpr int KC = 32;
constexpr int STAGES = 4;

struct TnArgs {
  int64_t M, N, K;
  int nt, ntiles_n, tmem_cols;
  float* C;
  int64_t ldc;
  int* err;
  uint64_t wait_ns;  // bound of every mbarrier wait
  int stall;         // test only: the producer issues no loads
};

// C[M][N] = A[M][K] * B[N][K]^T (BF16 in, FP32 out), one 128 x nt tile per
// CTA over the full K; warp 0: TMEM + TMA, warp 1: MMA, all: epilogue.
__global__ void __launch_bounds__(tc::THREADS, 1)
bf16_tn_kernel(const __grid_constant__ CUtensorMap map_a,
               const __grid_constant__ CUtensorMap map_b, TnArgs args) {
  using namespace tc;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nt = args.nt;
  const uint32_t a_bytes = TM * KC * 2, b_bytes = (uint32_t)nt * KC * 2;
  uint8_t* sa = smem;
  uint8_t* sb = smem + STAGES * a_bytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(sb + STAGES * b_bytes);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int tm = blockIdx.x / args.ntiles_n, tn = blockIdx.x % args.ntiles_n;
  const int64_t nk = args.K / KC;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
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
    int64_t issued = 0;
    for (int64_t i = 0; i < nk && !args.stall; ++i) {
      const int s = (int)(i % STAGES);
      const uint32_t ph = (uint32_t)((i / STAGES) & 1);
      if (!mbar_wait(&empty[s], ph ^ 1, args.err, 1, args.wait_ns)) break;
      mbar_expect_tx(&full[s], a_bytes + b_bytes);
      tma_load_2d(sa + s * a_bytes, &map_a, &full[s], (int)(i * KC), tm * TM);
      tma_load_2d(sb + s * b_bytes, &map_b, &full[s], (int)(i * KC), tn * nt);
      ++issued;
    }
    drain_loads(full, STAGES, issued, args.err, args.wait_ns);
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = instr_desc(nt, false);
    for (int64_t i = 0; i < nk; ++i) {
      const int s = (int)(i % STAGES);
      const uint32_t ph = (uint32_t)((i / STAGES) & 1);
      if (!mbar_wait(&full[s], ph, args.err, 2, args.wait_ns)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(sa + s * a_bytes);
      const uint32_t b0 = smem_u32(sb + s * b_bytes);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ++ks)
        mma_bf16(tmem, smem_desc<KC>(a0 + ks * 32), smem_desc<KC>(b0 + ks * 32),
                 idesc, (i > 0 || ks > 0) ? 1u : 0u);
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  // one thread decides for the CTA (warp-uniform tensor-memory loads)
  __shared__ int go;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool ok = mbar_wait_all(done, 0, args.wait_ns);
    if (!ok) atomicCAS(args.err, 0, 3);
    go = ok && nk > 0 && *(volatile int*)args.err == 0;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (go) {
    const int64_t row = (int64_t)tm * TM + warp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    for (int c = 0; c < nt; c += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
            "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
            "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
            "=r"(r[15])
          : "r"(tmem + lane_base + (uint32_t)c));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < args.M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t col = (int64_t)tn * nt + c + j;
          if (col < args.N)
            args.C[row * args.ldc + col] = __uint_as_float(r[j]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile(
        "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
        "r"(args.tmem_cols));
}

// 2D map over a row-major [rows][K] bf16 matrix, box {KC, box_rows}
static int make_map2d(CUtensorMap* map, const bf16* p, int64_t rows,
                      int64_t K, int box_rows) {
  auto fn = tc::encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled unavailable");
    return KPM_ECUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {(cuuint32_t)KC, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)p, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return KPM_ECUDA;
  }
  return KPM_OK;
}

// ------------------------------------------------------ elementwise kernels
__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) +
         z * 0.3989422804014327f * expf(-0.5f * z * z);
}

// W [N][K] fp32 -> Wb [N][Kp] and WTb [Kp][N] bf16 (zero padding)
__global__ void weights_kernel(const float* __restrict__ W, int N, int K,
                               int Kp, bf16* __restrict__ Wb,
                               bf16* __restrict__ WTb) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)N * Kp) return;
  const int n = (int)(idx / Kp), k = (int)(idx % Kp);
  const float v = k < K ? W[(int64_t)n * K + k] : 0.f;
  const bf16 b = __float2bfloat16_rn(v);
  Wb[idx] = b;
  WTb[(int64_t)k * N + n] = b;
}

// rows (gathered by idx) of x [n][K] fp32 -> Hb [B][Kp], HTb [Kp][B]
__global__ void input_kernel(const float* __restrict__ x,
                             const int32_t* __restrict__ idx, int B, int K,
                             int Kp, bf16* __restrict__ Hb,
                             bf16* __restrict__ HTb) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * Kp) return;
  const int b = (int)(t / Kp), k = (int)(t % Kp);
  const int src = idx ? idx[b] : b;
  const float v = k < K ? x[(int64_t)src * K + k] : 0.f;
  const bf16 h = __float2bfloat16_rn(v);
  Hb[t] = h;
  if (HTb) HTb[(int64_t)k * B + b] = h;
}

// Z += bias; hidden: H = GELU(Z) to Hb [B][N] / HTb [N][B]; output: Z kept
__global__ void bias_act_kernel(float* __restrict__ Z,
                                const float* __restrict__ bias, int B, int N,
                                int hidden, bf16* __restrict__ Hb,
                                bf16* __restrict__ HTb) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * N) return;
  const int b = (int)(t / N), n = (int)(t % N);
  const float z = Z[t] + bias[n];
  Z[t] = z;
  if (hidden) {
    const bf16 h = __float2bfloat16_rn(gelu(z));
    Hb[t] = h;
    if (HTb) HTb[(int64_t)n * B + b] = h;
  }
}

// dOut = 2 (pred - y) / (B D); per-block partial sums of squared error
__global__ void mse_kernel(const float* __restrict__ pred,
                           const float* __restrict__ y,
                           const int32_t* __restrict__ idx, int B, int D,
                           float* __restrict__ dout,
                           double* __restrict__ part) {
  __shared__ double s[256];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0.0;
  if (t < (int64_t)B * D) {
    const int b = (int)(t / D), d = (int)(t % D);
    const int src = idx ? idx[b] : b;
    const float e = pred[t] - y[(int64_t)src * D + d];
    dout[t] = 2.f * e / ((float)B * (float)D);
    e2 = (double)e * (double)e;
  }
  s[threadIdx.x] = e2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// *acc += sum(part[0..n)) * scale (one block, fixed order)
__global__ void loss_acc_kernel(const double* __restrict__ part, int n,
                                double scale, double* __restrict__ acc) {
  __shared__ double s[256];
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) t += part[i];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc += s[0] * scale;
}

// dZ = dH * GELU'(Z) (hidden) or dZ = dH (output); also bf16 copies
__global__ void act_back_kernel(const float* __restrict__ dH,
                                const float* __restrict__ Z, int64_t ldh,
                                int B, int N, int hidden,
                                float* __restrict__ dZ, bf16* __restrict__ dZb,
                                bf16* __restrict__ dZTb) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * N) return;
  const int b = (int)(t / N), n = (int)(t % N);
  float g = dH[(int64_t)b * ldh + n];
  if (hidden) g *= gelu_grad(Z[t]);
  dZ[t] = g;
  const bf16 h = __float2bfloat16_rn(g);
  dZb[t] = h;
  dZTb[(int64_t)n * B + b] = h;
}

// db[n] = sum_b dZ[b][n] (fixed order)
__global__ void bias_grad_kernel(const float* __restrict__ dZ, int B, int N,
                                 float* __restrict__ db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += dZ[(int64_t)b * N + n];
  db[n] = s;
}

// dW [N][K] from the padded GEMM output [N][Kp]
__global__ void strip_kernel(const float* __restrict__ src, int N, int K,
                             int Kp, float* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)N * K) return;
  const int n = (int)(t / K), k = (int)(t % K);
  dst[t] = src[(int64_t)n * Kp + k];
}

// Adam step t = *step + 1 (the counter is advanced by adam_count_kernel
// afterwards, so that a captured epoch replays with the right t)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v,
                            int64_t n, float lr, float b1, float b2,
                            float eps, const int64_t* __restrict__ step) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float t = (float)(*step + 1);
  const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void adam_count_kernel(int64_t* step) { *step += 1; }

}  // namespace mlp
}  // namespace kpm

using namespace kpm;
using namespace kpm::mlp;

struct kpm_mlp {
  int L = 0;
  std::vector<int> w, wp;            // widths, K-padded widths
  std::vector<int64_t> woff, boff;   // parameter offsets
  int64_t nparams = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  int64_t step = 0;
  int Bcap = 0;
  std::vector<bf16*> Wb, WTb, Hb, HTb;
  std::vector<float*> Z, dZ;
  bf16 *dZb = nullptr, *dZTb = nullptr;
  float *dH = nullptr, *tmp = nullptr;
  double* part = nullptr;
  double* loss_acc = nullptr;  // sum of batch losses since the last reset
  int64_t* dstep = nullptr;    // Adam step counter on the device
  int* err = nullptr;
  int num_sms = 0, device = 0;
  cudaStream_t stream = nullptr;
};

namespace {

template <typename T>
int alloc(T** p, size_t count, cudaStream_t s) {
  return dev_alloc((void**)p, count * sizeof(T), s);
}

size_t gemm_smem(int nt) {
  return 1024 + STAGES * (tc::TM * KC * 2 + (size_t)nt * KC * 2) +
         (2 * STAGES + 1) * 8 + 16;
}

// C[M][N] = A[M][K] B[N][K]^T  (A, B bf16 row-major, K multiple of 32)
int gemm_tn(kpm_mlp* net, const bf16* A, int64_t M, const bf16* B,
            int64_t N, int64_t K, float* C, int64_t ldc) {
  // power-of-two tile width: the shared memory per CTA then limits
  // residency so that the resident CTAs' TMEM columns never exceed 512
  int nt = 16;
  while (nt < N && nt < 256) nt *= 2;
  const int ntiles_n = (int)ceil_div(N, nt);
  const int tmem_cols = nt < 32 ? 32 : nt;
  CUtensorMap ma, mb;
  KPM_TRY(make_map2d(&ma, A, M, K, tc::TM));
  KPM_TRY(make_map2d(&mb, B, N, K, nt));
  const size_t smem = gemm_smem(nt);   // attribute set at create
  const tc::WaitCfg wc = tc::wait_cfg();
  TnArgs args{M, N, K, nt, ntiles_n, tmem_cols, C, ldc, net->err, wc.ns,
              wc.stall};
  const int grid = (int)(ceil_div(M, tc::TM) * ntiles_n);
  bf16_tn_kernel<<<grid, tc::THREADS, smem, net->stream>>>(ma, mb, args);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

unsigned blocks(int64_t n) { return (unsigned)ceil_div(n, 256); }

int upload_weights(kpm_mlp* net) {
  for (int l = 0; l < net->L; ++l) {
    const int N = net->w[l + 1], K = net->w[l], Kp = net->wp[l];
    weights_kernel<<<blocks((int64_t)N * Kp), 256, 0, net->stream>>>(
        net->params + net->woff[l], N, K, Kp, net->Wb[l], net->WTb[l]);
    count_launch(1);
  }
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// forward on B rows of x (gathered by idx when non-null); prediction in Z[L-1]
int forward(kpm_mlp* net, const float* x, const int32_t* idx, int B,
            bool train) {
  KPM_TRY(upload_weights(net));
  input_kernel<<<blocks((int64_t)B * net->wp[0]), 256, 0, net->stream>>>(
      x, idx, B, net->w[0], net->wp[0], net->Hb[0],
      train ? net->HTb[0] : nullptr);
  count_launch(1);
  for (int l = 0; l < net->L; ++l) {
    const int N = net->w[l + 1], Kp = net->wp[l];
    KPM_TRY(gemm_tn(net, net->Hb[l], B, net->Wb[l], N, Kp, net->Z[l], N));
    const bool hidden = l + 1 < net->L;
    bias_act_kernel<<<blocks((int64_t)B * N), 256, 0, net->stream>>>(
        net->Z[l], net->params + net->boff[l], B, N, hidden ? 1 : 0,
        hidden ? net->Hb[l + 1] : nullptr,
        hidden && train ? net->HTb[l + 1] : nullptr);
    count_launch(1);
  }
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// gradients of the MSE loss for the batch last forwarded; the batch loss is
// added to net->loss_acc on the device (no host synchronisation)
int backward(kpm_mlp* net, const float* y, const int32_t* idx, int B) {
  const int D = net->w[net->L];
  const int nb = (int)blocks((int64_t)B * D);
  mse_kernel<<<nb, 256, 0, net->stream>>>(net->Z[net->L - 1], y, idx, B, D,
                                          net->dH, net->part);
  loss_acc_kernel<<<1, 256, 0, net->stream>>>(net->part, nb,
                                              1.0 / ((double)B * D),
                                              net->loss_acc);
  count_launch(2);
  int64_t ldh = D;
  for (int l = net->L - 1; l >= 0; --l) {
    const int N = net->w[l + 1], K = net->w[l], Kp = net->wp[l];
    const bool hidden = l + 1 < net->L;
    act_back_kernel<<<blocks((int64_t)B * N), 256, 0, net->stream>>>(
        net->dH, net->Z[l], ldh, B, N, hidden ? 1 : 0, net->dZ[0], net->dZb,
        net->dZTb);
    bias_grad_kernel<<<blocks(N), 256, 0, net->stream>>>(
        net->dZ[0], B, N, net->grads + net->boff[l]);
    count_launch(2);
    // dW [N][Kp] = dZ^T [N][B] . (H^T [Kp][B])^T
    KPM_TRY(gemm_tn(net, net->dZTb, N, net->HTb[l], Kp, B, net->tmp, Kp));
    strip_kernel<<<blocks((int64_t)N * K), 256, 0, net->stream>>>(
        net->tmp, N, K, Kp, net->grads + net->woff[l]);
    count_launch(1);
    if (l > 0) {
      // dH_prev [B][Kp] = dZ [B][N] . (W^T [Kp][N])^T
      KPM_TRY(gemm_tn(net, net->dZb, B, net->WTb[l], Kp, N, net->dH, Kp));
      ldh = Kp;
    }
  }
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

int read_loss(kpm_mlp* net, double* out, bool reset) {
  double v = 0.0;
  KPM_CUDA(cudaMemcpyAsync(&v, net->loss_acc, sizeof(double),
                           cudaMemcpyDeviceToHost, net->stream));
  if (reset) KPM_CUDA(cudaMemsetAsync(net->loss_acc, 0, sizeof(double),
                                      net->stream));
  KPM_CUDA(cudaStreamSynchronize(net->stream));
  if (out) *out = v;
  return KPM_OK;
}

int check_err(kpm_mlp* net) {
  int herr = 0;
  KPM_CUDA(cudaMemcpyAsync(&herr, net->err, sizeof(int),
                           cudaMemcpyDeviceToHost, net->stream));
  KPM_CUDA(cudaStreamSynchronize(net->stream));
  if (herr) {
    set_error("surrogate GEMM: a bounded wait expired (code %d)", herr);
    return KPM_ETIMEOUT;
  }
  return KPM_OK;
}

}  // namespace

extern "C" {

int kpm_mlp_create(int num_layers, const int32_t* widths, int max_batch,
                   uint64_t seed, kpm_mlp** out) {
  KPM_REQUIRE(out && widths && num_layers >= 1 && num_layers <= 16,
              "kpm_mlp_create: invalid layer count");
  KPM_REQUIRE(max_batch >= 32 && max_batch % 32 == 0 && max_batch <= 65536,
              "kpm_mlp_create: max_batch must be a multiple of 32");
  for (int l = 0; l <= num_layers; ++l)
    KPM_REQUIRE(widths[l] >= 1 && widths[l] <= 4096,
                "kpm_mlp_create: invalid width");
  for (int l = 1; l <= num_layers; ++l)
    KPM_REQUIRE(widths[l] % 32 == 0,
                "kpm_mlp_create: hidden and output widths must be multiples "
                "of 32");
  auto* net = new kpm_mlp();
  net->L = num_layers;
  net->Bcap = max_batch;
  int st = init_device(&net->device, &net->num_sms);
  if (st == KPM_OK &&
      cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) !=
          cudaSuccess) {
    set_error("kpm_mlp_create: stream creation failed");
    st = KPM_ECUDA;
  }
  if (st != KPM_OK) {
    delete net;
    return st;
  }
  // the largest GEMM tile (256 columns) needs this much dynamic shared
  // memory; set it (and resolve the tensor-map encoder) before any stream
  // capture of a training epoch
  tc::encode_fn();
  if (cudaFuncSetAttribute(bf16_tn_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_smem(256)) != cudaSuccess) {
    set_error("kpm_mlp_create: shared memory attribute failed");
    cudaStreamDestroy(net->stream);
    delete net;
    return KPM_ECUDA;
  }
  net->w.assign(widths, widths + num_layers + 1);
  net->wp.resize(num_layers + 1);
  for (int l = 0; l <= num_layers; ++l)
    net->wp[l] = (int)round_up(net->w[l], 32);
  int64_t off = 0;
  for (int l = 0; l < num_layers; ++l) {
    net->woff.push_back(off);
    off += (int64_t)net->w[l + 1] * net->w[l];
    net->boff.push_back(off);
    off += net->w[l + 1];
  }
  net->nparams = off;
  // Glorot-uniform weights, zero biases, from seed
  std::vector<float> p(off, 0.f);
  std::mt19937_64 gen(seed);
  for (int l = 0; l < num_layers; ++l) {
    const double lim = std::sqrt(6.0 / (net->w[l] + net->w[l + 1]));
    std::uniform_real_distribution<double> U(-lim, lim);
    for (int64_t i = 0; i < (int64_t)net->w[l + 1] * net->w[l]; ++i)
      p[net->woff[l] + i] = (float)U(gen);
  }
  cudaStream_t s = net->stream;
  const int B = max_batch;
  int maxw = 0, maxwp = 0;
  for (int l = 0; l <= num_layers; ++l) {
    maxw = std::max(maxw, net->w[l]);
    maxwp = std::max(maxwp, net->wp[l]);
  }
  net->Wb.resize(num_layers);
  net->WTb.resize(num_layers);
  net->Hb.resize(num_layers + 1);
  net->HTb.resize(num_layers + 1);
  net->Z.resize(num_layers);
  net->dZ.resize(1);
  if (st == KPM_OK) st = alloc(&net->params, off, s);
  if (st == KPM_OK) st = alloc(&net->grads, off, s);
  if (st == KPM_OK) st = alloc(&net->m, off, s);
  if (st == KPM_OK) st = alloc(&net->v, off, s);
  for (int l = 0; st == KPM_OK && l < num_layers; ++l) {
    st = alloc(&net->Wb[l], (size_t)net->w[l + 1] * net->wp[l], s);
    if (st == KPM_OK)
      st = alloc(&net->WTb[l], (size_t)net->w[l + 1] * net->wp[l], s);
    if (st == KPM_OK) st = alloc(&net->Z[l], (size_t)B * net->w[l + 1], s);
  }
  for (int l = 0; st == KPM_OK && l <= num_layers; ++l) {
    st = alloc(&net->Hb[l], (size_t)B * net->wp[l], s);
    if (st == KPM_OK) st = alloc(&net->HTb[l], (size_t)B * net->wp[l], s);
  }
  if (st == KPM_OK) st = alloc(&net->dZ[0], (size_t)B * maxw, s);
  if (st == KPM_OK) st = alloc(&net->dZb, (size_t)B * maxw, s);
  if (st == KPM_OK) st = alloc(&net->dZTb, (size_t)B * maxw, s);
  if (st == KPM_OK) st = alloc(&net->dH, (size_t)B * maxwp, s);
  if (st == KPM_OK)
    st = alloc(&net->tmp, (size_t)std::max(maxw * maxwp, B * maxwp), s);
  if (st == KPM_OK) st = alloc(&net->part, (size_t)ceil_div(B * maxw, 256), s);
  if (st == KPM_OK) st = alloc(&net->err, 1, s);
  if (st == KPM_OK) st = alloc(&net->loss_acc, 1, s);
  if (st == KPM_OK) st = alloc(&net->dstep, 1, s);
  if (st == KPM_OK) {
    cudaMemsetAsync(net->m, 0, off * sizeof(float), s);
    cudaMemsetAsync(net->v, 0, off * sizeof(float), s);
    cudaMemsetAsync(net->err, 0, sizeof(int), s);
    cudaMemsetAsync(net->loss_acc, 0, sizeof(double), s);
    cudaMemsetAsync(net->dstep, 0, sizeof(int64_t), s);
    // zero activations (padding columns must stay zero)
    for (int l = 0; l <= num_layers; ++l) {
      cudaMemsetAsync(net->Hb[l], 0, (size_t)B * net->wp[l] * 2, s);
      cudaMemsetAsync(net->HTb[l], 0, (size_t)B * net->wp[l] * 2, s);
    }
    cudaMemcpyAsync(net->params, p.data(), off * sizeof(float),
                    cudaMemcpyHostToDevice, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      set_error("kpm_mlp_create: initialisation failed");
      st = KPM_ECUDA;
    }
  }
  if (st != KPM_OK) {
    kpm_mlp_destroy(net);
    return st;
  }
  *out = net;
  return KPM_OK;
}

int kpm_mlp_num_params(kpm_mlp* net, int64_t* count) {
  KPM_REQUIRE(net && count, "kpm_mlp_num_params: null argument");
  *count = net->nparams;
  return KPM_OK;
}

int kpm_mlp_get_params(kpm_mlp* net, float* out) {
  KPM_REQUIRE(net && out, "kpm_mlp_get_params: null argument");
  KPM_CUDA(cudaMemcpyAsync(out, net->params, net->nparams * sizeof(float),
                           cudaMemcpyDeviceToHost, net->stream));
  KPM_CUDA(cudaStreamSynchronize(net->stream));
  return KPM_OK;
}

int kpm_mlp_set_params(kpm_mlp* net, const float* in) {
  KPM_REQUIRE(net && in, "kpm_mlp_set_params: null argument");
  KPM_CUDA(cudaMemcpyAsync(net->params, in, net->nparams * sizeof(float),
                           cudaMemcpyHostToDevice, net->stream));
  KPM_CUDA(cudaStreamSynchronize(net->stream));
  net->step = 0;
  KPM_CUDA(cudaMemsetAsync(net->dstep, 0, sizeof(int64_t), net->stream));
  KPM_CUDA(cudaMemsetAsync(net->m, 0, net->nparams * sizeof(float),
                           net->stream));
  KPM_CUDA(cudaMemsetAsync(net->v, 0, net->nparams * sizeof(float),
                           net->stream));
  return KPM_OK;
}

int kpm_mlp_forward(kpm_mlp* net, const float* x, int64_t n, float* y) {
  KPM_REQUIRE(net && x && y && n > 0, "kpm_mlp_forward: invalid argument");
  const int D = net->w[net->L], K0 = net->w[0];
  float* dx = nullptr;
  KPM_TRY(alloc(&dx, (size_t)n * K0, net->stream));
  int st = KPM_OK;
  cudaError_t e = cudaMemcpyAsync(dx, x, (size_t)n * K0 * sizeof(float),
                                  cudaMemcpyHostToDevice, net->stream);
  if (e != cudaSuccess) st = KPM_ECUDA;
  for (int64_t b0 = 0; st == KPM_OK && b0 < n; b0 += net->Bcap) {
    const int B = (int)std::min<int64_t>(net->Bcap, n - b0);
    st = forward(net, dx + b0 * K0, nullptr, B, false);
    if (st == KPM_OK)
      e = cudaMemcpyAsync(y + b0 * D, net->Z[net->L - 1],
                          (size_t)B * D * sizeof(float),
                          cudaMemcpyDeviceToHost, net->stream);
    if (st == KPM_OK && e != cudaSuccess) st = KPM_ECUDA;
  }
  if (st == KPM_OK) st = check_err(net);
  dev_free(dx, net->stream);
  cudaStreamSynchronize(net->stream);
  if (e != cudaSuccess) {
    set_error("kpm_mlp_forward: %s", cudaGetErrorString(e));
    return KPM_ECUDA;
  }
  return st;
}

int kpm_mlp_gradients(kpm_mlp* net, const float* x, const float* y,
                      int64_t n, float* grads, double* loss) {
  KPM_REQUIRE(net && x && y && grads && n > 0 && n <= net->Bcap && n % 32 == 0,
              "kpm_mlp_gradients: n must be a multiple of 32 up to max_batch");
  const int D = net->w[net->L], K0 = net->w[0];
  float *dx = nullptr, *dy = nullptr;
  KPM_TRY(alloc(&dx, (size_t)n * K0, net->stream));
  int st = alloc(&dy, (size_t)n * D, net->stream);
  if (st == KPM_OK &&
      (cudaMemcpyAsync(dx, x, (size_t)n * K0 * 4, cudaMemcpyHostToDevice,
                       net->stream) != cudaSuccess ||
       cudaMemcpyAsync(dy, y, (size_t)n * D * 4, cudaMemcpyHostToDevice,
                       net->stream) != cudaSuccess)) {
    set_error("kpm_mlp_gradients: upload failed");
    st = KPM_ECUDA;
  }
  if (st == KPM_OK) st = read_loss(net, nullptr, true);
  if (st == KPM_OK) st = forward(net, dx, nullptr, (int)n, true);
  if (st == KPM_OK) st = backward(net, dy, nullptr, (int)n);
  if (st == KPM_OK) st = read_loss(net, loss, true);
  if (st == KPM_OK) st = check_err(net);
  if (st == KPM_OK &&
      cudaMemcpy(grads, net->grads, net->nparams * 4,
                 cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("kpm_mlp_gradients: download failed");
    st = KPM_ECUDA;
  }
  dev_free(dx, net->stream);
  dev_free(dy, net->stream);
  cudaStreamSynchronize(net->stream);
  return st;
}

int kpm_mlp_train(kpm_mlp* net, const float* x, const float* y, int64_t n,
                  int batch, int64_t epochs, double lr, uint64_t seed,
                  double* final_loss) {
  KPM_REQUIRE(net && x && y && n >= batch && batch >= 32 && batch % 32 == 0 &&
                  batch <= net->Bcap && epochs > 0 && lr > 0,
              "kpm_mlp_train: invalid argument");
  const int D = net->w[net->L], K0 = net->w[0];
  cudaStream_t s = net->stream;
  float *dx = nullptr, *dy = nullptr;
  int32_t* didx = nullptr;
  const int64_t per_epoch = n / batch;
  KPM_TRY(alloc(&dx, (size_t)n * K0, s));
  int st = alloc(&dy, (size_t)n * D, s);
  if (st == KPM_OK) st = alloc(&didx, (size_t)per_epoch * batch, s);
  if (st == KPM_OK &&
      (cudaMemcpyAsync(dx, x, (size_t)n * K0 * 4, cudaMemcpyHostToDevice, s) !=
           cudaSuccess ||
       cudaMemcpyAsync(dy, y, (size_t)n * D * 4, cudaMemcpyHostToDevice, s) !=
           cudaSuccess)) {
    set_error("kpm_mlp_train: upload failed");
    st = KPM_ECUDA;
  }
  std::mt19937_64 gen(seed);
  std::vector<int32_t> perm(n);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  // One epoch (per_epoch forward / backward / Adam steps over the shuffled
  // index buffer) is captured once as a CUDA graph and replayed; only the
  // shuffled indices change between epochs.
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t nodes = 0;
  int64_t counted0 = 0, counted1 = 0;
  kpm_launch_count(&counted0);
  if (st == KPM_OK) {
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
      set_error("kpm_mlp_train: stream capture failed");
      st = KPM_ECUDA;
    } else {
      int cst = KPM_OK;
      for (int64_t it = 0; cst == KPM_OK && it < per_epoch; ++it) {
        const int32_t* idx = didx + it * batch;
        cst = forward(net, dx, idx, batch, true);
        if (cst == KPM_OK) cst = backward(net, dy, idx, batch);
        if (cst != KPM_OK) break;
        adam_kernel<<<blocks(net->nparams), 256, 0, s>>>(
            net->params, net->grads, net->m, net->v, net->nparams,
            (float)lr, b1, b2, eps, net->dstep);
        adam_count_kernel<<<1, 1, 0, s>>>(net->dstep);
        if (cudaGetLastError() != cudaSuccess) {
          set_error("kpm_mlp_train: Adam launch failed");
          cst = KPM_ECUDA;
        }
      }
      const cudaError_t ce = cudaStreamEndCapture(s, &graph);
      st = cst;
      if (st == KPM_OK && ce != cudaSuccess) {
        set_error("kpm_mlp_train: stream capture failed: %s",
                  cudaGetErrorString(ce));
        st = KPM_ECUDA;
      }
      if (st == KPM_OK &&
          (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess ||
           cudaGraphGetNodes(graph, nullptr, &nodes) != cudaSuccess)) {
        set_error("kpm_mlp_train: graph instantiation failed");
        st = KPM_ECUDA;
      }
    }
  }
  // launches are counted when the graph replays, not when it is captured
  kpm_launch_count(&counted1);
  count_launch(-(int)(counted1 - counted0));
  for (int64_t ep = 0; st == KPM_OK && ep < epochs; ++ep) {
    for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
    std::shuffle(perm.begin(), perm.end(), gen);
    if (cudaMemcpyAsync(didx, perm.data(), per_epoch * batch * 4,
                        cudaMemcpyHostToDevice, s) != cudaSuccess) {
      set_error("kpm_mlp_train: index upload failed");
      st = KPM_ECUDA;
      break;
    }
    if (ep + 1 == epochs && st == KPM_OK) st = read_loss(net, nullptr, true);
    if (st == KPM_OK && cudaGraphLaunch(exec, s) != cudaSuccess) {
      set_error("kpm_mlp_train: graph launch failed");
      st = KPM_ECUDA;
    }
    count_launch((int)nodes);
    net->step += per_epoch;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  double last = 0.0;
  if (st == KPM_OK) st = read_loss(net, &last, true);
  if (st == KPM_OK) st = check_err(net);
  if (final_loss) *final_loss = last / std::max<int64_t>(per_epoch, 1);
  dev_free(dx, s);
  dev_free(dy, s);
  dev_free(didx, s);
  cudaStreamSynchronize(s);
  return st;
}

int kpm_mlp_destroy(kpm_mlp* net) {
  if (!net) return KPM_OK;
  cudaStream_t s = net->stream;
  for (auto* p : net->Wb) dev_free(p, s);
  for (auto* p : net->WTb) dev_free(p, s);
  for (auto* p : net->Hb) dev_free(p, s);
  for (auto* p : net->HTb) dev_free(p, s);
  for (auto* p : net->Z) dev_free(p, s);
  for (auto* p : net->dZ) dev_free(p, s);
  dev_free(net->dZb, s);
  dev_free(net->dZTb, s);
  dev_free(net->dH, s);
  dev_free(net->tmp, s);
  dev_free(net->part, s);
  dev_free(net->err, s);
  dev_free(net->loss_acc, s);
  dev_free(net->dstep, s);
  dev_free(net->params, s);
  dev_free(net->grads, s);
  dev_free(net->m, s);
  dev_free(net->v, s);
  if (s) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  cudaGetLastError();
  delete net;
  return KPM_OK;
}

}  // extern "C"
