// Vector stores and CUDA-core contractions of the correlator moments matrix
// (Correlator._calculate_moments_matrix, kwant/kpm.py:685-695):
//   mu_mn = (1/R) sum_K conj(Omega[m][K]) Psi[n][K],  K = orbital * R + vector.
// Split-K over the grid; the split partials are summed in a fixed order, so
// the result is deterministic.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_gemm.cuh"

namespace kpm {

int store_alloc(Store* s, int kind, int64_t M, int64_t K, cudaStream_t st) {
  s->kind = kind;
  s->M = M;
  s->K = K;
  if (kind == STORE_C128) {
    s->Kp = K;
    return dev_alloc((void**)&s->c128, (size_t)M * K * sizeof(double2), st);
  }
  s->Kp = round_up(K, STORE_KPAD);
  const size_t bytes = (size_t)4 * M * s->Kp * sizeof(__nv_bfloat16);
  KPM_TRY(dev_alloc((void**)&s->planes, bytes, st));
  KPM_CUDA(cudaMemsetAsync(s->planes, 0, bytes, st));
  return KPM_OK;
}

void store_free(Store* s, cudaStream_t st) {
  dev_free(s->c128, st);
  dev_free(s->planes, st);
  s->c128 = nullptr;
  s->planes = nullptr;
}

constexpr int GT = 32;  // output tile (GT x GT complex)
constexpr int GK = 16;  // K chunk staged in shared memory

// part[split][m][n] = sum_{kk in split} conj(A[m][off + kk*stride]) B[n][...]
__global__ void __launch_bounds__(256)
gemm_c128_kernel(const double2* __restrict__ A, const double2* __restrict__ B,
                 int64_t M, int64_t ld, int64_t k_off, int64_t k_len,
                 int64_t k_stride, double2* __restrict__ part) {
  const int64_t tm = blockIdx.x, tn = blockIdx.y, sp = blockIdx.z;
  const int64_t splits = gridDim.z;
  const int64_t chunk = ceil_div(k_len, splits);
  const int64_t ks = sp * chunk;
  const int64_t ke = ks + chunk < k_len ? ks + chunk : k_len;
  __shared__ double2 As[GT][GK + 1], Bs[GT][GK + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
  for (int64_t k0 = ks; k0 < ke; k0 += GK) {
    for (int e = threadIdx.x; e < GT * GK; e += blockDim.x) {
      const int r = e / GK, c = e % GK;
      const int64_t kk = k0 + c;
      const int64_t ma = tm * GT + r, nb = tn * GT + r;
      const bool ok = kk < ke;
      As[r][c] = (ok && ma < M) ? A[ma * ld + k_off + kk * k_stride]
                                : make_double2(0.0, 0.0);
      Bs[r][c] = (ok && nb < M) ? B[nb * ld + k_off + kk * k_stride]
                                : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < GK; ++c) {
      const double2 a0 = As[ty * 2][c], a1 = As[ty * 2 + 1][c];
      const double2 b0 = Bs[tx * 2][c], b1 = Bs[tx * 2 + 1][c];
      const double2 a[2] = {a0, a1}, b[2] = {b0, b1};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // conj(a) * b
          ar[i][j] = fma(a[i].x, b[j].x, fma(a[i].y, b[j].y, ar[i][j]));
          ai[i][j] = fma(a[i].x, b[j].y, fma(-a[i].y, b[j].x, ai[i][j]));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int64_t m = tm * GT + ty * 2 + i, n = tn * GT + tx * 2 + j;
      if (m < M && n < M)
        part[(sp * M + m) * M + n] = make_double2(ar[i][j], ai[i][j]);
    }
}

// 16-bit plane element as float: bfloat16, or FP16 when f16
__device__ __forceinline__ float plane_value(const __nv_bfloat16* p,
                                             int64_t i, int f16) {
  return f16 ? __half2float(reinterpret_cast<const __half*>(p)[i])
             : __bfloat162float(p[i]);
}

// Same contraction on BF16x3 planes (bfloat16, or FP16 when f16) with FP32
// products/accumulation per split (hi*hi + hi*lo + lo*hi for every real
// product).
__global__ void __launch_bounds__(256)
gemm_bf16x3_simt_kernel(const __nv_bfloat16* __restrict__ A,
                        const __nv_bfloat16* __restrict__ B, int64_t M,
                        int64_t Kp, int64_t K, int f16,
                        double2* __restrict__ part) {
  const int64_t tm = blockIdx.x, tn = blockIdx.y, sp = blockIdx.z;
  const int64_t splits = gridDim.z;
  const int64_t chunk = ceil_div(K, splits);
  const int64_t ks = sp * chunk;
  const int64_t ke = ks + chunk < K ? ks + chunk : K;
  __shared__ float As[4][GT][GK + 1], Bs[4][GT][GK + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
  for (int64_t k0 = ks; k0 < ke; k0 += GK) {
    for (int e = threadIdx.x; e < GT * GK; e += blockDim.x) {
      const int r = e / GK, c = e % GK;
      const int64_t kk = k0 + c;
      const int64_t ma = tm * GT + r, nb = tn * GT + r;
      for (int q = 0; q < 4; ++q) {
        As[q][r][c] = (kk < ke && ma < M)
                          ? plane_value(A, store_index(M, q, ma, kk), f16)
                          : 0.f;
        Bs[q][r][c] = (kk < ke && nb < M)
                          ? plane_value(B, store_index(M, q, nb, kk), f16)
                          : 0.f;
      }
    }
    __syncthreads();
    for (int c = 0; c < GK; ++c) {
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int ra = ty * 2 + i, rb = tx * 2 + j;
          const float arh = As[0][ra][c], arl = As[1][ra][c];
          const float aih = As[2][ra][c], ail = As[3][ra][c];
          const float brh = Bs[0][rb][c], brl = Bs[1][rb][c];
          const float bih = Bs[2][rb][c], bil = Bs[3][rb][c];
          // Re: Ar Br + Ai Bi ;  Im: Ar Bi - Ai Br
          ar[i][j] += arh * brh + arh * brl + arl * brh;
          ar[i][j] += aih * bih + aih * bil + ail * bih;
          ai[i][j] += arh * bih + arh * bil + arl * bih;
          ai[i][j] -= aih * brh + aih * brl + ail * brh;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int64_t m = tm * GT + ty * 2 + i, n = tn * GT + tx * 2 + j;
      if (m < M && n < M)
        part[(sp * M + m) * M + n] =
            make_double2((double)ar[i][j], (double)ai[i][j]);
    }
}

// out[m][n] = scale * sum_sp part[sp][m][n]   (sp in order)
__global__ void split_reduce_kernel(const double2* __restrict__ part,
                                    int64_t splits, int64_t MM, double scale,
                                    double2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MM) return;
  double r = 0.0, im = 0.0;
  for (int64_t s = 0; s < splits; ++s) {
    const double2 p = part[s * MM + i];
    r += p.x;
    im += p.y;
  }
  out[i] = make_double2(r * scale, im * scale);
}

static int64_t choose_splits(kpm_handle* h, int64_t tiles, int64_t k_len) {
  int64_t target = (int64_t)h->num_sms * 8;
  int64_t s = ceil_div(target, tiles);
  int64_t kmax = ceil_div(k_len, 4 * GK);
  if (s > kmax) s = kmax;
  if (s < 1) s = 1;
  if (s > 4096) s = 4096;
  return s;
}

static int finish(kpm_handle* h, double2* part, int64_t splits, int64_t M,
                  double scale, double* mu_host) {
  double2* mu = nullptr;
  KPM_TRY(dev_alloc((void**)&mu, (size_t)M * M * sizeof(double2), h->stream));
  split_reduce_kernel<<<(unsigned)ceil_div(M * M, 256), 256, 0, h->stream>>>(
      part, splits, M * M, scale, mu);
  count_launch(1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(mu_host, mu, (size_t)M * M * sizeof(double2),
                        cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dev_free(mu, h->stream);
  KPM_CUDA(e);
  return KPM_OK;
}

int gemm_fp64(kpm_handle* h, const Store* omega, const Store* psi, int64_t M,
              int64_t K, int64_t R, int per_vector, double* mu_host) {
  const int64_t tiles1 = ceil_div(M, GT);
  const int64_t nvec = per_vector ? R : 1;
  const int64_t k_len = per_vector ? K / R : K;
  const int64_t splits = choose_splits(h, tiles1 * tiles1, k_len);
  double2* part = nullptr;
  KPM_TRY(dev_alloc((void**)&part, (size_t)splits * M * M * sizeof(double2),
                    h->stream));
  int st = KPM_OK;
  for (int64_t r = 0; st == KPM_OK && r < nvec; ++r) {
    dim3 grid((unsigned)tiles1, (unsigned)tiles1, (unsigned)splits);
    gemm_c128_kernel<<<grid, 256, 0, h->stream>>>(
        omega->c128, psi->c128, M, K, per_vector ? r : 0, k_len,
        per_vector ? R : 1, part);
    count_launch(1);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("gemm_fp64: launch failed");
      st = KPM_ECUDA;
      break;
    }
    st = finish(h, part, splits, M, per_vector ? 1.0 : 1.0 / (double)R,
                mu_host + (per_vector ? 2 * r * M * M : 0));
  }
  dev_free(part, h->stream);
  return st;
}

int gemm_bf16x3_simt(kpm_handle* h, const Store* omega, const Store* psi,
                     int64_t M, int64_t K, int64_t R, double* mu_host) {
  const int64_t tiles1 = ceil_div(M, GT);
  const int64_t splits = choose_splits(h, tiles1 * tiles1, K);
  double2* part = nullptr;
  KPM_TRY(dev_alloc((void**)&part, (size_t)splits * M * M * sizeof(double2),
                    h->stream));
  dim3 grid((unsigned)tiles1, (unsigned)tiles1, (unsigned)splits);
  KPM_REQUIRE(omega->f16 == psi->f16, "gemm_bf16x3_simt: plane types differ");
  gemm_bf16x3_simt_kernel<<<grid, 256, 0, h->stream>>>(
      omega->planes, psi->planes, M, omega->Kp, K, omega->f16, part);
  count_launch(1);
  int st = KPM_OK;
  if (cudaGetLastError() != cudaSuccess) {
    set_error("gemm_bf16x3_simt: launch failed");
    st = KPM_ECUDA;
  }
  if (st == KPM_OK) st = finish(h, part, splits, M, 1.0 / (double)R, mu_host);
  dev_free(part, h->stream);
  return st;
}

}  // namespace kpm
