// Chebyshev recursion of the kernel polynomial method on GB300 (sm_103a).
//
// Replaces the per-vector loop of SpectralDensity._update_moments_list
// (kwant/kpm.py:390-490) and the rescaled matvec of _rescale
// (kwant/kpm.py:1182-1183) with one fused, batched sparse-matrix x
// multi-vector pass per Chebyshev step:
//
//   alpha_{n+1} = 2 (H alpha_n - b alpha_n) / a - alpha_{n-1}
//
// over all R vectors at once.  Vectors are stored interleaved, [row][vector],
// so a 16-lane slot reads one row of one vector group with 16-byte loads
// (1 complex128 or 2 complex64 per lane); every neighbour row is a 256-byte
// coalesced segment.  The per-vector dot products that give the DOS moments
// (<a_n|a_n>, <a_n+1|a_n>) are accumulated in FP64 in the same pass.
//
// Determinism: rows are split into a number of row partitions that depends
// only on the number of rows; each slot sums its rows in increasing order,
// slots are summed in order, partitions are summed in order.  A vector's
// moments therefore do not depend on how many other vectors share the batch
// or on the launch shape, which keeps add_vectors / add_moments bit-identical
// to a fresh run (kwant/tests/test_kpm.py:481-535).

#include <cstdarg>
#include <mutex>
#include <vector>
#include <atomic>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_tc.cuh"

namespace kpm {

// ---------------------------------------------------------------- errors
static thread_local char g_err[1024] = "";
static std::atomic<uint64_t> g_wait_ns{2000000000ull};
static std::atomic<int> g_stall_tma{0};
static std::atomic<int64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char* last_error() { return g_err; }
void count_launch(int n) { g_launches += n; }

namespace tc {
WaitCfg wait_cfg() { return WaitCfg{g_wait_ns.load(), g_stall_tma.load()}; }
}  // namespace tc

// ------------------------------------------------------------- allocation
int dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (bytes == 0) return KPM_OK;
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation of %zu bytes failed: %s", bytes,
              cudaGetErrorString(e));
    return KPM_ENOMEM;
  }
  return KPM_OK;
}

void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

int init_device(int* device, int* num_sms) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device available (%s); kwant_gb300 has no CPU path",
              e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    return KPM_ECUDA;
  }
  KPM_CUDA(cudaGetDevice(device));
  KPM_CUDA(cudaDeviceGetAttribute(num_sms, cudaDevAttrMultiProcessorCount,
                                  *device));
  static std::once_flag once;
  static int pool_status = KPM_OK;
  std::call_once(once, [&]() {
    // Keep freed blocks in the stream-ordered pool so that repeated
    // create/destroy cycles do not return memory to the driver.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, *device) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
  });
  return pool_status;
}

// ---------------------------------------------------------------- matrices
__global__ void scale_to_c64_kernel(const double2* __restrict__ in,
                                    float2* __restrict__ out, int64_t n,
                                    double scale) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = make_float2((float)(in[i].x * scale), (float)(in[i].y * scale));
}

// Validate a CSR on the host so that no kernel ever indexes out of bounds.
int validate_csr(const kpm_csr_desc* m) {
  KPM_REQUIRE(m->rows > 0 && m->nnz >= 0 && m->indptr && m->indices,
              "invalid CSR descriptor");
  KPM_REQUIRE(m->indptr[0] == 0 && m->indptr[m->rows] == m->nnz,
              "CSR indptr must start at 0 and end at nnz");
  for (int64_t i = 0; i < m->rows; ++i)
    KPM_REQUIRE(m->indptr[i] <= m->indptr[i + 1],
                "CSR indptr not monotone at row %lld", (long long)i);
  for (int64_t k = 0; k < m->nnz; ++k)
    KPM_REQUIRE(m->indices[k] >= 0 && m->indices[k] < m->rows,
                "CSR column index out of range at entry %lld", (long long)k);
  return KPM_OK;
}

namespace {

// device staging buffer released on every exit path
struct Staging {
  void* p = nullptr;
  cudaStream_t s;
  explicit Staging(cudaStream_t st) : s(st) {}
  ~Staging() { dev_free(p, s); }
  int alloc(size_t bytes) { return dev_alloc(&p, bytes, s); }
};

}  // namespace

// new row p = old row perm[p], columns renumbered by iperm, entry order
// within each row kept; values complex128 (C64 false) or complex64 * scale
template <bool C64>
__global__ void permute_rows_kernel(int64_t n, const int32_t* __restrict__ perm,
                                    const int32_t* __restrict__ iperm,
                                    const int32_t* __restrict__ oip,
                                    const int32_t* __restrict__ oix,
                                    const double2* __restrict__ oval,
                                    const int32_t* __restrict__ nip,
                                    int32_t* __restrict__ nix,
                                    void* __restrict__ nval, double scale) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t o = perm[p];
  int32_t dst = nip[p];
  for (int32_t k = oip[o]; k < oip[o + 1]; ++k, ++dst) {
    nix[dst] = iperm[oix[k]];
    const double2 v = oval[k];
    if constexpr (C64)
      static_cast<float2*>(nval)[dst] =
          make_float2((float)(v.x * scale), (float)(v.y * scale));
    else
      static_cast<double2*>(nval)[dst] = v;
  }
}

// ELL rows of width K from a device CSR with complex64 values; padding
// entries point at the row itself with value 0
__global__ void ell_from_csr_kernel(int64_t n, int K,
                                    const int32_t* __restrict__ ip,
                                    const int32_t* __restrict__ ix,
                                    const float2* __restrict__ val,
                                    int32_t* __restrict__ eidx,
                                    float2* __restrict__ eval) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int q = 0;
  for (int32_t k = ip[p]; k < ip[p + 1]; ++k, ++q) {
    eidx[p * K + q] = ix[k];
    eval[p * K + q] = val[k];
  }
  for (; q < K; ++q) {
    eidx[p * K + q] = (int32_t)p;
    eval[p * K + q] = make_float2(0.f, 0.f);
  }
}

int upload_matrix(kpm_handle* h, const kpm_csr_desc* m, double scale,
                  Matrix* out, bool with_ell) {
  return upload_matrix_perm(h, m, scale, out, with_ell, nullptr, nullptr,
                            true);
}

int upload_matrix_perm(kpm_handle* h, const kpm_csr_desc* m, double scale,
                       Matrix* out, bool with_ell, const int32_t* perm,
                       const int32_t* iperm, bool validate) {
  if (validate) KPM_TRY(validate_csr(m));
  cudaStream_t s = h->stream;
  const int64_t n = m->rows;
  const int64_t nz = m->nnz > 0 ? m->nnz : 1;
  const bool c64 = scale != 0.0;
  out->rows = n;
  out->nnz = m->nnz;
  KPM_TRY(dev_alloc((void**)&out->indptr, (n + 1) * sizeof(int32_t), s));
  KPM_TRY(dev_alloc((void**)&out->indices, nz * sizeof(int32_t), s));
  KPM_TRY(dev_alloc(&out->data, nz * (c64 ? sizeof(float2) : sizeof(double2)),
                    s));
  Staging vals(s);
  if (!perm) {
    KPM_CUDA(cudaMemcpyAsync(out->indptr, m->indptr, (n + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    if (m->nnz > 0)
      KPM_CUDA(cudaMemcpyAsync(out->indices, m->indices,
                               m->nnz * sizeof(int32_t),
                               cudaMemcpyHostToDevice, s));
    if (!c64) {
      if (m->nnz > 0)
        KPM_CUDA(cudaMemcpyAsync(out->data, m->data, m->nnz * sizeof(double2),
                                 cudaMemcpyHostToDevice, s));
    } else if (m->nnz > 0) {
      KPM_TRY(vals.alloc(m->nnz * sizeof(double2)));
      KPM_CUDA(cudaMemcpyAsync(vals.p, m->data, m->nnz * sizeof(double2),
                               cudaMemcpyHostToDevice, s));
      scale_to_c64_kernel<<<(unsigned)ceil_div(m->nnz, 256), 256, 0, s>>>(
          (const double2*)vals.p, (float2*)out->data, m->nnz, scale);
      count_launch(1);
      KPM_CHECK_LAUNCH();
    }
  } else {
    // row pointers of the permuted matrix (host, O(rows)); the entries are
    // moved on the device
    std::vector<int32_t> nip(n + 1);
    nip[0] = 0;
    for (int64_t p = 0; p < n; ++p)
      nip[p + 1] = nip[p] + (m->indptr[perm[p] + 1] - m->indptr[perm[p]]);
    KPM_CUDA(cudaMemcpyAsync(out->indptr, nip.data(),
                             (n + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    Staging oip(s), oix(s), dperm(s), diperm(s);
    KPM_TRY(oip.alloc((n + 1) * sizeof(int32_t)));
    KPM_TRY(oix.alloc(nz * sizeof(int32_t)));
    KPM_TRY(vals.alloc(nz * sizeof(double2)));
    KPM_TRY(dperm.alloc(n * sizeof(int32_t)));
    KPM_TRY(diperm.alloc(n * sizeof(int32_t)));
    KPM_CUDA(cudaMemcpyAsync(oip.p, m->indptr, (n + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    if (m->nnz > 0) {
      KPM_CUDA(cudaMemcpyAsync(oix.p, m->indices, m->nnz * sizeof(int32_t),
                               cudaMemcpyHostToDevice, s));
      KPM_CUDA(cudaMemcpyAsync(vals.p, m->data, m->nnz * sizeof(double2),
                               cudaMemcpyHostToDevice, s));
    }
    KPM_CUDA(cudaMemcpyAsync(dperm.p, perm, n * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    KPM_CUDA(cudaMemcpyAsync(diperm.p, iperm, n * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    const unsigned blocks = (unsigned)ceil_div(n, 256);
    if (c64)
      permute_rows_kernel<true><<<blocks, 256, 0, s>>>(
          n, (const int32_t*)dperm.p, (const int32_t*)diperm.p,
          (const int32_t*)oip.p, (const int32_t*)oix.p,
          (const double2*)vals.p, out->indptr, out->indices, out->data, scale);
    else
      permute_rows_kernel<false><<<blocks, 256, 0, s>>>(
          n, (const int32_t*)dperm.p, (const int32_t*)diperm.p,
          (const int32_t*)oip.p, (const int32_t*)oix.p,
          (const double2*)vals.p, out->indptr, out->indices, out->data, 0.0);
    count_launch(1);
    KPM_CHECK_LAUNCH();
    // the staging buffers are released (stream-ordered) when this scope
    // ends, after the kernel that reads them
  }
  if (c64 && with_ell) KPM_TRY(build_ell(h, m, out));
  KPM_CUDA(cudaStreamSynchronize(s));
  return KPM_OK;
}

// ELL copy (complex64) of a device CSR whose rows have at most ELL_MAX
// entries; the width comes from the host row pointers.
int build_ell(kpm_handle* h, const kpm_csr_desc* m, Matrix* out) {
  int64_t maxnnz = 0;
  for (int64_t i = 0; i < m->rows; ++i)
    maxnnz = std::max<int64_t>(maxnnz, m->indptr[i + 1] - m->indptr[i]);
  const int64_t K = round_up(maxnnz > 0 ? maxnnz : 1, 4);
  if (K > ELL_MAX) return KPM_OK;  // the CSR kernel handles wide rows
  const size_t cnt = (size_t)m->rows * K;
  KPM_TRY(dev_alloc((void**)&out->ell_idx, cnt * sizeof(int32_t), h->stream));
  KPM_TRY(dev_alloc((void**)&out->ell_val, cnt * sizeof(float2), h->stream));
  ell_from_csr_kernel<<<(unsigned)ceil_div(m->rows, 256), 256, 0,
                        h->stream>>>(m->rows, (int)K, out->indptr, out->indices,
                                     (const float2*)out->data, out->ell_idx,
                                     out->ell_val);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  out->ell_k = (int)K;
  return KPM_OK;
}

void free_matrix(Matrix* m, cudaStream_t s) {
  dev_free(m->indptr, s);
  dev_free(m->indices, s);
  dev_free(m->data, s);
  dev_free(m->ell_idx, s);
  dev_free(m->ell_val, s);
  m->ell_idx = nullptr;
  m->ell_val = nullptr;
  m->ell_k = 0;
  m->indptr = nullptr;
  m->indices = nullptr;
  m->data = nullptr;
}

// ----------------------------------------------------------- vector layout
// [R][N] complex128 (host order)  ->  [N][Rpad] complex (device order)
template <typename OutT>
__global__ void to_interleaved_kernel(const double2* __restrict__ in,
                                      OutT* __restrict__ out, int64_t N,
                                      int64_t R, int64_t Rpad,
                                      const int32_t* __restrict__ perm) {
  __shared__ double2 tile[32][33];
  const int64_t n0 = (int64_t)blockIdx.x * 32;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t r = r0 + k, n = n0 + threadIdx.x;
    double2 v = make_double2(0.0, 0.0);
    if (r < R && n < N) v = in[r * N + (perm ? perm[n] : n)];
    tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t n = n0 + k, r = r0 + threadIdx.x;
    if (n < N && r < Rpad) {
      double2 v = tile[threadIdx.x][k];
      if constexpr (sizeof(OutT) == 16) {
        out[n * Rpad + r] = *reinterpret_cast<OutT*>(&v);
      } else {
        float2 f = make_float2((float)v.x, (float)v.y);
        out[n * Rpad + r] = *reinterpret_cast<OutT*>(&f);
      }
    }
  }
}

// [N][Rpad] complex (device order) -> [R][N] complex128
template <typename InT>
__global__ void from_interleaved_kernel(const InT* __restrict__ in,
                                        double2* __restrict__ out, int64_t N,
                                        int64_t R, int64_t Rpad,
                                        const int32_t* __restrict__ perm) {
  __shared__ double2 tile[32][33];
  const int64_t n0 = (int64_t)blockIdx.x * 32;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t n = n0 + k, r = r0 + threadIdx.x;
    double2 v = make_double2(0.0, 0.0);
    if (n < N && r < Rpad) {
      if constexpr (sizeof(InT) == 16) {
        v = *reinterpret_cast<const double2*>(&in[n * Rpad + r]);
      } else {
        float2 f = *reinterpret_cast<const float2*>(&in[n * Rpad + r]);
        v = make_double2((double)f.x, (double)f.y);
      }
    }
    tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t r = r0 + k, n = n0 + threadIdx.x;
    if (r < R && n < N) out[r * N + (perm ? perm[n] : n)] = tile[threadIdx.x][k];
  }
}

// [R][N] complex128 -> hi [N][Rpad] complex64 + lo [N][Rpad] bfloat16 x 2:
// hi = RN(v), lo = RZ_bf16(RZ_f32(v - hi)) (v - hi is exact in FP64).  The
// split of hi + lo (as downloaded) gives back the same hi and lo.
__device__ __forceinline__ float lo_part(double v, float hi) {
  const float d = __double2float_rz(v - (double)hi);
  return __uint_as_float(__float_as_uint(d) & 0xffff0000u);
}
__global__ void to_interleaved_hilo_kernel(const double2* __restrict__ in,
                                           float2* __restrict__ out,
                                           uint32_t* __restrict__ lo,
                                           int64_t N, int64_t R, int64_t Rpad,
                                           const int32_t* __restrict__ perm) {
  __shared__ double2 tile[32][33];
  const int64_t n0 = (int64_t)blockIdx.x * 32;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t r = r0 + k, n = n0 + threadIdx.x;
    double2 v = make_double2(0.0, 0.0);
    if (r < R && n < N) v = in[r * N + (perm ? perm[n] : n)];
    tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t n = n0 + k, r = r0 + threadIdx.x;
    if (n < N && r < Rpad) {
      const double2 v = tile[threadIdx.x][k];
      const float hr = (float)v.x, hi = (float)v.y;
      out[n * Rpad + r] = make_float2(hr, hi);
      lo[n * Rpad + r] = (__float_as_uint(lo_part(v.x, hr)) >> 16) |
                         (__float_as_uint(lo_part(v.y, hi)) & 0xffff0000u);
    }
  }
}

// hi + lo [N][Rpad] -> [R][N] complex128 (exact)
__global__ void from_interleaved_hilo_kernel(const float2* __restrict__ in,
                                             const uint32_t* __restrict__ lo,
                                             double2* __restrict__ out,
                                             int64_t N, int64_t R,
                                             int64_t Rpad,
                                             const int32_t* __restrict__ perm) {
  __shared__ double2 tile[32][33];
  const int64_t n0 = (int64_t)blockIdx.x * 32;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t n = n0 + k, r = r0 + threadIdx.x;
    double2 v = make_double2(0.0, 0.0);
    if (n < N && r < Rpad) {
      const float2 f = in[n * Rpad + r];
      const uint32_t w = lo[n * Rpad + r];
      v = make_double2((double)f.x + (double)__uint_as_float(w << 16),
                       (double)f.y + (double)__uint_as_float(w & 0xffff0000u));
    }
    tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int64_t r = r0 + k, n = n0 + threadIdx.x;
    if (r < R && n < N) out[r * N + (perm ? perm[n] : n)] = tile[threadIdx.x][k];
  }
}

int upload_vectors(kpm_handle* h, const double* host, int64_t R, int64_t N,
                   int64_t Rpad, void* dst) {
  return upload_vectors_lo(h, host, R, N, Rpad, dst, nullptr);
}

int upload_vectors_lo(kpm_handle* h, const double* host, int64_t R,
                      int64_t N, int64_t Rpad, void* dst, uint32_t* lo) {
  void* staging = nullptr;
  size_t bytes = (size_t)R * N * 16;
  cudaError_t e = cudaSuccess;
  if (h->vec_staging && h->vec_staging_src == host &&
      h->vec_staging_bytes == bytes) {
    staging = h->vec_staging;          // copied ahead of time
    h->vec_staging = nullptr;
    h->vec_staging_src = nullptr;
    h->vec_staging_bytes = 0;
  } else {
    KPM_TRY(dev_alloc(&staging, bytes, h->stream));
    e = cudaMemcpyAsync(staging, host, bytes, cudaMemcpyHostToDevice,
                        h->stream);
  }
  if (e != cudaSuccess) {
    dev_free(staging, h->stream);
    KPM_CUDA(e);
  }
  dim3 blk(32, 8), grd((unsigned)ceil_div(N, 32), (unsigned)ceil_div(Rpad, 32));
  if (h->precision == KPM_PREC_MIXED && lo)
    to_interleaved_hilo_kernel<<<grd, blk, 0, h->stream>>>(
        (const double2*)staging, (float2*)dst, lo, N, R, Rpad, h->perm);
  else if (h->precision == KPM_PREC_MIXED)
    to_interleaved_kernel<float2><<<grd, blk, 0, h->stream>>>(
        (const double2*)staging, (float2*)dst, N, R, Rpad, h->perm);
  else
    to_interleaved_kernel<double2><<<grd, blk, 0, h->stream>>>(
        (const double2*)staging, (double2*)dst, N, R, Rpad, h->perm);
  count_launch(1);
  e = cudaGetLastError();
  dev_free(staging, h->stream);
  KPM_CUDA(e);
  return KPM_OK;
}

int download_vectors(kpm_handle* h, const void* src, int64_t R, int64_t N,
                     int64_t Rpad, double* host) {
  return download_vectors_lo(h, src, nullptr, R, N, Rpad, host);
}

int download_vectors_lo(kpm_handle* h, const void* src, const uint32_t* lo,
                        int64_t R, int64_t N, int64_t Rpad, double* host) {
  void* staging = nullptr;
  size_t bytes = (size_t)R * N * 16;
  KPM_TRY(dev_alloc(&staging, bytes, h->stream));
  dim3 blk(32, 8), grd((unsigned)ceil_div(N, 32), (unsigned)ceil_div(Rpad, 32));
  if (h->precision == KPM_PREC_MIXED && lo)
    from_interleaved_hilo_kernel<<<grd, blk, 0, h->stream>>>(
        (const float2*)src, lo, (double2*)staging, N, R, Rpad, h->perm);
  else if (h->precision == KPM_PREC_MIXED)
    from_interleaved_kernel<float2><<<grd, blk, 0, h->stream>>>(
        (const float2*)src, (double2*)staging, N, R, Rpad, h->perm);
  else
    from_interleaved_kernel<double2><<<grd, blk, 0, h->stream>>>(
        (const double2*)src, (double2*)staging, N, R, Rpad, h->perm);
  count_launch(1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host, staging, bytes, cudaMemcpyDeviceToHost,
                        h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dev_free(staging, h->stream);
  KPM_CUDA(e);
  return KPM_OK;
}

// ------------------------------------------------------------ step kernel
template <bool MIXED, int VPL> struct Traits;
template <> struct Traits<false, 1> {
  using PT = double2;
  using VT = double2;
  static constexpr int VPL = 1;
  static constexpr int G = GROUP_FP64;
};
template <> struct Traits<true, 2> {
  using PT = float4;
  using VT = float2;
  static constexpr int VPL = 2;
  static constexpr int G = GROUP_FP32;
};
template <> struct Traits<true, 1> {
  using PT = float2;
  using VT = float2;
  static constexpr int VPL = 1;
  static constexpr int G = GROUP_FP64;
};

// complex64 payload access: vector k (0 or 1) of a lane's payload
__device__ __forceinline__ float c64_re(const float4& v, int k) {
  return k ? v.z : v.x;
}
__device__ __forceinline__ float c64_im(const float4& v, int k) {
  return k ? v.w : v.y;
}
__device__ __forceinline__ float c64_re(const float2& v, int) { return v.x; }
__device__ __forceinline__ float c64_im(const float2& v, int) { return v.y; }
template <int VPL> struct C64Pay;
template <> struct C64Pay<2> {
  __device__ static float4 make(const float (&r)[2], const float (&i)[2]) {
    return make_float4(r[0], i[0], r[1], i[1]);
  }
};
template <> struct C64Pay<1> {
  __device__ static float2 make(const float (&r)[1], const float (&i)[1]) {
    return make_float2(r[0], i[0]);
  }
};

// sum += h x in CSR order (scipy's csr_matvec, kwant/kpm.py:1182), as four
// FMAs.  GB300's FP64 pipe issues an FMA at the rate of a multiply or an
// add, so this is half the instructions of scipy's separately rounded
// (hr xr - hi xi) + i (hr xi + hi xr): the FP64 step is FP64-pipe bound, and
// the fused form took it from 11.7 to 7.1 ms per step on the 2e6-orbital
// graphene workload (R = 64).  Results stay within 1e-15 relative of the
// reference's arithmetic per step.
__device__ __forceinline__ void cmul_acc_fma(double& ar, double& ai,
                                             double2 h, double2 x) {
  ar = fma(h.x, x.x, fma(-h.y, x.y, ar));
  ai = fma(h.x, x.y, fma(h.y, x.x, ai));
}

template <bool MIXED, int MODE, bool DOTS, int VPL_ = (MIXED ? 2 : 1)>
__global__ void __launch_bounds__(STEP_THREADS)
cheb_step_kernel(StepArgs p) {
  using T = Traits<MIXED, VPL_>;
  using PT = typename T::PT;
  using VT = typename T::VT;
  constexpr int VPL = T::VPL;
  constexpr int G = T::G;
  const int lane = threadIdx.x & (LANES - 1);
  const int slot = threadIdx.x / LANES;
  // per-slot dot-product partials (DOS dots, or the norm of the odd tail)
  constexpr bool RED = DOTS || MODE == STEP_NORM;
  __shared__ double red[RED ? SLOTS : 1][RED ? G * 3 : 1];

  const PT* __restrict__ x = reinterpret_cast<const PT*>(p.x);
  const PT* prev = reinterpret_cast<const PT*>(p.prev);
  PT* out = reinterpret_cast<PT*>(p.out);
  const VT* __restrict__ vals = reinterpret_cast<const VT*>(p.vals);
  const int32_t* __restrict__ indptr = p.indptr;
  const int32_t* __restrict__ indices = p.indices;
  const int64_t work = (int64_t)p.xitems * p.groups;
  const int64_t stride = (int64_t)p.xitems * SLOTS;

  for (int64_t w = blockIdx.x; w < work; w += gridDim.x) {
    const int xi = (int)(w / p.groups);
    const int g = (int)(w - (int64_t)xi * p.groups);
    const int64_t col = (int64_t)g * LANES + lane;
    double nrm[VPL], cre[VPL], cim[VPL];
    // complex64 path: FP32 partials over at most FLUSH rows, then added to
    // the FP64 accumulators.  GB300's FP64 pipe is narrow; per-row FP64 dot
    // products would bound the kernel.
    float fn[VPL], fcr[VPL], fci[VPL];
    int pending = 0;
    constexpr int FLUSH = 32;
#pragma unroll
    for (int k = 0; k < VPL; ++k) {
      nrm[k] = cre[k] = cim[k] = 0.0;
      fn[k] = fcr[k] = fci[k] = 0.f;
    }
    auto flush = [&]() {
#pragma unroll
      for (int k = 0; k < VPL; ++k) {
        nrm[k] += (double)fn[k];
        cre[k] += (double)fcr[k];
        cim[k] += (double)fci[k];
        fn[k] = fcr[k] = fci[k] = 0.f;
      }
      pending = 0;
    };

    for (int64_t i = (int64_t)xi * SLOTS + slot; i < p.rows; i += stride) {
      const PT xv = x[i * p.rp + col];
      if constexpr (MODE == STEP_NORM) {
        if constexpr (MIXED) {
#pragma unroll
          for (int k = 0; k < VPL; ++k)
            fn[k] = fmaf(c64_re(xv, k), c64_re(xv, k),
                         fmaf(c64_im(xv, k), c64_im(xv, k), fn[k]));
          if (++pending == FLUSH) flush();
        } else {
          nrm[0] = fma(xv.x, xv.x, fma(xv.y, xv.y, nrm[0]));
        }
        continue;
      }
      const int beg = __ldg(indptr + i), end = __ldg(indptr + i + 1);
      PT o;
      if constexpr (!MIXED) {
        double ar = 0.0, ai = 0.0;
        int jj = beg;
        for (; jj + 4 <= end; jj += 4) {
          int c0 = col_index(p, __ldg(indices + jj)), c1 = col_index(p, __ldg(indices + jj + 1));
          int c2 = col_index(p, __ldg(indices + jj + 2)), c3 = col_index(p, __ldg(indices + jj + 3));
          double2 h0 = vals[jj], h1 = vals[jj + 1];
          double2 h2 = vals[jj + 2], h3 = vals[jj + 3];
          double2 x0 = x[(int64_t)c0 * p.rp + col];
          double2 x1 = x[(int64_t)c1 * p.rp + col];
          double2 x2 = x[(int64_t)c2 * p.rp + col];
          double2 x3 = x[(int64_t)c3 * p.rp + col];
          cmul_acc_fma(ar, ai, h0, x0);
          cmul_acc_fma(ar, ai, h1, x1);
          cmul_acc_fma(ar, ai, h2, x2);
          cmul_acc_fma(ar, ai, h3, x3);
        }
        for (; jj < end; ++jj) {
          int c = col_index(p, __ldg(indices + jj));
          cmul_acc_fma(ar, ai, vals[jj], x[(int64_t)c * p.rp + col]);
        }
        // (H v - b v) * (1/a): numpy's order (kwant/kpm.py:1183; complex
        // division by a real is a multiplication by the rounded reciprocal)
        double tr = __dmul_rn(fma(-p.b, xv.x, ar), p.inv_a);
        double ti = __dmul_rn(fma(-p.b, xv.y, ai), p.inv_a);
        if constexpr (MODE == STEP_FIRST) {
          o = make_double2(tr, ti);
        } else {
          const double2 pv = prev[i * p.rp + col];
          o = make_double2(__dsub_rn(__dmul_rn(2.0, tr), pv.x),
                           __dsub_rn(__dmul_rn(2.0, ti), pv.y));
        }
      } else {
        // complex64: values are 2H/a, shift = -2b/a; FMA everywhere (the
        // same sequence for every vector whatever the vectors per lane).
        float ar[VPL], ai[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          ar[k] = p.shift * c64_re(xv, k);
          ai[k] = p.shift * c64_im(xv, k);
        }
        auto mac = [&](const float2 h, const PT xx) {
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            ar[k] = fmaf(h.x, c64_re(xx, k), ar[k]);
            ar[k] = fmaf(-h.y, c64_im(xx, k), ar[k]);
            ai[k] = fmaf(h.x, c64_im(xx, k), ai[k]);
            ai[k] = fmaf(h.y, c64_re(xx, k), ai[k]);
          }
        };
        int jj = beg;
        for (; jj + 4 <= end; jj += 4) {
          int c[4];
          float2 h[4];
          PT xx[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            c[u] = col_index(p, __ldg(indices + jj + u));
            h[u] = vals[jj + u];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) xx[u] = x[(int64_t)c[u] * p.rp + col];
#pragma unroll
          for (int u = 0; u < 4; ++u) mac(h[u], xx[u]);
        }
        for (; jj < end; ++jj) {
          int c = col_index(p, __ldg(indices + jj));
          mac(vals[jj], x[(int64_t)c * p.rp + col]);
        }
        float orr[VPL], oii[VPL];
        if constexpr (MODE == STEP_FIRST) {
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            orr[k] = 0.5f * ar[k];
            oii[k] = 0.5f * ai[k];
          }
        } else {
          const PT pv = prev[i * p.rp + col];
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            orr[k] = ar[k] - c64_re(pv, k);
            oii[k] = ai[k] - c64_im(pv, k);
          }
        }
        o = C64Pay<VPL>::make(orr, oii);
      }
      out[i * p.rp + col] = o;
      if constexpr (DOTS) {
        // <x|x> and <o|x> = sum conj(o) x
        if constexpr (MIXED) {
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            const float xr = c64_re(xv, k), xi = c64_im(xv, k);
            const float or_ = c64_re(o, k), oi = c64_im(o, k);
            fn[k] = fmaf(xr, xr, fmaf(xi, xi, fn[k]));
            fcr[k] = fmaf(or_, xr, fmaf(oi, xi, fcr[k]));
            fci[k] = fmaf(or_, xi, fmaf(-oi, xr, fci[k]));
          }
          if (++pending == FLUSH) flush();
        } else {
          nrm[0] = fma(xv.x, xv.x, fma(xv.y, xv.y, nrm[0]));
          cre[0] = fma(o.x, xv.x, fma(o.y, xv.y, cre[0]));
          cim[0] = fma(o.x, xv.y, fma(-o.y, xv.x, cim[0]));
        }
      }
    }
    if constexpr (RED) {
      if constexpr (MIXED) flush();
#pragma unroll
      for (int k = 0; k < VPL; ++k) {
        red[slot][(lane * VPL + k) * 3 + 0] = nrm[k];
        red[slot][(lane * VPL + k) * 3 + 1] = cre[k];
        red[slot][(lane * VPL + k) * 3 + 2] = cim[k];
      }
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

// Sum the row-partition partials of every vector in a fixed order and turn
// them into moments.  One block per vector.
__global__ void dos_finalize_kernel(const double* __restrict__ partials,
                                    int G, int xitems, int64_t Rpad,
                                    int mode, double2* mu01,
                                    double2* mom, int64_t mom_stride,
                                    int64_t slot_even, int64_t slot_odd) {
  const int64_t v = blockIdx.x;
  const int g = (int)(v / G), e0 = (int)(v % G) * 3;
  __shared__ double s[3][128];
  double acc[3] = {0.0, 0.0, 0.0};
  const double* src = partials + ((int64_t)g * (G * 3) + e0) * xitems;
  for (int xi = threadIdx.x; xi < xitems; xi += blockDim.x) {
    acc[0] += src[xi];
    acc[1] += src[xitems + xi];
    acc[2] += src[2 * (int64_t)xitems + xi];
  }
  for (int c = 0; c < 3; ++c) s[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 3; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double nrm = s[0][0], cre = s[1][0], cim = s[2][0];
  if (mode == STEP_FIRST) {
    double2 m0 = make_double2(nrm, 0.0);
    double2 m1 = make_double2(cre, -cim);  // <a0|a1> = conj(<a1|a0>)
    mu01[2 * v] = m0;
    mu01[2 * v + 1] = m1;
    if (slot_even >= 0) mom[slot_even * mom_stride + v] = m0;
    if (slot_odd >= 0) mom[slot_odd * mom_stride + v] = m1;
  } else if (mode == STEP_RECUR) {
    const double2 m0 = mu01[2 * v], m1 = mu01[2 * v + 1];
    if (slot_even >= 0)
      mom[slot_even * mom_stride + v] =
          make_double2(2.0 * nrm - m0.x, 0.0 - m0.y);
    if (slot_odd >= 0)
      mom[slot_odd * mom_stride + v] =
          make_double2(2.0 * cre - m1.x, 2.0 * cim - m1.y);
  } else {  // STEP_NORM: odd tail
    const double2 m0 = mu01[2 * v];
    if (slot_even >= 0)
      mom[slot_even * mom_stride + v] =
          make_double2(2.0 * nrm - m0.x, 0.0 - m0.y);
  }
}

// [count][Rpad] complex -> [R][count] complex
__global__ void moments_to_host_order_kernel(const double2* __restrict__ in,
                                             double2* __restrict__ out,
                                             int64_t count, int64_t R,
                                             int64_t Rpad, int64_t W) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = R * count * W;
  if (idx >= total) return;
  int64_t w = idx % W;
  int64_t m = (idx / W) % count;
  int64_t r = idx / (W * count);
  out[idx] = in[(m * W + w) * Rpad + r];
}

// --------------------------------------------------------------- dispatch

// Per-launch profiling (kpm_profile): an event pair around the next
// step launch on the handle's stream; *e1 = the closing event, or nullptr
// when profiling is off.
int dos_xitems(const kpm_handle* h, int64_t rows) {
  return xitems_for_rows(rows, h->num_sms,
                         h->compensated && h->H.ell_k > 0 ? 2
                                                          : XITEMS_PER_SM);
}

int prof_begin(kpm_handle* h, cudaEvent_t* e1) {
  *e1 = nullptr;
  if (!h->profiling) return KPM_OK;
  while (h->prof_events.size() < h->prof_used + 2) {
    cudaEvent_t e;
    KPM_CUDA(cudaEventCreate(&e));
    h->prof_events.push_back(e);
  }
  KPM_CUDA(cudaEventRecord(h->prof_events[h->prof_used], h->stream));
  *e1 = h->prof_events[h->prof_used + 1];
  h->prof_used += 2;
  return KPM_OK;
}

template <bool MIXED, int MODE, bool DOTS, int VPL = (MIXED ? 2 : 1)>
static int launch_step_t(kpm_handle* h, const StepArgs& a) {
  static int occ = -1;
  if (occ < 0) {
    int blocks = 0;
    KPM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks, cheb_step_kernel<MIXED, MODE, DOTS, VPL>, STEP_THREADS, 0));
    occ = blocks > 0 ? blocks : 1;
  }
  int64_t work = (int64_t)a.xitems * a.groups;
  int64_t grid = (int64_t)occ * h->num_sms;
  if (grid > work) grid = work;
  cudaEvent_t e1 = nullptr;
  KPM_TRY(prof_begin(h, &e1));
  cheb_step_kernel<MIXED, MODE, DOTS, VPL>
      <<<(unsigned)grid, STEP_THREADS, 0, h->stream>>>(a);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (e1) KPM_CUDA(cudaEventRecord(e1, h->stream));
  return KPM_OK;
}

int launch_step(kpm_handle* h, int mode, bool dots, const StepArgs& a) {
  const bool mixed = h->precision == KPM_PREC_MIXED;
  if (mixed && h->H.ell_k > 0 && mode != STEP_NORM && a.vals == h->H.data)
    return launch_step_ell(h, mode, dots, a);
  if (mixed && a.vpl == 1) {
    if (mode == STEP_FIRST)
      return dots ? launch_step_t<true, STEP_FIRST, true, 1>(h, a)
                  : launch_step_t<true, STEP_FIRST, false, 1>(h, a);
    if (mode == STEP_RECUR)
      return dots ? launch_step_t<true, STEP_RECUR, true, 1>(h, a)
                  : launch_step_t<true, STEP_RECUR, false, 1>(h, a);
    return launch_step_t<true, STEP_NORM, false, 1>(h, a);
  }
  if (mixed) {
    if (mode == STEP_FIRST)
      return dots ? launch_step_t<true, STEP_FIRST, true>(h, a)
                  : launch_step_t<true, STEP_FIRST, false>(h, a);
    if (mode == STEP_RECUR)
      return dots ? launch_step_t<true, STEP_RECUR, true>(h, a)
                  : launch_step_t<true, STEP_RECUR, false>(h, a);
    return launch_step_t<true, STEP_NORM, false>(h, a);
  }
  if (mode == STEP_FIRST)
    return dots ? launch_step_t<false, STEP_FIRST, true>(h, a)
                : launch_step_t<false, STEP_FIRST, false>(h, a);
  if (mode == STEP_RECUR)
    return dots ? launch_step_t<false, STEP_RECUR, true>(h, a)
                : launch_step_t<false, STEP_RECUR, false>(h, a);
  return launch_step_t<false, STEP_NORM, false>(h, a);
}

int ensure_partials(kpm_handle* h, int groups, int xitems) {
  size_t need = (size_t)groups * xitems * group_size(h->precision) * 3;
  if (need <= h->partials_cap) return KPM_OK;
  dev_free(h->partials, h->stream);
  h->partials = nullptr;
  h->partials_cap = 0;
  KPM_TRY(dev_alloc((void**)&h->partials, need * sizeof(double), h->stream));
  h->partials_cap = need;
  return KPM_OK;
}

StepArgs step_args(kpm_block* b, const void* x, const void* prev, void* out) {
  kpm_handle* h = b->h;
  StepArgs a{};
  a.rows = b->N;
  a.indptr = h->H.indptr;
  a.indices = h->H.indices;
  a.vals = h->H.data;
  a.b = h->b;
  a.inv_a = 1.0 / h->a;
  a.shift = (float)(-2.0 * h->b / h->a);
  a.x = x;
  a.prev = prev;
  a.out = out;
  a.vpl = h->precision == KPM_PREC_MIXED ? b->G / GROUP_FP64 : 1;
  a.rp = b->Rpad / a.vpl;
  a.groups = b->groups;
  a.xitems = dos_xitems(h, b->N);
  a.partials = h->partials;
  a.check = h->check;
  return a;
}

int check_bounds(kpm_handle* h, const char* where) {
#ifdef KPM_CHECK
  if (!h->check) return KPM_OK;
  unsigned long long v = 0;
  KPM_CUDA(cudaMemcpyAsync(&v, h->check, sizeof(v), cudaMemcpyDeviceToHost,
                           h->stream));
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  if (v) {
    KPM_CUDA(cudaMemsetAsync(h->check, 0, sizeof(v), h->stream));
    set_error("%s: bounds check: column index %llu outside [0, %lld)", where,
              v - 1, (long long)h->H.rows);
    return KPM_EINVAL;
  }
#else
  (void)h;
  (void)where;
#endif
  return KPM_OK;
}

// The output buffer of the step that advances a block from p_cur, its
// alpha_{n-1} input and the step mode: alpha_1 goes to buf[0]; afterwards
// alpha_{n+1} overwrites alpha_{n-1} in place, except a kept alpha_0.
static void* next_out(kpm_block* b, const void** prev, int* mode) {
  if (b->steps_done == 0) {
    *prev = nullptr;
    *mode = STEP_FIRST;
    return b->buf[0];
  }
  *prev = b->p_prev;
  *mode = STEP_RECUR;
  if (b->p_prev == b->a0 && b->keep_a0)
    return (b->p_cur == b->buf[0]) ? b->buf[1] : b->buf[0];
  return b->p_prev;
}

static void rotate(kpm_block* b, void* out) {
  b->p_prev = b->p_cur;
  b->p_cur = out;
  b->steps_done += 1;
}

// Advance the block's recursion by one matvec.  On the first call alpha_1 =
// H~ alpha_0; afterwards alpha_{n+1} = 2 H~ alpha_n - alpha_{n-1}.
int block_advance(kpm_block* b, bool dots) {
  const void* prev;
  int mode;
  void* out = next_out(b, &prev, &mode);
  StepArgs a = step_args(b, b->p_cur, prev, out);
  KPM_TRY(launch_step(b->h, mode, dots, a));
  rotate(b, out);
  return KPM_OK;
}

uint32_t* block_lo(const kpm_block* b, const void* hi) {
  if (!b->lo_a0 || !hi) return nullptr;
  if (hi == b->buf[0]) return b->lo_buf[0];
  if (hi == b->buf[1]) return b->lo_buf[1];
  if (hi == b->a0) return b->lo_a0;
  return nullptr;
}

// block_advance on hi + lo vectors: the same buffer rotation, with each lo
// part following its hi part.
int block_advance_hilo(kpm_block* b) {
  const void* prev;
  int mode;
  void* out = next_out(b, &prev, &mode);
  HiloArgs q{};
  q.xlo = block_lo(b, b->p_cur);
  q.plo = block_lo(b, prev);
  q.olo = block_lo(b, out);
  if (!q.xlo || !q.olo || (mode == STEP_RECUR && !q.plo)) {
    set_error("compensated step: block has no lo part for its buffers");
    return KPM_ESTATE;
  }
  StepArgs a = step_args(b, b->p_cur, prev, out);
  KPM_TRY(launch_step_hilo(b->h, mode, a, q));
  rotate(b, out);
  return KPM_OK;
}

int block_advance_store(kpm_block* b, int smode, const float2* vell,
                        const StoreRow& row, int64_t R) {
  kpm_handle* h = b->h;
  if (h->precision != KPM_PREC_MIXED || h->H.ell_k == 0) {
    set_error("fused store needs a complex64 ELL handle");
    return KPM_EUNSUPPORTED;
  }
  const void* prev;
  int mode;
  void* out = next_out(b, &prev, &mode);
  StepArgs a = step_args(b, b->p_cur, prev, out);
  StoreArgs sa{smode, vell, row, R};
  KPM_TRY(launch_step_ell(h, mode, false, a, &sa));
  rotate(b, out);
  return KPM_OK;
}

int block_norm(kpm_block* b) {
  StepArgs a = step_args(b, b->p_cur, nullptr, nullptr);
  return launch_step(b->h, STEP_NORM, false, a);
}

int finalize(kpm_block* b, int mode, double2* mom, int64_t slot_even,
             int64_t slot_odd) {
  kpm_handle* h = b->h;
  dos_finalize_kernel<<<(unsigned)b->Rpad, 128, 0, h->stream>>>(
      h->partials, b->G, dos_xitems(h, b->N), b->Rpad,
      mode, (double2*)b->mu01, mom, b->Rpad, slot_even, slot_odd);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

int moments_to_host(kpm_handle* h, const double2* dev, int64_t count,
                    int64_t R, int64_t Rpad, int64_t W, double* host) {
  if (count == 0) return KPM_OK;
  double2* tmp = nullptr;
  size_t n = (size_t)R * count * W;
  KPM_TRY(dev_alloc((void**)&tmp, n * sizeof(double2), h->stream));
  moments_to_host_order_kernel<<<(unsigned)ceil_div(n, 256), 256, 0,
                                 h->stream>>>(dev, tmp, count, R, Rpad, W);
  count_launch(1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host, tmp, n * sizeof(double2),
                        cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dev_free(tmp, h->stream);
  KPM_CUDA(e);
  return KPM_OK;
}

int timed_begin(kpm_handle* h) {
  if (!h->ev_start) {
    KPM_CUDA(cudaEventCreate(&h->ev_start));
    KPM_CUDA(cudaEventCreate(&h->ev_stop));
  }
  KPM_CUDA(cudaEventRecord(h->ev_start, h->stream));
  return KPM_OK;
}

int timed_end(kpm_handle* h) {
  KPM_CUDA(cudaEventRecord(h->ev_stop, h->stream));
  h->timed = true;
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

// ======================================================================
//                                C ABI
// ======================================================================
namespace kpm {
// Random-phase vectors exp(2 pi i u) in the device layout [N][Rpad] (device
// row order), padding vectors zero; u from SplitMix64 of (key, vector) then
// row: the top 24 bits (complex64) or 53 bits (complex128).
template <typename T>
__global__ void random_phase_kernel(T* __restrict__ a0, int64_t N, int64_t R,
                                    int64_t Rpad, uint64_t key) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * Rpad) return;
  const int64_t n = idx / Rpad, r = idx % Rpad;
  const uint64_t hsh = mix64(mix64(key ^ (uint64_t)r) + (uint64_t)n);
  T v;
  if constexpr (sizeof(T) == 8) {
    float s = 0.f, c = 0.f;
    if (r < R) sincospif(2.0f * ((float)(hsh >> 40) * 0x1.0p-24f), &s, &c);
    v.x = c;
    v.y = s;
  } else {
    double s = 0.0, c = 0.0;
    if (r < R) sincospi(2.0 * ((double)(hsh >> 11) * 0x1.0p-53), &s, &c);
    v.x = c;
    v.y = s;
  }
  a0[idx] = v;
}
}  // namespace kpm

extern "C" {

int kpm_version(void) { return 10000; }

int kpm_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return KPM_EINVAL;
  strncpy(buf, g_err, len - 1);
  buf[len - 1] = '\0';
  return KPM_OK;
}

int kpm_device_count(int* count) {
  if (!count) return KPM_EINVAL;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return KPM_OK;
}

int kpm_debug_set(int key, int64_t value) {
  switch (key) {
    case KPM_DEBUG_WAIT_NS:
      KPM_REQUIRE(value > 0, "kpm_debug_set: wait limit must be positive");
      g_wait_ns = (uint64_t)value;
      return KPM_OK;
    case KPM_DEBUG_STALL_TMA:
      g_stall_tma = value != 0;
      return KPM_OK;
  }
  set_error("kpm_debug_set: unknown key %d", key);
  return KPM_EINVAL;
}

int kpm_build_checks(int* enabled) {
  KPM_REQUIRE(enabled, "kpm_build_checks: null argument");
#ifdef KPM_CHECK
  *enabled = 1;
#else
  *enabled = 0;
#endif
  return KPM_OK;
}

int kpm_launch_count(int64_t* count) {
  if (!count) return KPM_EINVAL;
  *count = g_launches.load();
  return KPM_OK;
}

int kpm_create(const kpm_csr_desc* ham, double a, double b, int precision,
               kpm_handle** out) {
  return kpm_create_ex(ham, a, b, precision, 0, out);
}

int kpm_create_ex(const kpm_csr_desc* ham, double a, double b, int precision,
                  int flags, kpm_handle** out) {
  KPM_REQUIRE(ham && out, "kpm_create: null argument");
  KPM_REQUIRE(ham->rows > 0 && ham->nnz >= 0 && ham->indptr && ham->indices &&
                  (ham->nnz == 0 || ham->data),
              "kpm_create: invalid CSR descriptor");
  // (the step kernels walk rows in 32-bit counters that run up to 2^17
  // past the last row)
  KPM_REQUIRE(ham->rows < INT32_MAX - (1 << 17) && ham->nnz < INT32_MAX,
              "kpm_create: CSR exceeds int32 indexing (rows=%lld nnz=%lld)",
              (long long)ham->rows, (long long)ham->nnz);
  KPM_REQUIRE(precision == KPM_PREC_FP64 || precision == KPM_PREC_MIXED,
              "kpm_create: unknown precision %d", precision);
  KPM_REQUIRE(a > 0 && std::isfinite(a) && std::isfinite(b),
              "kpm_create: scale a must be positive and finite");
  *out = nullptr;
  auto* h = new kpm_handle();
  h->precision = precision;
  h->a = a;
  h->b = b;
  int st = init_device(&h->device, &h->num_sms);
  if (st != KPM_OK) {
    delete h;
    return st;
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) !=
      cudaSuccess) {
    delete h;
    set_error("kpm_create: stream creation failed");
    return KPM_ECUDA;
  }
  h->own_stream = true;
  h->compensated =
      precision == KPM_PREC_MIXED && !(flags & KPM_FLAG_PLAIN_C64);
#ifdef KPM_CHECK
  st = dev_alloc((void**)&h->check, sizeof(unsigned long long), h->stream);
  if (st == KPM_OK &&
      cudaMemsetAsync(h->check, 0, sizeof(unsigned long long), h->stream) !=
          cudaSuccess)
    st = KPM_ECUDA;
  if (st != KPM_OK) {
    kpm_destroy(h);
    return st;
  }
#endif
  if (const char* kc = getenv("KPM_TC_KC")) h->tc_kc = atoi(kc) == 32 ? 32 : 16;
  const double scale = h->precision == KPM_PREC_MIXED ? 2.0 / a : 0.0;
  if (flags & KPM_FLAG_REORDER) {
    st = validate_csr(ham);
    std::vector<int32_t> perm;
    if (st == KPM_OK) st = setup_reorder(h, ham, perm);
    if (st == KPM_OK)
      st = upload_matrix_perm(h, ham, scale, &h->H, true, perm.data(),
                              h->h_iperm.data(), false);
  } else {
    st = upload_matrix(h, ham, scale, &h->H);
  }
  if (st != KPM_OK) {
    kpm_destroy(h);
    return st;
  }
  *out = h;
  return KPM_OK;
}

int kpm_set_stream(kpm_handle* h, void* stream) {
  KPM_REQUIRE(h, "kpm_set_stream: null handle");
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->stream = (cudaStream_t)stream;
  h->own_stream = false;
  return KPM_OK;
}

int kpm_get_stream(kpm_handle* h, void** stream) {
  KPM_REQUIRE(h && stream, "kpm_get_stream: null argument");
  *stream = (void*)h->stream;
  return KPM_OK;
}

int kpm_synchronize(kpm_handle* h) {
  KPM_REQUIRE(h, "kpm_synchronize: null handle");
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  return KPM_OK;
}

int kpm_destroy(kpm_handle* h) {
  if (!h) return KPM_OK;
  free_matrix(&h->H, h->stream);
  free_family(h);
  dev_free(h->vec_staging, h->stream);
  dev_free(h->partials, h->stream);
  dev_free(h->perm, h->stream);
  dev_free(h->check, h->stream);
  dev_free(h->dg_idx, h->stream);
  dev_free(h->dg_val, h->stream);
  dev_free(h->dg_flag, h->stream);
  if (h->ev_start) cudaEventDestroy(h->ev_start);
  if (h->ev_stop) cudaEventDestroy(h->ev_stop);
  for (cudaEvent_t e : h->prof_events) cudaEventDestroy(e);
  if (h->ev_gemm0) cudaEventDestroy(h->ev_gemm0);
  if (h->ev_gemm1) cudaEventDestroy(h->ev_gemm1);
  cudaStreamSynchronize(h->stream);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  cudaGetLastError();
  delete h;
  return KPM_OK;
}

int kpm_profile(kpm_handle* h, int enable) {
  KPM_REQUIRE(h, "kpm_profile: null handle");
  h->profiling = enable != 0;
  h->prof_used = 0;
  return KPM_OK;
}

int kpm_profile_read(kpm_handle* h, int64_t* launches, double* total_ms) {
  KPM_REQUIRE(h && launches && total_ms, "kpm_profile_read: null argument");
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  double tot = 0.0;
  for (size_t i = 0; i + 1 < h->prof_used; i += 2) {
    float f = 0.f;
    KPM_CUDA(cudaEventElapsedTime(&f, h->prof_events[i],
                                  h->prof_events[i + 1]));
    tot += f;
  }
  *launches = (int64_t)(h->prof_used / 2);
  *total_ms = tot;
  h->prof_used = 0;
  return KPM_OK;
}

int kpm_last_gemm(kpm_handle* h, double* ms, double* flops) {
  KPM_REQUIRE(h && ms && flops, "kpm_last_gemm: null argument");
  *ms = h->last_gemm_ms;
  *flops = h->last_gemm_flops;
  return KPM_OK;
}

int kpm_last_kernel_ms(kpm_handle* h, double* ms) {
  KPM_REQUIRE(h && ms, "kpm_last_kernel_ms: null argument");
  KPM_REQUIRE(h->timed, "kpm_last_kernel_ms: nothing timed yet");
  float f = 0.f;
  KPM_CUDA(cudaEventSynchronize(h->ev_stop));
  KPM_CUDA(cudaEventElapsedTime(&f, h->ev_start, h->ev_stop));
  *ms = f;
  return KPM_OK;
}

int kpm_block_create(kpm_handle* h, const double* vecs, int64_t R,
                     int keep_a0, kpm_block** out) {
  KPM_REQUIRE(h && out, "kpm_block_create: null argument");
  KPM_REQUIRE(R > 0, "kpm_block_create: num_vectors must be positive");
  *out = nullptr;
  auto* b = new kpm_block();
  b->h = h;
  b->R = R;
  b->N = h->H.rows;
  const int G = group_size(h->precision, R);
  b->G = G;
  b->Rpad = round_up(R, G);
  b->groups = (int)(b->Rpad / G);
  b->keep_a0 = keep_a0 != 0;
  const size_t csz = h->precision == KPM_PREC_MIXED ? 8 : 16;
  const size_t vbytes = (size_t)b->N * b->Rpad * csz;
  int st = KPM_OK;
  if (st == KPM_OK) st = dev_alloc(&b->buf[0], vbytes, h->stream);
  if (st == KPM_OK) st = dev_alloc(&b->buf[1], vbytes, h->stream);
  if (st == KPM_OK && b->keep_a0) st = dev_alloc(&b->a0, vbytes, h->stream);
  if (st == KPM_OK && !b->keep_a0) b->a0 = b->buf[1];
  if (st == KPM_OK)
    st = dev_alloc((void**)&b->mu01, (size_t)b->Rpad * 2 * sizeof(double2),
                   h->stream);
  if (st == KPM_OK && h->compensated && h->H.ell_k > 0) {
    const size_t lbytes = (size_t)b->N * b->Rpad * sizeof(uint32_t);
    st = dev_alloc((void**)&b->lo_buf[0], lbytes, h->stream);
    if (st == KPM_OK) st = dev_alloc((void**)&b->lo_buf[1], lbytes, h->stream);
    if (st == KPM_OK && b->keep_a0)
      st = dev_alloc((void**)&b->lo_a0, lbytes, h->stream);
    if (st == KPM_OK && !b->keep_a0) b->lo_a0 = b->lo_buf[1];
  }
  if (st == KPM_OK && vecs) {
    st = upload_vectors_lo(h, vecs, R, b->N, b->Rpad, b->a0, b->lo_a0);
  } else if (st == KPM_OK) {
    // no host vectors: zero, until kpm_block_randomize sets them
    cudaError_t e = cudaMemsetAsync(b->a0, 0, vbytes, h->stream);
    if (e == cudaSuccess && b->lo_a0)
      e = cudaMemsetAsync(b->lo_a0, 0,
                          (size_t)b->N * b->Rpad * sizeof(uint32_t),
                          h->stream);
    if (e != cudaSuccess) {
      set_error("kpm_block_create: %s", cudaGetErrorString(e));
      st = KPM_ECUDA;
    }
  }
  if (st == KPM_OK) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      set_error("kpm_block_create: %s", cudaGetErrorString(e));
      st = KPM_ECUDA;
    }
  }
  if (st != KPM_OK) {
    kpm_block_destroy(b);
    return st;
  }
  b->p_cur = b->a0;
  b->p_prev = nullptr;
  *out = b;
  return KPM_OK;
}

int kpm_block_randomize(kpm_block* b, uint64_t seed) {
  KPM_REQUIRE(b, "kpm_block_randomize: null block");
  if (!b->keep_a0) {
    set_error("kpm_block_randomize: block was created without keep_a0");
    return KPM_ESTATE;
  }
  kpm_handle* h = b->h;
  const int64_t total = b->N * b->Rpad;
  const unsigned grid = (unsigned)ceil_div(total, 256);
  const uint64_t key = mix64(seed ^ 0x5EEDB10Cull);
  if (h->precision == KPM_PREC_MIXED)
    random_phase_kernel<float2><<<grid, 256, 0, h->stream>>>(
        static_cast<float2*>(b->a0), b->N, b->R, b->Rpad, key);
  else
    random_phase_kernel<double2><<<grid, 256, 0, h->stream>>>(
        static_cast<double2*>(b->a0), b->N, b->R, b->Rpad, key);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  if (b->lo_a0)  // the generated complex64 vectors are exact: lo = 0
    KPM_CUDA(cudaMemsetAsync(b->lo_a0, 0, (size_t)total * sizeof(uint32_t),
                             h->stream));
  return kpm_block_rewind(b);
}

int kpm_block_rewind(kpm_block* b) {
  KPM_REQUIRE(b, "kpm_block_rewind: null block");
  if (!b->keep_a0) {
    set_error("kpm_block_rewind: block was created without keep_a0");
    return KPM_ESTATE;
  }
  b->p_cur = b->a0;
  b->p_prev = nullptr;
  b->steps_done = 0;
  b->mode = -1;
  return KPM_OK;
}

int kpm_block_destroy(kpm_block* b) {
  if (!b) return KPM_OK;
  cudaStream_t s = b->h->stream;
  dev_free(b->buf[0], s);
  dev_free(b->buf[1], s);
  if (b->keep_a0) dev_free(b->a0, s);
  dev_free(b->lo_buf[0], s);
  dev_free(b->lo_buf[1], s);
  if (b->keep_a0) dev_free(b->lo_a0, s);
  dev_free(b->mu01, s);
  dev_free(b->op_coef, s);
  cudaStreamSynchronize(s);
  cudaGetLastError();
  delete b;
  return KPM_OK;
}

int kpm_block_checkpoint(kpm_block* b, int64_t* steps_done, int* mode,
                         double* mu01) {
  KPM_REQUIRE(b && steps_done && mode, "kpm_block_checkpoint: null argument");
  *steps_done = b->steps_done;
  *mode = b->mode;
  if (mu01) {
    KPM_CUDA(cudaMemcpyAsync(mu01, b->mu01, (size_t)b->R * 2 * sizeof(double2),
                             cudaMemcpyDeviceToHost, b->h->stream));
    KPM_CUDA(cudaStreamSynchronize(b->h->stream));
  }
  return KPM_OK;
}

int kpm_block_restore(kpm_block* b, int64_t steps_done, int mode,
                      const double* alpha_prev, const double* alpha_cur,
                      const double* mu01) {
  KPM_REQUIRE(b, "kpm_block_restore: null block");
  KPM_REQUIRE(steps_done >= 0 && mode >= -1 && mode <= 1,
              "kpm_block_restore: invalid state (steps %lld, mode %d)",
              (long long)steps_done, mode);
  kpm_handle* h = b->h;
  if (steps_done == 0) {
    if (!b->keep_a0 && b->steps_done != 0) {
      set_error("kpm_block_restore: block was created without keep_a0");
      return KPM_ESTATE;
    }
    b->p_cur = b->a0;
    b->p_prev = nullptr;
  } else {
    KPM_REQUIRE(alpha_prev && alpha_cur,
                "kpm_block_restore: both Chebyshev vectors are needed");
    // alpha_n in buf[0], alpha_{n-1} in buf[1]; the next step writes
    // alpha_{n+1} over alpha_{n-1} (when the block does not keep a0, a0
    // is buf[1] and is not needed again)
    KPM_TRY(upload_vectors_lo(h, alpha_cur, b->R, b->N, b->Rpad, b->buf[0],
                              b->lo_buf[0]));
    KPM_TRY(upload_vectors_lo(h, alpha_prev, b->R, b->N, b->Rpad, b->buf[1],
                              b->lo_buf[1]));
    b->p_cur = b->buf[0];
    b->p_prev = b->buf[1];
  }
  if (mu01) {
    KPM_CUDA(cudaMemsetAsync(b->mu01, 0, (size_t)b->Rpad * 2 * sizeof(double2),
                             h->stream));
    KPM_CUDA(cudaMemcpyAsync(b->mu01, mu01, (size_t)b->R * 2 * sizeof(double2),
                             cudaMemcpyHostToDevice, h->stream));
  }
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  b->steps_done = steps_done;
  b->mode = mode;
  return KPM_OK;
}

int kpm_block_state(kpm_block* b, double* alpha_prev, double* alpha_cur) {
  KPM_REQUIRE(b && alpha_cur, "kpm_block_state: null argument");
  // lo parts are kept by the DOS recursion (and exist for a0 from the start)
  const bool lo = b->lo_a0 && (b->mode == 0 || b->steps_done == 0);
  if (alpha_prev) {
    if (!b->p_prev) {
      set_error("kpm_block_state: no previous vector before the first step");
      return KPM_ESTATE;
    }
    KPM_TRY(download_vectors_lo(b->h, b->p_prev,
                                lo ? block_lo(b, b->p_prev) : nullptr, b->R,
                                b->N, b->Rpad, alpha_prev));
  }
  return download_vectors_lo(b->h, b->p_cur,
                             lo ? block_lo(b, b->p_cur) : nullptr, b->R, b->N,
                             b->Rpad, alpha_cur);
}

// Failure detection for spectral bounds that do not enclose the spectrum:
// with the rescaled spectrum inside [-1, 1], |T_n| <= 1 there and every DOS
// moment of a vector obeys |mu_n| <= mu_0; eigenvalues left outside make
// T_n grow exponentially.  The reference has no such check (its only guard
// is the eigsh bound itself, kwant/kpm.py:1177-1180).  The moments are
// written either way; KPM_EDIVERGED reports the first offending moment.
static int check_divergence(kpm_block* b, int64_t m_start, int64_t count,
                            const double* out) {
  std::vector<double> mu01;
  if (m_start > 0) {
    mu01.resize((size_t)b->R * 4);
    KPM_CUDA(cudaMemcpyAsync(mu01.data(), b->mu01,
                             (size_t)b->R * 2 * sizeof(double2),
                             cudaMemcpyDeviceToHost, b->h->stream));
    KPM_CUDA(cudaStreamSynchronize(b->h->stream));
  }
  for (int64_t r = 0; r < b->R; ++r) {
    const double* v = out + 2 * r * count;
    const double mu0 = m_start == 0 ? v[0] : mu01[4 * r];
    const double lim = 1.001 * fabs(mu0) + 1e-300;
    for (int64_t m = 0; m < count; ++m) {
      const double mag = hypot(v[2 * m], v[2 * m + 1]);
      if (!(mag <= lim)) {
        set_error("moment %lld of vector %lld: |mu| = %g exceeds mu_0 = %g: "
                  "the spectral bounds do not enclose the spectrum and the "
                  "recursion diverged", (long long)(m_start + m),
                  (long long)r, mag, mu0);
        return KPM_EDIVERGED;
      }
    }
  }
  return KPM_OK;
}

int kpm_block_dos_moments(kpm_block* b, int64_t m_start, int64_t m_end,
                          double* out) {
  NvtxRange nvtx("kpm_block_dos_moments");
  KPM_REQUIRE(b && out, "kpm_block_dos_moments: null argument");
  KPM_REQUIRE(m_end >= 2 && m_start >= 0 && m_start < m_end,
              "kpm_block_dos_moments: need 0 <= m_start < m_end, m_end >= 2 "
              "(got %lld, %lld)", (long long)m_start, (long long)m_end);
  kpm_handle* h = b->h;
  if (m_start == 0) {
    if (b->steps_done != 0) {
      set_error("kpm_block_dos_moments: block already advanced; rewind it");
      return KPM_ESTATE;
    }
  } else if (b->mode != 0 || m_start / 2 != b->steps_done) {
    set_error("kpm_block_dos_moments: cannot resume at moment %lld "
              "(state after %lld matvecs, mode %d)", (long long)m_start,
              (long long)b->steps_done, b->mode);
    return KPM_ESTATE;
  }
  b->mode = 0;
  const int64_t count = m_end - m_start;
  const int G = group_size(h->precision);
  KPM_TRY(ensure_partials(h, b->groups, dos_xitems(h, b->N)));
  double2* mom = nullptr;
  KPM_TRY(dev_alloc((void**)&mom, (size_t)count * b->Rpad * sizeof(double2),
                    h->stream));
  (void)G;
  int st = timed_begin(h);
  auto slot = [&](int64_t m) -> int64_t {
    return (m >= m_start && m < m_end) ? m - m_start : -1;
  };
  // compensated blocks: hi + lo vectors and error-free steps
  const bool hilo = b->lo_a0 != nullptr;
  if (st == KPM_OK && hilo) st = prepare_hilo(h);
  if (st == KPM_OK && m_start == 0) {
    st = hilo ? block_advance_hilo(b) : block_advance(b, true);
    if (st == KPM_OK) st = finalize(b, STEP_FIRST, mom, slot(0), slot(1));
  }
  int64_t n0 = m_start / 2 > 1 ? m_start / 2 : 1;
  for (int64_t n = n0; st == KPM_OK && n < m_end / 2; ++n) {
    st = hilo ? block_advance_hilo(b) : block_advance(b, true);
    if (st == KPM_OK)
      st = finalize(b, STEP_RECUR, mom, slot(2 * n), slot(2 * n + 1));
  }
  if (st == KPM_OK && (m_end % 2)) {
    st = block_norm(b);
    if (st == KPM_OK)
      st = finalize(b, STEP_NORM, mom, slot(m_end - 1), -1);
  }
  if (st == KPM_OK) st = timed_end(h);
  if (st == KPM_OK) st = moments_to_host(h, mom, count, b->R, b->Rpad, 1, out);
  dev_free(mom, h->stream);
  if (st == KPM_OK) st = check_bounds(h, "kpm_block_dos_moments");
  if (st == KPM_OK) st = check_divergence(b, m_start, count, out);
  return st;
}

}  // extern "C"
