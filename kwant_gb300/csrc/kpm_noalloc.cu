// DOS moments without any device allocation (kpm_dos_moments_noalloc).
//
// Some callers cannot let a library allocate device memory: an application
// or framework that owns every byte of device memory through its own arena
// and hands its libraries preallocated buffers (a custom-call interface of a
// tensor framework, a service with a fixed, audited device-memory budget).
// For them this entry point runs the DOS recursion of kpm_block_dos_moments
// with caller-provided inputs, work buffers and outputs.  The only other
// memory it touches is the scratch below: a file-scope device array of
// KPM_NOALLOC_SCRATCH_BYTES that every device which loads the library holds
// until the process exits.
//
// The scratch holds the per-row-partition dot-product partials and mu_0,
// mu_1 of each vector.  Each call writes every element it later reads, so
// nothing needs clearing; the array keeps the last call's contents.  All
// calls share it: calls whose GPU work overlaps in time (different streams,
// threads or processes sharing the device context) race on it.

#include <cuda.h>

#include <mutex>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

static __device__ __align__(256) double
    g_noalloc_scratch[KPM_NOALLOC_SCRATCH_BYTES / sizeof(double)];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mutex;
static double* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {nullptr};
static unsigned long long g_noalloc_ctx[NOALLOC_MAX_DEVICES] = {0};
static int g_noalloc_sms[NOALLOC_MAX_DEVICES] = {0};

// Id of the current device context (unique over the process lifetime), 0
// when none is current yet.  The driver calls come through the runtime's
// entry-point lookup, so the library needs no link to the driver library.
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent",
                                         (void**)&get_current, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_current = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&get_id, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_id = nullptr;
    cudaGetLastError();
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
      get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch array in the current device context.  The
// name g_noalloc_scratch in host code is only a host-side stand-in, so the
// address is looked up (with the device current) on the first call in each
// context and cached with the context's id: after cudaDeviceReset, or in a
// context the caller made current, the module can sit at another address,
// and the next call looks it up again.
static int noalloc_scratch(double** scratch, int* sms) {
  int dev = -1;
  KPM_CUDA(cudaGetDevice(&dev));
  KPM_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES,
              "kpm_dos_moments_noalloc: device ordinal %d not supported", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned long long ctx = current_context_id();
  if (!g_noalloc_addr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      set_error("kpm_dos_moments_noalloc: cudaGetSymbolAddress failed: %s",
                cudaGetErrorString(e));
      return KPM_ECUDA;
    }
    int n = 0;
    KPM_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    g_noalloc_sms[dev] = n;
    g_noalloc_addr[dev] = static_cast<double*>(p);
    // the lookup made a context current if none was
    g_noalloc_ctx[dev] = ctx ? ctx : current_context_id();
  }
  *scratch = g_noalloc_addr[dev];
  *sms = g_noalloc_sms[dev];
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_dos_moments_noalloc(const kpm_device_csr* ham, double a, double b,
                            int precision, const void* vecs, int64_t R,
                            int64_t M, void* work, double* moments,
                            void* stream) {
  KPM_REQUIRE(ham && vecs && work && moments,
              "kpm_dos_moments_noalloc: null argument");
  KPM_REQUIRE(ham->rows > 0 && ham->rows < INT32_MAX && ham->nnz >= 0 &&
                  ham->nnz < INT32_MAX && ham->indptr && ham->indices &&
                  (ham->nnz == 0 || ham->data),
              "kpm_dos_moments_noalloc: invalid device CSR descriptor");
  KPM_REQUIRE(precision == KPM_PREC_FP64 || precision == KPM_PREC_MIXED,
              "kpm_dos_moments_noalloc: unknown precision %d", precision);
  KPM_REQUIRE(a > 0 && std::isfinite(a) && std::isfinite(b),
              "kpm_dos_moments_noalloc: scale a must be positive and finite");
  KPM_REQUIRE(R > 0 && M >= 2,
              "kpm_dos_moments_noalloc: need num_vectors > 0 and "
              "num_moments >= 2");

  double* scratch = nullptr;
  int sms = 0;
  KPM_TRY(noalloc_scratch(&scratch, &sms));

  const int G = group_size(precision);
  const int64_t N = ham->rows;
  const int64_t Rpad = round_up(R, G);
  const int groups = (int)(Rpad / G);
  const int xitems = xitems_for_rows(N, sms);   // plain steps: 4 per SM
  const size_t partials = (size_t)groups * xitems * G * 3;  // doubles
  const size_t need = partials + (size_t)Rpad * 4;          // + mu0, mu1
  const size_t cap = KPM_NOALLOC_SCRATCH_BYTES / sizeof(double);
  KPM_REQUIRE(need <= cap,
              "kpm_dos_moments_noalloc: %lld vectors over %lld rows need "
              "%zu bytes of scratch, more than the %zu bytes this entry point "
              "holds; use fewer vectors per call", (long long)R,
              (long long)N, need * sizeof(double),
              (size_t)KPM_NOALLOC_SCRATCH_BYTES);

  // Stack descriptors over the caller's buffers: nothing is allocated.
  kpm_handle h;
  h.precision = precision;
  h.num_sms = sms;
  h.a = a;
  h.b = b;
  h.stream = static_cast<cudaStream_t>(stream);
  h.own_stream = false;
  h.H.rows = N;
  h.H.nnz = ham->nnz;
  h.H.indptr = const_cast<int32_t*>(ham->indptr);
  h.H.indices = const_cast<int32_t*>(ham->indices);
  h.H.data = const_cast<void*>(ham->data);
  h.partials = scratch;
  h.partials_cap = partials;

  const size_t csz = precision == KPM_PREC_MIXED ? 8 : 16;
  kpm_block blk;
  blk.h = &h;
  blk.R = R;
  blk.Rpad = Rpad;
  blk.G = G;
  blk.groups = groups;
  blk.N = N;
  blk.keep_a0 = true;  // the caller's vectors are only read
  blk.a0 = const_cast<void*>(vecs);
  blk.buf[0] = work;
  blk.buf[1] = static_cast<char*>(work) + (size_t)N * Rpad * csz;
  blk.p_cur = blk.a0;
  blk.p_prev = nullptr;
  blk.mu01 = scratch + partials;
  blk.mode = 0;

  double2* mom = reinterpret_cast<double2*>(moments);
  int st = block_advance(&blk, true);
  if (st == KPM_OK) st = finalize(&blk, STEP_FIRST, mom, 0, 1);
  for (int64_t n = 1; st == KPM_OK && n < M / 2; ++n) {
    st = block_advance(&blk, true);
    if (st == KPM_OK) st = finalize(&blk, STEP_RECUR, mom, 2 * n, 2 * n + 1);
  }
  if (st == KPM_OK && (M % 2)) {
    st = block_norm(&blk);
    if (st == KPM_OK) st = finalize(&blk, STEP_NORM, mom, M - 1, -1);
  }
  // the stack descriptors own nothing: make sure nothing is released
  h.H.indptr = nullptr;
  h.H.indices = nullptr;
  h.H.data = nullptr;
  h.partials = nullptr;
  return st;
}

}  // extern "C"
