// Internal interfaces shared by the KPM translation units.
#pragma once

#include "kpm_common.cuh"
#include "kpm_gemm.cuh"

namespace kpm {

enum { STEP_FIRST = 0, STEP_RECUR = 1, STEP_NORM = 2 };

struct StepArgs {
  int64_t rows;
  const int32_t* indptr;
  const int32_t* indices;
  const void* vals;
  double b, inv_a;  // complex128: (H v - b v) * inv_a
  float shift;      // complex64: values are 2H/a, diagonal shift -2b/a
  const void* x;    // alpha_n        [rows][Rpad]
  const void* prev; // alpha_{n-1}    (may alias out)
  void* out;        // alpha_{n+1}
  int64_t rp;       // payloads per row (16 bytes, or 8 when vpl == 1)
  int vpl;          // complex64 vectors per lane: 2 (groups of 32) or 1
  int groups;
  int xitems;
  double* partials; // [group][vector*3 + component][xitems]
  unsigned long long* check;  // KPM_CHECK builds: first bad index + 1
};

// Column index of a gathered row.  Bounds-checked builds (-DKPM_CHECK)
// validate it: an index outside [0, rows) is recorded in p.check and row 0
// is read instead; other builds use it as is.
__device__ __forceinline__ int col_index(const StepArgs& p, int c) {
#ifdef KPM_CHECK
  if ((uint32_t)c >= (uint32_t)p.rows) {
    if (p.check)
      atomicCAS(p.check, 0ull, 1ull + (unsigned long long)(uint32_t)c);
    return 0;
  }
#endif
  return c;
}

// KPM_CHECK builds: KPM_EINVAL if a step kernel of h met a bad index
// (then cleared); KPM_OK otherwise and in other builds
int check_bounds(kpm_handle* h, const char* where);

// Fused store of alpha_n's row (the correlator's recursions, ELL step,
// BF16x3 store): smode 0 none, 1 alpha_n itself, 2 V alpha_n with V's values
// in an ELL copy aligned entry for entry with H's (vell).  A separate
// kernel argument: inside StepArgs it made the plain step kernel spill.
struct StoreArgs {
  int smode;
  const float2* vell;
  StoreRow store;
  int64_t R;
};

// bfloat16 lo parts of a compensated (hi + lo) mixed-precision block:
// [rows][Rpad] words, bf16 re in the low half, im in the high half
struct HiloArgs {
  const uint32_t* xlo;  // lo of alpha_n
  const uint32_t* plo;  // lo of alpha_{n-1} (may alias olo)
  uint32_t* olo;        // lo of alpha_{n+1}
  int64_t lrp;          // lane payloads per row (set by the launcher)
};

void count_launch(int n);
// Row partitions of the steps that write moment dot partials (the DOS dots
// and norms, and their finalize): fixed for a handle and its row count, so
// the reduction order never depends on R or on the launch shape.  The
// compensated step runs two 256-thread blocks per SM, and 2 partitions per
// SM give each block half as many pipeline starts and block reductions as 4
// (graphene, 2e6 orbitals, R = 64: 1.000 -> 0.985 ms per step); the other
// steps keep 4.  One partition per SM is faster still when the blocks hold
// two or more 16-vector sub-groups (0.971 -> 0.921 ms at R = 64, 0.479 ->
// 0.457 at R = 32) but leaves half of the resident blocks idle at R <= 16
// (0.232 -> 0.336 ms at R = 16); since the count must not depend on R, it
// stays at 2.
int dos_xitems(const kpm_handle* h, int64_t rows);
// event pair around the next launch when profiling (*e1: closing event)
int prof_begin(kpm_handle* h, cudaEvent_t* e1);
int dev_alloc(void** p, size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);
int init_device(int* device, int* num_sms);

int validate_csr(const kpm_csr_desc* m);
// CSR upload.  scale == 0 keeps complex128 values; otherwise values are
// stored as complex64 multiplied by scale.
int upload_matrix(kpm_handle* h, const kpm_csr_desc* m, double scale,
                  Matrix* out, bool with_ell = true);
// upload_matrix in a row order: new row p = old row perm[p] (host arrays
// perm / iperm, or both null for the caller's order); the rows are moved
// on the device.  validate false: m was validated by the caller.
int upload_matrix_perm(kpm_handle* h, const kpm_csr_desc* m, double scale,
                       Matrix* out, bool with_ell, const int32_t* perm,
                       const int32_t* iperm, bool validate);
void free_matrix(Matrix* m, cudaStream_t s);
// upload_matrix in the handle's row order (reordered handles permute rows
// and columns)
int upload_matrix_for(kpm_handle* h, const kpm_csr_desc* m, double scale,
                      Matrix* out, bool with_ell = true);
// compute the RCM order of m (perm[new] = old), set h->perm / h->h_iperm
int setup_reorder(kpm_handle* h, const kpm_csr_desc* m,
                  std::vector<int32_t>& perm);

void free_family(kpm_handle* h);

int upload_vectors(kpm_handle* h, const double* host, int64_t R, int64_t N,
                   int64_t Rpad, void* dst);
int download_vectors(kpm_handle* h, const void* src, int64_t R, int64_t N,
                     int64_t Rpad, double* host);
// the same for compensated blocks: lo (bfloat16 x 2 words, [N][Rpad]) is
// written on upload (exact split of the complex128 input into hi + lo) and
// added on download (exact); lo null: complex64 only
int upload_vectors_lo(kpm_handle* h, const double* host, int64_t R,
                      int64_t N, int64_t Rpad, void* dst, uint32_t* lo);
int download_vectors_lo(kpm_handle* h, const void* src, const uint32_t* lo,
                        int64_t R, int64_t N, int64_t Rpad, double* host);
// lo part belonging to one of the block's hi buffers (null if none)
uint32_t* block_lo(const kpm_block* b, const void* hi);
// block_advance of a compensated block (DOS dots always fused)
int block_advance_hilo(kpm_block* b);

int launch_step(kpm_handle* h, int mode, bool dots, const StepArgs& a);
// widest ELL row (entries) the complex64 ELL step kernel is built for
constexpr int ELL_MAX = 16;
// ELL copy of out's device CSR (complex64 values already in out)
int build_ell(kpm_handle* h, const kpm_csr_desc* m, Matrix* out);
int launch_step_ell(kpm_handle* h, int mode, bool dots, const StepArgs& a,
                    const StoreArgs* sa = nullptr);
// compensated DOS step on a hi + lo block (complex64 ELL handle), dots fused
int launch_step_hilo(kpm_handle* h, int mode, const StepArgs& a,
                     const HiloArgs& q);
// (re)build the handle's diagonal-first ELL copy for the compensated step
// from its current complex64 ELL values
int prepare_hilo(kpm_handle* h);
StepArgs step_args(kpm_block* b, const void* x, const void* prev, void* out);
int block_advance(kpm_block* b, bool dots);
// block_advance without dot products that also writes the store row of the
// current vector (StepArgs::smode); KPM_EUNSUPPORTED when the handle has no
// complex64 ELL copy (the caller then stores with a separate kernel)
int block_advance_store(kpm_block* b, int smode, const float2* vell,
                        const StoreRow& row, int64_t R);
int block_norm(kpm_block* b);
// sum the dot-product partials and write DOS moments (slots < 0 skipped)
int finalize(kpm_block* b, int mode, double2* mom, int64_t slot_even,
             int64_t slot_odd);
int ensure_partials(kpm_handle* h, int groups, int xitems);
int moments_to_host(kpm_handle* h, const double2* dev, int64_t count,
                    int64_t R, int64_t Rpad, int64_t W, double* host);
int timed_begin(kpm_handle* h);
int timed_end(kpm_handle* h);

// Device reconstruction of kpm_reconstruct from device moments laid out as
// [R][M][W] complex128.
int reconstruct_on_device(cudaStream_t s, int64_t R, int64_t M, int64_t W,
                          const double2* moments, int mean, int is_real,
                          double a, int kernel, double lorentz_l,
                          const double* nodes,
                          double* gammas_out, double* densities_out);

}  // namespace kpm
