/*
 * kwant_gb300 — C ABI of the GB300 (sm_103a) kernel-polynomial-method path.
 *
 * This is the drop-in boundary for the KPM hot path of Kwant
 * (kwant/kpm.py: SpectralDensity, Correlator, conductivity; with
 * kwant/operator.pyx Density/Current as local operators).  The Python
 * package kwant_gb300 binds it through ctypes; any other host language
 * binds the same symbols.
 *
 * Conventions
 *  - Every function returns an int status: KPM_OK (0) or a negative error
 *    code; kpm_last_error() returns the message of the last failure on the
 *    calling thread.
 *  - Complex numbers are interleaved (re, im) doubles, like numpy
 *    complex128.  Indices are int32 (Kwant's gint, kwant/graph/defs.h:15).
 *  - Host pointers are owned by the caller and only read/written during the
 *    call.  Device memory is owned by the handle / block / operator objects.
 *  - Calls are synchronous with respect to the host (results are in the
 *    output buffers on return).  Each handle issues its work on one CUDA
 *    stream.  A handle and the objects created from it must be used from one
 *    host thread at a time.
 *  - There is no CPU fallback: without a usable CUDA device every call that
 *    would compute returns KPM_ECUDA.
 */
#ifndef KWANT_GB300_H
#define KWANT_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define KPM_API __attribute__((visibility("default")))
#else
#define KPM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define KPM_OK 0
#define KPM_EINVAL (-1)      /* invalid argument (reference: ValueError)   */
#define KPM_ECUDA (-2)       /* CUDA runtime / device error                */
#define KPM_ENOMEM (-3)      /* device allocation failed                   */
#define KPM_EDIVERGED (-4)   /* moments left [-mu0, mu0]: bounds too tight */
#define KPM_ETIMEOUT (-5)    /* a bounded device wait gave up              */
#define KPM_ESTATE (-6)      /* call out of order (e.g. resume mismatch)   */
#define KPM_EUNSUPPORTED (-7)

/* ---- enums ------------------------------------------------------------- */
/* Recursion precision.  FP64: complex128 vectors and matrix, reference
 * operation order.  MIXED: complex64 vectors and matrix (pre-scaled by
 * 2/a), FP64 accumulation of every dot product. */
#define KPM_PREC_FP64 0
#define KPM_PREC_MIXED 1

#define KPM_KERNEL_NONE 0
#define KPM_KERNEL_JACKSON 1   /* kwant/kpm.py:1106-1123 */
#define KPM_KERNEL_LORENTZ 2   /* kwant/kpm.py:1126-1142 */

typedef struct kpm_handle kpm_handle; /* a rescaled Hamiltonian on device  */
typedef struct kpm_block kpm_block;   /* R vectors + recursion state       */
typedef struct kpm_op kpm_op;         /* a lowered sesquilinear operator   */

/* CSR matrix on the host: rows x rows, complex128 values (interleaved). */
typedef struct kpm_csr_desc {
  int64_t rows;
  int64_t nnz;
  const int32_t* indptr;   /* rows + 1 */
  const int32_t* indices;  /* nnz      */
  const double* data;      /* 2 * nnz  */
} kpm_csr_desc;

/* A sesquilinear operator q_w(bra, ket) lowered to "terms" (see
 * kwant_gb300/operator.py for the lowering of Density, Current and
 * matrix operators):
 *   coef_t  = sum_{e in bra_ptr[t]..bra_ptr[t+1]} conj(bra_val[e]) * bra[bra_col[e]]
 *   q_w     = sum_{t : term_out[t] == w} conj(coef_t) * ket[term_row[t]]
 * Terms are sorted by output; chunk_ptr splits them into chunks of
 * consecutive terms of one output (chunk_out[c]); outputs with several
 * chunks are summed in chunk order.  real0 = 1 takes the real part of the
 * n = 0 moment (reference kwant/operator.pyx:556-558, bra is ket). */
typedef struct kpm_op_desc {
  int64_t num_terms;
  int64_t num_outputs;
  int64_t num_chunks;
  const int32_t* term_row;   /* num_terms     */
  const int64_t* bra_ptr;    /* num_terms + 1 */
  const int32_t* bra_col;    /* bra_ptr[num_terms] */
  const double* bra_val;     /* 2 * bra_ptr[num_terms] */
  const int64_t* chunk_ptr;  /* num_chunks + 1 (term offsets) */
  const int32_t* chunk_out;  /* num_chunks */
  int32_t real0;
} kpm_op_desc;

/* ---- library ------------------------------------------------------------ */
KPM_API int kpm_version(void);
/* Copies the last error message of this thread (NUL-terminated). */
KPM_API int kpm_last_error(char* buf, size_t len);
/* Number of CUDA devices visible (0 when none). */
KPM_API int kpm_device_count(int* count);

/* Diagnostics (no reference counterpart).  KPM_DEBUG_WAIT_NS: limit, in ns
 * of GPU time, of every bounded mbarrier wait in the tensor-core kernels
 * (default 2e9).  KPM_DEBUG_STALL_TMA (tests only): when nonzero their TMA
 * producers issue no loads, so the MMA thread's wait runs out; the kernel
 * records the expiry, releases its tensor memory and returns, the call
 * reports KPM_ETIMEOUT, and the CUDA context stays usable.  Process-wide
 * settings, read at each launch. */
#define KPM_DEBUG_WAIT_NS 1
#define KPM_DEBUG_STALL_TMA 2
KPM_API int kpm_debug_set(int key, int64_t value);
/* 1 if this library was built with -DKPM_CHECK: its Chebyshev step kernels
 * validate every gathered column index, and the moment calls return
 * KPM_EINVAL naming the first index out of range (no reference
 * counterpart; the reference's Cython loops run with boundscheck off). */
KPM_API int kpm_build_checks(int* enabled);

/* ---- Hamiltonian handle ---------------------------------------------------
 * Replaces the rescaled LinearOperator of _rescale (kwant/kpm.py:1145-1187):
 * the device applies (H v - b v) / a.  a, b as computed by the caller from
 * the spectral bounds (kwant/kpm.py:1174-1175). */
KPM_API int kpm_create(const kpm_csr_desc* ham, double a, double b, int precision,
                       kpm_handle** out);
/* kpm_create with flags.  KPM_FLAG_REORDER: store the Hamiltonian in a
 * reverse Cuthill-McKee order of its sparsity pattern (computed on the
 * host), so that the neighbours of a row are close in memory and stay in L2
 * during a step.  Vectors, operators and results are permuted on the device
 * transparently; moments are invariant under the reordering.  No reference
 * counterpart (the reference multiplies in the given order). */
#define KPM_FLAG_REORDER 1
/* KPM_PREC_MIXED only: run the DOS recursion on plain complex64 vectors
 * instead of the default compensated form.  The default keeps a bfloat16
 * correction next to every complex64 element (12 instead of 8 bytes) and
 * computes each step and the moment dot products with error-free FP32
 * transformations, which keeps the per-orbital DOS within ~1e-6 of the
 * FP64 recursion at every Chebyshev node; the plain form moves a third
 * fewer bytes and is off by up to ~1e-4 at the outermost nodes, where the
 * reconstruction divides by sqrt(1 - x^2).  No reference counterpart (the
 * reference computes in complex128). */
#define KPM_FLAG_PLAIN_C64 2
KPM_API int kpm_create_ex(const kpm_csr_desc* ham, double a, double b,
                          int precision, int flags, kpm_handle** out);
/* Use an external CUDA stream (cudaStream_t) for all work of the handle. */
KPM_API int kpm_set_stream(kpm_handle* h, void* stream);
KPM_API int kpm_get_stream(kpm_handle* h, void** stream);
KPM_API int kpm_synchronize(kpm_handle* h);
KPM_API int kpm_destroy(kpm_handle* h);

/* ---- vector blocks ---------------------------------------------------------
 * R starting vectors |r> (host, R x N complex128, one vector after another:
 * the stacked output of the reference's vector factory, kwant/kpm.py:437).
 * vecs == NULL allocates the block with zero vectors, for a following
 * kpm_block_randomize (no host upload).
 * keep_a0 keeps |r> resident (needed for operators and for rewinding). */
KPM_API int kpm_block_create(kpm_handle* h, const double* vecs, int64_t R,
                             int keep_a0, kpm_block** out);
/* Restart the recursion from |r> (requires keep_a0). */
KPM_API int kpm_block_rewind(kpm_block* blk);
/* Replace the starting vectors with new random-phase vectors generated on
 * the device (exp(2 pi i u), u from SplitMix64 of (seed, vector, device
 * row); 24 random bits for MIXED, 53 for FP64) and rewind (requires
 * keep_a0).  A fresh, independent vector set per sweep point without a
 * host upload; not the reference's MT19937 stream (RandomVectors,
 * kwant/kpm.py:932-952, draws from numpy). */
KPM_API int kpm_block_randomize(kpm_block* blk, uint64_t seed);
KPM_API int kpm_block_destroy(kpm_block* blk);
/* Copy the current recursion state (alpha_{n-1}, alpha_n) to the host, each
 * R x N complex128 (the reference's _last_two_alphas, kwant/kpm.py:486-488). */
KPM_API int kpm_block_state(kpm_block* blk, double* alpha_prev, double* alpha_cur);
/* Checkpoint / restore of a block's recursion, for resuming long moment runs
 * in another process (the reference keeps _moments_list and
 * _last_two_alphas in memory only, kwant/kpm.py:486-490).  checkpoint
 * reports the number of matvecs applied, the mode (-1 none, 0 DOS,
 * 1 operator) and, if mu01 is not NULL, the per-vector mu_0, mu_1 of the DOS
 * doubling (R x 2 complex128).  restore sets that state on a block created
 * with the same starting vectors and handle: alpha_prev, alpha_cur as
 * returned by kpm_block_state (R x N complex128; not needed when
 * steps_done is 0). */
KPM_API int kpm_block_checkpoint(kpm_block* blk, int64_t* steps_done, int* mode,
                                 double* mu01);
KPM_API int kpm_block_restore(kpm_block* blk, int64_t steps_done, int mode,
                              const double* alpha_prev, const double* alpha_cur,
                              const double* mu01);

/* ---- moments -----------------------------------------------------------------
 * DOS moments (operator=None) of SpectralDensity._update_moments_list,
 * kwant/kpm.py:436-477: mu_0 = <a0|a0>, mu_1 = <a0|a1>,
 * mu_2n = 2<a_n|a_n> - mu_0, mu_2n+1 = 2<a_n+1|a_n> - mu_1 (odd tail:
 * 2<a_last|a_last> - mu_0).  Computes moments [m_start, m_end) of every
 * vector; m_start is 0 on the first call and the previous m_end when
 * resuming (add_moments, kwant/kpm.py:318-358).  out: R x (m_end - m_start)
 * complex128.  Returns KPM_EDIVERGED (with out written) when a moment
 * exceeds 1.001 mu_0 in magnitude or is not finite: the spectral bounds
 * do not enclose the spectrum (|T_n| <= 1 holds only inside it). */
KPM_API int kpm_block_dos_moments(kpm_block* blk, int64_t m_start, int64_t m_end,
                                  double* out);

/* Operator moments mu_n = op(a0, T_n(H~) a0), kwant/kpm.py:439-448 and
 * :478-484 (operator a lowered kwant.operator Density / Current / matrix).
 * out: R x (m_end - m_start) x num_outputs complex128. */
KPM_API int kpm_op_create(kpm_handle* h, const kpm_op_desc* desc, kpm_op** out);
KPM_API int kpm_op_destroy(kpm_op* op);
KPM_API int kpm_block_op_moments(kpm_block* blk, kpm_op* op, int64_t m_start,
                                 int64_t m_end, double* out);
/* op(bra, ket) for single host vectors (reference _LocalOperator.__call__,
 * kwant/operator.pyx:470-559, MAT_ELS): out num_outputs complex128. */
KPM_API int kpm_op_apply(kpm_op* op, const double* bra, const double* ket,
                         double* out);

/* One-shot DOS (the C-ABI form of SpectralDensity with operator=None and
 * explicit bounds): uploads ham and vecs, runs the recursion, reduces the
 * moments (mean over vectors, /a, kernel) and reconstructs the density at
 * the 2M Chebyshev nodes on the device.  KPM_PREC_MIXED uses
 * KPM_FLAG_REORDER.  moments_out: R x M complex128 (may
 * be NULL); gammas_out / densities_out: 2M complex128 (may be NULL).
 * KPM_EDIVERGED as kpm_block_dos_moments, with every output written. */
KPM_API int kpm_dos(const kpm_csr_desc* ham, double a, double b, int precision,
                    const double* vecs, int64_t R, int64_t M, int kernel,
                    double* moments_out, double* gammas_out, double* densities_out);

/* ---- DOS moments without allocation ----------------------------------------
 * No counterpart in the reference.  For callers that cannot let this library
 * allocate device memory -- an application or framework that owns all device
 * memory through its own arena and passes its libraries preallocated buffers,
 * or a service with a fixed, audited device-memory budget -- this runs the
 * same DOS recursion as kpm_block_dos_moments with nothing allocated: no
 * cudaMalloc/cudaFree, no library allocator, no stream or event creation.
 * Apart from the caller's buffers it uses one file-scope device array of
 * KPM_NOALLOC_SCRATCH_BYTES (held by every device that loads the library
 * until the process exits) for the dot-product partials.
 *
 * All pointers are device pointers on the current device:
 *   ham->indptr/indices: int32 CSR of the Hamiltonian (must be valid: it is
 *     not checked on the device); ham->data: complex128 H (KPM_PREC_FP64) or
 *     complex64 values 2H/a (KPM_PREC_MIXED);
 *   vecs: the R starting vectors in the device layout [N][Rpad] (row-major,
 *     vectors fastest), complex128 (FP64) or complex64 (MIXED), Rpad = R
 *     rounded up to 16 (FP64) or 32 (MIXED), padding vectors zero; only read;
 *   work: 2 * N * Rpad complex elements of the same type; on return it holds
 *     the last two Chebyshev vectors;
 *   moments: M * Rpad complex128, written as [moment][vector].
 * Work is enqueued on `stream` (a cudaStream_t; NULL = default stream) and
 * the call returns without waiting: results are valid once the stream has
 * completed.  The first call in each device context looks up the scratch
 * array's device address (cudaGetSymbolAddress, with that device current)
 * and caches it with the context's id, so a new context (after
 * cudaDeviceReset, or one the caller made current) gets its own lookup;
 * make the first call in a context before any stream capture.  Calls whose
 * GPU work overlaps in time (different streams, threads or processes
 * sharing the device context) share the scratch array and race: serialise
 * them.  The array keeps the last call's contents, and every call writes
 * what it reads.  Sizes whose
 * scratch would exceed KPM_NOALLOC_SCRATCH_BYTES (more than about 500
 * vectors at the largest row-partition count) are rejected with KPM_EINVAL. */
typedef struct kpm_device_csr {
  int64_t rows;
  int64_t nnz;
  const int32_t* indptr;
  const int32_t* indices;
  const void* data;
} kpm_device_csr;
#define KPM_NOALLOC_SCRATCH_BYTES (8u << 20)
KPM_API int kpm_dos_moments_noalloc(const kpm_device_csr* ham, double a,
                                    double b, int precision, const void* vecs,
                                    int64_t R, int64_t M, void* work,
                                    double* moments, void* stream);

/* ---- batched multi-system DOS ------------------------------------------------
 * Many independent systems (disorder realisations, parameter points,
 * lattices of different size) advanced together: every Chebyshev step of all
 * systems is one launch (work items of all systems in one index space), and
 * the whole step loop is captured once in a CUDA graph and replayed.  The
 * matrices are block-sparse with 4 x 4 blocks (BSR4), the recursion is
 * complex64 with FP64 moment accumulation, and the R random-phase vectors of
 * every system come from a counter-based generator on the device (SplitMix64
 * of (seed, system, vector, orbital); u = top 24 bits / 2^24, vector entry
 * exp(2 pi i u)), not from the reference's MT19937 stream.  Replaces running
 * SpectralDensity (kwant/kpm.py:163-252) once per realisation. */
typedef struct kpm_batch kpm_batch;
typedef struct kpm_bsr_desc {
  int64_t block_rows;      /* orbitals = 4 * block_rows */
  int64_t nnzb;
  const int32_t* indptr;   /* block_rows + 1 */
  const int32_t* indices;  /* nnzb block columns */
  const double* data;      /* nnzb row-major 4x4 blocks, complex128 */
} kpm_bsr_desc;
KPM_API int kpm_batch_create(int64_t num_vectors, int64_t num_moments,
                             uint64_t seed, kpm_batch** out);
/* Add a system given as a host BSR4 matrix with its rescaling (a, b). */
KPM_API int kpm_batch_add_bsr(kpm_batch* bt, const kpm_bsr_desc* ham,
                              double a, double b);
/* Add an L^3 Wilson-Dirac system generated on the device: onsite
 * (m - 3) G0 + w 1, hopping H[r + e_j, r] = (G0 - i Gj) / 2, open
 * boundaries, G0 = tau_z (x) sigma_0, Gj = tau_x (x) sigma_j; disorder
 * w = W (u - 1/2), u = SplitMix64(seed, site) / 2^64 (53 bits).  Rescaled
 * with (a, b). */
KPM_API int kpm_batch_add_wilson_dirac(kpm_batch* bt, int64_t L, double m,
                                       double W, uint64_t seed, double a,
                                       double b);
/* Run the DOS recursion of every system (moments averaged over the R
 * vectors): out is num_systems x num_moments complex128.  The first call
 * allocates the vectors, picks the kernel variant (autotuner over variants
 * with identical arithmetic) and captures the step loop in a CUDA graph;
 * later calls replay the graph. */
KPM_API int kpm_batch_run(kpm_batch* bt, double* out);
/* Device time (ms) of the last kpm_batch_run's graph and the number of
 * kernel nodes it contains; the chosen variant (vectors per lane). */
KPM_API int kpm_batch_stats(kpm_batch* bt, double* ms, int64_t* nodes,
                            int* vectors_per_lane);
/* Step format chosen at the first kpm_batch_run.  When every row of every
 * system has at most 16 non-zero entries, two sparse forms are built on the
 * device besides the dense 4 x 4 blocks (format 0): an orbital-row ELL
 * (format 1, ell_width its width) and sparse blocks (format 2: the block
 * rows' vector rows staged in shared memory, products over the non-zero
 * entries only); the autotuner times all of them and keeps the fastest. */
KPM_API int kpm_batch_format(kpm_batch* bt, int* format, int* ell_width);
/* Work order chosen at the first kpm_batch_run (formats 0 and 1): 0 when
 * the vector groups of a row partition run side by side (they share its
 * matrix rows in L2), 1 when all partitions of one vector group do (the
 * resident blocks then cover a band of rows wide enough that the gathered
 * rows of distant neighbours, e.g. L^2 block rows away on an L^3 lattice,
 * are still in L2).  Results do not depend on it. */
KPM_API int kpm_batch_order(kpm_batch* bt, int* group_major);
KPM_API int kpm_batch_destroy(kpm_batch* bt);

/* ---- reconstruction (device) -------------------------------------------------
 * _moments + _calc_fft_moments, kwant/kpm.py:378-388 and :1197-1222:
 * moments (R x M x W complex128, host) -> mean over R (if mean) -> / a ->
 * kernel -> zero-pad to 2M -> DCT-III -> reversed ("gammas", 2M x W') ->
 * divided by pi sqrt(1 - x_k^2) at the nodes x_k ("densities").
 * W' = W if mean else R x W.  nodes: the 2M ascending Chebyshev nodes.
 * is_real: the moments passed numpy's real_if_close (kwant/kpm.py:379);
 * imaginary parts are ignored and divisions are true divisions (numpy's
 * real arithmetic) instead of reciprocal multiplications (its complex
 * arithmetic).  Outputs are complex128; gammas_out or densities_out may be
 * NULL. */
KPM_API int kpm_reconstruct(int64_t R, int64_t M, int64_t W, const double* moments,
                            int mean, int is_real, double a, int kernel,
                            double lorentz_l, const double* nodes, double* gammas_out,
                            double* densities_out);
/* Chebyshev series sum_n c[n][w] T_n(x_e) at E arbitrary points (the
 * chebval of SpectralDensity.__call__, kwant/kpm.py:263-295): coefs M x W
 * complex128, x E doubles in [-1, 1], out E x W complex128.  numpy's
 * Clenshaw recursion with the same rounding (results equal numpy's). */
KPM_API int kpm_chebval(int64_t M, int64_t W, const double* coefs, int64_t E,
                        const double* x, double* out);
/* Kernel weights g_m (M doubles) as applied by kpm_reconstruct. */
KPM_API int kpm_kernel_weights(int64_t M, int kernel, double lorentz_l, double* g);

/* ---- spectral bounds -------------------------------------------------------
 * Extremal eigenvalues of the Hermitian ham by FP64 Lanczos on the device,
 * started from v0 (N complex128, the reference's _v0, kwant/kpm.py:203),
 * until the Ritz residual of both extremes is below tol * max|theta|
 * (replaces the two ARPACK eigsh calls of kwant/kpm.py:1169-1172).
 * Returns the Ritz values widened by their residual norms. */
KPM_API int kpm_bounds(const kpm_csr_desc* ham, const double* v0, double tol,
                       int max_iter, double* lmin, double* lmax, int* iterations);

/* Single-vector FP64 matvec y = ham x on the device (x, y host, N complex128);
 * the matvec that an ARPACK driver on the host calls (bounds_method
 * "arpack" of the Python layer). */
KPM_API int kpm_handle_matvec(kpm_handle* h, const double* x, double* y);

/* ---- correlator / Kubo-Bastin ----------------------------------------------
 * Correlator moments matrix (kwant/kpm.py:557-606, :685-695):
 *   Psi_n = v_beta T_n(H~)|r>,  Omega_m = T_m(H~') v_alpha|r>,
 *   mu_mn = (1/R) sum_r <Omega_m | Psi_n>        (M x M complex128).
 * H~ uses the handle's (a, b); H~' uses (a2, b2) (the re-derived bounds of
 * kwant/kpm.py:576-579).  v_alpha, v_beta are CSR (e.g. the velocity of
 * _velocity, kwant/kpm.py:1042-1085).  gemm selects the contraction:
 *   0 = FP64 CUDA-core GEMM, 1 = tensor-core split-BF16 (hi+lo) GEMM with
 *   FP32 accumulation (tcgen05), 2 = automatic (1 for MIXED, 0 for FP64),
 *   3 = the same BF16 hi/lo products on CUDA cores (checks gemm 1),
 *   4 = tensor-core split-FP16 (hi+lo) GEMM: gemm 1's layout, MMAs and
 *   time with 11 instead of 8 significant bits per part, 5 = gemm 4's
 *   products on CUDA cores (checks gemm 4).  With gemm 4 / 5 a vector entry
 *   above the FP16 range (65504) makes mu non-finite: KPM_EDIVERGED, with
 *   mu_out written.
 * mu_out is the mean over vectors (or R x M x M when per_vector). */
KPM_API int kpm_correlator_moments(kpm_handle* h, double a2, double b2,
                                   const kpm_csr_desc* v_alpha,
                                   const kpm_csr_desc* v_beta, const double* vecs,
                                   int64_t R, int64_t M, int gemm, int per_vector,
                                   double* mu_out);

/* Fermi-weighted node sums for a grid of (mu, T) points, the device form
 * of SpectralDensity.integrate (Gauss-Chebyshev sum, kwant/kpm.py:297-316)
 * and of Correlator.__call__ (Simpson over the nodes, kwant/kpm.py:
 * 608-630) with fermi_distribution (kwant/kpm.py:990-1009):
 *   out[p][w] = sum_k weights[k] * f(energies[k]; mu[p], T[p]) * values[k][w]
 * energies, weights: n doubles; values: n x W complex128; out: P x W
 * complex128.  mu and temperature: P doubles (T >= 0; T = 0 is the step
 * E - mu < 0), or both NULL for f = 1 (then P = 1).  The caller folds the
 * quadrature weights and any energy-dependent factor into weights. */
KPM_API int kpm_fermi_sums(int64_t n, const double* energies,
                           const double* weights, int64_t W,
                           const double* values, int64_t P, const double* mu,
                           const double* temperature, double* out);

/* Learned-surrogate ensemble on the device (no reference counterpart): the
 * DOS of each of E members (E <= 8) at K energies is members[e][p] . At[:,k]
 * (members E x P x M, At M x K, both FP64 row-major); spread[p] = the
 * largest over k of the members' standard deviation (ddof 1); with ref
 * (P x M moments), err[p] = the largest |member mean - ref[p] . At[:,k]|.
 * err may be NULL; it needs ref. */
KPM_API int kpm_ensemble_dos(int64_t E, int64_t P, int64_t M, int64_t K,
                             const double* members, const double* At,
                             const double* ref, double* spread, double* err);

/* Integral factor of Correlator._build_integral_factor (kwant/kpm.py:
 * 720-760) on the device: mu (M x M complex128), kernel weights g (M, with
 * g[0] already halved), nodes x_k (2M) -> factor (2M complex128). */
KPM_API int kpm_integral_factor(int64_t M, const double* mu, const double* g,
                                const double* nodes, double* factor_out);

/* ---- parametric Hamiltonian family (parameter sweeps) -----------------------
 * A three-parameter family on the handle's sparsity structure,
 *   H(phi, s1, s2) = B .* exp(i phi Theta) + s1 D1 + s2 D2,
 * e.g. hoppings B with Peierls phases Theta per unit flux phi, and onsite
 * terms D1 (a fixed disorder pattern, s1 = its strength) and D2 (a staggered
 * mass, s2 = the mass).  The four CSR matrices must have exactly the
 * structure (indptr, indices) the handle was created with; Theta must be
 * real.  kpm_family_point regenerates the handle's matrix values on the
 * device for one parameter point (FP64: H; MIXED: 2H/a, the ELL copy
 * included); the handle's (a, b) must bound the spectrum of every point
 * used.  Blocks created on the handle must be rewound after a point change.
 * Replaces re-running the reference's Hamiltonian assembly
 * (hamiltonian_submatrix, kwant/_system.pyx:233-338) with new params per
 * sweep point. */
KPM_API int kpm_family_set(kpm_handle* h, const kpm_csr_desc* base,
                           const kpm_csr_desc* theta, const kpm_csr_desc* d1,
                           const kpm_csr_desc* d2);
KPM_API int kpm_family_point(kpm_handle* h, double phi, double s1, double s2);

/* ---- learned moment surrogate: multilayer perceptron ---------------------
 * widths[0] -> widths[1] -> ... -> widths[num_layers] with exact-erf GELU
 * after every hidden layer and a linear output.  Parameters (FP32 master
 * copy, flat): for each layer l, W_l (widths[l+1] x widths[l], row-major)
 * then b_l (widths[l+1]).  Matmuls in BF16 with FP32 accumulation on the
 * tensor cores (tcgen05, TMA-fed); loss = mean squared error over all
 * outputs; optimiser Adam (beta1 0.9, beta2 0.999, eps 1e-8).  Hidden and
 * output widths must be multiples of 32; batches multiples of 32.
 * x: n x widths[0] float32, y: n x widths[num_layers] float32 (host).
 * No counterpart in the reference: the plain KPM path is its fallback. */
typedef struct kpm_mlp kpm_mlp;
KPM_API int kpm_mlp_create(int num_layers, const int32_t* widths,
                           int max_batch, uint64_t seed, kpm_mlp** out);
KPM_API int kpm_mlp_num_params(kpm_mlp* net, int64_t* count);
KPM_API int kpm_mlp_get_params(kpm_mlp* net, float* out);
/* Sets the parameters and resets the Adam state. */
KPM_API int kpm_mlp_set_params(kpm_mlp* net, const float* in);
KPM_API int kpm_mlp_forward(kpm_mlp* net, const float* x, int64_t n,
                            float* y);
/* Gradient of the loss on one batch (n <= max_batch) at the current
 * parameters (flat, like the parameters) and the loss itself. */
KPM_API int kpm_mlp_gradients(kpm_mlp* net, const float* x, const float* y,
                              int64_t n, float* grads, double* loss);
/* Mini-batch Adam over (x, y): every epoch shuffles the n samples
 * (mt19937_64 from seed) and takes floor(n / batch) steps; final_loss is
 * the mean batch loss of the last epoch. */
KPM_API int kpm_mlp_train(kpm_mlp* net, const float* x, const float* y,
                          int64_t n, int batch, int64_t epochs, double lr,
                          uint64_t seed, double* final_loss);
KPM_API int kpm_mlp_destroy(kpm_mlp* net);

/* ---- diagnostics -------------------------------------------------------------- */
/* Device time (ms) of the last recursion call on the handle, measured with
 * CUDA events on the handle's stream around the kernels only. */
KPM_API int kpm_last_kernel_ms(kpm_handle* h, double* ms);
/* Per-launch profiling of the Chebyshev step kernels of a handle: while
 * enabled, every step-kernel launch is bracketed by CUDA events on the
 * handle's stream.  kpm_profile_read returns (and resets) the number of
 * timed launches and their summed device time in ms. */
KPM_API int kpm_profile(kpm_handle* h, int enable);
KPM_API int kpm_profile_read(kpm_handle* h, int64_t* launches,
                             double* total_ms);
/* Device time (CUDA events around the kernel) of the last tensor-core
 * moments-matrix contraction of the handle, and the BF16 MMA flops it
 * executed (12 real products x 2 M^2 K_padded); 0 if none ran. */
KPM_API int kpm_last_gemm(kpm_handle* h, double* ms, double* flops);
/* Number of kernel launches issued by this library since load. */
KPM_API int kpm_launch_count(int64_t* count);

#ifdef __cplusplus
}
#endif

#endif /* KWANT_GB300_H */
