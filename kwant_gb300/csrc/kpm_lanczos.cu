// Spectral bounds by FP64 Lanczos on the device.
//
// Replaces the two ARPACK eigsh calls of _rescale (kwant/kpm.py:1169-1172,
// which="LA" and "SA", tol = eps/2, started from _v0).  A plain Lanczos
// recurrence (no reorthogonalisation: loss of orthogonality only produces
// duplicate copies of converged Ritz values and does not move the extreme
// ones) runs on the device; every CHECK iterations the host computes the
// extreme eigenvalues of the tridiagonal matrix by Sturm bisection, their
// eigenvectors by inverse iteration, and the Ritz residuals
// beta_k |s_k|.  Iteration stops when both residuals are below
// tol * max(|theta|); the returned bounds are the Ritz values widened
// outward by their residuals, so that a bound that is too tight (which makes
// the Chebyshev recursion diverge) is unlikely.

#include <algorithm>
#include <cmath>
#include <vector>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// y = H x (- beta q_prev); complex128, 4 threads per row.
__global__ void lz_spmv_kernel(int64_t rows, const int32_t* __restrict__ ip,
                               const int32_t* __restrict__ ix,
                               const double2* __restrict__ v,
                               const double2* __restrict__ x,
                               const double2* __restrict__ qprev,
                               const double* __restrict__ beta_j,
                               double2* __restrict__ y) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = t >> 2;
  const int sub = threadIdx.x & 3;
  double ar = 0.0, ai = 0.0;
  if (row < rows) {
    for (int jj = ip[row] + sub; jj < ip[row + 1]; jj += 4) {
      const double2 h = v[jj];
      const double2 xv = x[ix[jj]];
      ar = fma(h.x, xv.x, fma(-h.y, xv.y, ar));
      ai = fma(h.x, xv.y, fma(h.y, xv.x, ai));
    }
  }
  ar += __shfl_xor_sync(0xffffffffu, ar, 1);
  ai += __shfl_xor_sync(0xffffffffu, ai, 1);
  ar += __shfl_xor_sync(0xffffffffu, ar, 2);
  ai += __shfl_xor_sync(0xffffffffu, ai, 2);
  if (row < rows && sub == 0) {
    if (qprev) {
      const double b = *beta_j;
      const double2 q = qprev[row];
      ar -= b * q.x;
      ai -= b * q.y;
    }
    y[row] = make_double2(ar, ai);
  }
}

// y = H x, one thread per row, CSR order, every operation rounded (no FMA):
// the same arithmetic as scipy's csr_matvec, so that a host ARPACK driver
// sees the reference's matvec.
__global__ void exact_spmv_kernel(int64_t rows, const int32_t* __restrict__ ip,
                                  const int32_t* __restrict__ ix,
                                  const double2* __restrict__ v,
                                  const double2* __restrict__ x,
                                  double2* __restrict__ y) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double ar = 0.0, ai = 0.0;
  for (int jj = ip[row]; jj < ip[row + 1]; ++jj) {
    const double2 h = v[jj];
    const double2 xv = x[ix[jj]];
    ar = __dadd_rn(ar, __dsub_rn(__dmul_rn(h.x, xv.x), __dmul_rn(h.y, xv.y)));
    ai = __dadd_rn(ai, __dadd_rn(__dmul_rn(h.x, xv.y), __dmul_rn(h.y, xv.x)));
  }
  y[row] = make_double2(ar, ai);
}

// partial sums of Re<a|b> (or |a|^2 when b == a) per block
__global__ void lz_dot_partial_kernel(int64_t n, const double2* __restrict__ a,
                                      const double2* __restrict__ b,
                                      double* __restrict__ part) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 u = a[i], w = b[i];
    acc = fma(u.x, w.x, fma(u.y, w.y, acc));
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// out = sum(part); if sq, out = sqrt(out)
__global__ void lz_finish_kernel(const double* __restrict__ part, int nparts,
                                 double* out, int sq) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sq ? sqrt(s[0]) : s[0];
}

// w -= alpha q
__global__ void lz_axpy_kernel(int64_t n, const double* __restrict__ alpha,
                               const double2* __restrict__ q,
                               double2* __restrict__ w) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double a = *alpha;
    double2 v = w[i];
    const double2 u = q[i];
    v.x -= a * u.x;
    v.y -= a * u.y;
    w[i] = v;
  }
}

// q = w / beta (beta > 0), else leaves q unchanged
__global__ void lz_scale_kernel(int64_t n, const double* __restrict__ beta,
                                const double2* __restrict__ w,
                                double2* __restrict__ q) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double b = *beta;
  if (i < n && b > 0.0) {
    const double2 v = w[i];
    q[i] = make_double2(v.x / b, v.y / b);
  }
}

// --------------------------------------------------- tridiagonal (host)
// Number of eigenvalues of T (diag d, offdiag e, e[i] couples i, i+1) < x.
static int sturm_count(const std::vector<double>& d,
                       const std::vector<double>& e, int k, double x) {
  int cnt = 0;
  double q = 1.0;
  for (int i = 0; i < k; ++i) {
    const double off = i > 0 ? e[i - 1] * e[i - 1] : 0.0;
    q = d[i] - x - (i > 0 ? off / q : 0.0);
    if (q == 0.0) q = -1e-300;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// i-th smallest eigenvalue (0-based) by bisection
static double bisect_eig(const std::vector<double>& d,
                         const std::vector<double>& e, int k, int i) {
  double lo = 1e300, hi = -1e300;
  for (int j = 0; j < k; ++j) {
    const double r = (j > 0 ? fabs(e[j - 1]) : 0.0) +
                     (j + 1 < k ? fabs(e[j]) : 0.0);
    lo = std::min(lo, d[j] - r);
    hi = std::max(hi, d[j] + r);
  }
  const double scale = std::max(fabs(lo), fabs(hi));
  lo -= 1e-12 * scale + 1e-300;
  hi += 1e-12 * scale + 1e-300;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid == lo || mid == hi) break;
    if (sturm_count(d, e, k, mid) > i)
      hi = mid;
    else
      lo = mid;
  }
  return 0.5 * (lo + hi);
}

// |last component| of the unit eigenvector of T for eigenvalue theta, by
// inverse iteration (tridiagonal LU without pivoting, shifted slightly).
static double last_component(const std::vector<double>& d,
                             const std::vector<double>& e, int k,
                             double theta) {
  if (k == 1) return 1.0;
  double scale = 0.0;
  for (int j = 0; j < k; ++j) scale = std::max(scale, fabs(d[j]));
  for (int j = 0; j + 1 < k; ++j) scale = std::max(scale, fabs(e[j]));
  const double shift = theta + 1e-10 * (scale > 0 ? scale : 1.0);
  std::vector<double> x(k, 1.0), c(k), dd(k), y(k);
  for (int it = 0; it < 4; ++it) {
    // solve (T - shift) y = x  (Thomas algorithm)
    dd[0] = d[0] - shift;
    if (dd[0] == 0.0) dd[0] = 1e-300;
    y[0] = x[0];
    for (int j = 1; j < k; ++j) {
      const double m = e[j - 1] / dd[j - 1];
      dd[j] = d[j] - shift - m * e[j - 1];
      if (dd[j] == 0.0) dd[j] = 1e-300;
      y[j] = x[j] - m * y[j - 1];
    }
    x[k - 1] = y[k - 1] / dd[k - 1];
    for (int j = k - 2; j >= 0; --j) x[j] = (y[j] - e[j] * x[j + 1]) / dd[j];
    double nrm = 0.0;
    for (int j = 0; j < k; ++j) nrm += x[j] * x[j];
    nrm = sqrt(nrm);
    for (int j = 0; j < k; ++j) x[j] /= nrm;
  }
  return fabs(x[k - 1]);
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_bounds(const kpm_csr_desc* ham, const double* v0, double tol,
               int max_iter, double* lmin, double* lmax, int* iterations) {
  NvtxRange nvtx("kpm_bounds");
  KPM_REQUIRE(ham && v0 && lmin && lmax, "kpm_bounds: null argument");
  KPM_REQUIRE(tol > 0 && max_iter >= 2, "kpm_bounds: invalid tol/max_iter");
  kpm_handle* h = nullptr;
  KPM_TRY(kpm_create(ham, 1.0, 0.0, KPM_PREC_FP64, &h));
  const int64_t N = ham->rows;
  cudaStream_t s = h->stream;
  const int CHECK = 10;
  const int nparts = 256;
  double2 *q0 = nullptr, *q1 = nullptr, *w = nullptr;
  double *coefs = nullptr, *part = nullptr;
  int st = dev_alloc((void**)&q0, N * 16, s);
  if (st == KPM_OK) st = dev_alloc((void**)&q1, N * 16, s);
  if (st == KPM_OK) st = dev_alloc((void**)&w, N * 16, s);
  // coefs[2j] = alpha_j, coefs[2j+1] = beta_{j+1}; coefs[-1] slot: beta_0
  if (st == KPM_OK)
    st = dev_alloc((void**)&coefs, (2 * (int64_t)max_iter + 2) * 8, s);
  if (st == KPM_OK) st = dev_alloc((void**)&part, nparts * 8, s);
  cudaError_t e = cudaSuccess;
  std::vector<double> hc(2 * (size_t)max_iter + 2, 0.0);
  int k = 0;
  double th_lo = 0, th_hi = 0, r_lo = 0, r_hi = 0;
  bool converged = false;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(w, v0, N * 16, cudaMemcpyHostToDevice, s);
    // q0 = v0 / |v0|
    const unsigned gb = (unsigned)ceil_div(N, 256);
    if (e == cudaSuccess) {
      lz_dot_partial_kernel<<<nparts, 256, 0, s>>>(N, w, w, part);
      lz_finish_kernel<<<1, 256, 0, s>>>(part, nparts, coefs + 1, 1);
      lz_scale_kernel<<<gb, 256, 0, s>>>(N, coefs + 1, w, q0);
      cudaMemsetAsync(coefs + 1, 0, 8, s);  // beta_0 = 0
      count_launch(3);
      e = cudaGetLastError();
    }
    double2* qj = q0;
    double2* qp = q1;
    const unsigned gs = (unsigned)ceil_div(N * 4, 256);
    while (e == cudaSuccess && k < max_iter) {
      // beta_j lives at coefs[2j-1] (coefs[1] = beta_0 = 0 for j = 0)
      const double* beta_j = coefs + (k == 0 ? 1 : 2 * k - 1);
      lz_spmv_kernel<<<gs, 256, 0, s>>>(N, h->H.indptr, h->H.indices,
                                        (const double2*)h->H.data, qj,
                                        k == 0 ? nullptr : qp, beta_j, w);
      lz_dot_partial_kernel<<<nparts, 256, 0, s>>>(N, qj, w, part);
      lz_finish_kernel<<<1, 256, 0, s>>>(part, nparts, coefs + 2 * k, 0);
      lz_axpy_kernel<<<gb, 256, 0, s>>>(N, coefs + 2 * k, qj, w);
      lz_dot_partial_kernel<<<nparts, 256, 0, s>>>(N, w, w, part);
      lz_finish_kernel<<<1, 256, 0, s>>>(part, nparts, coefs + 2 * k + 1, 1);
      // q_{j+1} overwrites q_{j-1}
      lz_scale_kernel<<<gb, 256, 0, s>>>(N, coefs + 2 * k + 1, w, qp);
      count_launch(7);
      e = cudaGetLastError();
      std::swap(qj, qp);
      ++k;
      if (e != cudaSuccess) break;
      if (k % CHECK == 0 || k == max_iter || k == N) {
        e = cudaMemcpyAsync(hc.data(), coefs, 2 * (size_t)k * 8,
                            cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) break;
        std::vector<double> d(k), off(k);
        for (int j = 0; j < k; ++j) {
          d[j] = hc[2 * j];
          off[j] = hc[2 * j + 1];
        }
        // breakdown: beta_j ~ 0 (relative to the coefficients so far) means
        // span(q_0..q_j) is invariant and its Ritz values are exact
        // eigenvalues; the coefficients computed after it (from an
        // unnormalised q) are discarded
        int kk = k;
        double mag = 0.0;
        for (int j = 0; j < k; ++j) {
          mag = std::max(mag, fabs(d[j]));
          if (j > 0) mag = std::max(mag, fabs(off[j - 1]));
          if (off[j] <= 1e-14 * (mag > 0 ? mag : 1.0)) {
            kk = j + 1;
            break;
          }
        }
        const double beta_k = off[kk - 1];
        th_lo = bisect_eig(d, off, kk, 0);
        th_hi = bisect_eig(d, off, kk, kk - 1);
        r_lo = beta_k * last_component(d, off, kk, th_lo);
        r_hi = beta_k * last_component(d, off, kk, th_hi);
        const double sc = std::max(fabs(th_lo), fabs(th_hi));
        const double small = 1e-14 * (sc > 0 ? sc : 1.0);
        if (kk < k || (r_lo <= tol * sc && r_hi <= tol * sc) ||
            beta_k <= small || k == N) {
          converged = true;
          break;
        }
      }
    }
  }
  dev_free(q0, s);
  dev_free(q1, s);
  dev_free(w, s);
  dev_free(coefs, s);
  dev_free(part, s);
  cudaStreamSynchronize(s);
  kpm_destroy(h);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  if (iterations) *iterations = k;
  if (!converged) {
    set_error("kpm_bounds: Lanczos did not converge in %d iterations "
              "(residuals %.3g, %.3g)", k, r_lo, r_hi);
    return KPM_ETIMEOUT;
  }
  *lmin = th_lo - r_lo;
  *lmax = th_hi + r_hi;
  return KPM_OK;
}

int kpm_handle_matvec(kpm_handle* h, const double* x, double* y) {
  KPM_REQUIRE(h && x && y, "kpm_handle_matvec: null argument");
  if (h->precision != KPM_PREC_FP64 || h->perm) {
    set_error("kpm_handle_matvec: needs a KPM_PREC_FP64 handle without "
              "reordering");
    return KPM_EUNSUPPORTED;
  }
  const int64_t N = h->H.rows;
  cudaStream_t s = h->stream;
  double2 *dx = nullptr, *dy = nullptr;
  int st = dev_alloc((void**)&dx, N * 16, s);
  if (st == KPM_OK) st = dev_alloc((void**)&dy, N * 16, s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(dx, x, N * 16, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      exact_spmv_kernel<<<(unsigned)ceil_div(N, 128), 128, 0, s>>>(
          N, h->H.indptr, h->H.indices, (const double2*)h->H.data, dx, dy);
      count_launch(1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(y, dy, N * 16, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(dx, s);
  dev_free(dy, s);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  return KPM_OK;
}

}  // extern "C"
