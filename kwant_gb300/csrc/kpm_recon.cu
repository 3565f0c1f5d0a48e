// Device-side moment reduction, kernel damping and DCT reconstruction.
//
// SpectralDensity._moments (kwant/kpm.py:378-388): mean over vectors, / a,
// kernel (jackson_kernel kwant/kpm.py:1106-1123, lorentz_kernel :1126-1142);
// _calc_fft_moments (kwant/kpm.py:1197-1222): zero-pad to 2M, DCT-III,
// reverse, divide by pi sqrt(1 - x^2).
//
// The DCT-III of a length-2M input whose upper half is zero is evaluated
// directly, y_k = x_0 + 2 sum_{n=1}^{M-1} x_n cos(pi n (2k+1) / (4M)), with
// the cosine argument reduced exactly in integers (n (2k+1) mod 8M) and read
// from a table of cos(pi q / 4M), q < 8M, built with cospi.  That costs
// O(M^2 W) FP64 work, negligible next to the recursion, and is more accurate
// than an FFT-based transform.
//
// Numerics follow numpy where it matters for parity: for complex data,
// division by a real number is a multiplication by its rounded reciprocal
// (numpy's complex division with a zero imaginary divisor); for real data it
// is a true division.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

__global__ void kernel_weights_kernel(int64_t M, int kind, double l,
                                      double* g) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  double v = 1.0;
  if (kind == KPM_KERNEL_JACKSON) {
    const double n1 = (double)(M + 1);
    const double ang = M_PI * (double)m / n1;
    v = ((double)(M - m + 1) * cos(ang) + sin(ang) / tan(M_PI / n1)) / n1;
  } else if (kind == KPM_KERNEL_LORENTZ) {
    v = sinh(l * (1.0 - (double)m / (double)M)) / sinh(l);
  }
  g[m] = v;
}

// mean over R (sequential in r), scale by 1/a, kernel weight.
// in: [R][M][W] complex; out: [M][Wo] complex, Wo = W (mean) or R*W with the
// vector axis second (kwant/kpm.py:381: swapaxes(0, 1)).
__global__ void reduce_scale_kernel(const double2* __restrict__ in,
                                    double2* __restrict__ out, int64_t R,
                                    int64_t M, int64_t W, int mean,
                                    int is_real, double a,
                                    const double* __restrict__ g) {
  const int64_t Wo = mean ? W : R * W;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * Wo) return;
  const int64_t m = idx / Wo, c = idx % Wo;
  double re, im;
  if (mean) {
    re = 0.0;
    im = 0.0;
    for (int64_t r = 0; r < R; ++r) {
      double2 v = in[(r * M + m) * W + c];
      re += v.x;
      im += v.y;
    }
    if (is_real) {
      re = re / (double)R;
      im = 0.0;
    } else {
      const double inv = 1.0 / (double)R;
      re = re * inv;
      im = im * inv;
    }
  } else {
    const int64_t r = c / W, w = c % W;
    double2 v = in[(r * M + m) * W + w];
    re = v.x;
    im = is_real ? 0.0 : v.y;
  }
  if (is_real) {
    re = re / a;
  } else {
    const double inv = 1.0 / a;
    re = re * inv;
    im = im * inv;
  }
  const double gm = g[m];
  out[idx] = make_double2(re * gm, im * gm);
}

__global__ void cos_table_kernel(int64_t M, double* tab) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < 8 * M) tab[q] = cospi((double)q / (double)(4 * M));
}

// gammas[j][w] = y[2M-1-j][w];  rho = gammas / (pi sqrt(1 - x_j^2))
__global__ void dct3_kernel(const double2* __restrict__ x,
                            const double* __restrict__ tab, int64_t M,
                            int64_t W, const double* __restrict__ nodes,
                            int is_real, double2* __restrict__ gammas,
                            double2* __restrict__ rho) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t K = 2 * M;
  if (idx >= K * W) return;
  const int64_t j = idx / W, w = idx % W;
  const int64_t k = K - 1 - j;
  const int64_t step = 2 * k + 1, period = 8 * M;
  double sr = 0.0, si = 0.0;
  int64_t q = 0;
  for (int64_t n = 1; n < M; ++n) {
    q += step;
    if (q >= period) q %= period;
    const double c = tab[q];
    const double2 v = x[n * W + w];
    sr = fma(v.x, c, sr);
    si = fma(v.y, c, si);
  }
  const double2 x0 = x[w];
  const double yr = x0.x + 2.0 * sr, yi = x0.y + 2.0 * si;
  if (gammas) gammas[idx] = make_double2(yr, yi);
  if (rho) {
    const double e = nodes[j];
    // numpy: pi * sqrt(1 - e**2), each operation rounded (no FMA: near
    // |e| = 1 the contraction would change 1 - e^2 in its leading digits)
    const double gk = __dmul_rn(M_PI, sqrt(__dsub_rn(1.0, __dmul_rn(e, e))));
    if (is_real) {
      rho[idx] = make_double2(yr / gk, 0.0);
    } else {
      const double inv = 1.0 / gk;
      rho[idx] = make_double2(yr * inv, yi * inv);
    }
  }
}

int reconstruct_on_device(cudaStream_t s, int64_t R, int64_t M, int64_t W,
                          const double2* moments, int mean, int is_real,
                          double a, int kernel, double lorentz_l,
                          const double* nodes_host, double* gammas_out,
                          double* densities_out) {
  const int64_t Wo = mean ? W : R * W;
  const int64_t K = 2 * M;
  double *g = nullptr, *tab = nullptr, *nodes = nullptr;
  double2 *red = nullptr, *gam = nullptr, *rho = nullptr;
  int st = KPM_OK;
  st = dev_alloc((void**)&g, M * sizeof(double), s);
  if (st == KPM_OK) st = dev_alloc((void**)&tab, 8 * M * sizeof(double), s);
  if (st == KPM_OK) st = dev_alloc((void**)&nodes, K * sizeof(double), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&red, M * Wo * sizeof(double2), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&gam, K * Wo * sizeof(double2), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&rho, K * Wo * sizeof(double2), s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(nodes, nodes_host, K * sizeof(double),
                        cudaMemcpyHostToDevice, s);
  }
  if (st == KPM_OK && e == cudaSuccess) {
    kernel_weights_kernel<<<(unsigned)ceil_div(M, 256), 256, 0, s>>>(
        M, kernel, lorentz_l, g);
    cos_table_kernel<<<(unsigned)ceil_div(8 * M, 256), 256, 0, s>>>(M, tab);
    reduce_scale_kernel<<<(unsigned)ceil_div(M * Wo, 256), 256, 0, s>>>(
        moments, red, R, M, W, mean, is_real, a, g);
    dct3_kernel<<<(unsigned)ceil_div(K * Wo, 128), 128, 0, s>>>(
        red, tab, M, Wo, nodes, is_real, gam, rho);
    count_launch(4);
    e = cudaGetLastError();
    if (e == cudaSuccess && gammas_out)
      e = cudaMemcpyAsync(gammas_out, gam, K * Wo * sizeof(double2),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && densities_out)
      e = cudaMemcpyAsync(densities_out, rho, K * Wo * sizeof(double2),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(g, s);
  dev_free(tab, s);
  dev_free(nodes, s);
  dev_free(red, s);
  dev_free(gam, s);
  dev_free(rho, s);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  return KPM_OK;
}

// ---------------------------------------------------------- integral factor
// Correlator._build_integral_factor (kwant/kpm.py:720-760), rewritten as
//   factor(e) = sum_m e+_m (mu~ t)_m + sum_n conj(e+_n) (mu~^T t)_n,
// t_n = T_n(e), e+_n = (e - i n sqrt(1-e^2)) exp(i n arccos e),
// mu~ = g g^T o mu.  One block per energy node.
__global__ void integral_factor_kernel(int64_t M,
                                       const double2* __restrict__ mu,
                                       const double* __restrict__ g,
                                       const double* __restrict__ nodes,
                                       double2* __restrict__ factor) {
  extern __shared__ double sh[];
  double* t = sh;                 // M
  double* ep = sh + M;            // 2M (re, im)
  double* red = sh + 3 * M;       // 2 * blockDim
  const int64_t k = blockIdx.x;
  const double e = nodes[k];
  const double se = sqrt(1.0 - e * e);
  const double th = acos(e);
  for (int64_t n = threadIdx.x; n < M; n += blockDim.x) {
    double sn, cn;
    sincos(th * (double)n, &sn, &cn);
    t[n] = cn;
    // (e - i n se) * (cn + i sn)
    const double br = e, bi = -(double)n * se;
    ep[2 * n] = br * cn - bi * sn;
    ep[2 * n + 1] = br * sn + bi * cn;
  }
  __syncthreads();
  double accr = 0.0, acci = 0.0;
  for (int64_t m = threadIdx.x; m < M; m += blockDim.x) {
    // u_m = sum_n mu~[m,n] t_n ;  w_m = sum_n mu~[n,m] t_n
    double ur = 0.0, ui = 0.0, wr = 0.0, wi = 0.0;
    const double gm = g[m];
    for (int64_t n = 0; n < M; ++n) {
      const double gn = g[n] * t[n];
      const double2 a1 = mu[m * M + n];
      const double2 a2 = mu[n * M + m];
      ur = fma(a1.x, gn, ur);
      ui = fma(a1.y, gn, ui);
      wr = fma(a2.x, gn, wr);
      wi = fma(a2.y, gn, wi);
    }
    ur *= gm; ui *= gm; wr *= gm; wi *= gm;
    const double er = ep[2 * m], ei = ep[2 * m + 1];
    // e+_m u_m + conj(e+_m) w_m
    accr += er * ur - ei * ui + er * wr + ei * wi;
    acci += er * ui + ei * ur + er * wi - ei * wr;
  }
  red[threadIdx.x] = accr;
  red[blockDim.x + threadIdx.x] = acci;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[threadIdx.x] += red[threadIdx.x + w];
      red[blockDim.x + threadIdx.x] += red[blockDim.x + threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) factor[k] = make_double2(red[0], red[blockDim.x]);
}

}  // namespace kpm

using namespace kpm;

// Chebyshev series at arbitrary points, one thread per (point, column):
// numpy.polynomial.chebyshev.chebval's Clenshaw recursion (c0 = c[-2],
// c1 = c[-1]; c0, c1 = c[-i] - c1, c0 + c1 * 2x; result c0 + c1 x) with
// the same separately rounded products and sums, so results are those of
// numpy bit for bit.
__global__ void chebval_kernel(int64_t M, int64_t W,
                               const double2* __restrict__ c, int64_t E,
                               const double* __restrict__ x,
                               double2* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= E * W) return;
  const int64_t e = t / W, w = t % W;
  const double xe = x[e];
  double2 c0, c1;
  if (M == 1) {
    c0 = c[w];
    c1 = make_double2(0.0, 0.0);
  } else {
    const double x2 = __dmul_rn(2.0, xe);
    c0 = c[(M - 2) * W + w];
    c1 = c[(M - 1) * W + w];
    for (int64_t i = 3; i <= M; ++i) {
      const double2 tmp = c0;
      const double2 ci = c[(M - i) * W + w];
      c0 = make_double2(__dsub_rn(ci.x, c1.x), __dsub_rn(ci.y, c1.y));
      c1 = make_double2(__dadd_rn(tmp.x, __dmul_rn(c1.x, x2)),
                        __dadd_rn(tmp.y, __dmul_rn(c1.y, x2)));
    }
  }
  out[t] = make_double2(__dadd_rn(c0.x, __dmul_rn(c1.x, xe)),
                        __dadd_rn(c0.y, __dmul_rn(c1.y, xe)));
}

// Fermi-weighted sums over the energy nodes for a grid of (mu, T) points:
// out[p][w] = sum_k weight[k] * f(E_k; mu_p, T_p) * values[k][w], with
// f = fermi_distribution of kwant/kpm.py:990-1009 (T = 0: the step
// E - mu < 0; otherwise 1 / (1 + exp((E - mu) / T))), or f = 1 when mu is
// null.  One block per (p, w); each thread sums a strided share of the nodes
// in FP64 and the block reduces in a fixed order.
__global__ void fermi_sums_kernel(int64_t n, const double* __restrict__ e,
                                  const double* __restrict__ wt,
                                  const double2* __restrict__ vals, int64_t W,
                                  const double* __restrict__ mu,
                                  const double* __restrict__ temp,
                                  double2* __restrict__ out) {
  const int64_t p = blockIdx.x / W, w = blockIdx.x % W;
  const double m = mu ? mu[p] : 0.0, T = mu ? temp[p] : 0.0;
  double sr = 0.0, si = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    double f = 1.0;
    if (mu) {
      const double d = e[k] - m;
      f = T == 0.0 ? (d < 0.0 ? 1.0 : 0.0) : 1.0 / (1.0 + exp(d / T));
    }
    const double c = wt[k] * f;
    const double2 v = vals[k * W + w];
    sr += c * v.x;
    si += c * v.y;
  }
  __shared__ double rr[256], ri[256];
  rr[threadIdx.x] = sr;
  ri[threadIdx.x] = si;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      rr[threadIdx.x] += rr[threadIdx.x + s];
      ri[threadIdx.x] += ri[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = make_double2(rr[0], ri[0]);
}

namespace kpm {

// Surrogate ensemble DOS, one block per point p: the DOS of member e at
// energy k is d_e(k) = sum_n mem[e][p][n] At[n][k]; out the largest (over
// k) standard deviation over the members (ddof 1) and, with reference
// moments, the largest |mean_e d_e(k) - sum_n ref[p][n] At[n][k]|.  FP64,
// the point's moments staged in shared memory, At read along k
// (coalesced).
constexpr int ENS_MAX = 8;
__global__ void ensemble_dos_kernel(int64_t E, int64_t P, int64_t M,
                                    int64_t K, const double* __restrict__ mem,
                                    const double* __restrict__ At,
                                    const double* __restrict__ ref,
                                    double* __restrict__ spread,
                                    double* __restrict__ err) {
  extern __shared__ double sm[];              // (E + 1) x M
  const int64_t p = blockIdx.x;
  for (int64_t i = threadIdx.x; i < E * M; i += blockDim.x) {
    const int64_t e = i / M, n = i % M;
    sm[i] = mem[(e * P + p) * M + n];
  }
  if (ref)
    for (int64_t n = threadIdx.x; n < M; n += blockDim.x)
      sm[E * M + n] = ref[p * M + n];
  __syncthreads();
  double smax = 0.0, emax = 0.0;
  for (int64_t k = threadIdx.x; k < K; k += blockDim.x) {
    double d[ENS_MAX], dr = 0.0;
    for (int e = 0; e < ENS_MAX; ++e) d[e] = 0.0;
    for (int64_t n = 0; n < M; ++n) {
      const double a = At[n * K + k];
#pragma unroll
      for (int e = 0; e < ENS_MAX; ++e)
        if (e < E) d[e] = fma(sm[e * M + n], a, d[e]);
      if (ref) dr = fma(sm[E * M + n], a, dr);
    }
    double mean = 0.0;
    for (int e = 0; e < E; ++e) mean += d[e];
    mean /= (double)E;
    double var = 0.0;
    for (int e = 0; e < E; ++e) var += (d[e] - mean) * (d[e] - mean);
    if (E > 1) smax = fmax(smax, sqrt(var / (double)(E - 1)));
    if (ref) emax = fmax(emax, fabs(mean - dr));
  }
  __shared__ double rs[256], re[256];
  rs[threadIdx.x] = smax;
  re[threadIdx.x] = emax;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      rs[threadIdx.x] = fmax(rs[threadIdx.x], rs[threadIdx.x + s]);
      re[threadIdx.x] = fmax(re[threadIdx.x], re[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    spread[p] = rs[0];
    if (err) err[p] = re[0];
  }
}

}  // namespace kpm

extern "C" {

int kpm_chebval(int64_t M, int64_t W, const double* coefs, int64_t E,
                const double* x, double* out) {
  KPM_REQUIRE(M > 0 && W > 0 && E >= 0 && coefs && (E == 0 || (x && out)),
              "kpm_chebval: invalid argument");
  if (E == 0) return KPM_OK;
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double2 *dc = nullptr, *dout = nullptr;
  double* dx = nullptr;
  int st = dev_alloc((void**)&dc, (size_t)M * W * sizeof(double2), s);
  if (st == KPM_OK) st = dev_alloc((void**)&dx, (size_t)E * sizeof(double), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&dout, (size_t)E * W * sizeof(double2), s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(dc, coefs, (size_t)M * W * sizeof(double2),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dx, x, (size_t)E * sizeof(double),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      chebval_kernel<<<(unsigned)ceil_div(E * W, 256), 256, 0, s>>>(
          M, W, dc, E, dx, dout);
      count_launch(1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(out, dout, (size_t)E * W * sizeof(double2),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(dc, s);
  dev_free(dx, s);
  dev_free(dout, s);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  return KPM_OK;
}

int kpm_kernel_weights(int64_t M, int kernel, double lorentz_l, double* g) {
  KPM_REQUIRE(M > 0 && g, "kpm_kernel_weights: invalid argument");
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double* d = nullptr;
  KPM_TRY(dev_alloc((void**)&d, M * sizeof(double), s));
  kernel_weights_kernel<<<(unsigned)ceil_div(M, 256), 256, 0, s>>>(
      M, kernel, lorentz_l, d);
  count_launch(1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g, d, M * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  dev_free(d, s);
  KPM_CUDA(e);
  return KPM_OK;
}

int kpm_reconstruct(int64_t R, int64_t M, int64_t W, const double* moments,
                    int mean, int is_real, double a, int kernel,
                    double lorentz_l, const double* nodes, double* gammas_out,
                    double* densities_out) {
  NvtxRange nvtx("kpm_reconstruct");
  KPM_REQUIRE(R > 0 && M > 0 && W > 0 && moments && nodes && a > 0,
              "kpm_reconstruct: invalid argument");
  KPM_REQUIRE(kernel >= KPM_KERNEL_NONE && kernel <= KPM_KERNEL_LORENTZ,
              "kpm_reconstruct: unknown kernel %d", kernel);
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double2* d = nullptr;
  const size_t bytes = (size_t)R * M * W * sizeof(double2);
  KPM_TRY(dev_alloc((void**)&d, bytes, s));
  cudaError_t e = cudaMemcpyAsync(d, moments, bytes, cudaMemcpyHostToDevice,
                                  s);
  int st = KPM_OK;
  if (e == cudaSuccess)
    st = reconstruct_on_device(s, R, M, W, d, mean, is_real, a, kernel,
                               lorentz_l, nodes, gammas_out, densities_out);
  dev_free(d, s);
  cudaStreamSynchronize(s);
  KPM_CUDA(e);
  return st;
}

int kpm_fermi_sums(int64_t n, const double* energies, const double* weights,
                   int64_t W, const double* values, int64_t P,
                   const double* mu, const double* temperature, double* out) {
  NvtxRange nvtx("kpm_fermi_sums");
  KPM_REQUIRE(n > 0 && W > 0 && P > 0 && energies && weights && values &&
                  out && (mu == nullptr) == (temperature == nullptr) &&
                  (mu != nullptr || P == 1),
              "kpm_fermi_sums: invalid argument");
  KPM_REQUIRE(P * W < (int64_t)1 << 31, "kpm_fermi_sums: grid too large");
  for (int64_t p = 0; mu && p < P; ++p)
    KPM_REQUIRE(temperature[p] >= 0.0,
                "kpm_fermi_sums: temperature must be non-negative");
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double *de = nullptr, *dw = nullptr, *dmu = nullptr, *dT = nullptr;
  double2 *dv = nullptr, *dout = nullptr;
  int st = dev_alloc((void**)&de, n * sizeof(double), s);
  if (st == KPM_OK) st = dev_alloc((void**)&dw, n * sizeof(double), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&dv, (size_t)n * W * sizeof(double2), s);
  if (st == KPM_OK && mu) st = dev_alloc((void**)&dmu, P * sizeof(double), s);
  if (st == KPM_OK && mu) st = dev_alloc((void**)&dT, P * sizeof(double), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&dout, (size_t)P * W * sizeof(double2), s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(de, energies, n * sizeof(double),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dw, weights, n * sizeof(double),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dv, values, (size_t)n * W * sizeof(double2),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && mu)
      e = cudaMemcpyAsync(dmu, mu, P * sizeof(double), cudaMemcpyHostToDevice,
                          s);
    if (e == cudaSuccess && mu)
      e = cudaMemcpyAsync(dT, temperature, P * sizeof(double),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      fermi_sums_kernel<<<(unsigned)(P * W), 256, 0, s>>>(n, de, dw, dv, W,
                                                          dmu, dT, dout);
      count_launch(1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(out, dout, (size_t)P * W * sizeof(double2),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(de, s);
  dev_free(dw, s);
  dev_free(dv, s);
  dev_free(dmu, s);
  dev_free(dT, s);
  dev_free(dout, s);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  return KPM_OK;
}


int kpm_ensemble_dos(int64_t E, int64_t P, int64_t M, int64_t K,
                     const double* members, const double* At,
                     const double* ref, double* spread, double* err) {
  NvtxRange nvtx("kpm_ensemble_dos");
  KPM_REQUIRE(E > 0 && E <= kpm::ENS_MAX && P > 0 && M > 0 && K > 0 &&
                  members && At && spread && (err == nullptr || ref),
              "kpm_ensemble_dos: invalid argument");
  KPM_REQUIRE(P < (int64_t)1 << 31 && (E + 1) * M * 8 <= 160 * 1024,
              "kpm_ensemble_dos: sizes too large");
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double *dm = nullptr, *da = nullptr, *dr = nullptr, *ds = nullptr,
         *de = nullptr;
  int st = dev_alloc((void**)&dm, (size_t)E * P * M * 8, s);
  if (st == KPM_OK) st = dev_alloc((void**)&da, (size_t)M * K * 8, s);
  if (st == KPM_OK && ref) st = dev_alloc((void**)&dr, (size_t)P * M * 8, s);
  if (st == KPM_OK) st = dev_alloc((void**)&ds, (size_t)P * 8, s);
  if (st == KPM_OK && err) st = dev_alloc((void**)&de, (size_t)P * 8, s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(dm, members, (size_t)E * P * M * 8,
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(da, At, (size_t)M * K * 8, cudaMemcpyHostToDevice,
                          s);
    if (e == cudaSuccess && ref)
      e = cudaMemcpyAsync(dr, ref, (size_t)P * M * 8, cudaMemcpyHostToDevice,
                          s);
    const size_t smem = (size_t)(E + 1) * M * 8;
    if (e == cudaSuccess && smem > 48 * 1024)
      e = cudaFuncSetAttribute(ensemble_dos_kernel,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    if (e == cudaSuccess) {
      ensemble_dos_kernel<<<(unsigned)P, 256, smem, s>>>(E, P, M, K, dm, da,
                                                        dr, ds, de);
      count_launch(1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(spread, ds, (size_t)P * 8, cudaMemcpyDeviceToHost,
                          s);
    if (e == cudaSuccess && err)
      e = cudaMemcpyAsync(err, de, (size_t)P * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(dm, s);
  dev_free(da, s);
  dev_free(dr, s);
  dev_free(ds, s);
  dev_free(de, s);
  if (st != KPM_OK) return st;
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("kpm_ensemble_dos: %s", cudaGetErrorString(e));
    return KPM_ECUDA;
  }
  return KPM_OK;
}

int kpm_integral_factor(int64_t M, const double* mu, const double* g,
                        const double* nodes, double* factor_out) {
  NvtxRange nvtx("kpm_integral_factor");
  KPM_REQUIRE(M > 0 && mu && g && nodes && factor_out,
              "kpm_integral_factor: invalid argument");
  int dev, sms;
  KPM_TRY(init_device(&dev, &sms));
  cudaStream_t s = 0;
  double2 *dmu = nullptr, *dout = nullptr;
  double *dg = nullptr, *dn = nullptr;
  int st = dev_alloc((void**)&dmu, (size_t)M * M * sizeof(double2), s);
  if (st == KPM_OK) st = dev_alloc((void**)&dg, M * sizeof(double), s);
  if (st == KPM_OK) st = dev_alloc((void**)&dn, 2 * M * sizeof(double), s);
  if (st == KPM_OK)
    st = dev_alloc((void**)&dout, 2 * M * sizeof(double2), s);
  cudaError_t e = cudaSuccess;
  if (st == KPM_OK) {
    e = cudaMemcpyAsync(dmu, mu, (size_t)M * M * sizeof(double2),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dg, g, M * sizeof(double), cudaMemcpyHostToDevice,
                          s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dn, nodes, 2 * M * sizeof(double),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      const int threads = 256;
      const size_t shm = (3 * M + 2 * threads) * sizeof(double);
      if (shm > 48 * 1024)
        e = cudaFuncSetAttribute(integral_factor_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)shm);
      if (e == cudaSuccess) {
        integral_factor_kernel<<<(unsigned)(2 * M), threads, shm, s>>>(
            M, dmu, dg, dn, dout);
        count_launch(1);
        e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(factor_out, dout, 2 * M * sizeof(double2),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  dev_free(dmu, s);
  dev_free(dg, s);
  dev_free(dn, s);
  dev_free(dout, s);
  if (st != KPM_OK) return st;
  KPM_CUDA(e);
  return KPM_OK;
}

int kpm_dos(const kpm_csr_desc* ham, double a, double b, int precision,
            const double* vecs, int64_t R, int64_t M, int kernel,
            double* moments_out, double* gammas_out, double* densities_out) {
  NvtxRange nvtx("kpm_dos");
  KPM_REQUIRE(ham && vecs && R > 0 && M >= 2, "kpm_dos: invalid argument");
  KPM_REQUIRE(ham->rows > 0, "kpm_dos: invalid CSR descriptor");
  // Copy the vectors to the device on a stream of their own first, so that
  // the copy overlaps the handle set-up (the RCM order is computed on the
  // host); the handle's stream waits for it before the block uses it.
  const size_t vbytes = (size_t)R * ham->rows * 16;
  cudaStream_t vs = nullptr;
  cudaEvent_t vdone = nullptr;
  void* vstage = nullptr;
  if (cudaStreamCreateWithFlags(&vs, cudaStreamNonBlocking) == cudaSuccess &&
      cudaEventCreateWithFlags(&vdone, cudaEventDisableTiming) ==
          cudaSuccess &&
      cudaMallocAsync(&vstage, vbytes, vs) == cudaSuccess &&
      cudaMemcpyAsync(vstage, vecs, vbytes, cudaMemcpyHostToDevice, vs) ==
          cudaSuccess &&
      cudaEventRecord(vdone, vs) == cudaSuccess) {
  } else {
    cudaGetLastError();
    if (vstage) cudaFreeAsync(vstage, vs);
    vstage = nullptr;                   // the block copies them itself
  }
  kpm_handle* h = nullptr;
  // the mixed-precision one-shot path stores the Hamiltonian in RCM order
  int cst = kpm_create_ex(ham, a, b, precision,
                          precision == KPM_PREC_MIXED ? KPM_FLAG_REORDER : 0,
                          &h);
  if (cst == KPM_OK && vstage &&
      cudaStreamWaitEvent(h->stream, vdone, 0) == cudaSuccess) {
    h->vec_staging = vstage;            // freed by the upload or the handle
    h->vec_staging_src = vecs;
    h->vec_staging_bytes = vbytes;
    vstage = nullptr;
  }
  if (vstage) cudaFreeAsync(vstage, vs);
  if (vdone) cudaEventDestroy(vdone);
  if (vs) cudaStreamDestroy(vs);
  if (cst != KPM_OK) return cst;
  kpm_block* blk = nullptr;
  int st = kpm_block_create(h, vecs, R, 0, &blk);
  double* mom = nullptr;
  if (st == KPM_OK) {
    mom = moments_out ? moments_out : new double[2 * R * M];
    st = kpm_block_dos_moments(blk, 0, M, mom);
  }
  // a diverged recursion still returns its moments and densities
  const bool diverged = st == KPM_EDIVERGED;
  std::string diverged_msg = diverged ? last_error() : "";
  if (diverged) st = KPM_OK;
  if (st == KPM_OK && (gammas_out || densities_out)) {
    // real_if_close(tol=100): real when every |imag| < 100 * eps
    double mx = 0.0;
    for (int64_t i = 0; i < R * M; ++i) mx = fmax(mx, fabs(mom[2 * i + 1]));
    const int is_real = mx < 100.0 * 2.220446049250313e-16;
    double* nodes = new double[2 * M];
    // _chebyshev_nodes (kwant/kpm.py:1190-1194)
    const int64_t K = 2 * M;
    const double step = -M_PI / (double)K;
    for (int64_t k = 0; k < K; ++k)
      nodes[k] = cos((M_PI + (double)k * step) + step / 2);
    double2* dmom = nullptr;
    st = dev_alloc((void**)&dmom, (size_t)R * M * sizeof(double2), h->stream);
    if (st == KPM_OK) {
      cudaError_t e = cudaMemcpyAsync(dmom, mom, (size_t)R * M * 16,
                                      cudaMemcpyHostToDevice, h->stream);
      if (e != cudaSuccess) {
        set_error("kpm_dos: %s", cudaGetErrorString(e));
        st = KPM_ECUDA;
      } else {
        st = reconstruct_on_device(h->stream, R, M, 1, dmom, 1, is_real, a,
                                   kernel, 4.0, nodes, gammas_out,
                                   densities_out);
      }
      dev_free(dmom, h->stream);
    }
    delete[] nodes;
  }
  if (mom && mom != moments_out) delete[] mom;
  kpm_block_destroy(blk);
  kpm_destroy(h);
  if (st == KPM_OK && diverged) {
    set_error("kpm_dos: %s", diverged_msg.c_str());
    return KPM_EDIVERGED;
  }
  return st;
}

}  // extern "C"
