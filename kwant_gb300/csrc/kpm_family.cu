// Parametric Hamiltonian family on a fixed sparsity structure:
//   H(phi, s1, s2) = B .* exp(i phi Theta) + s1 D1 + s2 D2.
// The four coefficient matrices stay resident in HBM (CSR order of the
// handle, reordering applied); a sweep point rewrites the handle's matrix
// values in place with one kernel instead of re-assembling and re-uploading
// the Hamiltonian (the reference re-runs hamiltonian_submatrix,
// kwant/_system.pyx:233-338, for every params value).

#include <vector>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {
namespace {

__global__ void same_structure_kernel(const int32_t* __restrict__ a,
                                      const int32_t* __restrict__ b,
                                      int64_t n, int* __restrict__ diff) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && a[i] != b[i]) atomicExch(diff, 1);
}

// One thread per row: value of every CSR entry at the point, written as raw
// complex128 (FP64 handles) or as complex64 values * scale into the CSR
// array and, when present, the ELL copy (entry q of row i at i * ell_k + q).
template <bool MIXED>
__global__ void family_point_kernel(
    int64_t rows, const int32_t* __restrict__ indptr,
    const double2* __restrict__ base, const double2* __restrict__ theta,
    const double2* __restrict__ d1, const double2* __restrict__ d2,
    double phi, double s1, double s2, double scale, void* __restrict__ data,
    int ell_k, float2* __restrict__ ell_val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const int32_t k0 = indptr[i], k1 = indptr[i + 1];
  for (int32_t k = k0; k < k1; ++k) {
    double sn, cs;
    sincos(phi * theta[k].x, &sn, &cs);
    const double2 bk = base[k], a1 = d1[k], a2 = d2[k];
    double2 v;
    v.x = bk.x * cs - bk.y * sn + s1 * a1.x + s2 * a2.x;
    v.y = bk.x * sn + bk.y * cs + s1 * a1.y + s2 * a2.y;
    if (MIXED) {
      const float2 f = make_float2((float)(v.x * scale), (float)(v.y * scale));
      static_cast<float2*>(data)[k] = f;
      if (ell_val) ell_val[i * ell_k + (k - k0)] = f;
    } else {
      static_cast<double2*>(data)[k] = v;
    }
  }
}

// Upload one coefficient matrix in the handle's order and check that its
// structure is the handle's; on success *out owns the complex128 values.
int upload_channel(kpm_handle* h, const kpm_csr_desc* m, double2** out,
                   int* diff) {
  KPM_REQUIRE(m && m->rows == h->H.rows && m->nnz == h->H.nnz,
              "kpm_family_set: matrix size differs from the handle's");
  Matrix t;
  int st = upload_matrix_for(h, m, 0.0, &t, false);
  if (st == KPM_OK && m->nnz > 0) {
    same_structure_kernel<<<(unsigned)ceil_div(m->nnz, 256), 256, 0,
                            h->stream>>>(t.indices, h->H.indices, m->nnz,
                                         diff);
    same_structure_kernel<<<(unsigned)ceil_div(m->rows + 1, 256), 256, 0,
                            h->stream>>>(t.indptr, h->H.indptr, m->rows + 1,
                                         diff);
    count_launch(2);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("kpm_family_set: structure check launch failed");
      st = KPM_ECUDA;
    }
  }
  if (st == KPM_OK) {
    *out = static_cast<double2*>(t.data);
    t.data = nullptr;
  }
  free_matrix(&t, h->stream);
  return st;
}

}  // namespace

void free_family(kpm_handle* h) {
  dev_free(h->fam_base, h->stream);
  dev_free(h->fam_theta, h->stream);
  dev_free(h->fam_d1, h->stream);
  dev_free(h->fam_d2, h->stream);
  h->fam_base = h->fam_theta = h->fam_d1 = h->fam_d2 = nullptr;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_family_set(kpm_handle* h, const kpm_csr_desc* base,
                   const kpm_csr_desc* theta, const kpm_csr_desc* d1,
                   const kpm_csr_desc* d2) {
  KPM_REQUIRE(h && base && theta && d1 && d2, "kpm_family_set: null argument");
  KPM_REQUIRE(theta->nnz == 0 || theta->data, "kpm_family_set: null data");
  for (int64_t k = 0; k < theta->nnz; ++k)
    KPM_REQUIRE(theta->data[2 * k + 1] == 0.0,
                "kpm_family_set: Theta must be real");
  free_family(h);
  int* diff = nullptr;
  KPM_TRY(dev_alloc((void**)&diff, sizeof(int), h->stream));
  int st = cudaMemsetAsync(diff, 0, sizeof(int), h->stream) == cudaSuccess
               ? KPM_OK
               : KPM_ECUDA;
  double2* ch[4] = {nullptr, nullptr, nullptr, nullptr};
  const kpm_csr_desc* src[4] = {base, theta, d1, d2};
  for (int c = 0; c < 4 && st == KPM_OK; ++c)
    st = upload_channel(h, src[c], &ch[c], diff);
  int hdiff = 0;
  if (st == KPM_OK &&
      (cudaMemcpyAsync(&hdiff, diff, sizeof(int), cudaMemcpyDeviceToHost,
                       h->stream) != cudaSuccess ||
       cudaStreamSynchronize(h->stream) != cudaSuccess)) {
    set_error("kpm_family_set: structure check failed to run");
    st = KPM_ECUDA;
  }
  if (st == KPM_OK && hdiff) {
    set_error("kpm_family_set: matrix structure differs from the handle's");
    st = KPM_EINVAL;
  }
  dev_free(diff, h->stream);
  if (st != KPM_OK) {
    for (auto* p : ch) dev_free(p, h->stream);
    return st;
  }
  h->fam_base = ch[0];
  h->fam_theta = ch[1];
  h->fam_d1 = ch[2];
  h->fam_d2 = ch[3];
  return KPM_OK;
}

int kpm_family_point(kpm_handle* h, double phi, double s1, double s2) {
  KPM_REQUIRE(h, "kpm_family_point: null handle");
  KPM_REQUIRE(h->fam_base, "kpm_family_point: no family set on the handle");
  KPM_REQUIRE(std::isfinite(phi) && std::isfinite(s1) && std::isfinite(s2),
              "kpm_family_point: parameters must be finite");
  const Matrix& H = h->H;
  if (H.rows == 0 || H.nnz == 0) return KPM_OK;
  const unsigned grid = (unsigned)ceil_div(H.rows, 256);
  if (h->precision == KPM_PREC_MIXED)
    family_point_kernel<true><<<grid, 256, 0, h->stream>>>(
        H.rows, H.indptr, h->fam_base, h->fam_theta, h->fam_d1, h->fam_d2,
        phi, s1, s2, 2.0 / h->a, H.data, H.ell_k, H.ell_val);
  else
    family_point_kernel<false><<<grid, 256, 0, h->stream>>>(
        H.rows, H.indptr, h->fam_base, h->fam_theta, h->fam_d1, h->fam_d2,
        phi, s1, s2, 0.0, H.data, 0, nullptr);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

}  // extern "C"
