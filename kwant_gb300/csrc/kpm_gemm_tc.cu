// Tensor-core (tcgen05) split-BF16 contraction of the correlator moments
// matrix.  Placeholder dispatch: the CUDA-core evaluation of the same BF16x3
// products is used until the tcgen05 kernel is enabled.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"
#include "kpm_gemm.cuh"

namespace kpm {

int gemm_bf16x3(kpm_handle* h, const Store* omega, const Store* psi,
                int64_t M, int64_t K, int64_t R, double* mu_host) {
  return gemm_bf16x3_simt(h, omega, psi, M, K, R, mu_host);
}

}  // namespace kpm
