// Locality reordering of the Hamiltonian (host side).
//
// Kwant numbers sites by family, then tag (kwant/builder.py:2178), so the
// two sublattices of a honeycomb flake are N/2 rows apart and every row's
// neighbours live in the other half of the vector block: during a step each
// vector row is then fetched from HBM twice (once as a row, once as a
// neighbour).  A reverse Cuthill-McKee (RCM) order of the sparsity pattern
// keeps the neighbours of a row within a band of about the lattice width,
// which a step's working window holds in L2.
//
// Only the order itself is computed on the host.  The matrix rows are
// moved and the vectors permuted on the device (at upload and download);
// the entry order inside each row is kept, so every row sum is evaluated in
// the caller's order.

#include <algorithm>
#include <numeric>
#include <vector>

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

namespace kpm {

// perm[new] = old
void rcm_order(int64_t n, const int32_t* indptr, const int32_t* indices,
               std::vector<int32_t>& perm) {
  std::vector<int32_t> deg(n);
  for (int64_t i = 0; i < n; ++i) deg[i] = indptr[i + 1] - indptr[i];
  // nodes by ascending degree (counting sort) to pick component seeds
  int32_t maxd = 0;
  for (int64_t i = 0; i < n; ++i) maxd = std::max(maxd, deg[i]);
  std::vector<int64_t> cnt(maxd + 2, 0);
  for (int64_t i = 0; i < n; ++i) cnt[deg[i] + 1]++;
  for (int32_t d = 0; d <= maxd; ++d) cnt[d + 1] += cnt[d];
  std::vector<int32_t> by_deg(n);
  for (int64_t i = 0; i < n; ++i) by_deg[cnt[deg[i]]++] = (int32_t)i;

  std::vector<char> seen(n, 0);
  perm.clear();
  perm.reserve(n);
  std::vector<int32_t> nb;
  int64_t seed_pos = 0;
  while ((int64_t)perm.size() < n) {
    while (seen[by_deg[seed_pos]]) ++seed_pos;
    const int32_t seed = by_deg[seed_pos];
    size_t head = perm.size();
    perm.push_back(seed);
    seen[seed] = 1;
    while (head < perm.size()) {
      const int32_t u = perm[head++];
      nb.clear();
      for (int32_t k = indptr[u]; k < indptr[u + 1]; ++k) {
        const int32_t v = indices[k];
        if (!seen[v]) {
          seen[v] = 1;
          nb.push_back(v);
        }
      }
      std::sort(nb.begin(), nb.end(), [&](int32_t p, int32_t q) {
        return deg[p] < deg[q] || (deg[p] == deg[q] && p < q);
      });
      perm.insert(perm.end(), nb.begin(), nb.end());
    }
  }
  std::reverse(perm.begin(), perm.end());
}

int upload_matrix_for(kpm_handle* h, const kpm_csr_desc* m, double scale,
                      Matrix* out, bool with_ell) {
  if (!h->perm) return upload_matrix(h, m, scale, out, with_ell);
  KPM_REQUIRE(m->rows == (int64_t)h->h_iperm.size(),
              "matrix size does not match the handle");
  KPM_TRY(validate_csr(m));
  std::vector<int32_t> perm(m->rows);
  for (int64_t o = 0; o < m->rows; ++o) perm[h->h_iperm[o]] = (int32_t)o;
  return upload_matrix_perm(h, m, scale, out, with_ell, perm.data(),
                            h->h_iperm.data(), false);
}

int setup_reorder(kpm_handle* h, const kpm_csr_desc* m,
                  std::vector<int32_t>& perm) {
  rcm_order(m->rows, m->indptr, m->indices, perm);
  h->h_iperm.assign(m->rows, 0);
  for (int64_t p = 0; p < m->rows; ++p) h->h_iperm[perm[p]] = (int32_t)p;
  KPM_TRY(dev_alloc((void**)&h->perm, m->rows * sizeof(int32_t), h->stream));
  KPM_CUDA(cudaMemcpyAsync(h->perm, perm.data(), m->rows * sizeof(int32_t),
                           cudaMemcpyHostToDevice, h->stream));
  KPM_CUDA(cudaStreamSynchronize(h->stream));
  return KPM_OK;
}

}  // namespace kpm
