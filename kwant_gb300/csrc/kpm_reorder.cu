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

  // breadth-first from each component's lowest-degree node; the unseen
  // neighbours of a node are appended in (degree, index) order, sorted in
  // place by insertion (rows are short)
  std::vector<char> seen(n, 0);
  perm.assign(n, 0);
  auto before = [&](int32_t p, int32_t q) {
    return deg[p] < deg[q] || (deg[p] == deg[q] && p < q);
  };
  int64_t tail = 0, seed_pos = 0;
  while (tail < n) {
    while (seen[by_deg[seed_pos]]) ++seed_pos;
    const int32_t seed = by_deg[seed_pos];
    int64_t head = tail;
    perm[tail++] = seed;
    seen[seed] = 1;
    while (head < tail) {
      const int32_t u = perm[head++];
      const int64_t first = tail;
      for (int32_t k = indptr[u]; k < indptr[u + 1]; ++k) {
        const int32_t v = indices[k];
        if (seen[v]) continue;
        seen[v] = 1;
        int64_t j = tail++;
        while (j > first && before(v, perm[j - 1])) {
          perm[j] = perm[j - 1];
          --j;
        }
        perm[j] = v;
      }
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
