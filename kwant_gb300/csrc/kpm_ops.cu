// Local-operator moments on the device.
//
// Every operator of the KPM path is a sesquilinear map q_w(bra, ket):
// Density MAT_ELS (kwant/operator.pyx:785-807), Current MAT_ELS
// (kwant/operator.pyx:977-987), a matrix operator vdot(bra, O ket)
// (kwant/kpm.py:195).  The host lowers each one to "terms" (see
// include/kwant_gb300.h, kpm_op_desc): the bra-side factor of each term,
// coef_t = sum_e conj(v_e) bra[col_e], depends only on the starting vector
// alpha_0, so it is computed once per vector block; every Chebyshev step then
// only gathers
//     q_w(alpha_0, alpha_n) = sum_{t in w} conj(coef_t) alpha_n[row_t]
// for all R vectors at once (rows are [row][vector], so the gather reads
// contiguous 16-byte payloads).  Accumulation is FP64 in term order.

#include "kpm_common.cuh"
#include "kpm_internal.cuh"

struct kpm_op {
  kpm_handle* h = nullptr;
  int64_t T = 0, W = 0, C = 0, E = 0;
  int32_t* term_row = nullptr;
  int64_t* bra_ptr = nullptr;
  int32_t* bra_col = nullptr;
  double2* bra_val = nullptr;
  int64_t* chunk_ptr = nullptr;
  int64_t* out_chunk_ptr = nullptr;  // W + 1 (chunks of each output)
  bool direct = false;               // one chunk per output, in order
  int real0 = 0;
};

namespace kpm {

template <bool MIXED>
__global__ void op_coef_kernel(int64_t T, const int64_t* __restrict__ bra_ptr,
                               const int32_t* __restrict__ bra_col,
                               const double2* __restrict__ bra_val,
                               const void* __restrict__ a0, int64_t rp,
                               int64_t Rpad, double2* __restrict__ coef) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * rp) return;
  const int64_t t = idx / rp, l = idx % rp;
  const int64_t e0 = bra_ptr[t], e1 = bra_ptr[t + 1];
  if constexpr (MIXED) {
    const float4* A = reinterpret_cast<const float4*>(a0);
    double r0 = 0, i0 = 0, r1 = 0, i1 = 0;
    for (int64_t e = e0; e < e1; ++e) {
      const double2 v = bra_val[e];
      const float4 x = A[(int64_t)bra_col[e] * rp + l];
      // conj(v) * x
      r0 += v.x * x.x + v.y * x.y;
      i0 += v.x * x.y - v.y * x.x;
      r1 += v.x * x.z + v.y * x.w;
      i1 += v.x * x.w - v.y * x.z;
    }
    coef[t * Rpad + 2 * l] = make_double2(r0, i0);
    coef[t * Rpad + 2 * l + 1] = make_double2(r1, i1);
  } else {
    const double2* A = reinterpret_cast<const double2*>(a0);
    double r0 = 0, i0 = 0;
    for (int64_t e = e0; e < e1; ++e) {
      const double2 v = bra_val[e];
      const double2 x = A[(int64_t)bra_col[e] * rp + l];
      r0 += v.x * x.x + v.y * x.y;
      i0 += v.x * x.y - v.y * x.x;
    }
    coef[t * Rpad + l] = make_double2(r0, i0);
  }
}

// out[c][v] = sum_{t in chunk c} conj(coef[t][v]) * alpha[row_t][v]
template <bool MIXED>
__global__ void op_gather_kernel(int64_t C,
                                 const int64_t* __restrict__ chunk_ptr,
                                 const int32_t* __restrict__ term_row,
                                 const double2* __restrict__ coef,
                                 const void* __restrict__ alpha, int64_t rp,
                                 int64_t Rpad, double2* __restrict__ out,
                                 int real_part) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= C * rp) return;
  const int64_t c = idx / rp, l = idx % rp;
  const int64_t t0 = chunk_ptr[c], t1 = chunk_ptr[c + 1];
  if constexpr (MIXED) {
    const float4* A = reinterpret_cast<const float4*>(alpha);
    double r0 = 0, i0 = 0, r1 = 0, i1 = 0;
    for (int64_t t = t0; t < t1; ++t) {
      const float4 x = A[(int64_t)term_row[t] * rp + l];
      const double2 k0 = coef[t * Rpad + 2 * l];
      const double2 k1 = coef[t * Rpad + 2 * l + 1];
      r0 += k0.x * x.x + k0.y * x.y;
      i0 += k0.x * x.y - k0.y * x.x;
      r1 += k1.x * x.z + k1.y * x.w;
      i1 += k1.x * x.w - k1.y * x.z;
    }
    if (real_part) i0 = i1 = 0.0;
    out[c * Rpad + 2 * l] = make_double2(r0, i0);
    out[c * Rpad + 2 * l + 1] = make_double2(r1, i1);
  } else {
    const double2* A = reinterpret_cast<const double2*>(alpha);
    double r0 = 0, i0 = 0;
    for (int64_t t = t0; t < t1; ++t) {
      const double2 x = A[(int64_t)term_row[t] * rp + l];
      const double2 k = coef[t * Rpad + l];
      r0 += k.x * x.x + k.y * x.y;
      i0 += k.x * x.y - k.y * x.x;
    }
    if (real_part) i0 = 0.0;
    out[c * Rpad + l] = make_double2(r0, i0);
  }
}

// out[w][v] = sum over the chunks of output w, fixed tree order.
__global__ void op_combine_kernel(const int64_t* __restrict__ out_chunk_ptr,
                                  const double2* __restrict__ part,
                                  int64_t Rpad, double2* __restrict__ out,
                                  int real_part) {
  const int64_t w = blockIdx.x, v = blockIdx.y;
  const int64_t c0 = out_chunk_ptr[w], c1 = out_chunk_ptr[w + 1];
  __shared__ double sr[128], si[128];
  double r = 0.0, i = 0.0;
  for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
    const double2 p = part[c * Rpad + v];
    r += p.x;
    i += p.y;
  }
  sr[threadIdx.x] = r;
  si[threadIdx.x] = i;
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    out[w * Rpad + v] = make_double2(sr[0], real_part ? 0.0 : si[0]);
}

static int op_coef(kpm_op* op, const void* a0, int64_t Rpad, double2* coef) {
  kpm_handle* h = op->h;
  const bool mixed = h->precision == KPM_PREC_MIXED;
  const int64_t rp = Rpad / (mixed ? 2 : 1);
  const int64_t n = op->T * rp;
  if (n == 0) return KPM_OK;
  if (mixed)
    op_coef_kernel<true><<<(unsigned)ceil_div(n, 256), 256, 0, h->stream>>>(
        op->T, op->bra_ptr, op->bra_col, op->bra_val, a0, rp, Rpad, coef);
  else
    op_coef_kernel<false><<<(unsigned)ceil_div(n, 256), 256, 0, h->stream>>>(
        op->T, op->bra_ptr, op->bra_col, op->bra_val, a0, rp, Rpad, coef);
  count_launch(1);
  KPM_CHECK_LAUNCH();
  return KPM_OK;
}

// Evaluate the operator against alpha for all vectors into out [W][Rpad].
static int op_eval(kpm_op* op, const double2* coef, const void* alpha,
                   int64_t Rpad, double2* part, double2* out, int real_part) {
  kpm_handle* h = op->h;
  const bool mixed = h->precision == KPM_PREC_MIXED;
  const int64_t rp = Rpad / (mixed ? 2 : 1);
  double2* dst = op->direct ? out : part;
  const int64_t n = op->C * rp;
  if (n > 0) {
    if (mixed)
      op_gather_kernel<true><<<(unsigned)ceil_div(n, 256), 256, 0,
                               h->stream>>>(op->C, op->chunk_ptr,
                                            op->term_row, coef, alpha, rp,
                                            Rpad, dst, real_part);
    else
      op_gather_kernel<false><<<(unsigned)ceil_div(n, 256), 256, 0,
                                h->stream>>>(op->C, op->chunk_ptr,
                                             op->term_row, coef, alpha, rp,
                                             Rpad, dst, real_part);
    count_launch(1);
    KPM_CHECK_LAUNCH();
  }
  if (!op->direct) {
    dim3 grid((unsigned)op->W, (unsigned)Rpad);
    op_combine_kernel<<<grid, 128, 0, h->stream>>>(op->out_chunk_ptr, part,
                                                   Rpad, out, real_part);
    count_launch(1);
    KPM_CHECK_LAUNCH();
  }
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_op_create(kpm_handle* h, const kpm_op_desc* d, kpm_op** out) {
  KPM_REQUIRE(h && d && out, "kpm_op_create: null argument");
  KPM_REQUIRE(d->num_terms >= 0 && d->num_outputs > 0 && d->num_chunks >= 0,
              "kpm_op_create: invalid sizes");
  KPM_REQUIRE(d->num_outputs < INT32_MAX, "kpm_op_create: too many outputs");
  const int64_t T = d->num_terms, C = d->num_chunks, W = d->num_outputs;
  KPM_REQUIRE(T == 0 || (d->term_row && d->bra_ptr && d->chunk_ptr &&
                         d->chunk_out),
              "kpm_op_create: missing arrays");
  const int64_t E = T ? d->bra_ptr[T] : 0;
  // validate on the host: indices in range, chunks sorted by output
  for (int64_t t = 0; t < T; ++t) {
    KPM_REQUIRE(d->term_row[t] >= 0 && d->term_row[t] < h->H.rows,
                "kpm_op_create: term %lld row out of range", (long long)t);
    KPM_REQUIRE(d->bra_ptr[t] <= d->bra_ptr[t + 1],
                "kpm_op_create: bra_ptr not monotone");
  }
  for (int64_t e = 0; e < E; ++e)
    KPM_REQUIRE(d->bra_col[e] >= 0 && d->bra_col[e] < h->H.rows,
                "kpm_op_create: bra column out of range");
  KPM_REQUIRE(C == 0 || (d->chunk_ptr[0] == 0 && d->chunk_ptr[C] == T),
              "kpm_op_create: chunk_ptr must span all terms");
  std::vector<int64_t> ocp(W + 1, 0);
  bool direct = (C == W);
  for (int64_t c = 0; c < C; ++c) {
    KPM_REQUIRE(d->chunk_ptr[c] <= d->chunk_ptr[c + 1],
                "kpm_op_create: chunk_ptr not monotone");
    KPM_REQUIRE(d->chunk_out[c] >= 0 && d->chunk_out[c] < W,
                "kpm_op_create: chunk output out of range");
    KPM_REQUIRE(c == 0 || d->chunk_out[c] >= d->chunk_out[c - 1],
                "kpm_op_create: chunks must be sorted by output");
    if (d->chunk_out[c] != c) direct = false;
    ocp[d->chunk_out[c] + 1] += 1;
  }
  for (int64_t w = 0; w < W; ++w) ocp[w + 1] += ocp[w];

  auto* op = new kpm_op();
  op->h = h;
  op->T = T;
  op->W = W;
  op->C = C;
  op->E = E;
  op->direct = direct;
  op->real0 = d->real0;
  cudaStream_t s = h->stream;
  int st = KPM_OK;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (st != KPM_OK) return;
    st = dev_alloc(dst, bytes ? bytes : 8, s);
    if (st == KPM_OK && bytes) {
      cudaError_t e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice,
                                      s);
      if (e != cudaSuccess) {
        set_error("kpm_op_create: %s", cudaGetErrorString(e));
        st = KPM_ECUDA;
      }
    }
  };
  // reordered handles: map orbital indices to the device row order
  std::vector<int32_t> rows_m, cols_m;
  const int32_t* trow = d->term_row;
  const int32_t* bcol = d->bra_col;
  if (h->perm) {
    rows_m.resize(T);
    cols_m.resize(E);
    for (int64_t t = 0; t < T; ++t) rows_m[t] = h->h_iperm[d->term_row[t]];
    for (int64_t e = 0; e < E; ++e) cols_m[e] = h->h_iperm[d->bra_col[e]];
    trow = rows_m.data();
    bcol = cols_m.data();
  }
  up((void**)&op->term_row, trow, T * sizeof(int32_t));
  up((void**)&op->bra_ptr, d->bra_ptr, T ? (T + 1) * sizeof(int64_t) : 0);
  up((void**)&op->bra_col, bcol, E * sizeof(int32_t));
  up((void**)&op->bra_val, d->bra_val, E * sizeof(double2));
  up((void**)&op->chunk_ptr, d->chunk_ptr, C ? (C + 1) * sizeof(int64_t) : 0);
  up((void**)&op->out_chunk_ptr, ocp.data(), (W + 1) * sizeof(int64_t));
  if (st == KPM_OK && cudaStreamSynchronize(s) != cudaSuccess) {
    set_error("kpm_op_create: upload failed");
    st = KPM_ECUDA;
  }
  if (st != KPM_OK) {
    kpm_op_destroy(op);
    return st;
  }
  *out = op;
  return KPM_OK;
}

int kpm_op_destroy(kpm_op* op) {
  if (!op) return KPM_OK;
  cudaStream_t s = op->h->stream;
  dev_free(op->term_row, s);
  dev_free(op->bra_ptr, s);
  dev_free(op->bra_col, s);
  dev_free(op->bra_val, s);
  dev_free(op->chunk_ptr, s);
  dev_free(op->out_chunk_ptr, s);
  cudaStreamSynchronize(s);
  cudaGetLastError();
  delete op;
  return KPM_OK;
}

int kpm_block_op_moments(kpm_block* b, kpm_op* op, int64_t m_start,
                         int64_t m_end, double* out) {
  NvtxRange nvtx("kpm_block_op_moments");
  KPM_REQUIRE(b && op && out, "kpm_block_op_moments: null argument");
  KPM_REQUIRE(op->h == b->h, "kpm_block_op_moments: operator of another "
              "handle");
  KPM_REQUIRE(m_end >= 2 && m_start >= 0 && m_start < m_end,
              "kpm_block_op_moments: need 0 <= m_start < m_end, m_end >= 2");
  KPM_REQUIRE(b->keep_a0, "kpm_block_op_moments: block needs keep_a0");
  kpm_handle* h = b->h;
  if (m_start == 0) {
    if (b->steps_done != 0) {
      set_error("kpm_block_op_moments: block already advanced; rewind it");
      return KPM_ESTATE;
    }
  } else if (b->mode != 1 || b->steps_done != m_start - 1 ||
             (b->op_tag != nullptr && b->op_tag != (const void*)op)) {
    // (a block restored from a checkpoint has no operator yet: its bra
    // factors are recomputed below from a0)
    set_error("kpm_block_op_moments: cannot resume at moment %lld",
              (long long)m_start);
    return KPM_ESTATE;
  }
  b->mode = 1;
  const int64_t count = m_end - m_start, W = op->W;
  double2 *mom = nullptr, *part = nullptr;
  int st = dev_alloc((void**)&mom, (size_t)count * W * b->Rpad * 16,
                     h->stream);
  if (st == KPM_OK && !op->direct)
    st = dev_alloc((void**)&part, (size_t)op->C * b->Rpad * 16, h->stream);
  if (st == KPM_OK && (m_start == 0 || b->op_coef == nullptr)) {
    dev_free(b->op_coef, h->stream);
    b->op_coef = nullptr;
    st = dev_alloc((void**)&b->op_coef,
                   (size_t)(op->T ? op->T : 1) * b->Rpad * 16, h->stream);
    if (st == KPM_OK) st = op_coef(op, b->a0, b->Rpad, (double2*)b->op_coef);
    b->op_tag = op;
  }
  if (st == KPM_OK) st = timed_begin(h);
  if (st == KPM_OK && m_start == 0) {
    // mu_0 = op(a0, a0) (real part when Hermitian, bra is ket)
    st = op_eval(op, (double2*)b->op_coef, b->a0, b->Rpad, part, mom,
                 op->real0);
    if (st == KPM_OK) st = block_advance(b, false);
    if (st == KPM_OK && m_end > 1)
      st = op_eval(op, (double2*)b->op_coef, b->p_cur, b->Rpad, part,
                   mom + (size_t)W * b->Rpad, 0);
  }
  for (int64_t n = (m_start > 2 ? m_start : 2); st == KPM_OK && n < m_end;
       ++n) {
    st = block_advance(b, false);
    if (st == KPM_OK)
      st = op_eval(op, (double2*)b->op_coef, b->p_cur, b->Rpad, part,
                   mom + (size_t)(n - m_start) * W * b->Rpad, 0);
  }
  if (st == KPM_OK) st = timed_end(h);
  if (st == KPM_OK) st = moments_to_host(h, mom, count, b->R, b->Rpad, W, out);
  dev_free(mom, h->stream);
  dev_free(part, h->stream);
  if (st == KPM_OK) st = check_bounds(h, "kpm_block_op_moments");
  return st;
}

int kpm_op_apply(kpm_op* op, const double* bra, const double* ket,
                 double* out) {
  KPM_REQUIRE(op && bra && ket && out, "kpm_op_apply: null argument");
  kpm_handle* h = op->h;
  const int64_t N = h->H.rows;
  const int64_t Rpad = group_size(h->precision);
  const size_t csz = h->precision == KPM_PREC_MIXED ? 8 : 16;
  void *dbra = nullptr, *dket = nullptr;
  double2 *coef = nullptr, *part = nullptr, *res = nullptr;
  int st = dev_alloc(&dbra, N * Rpad * csz, h->stream);
  if (st == KPM_OK) st = dev_alloc(&dket, N * Rpad * csz, h->stream);
  if (st == KPM_OK)
    st = dev_alloc((void**)&coef, (op->T ? op->T : 1) * Rpad * 16, h->stream);
  if (st == KPM_OK && !op->direct)
    st = dev_alloc((void**)&part, op->C * Rpad * 16, h->stream);
  if (st == KPM_OK) st = dev_alloc((void**)&res, op->W * Rpad * 16, h->stream);
  if (st == KPM_OK) st = upload_vectors(h, bra, 1, N, Rpad, dbra);
  if (st == KPM_OK) st = upload_vectors(h, ket, 1, N, Rpad, dket);
  if (st == KPM_OK) st = op_coef(op, dbra, Rpad, coef);
  if (st == KPM_OK) st = op_eval(op, coef, dket, Rpad, part, res, 0);
  if (st == KPM_OK) st = moments_to_host(h, res, 1, 1, Rpad, op->W, out);
  dev_free(dbra, h->stream);
  dev_free(dket, h->stream);
  dev_free(coef, h->stream);
  dev_free(part, h->stream);
  dev_free(res, h->stream);
  return st;
}

}  // extern "C"
