// Device build of the bilinear alpha x beta determinant index.
//
// Mirrors the providers of src/Determinants/spindeterminants.irp.f:
//   psi_det_alpha_unique / _beta_unique          :56-136
//   psi_bilinear_matrix_rows/_columns/_order     :387-445  (beta-major)
//   psi_bilinear_matrix_columns_loc              :465-494
//   psi_bilinear_matrix_transp_*  (alpha-major)  :496-555
//   psi_bilinear_matrix_transp_rows_loc          :557-578
//   singles_alpha_csc (singles among unique strings) :843-915
// Unique strings are ordered by their bit pattern (a 64*N_int-bit integer)
// instead of spin_det_search_key; sigma does not depend on that order.
//
// The singles adjacency is found without the reference's quadratic scan:
// two strings with the same electron count are singly connected iff they
// share an (N-1)-electron subset, so every string emits its N "deletion
// keys" (itself minus one electron); after a radix sort, strings in a run of
// equal keys are exactly the singles of each other, and each single pair
// occurs in exactly one run.
#include <cub/cub.cuh>

#include "qpgpu_internal.cuh"

namespace {

constexpr int TPB = 256;

inline unsigned grid_for(int64_t n, int tpb = TPB) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > (1 << 30)) g = 1 << 30;
  return (unsigned)g;
}

template <class T>
struct Scoped {
  T* p = nullptr;
  ~Scoped() { dev_free(p); }
};

__global__ void k_iota(int* a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (int)i;
}

// word w of spin s of det perm[i]
__global__ void k_gather_word(const u64* dets, int nint, int spin, int w, const int* perm, u64* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = perm ? perm[i] : i;
    out[i] = dets[k * 2 * nint + spin * nint + w];
  }
}

__global__ void k_unique_flags(const u64* dets, int nint, int spin, const int* perm, int* flag, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int f = 1;
    if (i > 0) {
      const u64* a = dets + (int64_t)perm[i] * 2 * nint + spin * nint;
      const u64* b = dets + (int64_t)perm[i - 1] * 2 * nint + spin * nint;
      f = 0;
      for (int w = 0; w < nint; ++w) f |= (a[w] != b[w]);
    }
    flag[i] = f;
  }
}

// uid_sorted = inclusive_scan(flag) - 1 ; id[perm[i]] = uid ; unique[uid] = string
__global__ void k_unique_scatter(const u64* dets, int nint, int spin, const int* perm, const int* incl,
                                 const int* flag, int* id, u64* uniq, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int u = incl[i] - 1;
    id[perm[i]] = u;
    if (flag[i]) {
      const u64* a = dets + (int64_t)perm[i] * 2 * nint + spin * nint;
      for (int w = 0; w < nint; ++w) uniq[(int64_t)u * nint + w] = a[w];
    }
  }
}

__global__ void k_make_key(const int* hi, const int* lo, int64_t mul, u64* key, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    key[i] = (u64)hi[i] * (u64)mul + (u64)lo[i];
}

// bilinear (beta-major): rows/cols at position p from the sorted permutation
__global__ void k_bilinear(const int* order, const int* aid, const int* bid, int* rows, int* cols, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    int k = order[p];
    rows[p] = aid[k];
    cols[p] = bid[k];
  }
}

// first position of each segment id (ids sorted ascending, every id present)
__global__ void k_seg_starts(const int* ids, int* loc, int64_t n, int nseg) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (p == 0 || ids[p] != ids[p - 1]) loc[ids[p]] = (int)p;
    if (p == n - 1) loc[nseg] = (int)n;
  }
}

__global__ void k_gather_u64(const u64* src, const int* idx, u64* dst, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    dst[p] = src[idx[p]];
}

__global__ void k_gather_int(const int* src, const int* idx, int* dst, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    dst[p] = src[idx[p]];
}

// deletion keys: entry e = u*ne + j -> string u with its j-th electron removed
__global__ void k_deletion_word(const u64* uniq, int nint, int ne, int w, const int* perm, u64* out, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t e = perm ? perm[i] : i;
    int64_t u = e / ne;
    int j = (int)(e % ne);
    const u64* s = uniq + u * nint;
    // locate the j-th set bit
    int cnt = 0, wj = -1, bj = 0;
    for (int x = 0; x < nint && wj < 0; ++x) {
      int c = __popcll(s[x]);
      if (j < cnt + c) {
        u64 v = s[x];
        for (int t = 0; t < j - cnt; ++t) v &= v - 1;
        wj = x;
        bj = __ffsll((long long)v) - 1;
      }
      cnt += c;
    }
    u64 word = s[w];
    if (w == wj) word &= ~(1ull << bj);
    out[i] = word;
  }
}

// run boundaries of equal deletion keys (all words compared)
__global__ void k_run_flags(const u64* uniq, int nint, int ne, const int* perm, int* flag, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    if (i == 0) { flag[i] = 1; continue; }
    int f = 0;
    {
      int64_t e1 = perm[i], e0 = perm[i - 1];
      // recompute both keys word by word
      for (int w = 0; w < nint; ++w) {
        u64 k1, k0;
        {
          int64_t u = e1 / ne; int j = (int)(e1 % ne); const u64* s = uniq + u * nint;
          int cnt = 0, wj = -1, bj = 0;
          for (int x = 0; x < nint && wj < 0; ++x) { int c = __popcll(s[x]); if (j < cnt + c) { u64 v = s[x]; for (int t = 0; t < j - cnt; ++t) v &= v - 1; wj = x; bj = __ffsll((long long)v) - 1; } cnt += c; }
          k1 = s[w]; if (w == wj) k1 &= ~(1ull << bj);
        }
        {
          int64_t u = e0 / ne; int j = (int)(e0 % ne); const u64* s = uniq + u * nint;
          int cnt = 0, wj = -1, bj = 0;
          for (int x = 0; x < nint && wj < 0; ++x) { int c = __popcll(s[x]); if (j < cnt + c) { u64 v = s[x]; for (int t = 0; t < j - cnt; ++t) v &= v - 1; wj = x; bj = __ffsll((long long)v) - 1; } cnt += c; }
          k0 = s[w]; if (w == wj) k0 &= ~(1ull << bj);
        }
        f |= (k1 != k0);
      }
    }
    flag[i] = f;
  }
}

// per entry: run id -> run start/end (runs are contiguous)
__global__ void k_run_bounds(const int* run_incl, int* run_start, int* run_end, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int r = run_incl[i] - 1;
    if (i == 0 || run_incl[i - 1] != run_incl[i]) run_start[r] = (int)i;
    if (i == m - 1 || run_incl[i + 1] != run_incl[i]) run_end[r] = (int)i + 1;
  }
}

__global__ void k_pair_counts(const int* run_incl, const int* run_start, const int* run_end, int64_t* cnt, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int r = run_incl[i] - 1;
    cnt[i] = run_end[r] - run_start[r] - 1;
  }
}

// emit (u_i, u_j) for every other member j of i's run, key = u_i * U + u_j
__global__ void k_pair_emit(const int* perm, int ne, const int* run_incl, const int* run_start, const int* run_end,
                            const int64_t* off, u64* keys, int U, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int r = run_incl[i] - 1;
    int64_t o = off[i];
    u64 ui = (u64)(perm[i] / ne);
    for (int j = run_start[r]; j < run_end[r]; ++j) {
      if (j == i) continue;
      keys[o++] = ui * (u64)U + (u64)(perm[j] / ne);
    }
  }
}

__global__ void k_split_pairs(const u64* keys, int U, int* src, int* dst, int64_t t) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t; i += (int64_t)gridDim.x * blockDim.x) {
    src[i] = (int)(keys[i] / (u64)U);
    dst[i] = (int)(keys[i] % (u64)U);
  }
}

__global__ void k_csr_ptr(const int* src, int* ptr, int64_t t, int U) {
  // ptr[u] = first index with src >= u (src sorted)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= t; i += (int64_t)gridDim.x * blockDim.x) {
    int cur = (i < t) ? src[i] : U;
    int prev = (i > 0) ? src[i - 1] : -1;
    for (int u = prev + 1; u <= cur; ++u) ptr[u] = (int)i;
  }
}

// cost of the alpha-beta scan strategies, summed over the singles of each
// string: the length of each single's line, or keycost for a line with a
// 1-deletion table (probes of the ne keys, about one warp step each)
__global__ void k_single_costs(const int* ptr, const int* idx, const int* loc, const unsigned char* lkey,
                               int64_t keycost, int64_t* cost, int U) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < U; u += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = 0;
    for (int t = ptr[u]; t < ptr[u + 1]; ++t)
      c += (lkey && (lkey[idx[t]] & KEY_SINGLE)) ? keycost : loc[idx[t] + 1] - loc[idx[t]];
    cost[u] = c;
  }
}

// LSD radix sort of multi-word keys produced by `word_fn(w, perm, out)`; perm is the result.
template <class WordFn>
int sort_multiword(qpgpu_ctx* c, int64_t n, int nwords, WordFn word_fn, int* perm_out) {
  cudaStream_t st = c->stream;
  Scoped<u64> ka, kb;
  Scoped<int> pa, pb;
  Scoped<char> tmp;
  QP_CUDA(c, dev_alloc(&ka.p, n));
  QP_CUDA(c, dev_alloc(&kb.p, n));
  QP_CUDA(c, dev_alloc(&pa.p, n));
  QP_CUDA(c, dev_alloc(&pb.p, n));
  size_t tbytes = 0;
  QP_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tbytes, ka.p, kb.p, pa.p, pb.p, (int)n, 0, 64, st));
  QP_CUDA(c, dev_alloc(&tmp.p, tbytes));
  k_iota<<<grid_for(n), TPB, 0, st>>>(pa.p, n);
  for (int w = 0; w < nwords; ++w) {
    word_fn(w, pa.p, ka.p);  // keys of the current permutation
    QP_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tbytes, ka.p, kb.p, pa.p, pb.p, (int)n, 0, 64, st));
    std::swap(pa.p, pb.p);
  }
  QP_CUDA(c, cudaMemcpyAsync(perm_out, pa.p, n * sizeof(int), cudaMemcpyDeviceToDevice, st));
  return 0;
}

int unique_spin(qpgpu_ctx* c, int spin, int* id_out, u64** uniq_out, int* nu_out) {
  const int64_t N = c->N;
  const int nint = c->nint;
  cudaStream_t st = c->stream;
  Scoped<int> perm, flag, incl;
  QP_CUDA(c, dev_alloc(&perm.p, N));
  QP_CUDA(c, dev_alloc(&flag.p, N));
  QP_CUDA(c, dev_alloc(&incl.p, N));
  int rc = sort_multiword(c, N, nint, [&](int w, const int* p, u64* out) {
    k_gather_word<<<grid_for(N), TPB, 0, st>>>(c->d_dets, nint, spin, w, p, out, N);
  }, perm.p);
  if (rc) return rc;
  k_unique_flags<<<grid_for(N), TPB, 0, st>>>(c->d_dets, nint, spin, perm.p, flag.p, N);
  size_t tb = 0;
  QP_CUDA(c, cub::DeviceScan::InclusiveSum(nullptr, tb, flag.p, incl.p, (int)N, st));
  Scoped<char> tmp;
  QP_CUDA(c, dev_alloc(&tmp.p, tb));
  QP_CUDA(c, cub::DeviceScan::InclusiveSum(tmp.p, tb, flag.p, incl.p, (int)N, st));
  int nu = 0;
  QP_CUDA(c, cudaMemcpyAsync(&nu, incl.p + N - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  u64* uniq = nullptr;
  QP_CUDA(c, dev_alloc(&uniq, (size_t)nu * nint));
  k_unique_scatter<<<grid_for(N), TPB, 0, st>>>(c->d_dets, nint, spin, perm.p, incl.p, flag.p, id_out, uniq, N);
  *uniq_out = uniq;
  *nu_out = nu;
  return 0;
}

// singles adjacency (CSR) among U unique strings with ne electrons each
int singles_adjacency(qpgpu_ctx* c, const u64* uniq, int U, int ne, int** ptr_out, int** idx_out, int64_t* nnz) {
  cudaStream_t st = c->stream;
  const int nint = c->nint;
  const int64_t m = (int64_t)U * ne;
  *ptr_out = nullptr;
  *idx_out = nullptr;
  *nnz = 0;
  int* ptr = nullptr;
  QP_CUDA(c, dev_alloc(&ptr, (size_t)U + 1));
  if (ne == 0 || m == 0) {
    QP_CUDA(c, cudaMemsetAsync(ptr, 0, sizeof(int) * ((size_t)U + 1), st));
    *ptr_out = ptr;
    QP_CUDA(c, dev_alloc(idx_out, 1));
    return 0;
  }
  Scoped<int> perm, flag, incl, rs, re;
  QP_CUDA(c, dev_alloc(&perm.p, m));
  QP_CUDA(c, dev_alloc(&flag.p, m));
  QP_CUDA(c, dev_alloc(&incl.p, m));
  int rc = sort_multiword(c, m, nint, [&](int w, const int* p, u64* out) {
    k_deletion_word<<<grid_for(m), TPB, 0, st>>>(uniq, nint, ne, w, p, out, m);
  }, perm.p);
  if (rc) return rc;
  k_run_flags<<<grid_for(m), TPB, 0, st>>>(uniq, nint, ne, perm.p, flag.p, m);
  size_t tb = 0;
  QP_CUDA(c, cub::DeviceScan::InclusiveSum(nullptr, tb, flag.p, incl.p, (int)m, st));
  Scoped<char> tmp;
  QP_CUDA(c, dev_alloc(&tmp.p, tb));
  QP_CUDA(c, cub::DeviceScan::InclusiveSum(tmp.p, tb, flag.p, incl.p, (int)m, st));
  int nruns = 0;
  QP_CUDA(c, cudaMemcpyAsync(&nruns, incl.p + m - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  QP_CUDA(c, dev_alloc(&rs.p, nruns));
  QP_CUDA(c, dev_alloc(&re.p, nruns));
  k_run_bounds<<<grid_for(m), TPB, 0, st>>>(incl.p, rs.p, re.p, m);
  Scoped<int64_t> cnt, off;
  QP_CUDA(c, dev_alloc(&cnt.p, m + 1));
  QP_CUDA(c, dev_alloc(&off.p, m + 1));
  QP_CUDA(c, cudaMemsetAsync(cnt.p + m, 0, sizeof(int64_t), st));
  k_pair_counts<<<grid_for(m), TPB, 0, st>>>(incl.p, rs.p, re.p, cnt.p, m);
  size_t tb2 = 0;
  QP_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb2, cnt.p, off.p, (int)(m + 1), st));
  Scoped<char> tmp2;
  QP_CUDA(c, dev_alloc(&tmp2.p, tb2));
  QP_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp2.p, tb2, cnt.p, off.p, (int)(m + 1), st));
  int64_t T = 0;
  QP_CUDA(c, cudaMemcpyAsync(&T, off.p + m, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  if (T >= ((int64_t)1 << 31)) return qpgpu_fail(c, QPGPU_ERR_NOMEM, "singles adjacency too large");
  int* idx = nullptr;
  QP_CUDA(c, dev_alloc(&idx, (size_t)(T > 0 ? T : 1)));
  if (T > 0) {
    Scoped<u64> k1, k2;
    QP_CUDA(c, dev_alloc(&k1.p, T));
    QP_CUDA(c, dev_alloc(&k2.p, T));
    k_pair_emit<<<grid_for(m), TPB, 0, st>>>(perm.p, ne, incl.p, rs.p, re.p, off.p, k1.p, U, m);
    size_t tb3 = 0;
    QP_CUDA(c, cub::DeviceRadixSort::SortKeys(nullptr, tb3, k1.p, k2.p, (int)T, 0, 64, st));
    Scoped<char> tmp3;
    QP_CUDA(c, dev_alloc(&tmp3.p, tb3));
    QP_CUDA(c, cub::DeviceRadixSort::SortKeys(tmp3.p, tb3, k1.p, k2.p, (int)T, 0, 64, st));
    Scoped<int> src;
    QP_CUDA(c, dev_alloc(&src.p, T));
    k_split_pairs<<<grid_for(T), TPB, 0, st>>>(k2.p, U, src.p, idx, T);
    k_csr_ptr<<<grid_for(T + 1), TPB, 0, st>>>(src.p, ptr, T, U);
    QP_CUDA(c, cudaStreamSynchronize(st));
  } else {
    QP_CUDA(c, cudaMemsetAsync(ptr, 0, sizeof(int) * ((size_t)U + 1), st));
  }
  *ptr_out = ptr;
  *idx_out = idx;
  *nnz = T;
  return 0;
}

}  // namespace

void qp_free_dets(qpgpu_ctx* c) {
  qp_free_line_keys(c);
  void** ps[] = {(void**)&c->d_dets, (void**)&c->d_alpha, (void**)&c->d_beta, (void**)&c->d_rows,
                 (void**)&c->d_cols, (void**)&c->d_order, (void**)&c->d_col_loc, (void**)&c->d_t_order,
                 (void**)&c->d_t_cols, (void**)&c->d_row_loc, (void**)&c->d_sa_ptr, (void**)&c->d_sa_idx,
                 (void**)&c->d_sb_ptr, (void**)&c->d_sb_idx, (void**)&c->d_cost_a, (void**)&c->d_cost_b,
                 (void**)&c->d_detfeat, (void**)&c->d_alpha_pos, (void**)&c->d_beta_tpos};
  for (auto p : ps) {
    dev_free(*p);
    *p = nullptr;
  }
  c->have_dets = false;
  c->N = 0;
}

namespace {
// out[i] = strings[id[p(i)]] (p = perm, or the identity), nint words each
__global__ void k_gather_strings(const u64* strings, const int* id, const int* perm, u64* out, int64_t N, int nint) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * nint; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / nint;
    const int w = (int)(t % nint);
    const int64_t p = perm ? perm[i] : i;
    out[t] = strings[(int64_t)id[p] * nint + w];
  }
}
}  // namespace

// Requires c->d_dets and c->N set.
int qp_build_index(qpgpu_ctx* c) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  Scoped<int> aid, bid;
  QP_CUDA(c, dev_alloc(&aid.p, N));
  QP_CUDA(c, dev_alloc(&bid.p, N));
  int rc = unique_spin(c, 0, aid.p, &c->d_alpha, &c->Ua);
  if (rc) return rc;
  rc = unique_spin(c, 1, bid.p, &c->d_beta, &c->Ub);
  if (rc) return rc;
  qp_mark(c, "unique strings");
  const int Ua = c->Ua, Ub = c->Ub;
  // beta-major bilinear order: key = beta_id * Ua + alpha_id (spindeterminants.irp.f:417)
  QP_CUDA(c, dev_alloc(&c->d_order, N));
  QP_CUDA(c, dev_alloc(&c->d_rows, N));
  QP_CUDA(c, dev_alloc(&c->d_cols, N));
  {
    Scoped<u64> key;
    QP_CUDA(c, dev_alloc(&key.p, N));
    k_make_key<<<grid_for(N), TPB, 0, st>>>(bid.p, aid.p, Ua, key.p, N);
    rc = sort_multiword(c, N, 1, [&](int, const int* p, u64* out) {
      k_gather_u64<<<grid_for(N), TPB, 0, st>>>(key.p, p, out, N);
    }, c->d_order);
    if (rc) return rc;
  }
  k_bilinear<<<grid_for(N), TPB, 0, st>>>(c->d_order, aid.p, bid.p, c->d_rows, c->d_cols, N);
  QP_CUDA(c, dev_alloc(&c->d_col_loc, (size_t)Ub + 1));
  k_seg_starts<<<grid_for(N), TPB, 0, st>>>(c->d_cols, c->d_col_loc, N, Ub);
  // alpha-major (transposed) order over bilinear positions: key = alpha_id * Ub + beta_id
  QP_CUDA(c, dev_alloc(&c->d_t_order, N));
  QP_CUDA(c, dev_alloc(&c->d_t_cols, N));
  QP_CUDA(c, dev_alloc(&c->d_row_loc, (size_t)Ua + 1));
  {
    Scoped<u64> key;
    QP_CUDA(c, dev_alloc(&key.p, N));
    k_make_key<<<grid_for(N), TPB, 0, st>>>(c->d_rows, c->d_cols, Ub, key.p, N);
    rc = sort_multiword(c, N, 1, [&](int, const int* p, u64* out) {
      k_gather_u64<<<grid_for(N), TPB, 0, st>>>(key.p, p, out, N);
    }, c->d_t_order);
    if (rc) return rc;
    Scoped<int> trows;
    QP_CUDA(c, dev_alloc(&trows.p, N));
    k_gather_int<<<grid_for(N), TPB, 0, st>>>(c->d_rows, c->d_t_order, trows.p, N);
    k_gather_int<<<grid_for(N), TPB, 0, st>>>(c->d_cols, c->d_t_order, c->d_t_cols, N);
    k_seg_starts<<<grid_for(N), TPB, 0, st>>>(trows.p, c->d_row_loc, N, Ua);
  }
  // spin strings in scan order: the pair kernels read the strings of a
  // column (row) as one contiguous span instead of index -> string gathers
  QP_CUDA(c, dev_alloc(&c->d_alpha_pos, (size_t)N * c->nint));
  QP_CUDA(c, dev_alloc(&c->d_beta_tpos, (size_t)N * c->nint));
  k_gather_strings<<<grid_for(N * c->nint), TPB, 0, st>>>(c->d_alpha, c->d_rows, nullptr, c->d_alpha_pos, N,
                                                          c->nint);
  k_gather_strings<<<grid_for(N * c->nint), TPB, 0, st>>>(c->d_beta, c->d_cols, c->d_t_order, c->d_beta_tpos, N,
                                                          c->nint);
  qp_mark(c, "bilinear index");
  // singles among unique strings, and the per-string costs of the two
  // alpha-beta scan strategies
  rc = singles_adjacency(c, c->d_alpha, Ua, c->na, &c->d_sa_ptr, &c->d_sa_idx, &c->n_sa);
  if (rc) return rc;
  rc = singles_adjacency(c, c->d_beta, Ub, c->nb, &c->d_sb_ptr, &c->d_sb_idx, &c->n_sb);
  if (rc) return rc;
  qp_mark(c, "singles adjacency");
  rc = qp_build_line_keys(c);
  if (rc) return rc;
  qp_mark(c, "deletion-key tables");
  QP_CUDA(c, dev_alloc(&c->d_cost_a, (size_t)Ua));
  QP_CUDA(c, dev_alloc(&c->d_cost_b, (size_t)Ub));
  k_single_costs<<<grid_for(Ua), TPB, 0, st>>>(c->d_sa_ptr, c->d_sa_idx, c->d_row_loc, c->d_rowkey,
                                               32 * (int64_t)(c->nb + 2), c->d_cost_a, Ua);
  k_single_costs<<<grid_for(Ub), TPB, 0, st>>>(c->d_sb_ptr, c->d_sb_idx, c->d_col_loc, c->d_colkey,
                                               32 * (int64_t)(c->na + 2), c->d_cost_b, Ub);
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaStreamSynchronize(st));
  return 0;
}
