// Deletion-key tables of the heavy lines of a determinant set.
//
// The pair scans of pairs.cu test, for every determinant, every string of its
// beta column (same-beta pairs), of its alpha row (same-alpha pairs) and of
// the columns of its beta singles (alpha x beta pairs), as the reference's
// loops do (src/Davidson/u0Hu0.irp.f:177-332).  The cost of a line is the
// square of its length, and a few lines dominate: in the seeded 2e7-determinant
// set the reference beta column holds 4.4e6 determinants, about 2e13 string
// tests per sigma for that column alone, against 1e10 same-beta pairs in the
// whole set.  For the lines above a length threshold this file builds hash
// tables of deletion keys (the KeySlot comment in qpgpu_internal.cuh gives the
// principle); the scans then visit only the strings that share a key with the
// determinant, which are about the pairs themselves.
//
//   KT_COL1  alpha strings of a heavy column, one electron removed: the
//            alpha x beta scan probes a determinant's alpha string, minus each
//            electron, in the columns of its beta singles
//   KT_ROW1  the same for the beta strings of a heavy row
//   KT_COL2  alpha strings of a heavy column, two electrons removed: the
//            same-beta pairs of the column's own determinants
//   KT_ROW2  the same for the beta strings of a heavy row
//
// Build: one entry (hash, position) per string and removed electron (pair),
// a radix sort by hash, runs of equal hashes as groups, and an open-addressing
// table hash -> (first member, members).  2-deletion groups with one member
// hold no pair and are left out of the table.
#include <algorithm>
#include <climits>

#include <cub/cub.cuh>

#include "qpgpu_internal.cuh"

namespace {

constexpr int TPB = 256;

inline unsigned grid_n(int64_t n) {
  const int64_t g = (n + TPB - 1) / TPB;
  return (unsigned)std::min<int64_t>(std::max<int64_t>(g, 1), (int64_t)1 << 20);
}

template <class T>
struct Scoped {
  T* p = nullptr;
  ~Scoped() { dev_free(p); }
};

// flags of each line (n = loc[l+1] - loc[l] determinants): KEY_SINGLE when
// n > t1, KEY_DOUBLE when n > t2; sums[0], sums[1]: positions of the flagged
// lines
__global__ void k_line_flags(const int* loc, int nl, int64_t t1, int64_t t2, unsigned char* f,
                             unsigned long long* sums) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nl; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = loc[l + 1] - loc[l];
    unsigned char v = 0;
    if (n > t1) {
      v |= KEY_SINGLE;
      atomicAdd(&sums[0], (unsigned long long)n);
    }
    if (n > t2) {
      v |= KEY_DOUBLE;
      atomicAdd(&sums[1], (unsigned long long)n);
    }
    f[l] = v;
  }
}

__global__ void k_clear_flag(unsigned char* f, int nl, unsigned char bit) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nl; l += (int64_t)gridDim.x * blockDim.x)
    f[l] &= (unsigned char)~bit;
}

__global__ void k_count_flagged(const unsigned char* f, int nl, unsigned long long* n) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nl; l += (int64_t)gridDim.x * blockDim.x)
    if (f[l]) atomicAdd(n, 1ull);
}

// 1 for the positions whose line carries `bit`.  SPIN 0: bilinear positions
// (line = beta column), SPIN 1: alpha-major positions (line = alpha row)
template <int SPIN>
__global__ void k_pos_flags(const int* lineof, const int* t_order, const unsigned char* lf, unsigned char bit,
                            int* pf, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    const int line = SPIN == 0 ? lineof[p] : lineof[t_order[p]];
    pf[p] = (lf[line] & bit) ? 1 : 0;
  }
}

__global__ void k_pos_compact(const int* pf, const int* off, int* kpos, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x)
    if (pf[p]) kpos[off[p]] = (int)p;
}

// entry e = idx * nc + c: the string at position kpos[idx] with its c-th
// electron (dele 1) or c-th electron pair (dele 2) removed
template <int NINT, int SPIN>
__global__ void k_key_emit(const u64* strs, const int* lineof, const int* t_order, const int* kpos, int64_t M,
                           int ne, int dele, int kind, u64 hmask, u64* keys, int* vals) {
  const int nc = dele == 1 ? ne : ne * (ne - 1) / 2;
  const int64_t E = M * nc;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t idx = e / nc;
    const int c = (int)(e - idx * nc);
    const int p = kpos[idx];
    const int line = SPIN == 0 ? lineof[p] : lineof[t_order[p]];
    u64 K[NINT];
#pragma unroll
    for (int w = 0; w < NINT; ++w) K[w] = strs[(int64_t)p * NINT + w];
    if (dele == 1) {
      const int b = nth_electron<NINT>(K, c);
      clear_orbital<NINT>(K, b);
    } else {
      int i, j;
      pair_of_combo(c, ne, i, j);
      const int bi = nth_electron<NINT>(K, i), bj = nth_electron<NINT>(K, j);
      clear_orbital<NINT>(K, bi);
      clear_orbital<NINT>(K, bj);
    }
    keys[e] = key_hash<NINT>(kind, line, K, hmask);
    vals[e] = p;
  }
}

// groups are runs of equal hashes in the sorted keys: count (insert = 0) or
// insert (insert = 1) those with at least minlen members.  A group holds at
// most n_mo - ne + 2 choose 2 members (the strings that contain a given key),
// so the thread at a run start walks to its end.
__global__ void k_key_groups(const u64* keys, int64_t E, int minlen, unsigned long long* ng, KeySlot* slot,
                             u64 mask, int insert) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x) {
    const u64 h = keys[i];
    if (i > 0 && keys[i - 1] == h) continue;
    int64_t j = i + 1;
    while (j < E && keys[j] == h) ++j;
    if (j - i < minlen) continue;
    if (!insert) {
      atomicAdd(ng, 1ull);
      continue;
    }
    u64 s = h & mask;
    for (u64 it = 0; it <= mask; ++it) {
      const u64 prev = atomicCAS(&slot[s].h, 0ull, h);
      if (prev == 0ull) {
        slot[s].start = (unsigned)i;
        slot[s].len = (unsigned)(j - i);
        break;
      }
      s = (s + 1) & mask;
    }
  }
}

template <int NINT>
int build_table(qpgpu_ctx* c, int kind, unsigned char* lflags, int nlines, int64_t M, u64 hmask) {
  const int spin = (kind == KT_COL1 || kind == KT_COL2) ? 0 : 1;
  const int dele = (kind == KT_COL2 || kind == KT_ROW2) ? 2 : 1;
  const unsigned char bit = dele == 1 ? KEY_SINGLE : KEY_DOUBLE;
  const int ne = spin == 0 ? c->na : c->nb;
  const int64_t nc = dele == 1 ? ne : (int64_t)ne * (ne - 1) / 2;
  const int64_t E = M * nc;
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  if (M == 0) return 0;
  if (nc == 0) {  // no electron (pair) to remove: the lines stay with the scans
    k_clear_flag<<<grid_n(nlines), TPB, 0, st>>>(lflags, nlines, bit);
    QP_CUDA(c, cudaGetLastError());
    return 0;
  }
  // cut hashes merge most keys into a few groups and make the probes walk
  // them whole: a test hook for small sets only
  if (c->key_hash_bits < 64 && E > ((int64_t)1 << 22))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "line keys: hash_bits below 64 is a test hook for tables of at most 2^22 keys");
  // the sort holds two copies of (hash, position): leave the lines to the
  // scans when that would take more than half of the free memory or the
  // member offsets would not fit 32 bits
  size_t fr = 0, total = 0;
  QP_CUDA(c, cudaMemGetInfo(&fr, &total));
  const double need = 26.0 * (double)E + 12.0 * (double)N;
  if (E >= (int64_t)INT_MAX || need > 0.5 * (double)fr) {
    k_clear_flag<<<grid_n(nlines), TPB, 0, st>>>(lflags, nlines, bit);
    QP_CUDA(c, cudaGetLastError());
    return 0;
  }
  Scoped<int> kpos;
  QP_CUDA(c, dev_alloc(&kpos.p, (size_t)M));
  {
    Scoped<int> pf, off;
    Scoped<char> tmp;
    QP_CUDA(c, dev_alloc(&pf.p, (size_t)N));
    QP_CUDA(c, dev_alloc(&off.p, (size_t)N));
    if (spin == 0)
      k_pos_flags<0><<<grid_n(N), TPB, 0, st>>>(c->d_cols, c->d_t_order, lflags, bit, pf.p, N);
    else
      k_pos_flags<1><<<grid_n(N), TPB, 0, st>>>(c->d_rows, c->d_t_order, lflags, bit, pf.p, N);
    size_t tb = 0;
    QP_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, pf.p, off.p, (int)N, st));
    QP_CUDA(c, dev_alloc(&tmp.p, tb));
    QP_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, pf.p, off.p, (int)N, st));
    k_pos_compact<<<grid_n(N), TPB, 0, st>>>(pf.p, off.p, kpos.p, N);
    QP_CUDA(c, cudaGetLastError());
    QP_CUDA(c, cudaStreamSynchronize(st));
  }
  Scoped<u64> ka, kb;
  Scoped<int> va, vb;
  QP_CUDA(c, dev_alloc(&ka.p, (size_t)E));
  QP_CUDA(c, dev_alloc(&kb.p, (size_t)E));
  QP_CUDA(c, dev_alloc(&va.p, (size_t)E));
  QP_CUDA(c, dev_alloc(&vb.p, (size_t)E));
  if (spin == 0)
    k_key_emit<NINT, 0><<<grid_n(E), TPB, 0, st>>>(c->d_alpha_pos, c->d_cols, c->d_t_order, kpos.p, M, ne, dele,
                                                   kind, hmask, ka.p, va.p);
  else
    k_key_emit<NINT, 1><<<grid_n(E), TPB, 0, st>>>(c->d_beta_tpos, c->d_rows, c->d_t_order, kpos.p, M, ne, dele,
                                                   kind, hmask, ka.p, va.p);
  QP_CUDA(c, cudaGetLastError());
  const int bits = std::max(1, std::min(64, c->key_hash_bits));
  cub::DoubleBuffer<u64> dk(ka.p, kb.p);
  cub::DoubleBuffer<int> dv(va.p, vb.p);
  {
    size_t tb = 0;
    QP_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, dk, dv, (int)E, 0, bits, st));
    Scoped<char> tmp;
    QP_CUDA(c, dev_alloc(&tmp.p, tb));
    QP_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, dk, dv, (int)E, 0, bits, st));
  }
  const int minlen = dele == 2 ? 2 : 1;
  Scoped<unsigned long long> ng;
  QP_CUDA(c, dev_alloc(&ng.p, 1));
  QP_CUDA(c, cudaMemsetAsync(ng.p, 0, sizeof(unsigned long long), st));
  k_key_groups<<<grid_n(E), TPB, 0, st>>>(dk.Current(), E, minlen, ng.p, nullptr, 0, 0);
  unsigned long long G = 0;
  QP_CUDA(c, cudaMemcpyAsync(&G, ng.p, sizeof(G), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  int64_t nslot = 16;
  while (nslot < 2 * (int64_t)G) nslot <<= 1;
  KeySlot* slot = nullptr;
  QP_CUDA(c, dev_alloc(&slot, (size_t)nslot));
  QP_CUDA(c, cudaMemsetAsync(slot, 0, sizeof(KeySlot) * (size_t)nslot, st));
  c->d_kslot[kind] = slot;
  c->kslots[kind] = nslot;
  k_key_groups<<<grid_n(E), TPB, 0, st>>>(dk.Current(), E, minlen, ng.p, slot, (u64)(nslot - 1), 1);
  QP_CUDA(c, cudaGetLastError());
  // keep the sorted positions as the member array
  int* mem = dv.Current();
  if (mem == va.p)
    va.p = nullptr;
  else
    vb.p = nullptr;
  c->d_kmem[kind] = mem;
  c->kmem_n[kind] = E;
  QP_CUDA(c, cudaStreamSynchronize(st));
  return 0;
}

template <int NINT>
int build_line_keys_t(qpgpu_ctx* c) {
  cudaStream_t st = c->stream;
  const int64_t big = INT64_MAX;
  const int64_t t1_col = c->key_min_single >= 0 ? c->key_min_single : 64 * (int64_t)(c->na + 2);
  const int64_t t1_row = c->key_min_single >= 0 ? c->key_min_single : 64 * (int64_t)(c->nb + 2);
  const int64_t t2 = c->key_min_double >= 0 ? c->key_min_double : 16384;
  const u64 hmask = c->key_hash_bits >= 64 ? ~0ull : ((1ull << std::max(1, c->key_hash_bits)) - 1ull);
  QP_CUDA(c, dev_alloc(&c->d_colkey, (size_t)c->Ub));
  QP_CUDA(c, dev_alloc(&c->d_rowkey, (size_t)c->Ua));
  Scoped<unsigned long long> sums;
  QP_CUDA(c, dev_alloc(&sums.p, 5));
  QP_CUDA(c, cudaMemsetAsync(sums.p, 0, 5 * sizeof(unsigned long long), st));
  k_line_flags<<<grid_n(c->Ub), TPB, 0, st>>>(c->d_col_loc, c->Ub, t1_col, c->na >= 2 ? t2 : big, c->d_colkey,
                                               sums.p);
  k_line_flags<<<grid_n(c->Ua), TPB, 0, st>>>(c->d_row_loc, c->Ua, t1_row, c->nb >= 2 ? t2 : big, c->d_rowkey,
                                               sums.p + 2);
  QP_CUDA(c, cudaGetLastError());
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  QP_CUDA(c, cudaMemcpyAsync(h, sums.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  int rc = build_table<NINT>(c, KT_COL1, c->d_colkey, c->Ub, (int64_t)h[0], hmask);
  if (!rc) rc = build_table<NINT>(c, KT_ROW1, c->d_rowkey, c->Ua, (int64_t)h[2], hmask);
  if (!rc) rc = build_table<NINT>(c, KT_COL2, c->d_colkey, c->Ub, (int64_t)h[1], hmask);
  if (!rc) rc = build_table<NINT>(c, KT_ROW2, c->d_rowkey, c->Ua, (int64_t)h[3], hmask);
  if (rc) return rc;
  k_count_flagged<<<grid_n(c->Ub), TPB, 0, st>>>(c->d_colkey, c->Ub, sums.p + 4);
  k_count_flagged<<<grid_n(c->Ua), TPB, 0, st>>>(c->d_rowkey, c->Ua, sums.p + 4);
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaMemcpyAsync(&h[4], sums.p + 4, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  c->n_keyed_lines = (int)h[4];
  return 0;
}

}  // namespace

int qp_build_line_keys(qpgpu_ctx* c) {
  if (c->nint == 1) return build_line_keys_t<1>(c);
  if (c->nint == 2) return build_line_keys_t<2>(c);
  return qpgpu_fail(c, QPGPU_ERR_ARG, "n_int > 2 is not supported");
}

void qp_free_line_keys(qpgpu_ctx* c) {
  for (int k = 0; k < KT_N; ++k) {
    dev_free(c->d_kslot[k]);
    dev_free(c->d_kmem[k]);
    c->d_kslot[k] = nullptr;
    c->d_kmem[k] = nullptr;
    c->kslots[k] = c->kmem_n[k] = 0;
  }
  dev_free(c->d_colkey);
  dev_free(c->d_rowkey);
  c->d_colkey = c->d_rowkey = nullptr;
  c->n_keyed_lines = 0;
}
