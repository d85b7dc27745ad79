// CIPSI selection with the Epstein-Nesbet second-order energy on the device
// (plugins/Full_CI_ZMQ/selection.irp.f: select_connected :24-79, the
// per-generator walk :258-580, splash_pq and get_d0/d1/d2 :647-1086, the
// banned masks :1088-1172, fill_buffer_double :582-645, and the buffer of
// selection_buffer.irp.f:33-138).
//
// The wave function held by the context must be in psi_det_sorted order:
// generators are determinants 0..n_gen-1 and selectors 0..n_sel-1.
//
// Work items.  For a generator g, an external determinant a is a single
// excitation (g minus a hole h, plus a particle p) or a double one (g minus
// holes h1, h2, plus particles p1, p2).  The particles are orbitals empty in
// g, so each a has exactly one (holes, particles) description.  One CTA
// takes one item (g, holes, range of particle entries):
//  * single: entries p over the empty orbitals of the hole's spin;
//  * same-spin double: entries p1 < p2 over the empty orbitals of the
//    holes' spin;
//  * alpha-beta double: entries (p1 alpha, p2 beta).
// The entry range of an item is cut so that its numerator tile (entries x
// states, FP64) fits the CTA's shared memory.
//
// Numerators.  mask = g without the holes.  A selector D can be connected
// (excitation degree <= 2) to some a = mask + particles only if D lacks at
// most two of mask's electrons (k = |mask \ D| <= 2).  For a double item,
// a and D are then connected iff k + [p1 not in D] + [p2 not in D] <= 2; for
// a single item, iff k + [p not in D] <= 2.  This is the case split of
// get_d0 / get_d1 / get_d2 with k = 0, 1, 2.  Only selectors within a
// quadruple excitation of g can pass, so those are listed once per
// generator (k_sel_lists).  The CTA filters them per item (k <= 2), in
// selector order.  Every thread owns a fixed set of entries and adds
// c_D <a|H|D> for its connected entries, selector after selector, so each
// numerator is summed in selector order with no atomics.  <a|H|D> is the
// generic i_H_j (slater_rules.irp.f:478-570) with a as the first
// determinant.
//
// Banned determinants.  a is dropped when it is in the wave function
// (device hash set of psi_det) or within a double excitation of an earlier
// generator, so that every external determinant is counted once, by the
// first generator that reaches it.  The earlier generators within a
// quadruple excitation of g are listed once per generator; the CTA keeps
// those that lack at most two of mask's electrons.
//
// Energy.  H_aa = diag_H_mat_elem_fock(g, a) (slater_rules.irp.f:1800-1866)
// from the generator's build_fock_tmp (Fock_diag.irp.f:1-98).  For each state,
// e = (sign(delta) sqrt(delta^2 + (2 mat)^2) - delta) / 2 with
// delta = E0 - H_aa.  pt2 sums e.  The buffer gets a with min(0, min_st e)
// when some numerator is non-zero, and keeps the most negative values: a
// device radix sort by value, with ties put in determinant-bit order on the
// host.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "qpgpu_internal.cuh"

namespace {

constexpr int SBLK = 256;
constexpr int SEL_TILE = 16384;    // FP64 numerators per CTA at most (128 KB of shared memory)
constexpr int SEL_DTILE = 256;     // selectors staged per filtering pass
constexpr int SEL_MAXST = 8;       // states
constexpr int SEL_MAXFG = 2048;    // earlier generators kept per item in shared memory (else read from the global list)

enum { IT_SINGLE = 0, IT_SAME = 1, IT_AB = 2 };

struct SelItem {
  int g;         // generator (psi_det index)
  int gl;        // its position in the generator list of the call
  int kind;      // IT_*
  int spin;      // single / same-spin double: 0 alpha, 1 beta
  int h1, h2;    // holes (1-based); alpha-beta: h1 alpha, h2 beta
  int e0, e1;    // entry range
};

struct SelArgs {
  DevTables t;
  const u64* dets;       // (nint, 2, N)
  const double* coef;    // (N, n_st) row-major (state fastest)
  const double* e0;      // (n_st)
  int n_st;
  int64_t N;
  const SelItem* items;
  const int64_t* ilist_off;  // per listed generator: selectors within a quadruple excitation
  const int* ilist;
  const int64_t* flist_off;  // per listed generator: earlier generators within a quadruple excitation
  const int* flist;
  const double* fock;        // per listed generator: build_fock_tmp, [gl][2][n_mo + 2]
  const int* hslot;          // hash set of psi_det: det index or -1
  uint64_t hmask;
  double* pt2_part;          // [item][n_st]
  unsigned long long* n_ext;
  unsigned long long* n_cand;
  uint64_t cap;
  double* cand_val;
  u64* cand_det;             // (2 nint) per candidate
  int* err;
};

template <int NINT>
__device__ __forceinline__ uint64_t det_hash(const u64* d) {
  uint64_t h = 0x9e3779b97f4a7c15ull;
#pragma unroll
  for (int w = 0; w < 2 * NINT; ++w) {
    h ^= d[w] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h *= 0xbf58476d1ce4e5b9ull;
  }
  return h ^ (h >> 31);
}

template <int NINT>
__device__ __forceinline__ bool same_det(const u64* a, const u64* b) {
  bool eq = true;
#pragma unroll
  for (int w = 0; w < 2 * NINT; ++w) eq &= a[w] == b[w];
  return eq;
}

template <int NINT>
__global__ void k_hash_insert(const u64* dets, int64_t N, int* slot, uint64_t hmask) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const u64* d = dets + i * 2 * NINT;
    uint64_t s = det_hash<NINT>(d) & hmask;
    for (uint64_t probe = 0; probe <= hmask; ++probe) {
      const int prev = atomicCAS(&slot[s], -1, (int)i);
      if (prev == -1) break;
      s = (s + 1) & hmask;
    }
  }
}

template <int NINT>
__device__ __forceinline__ bool in_wf(const SelArgs& A, const u64* a) {
  uint64_t s = det_hash<NINT>(a) & A.hmask;
  for (uint64_t probe = 0; probe <= A.hmask; ++probe) {
    const int i = __ldg(&A.hslot[s]);
    if (i < 0) return false;
    if (same_det<NINT>(A.dets + (int64_t)i * 2 * NINT, a)) return true;
    s = (s + 1) & A.hmask;
  }
  return false;
}

template <int NINT>
__device__ __forceinline__ int exc_deg(const u64* a, const u64* b) {
  int d = 0;
#pragma unroll
  for (int w = 0; w < 2 * NINT; ++w) d += popc64(a[w] ^ b[w]);
  return d >> 1;
}

// per listed generator g = gens[l]: the candidates c < limit (selectors:
// limit = n_sel; earlier generators: limit = g) within a quadruple excitation
// of g, in increasing order.  mode 0 counts into cnt[l], mode 1 fills at off[l].
template <int NINT>
__global__ void __launch_bounds__(SBLK) k_sel_lists(const u64* dets, const int* gens, int n_list, int n_sel,
                                                    int earlier, int mode, int64_t* cnt, const int64_t* off,
                                                    int* out) {
  __shared__ int wsum[SBLK / 32];
  __shared__ int base_s;
  const int l = blockIdx.x;
  if (l >= n_list) return;
  const int g = gens[l];
  u64 gd[2 * NINT];
#pragma unroll
  for (int w = 0; w < 2 * NINT; ++w) gd[w] = dets[(int64_t)g * 2 * NINT + w];
  const int limit = earlier ? g : n_sel;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  for (int c0 = 0; c0 < limit; c0 += SBLK) {
    const int c = c0 + threadIdx.x;
    bool keep = false;
    if (c < limit) keep = exc_deg<NINT>(gd, dets + (int64_t)c * 2 * NINT) <= 4;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int before = base_s;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    if (mode == 1 && keep) out[off[l] + before + __popc(bal & ((1u << lane) - 1))] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < SBLK / 32; ++w) tot += wsum[w];
      base_s += tot;
    }
    __syncthreads();
  }
  if (mode == 0 && threadIdx.x == 0) cnt[l] = base_s;
}

// build_fock_tmp (Fock_diag.irp.f:1-98) of every listed generator:
// f[l][s][i], i = 1..n_mo, and f[l][s][n_mo + 1] = <g|H|g>
template <int NINT>
__global__ void k_sel_fock(DevTables t, const u64* dets, const int* gens, int n_list, double* fock) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n_list) return;
  const int n = t.n, st = n + 2;
  const u64* d = dets + (int64_t)gens[l] * 2 * NINT;
  double* f = fock + (int64_t)l * 2 * st;
  for (int i = 0; i < 2 * st; ++i) f[i] = 0.0;
  int occ[2][QPGPU_MAX_MO];
  int no[2] = {0, 0};
  for (int s = 0; s < 2; ++s)
    for (int w = 0; w < NINT; ++w)
      for (u64 x = d[s * NINT + w]; x; x &= x - 1) occ[s][no[s]++] = ctz64(x) + 1 + 64 * w;
  double e0 = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int o = 1 - s;
    for (int ii = 0; ii < no[s]; ++ii) {
      const int i = occ[s][ii];
      f[s * st + i] += tab2(t.h, n, i, i);
      e0 += tab2(t.h, n, i, i);
      for (int jj = 0; jj < no[s]; ++jj) {
        const int j = occ[s][jj];
        if (i == j) continue;
        f[s * st + i] += tab2(t.ja, n, i, j);
        e0 += 0.5 * tab2(t.ja, n, i, j);
      }
      for (int jj = 0; jj < no[o]; ++jj) {
        const int j = occ[o][jj];
        f[s * st + i] += tab2(t.jj, n, i, j);
        if (s == 0) e0 += tab2(t.jj, n, i, j);
      }
    }
  }
  for (int s = 0; s < 2; ++s) {
    const int o = 1 - s;
    for (int i = 1; i <= n; ++i) {
      if (f[s * st + i] != 0.0) continue;
      f[s * st + i] += tab2(t.h, n, i, i);
      for (int jj = 0; jj < no[s]; ++jj) f[s * st + i] += tab2(t.ja, n, i, occ[s][jj]);
      for (int jj = 0; jj < no[o]; ++jj) f[s * st + i] += tab2(t.jj, n, i, occ[o][jj]);
    }
  }
  f[n + 1] = e0;
  f[st + n + 1] = e0;
}

// <a|H|D>, generic path (degree from the words; a is the first determinant)
template <int NINT>
__device__ __forceinline__ double ihj(const DevTables& t, const u64* a, const u64* D) {
  int da = 0, db = 0;
#pragma unroll
  for (int w = 0; w < NINT; ++w) {
    da += popc64(a[w] ^ D[w]);
    db += popc64(a[NINT + w] ^ D[NINT + w]);
  }
  if (da + db == 4) {
    if (da == 4) return h_double_spin<NINT>(t, a, D, nullptr, nullptr);
    if (db == 4) return h_double_spin<NINT>(t, a + NINT, D + NINT, nullptr, nullptr);
    double s2;
    return h_double_ab<NINT>(t, a, D, &s2, nullptr, nullptr);
  }
  if (da + db == 2) return h_mono_spin<NINT>(t, a, D, da == 2 ? 1 : 2, nullptr, nullptr);
  if (da + db == 0) return diag_h<NINT>(t, a);
  return 0.0;
}

__device__ __forceinline__ bool has_orb(const u64* d, int nint, int spin, int orb) {
  return (d[spin * nint + ((orb - 1) >> 6)] >> ((orb - 1) & 63)) & 1ull;
}
__device__ __forceinline__ void set_orb(u64* d, int nint, int spin, int orb, bool on) {
  const u64 b = 1ull << ((orb - 1) & 63);
  u64& w = d[spin * nint + ((orb - 1) >> 6)];
  w = on ? (w | b) : (w & ~b);
}

// triangular entry e -> (i1 < i2)
__device__ __forceinline__ void tri_decode(int e, int& i1, int& i2) {
  int j = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)e)) * 0.5f);
  while (j * (j - 1) / 2 > e) --j;
  while ((j + 1) * j / 2 <= e) ++j;
  i2 = j;
  i1 = e - j * (j - 1) / 2;
}

template <int NINT>
__global__ void __launch_bounds__(SBLK) k_sel_items(SelArgs A) {
  extern __shared__ double tile[];  // [entry - e0][n_st]
  __shared__ u64 sdet[SEL_DTILE][2 * NINT];
  __shared__ int sidx[SEL_DTILE];
  __shared__ unsigned char sk[SEL_DTILE];
  __shared__ int vir[2][QPGPU_MAX_MO];
  __shared__ int nvir[2];
  __shared__ int fgen[SEL_MAXFG];
  __shared__ int nfg;
  __shared__ int wsum[SBLK / 32];
  __shared__ int nsel_s;
  const SelItem it = A.items[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nst = A.n_st, n = A.t.n;
  const u64* gd = A.dets + (int64_t)it.g * 2 * NINT;
  u64 mask[2 * NINT];
#pragma unroll
  for (int w = 0; w < 2 * NINT; ++w) mask[w] = gd[w];
  if (it.kind == IT_SINGLE) {
    set_orb(mask, NINT, it.spin, it.h1, false);
  } else if (it.kind == IT_SAME) {
    set_orb(mask, NINT, it.spin, it.h1, false);
    set_orb(mask, NINT, it.spin, it.h2, false);
  } else {
    set_orb(mask, NINT, 0, it.h1, false);
    set_orb(mask, NINT, 1, it.h2, false);
  }
  if (tid < 2) {
    int c = 0;
    for (int o = 1; o <= n; ++o)
      if (!has_orb(gd, NINT, tid, o)) vir[tid][c++] = o;
    nvir[tid] = c;
  }
  if (tid == 0) nfg = 0;
  __syncthreads();
  // the earlier generators that can reach a determinant of this item
  {
    const int64_t f0 = A.flist_off[it.gl], f1 = A.flist_off[it.gl + 1];
    for (int64_t f = f0 + tid; f < f1; f += SBLK) {
      const int gp = A.flist[f];
      const u64* q = A.dets + (int64_t)gp * 2 * NINT;
      int k = 0;
#pragma unroll
      for (int w = 0; w < 2 * NINT; ++w) k += popc64(mask[w] & ~q[w]);
      if (k <= 2) {
        const int slot = atomicAdd(&nfg, 1);
        if (slot < SEL_MAXFG) fgen[slot] = gp;  // past SEL_MAXFG the bans read the global list
      }
    }
  }
  // owned entries: e = it.e0 + tid + j SBLK
  const int ne = it.e1 - it.e0;
  for (int x = tid; x < ne * nst; x += SBLK) tile[x] = 0.0;
  __syncthreads();
  const int sp1 = it.kind == IT_AB ? 0 : it.spin;  // spin of particle 1
  const int sp2 = it.kind == IT_AB ? 1 : it.spin;  // spin of particle 2
  auto particles = [&](int e, int& p1, int& p2) {
    if (it.kind == IT_SINGLE) {
      p1 = vir[it.spin][e];
      p2 = 0;
    } else if (it.kind == IT_SAME) {
      int i1, i2;
      tri_decode(e, i1, i2);
      p1 = vir[it.spin][i1];
      p2 = vir[it.spin][i2];
    } else {
      const int nb = nvir[1];
      p1 = vir[0][e / nb];
      p2 = vir[1][e % nb];
    }
  };
  const int64_t i0 = A.ilist_off[it.gl], i1 = A.ilist_off[it.gl + 1];
  for (int64_t base = i0; base < i1; base += SEL_DTILE) {
    // stage the selectors of this pass with k = |mask \ D| <= 2, in order
    if (tid == 0) nsel_s = 0;
    __syncthreads();
    for (int sub = 0; sub < SEL_DTILE; sub += SBLK) {
      const int64_t q = base + sub + tid;
      int D = -1, k = 3;
      if (q < i1) {
        D = A.ilist[q];
        const u64* dd = A.dets + (int64_t)D * 2 * NINT;
        k = 0;
#pragma unroll
        for (int w = 0; w < 2 * NINT; ++w) k += popc64(mask[w] & ~dd[w]);
      }
      const bool keep = k <= 2;
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) wsum[warp] = __popc(bal);
      __syncthreads();
      int pos = nsel_s;
      for (int w = 0; w < warp; ++w) pos += wsum[w];
      pos += __popc(bal & ((1u << lane) - 1));
      if (keep) {
        const u64* dd = A.dets + (int64_t)D * 2 * NINT;
#pragma unroll
        for (int w = 0; w < 2 * NINT; ++w) sdet[pos][w] = dd[w];
        sidx[pos] = D;
        sk[pos] = (unsigned char)k;
      }
      __syncthreads();
      if (tid == 0) {
        int tot = 0;
        for (int w = 0; w < SBLK / 32; ++w) tot += wsum[w];
        nsel_s += tot;
      }
      __syncthreads();
    }
    const int ns = nsel_s;
    // every thread: its entries against the staged selectors, in order
    for (int e = tid; e < ne; e += SBLK) {
      int p1, p2;
      particles(it.e0 + e, p1, p2);
      u64 a[2 * NINT];
#pragma unroll
      for (int w = 0; w < 2 * NINT; ++w) a[w] = mask[w];
      set_orb(a, NINT, sp1, p1, true);
      if (it.kind != IT_SINGLE) set_orb(a, NINT, sp2, p2, true);
      double* m = tile + (size_t)e * nst;
      for (int j = 0; j < ns; ++j) {
        const u64* dd = sdet[j];
        int deg = sk[j] + (has_orb(dd, NINT, sp1, p1) ? 0 : 1);
        if (it.kind != IT_SINGLE) deg += has_orb(dd, NINT, sp2, p2) ? 0 : 1;
        if (deg > 2 || deg == 0) continue;  // deg 0: a = D, in the wave function
        u64 Dw[2 * NINT];
#pragma unroll
        for (int w = 0; w < 2 * NINT; ++w) Dw[w] = dd[w];
        const double h = ihj<NINT>(A.t, a, Dw);
        const double* cD = A.coef + (int64_t)sidx[j] * nst;
        for (int s = 0; s < nst; ++s) m[s] = fma(__ldg(&cD[s]), h, m[s]);
      }
    }
    __syncthreads();
  }
  // energies of this thread's entries
  double pt[SEL_MAXST];
#pragma unroll
  for (int s = 0; s < SEL_MAXST; ++s) pt[s] = 0.0;
  const int st = n + 2;
  const double* F = A.fock + (int64_t)it.gl * 2 * st;
  const double eg = F[n + 1];
  unsigned long long next = 0;
  for (int e = tid; e < ne; e += SBLK) {
    const double* m = tile + (size_t)e * nst;
    double sabs = 0.0;
    for (int s = 0; s < nst; ++s) sabs += fabs(m[s]);
    if (sabs == 0.0) continue;
    int p1, p2;
    particles(it.e0 + e, p1, p2);
    u64 a[2 * NINT];
#pragma unroll
    for (int w = 0; w < 2 * NINT; ++w) a[w] = mask[w];
    set_orb(a, NINT, sp1, p1, true);
    if (it.kind != IT_SINGLE) set_orb(a, NINT, sp2, p2, true);
    bool banned = in_wf<NINT>(A, a);
    if (nfg <= SEL_MAXFG) {
      for (int f = 0; f < nfg && !banned; ++f) banned = exc_deg<NINT>(a, A.dets + (int64_t)fgen[f] * 2 * NINT) <= 2;
    } else {  // more earlier generators reach this item than the shared list holds
      for (int64_t f = A.flist_off[it.gl]; f < A.flist_off[it.gl + 1] && !banned; ++f)
        banned = exc_deg<NINT>(a, A.dets + (int64_t)A.flist[f] * 2 * NINT) <= 2;
    }
    if (banned) continue;
    ++next;
    // diag_H_mat_elem_fock (slater_rules.irp.f:1800-1866); holes and
    // particles ascending within a spin, as decode_exc lists them
    double haa;
    const double* Fa = F;
    const double* Fb = F + st;
    if (it.kind == IT_SINGLE) {
      const double* Fs = it.spin ? Fb : Fa;
      haa = eg - Fs[it.h1] + (Fs[p1] - tab2(A.t.ja, n, it.h1, p1));
    } else if (it.kind == IT_SAME) {
      const double* Fs = it.spin ? Fb : Fa;
      const int h1 = it.h1, h2 = it.h2;  // h1 < h2, p1 < p2
      haa = eg - Fs[h1] + (Fs[p1] - tab2(A.t.ja, n, h1, p1)) -
            (Fs[h2] - tab2(A.t.ja, n, h1, h2) + tab2(A.t.ja, n, p1, h2)) +
            (Fs[p2] - tab2(A.t.ja, n, h1, p2) + tab2(A.t.ja, n, p1, p2) - tab2(A.t.ja, n, h2, p2));
    } else {
      const int h1 = it.h1, h2 = it.h2;
      haa = eg - Fa[h1] + (Fa[p1] - tab2(A.t.ja, n, h1, p1)) -
            (Fb[h2] - tab2(A.t.jj, n, h1, h2) + tab2(A.t.jj, n, p1, h2)) +
            (Fb[p2] - tab2(A.t.jj, n, h1, p2) + tab2(A.t.jj, n, p1, p2) - tab2(A.t.ja, n, h2, p2));
    }
    double mine = 0.0;
    for (int s = 0; s < nst; ++s) {
      const double delta = A.e0[s] - haa;
      const double val = m[s] + m[s];
      double tmp = sqrt(delta * delta + val * val);
      if (delta < 0.0) tmp = -tmp;
      const double ev = 0.5 * (tmp - delta);
      pt[s] += ev;
      mine = fmin(ev, mine);
    }
    const unsigned long long slot = atomicAdd(A.n_cand, 1ull);
    if (slot < A.cap) {
      A.cand_val[slot] = mine;
#pragma unroll
      for (int w = 0; w < 2 * NINT; ++w) A.cand_det[slot * 2 * NINT + w] = a[w];
    }
  }
  if (next) atomicAdd(A.n_ext, next);
  // the numerator tile is free now: it holds the per-thread sums (the
  // dynamic allocation is at least SBLK x n_st doubles)
  __syncthreads();
  for (int s = 0; s < nst; ++s) tile[tid * nst + s] = pt[s];
  __syncthreads();
  if (tid < nst) {
    double acc = 0.0;
    for (int x = 0; x < SBLK; ++x) acc += tile[x * nst + tid];
    A.pt2_part[(int64_t)blockIdx.x * nst + tid] = acc;
  }
}

// pt2[s] = sum over items, in order
__global__ void k_sel_pt2(const double* part, int64_t n_items, int nst, double* pt2) {
  const int s = threadIdx.x;
  if (s >= nst) return;
  double acc = 0.0;
  for (int64_t i = 0; i < n_items; ++i) acc += part[i * nst + s];
  pt2[s] = acc;
}

// ascending order of doubles as unsigned keys
__global__ void k_sel_keys(const double* v, uint64_t n, unsigned long long* key, long long* idx) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v[i]);
    key[i] = (b >> 63) ? ~b : (b | (1ull << 63));
    idx[i] = (long long)i;
  }
}

// the head of the sorted candidates, contiguous
__global__ void k_sel_gather(const long long* idx, uint64_t take, const double* cval, const u64* cdet, int w2,
                             double* vals, u64* dets) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < take; i += (uint64_t)gridDim.x * blockDim.x) {
    const long long j = idx[i];
    vals[i] = cval[j];
    for (int w = 0; w < w2; ++w) dets[i * w2 + w] = cdet[j * w2 + w];
  }
}

struct Dev {
  void* p = nullptr;
  ~Dev() { dev_free(p); }
};

}  // namespace

// The selection over the listed generators (psi_det indices, each banned by
// every generator before it, listed or not).  pt2 (n_st) sums all of them;
// per_gen (n_list x n_st, optional) holds each generator's share, summed over
// its items in order.  The buffer as qpgpu_select_pt2.  Returns the number of
// buffer entries written or a negative status.
static int run_selection(qpgpu_ctx* c, const double* coef, int n_st, const double* e0, int n_sel,
                         const std::vector<int>& gens, int buf_size, double* pt2, double* per_gen,
                         uint64_t* buf_dets, double* buf_vals, int64_t* n_ext) {
  const int64_t N = c->N;
  const int nint = c->nint, n = c->n_mo;
  const int n_list = (int)gens.size();
  cudaStream_t st = c->stream;
  // host copies of the listed generators (item list)
  std::vector<u64> gdet((size_t)n_list * 2 * nint);
  for (int l = 0; l < n_list; ++l)
    QP_CUDA(c, cudaMemcpyAsync(&gdet[(size_t)l * 2 * nint], c->d_dets + (int64_t)gens[l] * 2 * nint,
                               2 * nint * sizeof(u64), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  const int tile_entries = SEL_TILE / n_st;
  std::vector<SelItem> items;
  std::vector<int64_t> item_first(n_list + 1);
  auto push = [&](SelItem it, int ne) {
    for (int a = 0; a < ne; a += tile_entries) {
      it.e0 = a;
      it.e1 = std::min(ne, a + tile_entries);
      items.push_back(it);
    }
  };
  for (int l = 0; l < n_list; ++l) {
    item_first[l] = (int64_t)items.size();
    const int g = gens[l];
    std::vector<int> occ[2];
    for (int s = 0; s < 2; ++s)
      for (int o = 1; o <= n; ++o)
        if ((gdet[(size_t)l * 2 * nint + s * nint + ((o - 1) >> 6)] >> ((o - 1) & 63)) & 1ull) occ[s].push_back(o);
    const int nv[2] = {n - (int)occ[0].size(), n - (int)occ[1].size()};
    for (int s = 0; s < 2; ++s)
      for (int h : occ[s]) push(SelItem{g, l, IT_SINGLE, s, h, 0, 0, 0}, nv[s]);
    for (int s = 0; s < 2; ++s)
      for (size_t x = 0; x < occ[s].size(); ++x)
        for (size_t y = x + 1; y < occ[s].size(); ++y)
          push(SelItem{g, l, IT_SAME, s, occ[s][x], occ[s][y], 0, 0}, nv[s] * (nv[s] - 1) / 2);
    for (int ha : occ[0])
      for (int hb : occ[1]) push(SelItem{g, l, IT_AB, 0, ha, hb, 0, 0}, nv[0] * nv[1]);
  }
  item_first[n_list] = (int64_t)items.size();
  const int64_t n_items = (int64_t)items.size();
  for (int s = 0; s < n_st; ++s) pt2[s] = 0.0;
  if (n_ext) *n_ext = 0;
  if (n_items == 0) {
    if (per_gen)
      for (size_t x = 0; x < (size_t)n_list * n_st; ++x) per_gen[x] = 0.0;
    return 0;
  }
  // device arrays
  Dev d_items, d_gens, d_coef, d_e0, d_icnt, d_ioff, d_ilist, d_fcnt, d_foff, d_flist, d_fock, d_slot, d_part, d_cnt,
      d_err, d_pt2;
  uint64_t hcap = 1;
  while (hcap < (uint64_t)(2 * N)) hcap <<= 1;
  QP_CUDA(c, cudaMalloc(&d_items.p, items.size() * sizeof(SelItem)));
  QP_CUDA(c, cudaMemcpyAsync(d_items.p, items.data(), items.size() * sizeof(SelItem), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMalloc(&d_gens.p, n_list * sizeof(int)));
  QP_CUDA(c, cudaMemcpyAsync(d_gens.p, gens.data(), n_list * sizeof(int), cudaMemcpyHostToDevice, st));
  // coefficients: column-major (N, n_st) on the host -> (N, n_st) row-major
  std::vector<double> crow((size_t)N * n_st);
  for (int s = 0; s < n_st; ++s)
    for (int64_t i = 0; i < N; ++i) crow[(size_t)i * n_st + s] = coef[(size_t)s * N + i];
  QP_CUDA(c, cudaMalloc(&d_coef.p, crow.size() * sizeof(double)));
  QP_CUDA(c, cudaMemcpyAsync(d_coef.p, crow.data(), crow.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMalloc(&d_e0.p, n_st * sizeof(double)));
  QP_CUDA(c, cudaMemcpyAsync(d_e0.p, e0, n_st * sizeof(double), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMalloc(&d_slot.p, hcap * sizeof(int)));
  QP_CUDA(c, cudaMemsetAsync(d_slot.p, 0xff, hcap * sizeof(int), st));
  QP_CUDA(c, cudaMalloc(&d_fock.p, (size_t)n_list * 2 * (n + 2) * sizeof(double)));
  QP_CUDA(c, cudaMalloc(&d_icnt.p, (n_list + 1) * sizeof(int64_t)));
  QP_CUDA(c, cudaMalloc(&d_fcnt.p, (n_list + 1) * sizeof(int64_t)));
  QP_CUDA(c, cudaMalloc(&d_cnt.p, 2 * sizeof(unsigned long long)));
  QP_CUDA(c, cudaMalloc(&d_err.p, sizeof(int)));
  QP_CUDA(c, cudaMemsetAsync(d_err.p, 0, sizeof(int), st));
  QP_CUDA(c, cudaMalloc(&d_pt2.p, n_st * sizeof(double)));
  QP_CUDA(c, cudaMalloc(&d_part.p, (size_t)n_items * n_st * sizeof(double)));
  const u64* dets = c->d_dets;
  const int* dg = (const int*)d_gens.p;
  const int hb = (int)std::min<int64_t>((N + 255) / 256, (int64_t)c->n_sm * 8);
#define QP_SEL_NINT(NI)                                                                                          \
  k_hash_insert<NI><<<hb, 256, 0, st>>>(dets, N, (int*)d_slot.p, hcap - 1);                                     \
  k_sel_lists<NI><<<n_list, SBLK, 0, st>>>(dets, dg, n_list, n_sel, 0, 0, (int64_t*)d_icnt.p, nullptr, nullptr); \
  k_sel_lists<NI><<<n_list, SBLK, 0, st>>>(dets, dg, n_list, n_sel, 1, 0, (int64_t*)d_fcnt.p, nullptr, nullptr); \
  k_sel_fock<NI><<<(n_list + 63) / 64, 64, 0, st>>>(c->tab, dets, dg, n_list, (double*)d_fock.p);
  if (nint == 1) {
    QP_SEL_NINT(1)
  } else {
    QP_SEL_NINT(2)
  }
#undef QP_SEL_NINT
  QP_CUDA(c, cudaGetLastError());
  // list offsets on the host
  std::vector<int64_t> icnt(n_list), fcnt(n_list), ioff(n_list + 1), foff(n_list + 1);
  QP_CUDA(c, cudaMemcpyAsync(icnt.data(), d_icnt.p, n_list * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaMemcpyAsync(fcnt.data(), d_fcnt.p, n_list * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  ioff[0] = foff[0] = 0;
  for (int l = 0; l < n_list; ++l) {
    ioff[l + 1] = ioff[l] + icnt[l];
    foff[l + 1] = foff[l] + fcnt[l];
  }
  QP_CUDA(c, cudaMalloc(&d_ioff.p, (n_list + 1) * sizeof(int64_t)));
  QP_CUDA(c, cudaMalloc(&d_foff.p, (n_list + 1) * sizeof(int64_t)));
  QP_CUDA(c, cudaMemcpyAsync(d_ioff.p, ioff.data(), (n_list + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMemcpyAsync(d_foff.p, foff.data(), (n_list + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMalloc(&d_ilist.p, std::max<int64_t>(1, ioff[n_list]) * sizeof(int)));
  QP_CUDA(c, cudaMalloc(&d_flist.p, std::max<int64_t>(1, foff[n_list]) * sizeof(int)));
  // candidates (only when a buffer is asked for): at most one per entry
  uint64_t ub = 0;
  for (const SelItem& it : items) ub += (uint64_t)(it.e1 - it.e0);
  uint64_t cap = buf_size > 0 ? std::min<uint64_t>(ub, 1ull << 28) : 0;  // <= 10.7 GB of candidates
  Dev d_cval, d_cdet;
  SelArgs A{};
  A.t = c->tab;
  A.dets = dets;
  A.coef = (const double*)d_coef.p;
  A.e0 = (const double*)d_e0.p;
  A.n_st = n_st;
  A.N = N;
  A.items = (const SelItem*)d_items.p;
  A.ilist_off = (const int64_t*)d_ioff.p;
  A.ilist = (const int*)d_ilist.p;
  A.flist_off = (const int64_t*)d_foff.p;
  A.flist = (const int*)d_flist.p;
  A.fock = (const double*)d_fock.p;
  A.hslot = (const int*)d_slot.p;
  A.hmask = hcap - 1;
  A.pt2_part = (double*)d_part.p;
  A.n_ext = (unsigned long long*)d_cnt.p;
  A.n_cand = (unsigned long long*)d_cnt.p + 1;
  A.err = (int*)d_err.p;
  // dynamic shared memory: the largest item's numerator tile (at least the
  // SBLK x n_st doubles of the final reduction), so that several CTAs fit an SM
  int max_ne = 0;
  for (const SelItem& it : items) max_ne = std::max(max_ne, it.e1 - it.e0);
  const size_t smem = (size_t)std::max(max_ne * n_st, SBLK * n_st) * sizeof(double);
  unsigned long long hcnt[2] = {0, 0};
  for (int attempt = 0; attempt < 2; ++attempt) {
    dev_free(d_cval.p);
    dev_free(d_cdet.p);
    d_cval.p = d_cdet.p = nullptr;
    QP_CUDA(c, cudaMalloc(&d_cval.p, std::max<uint64_t>(1, cap) * sizeof(double)));
    QP_CUDA(c, cudaMalloc(&d_cdet.p, std::max<uint64_t>(1, cap) * 2 * nint * sizeof(u64)));
    A.cap = cap;
    A.cand_val = (double*)d_cval.p;
    A.cand_det = (u64*)d_cdet.p;
    QP_CUDA(c, cudaMemsetAsync(d_cnt.p, 0, 2 * sizeof(unsigned long long), st));
#define QP_SEL_RUN(NI)                                                                                             \
  k_sel_lists<NI><<<n_list, SBLK, 0, st>>>(dets, dg, n_list, n_sel, 0, 1, nullptr, (const int64_t*)d_ioff.p,       \
                                           (int*)d_ilist.p);                                                       \
  k_sel_lists<NI><<<n_list, SBLK, 0, st>>>(dets, dg, n_list, n_sel, 1, 1, nullptr, (const int64_t*)d_foff.p,       \
                                           (int*)d_flist.p);                                                       \
  QP_CUDA(c, cudaFuncSetAttribute(k_sel_items<NI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));       \
  k_sel_items<NI><<<(unsigned)n_items, SBLK, smem, st>>>(A);
    if (nint == 1) {
      QP_SEL_RUN(1)
    } else {
      QP_SEL_RUN(2)
    }
#undef QP_SEL_RUN
    QP_CUDA(c, cudaGetLastError());
    QP_CUDA(c, cudaMemcpyAsync(hcnt, d_cnt.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    if (buf_size == 0 || hcnt[1] <= cap) break;
    cap = hcnt[1];  // every candidate counted: run once more with room for all of them
  }
  k_sel_pt2<<<1, 32, 0, st>>>((const double*)d_part.p, n_items, n_st, (double*)d_pt2.p);
  QP_CUDA(c, cudaMemcpyAsync(pt2, d_pt2.p, n_st * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (per_gen) {
    std::vector<double> part((size_t)n_items * n_st);
    QP_CUDA(c, cudaMemcpyAsync(part.data(), d_part.p, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    for (int l = 0; l < n_list; ++l)
      for (int s = 0; s < n_st; ++s) {
        double acc = 0.0;
        for (int64_t i = item_first[l]; i < item_first[l + 1]; ++i) acc += part[(size_t)i * n_st + s];
        per_gen[(size_t)l * n_st + s] = acc;
      }
  }
  if (n_ext) *n_ext = (int64_t)hcnt[0];
  const uint64_t nc = std::min<uint64_t>(hcnt[1], cap);
  int nout = (int)std::min<uint64_t>(nc, (uint64_t)buf_size);
  if (nout > 0) {
    // sort by value on the device; the head (and any tie group crossing its
    // end) goes to the host, where equal values are put in determinant order
    Dev kin, kout, vin, vout, tmp;
    QP_CUDA(c, cudaMalloc(&kin.p, nc * 8));
    QP_CUDA(c, cudaMalloc(&kout.p, nc * 8));
    QP_CUDA(c, cudaMalloc(&vin.p, nc * 8));
    QP_CUDA(c, cudaMalloc(&vout.p, nc * 8));
    k_sel_keys<<<(unsigned)std::min<uint64_t>((nc + 255) / 256, (uint64_t)c->n_sm * 8), 256, 0, st>>>(
        (const double*)d_cval.p, nc, (unsigned long long*)kin.p, (long long*)vin.p);
    size_t tb = 0;
    QP_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned long long*)kin.p, (unsigned long long*)kout.p,
                                               (long long*)vin.p, (long long*)vout.p, (int64_t)nc, 0, 64, st));
    QP_CUDA(c, cudaMalloc(&tmp.p, tb));
    QP_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, (unsigned long long*)kin.p, (unsigned long long*)kout.p,
                                               (long long*)vin.p, (long long*)vout.p, (int64_t)nc, 0, 64, st));
    std::vector<unsigned long long> keys;
    uint64_t take = std::min<uint64_t>(nc, (uint64_t)nout + 64);
    while (true) {  // grow the head until it ends past the tie group of entry nout - 1
      keys.resize(take);
      QP_CUDA(c, cudaMemcpyAsync(keys.data(), kout.p, take * 8, cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaStreamSynchronize(st));
      if (take == nc || keys[take - 1] != keys[nout - 1]) break;
      take = std::min<uint64_t>(nc, take * 2);
    }
    std::vector<double> vals(take);
    std::vector<u64> dts(take * 2 * nint);
    Dev gv, gd;
    QP_CUDA(c, cudaMalloc(&gv.p, take * sizeof(double)));
    QP_CUDA(c, cudaMalloc(&gd.p, take * 2 * nint * sizeof(u64)));
    k_sel_gather<<<(unsigned)std::min<uint64_t>((take + 255) / 256, (uint64_t)c->n_sm * 8), 256, 0, st>>>(
        (const long long*)vout.p, take, (const double*)d_cval.p, (const u64*)d_cdet.p, 2 * nint, (double*)gv.p,
        (u64*)gd.p);
    QP_CUDA(c, cudaMemcpyAsync(vals.data(), gv.p, take * sizeof(double), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaMemcpyAsync(dts.data(), gd.p, take * 2 * nint * sizeof(u64), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    std::vector<uint64_t> ord(take);
    for (uint64_t i = 0; i < take; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](uint64_t x, uint64_t y) {
      if (vals[x] != vals[y]) return vals[x] < vals[y];
      for (int w = 0; w < 2 * nint; ++w)
        if (dts[x * 2 * nint + w] != dts[y * 2 * nint + w]) return dts[x * 2 * nint + w] < dts[y * 2 * nint + w];
      return false;
    });
    for (int i = 0; i < nout; ++i) {
      buf_vals[i] = vals[ord[i]];
      for (int w = 0; w < 2 * nint; ++w) buf_dets[(size_t)i * 2 * nint + w] = dts[ord[i] * 2 * nint + w];
    }
  }
  QP_CUDA(c, cudaStreamSynchronize(st));
  return nout;
}

extern "C" int qpgpu_select_pt2(qpgpu_ctx* c, const double* coef, int n_st, const double* e0, int n_gen, int n_sel,
                                int buf_size, double* pt2, uint64_t* buf_dets, double* buf_vals, int64_t* n_ext) {
  if (!c) return QPGPU_ERR_ARG;
  if (!coef || !e0 || !pt2 || n_st < 1 || n_st > SEL_MAXST || buf_size < 0 ||
      (buf_size > 0 && (!buf_dets || !buf_vals)))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "select_pt2: bad arguments (1 <= n_st <= 8, buffers for buf_size > 0)");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->have_ints || !c->have_dets)
    return qpgpu_fail(c, QPGPU_ERR_STATE, "select_pt2: integrals and determinants first");
  if (n_gen < 1 || n_gen > n_sel || n_sel > c->N)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "select_pt2: need 1 <= n_gen <= n_sel <= N_det");
  std::vector<int> gens(n_gen);
  for (int g = 0; g < n_gen; ++g) gens[g] = g;
  return run_selection(c, coef, n_st, e0, n_sel, gens, buf_size, pt2, nullptr, buf_dets, buf_vals, n_ext);
}

extern "C" int qpgpu_pt2_generators(qpgpu_ctx* c, const double* coef, int n_st, const double* e0, int n_sel,
                                    const int32_t* gens, int n_list, double* pt2_detail) {
  if (!c) return QPGPU_ERR_ARG;
  if (!coef || !e0 || !gens || !pt2_detail || n_st < 1 || n_st > SEL_MAXST || n_list < 0)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "pt2_generators: bad arguments (1 <= n_st <= 8)");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->have_ints || !c->have_dets)
    return qpgpu_fail(c, QPGPU_ERR_STATE, "pt2_generators: integrals and determinants first");
  if (n_sel < 1 || n_sel > c->N) return qpgpu_fail(c, QPGPU_ERR_ARG, "pt2_generators: need 1 <= n_sel <= N_det");
  std::vector<int> g(gens, gens + n_list);
  for (int x : g)
    if (x < 0 || x >= n_sel) return qpgpu_fail(c, QPGPU_ERR_ARG, "pt2_generators: generator outside 0..n_sel-1");
  if (n_list == 0) return QPGPU_OK;
  std::vector<double> tot(n_st);
  const int rc = run_selection(c, coef, n_st, e0, n_sel, g, 0, tot.data(), pt2_detail, nullptr, nullptr, nullptr);
  return rc < 0 ? rc : QPGPU_OK;
}
