// Internal declarations of the GB300 sigma library (not part of the C-ABI).
//
// Orbitals are 1-based as in Quantum Package: orbital p is bit (p-1)%64 of
// word (p-1)/64.  Determinants are psi_det(N_int,2,N): det[k*2*nint + s*nint + w].
// Every device routine that computes a matrix element follows the FP64
// operation order of the reference routine it cites, so FP64 matrix elements
// are bit-identical to the restatement of that routine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/qpgpu.h"

typedef unsigned long long u64;

#define QPGPU_MAX_NINT 2  // n_mo <= 128
#define QPGPU_MAX_MO (64 * QPGPU_MAX_NINT)

// ---------------------------------------------------------------------------
// Device integral tables (set by qpgpu_set_integrals)
// ---------------------------------------------------------------------------
struct DevTables {
  int n, nint, na, nb;
  const double* eri;   // chemist (pq|rs) at bielec_integrals_index key - 1
  const double* h;     // h(i,j) col-major
  const double* jj;    // mo_bielec_integral_jj(i,j)       (n*n col-major)
  const double* ja;    // mo_bielec_integral_jj_anti(i,j)
  const double* bc;    // big_array_coulomb_integrals(i,h,p), i fastest
  const double* bx;    // big_array_exchange_integrals(i,h,p)
  const double* fock;  // fock_operator_closed_shell_ref_bitmask(i,j)
  u64 ref[2 * QPGPU_MAX_NINT];     // ref_bitmask (alpha words, then beta words)
  u64 ref_cs[2 * QPGPU_MAX_NINT];  // ref_closed_shell_bitmask
  double e_ref;                    // ref_bitmask_energy
};

__host__ __device__ inline long long pair_idx(long long i, long long j) {
  long long p = i < j ? i : j, r = i < j ? j : i;
  return p + ((r * r - r) >> 1);
}

#ifdef __CUDACC__
// <ij|kl> physicist = (ik|jl) chemist  (get_mo_bielec_integral,
// src/Integrals_Bielec/map_integrals.irp.f:383-413; dense-cache path)
__device__ __forceinline__ double get_int(const DevTables& t, int i, int j, int k, int l) {
  return __ldg(&t.eri[pair_idx(pair_idx(i, k), pair_idx(j, l)) - 1]);
}
__device__ __forceinline__ double tab2(const double* a, int n, int i, int j) {
  return __ldg(&a[(i - 1) + (size_t)(j - 1) * n]);
}
__device__ __forceinline__ double tab3(const double* a, int n, int x, int y, int z) {
  return __ldg(&a[(x - 1) + (size_t)n * ((y - 1) + (size_t)n * (z - 1))]);
}

__device__ __forceinline__ int popc64(u64 x) { return __popcll(x); }
__device__ __forceinline__ int ctz64(u64 x) { return __ffsll((long long)x) - 1; }

// Electrons of det1 strictly between orbitals low < high (1-based), the nperm
// term of get_mono/double_excitation_spin (slater_rules.irp.f:2837-2860,2954-2969)
template <int NINT>
__device__ __forceinline__ int nperm_between(const u64* det1, int low, int high) {
  int j = (low - 1) >> 6, n = ((low - 1) & 63) + 1;
  int k = (high - 1) >> 6, m = ((high - 1) & 63) + 1;
  int np = 0;
  if (j == k) {
    u64 mask = ((1ull << (m - 1)) - 1ull) & (0ull - (1ull << n));
    np += popc64(det1[j] & mask);
  } else {
    np += popc64(det1[k] & ((1ull << (m - 1)) - 1ull));
    if (n < 64) np += popc64(det1[j] & (0ull - (1ull << n)));
#pragma unroll
    for (int i = 0; i < NINT; ++i)
      if (i > j && i < k) np += popc64(det1[i]);
  }
  return np;
}

// get_mono_excitation_spin, slater_rules.irp.f:2913-2987 (hole in d1, particle in d2)
template <int NINT>
__device__ __forceinline__ int mono_exc_spin(const u64* d1, const u64* d2, int* hole, int* part) {
  int h = 0, p = 0;
#pragma unroll
  for (int l = 0; l < NINT; ++l) {
    u64 tmp = d1[l] ^ d2[l];
    u64 particle = tmp & d2[l];
    u64 hl = tmp & d1[l];
    if (particle) p = ctz64(particle) + 1 + 64 * l;
    if (hl) h = ctz64(hl) + 1 + 64 * l;
  }
  *hole = h;
  *part = p;
  int low = h < p ? h : p, high = h < p ? p : h;
  return nperm_between<NINT>(d1, low, high) & 1;  // 1 => phase -1
}

// get_double_excitation_spin, slater_rules.irp.f:2783-2911 (holes/particles ascending)
template <int NINT>
__device__ __forceinline__ int double_exc_spin(const u64* d1, const u64* d2, int* h, int* p) {
  int ih = 0, ip = 0;
  h[0] = h[1] = p[0] = p[1] = 0;
#pragma unroll
  for (int l = 0; l < NINT; ++l) {
    u64 tmp = d1[l] ^ d2[l];
    u64 particle = tmp & d2[l];
    u64 hl = tmp & d1[l];
    while (particle) {
      if (ip < 2) p[ip] = ctz64(particle) + 1 + 64 * l;
      ++ip;
      particle &= particle - 1;
    }
    while (hl) {
      if (ih < 2) h[ih] = ctz64(hl) + 1 + 64 * l;
      ++ih;
      hl &= hl - 1;
    }
  }
  int np = 0;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    int low = h[i] < p[i] ? h[i] : p[i], high = h[i] < p[i] ? p[i] : h[i];
    np += nperm_between<NINT>(d1, low, high);
  }
  int a = min(h[0], p[0]), b = max(h[0], p[0]);
  int c = min(h[1], p[1]), d = max(h[1], p[1]);
  if (c > a && c < b && d > b) np += 1;
  return np & 1;
}

// get_mono_excitation_from_fock, src/Determinants/mono_excitations.irp.f:97-155
// det1: (nint,2) row determinant I.
template <int NINT>
__device__ __forceinline__ double mono_from_fock(const DevTables& t, const u64* det1, int h, int p,
                                                 int spin, int neg) {
  const int n = t.n;
  u64 hole[2][NINT], partcl[2][NINT];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int i = 0; i < NINT; ++i) {
      u64 diff = det1[s * NINT + i] ^ t.ref_cs[s * NINT + i];
      hole[s][i] = diff & t.ref_cs[s * NINT + i];
      partcl[s][i] = diff & det1[s * NINT + i];
    }
  double hij = tab2(t.fock, n, h, p);
  // holes: direct terms (alpha then beta), exchange terms (same spin)
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int w = 0; w < NINT; ++w)
      for (u64 x = hole[s][w]; x; x &= x - 1) hij = __dsub_rn(hij, tab3(t.bc, n, ctz64(x) + 1 + 64 * w, h, p));
#pragma unroll
  for (int w = 0; w < NINT; ++w)
    for (u64 x = hole[spin - 1][w]; x; x &= x - 1) hij = __dadd_rn(hij, tab3(t.bx, n, ctz64(x) + 1 + 64 * w, h, p));
  // particles: direct terms, exchange terms
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int w = 0; w < NINT; ++w)
      for (u64 x = partcl[s][w]; x; x &= x - 1) hij = __dadd_rn(hij, tab3(t.bc, n, ctz64(x) + 1 + 64 * w, h, p));
#pragma unroll
  for (int w = 0; w < NINT; ++w)
    for (u64 x = partcl[spin - 1][w]; x; x &= x - 1) hij = __dsub_rn(hij, tab3(t.bx, n, ctz64(x) + 1 + 64 * w, h, p));
  return neg ? -hij : hij;
}

// i_H_j_double_spin, slater_rules.irp.f:3008-3035 (si, sj: spin strings)
template <int NINT>
__device__ __forceinline__ double h_double_spin(const DevTables& t, const u64* si, const u64* sj, int* exc4,
                                                int* neg_out) {
  int h[2], p[2];
  int neg = double_exc_spin<NINT>(si, sj, h, p);
  double v = __dsub_rn(get_int(t, h[0], h[1], p[0], p[1]), get_int(t, h[0], h[1], p[1], p[0]));
  if (exc4) { exc4[0] = h[0]; exc4[1] = p[0]; exc4[2] = h[1]; exc4[3] = p[1]; }
  if (neg_out) *neg_out = neg;
  return neg ? -v : v;
}

// i_H_j_double_alpha_beta, slater_rules.irp.f:3037-3067.  The reference's
// big_array_exchange shortcuts (:3056-3060) read the same packed entry as the
// general lookup, so the general lookup is used for every case.
// Also returns <I|S+S-|J> of get_s2 (s2.irp.f:32-63): -phase when the alpha and
// beta excitations swap the same two orbitals, else 0.  (The phase of the
// reverse excitation J->I that get_s2 uses equals that of I->J: the electrons
// strictly between hole and particle are the same in I and J.)
template <int NINT>
__device__ __forceinline__ double h_double_ab(const DevTables& t, const u64* ki, const u64* kj, double* s2,
                                              int* exc4, int* neg_out) {
  int ha, pa, hb, pb;
  int na = mono_exc_spin<NINT>(ki, kj, &ha, &pa);
  int nb = mono_exc_spin<NINT>(ki + NINT, kj + NINT, &hb, &pb);
  int neg = na ^ nb;
  double v = get_int(t, ha, hb, pa, pb);
  *s2 = (pa == hb && pb == ha) ? (neg ? 1.0 : -1.0) : 0.0;
  if (exc4) { exc4[0] = ha; exc4[1] = pa; exc4[2] = hb; exc4[3] = pb; }
  if (neg_out) *neg_out = neg;
  return neg ? -v : v;
}

// i_H_j_mono_spin, slater_rules.irp.f:2989-3006 (ki, kj: (nint,2))
template <int NINT>
__device__ __forceinline__ double h_mono_spin(const DevTables& t, const u64* ki, const u64* kj, int spin,
                                              int* exc4, int* neg_out) {
  int h, p;
  int neg = mono_exc_spin<NINT>(ki + (spin - 1) * NINT, kj + (spin - 1) * NINT, &h, &p);
  if (exc4) { exc4[0] = h; exc4[1] = p; exc4[2] = 0; exc4[3] = 0; }
  if (neg_out) *neg_out = neg;
  return mono_from_fock<NINT>(t, ki, h, p, spin, neg);
}

// diag_H_mat_elem with a_operator / ac_operator, slater_rules.irp.f:1869-2022
template <int NINT>
__device__ __forceinline__ double diag_h(const DevTables& t, const u64* det) {
  const int n = t.n;
  u64 hole[2][NINT], particle[2][NINT];
  int nexc = 0;
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int i = 0; i < NINT; ++i) {
      u64 x = det[s * NINT + i] ^ t.ref[s * NINT + i];
      particle[s][i] = x & det[s * NINT + i];
      hole[s][i] = x & t.ref[s * NINT + i];
      nexc += popc64(hole[s][i]);
    }
  double e = t.e_ref;
  if (nexc == 0) return e;
  u64 tmp[2][NINT];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int i = 0; i < NINT; ++i) tmp[s][i] = t.ref[s * NINT + i];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int o = 1 - s;
    // the i-th particle and the i-th hole of this spin, ascending
    u64 pw[NINT], hw[NINT];
#pragma unroll
    for (int i = 0; i < NINT; ++i) { pw[i] = particle[s][i]; hw[i] = hole[s][i]; }
    while (true) {
      int porb = 0, horb = 0;
#pragma unroll
      for (int i = NINT - 1; i >= 0; --i) {
        if (pw[i]) porb = ctz64(pw[i]) + 1 + 64 * i;
        if (hw[i]) horb = ctz64(hw[i]) + 1 + 64 * i;
      }
      if (porb == 0) break;
      // ac_operator(particle): sums over the occupation before the bit is set
      e = __dadd_rn(e, tab2(t.h, n, porb, porb));
#pragma unroll
      for (int w = 0; w < NINT; ++w)
        for (u64 x = tmp[s][w]; x; x &= x - 1) e = __dadd_rn(e, tab2(t.ja, n, ctz64(x) + 1 + 64 * w, porb));
#pragma unroll
      for (int w = 0; w < NINT; ++w)
        for (u64 x = tmp[o][w]; x; x &= x - 1) e = __dadd_rn(e, tab2(t.jj, n, ctz64(x) + 1 + 64 * w, porb));
      tmp[s][(porb - 1) >> 6] |= 1ull << ((porb - 1) & 63);
      // a_operator(hole): sums over the occupation after the bit is cleared
      tmp[s][(horb - 1) >> 6] &= ~(1ull << ((horb - 1) & 63));
      e = __dsub_rn(e, tab2(t.h, n, horb, horb));
#pragma unroll
      for (int w = 0; w < NINT; ++w)
        for (u64 x = tmp[s][w]; x; x &= x - 1) e = __dsub_rn(e, tab2(t.ja, n, ctz64(x) + 1 + 64 * w, horb));
#pragma unroll
      for (int w = 0; w < NINT; ++w)
        for (u64 x = tmp[o][w]; x; x &= x - 1) e = __dsub_rn(e, tab2(t.jj, n, ctz64(x) + 1 + 64 * w, horb));
      pw[(porb - 1) >> 6] &= ~(1ull << ((porb - 1) & 63));
      hw[(horb - 1) >> 6] &= ~(1ull << ((horb - 1) & 63));
    }
  }
  return e;
}

// diag_S_mat_elem, s2.irp.f:1-30
template <int NINT>
__device__ __forceinline__ double diag_s(const u64* det) {
  int nup = 0;
#pragma unroll
  for (int i = 0; i < NINT; ++i) nup += popc64((det[i] ^ det[NINT + i]) & det[i]);
  return (double)nup;
}
#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// Deletion-key tables of heavy lines (built by keys.cu, read by the pair scans)
//
// Two spin strings one excitation apart share exactly one string with one
// electron removed (their intersection); two strings two excitations apart
// share exactly one string with two electrons removed.  For a line (a beta
// column or an alpha row) that holds many determinants, the pair scans look
// the line's strings up by these deletion keys instead of testing every
// string of the line: a table maps hash(kind, line, key) to the group of
// positions whose strings produced the key.  Every group member is verified
// exactly (position inside the line, popcount of the difference, the key
// itself), so hash collisions only add candidates, never pairs.
// ---------------------------------------------------------------------------
struct __align__(16) KeySlot {
  u64 h;           // hash of (kind, line, key); 0 = empty slot
  unsigned start;  // first member of the group in the table's member array
  unsigned len;    // members in the group
};
struct KeyView {
  const KeySlot* slot;  // open addressing, linear probing; nullptr = no table
  u64 mask;             // slots - 1 (a power of two)
  const int* mem;       // positions (bilinear for columns, alpha-major for rows), grouped
};
// tables: 1-deletion keys of the alpha strings of heavy columns / of the beta
// strings of heavy rows (alpha x beta pairs), 2-deletion keys (same-spin pairs)
enum { KT_COL1 = 0, KT_ROW1 = 1, KT_COL2 = 2, KT_ROW2 = 3, KT_N = 4 };
// per-line flags: the line has a 1-deletion / a 2-deletion table
constexpr unsigned char KEY_SINGLE = 1, KEY_DOUBLE = 2;

#ifdef __CUDACC__
// SplitMix64 output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) as the mixing step
__device__ __forceinline__ u64 key_mix(u64 z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
// never 0 (the empty slot); hmask keeps the low bits only (a test hook that
// makes distinct keys collide)
template <int NINT>
__device__ __forceinline__ u64 key_hash(int kind, int line, const u64* K, u64 hmask) {
  u64 h = key_mix((((u64)(unsigned)line) << 2 | (u64)kind) + 0x9e3779b97f4a7c15ull);
#pragma unroll
  for (int w = 0; w < NINT; ++w) h = key_mix(h ^ K[w]);
  return (h & hmask) | 1ull;
}
__device__ __forceinline__ bool key_find(const KeyView& kv, u64 h, unsigned& start, unsigned& len) {
  if (kv.slot == nullptr) return false;
  u64 s = h & kv.mask;
  for (u64 it = 0; it <= kv.mask; ++it) {
    const KeySlot sl = kv.slot[s];
    if (sl.h == h) {
      start = sl.start;
      len = sl.len;
      return true;
    }
    if (sl.h == 0) return false;
    s = (s + 1) & kv.mask;
  }
  return false;
}
// orbital index (word * 64 + bit) of the j-th electron (0-based) of s
template <int NINT>
__device__ __forceinline__ int nth_electron(const u64* s, int j) {
#pragma unroll
  for (int w = 0; w < NINT; ++w) {
    const int c = __popcll(s[w]);
    if (j < c) {
      u64 v = s[w];
      for (int t = 0; t < j; ++t) v &= v - 1;
      return w * 64 + __ffsll((long long)v) - 1;
    }
    j -= c;
  }
  return -1;
}
// clear orbital b (word * 64 + bit) of s, with constant word indices (s stays in registers)
template <int NINT>
__device__ __forceinline__ void clear_orbital(u64* s, int b) {
#pragma unroll
  for (int w = 0; w < NINT; ++w)
    if (w == (b >> 6)) s[w] &= ~(1ull << (b & 63));
}
// pair (i, j), i < j, of the c-th 2-electron combination of ne electrons
__device__ __forceinline__ void pair_of_combo(int c, int ne, int& i, int& j) {
  i = 0;
  while (c >= ne - 1 - i) {
    c -= ne - 1 - i;
    ++i;
  }
  j = i + 1 + c;
}
#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// Host-side context
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Rows are split into chunks of at most QP_SIGMA_CHUNK pairs, one warp each.
#define QP_SIGMA_CHUNK 2048

struct SigmaItems {
  int64_t n_items = 0;
  int n_multi = 0;
  int* row_nitems = nullptr;  // (N+1) chunks of each row
  int* row_item0 = nullptr;   // (N+1) first chunk of each row
  int* item_row = nullptr;
  int* item_sub = nullptr;
  int* multi_rows = nullptr;  // rows with more than one chunk
  double* pv = nullptr;       // partial sums (n_items, n_st)
  double* ps = nullptr;
  size_t partial_cap = 0;
  int sig32_variant[18] = {-1, -1, -1, -1, -1, -1, -1, -1, -1,
                           -1, -1, -1, -1, -1, -1, -1, -1, -1};  // tuned FP32 shape per n_st (+9: padded rows)
  void free_all() {
    void* ps_[] = {row_nitems, row_item0, item_row, item_sub, multi_rows, pv, ps};
    for (void* p : ps_)
      if (p) cudaFree(p);
    row_nitems = row_item0 = item_row = item_sub = multi_rows = nullptr;
    pv = ps = nullptr;
    partial_cap = 0;
    n_items = 0;
    n_multi = 0;
    for (int& v : sig32_variant) v = -1;
  }
};

// Learned preconditioner: MLP 8 -> 64 -> 64 -> 1 (GELU), FP32 parameters
// packed as W1[64][8], b1[64], W2[64][64], b2[64], W3[64], b3.
#define QP_MLP_IN 8
#define QP_MLP_H 64
#define QP_MLP_W1 0
#define QP_MLP_B1 (QP_MLP_W1 + QP_MLP_H * QP_MLP_IN)
#define QP_MLP_W2 (QP_MLP_B1 + QP_MLP_H)
#define QP_MLP_B2 (QP_MLP_W2 + QP_MLP_H * QP_MLP_H)
#define QP_MLP_W3 (QP_MLP_B2 + QP_MLP_H)
#define QP_MLP_B3 (QP_MLP_W3 + QP_MLP_H)
#define QP_MLP_NPARAM (QP_MLP_B3 + 1)

struct MlpState {
  float* params = nullptr;  // device
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int64_t adam_t = 0;
  bool ready = false;
  // training set: features X[n][8], target multiplier G[n], weight Wt[n]
  float* X = nullptr;
  float* G = nullptr;
  float* Wt = nullptr;
  int64_t n = 0, cap = 0;
  void free_all() {
    void* ps[] = {params, adam_m, adam_v, X, G, Wt};
    for (void* p : ps)
      if (p) cudaFree(p);
    params = adam_m = adam_v = X = G = Wt = nullptr;
    n = cap = 0;
    adam_t = 0;
    ready = false;
  }
};

// Dressing of one state (qpgpu_set_dressing), determinants as bilinear positions
struct Dressing {
  bool on = false;
  int n_ref = 0;
  int64_t n_nref = 0;
  int* ref = nullptr;        // (n_ref)
  int* nref = nullptr;       // (n_nref)
  double* d = nullptr;       // delta_ij (n_nref, n_ref) column-major
  double* ds = nullptr;      // delta_ij_s2
  double* dii = nullptr;     // delta_ii (n_ref)
  double* hdress = nullptr;  // H_jj with delta_ii added at the references (N)
};

struct qpgpu_ctx {
  std::mutex mu;
  int device = 0;
  int n_sm = 0;  // streaming multiprocessors of the device (read at create)
  cudaStream_t stream = nullptr;
  std::string last_error;

  int n_mo = 0, na = 0, nb = 0, nint = 0;
  bool have_ints = false;
  DevTables tab{};
  // owned device memory of the tables
  double *d_eri = nullptr, *d_h = nullptr, *d_jj = nullptr, *d_kk = nullptr, *d_ja = nullptr;
  double *d_bc = nullptr, *d_bx = nullptr, *d_fock = nullptr, *d_eref = nullptr;

  // determinant set
  bool have_dets = false;
  int64_t N = 0;
  int Ua = 0, Ub = 0;
  u64* d_dets = nullptr;       // (nint,2,N) original order
  u64* d_alpha = nullptr;      // (U_a, nint) unique alpha strings
  u64* d_beta = nullptr;       // (U_b, nint)
  int* d_rows = nullptr;       // bilinear (beta-major) position -> alpha id (0-based)
  int* d_cols = nullptr;       // -> beta id
  int* d_order = nullptr;      // bilinear position -> original index
  int* d_col_loc = nullptr;    // (U_b+1) first bilinear position of each beta column
  int* d_t_order = nullptr;    // alpha-major position -> bilinear position
  int* d_t_cols = nullptr;     // alpha-major position -> beta id
  int* d_row_loc = nullptr;    // (U_a+1) first alpha-major position of each alpha row
  u64* d_alpha_pos = nullptr;  // (N, nint) alpha string at each bilinear position (coalesced scans)
  u64* d_beta_tpos = nullptr;  // (N, nint) beta string at each alpha-major position
  int* d_sa_ptr = nullptr;     // singles adjacency of unique alpha strings (CSR)
  int* d_sa_idx = nullptr;
  int* d_sb_ptr = nullptr;
  int* d_sb_idx = nullptr;
  int64_t n_sa = 0, n_sb = 0;
  // per-row strategy cost of the alpha-beta class
  int64_t* d_cost_b = nullptr;  // per unique beta: sum of |col(b')| over singles b'
  int64_t* d_cost_a = nullptr;  // per unique alpha: sum of |row(a')| over singles a'
  // deletion-key tables of heavy lines (keys.cu)
  KeySlot* d_kslot[KT_N] = {nullptr, nullptr, nullptr, nullptr};
  int64_t kslots[KT_N] = {0, 0, 0, 0};
  int* d_kmem[KT_N] = {nullptr, nullptr, nullptr, nullptr};
  int64_t kmem_n[KT_N] = {0, 0, 0, 0};
  unsigned char* d_colkey = nullptr;  // per beta column: KEY_SINGLE | KEY_DOUBLE
  unsigned char* d_rowkey = nullptr;  // per alpha row
  int n_keyed_lines = 0;
  // qpgpu_set_line_keys: lines holding more determinants than these get
  // tables (-1: defaults), and the hash bits kept
  int64_t key_min_single = -1, key_min_double = -1;
  int key_hash_bits = 64;

  // Hamiltonian in CSR over bilinear rows (columns are bilinear positions)
  bool have_pairs = false;
  int sigma_mode = QPGPU_SIGMA_AUTO;  // qpgpu_set_sigma_mode
  bool direct = false;                // pairs not stored: sigma enumerates them (pairs.cu)
  double* d_direct_ut = nullptr;      // direct sigma: u in alpha-major order
  size_t direct_ut_n = 0;
  int* d_cntA = nullptr;              // direct sigma: same-beta / same-alpha pairs per row
  int* d_cntB = nullptr;
  std::vector<int64_t> h_rowptr;      // direct sigma: row starts (host)
  int* d_direct_cols = nullptr;       // direct sigma: columns of one chunk of rows
  int64_t direct_cols_cap = 0;
  int* d_direct_err = nullptr;
  int64_t P = 0;
  int64_t* d_rowptr = nullptr;  // N+1
  int* d_colidx = nullptr;      // P
  double* d_val64 = nullptr;    // P
  float* d_val32 = nullptr;     // P
  float* d_val32lo = nullptr;   // P, float-float sigma: val64 - val32 (built on first use)
  float* d_ffu = nullptr;       // float-float sigma: (hi, lo) rows of the coefficients
  size_t ffu_floats = 0;
  int64_t P_s2 = 0;             // alpha-beta spin-flip pairs (<I|S+S-|J> != 0)
  int64_t* d_s2ptr = nullptr;
  int* d_s2col = nullptr;
  float* d_s2val = nullptr;     // +-1 exactly
  double* d_hdiag = nullptr;    // H_II, bilinear order
  double* d_sdiag = nullptr;    // <I|S+S-|I>
  float* d_hdiag32 = nullptr;
  double setup_ms = 0.0;
  SigmaItems items;
  MlpState mlp;
  Dressing dress;
  float* d_detfeat = nullptr;  // (N, 4): alpha rank, beta rank, orbital-energy sum, log10(sum_J H_IJ^2)/4
  // optional phase timing of the set-up (environment QPGPU_PROFILE=1)
  bool profile = false;
  std::vector<std::pair<std::string, cudaEvent_t>> marks;

  int* d_flag = nullptr;  // NaN / Inf flag of the host-array entry points
  void* d_tc_scratch = nullptr;  // qpgpu_gram_tc: per-CTA partials, exponents, status
  size_t tc_scratch_bytes = 0;
  // scratch for the host-pointer sigma entry points
  double* d_work = nullptr;
  size_t work_bytes = 0;
  double* d_stage = nullptr;  // device copies of the host arrays of qpgpu_h_s2_u0
  size_t stage_bytes = 0;
};

// error helpers ---------------------------------------------------------------
int qpgpu_fail(qpgpu_ctx* c, int code, const std::string& msg);
#define QP_CUDA(c, call)                                                                      \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess)                                                                    \
      return qpgpu_fail((c), QPGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

template <class T>
inline cudaError_t dev_alloc(T** p, size_t count) {
  return cudaMalloc((void**)p, count * sizeof(T) + 16);
}
inline void dev_free(void* p) {
  if (p) cudaFree(p);
}

// entry points implemented across translation units
int qp_build_index(qpgpu_ctx* c);      // index.cu
int qp_build_line_keys(qpgpu_ctx* c);  // keys.cu (inside qp_build_index)
void qp_free_line_keys(qpgpu_ctx* c);  // keys.cu
int qp_build_pairs(qpgpu_ctx* c);      // pairs.cu
void qp_free_dets(qpgpu_ctx* c);       // index.cu
void qp_free_pairs(qpgpu_ctx* c);      // pairs.cu
int qp_build_sigma_items(qpgpu_ctx* c, SigmaItems* it);  // sigma.cu
// FP64 sigma without stored pairs (pairs.cu)
int qp_sigma_direct(qpgpu_ctx* c, double* v, double* s, const double* u, int nst, cudaStream_t st, int row_lo,
                    int row_hi, int row_first, int row_step);
// u32_ld: floats between FP32 rows (0: n_st; or n_st padded by qp_pad_states)
int qp_sigma_launch(qpgpu_ctx* c, SigmaItems* it, double* v, double* s, const double* u, const float* u32, int nst,
                    int precision, cudaStream_t st, int row_lo, int row_hi, int row_first, int row_step,
                    int u32_ld = 0, const float* u32lo = nullptr);
// float-float sigma of an FP64 block u (N, nst): splits u and the stored
// elements into FP32 pairs (scratch of the context) and runs k_sigma_ff
int qp_sigma_ff(qpgpu_ctx* c, SigmaItems* it, double* v, double* s, const double* u, int nst, cudaStream_t st,
                int row_lo, int row_hi, int row_first, int row_step);
// FP32 row length that keeps a row of n_st coefficients in one 32-byte sector
inline int qp_pad_states(int nst) { return nst <= 1 ? 1 : nst <= 2 ? 2 : nst <= 4 ? 4 : 8; }
// bad (optional, device int): set to 1 when an input coefficient is not finite
void qp_to_bilinear(const double* u0, int64_t ld, const int* order, double* ut, float* ut32, int nst, int64_t N,
                    cudaStream_t st, int* bad = nullptr);
void qp_flag_nonfinite(const double* x, int64_t n, int* bad, cudaStream_t st);
// device flag of the context for the NaN / Inf checks of host-array entry
// points (allocated on first use), cleared on stream st
int qp_numeric_flag(qpgpu_ctx* c, cudaStream_t st, int** flag);
void qp_from_bilinear(const double* vt, int64_t ld, const int* order, double* v0, int nst, int64_t N,
                      cudaStream_t st);
void qp_to_float(const double* x, float* y, int64_t N, int nst, int ld, cudaStream_t st);

// records a named event on the context stream when profiling is on
inline void qp_mark(qpgpu_ctx* c, const char* name) {
  if (!c->profile) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, c->stream);
  c->marks.emplace_back(name, e);
}
void qp_report_marks(qpgpu_ctx* c);  // ctx.cu

// dressing (dress.cu): adds the context's dressing to a bilinear-layout sigma
// v, s of u (nst states fastest); no-op without a dressing
int qp_dress(qpgpu_ctx* c, double* v, double* s, const double* u, int nst, cudaStream_t st);
void qp_free_dressing(qpgpu_ctx* c);

// FP64-accurate Gram blocks on the tensor cores (ozaki.cu)
int qp_gram_oz_prepare();
int qp_lincomb_oz(const double* A, int64_t sA, int m, int nsd, const double* C, double* O, int64_t ldO, int64_t N,
                  int ncta, const int* skip, int* status, cudaStream_t st);
void qp_col_maxexp(const double* X, int nblk, int64_t sX, int nsd, int ld, int64_t N, int* E, int col0,
                   const int* skip, cudaStream_t st, int n_sm);
void qp_gram_oz(const double* A, int64_t sA, int m, int nsdA, int ldA, const double* B0, const double* B1, int nbc,
                int nsdB, int ldB, int64_t N, const int* eA, const int* eB, double* partial, int ncta,
                const int* skip, int* status, cudaStream_t st);
void qp_oz_reduce(const double* partial, int ncta, int np, double* out, const int* skip, cudaStream_t st);

// learned preconditioner (mlp.cu)
int qp_det_features(qpgpu_ctx* c);
int qp_mlp_append(qpgpu_ctx* c, const float* X, const float* G, const float* W, int64_t n, bool device_src);
void qp_mlp_eval(const float* P, const float* X, float* y, int64_t n, cudaStream_t st, int n_sm);
#ifdef __CUDACC__
__device__ __forceinline__ float qp_gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float qp_gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}
// features of one (determinant, state): static (N,4) features + dynamic ones
__device__ __forceinline__ void qp_features(const float4 st, double hmL, double c, double r, double d, float* f) {
  f[0] = st.x * 0.25f;
  f[1] = st.y * 0.25f;
  f[2] = (float)(hmL * 0.1);
  f[3] = st.z * 0.1f;
  f[4] = st.w;
  f[5] = (float)(log10(fabs(c) + 1e-30) / 8.0);
  f[6] = (float)(log10(fabs(r) + 1e-30) / 8.0);
  f[7] = (float)(log10(fabs(d) + 1e-30) / 8.0);
}
// forward pass with the parameters in shared memory (P 16-byte aligned: the
// weight rows start at multiples of 4 floats, so each 16-byte broadcast load
// feeds four FMAs; the summation order is that of the plain loops)
static_assert(QP_MLP_W1 % 4 == 0 && QP_MLP_W2 % 4 == 0 && QP_MLP_IN % 4 == 0 && QP_MLP_H % 4 == 0,
              "MLP weight rows must be 16-byte aligned");
__device__ __forceinline__ float qp_mlp_forward(const float* P, const float* f) {
  float h1[QP_MLP_H];  // fully unrolled below, so it stays in registers
#pragma unroll
  for (int j = 0; j < QP_MLP_H; ++j) {
    float a = P[QP_MLP_B1 + j];
#pragma unroll
    for (int i = 0; i < QP_MLP_IN; i += 4) {
      const float4 w = *reinterpret_cast<const float4*>(&P[QP_MLP_W1 + j * QP_MLP_IN + i]);
      a = fmaf(w.x, f[i], a);
      a = fmaf(w.y, f[i + 1], a);
      a = fmaf(w.z, f[i + 2], a);
      a = fmaf(w.w, f[i + 3], a);
    }
    h1[j] = qp_gelu(a);
  }
  float y = P[QP_MLP_B3];
  for (int j = 0; j < QP_MLP_H; ++j) {
    float a = P[QP_MLP_B2 + j];
#pragma unroll
    for (int i = 0; i < QP_MLP_H; i += 4) {
      const float4 w = *reinterpret_cast<const float4*>(&P[QP_MLP_W2 + j * QP_MLP_H + i]);
      a = fmaf(w.x, h1[i], a);
      a = fmaf(w.y, h1[i + 1], a);
      a = fmaf(w.z, h1[i + 2], a);
      a = fmaf(w.w, h1[i + 3], a);
    }
    y = fmaf(P[QP_MLP_W3 + j], qp_gelu(a), y);
  }
  return y;
}
#endif

// small symmetric eigenproblem on the host (davidson.cu): ascending
// eigenvalues, eigenvectors in the columns of v (row-major n x n)
void qp_eigh(std::vector<double> a, int n, std::vector<double>& w, std::vector<double>& v);
