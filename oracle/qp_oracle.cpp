// CPU oracle for the Davidson sigma path of Quantum Package v1.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in C++17 + OpenMP, the
// reference's FP64 algorithm so that the CUDA path can be checked against it.
// Only the test-suite, the smoke check and the CPU-baseline leg of the bench
// load it; the product library never links or calls it.
//
// Parity status: the reference (Fortran + IRPF90) cannot be compiled in this
// environment, and its own test-suite holds no sigma / Slater-rule / phase
// level known-answer vectors (only end-to-end energies that need AO integrals
// and SCF).  The restatement is therefore pinned by independent checks that the
// test-suite runs: a second-quantisation Hamiltonian built from scratch
// (tests/golden fixtures), full-CI S^2 spectra, symmetry of H, and dense
// eigen-solves.  Parity with the reference's own binaries is UNPINNED.
//
// Every routine cites the reference file:line it follows (paths relative to
// the quantum_package source tree).  FP contraction is disabled at build time
// (-ffp-contract=off) so results are identical on x86-64 and aarch64.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t u64;

namespace {

inline int popc(u64 x) { return __builtin_popcountll(x); }
inline int ctz(u64 x) { return __builtin_ctzll(x); }

// pair index of bielec_integrals_index, src/Integrals_Bielec/map_integrals.irp.f:19-34
inline int64_t pair_idx(int64_t i, int64_t j) {
  int64_t p = std::min(i, j), r = std::max(i, j);
  return p + ((r * r - r) >> 1);
}

struct Ctx {
  int n_mo = 0, na = 0, nb = 0, nint = 0;
  std::vector<double> h;    // h(i,j) col-major, mo_mono_elec_integral
  std::vector<double> eri;  // chemist (pq|rs) at key-1
  std::vector<double> jj, kk, jj_anti;      // mo_bi_integrals.irp.f:1344-1369
  std::vector<double> big_coul, big_exch;   // integrals_3_index.irp.f:1-22
  std::vector<double> fock_cs;              // mono_excitations.irp.f:22-95
  std::vector<u64> ref, ref_cs;             // bitmasks.irp.f:89-95 ; mono_excitations.irp.f:2-19
  double e_ref = 0.0;                       // ref_bitmask.irp.f:1-56

  int64_t N = 0;
  std::vector<u64> dets;  // psi_det(N_int,2,N)
  int Ua = 0, Ub = 0;
  std::vector<u64> alpha_unique, beta_unique;  // (nint, U)
  // 1-based values, 0-based storage, as in spindeterminants.irp.f:387-596
  std::vector<int> rows, cols, order, order_reverse, col_loc;
  std::vector<int> t_rows, t_cols, t_order, row_loc, order_transp_reverse;

  // <ij|kl> physicist = (ik|jl), map_integrals.irp.f:383-413 (dense cache path)
  inline double get(int i, int j, int k, int l) const {
    return eri[pair_idx(pair_idx(i, k), pair_idx(j, l)) - 1];
  }
  inline double H(int i, int j) const { return h[(i - 1) + (size_t)(j - 1) * n_mo]; }
  inline double JJ(int i, int j) const { return jj[(i - 1) + (size_t)(j - 1) * n_mo]; }
  inline double JA(int i, int j) const { return jj_anti[(i - 1) + (size_t)(j - 1) * n_mo]; }
  inline double BC(int a, int b, int c) const {
    return big_coul[(a - 1) + (size_t)n_mo * ((b - 1) + (size_t)n_mo * (c - 1))];
  }
  inline double BX(int a, int b, int c) const {
    return big_exch[(a - 1) + (size_t)n_mo * ((b - 1) + (size_t)n_mo * (c - 1))];
  }
  inline double F(int i, int j) const { return fock_cs[(i - 1) + (size_t)(j - 1) * n_mo]; }
  inline const u64* det(int64_t k) const { return &dets[(size_t)k * 2 * nint]; }
  inline const u64* aun(int i) const { return &alpha_unique[(size_t)(i - 1) * nint]; }
  inline const u64* bun(int i) const { return &beta_unique[(size_t)(i - 1) * nint]; }
};

// bitstring_to_list, slater_rules.irp.f (bitstring_to_list_ab :400-430)
inline int to_list(const u64* s, int nint, int* list) {
  int n = 0;
  for (int i = 0; i < nint; ++i) {
    u64 l = s[i];
    while (l) {
      int j = ctz(l);
      l &= l - 1;
      list[n++] = 1 + 64 * i + j;
    }
  }
  return n;
}

// ---------------------------------------------------------------------------
// Slater rules (src/Determinants/slater_rules.irp.f)
// ---------------------------------------------------------------------------

// nperm contribution of one (hole, particle) pair, shared by the spin variants
// (slater_rules.irp.f:2837-2860, 2954-2969)
inline int nperm_between(const u64* det1, int low, int high) {
  int j = (low - 1) >> 6, n = ((low - 1) & 63) + 1;
  int k = (high - 1) >> 6, m = ((high - 1) & 63) + 1;
  int np = 0;
  if (j == k) {
    u64 mask = ((u64(1) << (m - 1)) - 1) & (u64(0) - (u64(1) << n));
    np += popc(det1[j] & mask);
  } else {
    np += popc(det1[k] & ((u64(1) << (m - 1)) - 1));
    if (n < 64) np += popc(det1[j] & (u64(0) - (u64(1) << n)));
    for (int i = j + 1; i < k; ++i) np += popc(det1[i]);
  }
  return np;
}

// get_mono_excitation_spin, slater_rules.irp.f:2913-2987
// exc[0]=hole, exc[1]=particle (1-based orbitals)
void mono_exc_spin(const u64* d1, const u64* d2, int nint, int* hole, int* part, double* phase) {
  int e01 = 0, e02 = 0, h = 0, p = 0;
  for (int l = 0; l < nint; ++l) {
    int ishift = 1 + 64 * l;
    if (d1[l] == d2[l]) continue;
    u64 tmp = d1[l] ^ d2[l];
    u64 particle = tmp & d2[l];
    u64 hl = tmp & d1[l];
    if (particle) { e02 = 1; p = ctz(particle) + ishift; }
    if (hl) { e01 = 1; h = ctz(hl) + ishift; }
    if ((e01 & e02) != 1) continue;
    int low = std::min(h, p), high = std::max(h, p);
    int np = nperm_between(d1, low, high);
    *hole = h; *part = p;
    *phase = (np & 1) ? -1.0 : 1.0;
    return;
  }
  *hole = h; *part = p; *phase = 1.0;
}

// get_double_excitation_spin, slater_rules.irp.f:2783-2911
// holes h[0..1], particles p[0..1] in order of discovery (increasing orbital)
void double_exc_spin(const u64* d1, const u64* d2, int nint, int* h, int* p, double* phase) {
  int e01 = 0, e02 = 0, ih = 0, ip = 0, np = 0;
  h[0] = h[1] = p[0] = p[1] = 0;
  for (int l = 0; l < nint; ++l) {
    int ishift = 1 + 64 * l;
    if (d1[l] == d2[l]) continue;
    u64 tmp = d1[l] ^ d2[l];
    u64 particle = tmp & d2[l];
    u64 hl = tmp & d1[l];
    while (particle) {
      int tz = ctz(particle);
      if (ip < 2) p[ip] = tz + ishift;
      ++ip; ++e02;
      particle &= particle - 1;
    }
    if ((e01 & e02) == 2) break;
    while (hl) {
      int tz = ctz(hl);
      if (ih < 2) h[ih] = tz + ishift;
      ++ih; ++e01;
      hl &= hl - 1;
    }
    if ((e01 & e02) == 2) break;
  }
  if (e01 == 1) {
    int low = std::min(h[0], p[0]), high = std::max(h[0], p[0]);
    np += nperm_between(d1, low, high);
  } else if (e01 == 2) {
    for (int i = 0; i < 2; ++i) {
      int low = std::min(h[i], p[i]), high = std::max(h[i], p[i]);
      np += nperm_between(d1, low, high);
    }
    int a = std::min(h[0], p[0]), b = std::max(h[0], p[0]);
    int c = std::min(h[1], p[1]), d = std::max(h[1], p[1]);
    if (c > a && c < b && d > b) np += 1;
  }
  *phase = (np & 1) ? -1.0 : 1.0;
}

// get_mono_excitation_from_fock, mono_excitations.irp.f:97-155
double mono_from_fock(const Ctx& c, const u64* det1 /*(nint,2)*/, int h, int p, int spin, double phase) {
  const int nint = c.nint;
  u64 hole[2 * 4], partcl[2 * 4];
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < nint; ++i) {
      u64 diff = det1[s * nint + i] ^ c.ref_cs[s * nint + i];
      hole[s * nint + i] = diff & c.ref_cs[s * nint + i];
      partcl[s * nint + i] = diff & det1[s * nint + i];
    }
  int oh[2][256], op[2][256], nh[2], npart[2];
  for (int s = 0; s < 2; ++s) {
    nh[s] = to_list(&hole[s * nint], nint, oh[s]);
    npart[s] = to_list(&partcl[s * nint], nint, op[s]);
  }
  double hij = c.F(h, p);
  for (int i = 0; i < nh[0]; ++i) hij -= c.BC(oh[0][i], h, p);
  for (int i = 0; i < nh[1]; ++i) hij -= c.BC(oh[1][i], h, p);
  for (int i = 0; i < nh[spin - 1]; ++i) hij += c.BX(oh[spin - 1][i], h, p);
  for (int i = 0; i < npart[0]; ++i) hij += c.BC(op[0][i], h, p);
  for (int i = 0; i < npart[1]; ++i) hij += c.BC(op[1][i], h, p);
  for (int i = 0; i < npart[spin - 1]; ++i) hij -= c.BX(op[spin - 1][i], h, p);
  return hij * phase;
}

// i_H_j_mono_spin, slater_rules.irp.f:2989-3006 (key_i, key_j: (nint,2))
double h_mono_spin(const Ctx& c, const u64* ki, const u64* kj, int spin) {
  int h, p;
  double phase;
  mono_exc_spin(ki + (spin - 1) * c.nint, kj + (spin - 1) * c.nint, c.nint, &h, &p, &phase);
  return mono_from_fock(c, ki, h, p, spin, phase);
}

// i_H_j_double_spin, slater_rules.irp.f:3008-3035 (spin strings)
double h_double_spin(const Ctx& c, const u64* si, const u64* sj) {
  int h[2], p[2];
  double phase;
  double_exc_spin(si, sj, c.nint, h, p, &phase);
  return phase * (c.get(h[0], h[1], p[0], p[1]) - c.get(h[0], h[1], p[1], p[0]));
}

// i_H_j_double_alpha_beta, slater_rules.irp.f:3037-3067
double h_double_ab(const Ctx& c, const u64* ki, const u64* kj) {
  int ha, pa, hb, pb;
  double pha, phb;
  mono_exc_spin(ki, kj, c.nint, &ha, &pa, &pha);
  mono_exc_spin(ki + c.nint, kj + c.nint, c.nint, &hb, &pb, &phb);
  double phase = pha * phb;
  if (ha == pb) return phase * c.BX(ha, hb, pa);
  if (pa == hb) return phase * c.BX(pa, ha, pb);
  return phase * c.get(ha, hb, pa, pb);
}

// get_excitation_degree, slater_rules.irp.f:1-56
int exc_degree(const u64* k1, const u64* k2, int nint) {
  int d = 0;
  for (int l = 0; l < 2 * nint; ++l) d += popc(k1[l] ^ k2[l]);
  return d >> 1;
}

// get_double_excitation (generic, both spins), slater_rules.irp.f:171-313
// exc[ispin][0=hole/1=particle][0..1]; nexc[ispin][hole/particle]
void double_exc_generic(const u64* d1, const u64* d2, int nint, int exc[2][2][2], int nexc[2][2],
                        double* phase) {
  int np = 0;
  for (int s = 0; s < 2; ++s) {
    nexc[s][0] = nexc[s][1] = 0;
    exc[s][0][0] = exc[s][0][1] = exc[s][1][0] = exc[s][1][1] = 0;
  }
  for (int s = 0; s < 2; ++s) {
    int ih = 0, ip = 0;
    const u64* a = d1 + s * nint;
    const u64* b = d2 + s * nint;
    for (int l = 0; l < nint; ++l) {
      int ishift = 1 + 64 * l;
      if (a[l] == b[l]) continue;
      u64 tmp = a[l] ^ b[l];
      u64 particle = tmp & b[l];
      u64 hl = tmp & a[l];
      while (particle) {
        if (ip < 2) exc[s][1][ip] = ctz(particle) + ishift;
        ++ip; ++nexc[s][1];
        particle &= particle - 1;
      }
      if ((nexc[s][0] & nexc[s][1]) == 2) break;
      while (hl) {
        if (ih < 2) exc[s][0][ih] = ctz(hl) + ishift;
        ++ih; ++nexc[s][0];
        hl &= hl - 1;
      }
      if ((nexc[s][0] & nexc[s][1]) == 2) break;
    }
    if (nexc[s][0] == 0) continue;
    if (nexc[s][0] == 1) {
      // slater_rules.irp.f:239-268 (high = max-1, low = min; mask form)
      int high = std::max(exc[s][0][0], exc[s][1][0]) - 1;
      int low = std::min(exc[s][0][0], exc[s][1][0]);
      int k = high >> 6, j = low >> 6, m = high & 63, n = low & 63;
      if (j == k) {
        np += popc(a[j] & (((u64(1) << m) - 1) & (~(u64(1) << n) + 1)));
      } else {
        np += popc(a[j] & (~u64(0) & (~(u64(1) << n) + 1))) + popc(a[k] & ((u64(1) << m) - 1));
        for (int i = j + 1; i < k; ++i) np += popc(a[i]);
      }
    } else if (nexc[s][0] == 2) {
      for (int l = 0; l < 2; ++l) {
        int high = std::max(exc[s][0][l], exc[s][1][l]) - 1;
        int low = std::min(exc[s][0][l], exc[s][1][l]);
        int k = high >> 6, j = low >> 6, m = high & 63, n = low & 63;
        if (j == k) {
          np += popc(a[j] & (((u64(1) << m) - 1) & (~(u64(1) << n) + 1)));
        } else {
          np += popc(a[j] & (~u64(0) & (~(u64(1) << n) + 1))) + popc(a[k] & ((u64(1) << m) - 1));
          for (int i = j + 1; i < k; ++i) np += popc(a[i]);
        }
      }
      int aa = std::min(exc[s][0][0], exc[s][1][0]), bb = std::max(exc[s][0][0], exc[s][1][0]);
      int cc = std::min(exc[s][0][1], exc[s][1][1]), dd = std::max(exc[s][0][1], exc[s][1][1]);
      if (aa < cc && cc < bb && bb < dd) np += 1;
      break;
    }
  }
  *phase = (np & 1) ? -1.0 : 1.0;
}

// get_mono_excitation (generic), slater_rules.irp.f:315-401
void mono_exc_generic(const u64* d1, const u64* d2, int nint, int* hole, int* part, int* spin,
                      double* phase) {
  for (int s = 0; s < 2; ++s) {
    int e01 = 0, e02 = 0, h = 0, p = 0;
    const u64* a = d1 + s * nint;
    const u64* b = d2 + s * nint;
    for (int l = 0; l < nint; ++l) {
      int ishift = 1 + 64 * l;
      if (a[l] == b[l]) continue;
      u64 tmp = a[l] ^ b[l];
      u64 particle = tmp & b[l];
      u64 hl = tmp & a[l];
      if (particle) { e02 = 1; p = ctz(particle) + ishift; }
      if (hl) { e01 = 1; h = ctz(hl) + ishift; }
      if ((e01 & e02) != 1) continue;
      int high = std::max(h, p) - 1, low = std::min(h, p);
      int k = high >> 6, j = low >> 6, m = high & 63, n = low & 63;
      int np = 0;
      if (j == k) {
        np += popc(a[j] & (((u64(1) << m) - 1) & (~(u64(1) << n) + 1)));
      } else {
        np += popc(a[j] & (~u64(0) & (~(u64(1) << n) + 1))) + popc(a[k] & ((u64(1) << m) - 1));
        for (int i = j + 1; i < k; ++i) np += popc(a[i]);
      }
      *hole = h; *part = p; *spin = s + 1;
      *phase = (np & 1) ? -1.0 : 1.0;
      return;
    }
  }
  *hole = *part = 0; *spin = 0; *phase = 1.0;
}

// diag_S_mat_elem, s2.irp.f:1-30
double diag_s(const Ctx& c, const u64* k) {
  int nup = 0;
  for (int i = 0; i < c.nint; ++i) nup += popc((k[i] ^ k[c.nint + i]) & k[i]);
  return (double)nup;
}

// a_operator / ac_operator, slater_rules.irp.f:1931-2022
void ac_operator(const Ctx& c, int iorb, int ispin, u64* key, double* hjj, int* na, int nb) {
  int occ[2][256];
  int n0 = to_list(key, c.nint, occ[0]);
  int n1 = to_list(key + c.nint, c.nint, occ[1]);
  (void)n0; (void)n1;
  int k = (iorb - 1) >> 6, l = (iorb - 1) & 63;
  key[(ispin - 1) * c.nint + k] |= (u64(1) << l);
  int other = (ispin == 1) ? 2 : 1;
  *hjj = *hjj + c.H(iorb, iorb);
  for (int i = 0; i < *na; ++i) *hjj = *hjj + c.JA(occ[ispin - 1][i], iorb);
  for (int i = 0; i < nb; ++i) *hjj = *hjj + c.JJ(occ[other - 1][i], iorb);
  *na += 1;
}

void a_operator(const Ctx& c, int iorb, int ispin, u64* key, double* hjj, int* na, int nb) {
  int k = (iorb - 1) >> 6, l = (iorb - 1) & 63;
  key[(ispin - 1) * c.nint + k] &= ~(u64(1) << l);
  int other = (ispin == 1) ? 2 : 1;
  int occ[2][256];
  to_list(key, c.nint, occ[0]);
  to_list(key + c.nint, c.nint, occ[1]);
  *na -= 1;
  *hjj = *hjj - c.H(iorb, iorb);
  for (int i = 0; i < *na; ++i) *hjj = *hjj - c.JA(occ[ispin - 1][i], iorb);
  for (int i = 0; i < nb; ++i) *hjj = *hjj - c.JJ(occ[other - 1][i], iorb);
}

// diag_H_mat_elem, slater_rules.irp.f:1869-1929
double diag_h(const Ctx& c, const u64* det_in) {
  const int nint = c.nint;
  u64 hole[8], particle[8];
  int nexc[2] = {0, 0};
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < nint; ++i) {
      u64 x = det_in[s * nint + i] ^ c.ref[s * nint + i];
      particle[s * nint + i] = x & det_in[s * nint + i];
      hole[s * nint + i] = x & c.ref[s * nint + i];
      nexc[s] += popc(hole[s * nint + i]);
    }
  double e = c.e_ref;
  if (nexc[0] + nexc[1] == 0) return e;
  int op[2][256], oh[2][256];
  for (int s = 0; s < 2; ++s) {
    to_list(&particle[s * nint], nint, op[s]);
    to_list(&hole[s * nint], nint, oh[s]);
  }
  u64 tmp[8];
  for (int i = 0; i < 2 * nint; ++i) tmp[i] = c.ref[i];
  const int elec[2] = {c.na, c.nb};
  for (int s = 1; s <= 2; ++s) {
    int na = elec[s - 1];
    int nb = elec[(s == 1) ? 1 : 0];
    for (int i = 0; i < nexc[s - 1]; ++i) {
      ac_operator(c, op[s - 1][i], s, tmp, &e, &na, nb);
      a_operator(c, oh[s - 1][i], s, tmp, &e, &na, nb);
    }
  }
  return e;
}

// get_s2, s2.irp.f:32-63
double get_s2(const Ctx& c, const u64* ki, const u64* kj) {
  int degree = exc_degree(ki, kj, c.nint);
  if (degree == 2) {
    int exc[2][2][2], nexc[2][2];
    double phase;
    double_exc_generic(kj, ki, c.nint, exc, nexc, &phase);
    if (nexc[0][0] == 1) {
      if (exc[0][0][0] == exc[1][1][0] && exc[1][0][0] == exc[0][1][0]) return -phase;
    }
    return 0.0;
  }
  if (degree == 0) return diag_s(c, ki);
  return 0.0;
}

// i_H_j (generic path), slater_rules.irp.f:478-570
double i_h_j(const Ctx& c, const u64* ki, const u64* kj) {
  int degree = exc_degree(ki, kj, c.nint);
  if (degree == 2) {
    int exc[2][2][2], nexc[2][2];
    double phase;
    double_exc_generic(ki, kj, c.nint, exc, nexc, &phase);
    if (nexc[0][0] == 1) {
      int ha = exc[0][0][0], pa = exc[0][1][0], hb = exc[1][0][0], pb = exc[1][1][0];
      if (ha == pb) return phase * c.BX(ha, hb, pa);
      if (pa == hb) return phase * c.BX(pa, ha, pb);
      return phase * c.get(ha, hb, pa, pb);
    } else if (nexc[0][0] == 2) {
      int h1 = exc[0][0][0], h2 = exc[0][0][1], p1 = exc[0][1][0], p2 = exc[0][1][1];
      return phase * (c.get(h1, h2, p1, p2) - c.get(h1, h2, p2, p1));
    } else if (nexc[1][0] == 2) {
      int h1 = exc[1][0][0], h2 = exc[1][0][1], p1 = exc[1][1][0], p2 = exc[1][1][1];
      return phase * (c.get(h1, h2, p1, p2) - c.get(h1, h2, p2, p1));
    }
    return 0.0;
  }
  if (degree == 1) {
    int h, p, spin;
    double phase;
    mono_exc_generic(ki, kj, c.nint, &h, &p, &spin, &phase);
    // the generic path passes (particle, hole), slater_rules.irp.f:561
    return mono_from_fock(c, ki, p, h, spin, phase);
  }
  if (degree == 0) return diag_h(c, ki);
  return 0.0;
}

// ---------------------------------------------------------------------------
// Integral tables
// ---------------------------------------------------------------------------
void build_tables(Ctx& c) {
  const int n = c.n_mo;
  c.jj.assign((size_t)n * n, 0.0);
  c.kk.assign((size_t)n * n, 0.0);
  c.jj_anti.assign((size_t)n * n, 0.0);
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) {
      size_t x = (i - 1) + (size_t)(j - 1) * n;
      c.jj[x] = c.get(i, j, i, j);
      c.kk[x] = c.get(i, j, j, i);
      c.jj_anti[x] = c.jj[x] - c.kk[x];
    }
  c.big_coul.assign((size_t)n * n * n, 0.0);
  c.big_exch.assign((size_t)n * n * n, 0.0);
  for (int k = 1; k <= n; ++k)
    for (int i = 1; i <= n; ++i)
      for (int j = 1; j <= n; ++j) {
        size_t x = (j - 1) + (size_t)n * ((i - 1) + (size_t)n * (k - 1));
        c.big_coul[x] = c.get(i, j, k, j);
        c.big_exch[x] = c.get(i, j, j, k);
      }
  // ref_bitmask = HF_bitmask, bitmasks.irp.f:71-95
  const int nint = c.nint;
  c.ref.assign(2 * nint, 0);
  for (int i = 0; i < c.na; ++i) c.ref[i >> 6] |= u64(1) << (i & 63);
  for (int i = 0; i < c.nb; ++i) c.ref[nint + (i >> 6)] |= u64(1) << (i & 63);
  // ref_closed_shell_bitmask, mono_excitations.irp.f:2-19
  c.ref_cs = c.ref;
  {
    int occ[256];
    to_list(&c.ref[0], nint, occ);
    for (int i0 = c.nb; i0 < c.na; ++i0) {
      int i = occ[i0];
      c.ref_cs[(i - 1) >> 6] &= ~(u64(1) << ((i - 1) & 63));
    }
  }
  // fock_operator_closed_shell_ref_bitmask, mono_excitations.irp.f:22-95
  c.fock_cs.assign((size_t)n * n, 0.0);
  {
    int docc[256] = {0}, virt[256] = {0};
    int nd = to_list(&c.ref_cs[0], nint, docc);
    std::vector<u64> kv(nint);
    for (int i = 0; i < nint; ++i) {
      u64 full = (i < nint - 1 || (n & 63) == 0) ? ~u64(0) : ((u64(1) << (n & 63)) - 1);
      kv[i] = full ^ c.ref_cs[i];
    }
    int nv = to_list(kv.data(), nint, virt);
    auto fill = [&](const int* la, int na_, const int* lb, int nb_) {
      for (int i0 = 0; i0 < na_; ++i0) {
        int i = la[i0];
        for (int j0 = 0; j0 < nb_; ++j0) {
          int j = lb[j0];
          double accu = 0.0;
          for (int k0 = 0; k0 < nd; ++k0) {
            int k = docc[k0];
            accu += 2.0 * c.get(i, k, j, k) - c.get(i, k, k, j);
          }
          c.fock_cs[(i - 1) + (size_t)(j - 1) * n] = accu + c.H(i, j);
          c.fock_cs[(j - 1) + (size_t)(i - 1) * n] = accu + c.H(i, j);
        }
      }
    };
    fill(docc, nd, virt, nv);
    fill(virt, nv, virt, nv);
    fill(docc, nd, docc, nd);
  }
  // ref_bitmask_energy, ref_bitmask.irp.f:1-56
  {
    int oa[256], ob[256];
    to_list(&c.ref[0], nint, oa);
    to_list(&c.ref[nint], nint, ob);
    double e = 0.0;
    for (int i = 0; i < c.nb; ++i) e += c.H(oa[i], oa[i]) + c.H(ob[i], ob[i]);
    for (int i = c.nb; i < c.na; ++i) e += c.H(oa[i], oa[i]);
    for (int j = 0; j < c.na; ++j)
      for (int i = j + 1; i < c.na; ++i) e += c.JA(oa[i], oa[j]);
    for (int j = 0; j < c.nb; ++j) {
      for (int i = j + 1; i < c.nb; ++i) e += c.JA(ob[i], ob[j]);
      for (int i = 0; i < c.na; ++i) e += c.JJ(oa[i], ob[j]);
    }
    c.e_ref = e;
  }
}

// ---------------------------------------------------------------------------
// Bilinear alpha x beta index (src/Determinants/spindeterminants.irp.f)
// ---------------------------------------------------------------------------

// spin_det_search_key, spindeterminants.irp.f:9-24 (wrapping add of -huge)
inline int64_t search_key(const u64* d, int nint) {
  u64 k = d[0];
  for (int i = 1; i < nint; ++i) k ^= d[i];
  return (int64_t)(k + (u64)(-(int64_t)0x7fffffffffffffffLL));
}

// psi_det_alpha_unique / psi_det_beta_unique, spindeterminants.irp.f:56-136
void unique_strings(const Ctx& c, int spin, std::vector<u64>& out, int& nu) {
  const int nint = c.nint;
  const int64_t N = c.N;
  std::vector<int64_t> key(N);
  std::vector<int64_t> ord(N);
  for (int64_t i = 0; i < N; ++i) {
    ord[i] = i;
    key[i] = search_key(c.det(i) + spin * nint, nint);
  }
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
  out.clear();
  // keep, in sorted order, the first occurrence of every distinct string
  int64_t i = 0;
  while (i < N) {
    int64_t j = i;
    while (j < N && key[ord[j]] == key[ord[i]]) ++j;
    size_t run_start = out.size() / nint;
    for (int64_t t = i; t < j; ++t) {
      const u64* s = c.det(ord[t]) + spin * nint;
      bool dup = false;
      for (size_t u = run_start; u < out.size() / nint && !dup; ++u)
        dup = std::equal(s, s + nint, &out[u * nint]);
      if (!dup) out.insert(out.end(), s, s + nint);
    }
    i = j;
  }
  nu = (int)(out.size() / nint);
}

// get_index_in_psi_det_alpha_unique, spindeterminants.irp.f:141-220
int index_in_unique(const std::vector<u64>& uni, int nu, const u64* key, int nint) {
  int64_t ref = search_key(key, nint);
  int lo = 0, hi = nu;  // first position with key >= ref
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (search_key(&uni[(size_t)mid * nint], nint) < ref) lo = mid + 1; else hi = mid;
  }
  for (int i = lo; i < nu && search_key(&uni[(size_t)i * nint], nint) == ref; ++i)
    if (std::equal(key, key + nint, &uni[(size_t)i * nint])) return i + 1;
  return 0;
}

void build_bilinear(Ctx& c) {
  const int64_t N = c.N;
  const int nint = c.nint;
  unique_strings(c, 0, c.alpha_unique, c.Ua);
  unique_strings(c, 1, c.beta_unique, c.Ub);
  std::vector<int> r(N), co(N);
  std::vector<int64_t> to_sort(N);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; ++k) {
    r[k] = index_in_unique(c.alpha_unique, c.Ua, c.det(k), nint);
    co[k] = index_in_unique(c.beta_unique, c.Ub, c.det(k) + nint, nint);
    to_sort[k] = (int64_t)c.Ua * (co[k] - 1) + r[k];
  }
  // psi_bilinear_matrix_*, spindeterminants.irp.f:387-445
  std::vector<int64_t> ord(N);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return to_sort[a] < to_sort[b]; });
  c.rows.resize(N); c.cols.resize(N); c.order.resize(N); c.order_reverse.resize(N);
  for (int64_t k = 0; k < N; ++k) {
    c.order[k] = (int)ord[k] + 1;
    c.rows[k] = r[ord[k]];
    c.cols[k] = co[ord[k]];
  }
  // order_reverse, :448-462
  for (int64_t k = 0; k < N; ++k) c.order_reverse[c.order[k] - 1] = (int)k + 1;
  // columns_loc, :465-494
  c.col_loc.assign(c.Ub + 1, 0);
  c.col_loc[c.cols[0] - 1] = 1;
  for (int64_t k = 1; k < N; ++k)
    if (c.cols[k] != c.cols[k - 1]) c.col_loc[c.cols[k] - 1] = (int)k + 1;
  c.col_loc[c.Ub] = (int)N + 1;
  // transp_*, :496-555
  std::vector<int64_t> ts(N);
  for (int64_t k = 0; k < N; ++k) ts[k] = (int64_t)c.Ub * (c.rows[k] - 1) + c.cols[k];
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return ts[a] < ts[b]; });
  c.t_rows.resize(N); c.t_cols.resize(N); c.t_order.resize(N);
  for (int64_t k = 0; k < N; ++k) {
    c.t_order[k] = (int)ord[k] + 1;
    c.t_rows[k] = c.rows[ord[k]];
    c.t_cols[k] = c.cols[ord[k]];
  }
  // transp_rows_loc, :557-578
  c.row_loc.assign(c.Ua + 1, 0);
  c.row_loc[c.t_rows[0] - 1] = 1;
  for (int64_t k = 1; k < N; ++k)
    if (c.t_rows[k] != c.t_rows[k - 1]) c.row_loc[c.t_rows[k] - 1] = (int)k + 1;
  c.row_loc[c.Ua] = (int)N + 1;
  // order_transp_reverse, :580-596
  c.order_transp_reverse.assign(N, -1);
  for (int64_t k = 0; k < N; ++k) c.order_transp_reverse[c.t_order[k] - 1] = (int)k + 1;
}

// get_all_spin_singles_$N_int / _and_doubles_$N_int, spindeterminants.irp.f:920-1183
// degree here counts differing bits (2 = single, 4 = double), as the reference does
inline int spin_bits(const u64* a, const u64* b, int nint) {
  int d = 0;
  for (int k = 0; k < nint; ++k) d += popc(a[k] ^ b[k]);
  return d;
}

// Pair record emitted by the sigma loops (for the connectivity comparison)
struct PairSink {
  std::vector<int32_t>* I = nullptr;  // bilinear positions (1-based)
  std::vector<int32_t>* J = nullptr;
  std::vector<int8_t>* cls = nullptr;
};

// H_S2_u_0_nstates_openmp_work_$N_int, src/Davidson/u0Hu0.irp.f:97-448
// v_t,s_t,u_t: (N_st, N) in bilinear order; rows istart..iend (1-based)
// row_list (optional): explicit bilinear rows (1-based, ascending) in place of
// the range istart+ishift, +istep, ..., <= iend; same loop bodies.
void sigma_work(const Ctx& c, double* v_t, double* s_t, const double* u_t, int N_st, int istart,
                int iend, int ishift, int istep, std::vector<std::vector<int64_t>>* pairs_out,
                const int* row_list = nullptr, int64_t n_list = 0) {
  const int64_t n_iter = row_list ? n_list
                                  : (iend >= istart + ishift ? (int64_t)(iend - istart - ishift) / istep + 1 : 0);
  const int nint = c.nint;
  const int maxab = std::max(c.Ua, c.Ub) + 1;
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  if (pairs_out) pairs_out->assign(nthreads, {});
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<int64_t>* rec = pairs_out ? &(*pairs_out)[tid] : nullptr;
    std::vector<u64> buffer((size_t)nint * maxab);
    std::vector<int> singles_a(maxab), singles_b(maxab), doubles(maxab), idx(maxab);
    u64 tmp_det[8], tmp_det2[8], spindet[4];
    int kcol_prev = -1, n_singles_b = 0;
    // Alpha/Beta double excitations, u0Hu0.irp.f:177-246
#pragma omp for schedule(dynamic, 64)
    for (int64_t it = 0; it < n_iter; ++it) {
      const int k_a = row_list ? row_list[it] : istart + ishift + (int)(it * istep);
      int krow = c.rows[k_a - 1], kcol = c.cols[k_a - 1];
      std::memcpy(tmp_det, c.aun(krow), 8 * nint);
      std::memcpy(tmp_det + nint, c.bun(kcol), 8 * nint);
      if (kcol != kcol_prev) {
        n_singles_b = 0;
        for (int i = 1; i <= c.Ub; ++i)
          if (spin_bits(tmp_det + nint, c.bun(i), nint) == 2) singles_b[n_singles_b++] = i;
      }
      kcol_prev = kcol;
      for (int i = 0; i < n_singles_b; ++i) {
        int lcol = singles_b[i];
        std::memcpy(tmp_det2 + nint, c.bun(lcol), 8 * nint);
        int l_a = c.col_loc[lcol - 1];
        int j = 0;
        for (; j < c.col_loc[lcol] - c.col_loc[lcol - 1]; ++j) {
          int lrow = c.rows[l_a - 1];
          std::memcpy(&buffer[(size_t)j * nint], c.aun(lrow), 8 * nint);
          idx[j] = l_a;
          ++l_a;
        }
        int n_singles_a = 0;
        for (int t = 0; t < j; ++t)
          if (spin_bits(tmp_det, &buffer[(size_t)t * nint], nint) == 2) singles_a[n_singles_a++] = idx[t];
        for (int k = 0; k < n_singles_a; ++k) {
          int la = singles_a[k];
          int lrow = c.rows[la - 1];
          std::memcpy(tmp_det2, c.aun(lrow), 8 * nint);
          double hij = h_double_ab(c, tmp_det, tmp_det2);
          double sij = get_s2(c, tmp_det, tmp_det2);
          for (int l = 0; l < N_st; ++l) {
            v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(la - 1) * N_st + l];
            s_t[(size_t)(k_a - 1) * N_st + l] = s_t[(size_t)(k_a - 1) * N_st + l] + sij * u_t[(size_t)(la - 1) * N_st + l];
          }
          if (rec) { rec->push_back(k_a); rec->push_back(la); rec->push_back(5); }
        }
      }
    }
    // Same-spin singles/doubles and diagonal, u0Hu0.irp.f:248-444
#pragma omp for schedule(dynamic, 64)
    for (int64_t it = 0; it < n_iter; ++it) {
      const int k_a = row_list ? row_list[it] : istart + ishift + (int)(it * istep);
      int krow = c.rows[k_a - 1], kcol = c.cols[k_a - 1];
      std::memcpy(tmp_det, c.aun(krow), 8 * nint);
      std::memcpy(tmp_det + nint, c.bun(kcol), 8 * nint);
      std::memcpy(spindet, tmp_det, 8 * nint);
      // gather the alpha strings of the beta column (:277-290)
      int lcol = c.cols[k_a - 1];
      int l_a = c.col_loc[lcol - 1];
      int i = 0;
      for (; i < c.Ua; ++i) {
        if (l_a > c.N) break;
        lcol = c.cols[l_a - 1];
        if (lcol != kcol) break;
        int lrow = c.rows[l_a - 1];
        std::memcpy(&buffer[(size_t)i * nint], c.aun(lrow), 8 * nint);
        idx[i] = l_a;
        ++l_a;
      }
      int n_sa = 0, n_d = 0;
      for (int t = 0; t < i; ++t) {
        int d = spin_bits(spindet, &buffer[(size_t)t * nint], nint);
        if (d == 4) doubles[n_d++] = idx[t];
        else if (d == 2) singles_a[n_sa++] = idx[t];
      }
      std::memcpy(tmp_det2 + nint, c.bun(kcol), 8 * nint);
      for (int t = 0; t < n_sa; ++t) {
        int la = singles_a[t];
        int lrow = c.rows[la - 1];
        std::memcpy(tmp_det2, c.aun(lrow), 8 * nint);
        double hij = h_mono_spin(c, tmp_det, tmp_det2, 1);
        for (int l = 0; l < N_st; ++l)
          v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(la - 1) * N_st + l];
        if (rec) { rec->push_back(k_a); rec->push_back(la); rec->push_back(1); }
      }
      for (int t = 0; t < n_d; ++t) {
        int la = doubles[t];
        int lrow = c.rows[la - 1];
        double hij = h_double_spin(c, tmp_det, c.aun(lrow));
        for (int l = 0; l < N_st; ++l)
          v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(la - 1) * N_st + l];
        if (rec) { rec->push_back(k_a); rec->push_back(la); rec->push_back(3); }
      }
      // beta singles/doubles in the alpha row (:336-415)
      std::memcpy(spindet, tmp_det + nint, 8 * nint);
      int k_b = c.order_transp_reverse[k_a - 1];
      int lrow = c.t_rows[k_b - 1];
      int l_b = c.row_loc[lrow - 1];
      i = 0;
      for (; i < c.Ub; ++i) {
        if (l_b > c.N) break;
        lrow = c.t_rows[l_b - 1];
        if (lrow != krow) break;
        int lc = c.t_cols[l_b - 1];
        std::memcpy(&buffer[(size_t)i * nint], c.bun(lc), 8 * nint);
        idx[i] = l_b;
        ++l_b;
      }
      int n_sb = 0;
      n_d = 0;
      for (int t = 0; t < i; ++t) {
        int d = spin_bits(spindet, &buffer[(size_t)t * nint], nint);
        if (d == 4) doubles[n_d++] = idx[t];
        else if (d == 2) singles_b[n_sb++] = idx[t];
      }
      std::memcpy(tmp_det2, c.aun(krow), 8 * nint);
      for (int t = 0; t < n_sb; ++t) {
        int lb = singles_b[t];
        int lc = c.t_cols[lb - 1];
        std::memcpy(tmp_det2 + nint, c.bun(lc), 8 * nint);
        double hij = h_mono_spin(c, tmp_det, tmp_det2, 2);
        int la = c.t_order[lb - 1];
        for (int l = 0; l < N_st; ++l)
          v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(la - 1) * N_st + l];
        if (rec) { rec->push_back(k_a); rec->push_back(la); rec->push_back(2); }
      }
      for (int t = 0; t < n_d; ++t) {
        int lb = doubles[t];
        int lc = c.t_cols[lb - 1];
        double hij = h_double_spin(c, tmp_det + nint, c.bun(lc));
        int la = c.t_order[lb - 1];
        for (int l = 0; l < N_st; ++l)
          v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(la - 1) * N_st + l];
        if (rec) { rec->push_back(k_a); rec->push_back(la); rec->push_back(4); }
      }
      // diagonal (:418-441)
      double hij = diag_h(c, tmp_det);
      double sij = diag_s(c, tmp_det);
      for (int l = 0; l < N_st; ++l) {
        v_t[(size_t)(k_a - 1) * N_st + l] = v_t[(size_t)(k_a - 1) * N_st + l] + hij * u_t[(size_t)(k_a - 1) * N_st + l];
        s_t[(size_t)(k_a - 1) * N_st + l] = s_t[(size_t)(k_a - 1) * N_st + l] + sij * u_t[(size_t)(k_a - 1) * N_st + l];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Small dense linear algebra (stand-ins for LAPACK dsyev / dgeqrf+dorgqr)
// ---------------------------------------------------------------------------

// Cyclic Jacobi eigen-solver; a (n x n col-major, lda) symmetric.  Eigenvalues
// ascending, eigenvectors in columns of v (like lapack_diag,
// src/Utils/LinearAlgebra.irp.f:446-512).
void jacobi_eigh(const double* a_in, int lda, int n, double* w, double* v, int ldv) {
  std::vector<double> a((size_t)n * n), q((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) a[i + (size_t)j * n] = a_in[i + (size_t)j * lda];
  for (int i = 0; i < n; ++i) q[i + (size_t)i * n] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double x = a[i + (size_t)j * n] * a[i + (size_t)j * n];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int r = p + 1; r < n; ++r) {
        double apr = a[p + (size_t)r * n];
        if (std::fabs(apr) < 1e-300) continue;
        double app = a[p + (size_t)p * n], arr = a[r + (size_t)r * n];
        double theta = (arr - app) / (2.0 * apr);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < n; ++k) {
          double akp = a[k + (size_t)p * n], akr = a[k + (size_t)r * n];
          a[k + (size_t)p * n] = cs * akp - sn * akr;
          a[k + (size_t)r * n] = sn * akp + cs * akr;
        }
        for (int k = 0; k < n; ++k) {
          double apk = a[p + (size_t)k * n], ark = a[r + (size_t)k * n];
          a[p + (size_t)k * n] = cs * apk - sn * ark;
          a[r + (size_t)k * n] = sn * apk + cs * ark;
        }
        for (int k = 0; k < n; ++k) {
          double qkp = q[k + (size_t)p * n], qkr = q[k + (size_t)r * n];
          q[k + (size_t)p * n] = cs * qkp - sn * qkr;
          q[k + (size_t)r * n] = sn * qkp + cs * qkr;
        }
      }
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a[x + (size_t)x * n] < a[y + (size_t)y * n]; });
  for (int j = 0; j < n; ++j) {
    w[j] = a[ord[j] + (size_t)ord[j] * n];
    for (int i = 0; i < n; ++i) v[i + (size_t)j * ldv] = q[i + (size_t)ord[j] * n];
  }
}

// Householder QR -> explicit Q in place (ortho_qr, LinearAlgebra.irp.f:123-153)
void householder_q(double* A, int64_t lda, int64_t m, int n) {
  std::vector<double> vs((size_t)m * n, 0.0), beta(n, 0.0);
  for (int k = 0; k < n; ++k) {
    double* col = A + (size_t)k * lda;
    double nrm = 0.0;
    for (int64_t i = k; i < m; ++i) nrm += col[i] * col[i];
    nrm = std::sqrt(nrm);
    double alpha = col[k] >= 0 ? -nrm : nrm;
    double* v = &vs[(size_t)k * m];
    for (int64_t i = k; i < m; ++i) v[i] = col[i];
    v[k] -= alpha;
    double vn = 0.0;
    for (int64_t i = k; i < m; ++i) vn += v[i] * v[i];
    beta[k] = vn > 0 ? 2.0 / vn : 0.0;
    for (int j = k; j < n; ++j) {
      double* cj = A + (size_t)j * lda;
      double d = 0.0;
      for (int64_t i = k; i < m; ++i) d += v[i] * cj[i];
      d *= beta[k];
      for (int64_t i = k; i < m; ++i) cj[i] -= d * v[i];
    }
  }
  // form Q = H_0 ... H_{n-1} [I; 0]
  for (int j = 0; j < n; ++j) {
    double* cj = A + (size_t)j * lda;
    for (int64_t i = 0; i < m; ++i) cj[i] = (i == j) ? 1.0 : 0.0;
  }
  for (int k = n - 1; k >= 0; --k) {
    const double* v = &vs[(size_t)k * m];
    for (int j = 0; j < n; ++j) {
      double* cj = A + (size_t)j * lda;
      double d = 0.0;
      for (int64_t i = k; i < m; ++i) d += v[i] * cj[i];
      d *= beta[k];
      for (int64_t i = k; i < m; ++i) cj[i] -= d * v[i];
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

struct qpo_ctx;

int qpo_create(int n_mo, int n_alpha, int n_beta, const double* h, const double* eri_packed,
               qpo_ctx** out) {
  if (n_mo <= 0 || n_mo > 256 || n_alpha < n_beta || n_beta < 0 || n_alpha > n_mo) return -1;
  Ctx* c = new Ctx();
  c->n_mo = n_mo; c->na = n_alpha; c->nb = n_beta; c->nint = (n_mo - 1) / 64 + 1;
  c->h.assign(h, h + (size_t)n_mo * n_mo);
  int64_t p2 = (int64_t)n_mo * (n_mo + 1) / 2;
  c->eri.assign(eri_packed, eri_packed + p2 * (p2 + 1) / 2);
  build_tables(*c);
  *out = reinterpret_cast<qpo_ctx*>(c);
  return 0;
}

void qpo_destroy(qpo_ctx* h) { delete reinterpret_cast<Ctx*>(h); }

int qpo_set_dets(qpo_ctx* h, const uint64_t* dets, int64_t n_det) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  if (n_det <= 0 || n_det >= (int64_t)1 << 31) return -1;
  c.N = n_det;
  c.dets.assign(dets, dets + (size_t)n_det * 2 * c.nint);
  build_bilinear(c);
  return 0;
}

double qpo_ref_energy(qpo_ctx* h) { return reinterpret_cast<Ctx*>(h)->e_ref; }

int qpo_n_unique(qpo_ctx* h, int* ua, int* ub) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  *ua = c.Ua; *ub = c.Ub;
  return 0;
}

// Integral tables, for table-level comparisons (n*n col-major / n^3)
int qpo_tables(qpo_ctx* h, double* fock, double* jj, double* kk, double* bcoul, double* bexch) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  size_t n = c.n_mo;
  if (fock) std::memcpy(fock, c.fock_cs.data(), 8 * n * n);
  if (jj) std::memcpy(jj, c.jj.data(), 8 * n * n);
  if (kk) std::memcpy(kk, c.kk.data(), 8 * n * n);
  if (bcoul) std::memcpy(bcoul, c.big_coul.data(), 8 * n * n * n);
  if (bexch) std::memcpy(bexch, c.big_exch.data(), 8 * n * n * n);
  return 0;
}

// 1-based index arrays of the bilinear representation
int qpo_bilinear(qpo_ctx* h, int32_t* rows, int32_t* cols, int32_t* order, int32_t* t_rows,
                 int32_t* t_cols, int32_t* t_order, int32_t* col_loc, int32_t* row_loc) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  size_t N = c.N;
  std::memcpy(rows, c.rows.data(), 4 * N);
  std::memcpy(cols, c.cols.data(), 4 * N);
  std::memcpy(order, c.order.data(), 4 * N);
  std::memcpy(t_rows, c.t_rows.data(), 4 * N);
  std::memcpy(t_cols, c.t_cols.data(), 4 * N);
  std::memcpy(t_order, c.t_order.data(), 4 * N);
  std::memcpy(col_loc, c.col_loc.data(), 4 * (c.Ub + 1));
  std::memcpy(row_loc, c.row_loc.data(), 4 * (c.Ua + 1));
  return 0;
}

int qpo_unique_strings(qpo_ctx* h, uint64_t* alpha, uint64_t* beta) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  std::memcpy(alpha, c.alpha_unique.data(), 8 * c.alpha_unique.size());
  std::memcpy(beta, c.beta_unique.data(), 8 * c.beta_unique.size());
  return 0;
}

// H_S2_u_0_nstates_openmp_work (range variant, bilinear order, states fastest)
int qpo_h_s2_u0_work(qpo_ctx* h, double* v_t, double* s_t, const double* u_t, int n_st,
                     int istart, int iend, int ishift, int istep) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  if (istart < 1 || iend > c.N || istep < 1 || n_st < 1) return -1;
  sigma_work(c, v_t, s_t, u_t, n_st, istart, iend, ishift, istep, nullptr);
  return 0;
}

// H_S2_u_0_nstates_openmp, src/Davidson/u0Hu0.irp.f:15-66.
// v0, s0, u0: (sze, N_st) column-major.  u0 is read only (the reference
// permutes it in place and restores it, which leaves it unchanged).
int qpo_h_s2_u0(qpo_ctx* h, double* v0, double* s0, const double* u0, int n_st, int64_t sze) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  const int64_t N = c.N;
  if (sze < N || n_st < 1) return -1;
  std::vector<double> u_t((size_t)N * n_st), v_t((size_t)N * n_st, 0.0), s_t((size_t)N * n_st, 0.0);
  for (int k = 0; k < n_st; ++k)
    for (int64_t i = 0; i < N; ++i) u_t[(size_t)i * n_st + k] = u0[(size_t)k * sze + (c.order[i] - 1)];
  sigma_work(c, v_t.data(), s_t.data(), u_t.data(), n_st, 1, (int)N, 0, 1, nullptr);
  for (int k = 0; k < n_st; ++k)
    for (int64_t i = 0; i < N; ++i) {
      v0[(size_t)k * sze + (c.order[i] - 1)] = v_t[(size_t)i * n_st + k];
      s0[(size_t)k * sze + (c.order[i] - 1)] = s_t[(size_t)i * n_st + k];
    }
  return 0;
}

// Connected pairs visited by the sigma loops, in original psi_det order
// (0-based I, J) with the class (1 a-single, 2 b-single, 3 aa-double,
// 4 bb-double, 5 ab-double).  Returns the count; fills at most cap records.
int64_t qpo_connected_pairs(qpo_ctx* h, int32_t* I, int32_t* J, int8_t* cls, int64_t cap) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  const int64_t N = c.N;
  std::vector<double> u_t((size_t)N, 0.0), v_t((size_t)N, 0.0), s_t((size_t)N, 0.0);
  std::vector<std::vector<int64_t>> rec;
  sigma_work(c, v_t.data(), s_t.data(), u_t.data(), 1, 1, (int)N, 0, 1, &rec);
  int64_t n = 0;
  for (auto& r : rec) {
    for (size_t t = 0; t + 2 < r.size(); t += 3) {
      if (n < cap) {
        I[n] = c.order[r[t] - 1] - 1;
        J[n] = c.order[r[t + 1] - 1] - 1;
        cls[n] = (int8_t)r[t + 2];
      }
      ++n;
    }
  }
  return n;
}

// Bilinear rows (1-based, ascending) of the psi_det indices psi_rows (0-based).
static std::vector<int> bilinear_rows(const Ctx& c, const int32_t* psi_rows, int64_t n) {
  std::vector<int> rl((size_t)n);
  for (int64_t i = 0; i < n; ++i) rl[i] = c.order_reverse[psi_rows[i]];
  std::sort(rl.begin(), rl.end());
  rl.erase(std::unique(rl.begin(), rl.end()), rl.end());
  return rl;
}

// Sigma of selected determinants only: the worker loops of
// u0Hu0.irp.f:177-444 run on the rows of psi_rows (0-based psi_det indices).
// u0: (n_st, sze) with determinants fastest (u_0(sze,N_st) column-major, psi_det
// order); v, s: (n, n_st) rows in the order of psi_rows.
int qpo_h_s2_u0_rows(qpo_ctx* h, double* v, double* s, const double* u0, int n_st, int64_t sze,
                     const int32_t* psi_rows, int64_t n) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  const int64_t N = c.N;
  if (sze < N || n_st < 1 || n < 0) return -1;
  for (int64_t i = 0; i < n; ++i)
    if (psi_rows[i] < 0 || psi_rows[i] >= N) return -1;
  std::vector<double> u_t((size_t)N * n_st), v_t((size_t)N * n_st, 0.0), s_t((size_t)N * n_st, 0.0);
  for (int k = 0; k < n_st; ++k)
    for (int64_t i = 0; i < N; ++i) u_t[(size_t)i * n_st + k] = u0[(size_t)k * sze + (c.order[i] - 1)];
  const std::vector<int> rl = bilinear_rows(c, psi_rows, n);
  sigma_work(c, v_t.data(), s_t.data(), u_t.data(), n_st, 1, (int)N, 0, 1, nullptr, rl.data(), (int64_t)rl.size());
  for (int64_t i = 0; i < n; ++i) {
    const int64_t b = c.order_reverse[psi_rows[i]] - 1;
    for (int k = 0; k < n_st; ++k) {
      v[(size_t)i * n_st + k] = v_t[(size_t)b * n_st + k];
      s[(size_t)i * n_st + k] = s_t[(size_t)b * n_st + k];
    }
  }
  return 0;
}

// Connected pairs of selected rows (psi_rows, 0-based psi_det indices), as
// qpo_connected_pairs records them.  Returns the count; fills at most cap.
int64_t qpo_connected_pairs_rows(qpo_ctx* h, const int32_t* psi_rows, int64_t n, int32_t* I, int32_t* J,
                                 int8_t* cls, int64_t cap) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  const int64_t N = c.N;
  for (int64_t i = 0; i < n; ++i)
    if (psi_rows[i] < 0 || psi_rows[i] >= N) return -1;
  std::vector<double> u_t((size_t)N, 0.0), v_t((size_t)N, 0.0), s_t((size_t)N, 0.0);
  std::vector<std::vector<int64_t>> rec;
  const std::vector<int> rl = bilinear_rows(c, psi_rows, n);
  sigma_work(c, v_t.data(), s_t.data(), u_t.data(), 1, 1, (int)N, 0, 1, &rec, rl.data(), (int64_t)rl.size());
  int64_t m = 0;
  for (auto& r : rec)
    for (size_t t = 0; t + 2 < r.size(); t += 3) {
      if (m < cap) {
        I[m] = c.order[r[t] - 1] - 1;
        J[m] = c.order[r[t + 1] - 1] - 1;
        cls[m] = (int8_t)r[t + 2];
      }
      ++m;
    }
  return m;
}

// Excitation data of a connected pair I -> J (0-based original indices), as
// the spin-specific routines used by the sigma compute it.  exc[0..3] =
// (h1,p1,h2,p2), 1-based (h2=p2=0 for singles); returns phase (+1/-1).
int qpo_pair_excitation(qpo_ctx* hc, int32_t I, int32_t J, int cls, int32_t* exc, double* hij,
                        double* sij) {
  Ctx& c = *reinterpret_cast<Ctx*>(hc);
  const u64* di = c.det(I);
  const u64* dj = c.det(J);
  const int nint = c.nint;
  double phase = 1.0;
  exc[0] = exc[1] = exc[2] = exc[3] = 0;
  *sij = 0.0;
  if (cls == 1 || cls == 2) {
    int s = cls - 1;
    mono_exc_spin(di + s * nint, dj + s * nint, nint, &exc[0], &exc[1], &phase);
    *hij = h_mono_spin(c, di, dj, cls);
  } else if (cls == 3 || cls == 4) {
    int s = cls - 3, hh[2], pp[2];
    double_exc_spin(di + s * nint, dj + s * nint, nint, hh, pp, &phase);
    exc[0] = hh[0]; exc[1] = pp[0]; exc[2] = hh[1]; exc[3] = pp[1];
    *hij = h_double_spin(c, di + s * nint, dj + s * nint);
  } else if (cls == 5) {
    double pb;
    mono_exc_spin(di, dj, nint, &exc[0], &exc[1], &phase);
    mono_exc_spin(di + nint, dj + nint, nint, &exc[2], &exc[3], &pb);
    phase *= pb;
    *hij = h_double_ab(c, di, dj);
    *sij = get_s2(c, di, dj);
  } else {
    return -1;
  }
  return phase > 0 ? 1 : -1;
}

// diag_H_mat_elem / diag_S_mat_elem for every det (original order)
int qpo_diag(qpo_ctx* h, double* hjj, double* sjj) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.N; ++i) {
    if (hjj) hjj[i] = diag_h(c, c.det(i));
    if (sjj) sjj[i] = diag_s(c, c.det(i));
  }
  return 0;
}

// Generic i_H_j and get_s2 on two arbitrary determinants (nint,2)
double qpo_i_h_j(qpo_ctx* h, const uint64_t* ki, const uint64_t* kj) {
  return i_h_j(*reinterpret_cast<Ctx*>(h), ki, kj);
}
double qpo_get_s2(qpo_ctx* h, const uint64_t* ki, const uint64_t* kj) {
  return get_s2(*reinterpret_cast<Ctx*>(h), ki, kj);
}

// H_matrix_all_dets (src/Determinants/utils.irp.f:1-21) through the generic
// i_H_j path, and the S^2 matrix through get_s2 (the pairs S2_u_0_nstates
// visits, src/Determinants/s2.irp.f:150-273).  N x N column-major.
int qpo_dense(qpo_ctx* h, double* H, double* S2) {
  Ctx& c = *reinterpret_cast<Ctx*>(h);
  const int64_t N = c.N;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < N; ++i)
    for (int64_t j = i; j < N; ++j) {
      if (H) {
        double hij = i_h_j(c, c.det(i), c.det(j));
        H[i + j * N] = hij;
        H[j + i * N] = hij;
      }
      if (S2) {
        double s = get_s2(c, c.det(i), c.det(j));
        S2[i + j * N] = s;
        S2[j + i * N] = s;
      }
    }
  return 0;
}

// davidson_diag_hjj_sjj, src/Davidson/diagonalization_hs2.irp.f:52-444.
// u_in(dim_in, N_st_diag) holds ALL guess vectors (the reference draws the
// extra ones with random_number, :188-200; here the caller supplies them).
// H_jj from diag_H_mat_elem (davidson_diag_hs2, :1-49).  energies/s2_out have
// N_st_diag entries.  Returns the number of sigma calls (>0) or <0 on error.
int qpo_davidson(qpo_ctx* hc, double* u_in, int64_t dim_in, double* energies, double* s2_out,
                 int n_st, int n_st_diag, int davidson_sze_max, double threshold, int s2_eig,
                 int max_sigma, double* res_out, int state_following) {
  Ctx& c = *reinterpret_cast<Ctx*>(hc);
  const int64_t sze = c.N;
  if (n_st_diag * 3 > sze) return -2;  // :110-114
  const int itermax = std::max(3, std::min(davidson_sze_max, (int)(sze / n_st_diag)));
  const int m = n_st_diag * itermax;
  std::vector<double> H_jj(sze);
  for (int64_t i = 0; i < sze; ++i) H_jj[i] = diag_h(c, c.det(i));
  const double Sz = 0.5 * (c.na - c.nb);
  const double S_z2_Sz = Sz * (Sz - 1.0);
  const double expected_s2 = Sz * (Sz + 1.0);
  std::vector<double> W((size_t)sze * m, 0.0), U((size_t)sze * m, 0.0), S((size_t)sze * m, 0.0);
  std::vector<double> hm((size_t)m * m), y((size_t)m * m), s_((size_t)m * m), s_tmp((size_t)m * m);
  std::vector<double> lambda(m), s2(m), residual_norm(n_st_diag, 0.0);
  std::vector<char> state_ok(m);
  // normalize guesses (:199-201)
  for (int k = 0; k < n_st_diag; ++k) {
    double nrm = 0.0;
    for (int64_t i = 0; i < sze; ++i) nrm += u_in[i + k * dim_in] * u_in[i + k * dim_in];
    nrm = 1.0 / std::sqrt(nrm);
    for (int64_t i = 0; i < sze; ++i) u_in[i + k * dim_in] *= nrm;
  }
  bool converged = false;
  int n_sigma = 0, shift2 = 0;
  auto gemm_tn = [&](const double* A, const double* B, double* C, int nn) {
    // C(nn,nn) = A^T B, A,B (sze, nn)
    for (int j = 0; j < nn; ++j)
      for (int i = 0; i < nn; ++i) {
        double d = 0.0;
        for (int64_t r = 0; r < sze; ++r) d += A[r + (size_t)i * sze] * B[r + (size_t)j * sze];
        C[i + (size_t)j * m] = d;
      }
  };
  auto small_nn = [&](const double* A, const double* B, double* C, int nn, bool ta) {
    for (int j = 0; j < nn; ++j)
      for (int i = 0; i < nn; ++i) {
        double d = 0.0;
        for (int k = 0; k < nn; ++k)
          d += (ta ? A[k + (size_t)i * m] : A[i + (size_t)k * m]) * B[k + (size_t)j * m];
        C[i + (size_t)j * m] = d;
      }
  };
  while (!converged) {
    for (int k = 0; k < n_st_diag; ++k)
      for (int64_t i = 0; i < sze; ++i) U[i + (size_t)k * sze] = u_in[i + k * dim_in];
    for (int iter = 1; iter <= itermax - 1; ++iter) {
      int shift = n_st_diag * (iter - 1);
      shift2 = n_st_diag * iter;
      householder_q(U.data(), sze, sze, shift2);  // :216
      // sigma on the new block (:222-226)
      {
        std::vector<double> u_t((size_t)sze * n_st_diag), v_t((size_t)sze * n_st_diag, 0.0),
            s_t((size_t)sze * n_st_diag, 0.0);
        for (int k = 0; k < n_st_diag; ++k)
          for (int64_t i = 0; i < sze; ++i)
            u_t[(size_t)i * n_st_diag + k] = U[(c.order[i] - 1) + (size_t)(shift + k) * sze];
        sigma_work(c, v_t.data(), s_t.data(), u_t.data(), n_st_diag, 1, (int)sze, 0, 1, nullptr);
        for (int k = 0; k < n_st_diag; ++k)
          for (int64_t i = 0; i < sze; ++i) {
            W[(c.order[i] - 1) + (size_t)(shift + k) * sze] = v_t[(size_t)i * n_st_diag + k];
            S[(c.order[i] - 1) + (size_t)(shift + k) * sze] = s_t[(size_t)i * n_st_diag + k];
          }
        ++n_sigma;
      }
      gemm_tn(U.data(), W.data(), hm.data(), shift2);  // :232-238
      gemm_tn(U.data(), S.data(), s_.data(), shift2);
      std::vector<double> w(shift2), vv((size_t)shift2 * shift2);
      jacobi_eigh(hm.data(), m, shift2, w.data(), vv.data(), shift2);  // :284
      for (int j = 0; j < shift2; ++j) {
        lambda[j] = w[j];
        for (int i = 0; i < shift2; ++i) y[i + (size_t)j * m] = vv[i + (size_t)j * shift2];
      }
      // S2 of each eigenvector (:289-301)
      small_nn(s_.data(), y.data(), s_tmp.data(), shift2, false);
      small_nn(y.data(), s_tmp.data(), s_.data(), shift2, true);
      for (int k = 0; k < shift2; ++k) s2[k] = s_[k + (size_t)k * m] + S_z2_Sz;
      for (int k = 0; k < shift2; ++k)
        state_ok[k] = s2_eig ? (std::fabs(s2[k] - expected_s2) < 0.6) : 1;
      for (int k = 0; k < shift2; ++k) {  // :312-326
        if (!state_ok[k]) {
          for (int l = k + 1; l < shift2; ++l) {
            if (state_ok[l]) {
              for (int i = 0; i < shift2; ++i) std::swap(y[i + (size_t)k * m], y[i + (size_t)l * m]);
              std::swap(s2[k], s2[l]);
              std::swap(lambda[k], lambda[l]);
              state_ok[k] = 1;
              state_ok[l] = 0;
              break;
            }
          }
        }
      }
      if (state_following) {  // :328-370, literally (order(k) is a row index used as a column)
        std::vector<double> ov((size_t)m * m, -1.0);
        for (int k = 0; k < shift2; ++k)
          for (int i = 0; i < shift2; ++i) ov[k + (size_t)i * m] = std::fabs(y[k + (size_t)i * m]);
        std::vector<int> order(n_st);
        for (int k = 0; k < n_st; ++k) {
          double cmax = -1.0;
          for (int i = 0; i < n_st; ++i)
            if (ov[i + (size_t)k * m] > cmax) {
              cmax = ov[i + (size_t)k * m];
              order[k] = i;
            }
          for (int i = 0; i < n_st_diag; ++i) ov[order[k] + (size_t)i * m] = -1.0;
        }
        const std::vector<double> y0 = y;
        std::vector<double> l0(lambda.begin(), lambda.begin() + n_st), s0(s2.begin(), s2.begin() + n_st);
        for (int k = 0; k < n_st; ++k) {
          const int l = order[k];
          if (k != l)
            for (int i = 0; i < shift2; ++i) y[i + (size_t)k * m] = y0[i + (size_t)l * m];
        }
        for (int k = 0; k < n_st; ++k) {
          const int l = order[k];
          if (k != l) {
            lambda[k] = l0[l];
            s2[k] = s0[l];
          }
        }
      }
      // Ritz vectors (:376-381)
      for (int k = 0; k < n_st_diag; ++k)
        for (int64_t i = 0; i < sze; ++i) {
          double a = 0.0, b = 0.0, d = 0.0;
          for (int l = 0; l < shift2; ++l) {
            double yl = y[l + (size_t)k * m];
            a += U[i + (size_t)l * sze] * yl;
            b += W[i + (size_t)l * sze] * yl;
            d += S[i + (size_t)l * sze] * yl;
          }
          U[i + (size_t)(shift2 + k) * sze] = a;
          W[i + (size_t)(shift2 + k) * sze] = b;
          S[i + (size_t)(shift2 + k) * sze] = d;
        }
      // residual / Davidson step (:386-401)
      for (int k = 0; k < n_st_diag; ++k) {
        double* uk = &U[(size_t)(shift2 + k) * sze];
        const double* wk = &W[(size_t)(shift2 + k) * sze];
        const double* sk = &S[(size_t)(shift2 + k) * sze];
        for (int64_t i = 0; i < sze; ++i)
          uk[i] = (lambda[k] * uk[i] - wk[i]) * (1.0 + s2[k] * uk[i] - sk[i] - S_z2_Sz) /
                  std::max(H_jj[i] - lambda[k], 1e-2);
        if (k < n_st) {
          double r = 0.0;
          for (int64_t i = 0; i < sze; ++i) r += uk[i] * uk[i];
          residual_norm[k] = r;
        }
      }
      // davidson_converged, parameters.irp.f:9-49 ('residual')
      converged = false;
      if (iter >= 2) {
        double mx = 0.0;
        for (int k = 0; k < n_st; ++k) mx = std::max(mx, residual_norm[k]);
        converged = std::fabs(mx) < threshold;
      }
      for (int k = 0; k < n_st; ++k)
        if (residual_norm[k] > 1e8) return -3;  // 'Davidson failed'
      if (converged || (max_sigma > 0 && n_sigma >= max_sigma)) break;
    }
    // re-contract (:419-420)
    for (int k = 0; k < n_st_diag; ++k)
      for (int64_t i = 0; i < sze; ++i) {
        double a = 0.0;
        for (int l = 0; l < shift2; ++l) a += U[i + (size_t)l * sze] * y[l + (size_t)k * m];
        u_in[i + k * dim_in] = a;
      }
    if (max_sigma > 0 && n_sigma >= max_sigma) break;
  }
  for (int k = 0; k < n_st_diag; ++k) {
    energies[k] = lambda[k];
    s2_out[k] = s2[k];
  }
  if (res_out)
    for (int k = 0; k < n_st; ++k) res_out[k] = residual_norm[k];
  return n_sigma;
}

int qpo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"

extern "C" {
// Batched qpo_pair_excitation over n pairs (OpenMP): phase (+1/-1), exc[4*i..], hij, sij.
int qpo_pair_excitations(qpo_ctx* hc, int64_t n, const int32_t* I, const int32_t* J, const int8_t* cls,
                         int8_t* phase, int32_t* exc, double* hij, double* sij) {
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t i = 0; i < n; ++i) {
    int ph = qpo_pair_excitation(hc, I[i], J[i], cls[i], exc + 4 * i, hij + i, sij + i);
    if (ph == -1 || ph == 1) phase[i] = (int8_t)ph; else bad = 1;
  }
  return bad ? -1 : 0;
}
}

// ---------------------------------------------------------------------------
// CIPSI selection with the Epstein-Nesbet second-order energy
// (plugins/Full_CI_ZMQ/selection.irp.f), restated on the determinant level.
//
// The reference walks, for each generator (the first N_det_generators
// determinants of psi_det_sorted), every pair of holes and every pair of
// particles, and for each external determinant a (a single or double
// excitation of the generator, not in the wave function):
//   * skips a when it is within a double excitation of an earlier generator
//     (spot_isinwf fullMatch, past_d1, past_d2: :1088-1172), so every external
//     determinant is counted once, by the first generator that reaches it;
//   * skips a when it is in the wave function (spot_isinwf banned, :1130-1172);
//   * forms mat(st) = sum over selectors D of c_D,st <a|H|D> (splash_pq,
//     get_d0/d1/d2: :647-1086), skipping a when every mat(st) is zero;
//   * H_aa = diag_H_mat_elem_fock(generator, a) (slater_rules.irp.f:1800-1866)
//     from the generator's build_fock_tmp (Fock_diag.irp.f:1-98);
//   * e(st) = (sign(delta) sqrt(delta^2 + (2 mat)^2) - delta) / 2 with
//     delta = E0(st) - H_aa, pt2(st) += e(st), and the buffer receives
//     a with the value min(0, min_st e(st)) (fill_buffer_double, :582-645);
//     the buffer keeps the most negative values (selection_buffer.irp.f:33-138).
// Here the same set of external determinants is enumerated generator by
// generator (a hash set stands in for the banned masks), <a|H|D> comes from
// the generic i_H_j path, and each external's numerator is summed over the
// selectors in their order.
// ---------------------------------------------------------------------------
namespace {

typedef std::array<u64, 4> DetKey;  // (alpha words, beta words), N_int <= 2

struct DetKeyHash {
  size_t operator()(const DetKey& k) const {
    u64 h = 0x9e3779b97f4a7c15ull;
    for (u64 w : k) {
      h ^= w + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
      h *= 0xbf58476d1ce4e5b9ull;
    }
    return (size_t)(h ^ (h >> 31));
  }
};

DetKey make_key(const u64* d, int nint) {
  DetKey k{};
  for (int i = 0; i < 2 * nint; ++i) k[i] = d[i];
  return k;
}

inline void flip_bit(u64* d, int nint, int spin, int orb) {  // orb 1-based, spin 0/1
  d[spin * nint + ((orb - 1) >> 6)] ^= u64(1) << ((orb - 1) & 63);
}

// every single and double excitation of det g (both spins), fn(const u64* a)
template <class Fn>
void for_each_excitation(const Ctx& c, const u64* g, Fn&& fn) {
  const int nint = c.nint, n = c.n_mo;
  int occ[2][256], vir[2][256], no[2], nv[2];
  for (int s = 0; s < 2; ++s) {
    no[s] = to_list(g + s * nint, nint, occ[s]);
    nv[s] = 0;
    for (int o = 1; o <= n; ++o)
      if (!((g[s * nint + ((o - 1) >> 6)] >> ((o - 1) & 63)) & 1)) vir[s][nv[s]++] = o;
  }
  u64 a[8];
  auto reset = [&]() { std::memcpy(a, g, sizeof(u64) * 2 * nint); };
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < no[s]; ++i)
      for (int j = 0; j < nv[s]; ++j) {
        reset();
        flip_bit(a, nint, s, occ[s][i]);
        flip_bit(a, nint, s, vir[s][j]);
        fn(a);
      }
  for (int s = 0; s < 2; ++s)
    for (int i1 = 0; i1 < no[s]; ++i1)
      for (int i2 = i1 + 1; i2 < no[s]; ++i2)
        for (int j1 = 0; j1 < nv[s]; ++j1)
          for (int j2 = j1 + 1; j2 < nv[s]; ++j2) {
            reset();
            flip_bit(a, nint, s, occ[s][i1]);
            flip_bit(a, nint, s, occ[s][i2]);
            flip_bit(a, nint, s, vir[s][j1]);
            flip_bit(a, nint, s, vir[s][j2]);
            fn(a);
          }
  for (int i1 = 0; i1 < no[0]; ++i1)
    for (int j1 = 0; j1 < nv[0]; ++j1)
      for (int i2 = 0; i2 < no[1]; ++i2)
        for (int j2 = 0; j2 < nv[1]; ++j2) {
          reset();
          flip_bit(a, nint, 0, occ[0][i1]);
          flip_bit(a, nint, 0, vir[0][j1]);
          flip_bit(a, nint, 1, occ[1][i2]);
          flip_bit(a, nint, 1, vir[1][j2]);
          fn(a);
        }
}

// build_fock_tmp, Fock_diag.irp.f:1-98: f[s * (n_mo + 2) + i], i = 1..n_mo, and
// f[s * (n_mo + 2) + n_mo + 1] = <g|H|g>
void build_fock_tmp(const Ctx& c, const u64* g, std::vector<double>& f) {
  const int n = c.n_mo, st = n + 2;
  f.assign(2 * (size_t)st, 0.0);
  int occ[2][256];
  to_list(g, c.nint, occ[0]);
  to_list(g + c.nint, c.nint, occ[1]);
  double e0 = 0.0;
  for (int ii = 0; ii < c.na; ++ii) {
    const int i = occ[0][ii];
    f[i] += c.H(i, i);
    e0 += c.H(i, i);
    for (int jj = 0; jj < c.na; ++jj) {
      const int j = occ[0][jj];
      if (i == j) continue;
      f[i] += c.JA(i, j);
      e0 += 0.5 * c.JA(i, j);
    }
    for (int jj = 0; jj < c.nb; ++jj) {
      const int j = occ[1][jj];
      f[i] += c.JJ(i, j);
      e0 += c.JJ(i, j);
    }
  }
  for (int ii = 0; ii < c.nb; ++ii) {
    const int i = occ[1][ii];
    f[st + i] += c.H(i, i);
    e0 += c.H(i, i);
    for (int jj = 0; jj < c.nb; ++jj) {
      const int j = occ[1][jj];
      if (i == j) continue;
      f[st + i] += c.JA(i, j);
      e0 += 0.5 * c.JA(i, j);
    }
    for (int jj = 0; jj < c.na; ++jj) f[st + i] += c.JJ(i, occ[0][jj]);
  }
  for (int i = 1; i <= n; ++i) {  // virtual MOs
    if (f[i] != 0.0) continue;
    f[i] += c.H(i, i);
    for (int jj = 0; jj < c.na; ++jj) f[i] += c.JA(i, occ[0][jj]);
    for (int jj = 0; jj < c.nb; ++jj) f[i] += c.JJ(i, occ[1][jj]);
  }
  for (int i = 1; i <= n; ++i) {
    if (f[st + i] != 0.0) continue;
    f[st + i] += c.H(i, i);
    for (int jj = 0; jj < c.nb; ++jj) f[st + i] += c.JA(i, occ[1][jj]);
    for (int jj = 0; jj < c.na; ++jj) f[st + i] += c.JJ(i, occ[0][jj]);
  }
  f[n + 1] = e0;
  f[st + n + 1] = e0;
}

// diag_H_mat_elem_fock, slater_rules.irp.f:1800-1866 (pert within a double
// excitation of ref)
double diag_h_fock(const Ctx& c, const u64* ref, const u64* pert, const std::vector<double>& f) {
  const int n = c.n_mo, st = n + 2;
  auto F = [&](int s, int i) { return f[(size_t)(s - 1) * st + i]; };
  const double e0 = F(1, n + 1);
  const int degree = exc_degree(ref, pert, c.nint);
  if (degree == 2) {
    int exc[2][2][2], nexc[2][2];
    double phase;
    double_exc_generic(ref, pert, c.nint, exc, nexc, &phase);
    int h1, h2, p1, p2, s1, s2;
    if (nexc[0][0] == 2) {  // decode_exc, slater_rules.irp.f:105-160
      h1 = exc[0][0][0]; h2 = exc[0][0][1]; p1 = exc[0][1][0]; p2 = exc[0][1][1]; s1 = s2 = 1;
    } else if (nexc[1][0] == 2) {
      h1 = exc[1][0][0]; h2 = exc[1][0][1]; p1 = exc[1][1][0]; p2 = exc[1][1][1]; s1 = s2 = 2;
    } else {
      h1 = exc[0][0][0]; h2 = exc[1][0][0]; p1 = exc[0][1][0]; p2 = exc[1][1][0]; s1 = 1; s2 = 2;
    }
    if (s1 == s2)
      return e0 - F(s1, h1) + (F(s1, p1) - c.JA(h1, p1)) - (F(s1, h2) - c.JA(h1, h2) + c.JA(p1, h2)) +
             (F(s1, p2) - c.JA(h1, p2) + c.JA(p1, p2) - c.JA(h2, p2));
    return e0 - F(1, h1) + (F(1, p1) - c.JA(h1, p1)) - (F(2, h2) - c.JJ(h1, h2) + c.JJ(p1, h2)) +
           (F(2, p2) - c.JJ(h1, p2) + c.JJ(p1, p2) - c.JA(h2, p2));
  }
  if (degree == 1) {
    int h, p, spin;
    double phase;
    mono_exc_generic(ref, pert, c.nint, &h, &p, &spin, &phase);
    return e0 - F(spin, h) + (F(spin, p) - c.JA(h, p));
  }
  return e0;
}

struct SelCand {
  double val;
  DetKey key;
};

}  // namespace

extern "C" {
// Selection over the wave function held by the context, whose determinants
// must be in psi_det_sorted order: generators = determinants 0..n_gen-1,
// selectors = 0..n_sel-1 (n_gen <= n_sel <= N).  coef(N, n_st) column-major
// (psi_coef_sorted), e0(n_st) the denominators (pt2_E0_denominator).  Writes
// pt2(n_st), the buf_size most negative buffer values (ascending, ties in
// determinant-bit order) with their determinants (N_int, 2) each, and the
// number of external determinants with a non-zero numerator.  Returns the
// number of buffer entries written, or -1 on bad arguments.
int qpo_select_pt2(qpo_ctx* hc, const double* coef, int n_st, const double* e0, int n_gen, int n_sel, int buf_size,
                   double* pt2, uint64_t* buf_dets, double* buf_vals, int64_t* n_ext) {
  if (!hc || !coef || !e0 || !pt2) return -1;
  const Ctx& c = *reinterpret_cast<Ctx*>(hc);
  const int64_t N = c.N;
  const int nint = c.nint;
  if (n_st < 1 || n_gen < 1 || n_gen > n_sel || n_sel > N || nint > 2 || buf_size < 0 ||
      (buf_size > 0 && (!buf_dets || !buf_vals)))
    return -1;
  std::unordered_set<DetKey, DetKeyHash> inwf;
  inwf.reserve((size_t)N * 2);
  for (int64_t i = 0; i < N; ++i) inwf.insert(make_key(c.det(i), nint));
  // external determinants in order of their (first) generator
  std::unordered_map<DetKey, int64_t, DetKeyHash> ext_index;
  std::vector<DetKey> ext;
  std::vector<int> ext_gen;
  for (int g = 0; g < n_gen; ++g)
    for_each_excitation(c, c.det(g), [&](const u64* a) {
      DetKey k = make_key(a, nint);
      if (inwf.count(k) || ext_index.count(k)) return;
      ext_index.emplace(k, (int64_t)ext.size());
      ext.push_back(k);
      ext_gen.push_back(g);
    });
  // numerators: sum over the selectors, in their order
  std::vector<double> v(ext.size() * (size_t)n_st, 0.0);
  for (int D = 0; D < n_sel; ++D)
    for_each_excitation(c, c.det(D), [&](const u64* a) {
      auto it = ext_index.find(make_key(a, nint));
      if (it == ext_index.end()) return;
      const double hij = i_h_j(c, a, c.det(D));
      for (int s = 0; s < n_st; ++s) v[(size_t)it->second * n_st + s] += coef[D + (size_t)N * s] * hij;
    });
  for (int s = 0; s < n_st; ++s) pt2[s] = 0.0;
  std::vector<SelCand> cand;
  std::vector<double> f;
  int fg = -1;
  int64_t nz = 0;
  for (size_t i = 0; i < ext.size(); ++i) {
    double sabs = 0.0;
    for (int s = 0; s < n_st; ++s) sabs += std::fabs(v[i * n_st + s]);
    if (sabs == 0.0) continue;
    ++nz;
    const int g = ext_gen[i];
    if (g != fg) {
      build_fock_tmp(c, c.det(g), f);
      fg = g;
    }
    const double haa = diag_h_fock(c, c.det(g), ext[i].data(), f);
    double mine = 0.0;
    for (int s = 0; s < n_st; ++s) {
      const double delta = e0[s] - haa;
      const double val = v[i * n_st + s] + v[i * n_st + s];
      double tmp = std::sqrt(delta * delta + val * val);
      if (delta < 0.0) tmp = -tmp;
      const double e = 0.5 * (tmp - delta);
      pt2[s] += e;
      mine = std::min(e, mine);
    }
    cand.push_back({mine, ext[i]});
  }
  if (n_ext) *n_ext = nz;
  const size_t nout = std::min(cand.size(), (size_t)buf_size);
  auto less = [](const SelCand& x, const SelCand& y) { return x.val < y.val || (x.val == y.val && x.key < y.key); };
  std::partial_sort(cand.begin(), cand.begin() + nout, cand.end(), less);
  for (size_t i = 0; i < nout; ++i) {
    buf_vals[i] = cand[i].val;
    for (int w = 0; w < 2 * nint; ++w) buf_dets[i * 2 * nint + w] = cand[i].key[w];
  }
  return (int)nout;
}
}
