// Build of the connected-pair Hamiltonian (CSR over bilinear rows).
//
// The pair set is the one H_S2_u_0_nstates_openmp_work visits
// (src/Davidson/u0Hu0.irp.f:177-444): for the determinant I = (a, b) at
// bilinear position k
//   class A  J in the same beta column, alpha strings 1 or 2 apart  (:277-332)
//   class B  J in the same alpha row, beta strings 1 or 2 apart      (:336-415)
//   class C  alpha single x beta single                              (:177-246)
// with the diagonal kept apart (:418-441).  The fill writes row k's A hits,
// then its B hits, then its C hits; the stored form then sorts each row's
// columns ascending (the direct sigma keeps the fill order).
//
// Two passes run the same deterministic traversal: the first counts hits per
// row, the second writes them (column = bilinear position of J, FP64 and FP32
// matrix elements).  A third mode (direct sigma, for determinant sets whose
// pairs do not fit in device memory) runs the traversal at every sigma call
// and accumulates h_IJ u_J for the row each thread (classes A, B) or warp
// (class C) owns: class A writes v, class B adds to it, class C adds its sum
// and the diagonal term and writes s, so no pair is stored and no atomic is
// needed.  Same-spin classes scan a column (row) with one thread per
// determinant; the column's strings are staged in shared memory and read by
// every thread of the block as broadcasts.  Class C gives one warp per row and
// compacts hits with __ballot_sync, scanning either the columns of the beta
// singles of b (as the reference does) or the rows of the alpha singles of a,
// whichever holds fewer determinants.
#include <algorithm>
#include <climits>
#include <vector>

#include <cub/cub.cuh>

#include "qpgpu_internal.cuh"

namespace {

constexpr int BLK = 256;
constexpr int TILE = 1024;

inline unsigned nblocks(int64_t n, int tpb) {
  int64_t g = (n + tpb - 1) / tpb;
  return (unsigned)(g < 1 ? 1 : g);
}

template <class T>
struct Scoped {
  T* p = nullptr;
  ~Scoped() { dev_free(p); }
};

struct BuildArgs {
  DevTables t;
  int64_t N;
  const u64* alpha;
  const u64* beta;
  const int* rows;
  const int* cols;
  const int* col_loc;
  const int* t_order;
  const int* t_cols;
  const int* row_loc;
  const u64* alpha_pos;  // alpha string at each bilinear position
  const u64* beta_tpos;  // beta string at each alpha-major position
  const int* sa_ptr;
  const int* sa_idx;
  const int* sb_ptr;
  const int* sb_idx;
  const int64_t* cost_a;
  const int64_t* cost_b;
  // counts (count pass output, fill pass input)
  int* cntA;
  int* cntB;
  int* cntC;
  int* cntS;
  // CSR (fill pass)
  const int64_t* rowptr;
  int* colidx;
  double* val64;
  float* val32;
  const int64_t* s2ptr;
  int* s2col;
  float* s2val;
  int* err;  // set when a fill pass would write past its row's segment
  // direct sigma (k_pair_sigma): v, s = H u, S^2 u for the selected rows, u (N, nst)
  const double* u;
  const double* uT;  // u in alpha-major order: same-alpha partners are contiguous there
  double* v;
  double* s;
  const double* hdiag;
  const double* sdiag;
  int nst;
  int row_lo, row_hi, row_first, row_step;
  // chunked direct sigma: the fill writes columns of rows [row_lo, row_hi) at
  // rowptr[k] - col_base, class A blocks start at block blk_off, and same-alpha
  // partners are written as alpha-major positions tagged with QP_TAG_T
  int64_t col_base;
  int64_t blk_off;
  int write_s2;
  int tag_t;
  // deletion-key tables of the heavy lines (keys.cu); colkey / rowkey null: none
  KeyView kv[KT_N];
  const unsigned char* colkey;
  const unsigned char* rowkey;
  u64 hmask;
};

constexpr unsigned QP_TAG_T = 0x80000000u;  // column given as alpha-major position

constexpr int MODE_COUNT = 0, MODE_FILL = 1;

__device__ __forceinline__ bool dsel(const BuildArgs& a, int64_t k) {
  return k >= a.row_lo && k < a.row_hi && ((k - a.row_first) % a.row_step) == 0;
}

// acc[st] += h * u[j][st] (j bilinear position; dacc_t: alpha-major position)
__device__ __forceinline__ void dacc_t(const BuildArgs& a, double h, int64_t q, double (&acc)[8]) {
  const double* uj = a.uT + q * a.nst;
#pragma unroll
  for (int st = 0; st < 8; ++st)
    if (st < a.nst) acc[st] = fma(h, __ldg(uj + st), acc[st]);
}
__device__ __forceinline__ void dacc(const BuildArgs& a, double h, int64_t j, double (&acc)[8]) {
  const double* uj = a.u + j * a.nst;
#pragma unroll
  for (int st = 0; st < 8; ++st)
    if (st < a.nst) acc[st] = fma(h, __ldg(uj + st), acc[st]);
}

// ---- class A: same beta column, alpha singles / doubles -------------------
template <int NINT, int MODE>
__global__ void __launch_bounds__(BLK) k_class_a(BuildArgs a) {
  constexpr bool FILL = MODE == MODE_FILL;
  __shared__ u64 tile[TILE * NINT];
  const int64_t r0 = ((int64_t)blockIdx.x + a.blk_off) * BLK;
  if (r0 >= a.N) return;
  const int64_t k = r0 + threadIdx.x;
  const bool valid = k < a.N;
  int cs = 0, ce = 0;
  u64 my[2 * NINT];
  int64_t out = 0;
  bool keyed = false;  // the column has a 2-deletion table: k_same_keyed takes the row
  if (valid) {
    const int b = a.cols[k];
    keyed = a.colkey && (a.colkey[b] & KEY_DOUBLE);
    cs = a.col_loc[b];
    ce = a.col_loc[b + 1];
    const int ai = a.rows[k];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      my[w] = a.alpha[(int64_t)ai * NINT + w];
      my[NINT + w] = a.beta[(int64_t)b * NINT + w];
    }
    if (FILL) out = a.rowptr[k] - a.col_base;
  }
  int cnt = 0;
  const bool act = valid && !keyed && (MODE == MODE_COUNT || dsel(a, k));
  // the tiles span the columns of the block's active rows
  __shared__ int s_lo, s_hi;
  if (threadIdx.x == 0) {
    s_lo = INT_MAX;
    s_hi = INT_MIN;
  }
  __syncthreads();
  if (act) {
    atomicMin(&s_lo, cs);
    atomicMax(&s_hi, ce);
  }
  __syncthreads();
  const int U0 = s_lo, U1 = s_hi;
  for (int t0 = U0; t0 < U1; t0 += TILE) {
    const int tn = min(TILE, U1 - t0);
    __syncthreads();
    for (int i = threadIdx.x; i < tn * NINT; i += BLK) tile[i] = a.alpha_pos[(int64_t)t0 * NINT + i];
    __syncthreads();
    if (act) {
      const int lo = max(cs, t0), hi = min(ce, t0 + tn);
      for (int pos = lo; pos < hi; ++pos) {
        const u64* c = &tile[(pos - t0) * NINT];
        int d = 0;
#pragma unroll
        for (int w = 0; w < NINT; ++w) d += popc64(my[w] ^ c[w]);
        if (d == 2 || d == 4) {
          if (FILL) {  // elements: k_pair_values (stored) or k_pair_sigma (direct)
            if (cnt < a.cntA[k])
              a.colidx[out + cnt] = pos;
            else
              atomicOr(a.err, 1);
          }
          ++cnt;
        }
      }
    }
  }
  if (MODE == MODE_COUNT && valid && !keyed) a.cntA[k] = cnt;
}

// ---- class B: same alpha row, beta singles / doubles ----------------------
template <int NINT, int MODE>
__global__ void __launch_bounds__(BLK) k_class_b(BuildArgs a) {
  constexpr bool FILL = MODE == MODE_FILL;
  __shared__ u64 tile[TILE * NINT];
  const int64_t q0 = (int64_t)blockIdx.x * BLK;
  if (q0 >= a.N) return;
  const int64_t q = q0 + threadIdx.x;
  const bool valid = q < a.N;
  int rs = 0, re = 0;
  int64_t k = 0, out = 0;
  u64 my[2 * NINT];
  bool keyed = false;  // the row has a 2-deletion table: k_same_keyed takes it
  if (valid) {
    k = a.t_order[q];
    const int ai = a.rows[k], bi = a.cols[k];
    keyed = a.rowkey && (a.rowkey[ai] & KEY_DOUBLE);
    rs = a.row_loc[ai];
    re = a.row_loc[ai + 1];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      my[w] = a.alpha[(int64_t)ai * NINT + w];
      my[NINT + w] = a.beta[(int64_t)bi * NINT + w];
    }
    if (FILL) out = a.rowptr[k] + a.cntA[k] - a.col_base;
  }
  int cnt = 0;
  const bool act = valid && !keyed && (MODE == MODE_COUNT || dsel(a, k));
  __shared__ int s_lo, s_hi;
  if (threadIdx.x == 0) {
    s_lo = INT_MAX;
    s_hi = INT_MIN;
  }
  __syncthreads();
  if (act) {
    atomicMin(&s_lo, rs);
    atomicMax(&s_hi, re);
  }
  __syncthreads();
  const int V0 = s_lo, V1 = s_hi;
  for (int t0 = V0; t0 < V1; t0 += TILE) {
    const int tn = min(TILE, V1 - t0);
    __syncthreads();
    for (int i = threadIdx.x; i < tn * NINT; i += BLK) tile[i] = a.beta_tpos[(int64_t)t0 * NINT + i];
    __syncthreads();
    if (act) {
      const int lo = max(rs, t0), hi = min(re, t0 + tn);
      for (int pos = lo; pos < hi; ++pos) {
        const u64* c = &tile[(pos - t0) * NINT];
        int d = 0;
#pragma unroll
        for (int w = 0; w < NINT; ++w) d += popc64(my[NINT + w] ^ c[w]);
        if (d == 2 || d == 4) {
          if (FILL) {  // elements: k_pair_values (stored) or k_pair_sigma (direct)
            if (cnt < a.cntB[k])
              a.colidx[out + cnt] = a.tag_t ? (int)(QP_TAG_T | (unsigned)pos) : a.t_order[pos];
            else
              atomicOr(a.err, 2);
          }
          ++cnt;
        }
      }
    }
  }
  if (MODE == MODE_COUNT && valid && !keyed) a.cntB[k] = cnt;
}

// spin flip test of an alpha-single x beta-single pair: the two excitations
// swap the same two orbitals between the spins (get_s2, s2.irp.f:46-55)
template <int NINT>
__device__ __forceinline__ bool spin_flip(const u64* my, const u64* ca, const u64* cb) {
  bool same = true, core = false;
#pragma unroll
  for (int w = 0; w < NINT; ++w) {
    u64 xa = my[w] ^ ca[w], xb = my[NINT + w] ^ cb[w];
    same &= (xa == xb);
    core |= (xa & my[w] & my[NINT + w]) != 0;
  }
  return same && !core;
}

// ---- class C: alpha single x beta single, one warp per row ----------------
// A column (row) with a 1-deletion table is not scanned: the lanes probe the
// row's alpha (beta) string with each electron removed, and the members of
// each group are the alpha (beta) singles of the row in that column (row).
template <int NINT, int MODE>
__global__ void __launch_bounds__(BLK, 3) k_class_c(BuildArgs a) {
  constexpr bool FILL = MODE == MODE_FILL;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * BLK + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * BLK) >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t k = warp; k < a.N; k += nwarp) {
    if (MODE != MODE_COUNT && !dsel(a, k)) continue;
    const int ai = a.rows[k], bi = a.cols[k];
    u64 my[2 * NINT];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      my[w] = a.alpha[(int64_t)ai * NINT + w];
      my[NINT + w] = a.beta[(int64_t)bi * NINT + w];
    }
    int64_t out = 0, sout = 0;
    if (FILL) {
      out = a.rowptr[k] + a.cntA[k] + a.cntB[k] - a.col_base;
      sout = a.s2ptr[k];
    }
    int cnt = 0, scnt = 0;
    // 32 candidates, one per lane: hit = (ca, cb) is an alpha single x beta
    // single of the row; col is what the fill writes, jpos the bilinear position
    auto step = [&](bool hit, const u64* ca, const u64* cb, int col, int jpos) {
      const unsigned bal = __ballot_sync(FULL, hit);
      const bool flip = hit && spin_flip<NINT>(my, ca, cb);
      const unsigned sbal = __ballot_sync(FULL, flip);
      if (FILL && hit) {  // elements: k_pair_values; S^2 values of spin flips here
        const int64_t o = out + cnt + __popc(bal & lt);
        if (o < a.rowptr[k + 1] - a.col_base)
          a.colidx[o] = col;
        else
          atomicOr(a.err, 4);
        if (flip && a.write_s2) {
          u64 J[2 * NINT];
#pragma unroll
          for (int w = 0; w < NINT; ++w) {
            J[w] = ca[w];
            J[NINT + w] = cb[w];
          }
          double s2;
          h_double_ab<NINT>(a.t, my, J, &s2, nullptr, nullptr);
          const int64_t so = sout + scnt + __popc(sbal & lt);
          if (so < a.s2ptr[k + 1]) {
            a.s2col[so] = jpos;
            a.s2val[so] = (float)s2;
          } else {
            atomicOr(a.err, 8);
          }
        }
      }
      cnt += __popc(bal);
      scnt += __popc(sbal);
    };
    // Lines of the row's singles, 32 at a time: the lanes read the bounds of
    // 32 lines at once, and the candidates of the scanned ones are packed
    // into full warp steps (lane prefix sums over the line lengths), since
    // most lines hold a few determinants; lines with a 1-deletion table are
    // probed afterwards, one after the other.
    const bool by_cols = a.cost_b[bi] <= a.cost_a[ai];
    const int t_beg = by_cols ? a.sb_ptr[bi] : a.sa_ptr[ai];
    const int t_end = by_cols ? a.sb_ptr[bi + 1] : a.sa_ptr[ai + 1];
    const int* lidx = by_cols ? a.sb_idx : a.sa_idx;
    const int* lloc = by_cols ? a.col_loc : a.row_loc;
    const unsigned char* lkey = by_cols ? a.colkey : a.rowkey;
    for (int t0 = t_beg; t0 < t_end; t0 += 32) {
      const int t = t0 + lane;
      int ln = -1, beg = 0, len = 0;
      bool kl = false;
      if (t < t_end) {
        ln = lidx[t];
        beg = lloc[ln];
        kl = lkey && (lkey[ln] & KEY_SINGLE);
        if (!kl) len = lloc[ln + 1] - beg;
      }
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(FULL, incl, 31);
      for (int c0 = 0; c0 < total; c0 += 32) {
        const int ci = c0 + lane;
        int src = 0;  // first lane whose inclusive prefix exceeds ci
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
          const int pr = __shfl_sync(FULL, incl, src + st - 1);
          if (pr <= ci) src += st;
        }
        const int sbeg = __shfl_sync(FULL, beg, src), slen = __shfl_sync(FULL, len, src);
        const int sinc = __shfl_sync(FULL, incl, src), sln = __shfl_sync(FULL, ln, src);
        bool hit = false;
        u64 ca[NINT], cb[NINT];
#pragma unroll
        for (int w = 0; w < NINT; ++w) ca[w] = cb[w] = 0;
        int col = 0, jpos = 0;
        if (ci < total) {
          const int pos = sbeg + (ci - (sinc - slen));
          int d = 0;
          if (by_cols) {  // column sln (a beta single): alpha singles of the row
#pragma unroll
            for (int w = 0; w < NINT; ++w) {
              ca[w] = a.alpha_pos[(int64_t)pos * NINT + w];
              d += popc64(my[w] ^ ca[w]);
            }
            hit = d == 2;
            if (hit) {
#pragma unroll
              for (int w = 0; w < NINT; ++w) cb[w] = a.beta[(int64_t)sln * NINT + w];
              col = jpos = pos;
            }
          } else {  // row sln (an alpha single): beta singles of the row
#pragma unroll
            for (int w = 0; w < NINT; ++w) {
              cb[w] = a.beta_tpos[(int64_t)pos * NINT + w];
              d += popc64(my[NINT + w] ^ cb[w]);
            }
            hit = d == 2;
            if (hit) {
#pragma unroll
              for (int w = 0; w < NINT; ++w) ca[w] = a.alpha[(int64_t)sln * NINT + w];
              jpos = a.t_order[pos];
              col = a.tag_t ? (int)(QP_TAG_T | (unsigned)pos) : jpos;
            }
          }
        }
        step(hit, ca, cb, col, jpos);
      }
      unsigned kb = __ballot_sync(FULL, kl);
      while (kb) {
        const int L = __ffs(kb) - 1;
        kb &= kb - 1;
        const int kln = __shfl_sync(FULL, ln, L);
        const int kbeg = lloc[kln], kend = lloc[kln + 1];
        // keyed line: the lanes probe the row's string (alpha in a column,
        // beta in a row) minus each electron; the members of a group are its
        // singles in that line
        u64 xs[NINT];  // the row's string of the probed spin
#pragma unroll
        for (int w = 0; w < NINT; ++w) xs[w] = by_cols ? my[w] : my[NINT + w];
        const int ne = by_cols ? a.t.na : a.t.nb;
        const int kind = by_cols ? KT_COL1 : KT_ROW1;
        const KeyView& kv = a.kv[kind];
        u64 fixed[NINT];  // the string of the line's other spin
#pragma unroll
        for (int w = 0; w < NINT; ++w) fixed[w] = by_cols ? a.beta[(int64_t)kln * NINT + w] : a.alpha[(int64_t)kln * NINT + w];
        for (int e0 = 0; e0 < ne; e0 += 32) {
          unsigned gs = 0, gl = 0;
          u64 K[NINT];
#pragma unroll
          for (int w = 0; w < NINT; ++w) K[w] = xs[w];
          if (e0 + lane < ne) {
            const int eb = nth_electron<NINT>(K, e0 + lane);
            clear_orbital<NINT>(K, eb);
            if (!key_find(kv, key_hash<NINT>(kind, kln, K, a.hmask), gs, gl)) gl = 0;
          }
          // the members of the 32 probed groups, packed into full warp steps
          int inc = (int)gl;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += y;
          }
          const int tot = __shfl_sync(FULL, inc, 31);
          for (int m0 = 0; m0 < tot; m0 += 32) {
            const int mi = m0 + lane;
            int src = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
              const int pr = __shfl_sync(FULL, inc, src + st - 1);
              if (pr <= mi) src += st;
            }
            const unsigned s0 = __shfl_sync(FULL, gs, src);
            const int i0 = __shfl_sync(FULL, inc, src) - (int)__shfl_sync(FULL, gl, src);
            u64 Kr[NINT];
#pragma unroll
            for (int w = 0; w < NINT; ++w) Kr[w] = __shfl_sync(FULL, K[w], src);
            {
              int pos = -1;
              if (mi < tot) {
                const unsigned tt = (unsigned)(mi - i0);
                pos = kv.mem[s0 + tt];
                if (tt > 0 && kv.mem[s0 + tt - 1] == pos) pos = -1;  // repeated member (colliding keys)
              }
              bool hit = false;
              u64 ca[NINT], cb[NINT];
#pragma unroll
              for (int w = 0; w < NINT; ++w) ca[w] = cb[w] = 0;
              int col = 0, jpos = 0;
              if (pos >= kbeg && pos < kend) {
                int d = 0;
                bool eq = true;
                u64 y[NINT];
#pragma unroll
                for (int w = 0; w < NINT; ++w) {
                  y[w] = by_cols ? a.alpha_pos[(int64_t)pos * NINT + w] : a.beta_tpos[(int64_t)pos * NINT + w];
                  d += popc64(xs[w] ^ y[w]);
                  eq &= (xs[w] & y[w]) == Kr[w];
                }
                hit = d == 2 && eq;
                if (hit) {
#pragma unroll
                  for (int w = 0; w < NINT; ++w) {
                    ca[w] = by_cols ? y[w] : fixed[w];
                    cb[w] = by_cols ? fixed[w] : y[w];
                  }
                  if (by_cols) {
                    col = jpos = pos;
                  } else {
                    jpos = a.t_order[pos];
                    col = a.tag_t ? (int)(QP_TAG_T | (unsigned)pos) : jpos;
                  }
                }
              }
              step(hit, ca, cb, col, jpos);
            }
          }
        }
      }
    }
    if (MODE == MODE_COUNT && lane == 0) {
      a.cntC[k] = cnt;
      a.cntS[k] = scnt;
    }
  }
}

// ---- same-spin pairs of the rows of keyed lines, one warp per row ----------
// SPIN 0: rows of a beta column with a 2-deletion table (class A), SPIN 1:
// rows of an alpha row with one (class B).  The lanes probe 32 of the row's
// C(ne,2) keys at a time; then the members of the 32 groups are packed into
// full warp steps (most groups hold a few strings).
// A member y of the key K of x is a double when |x ^ y| = 4 and x & y = K,
// and a single when |x ^ y| = 2 and K is x & y without its lowest electron:
// each pair is accepted under exactly one key, whatever the hash collisions.
template <int NINT, int MODE, int SPIN>
__global__ void __launch_bounds__(BLK) k_same_keyed(BuildArgs a) {
  constexpr bool FILL = MODE == MODE_FILL;
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int kind = SPIN == 0 ? KT_COL2 : KT_ROW2;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * BLK + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * BLK) >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const KeyView kv = a.kv[kind];
  const int ne = SPIN == 0 ? a.t.na : a.t.nb;
  const int nc = ne * (ne - 1) / 2;
  const unsigned char* lflag = SPIN == 0 ? a.colkey : a.rowkey;
  const u64* strs = SPIN == 0 ? a.alpha_pos : a.beta_tpos;
  const int64_t lo = MODE == MODE_COUNT ? 0 : a.row_lo, hi = MODE == MODE_COUNT ? a.N : a.row_hi;
  if (lflag == nullptr) return;
  for (int64_t k = lo + warp; k < hi; k += nwarp) {
    const int line = SPIN == 0 ? a.cols[k] : a.rows[k];
    if (!(lflag[line] & KEY_DOUBLE)) continue;
    if (MODE != MODE_COUNT && !dsel(a, k)) continue;
    u64 x[NINT];
#pragma unroll
    for (int w = 0; w < NINT; ++w)
      x[w] = SPIN == 0 ? a.alpha_pos[k * NINT + w] : a.beta[(int64_t)a.cols[k] * NINT + w];
    const int ls = SPIN == 0 ? a.col_loc[line] : a.row_loc[line];
    const int le = SPIN == 0 ? a.col_loc[line + 1] : a.row_loc[line + 1];
    int64_t out = 0;
    int cap = 0;
    if (FILL) {
      out = a.rowptr[k] + (SPIN == 0 ? 0 : a.cntA[k]) - a.col_base;
      cap = SPIN == 0 ? a.cntA[k] : a.cntB[k];
    }
    int cnt = 0;
    for (int c0 = 0; c0 < nc; c0 += 32) {
      unsigned gs = 0, gl = 0;
      u64 K[NINT];
#pragma unroll
      for (int w = 0; w < NINT; ++w) K[w] = 0;
      if (c0 + lane < nc) {
        int i, j;
        pair_of_combo(c0 + lane, ne, i, j);
        const int bi = nth_electron<NINT>(x, i), bj = nth_electron<NINT>(x, j);
#pragma unroll
        for (int w = 0; w < NINT; ++w) K[w] = x[w];
        clear_orbital<NINT>(K, bi);
        clear_orbital<NINT>(K, bj);
        if (!key_find(kv, key_hash<NINT>(kind, line, K, a.hmask), gs, gl)) gl = 0;
      }
      // the members of the 32 probed groups, packed into full warp steps
      int inc = (int)gl;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += y;
      }
      const int tot = __shfl_sync(FULL, inc, 31);
      for (int m0 = 0; m0 < tot; m0 += 32) {
        const int mi = m0 + lane;
        int src = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
          const int pr = __shfl_sync(FULL, inc, src + st - 1);
          if (pr <= mi) src += st;
        }
        const unsigned s0 = __shfl_sync(FULL, gs, src);
        const int i0 = __shfl_sync(FULL, inc, src) - (int)__shfl_sync(FULL, gl, src);
        u64 Kr[NINT];
#pragma unroll
        for (int w = 0; w < NINT; ++w) Kr[w] = __shfl_sync(FULL, K[w], src);
        {
          const unsigned t = (unsigned)(mi - i0);
          bool hit = false;
          int p = 0;
          if (mi < tot) {
            p = kv.mem[s0 + t];
            const bool dup = t > 0 && kv.mem[s0 + t - 1] == p;
            if (!dup && p >= ls && p < le) {
              u64 m[NINT];
              int d = 0;
#pragma unroll
              for (int w = 0; w < NINT; ++w) {
                const u64 y = strs[(int64_t)p * NINT + w];
                d += popc64(x[w] ^ y);
                m[w] = x[w] & y;
              }
              if (d == 2) {  // canonical key of a single: drop the lowest common electron
                bool done = false;
#pragma unroll
                for (int w = 0; w < NINT; ++w)
                  if (!done && m[w]) {
                    m[w] &= m[w] - 1;
                    done = true;
                  }
              }
              if (d == 2 || d == 4) {
                bool eq = true;
#pragma unroll
                for (int w = 0; w < NINT; ++w) eq &= m[w] == Kr[w];
                hit = eq;
              }
            }
          }
          const unsigned bal = __ballot_sync(FULL, hit);
          if (FILL && hit) {
            const int o = cnt + __popc(bal & lt);
            if (o < cap)
              a.colidx[out + o] = SPIN == 0 ? p : (a.tag_t ? (int)(QP_TAG_T | (unsigned)p) : a.t_order[p]);
            else
              atomicOr(a.err, SPIN == 0 ? 1 : 2);
          }
          cnt += __popc(bal);
        }
      }
    }
    if (MODE == MODE_COUNT && lane == 0) (SPIN == 0 ? a.cntA : a.cntB)[k] = cnt;
  }
}

// FP64 / FP32 elements of the stored pairs, after the fill pass has written
// their columns: one warp per row, lanes over the row's pairs, so that the
// dependent integral loads of 32 pairs are in flight at once (the fill's
// scanning thread would evaluate its row's pairs one after the other).  The
// class of a pair follows from the two determinants' strings, and each class
// calls the same Slater routine with the same arguments as the scans do, so
// the values are bit-identical.
template <int NINT>
__global__ void __launch_bounds__(BLK) k_pair_values(BuildArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * BLK + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * BLK) >> 5;
  for (int64_t k = warp; k < a.N; k += nwarp) {
    u64 my[2 * NINT];
    const int bi = a.cols[k];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      my[w] = a.alpha_pos[k * NINT + w];
      my[NINT + w] = a.beta[(int64_t)bi * NINT + w];
    }
    const int64_t e1 = a.rowptr[k + 1];
    for (int64_t e = a.rowptr[k] + lane; e < e1; e += 32) {
      const int j = a.colidx[e];
      u64 J[2 * NINT];
      const int bj = a.cols[j];
      bool samea = true, sameb = true;
      int da = 0, db = 0;
#pragma unroll
      for (int w = 0; w < NINT; ++w) {
        J[w] = a.alpha_pos[(int64_t)j * NINT + w];
        J[NINT + w] = a.beta[(int64_t)bj * NINT + w];
        samea &= J[w] == my[w];
        sameb &= J[NINT + w] == my[NINT + w];
        da += popc64(my[w] ^ J[w]);
        db += popc64(my[NINT + w] ^ J[NINT + w]);
      }
      double v;
      if (sameb)  // class A (same beta column)
        v = (da == 2) ? h_mono_spin<NINT>(a.t, my, J, 1, nullptr, nullptr)
                      : h_double_spin<NINT>(a.t, my, J, nullptr, nullptr);
      else if (samea)  // class B (same alpha row)
        v = (db == 2) ? h_mono_spin<NINT>(a.t, my, J, 2, nullptr, nullptr)
                      : h_double_spin<NINT>(a.t, my + NINT, J + NINT, nullptr, nullptr);
      else {  // class C (alpha single x beta single)
        double s2;
        v = h_double_ab<NINT>(a.t, my, J, &s2, nullptr, nullptr);
      }
      a.val64[e] = v;
      a.val32[e] = (float)v;
    }
  }
}

__global__ void k_row_totals(const int* A, const int* B, const int* C, const int* S, int64_t* tot, int64_t* stot,
                             int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= N; k += (int64_t)gridDim.x * blockDim.x) {
    tot[k] = (k < N) ? (int64_t)A[k] + B[k] + C[k] : 0;
    stot[k] = (k < N) ? (int64_t)S[k] : 0;
  }
}

// H_II and <I|S+S-|I> in bilinear order (diag_H_mat_elem, slater_rules.irp.f:1869;
// diag_S_mat_elem, s2.irp.f:1-30)
template <int NINT>
__global__ void k_diag(DevTables t, const u64* alpha, const u64* beta, const int* rows, const int* cols,
                       double* hd, double* sd, float* hd32, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    u64 det[2 * NINT];
    const int ai = rows[k], bi = cols[k];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      det[w] = alpha[(int64_t)ai * NINT + w];
      det[NINT + w] = beta[(int64_t)bi * NINT + w];
    }
    const double h = diag_h<NINT>(t, det);
    hd[k] = h;
    hd32[k] = (float)h;
    sd[k] = diag_s<NINT>(det);
  }
}

BuildArgs index_args(const qpgpu_ctx* c) {
  BuildArgs a{};
  a.t = c->tab;
  a.N = c->N;
  a.alpha = c->d_alpha;
  a.beta = c->d_beta;
  a.rows = c->d_rows;
  a.cols = c->d_cols;
  a.col_loc = c->d_col_loc;
  a.t_order = c->d_t_order;
  a.t_cols = c->d_t_cols;
  a.row_loc = c->d_row_loc;
  a.alpha_pos = c->d_alpha_pos;
  a.beta_tpos = c->d_beta_tpos;
  a.sa_ptr = c->d_sa_ptr;
  a.sa_idx = c->d_sa_idx;
  a.sb_ptr = c->d_sb_ptr;
  a.sb_idx = c->d_sb_idx;
  a.cost_a = c->d_cost_a;
  a.cost_b = c->d_cost_b;
  a.row_lo = 0;
  a.row_hi = (int)c->N;
  a.row_first = 0;
  a.row_step = 1;
  a.col_base = 0;
  a.blk_off = 0;
  a.write_s2 = 1;
  a.tag_t = 0;
  for (int t = 0; t < KT_N; ++t) {
    a.kv[t].slot = c->d_kslot[t];
    a.kv[t].mask = c->kslots[t] > 0 ? (u64)(c->kslots[t] - 1) : 0ull;
    a.kv[t].mem = c->d_kmem[t];
  }
  a.colkey = c->d_colkey;
  a.rowkey = c->d_rowkey;
  a.hmask = c->key_hash_bits >= 64 ? ~0ull : ((1ull << std::max(1, c->key_hash_bits)) - 1ull);
  return a;
}

__global__ void k_rel_offsets(const int64_t* rowptr, int64_t base, int* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int)(rowptr[i] - base);
}

// Each row's columns in ascending order (stored pairs, before the elements
// are evaluated): neighbouring lanes of the sigma gathers then read
// neighbouring coefficients, whatever order the scans and the deletion-key
// probes found the partners in.  Segmented sorts over batches of rows of at
// most 2^30 pairs.
int sort_row_columns(qpgpu_ctx* c) {
  const int64_t N = c->N, P = c->P;
  cudaStream_t st = c->stream;
  if (P == 0) return 0;
  std::vector<int64_t> rp(N + 1);
  QP_CUDA(c, cudaMemcpyAsync(rp.data(), c->d_rowptr, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  const int64_t cap = std::min<int64_t>(P, (int64_t)1 << 30);
  Scoped<int> tmp, offs;
  Scoped<char> work;
  size_t work_bytes = 0;
  QP_CUDA(c, dev_alloc(&tmp.p, (size_t)cap));
  QP_CUDA(c, dev_alloc(&offs.p, (size_t)N + 1));
  for (int64_t r0 = 0; r0 < N;) {
    int64_t r1 = std::upper_bound(rp.begin() + r0 + 1, rp.end(), rp[r0] + cap) - rp.begin() - 1;
    if (r1 <= r0) r1 = r0 + 1;
    const int64_t base = rp[r0], n = rp[r1] - base;
    if (n > cap) return qpgpu_fail(c, QPGPU_ERR_NOMEM, "a row holds more than 2^30 pairs");
    if (n > 0) {
      k_rel_offsets<<<nblocks(r1 - r0 + 1, 256), 256, 0, st>>>(c->d_rowptr + r0, base, offs.p, r1 - r0 + 1);
      size_t tb = 0;
      QP_CUDA(c, cub::DeviceSegmentedSort::SortKeys(nullptr, tb, c->d_colidx + base, tmp.p, (int)n, (int)(r1 - r0),
                                                    offs.p, offs.p + 1, st));
      if (tb > work_bytes) {
        dev_free(work.p);
        work.p = nullptr;
        QP_CUDA(c, dev_alloc(&work.p, tb));
        work_bytes = tb;
      }
      QP_CUDA(c, cub::DeviceSegmentedSort::SortKeys(work.p, tb, c->d_colidx + base, tmp.p, (int)n, (int)(r1 - r0),
                                                    offs.p, offs.p + 1, st));
      QP_CUDA(c, cudaMemcpyAsync(c->d_colidx + base, tmp.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, st));
    }
    r0 = r1;
  }
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaStreamSynchronize(st));
  return 0;
}

template <int NINT>
int build_pairs_t(qpgpu_ctx* c) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  BuildArgs a = index_args(c);
  Scoped<int> cA, cB, cC, cS;
  QP_CUDA(c, dev_alloc(&cA.p, N));
  QP_CUDA(c, dev_alloc(&cB.p, N));
  QP_CUDA(c, dev_alloc(&cC.p, N));
  QP_CUDA(c, dev_alloc(&cS.p, N));
  a.cntA = cA.p;
  a.cntB = cB.p;
  a.cntC = cC.p;
  a.cntS = cS.p;
  const unsigned gAB = nblocks(N, BLK);
  const unsigned gC = nblocks(N * 32, BLK);
  qp_mark(c, "pair setup");
  k_class_a<NINT, MODE_COUNT><<<gAB, BLK, 0, st>>>(a);
  k_same_keyed<NINT, MODE_COUNT, 0><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "count A (same beta)");
  k_class_b<NINT, MODE_COUNT><<<gAB, BLK, 0, st>>>(a);
  k_same_keyed<NINT, MODE_COUNT, 1><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "count B (same alpha)");
  k_class_c<NINT, MODE_COUNT><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "count C (alpha x beta)");
  QP_CUDA(c, cudaGetLastError());
  Scoped<int64_t> tot, stot;
  QP_CUDA(c, dev_alloc(&tot.p, N + 1));
  QP_CUDA(c, dev_alloc(&stot.p, N + 1));
  k_row_totals<<<nblocks(N + 1, 256), 256, 0, st>>>(cA.p, cB.p, cC.p, cS.p, tot.p, stot.p, N);
  QP_CUDA(c, dev_alloc(&c->d_rowptr, N + 1));
  QP_CUDA(c, dev_alloc(&c->d_s2ptr, N + 1));
  size_t tb = 0;
  QP_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, tot.p, c->d_rowptr, (int)(N + 1), st));
  Scoped<char> tmp;
  QP_CUDA(c, dev_alloc(&tmp.p, tb));
  QP_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, tot.p, c->d_rowptr, (int)(N + 1), st));
  QP_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, stot.p, c->d_s2ptr, (int)(N + 1), st));
  QP_CUDA(c, cudaMemcpyAsync(&c->P, c->d_rowptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaMemcpyAsync(&c->P_s2, c->d_s2ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  const int64_t P = c->P, PS = c->P_s2;
  // stored pairs (16 B each, S^2 pairs 8 B) or the direct sigma: forced by
  // qpgpu_set_sigma_mode, else direct when the stored pairs would leave less
  // than 1/16 of the device memory free
  bool direct = c->sigma_mode == QPGPU_SIGMA_DIRECT;
  if (c->sigma_mode == QPGPU_SIGMA_AUTO) {
    size_t fr = 0, total = 0;
    QP_CUDA(c, cudaMemGetInfo(&fr, &total));
    const double need = 16.0 * (double)P + 8.0 * (double)PS + 28.0 * (double)N;
    direct = need + (double)total / 16.0 > (double)fr;
  }
  c->direct = direct;
  if (direct) {
    // the direct sigma regenerates the columns chunk by chunk: keep the
    // per-row counts of the same-spin classes and the row starts on the host
    c->d_cntA = cA.p;
    cA.p = nullptr;
    c->d_cntB = cB.p;
    cB.p = nullptr;
    c->h_rowptr.resize(N + 1);
    QP_CUDA(c, cudaMemcpyAsync(c->h_rowptr.data(), c->d_rowptr, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                               st));
    QP_CUDA(c, dev_alloc(&c->d_hdiag, N));
    QP_CUDA(c, dev_alloc(&c->d_sdiag, N));
    QP_CUDA(c, dev_alloc(&c->d_hdiag32, N));
    k_diag<NINT><<<nblocks(N, 256), 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_hdiag,
                                                   c->d_sdiag, c->d_hdiag32, N);
    qp_mark(c, "diagonal (direct sigma: no pairs stored)");
    QP_CUDA(c, cudaGetLastError());
    QP_CUDA(c, cudaStreamSynchronize(st));
    return 0;
  }
  if (dev_alloc(&c->d_colidx, P) != cudaSuccess || dev_alloc(&c->d_val64, P) != cudaSuccess ||
      dev_alloc(&c->d_val32, P) != cudaSuccess || dev_alloc(&c->d_s2col, PS) != cudaSuccess ||
      dev_alloc(&c->d_s2val, PS) != cudaSuccess) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_NOMEM,
                      "not enough device memory for " + std::to_string(P) + " connected pairs");
  }
  a.rowptr = c->d_rowptr;
  a.colidx = c->d_colidx;
  a.val64 = c->d_val64;
  a.val32 = c->d_val32;
  a.s2ptr = c->d_s2ptr;
  a.s2col = c->d_s2col;
  a.s2val = c->d_s2val;
  Scoped<int> err;
  QP_CUDA(c, dev_alloc(&err.p, 1));
  QP_CUDA(c, cudaMemsetAsync(err.p, 0, sizeof(int), st));
  a.err = err.p;
  qp_mark(c, "scan + alloc");
  k_class_a<NINT, MODE_FILL><<<gAB, BLK, 0, st>>>(a);
  k_same_keyed<NINT, MODE_FILL, 0><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "fill A");
  k_class_b<NINT, MODE_FILL><<<gAB, BLK, 0, st>>>(a);
  k_same_keyed<NINT, MODE_FILL, 1><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "fill B");
  k_class_c<NINT, MODE_FILL><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "fill C");
  {
    int herr = 0;
    QP_CUDA(c, cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    if (herr)
      return qpgpu_fail(c, QPGPU_ERR_STATE, "pair fill disagrees with pair count (" + std::to_string(herr) + ")");
    const int rc = sort_row_columns(c);
    if (rc) return rc;
  }
  qp_mark(c, "row columns sorted");
  k_pair_values<NINT><<<gC, BLK, 0, st>>>(a);
  qp_mark(c, "pair elements");
  QP_CUDA(c, cudaGetLastError());
  int herr = 0;
  QP_CUDA(c, cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  if (herr) return qpgpu_fail(c, QPGPU_ERR_STATE, "pair fill disagrees with pair count (" + std::to_string(herr) + ")");
  QP_CUDA(c, dev_alloc(&c->d_hdiag, N));
  QP_CUDA(c, dev_alloc(&c->d_sdiag, N));
  QP_CUDA(c, dev_alloc(&c->d_hdiag32, N));
  k_diag<NINT><<<nblocks(N, 256), 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_hdiag,
                                                 c->d_sdiag, c->d_hdiag32, N);
  qp_mark(c, "diagonal");
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaStreamSynchronize(st));
  return 0;
}

__global__ void k_alpha_major(const double* u, const int* t_order, double* uT, int64_t N, int nst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * nst; t += (int64_t)gridDim.x * blockDim.x)
    uT[t] = u[(int64_t)t_order[t / nst] * nst + t % nst];
}

// Direct sigma of the rows [row_lo, row_hi) of one chunk, after the fill
// scans wrote their columns into pc (at rowptr[k] - col_base): one warp per
// row, lanes over its pairs; each pair's element is evaluated as in
// k_pair_values (same routines, same arguments), multiplied by the partner's
// coefficients (same-alpha partners, tagged with their alpha-major position,
// read from the alpha-major copy uT, where a row's partners are contiguous),
// and the lanes are combined in a fixed butterfly order.
template <int NINT>
__global__ void __launch_bounds__(BLK, 3) k_pair_sigma(BuildArgs a, const int* __restrict__ pc) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * BLK + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * BLK) >> 5;
  for (int64_t k = a.row_lo + warp; k < a.row_hi; k += nwarp) {
    if (((k - a.row_first) % a.row_step) != 0) continue;
    u64 my[2 * NINT];
    const int bi = a.cols[k];
#pragma unroll
    for (int w = 0; w < NINT; ++w) {
      my[w] = a.alpha_pos[k * NINT + w];
      my[NINT + w] = a.beta[(int64_t)bi * NINT + w];
    }
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, sacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t e0 = a.rowptr[k], e1 = a.rowptr[k + 1];
    // the fill wrote the row's same-beta partners, then its same-alpha
    // partners, then the alpha x beta ones: a same-spin partner shares one
    // string with the row, so only its other string is read
    const int64_t eA = e0 + a.cntA[k], eB = eA + a.cntB[k];
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      const unsigned cj = (unsigned)pc[e - a.col_base];
      const bool via_t = (cj & QP_TAG_T) != 0;
      const int q = (int)(cj & ~QP_TAG_T);
      u64 J[2 * NINT];
      bool samea, sameb;
      int da = 0, db = 0, j = q;
      if (e < eA) {  // same beta column: q is the partner's bilinear position
        samea = false;
        sameb = true;
#pragma unroll
        for (int w = 0; w < NINT; ++w) {
          J[w] = a.alpha_pos[(int64_t)q * NINT + w];
          J[NINT + w] = my[NINT + w];
          da += popc64(my[w] ^ J[w]);
        }
      } else if (e < eB) {  // same alpha row: q is the partner's alpha-major position
        samea = true;
        sameb = false;
#pragma unroll
        for (int w = 0; w < NINT; ++w) {
          J[w] = my[w];
          J[NINT + w] = a.beta_tpos[(int64_t)q * NINT + w];
          db += popc64(my[NINT + w] ^ J[NINT + w]);
        }
      } else {
        j = via_t ? a.t_order[q] : q;
        const int bj = a.cols[j];
        samea = sameb = false;
#pragma unroll
        for (int w = 0; w < NINT; ++w) {
          J[w] = a.alpha_pos[(int64_t)j * NINT + w];
          J[NINT + w] = a.beta[(int64_t)bj * NINT + w];
        }
      }
      double v, s2 = 0.0;
      if (sameb)
        v = (da == 2) ? h_mono_spin<NINT>(a.t, my, J, 1, nullptr, nullptr)
                      : h_double_spin<NINT>(a.t, my, J, nullptr, nullptr);
      else if (samea)
        v = (db == 2) ? h_mono_spin<NINT>(a.t, my, J, 2, nullptr, nullptr)
                      : h_double_spin<NINT>(a.t, my + NINT, J + NINT, nullptr, nullptr);
      else
        v = h_double_ab<NINT>(a.t, my, J, &s2, nullptr, nullptr);
      if (via_t) {
        dacc_t(a, v, q, acc);
        if (s2 != 0.0) dacc_t(a, s2, q, sacc);
      } else {
        dacc(a, v, j, acc);
        if (s2 != 0.0) dacc(a, s2, j, sacc);
      }
    }
#pragma unroll
    for (int st = 0; st < 8; ++st) {
      if (st >= a.nst) break;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        acc[st] += __shfl_xor_sync(0xffffffffu, acc[st], o);
        sacc[st] += __shfl_xor_sync(0xffffffffu, sacc[st], o);
      }
    }
    if (lane == 0) {
      const double hd = a.hdiag[k], sd = a.sdiag[k];
      for (int st = 0; st < a.nst; ++st) {
        const double uk = a.u[k * a.nst + st];
        a.v[k * a.nst + st] = acc[st] + hd * uk;
        a.s[k * a.nst + st] = sacc[st] + sd * uk;
      }
    }
  }
}

// chunks of rows whose columns fit the buffer: fill scans restricted to the
// chunk (S^2 lists not written), then k_pair_sigma
template <int NINT>
int sigma_direct_t(qpgpu_ctx* c, double* v, double* s, const double* u, const double* uT, int nst,
                   cudaStream_t st, int row_lo, int row_hi, int row_first, int row_step) {
  BuildArgs a = index_args(c);
  a.u = u;
  a.uT = uT;
  a.v = v;
  a.s = s;
  a.hdiag = c->d_hdiag;
  a.sdiag = c->d_sdiag;
  a.nst = nst;
  a.rowptr = c->d_rowptr;
  a.s2ptr = c->d_s2ptr;
  a.cntA = c->d_cntA;
  a.cntB = c->d_cntB;
  a.colidx = c->d_direct_cols;
  a.err = c->d_direct_err;
  a.write_s2 = 0;
  a.tag_t = 1;
  a.row_first = row_first;
  a.row_step = row_step;
  const int64_t N = c->N;
  const std::vector<int64_t>& rp = c->h_rowptr;
  const unsigned gAB = nblocks(N, BLK);
  const unsigned gC = nblocks(N * 32, BLK);
  int64_t clo = 0;
  while (clo < N) {
    // largest chi with rp[chi] - rp[clo] <= capacity (at least one row)
    const int64_t lim = rp[clo] + c->direct_cols_cap;
    int64_t chi = std::upper_bound(rp.begin() + clo + 1, rp.end(), lim) - rp.begin() - 1;
    if (chi <= clo) chi = clo + 1;
    const int64_t lo = std::max<int64_t>(clo, row_lo), hi = std::min<int64_t>(chi, row_hi);
    if (lo < hi) {
      a.row_lo = (int)lo;
      a.row_hi = (int)hi;
      a.col_base = rp[lo];
      a.blk_off = lo / BLK;
      const unsigned gA = (unsigned)((hi - 1) / BLK - lo / BLK + 1);
      const unsigned gK = nblocks((hi - lo) * 32, BLK);
      const bool marks = st == c->stream;  // QPGPU_PROFILE=1: phase times on the context stream
      if (marks) qp_mark(c, "direct: chunk start");
      k_class_a<NINT, MODE_FILL><<<gA, BLK, 0, st>>>(a);
      k_same_keyed<NINT, MODE_FILL, 0><<<gK, BLK, 0, st>>>(a);
      if (marks) qp_mark(c, "direct: scan A");
      k_class_b<NINT, MODE_FILL><<<gAB, BLK, 0, st>>>(a);
      k_same_keyed<NINT, MODE_FILL, 1><<<gK, BLK, 0, st>>>(a);
      if (marks) qp_mark(c, "direct: scan B");
      k_class_c<NINT, MODE_FILL><<<gC, BLK, 0, st>>>(a);
      if (marks) qp_mark(c, "direct: scan C");
      k_pair_sigma<NINT><<<nblocks((hi - lo) * 32, BLK), BLK, 0, st>>>(a, c->d_direct_cols);
      if (marks) qp_mark(c, "direct: elements");
    }
    clo = chi;
  }
  QP_CUDA(c, cudaGetLastError());
  return 0;
}

}  // namespace

// Direct sigma (FP64, nothing stored): v, s of the rows selected by (row_lo,
// row_hi, row_first, row_step), bilinear order, u (N, nst).
int qp_sigma_direct(qpgpu_ctx* c, double* v, double* s, const double* u, int nst, cudaStream_t st, int row_lo,
                    int row_hi, int row_first, int row_step) {
  if (nst < 1 || nst > 8) return qpgpu_fail(c, QPGPU_ERR_ARG, "n_st must be in 1..8 per sigma block");
  if (row_step < 1) return qpgpu_fail(c, QPGPU_ERR_ARG, "row step must be >= 1");
  const size_t need = (size_t)c->N * nst;
  if (c->direct_ut_n < need) {
    dev_free(c->d_direct_ut);
    c->d_direct_ut = nullptr;
    c->direct_ut_n = 0;
    QP_CUDA(c, dev_alloc(&c->d_direct_ut, need));
    c->direct_ut_n = need;
  }
  if (!c->d_direct_cols) {  // column buffer: the whole set if it fits in half the free memory
    size_t fr = 0, total = 0;
    QP_CUDA(c, cudaMemGetInfo(&fr, &total));
    int64_t maxrow = 0;
    for (int64_t k = 0; k < c->N; ++k) maxrow = std::max(maxrow, c->h_rowptr[k + 1] - c->h_rowptr[k]);
    int64_t cap = std::min<int64_t>(c->P, (int64_t)(fr / 2 / sizeof(int)));
    // QPGPU_DIRECT_CHUNK_COLS caps the buffer (a memory budget; small values
    // force many chunks)
    if (const char* e = getenv("QPGPU_DIRECT_CHUNK_COLS")) cap = std::min<int64_t>(cap, atoll(e) > 0 ? atoll(e) : cap);
    cap = std::max<int64_t>(cap, maxrow);
    QP_CUDA(c, dev_alloc(&c->d_direct_cols, (size_t)std::max<int64_t>(cap, 1)));
    QP_CUDA(c, dev_alloc(&c->d_direct_err, 1));
    QP_CUDA(c, cudaMemsetAsync(c->d_direct_err, 0, sizeof(int), st));
    c->direct_cols_cap = cap;
  }
  k_alpha_major<<<nblocks((int64_t)need, 256), 256, 0, st>>>(u, c->d_t_order, c->d_direct_ut, c->N, nst);
  const int rc = (c->nint == 1)
                     ? sigma_direct_t<1>(c, v, s, u, c->d_direct_ut, nst, st, row_lo, row_hi, row_first, row_step)
                     : sigma_direct_t<2>(c, v, s, u, c->d_direct_ut, nst, st, row_lo, row_hi, row_first, row_step);
  if (rc) return rc;
  QP_CUDA(c, cudaGetLastError());
  qp_report_marks(c);
  return 0;
}

void qp_free_pairs(qpgpu_ctx* c) {
  void** ps[] = {(void**)&c->d_rowptr, (void**)&c->d_colidx, (void**)&c->d_val64, (void**)&c->d_val32,
                 (void**)&c->d_val32lo,
                 (void**)&c->d_s2ptr, (void**)&c->d_s2col, (void**)&c->d_s2val, (void**)&c->d_hdiag,
                 (void**)&c->d_sdiag, (void**)&c->d_hdiag32};
  for (auto p : ps) {
    dev_free(*p);
    *p = nullptr;
  }
  c->have_pairs = false;
  c->direct = false;
  void** dp[] = {(void**)&c->d_cntA, (void**)&c->d_cntB, (void**)&c->d_direct_cols, (void**)&c->d_direct_err};
  for (auto p : dp) {
    dev_free(*p);
    *p = nullptr;
  }
  c->direct_cols_cap = 0;
  c->h_rowptr.clear();
  c->P = c->P_s2 = 0;
}

int qp_build_pairs(qpgpu_ctx* c) {
  if (c->nint == 1) return build_pairs_t<1>(c);
  if (c->nint == 2) return build_pairs_t<2>(c);
  return qpgpu_fail(c, QPGPU_ERR_ARG, "n_int > 2 is not supported");
}
