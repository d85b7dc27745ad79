// Batched CI problems: many independent determinant sets (each its own
// qpgpu_ctx) solved together.  Quantum Package solves one problem per
// process; callers that need many small CI solves (state-specific or
// multi-reference loops, many small selected spaces) would run them one
// after the other.  Here:
//  * sigma for all problems is ONE persistent launch: every warp pulls
//    (problem, row chunk) work items from a global atomic queue that spans
//    the whole batch, so problems of uneven size (1e3..1e5 determinants)
//    share the GPU without per-problem launches or tail effects;
//  * the Davidson algebra of all problems runs in batched kernels indexed by
//    problem (blockIdx.y), about twenty launches per iteration for the whole
//    batch; the device part of each iteration is captured as CUDA graphs
//    (one per position in the restart cycle) and replayed;
//  * an autotuner times the persistent kernel's launch shape (warps per
//    block x resident blocks per SM) on the first call and keeps the best.
// The Davidson per problem follows davidson_diag_hjj_sjj
// (src/Davidson/diagonalization_hs2.irp.f:52-444) exactly as davidson.cu does.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "qpgpu_internal.cuh"
#include "sigma_device.cuh"

using namespace qpsig;

namespace {

constexpr int BBLK = 256;
constexpr int BMAXS = 8;    // N_st_diag
constexpr int BMAXM = 64;   // N_st_diag * itermax
constexpr int BROWS = 2048; // rows per algebra CTA

inline unsigned gsz(int64_t n, int tpb = BBLK) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (unsigned)g;
}

// one problem of the batch, as the device sees it
struct BProb {
  int64_t N;
  int nst;
  int active;  // 0 once converged (kernels skip it)
  // stored-pair Hamiltonian of its context
  const int64_t* rowptr;
  const int* colidx;
  const double* val64;
  const float* val32;
  const int64_t* s2ptr;
  const int* s2col;
  const float* s2val;
  const double* hdiag;
  const double* sdiag;
  const int* item_row;
  const int* item_sub;
  const int* row_nitems;
  const int* row_item0;
  const int* multi_rows;
  int64_t n_items;
  int64_t item_base;  // first global work item of this problem
  int n_multi;
  // Davidson blocks (itermax blocks of (N, nsd)) and scratch
  double* U;
  double* W;
  double* S;
  double* R;
  float* u32;
  double* pv;
  double* ps;
  int ncta;  // algebra CTAs of this problem
};

// ---- persistent sigma over the whole batch ---------------------------------
template <int NST>
__device__ __forceinline__ void bstore(const BProb& P, int64_t it, int k, int lane, double hv, double sv, bool has_s2,
                                       const double* u, double* v, double* s) {
  constexpr int SH = 5 - Pow2<NST>::lg;
  const int st = lane >> SH;
  const bool owner = (lane & ((1 << SH) - 1)) == 0 && st < NST;
  if (!owner) return;
  if (P.row_nitems[k] == 1) {
    const double uk = u[(int64_t)k * NST + st];
    v[(int64_t)k * NST + st] = hv + P.hdiag[k] * uk;
    s[(int64_t)k * NST + st] = (has_s2 ? sv : 0.0) + P.sdiag[k] * uk;
  } else {
    P.pv[it * NST + st] = hv;
    P.ps[it * NST + st] = has_s2 ? sv : 0.0;
  }
}

// sigma of block `blk` of every active problem: v = W[blk], s = S[blk],
// u = U[blk] (FP64) or the FP32 copy.  Warps take work items from *counter
// (reset to 0 before the launch) until the batch's items are exhausted.
template <int NST, bool F32>
__global__ void k_bsigma(const BProb* __restrict__ probs, int np, int64_t total, int blk,
                         unsigned long long* counter) {
  __shared__ int64_t base[256];
  for (int i = threadIdx.x; i < np; i += blockDim.x) base[i] = probs[i].item_base;
  __syncthreads();
  constexpr int NP = Pow2<NST>::v;
  const int lane = threadIdx.x & 31;
  while (true) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(counter, 1ull);
    g = __shfl_sync(0xffffffffu, g, 0);
    if ((int64_t)g >= total) break;
    int lo = 0, hi = np;  // last problem with base <= g
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (base[mid] <= (int64_t)g) lo = mid; else hi = mid;
    }
    const BProb& P = probs[lo];
    if (!P.active) continue;
    const int64_t it = (int64_t)g - P.item_base;
    const int64_t off = (int64_t)blk * P.N * NST;
    const double* u = P.U + off;
    const float* u32 = P.u32;
    double* v = P.W + off;
    double* s = P.S + off;
    const int k = P.item_row[it];
    const int j = P.item_sub[it];
    const int64_t rb = P.rowptr[k], re = P.rowptr[k + 1];
    const int64_t beg = rb + (int64_t)j * QP_SIGMA_CHUNK;
    const int64_t end = min(beg + (int64_t)QP_SIGMA_CHUNK, re);
    double hsum;
    if (F32) {
      float sum[NP], cmp[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) sum[st] = cmp[st] = 0.f;
      constexpr int U4 = 4;  // independent loads in flight per lane
      for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * U4) {
        int col[U4];
        float hv[U4];
#pragma unroll
        for (int q = 0; q < U4; ++q) {
          const int64_t e = e0 + 32 * q;
          col[q] = e < end ? __ldg(&P.colidx[e]) : k;
          hv[q] = e < end ? __ldg(&P.val32[e]) : 0.f;
        }
#pragma unroll
        for (int q = 0; q < U4; ++q) {
          float x[NST];
          load_row<NST>(u32, col[q], x);
#pragma unroll
          for (int st = 0; st < NST; ++st) {
            const float y = __fmaf_rn(hv[q], x[st], -cmp[st]);
            const float t = __fadd_rn(sum[st], y);
            cmp[st] = __fsub_rn(__fsub_rn(t, sum[st]), y);
            sum[st] = t;
          }
        }
      }
#pragma unroll
      for (int st = 0; st < NP; ++st) cmp[st] = -cmp[st];
      float rh, rl;
      reduce_scatter_ff<NP>(sum, cmp, lane, rh, rl);
      hsum = (double)rh + (double)rl;
    } else {
      double acc[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) acc[st] = 0.0;
      constexpr int U2 = 2;
      for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * U2) {
        int col[U2];
        double hv[U2];
#pragma unroll
        for (int q = 0; q < U2; ++q) {
          const int64_t e = e0 + 32 * q;
          col[q] = e < end ? __ldg(&P.colidx[e]) : k;
          hv[q] = e < end ? __ldg(&P.val64[e]) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < U2; ++q) {
          double x[NST];
          load_row<NST>(u, col[q], x);
#pragma unroll
          for (int st = 0; st < NST; ++st) acc[st] = fma(hv[q], x[st], acc[st]);
        }
      }
      hsum = reduce_scatter64<NP>(acc, lane);
    }
    double ssum = 0.0;
    const int64_t sb = P.s2ptr[k], se = P.s2ptr[k + 1];
    const bool has_s2 = (j == 0) && (se > sb);
    if (has_s2) {
      double sacc[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) sacc[st] = 0.0;
      for (int64_t e = sb + lane; e < se; e += 32) {
        const double sv = (double)__ldg(&P.s2val[e]);
        double x[NST];
        load_row<NST>(u, __ldg(&P.s2col[e]), x);
#pragma unroll
        for (int st = 0; st < NST; ++st) sacc[st] = fma(sv, x[st], sacc[st]);
      }
      ssum = reduce_scatter64<NP>(sacc, lane);
    }
    bstore<NST>(P, it, k, lane, hsum, ssum, has_s2, u, v, s);
  }
}

// rows split over several work items: partials added in item order
__global__ void k_bcombine(const BProb* __restrict__ probs, int nst, int blk) {
  const BProb& P = probs[blockIdx.y];
  if (!P.active) return;
  const int64_t off = (int64_t)blk * P.N * nst;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)P.n_multi * nst;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = P.multi_rows[t / nst];
    const int st = (int)(t % nst);
    const int i0 = P.row_item0[k], ni = P.row_nitems[k];
    double av = 0.0, as = 0.0;
    for (int i = 0; i < ni; ++i) {
      av += P.pv[(int64_t)(i0 + i) * nst + st];
      as += P.ps[(int64_t)(i0 + i) * nst + st];
    }
    const double uk = P.U[off + (int64_t)k * nst + st];
    P.W[off + (int64_t)k * nst + st] = av + P.hdiag[k] * uk;
    P.S[off + (int64_t)k * nst + st] = as + P.sdiag[k] * uk;
  }
}

__global__ void k_bto_float(const BProb* __restrict__ probs, int nst, int blk) {
  const BProb& P = probs[blockIdx.y];
  if (!P.active) return;
  const double* u = P.U + (int64_t)blk * P.N * nst;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N * nst; i += (int64_t)gridDim.x * blockDim.x)
    P.u32[i] = (float)u[i];
}

// ---- batched Davidson algebra (one problem per blockIdx.y) ----------------
enum { AU = 0, AW = 1, AS = 2, AR = 3 };
__device__ __forceinline__ double* barr(const BProb& P, int sel) {
  return sel == AU ? P.U : sel == AW ? P.W : sel == AS ? P.S : P.R;
}

// partial Gram G[i][j] = sum_r A_i[r] B_j[r]: A = blocks a0..a0+nbA-1 of array
// asel, B = block bb of array bsel; rows [c*BROWS, ...) of CTA c; one partial
// per (problem, CTA).  As the single-problem k_gram: a lane owns one row at a
// time and CI = 32 / NSD columns of A for all NSD columns of B (every FP64 FMA
// useful), warps hold column groups (or split the rows when there are fewer
// groups), gridDim.z passes cover the rest, and the sums are combined in a
// fixed order (reduce-scatter over lanes, shared memory over warps).
template <int NSD>
__global__ void __launch_bounds__(BBLK) k_bgram(const BProb* __restrict__ probs, int asel, int a0, int nbA, int bsel,
                                                int bb, double* partial, int pstride,
                                                const int* skip /* per problem, stride sstride */, int sstride,
                                                int ncta_max) {
  constexpr int CI = 32 / NSD;
  constexpr int NW = BBLK / 32;
  __shared__ double red[NW][32];
  const BProb& P = probs[blockIdx.y];
  const int c = blockIdx.x;
  if (!P.active || c >= P.ncta) return;
  const int m = nbA * NSD;
  const int ncg = (m + CI - 1) / CI;
  const int cg0 = blockIdx.z * NW;
  if (cg0 >= ncg) return;
  double* out = partial + ((int64_t)blockIdx.y * ncta_max + c) * pstride;
  if (skip && skip[(int64_t)blockIdx.y * sstride]) {
    for (int p = cg0 * CI * NSD + threadIdx.x; p < min(m, (cg0 + NW) * CI) * NSD; p += BBLK) out[p] = 0.0;
    return;
  }
  const int64_t N = P.N;
  const double* A = barr(P, asel) + (int64_t)a0 * N * NSD;
  const double* B = barr(P, bsel) + (int64_t)bb * N * NSD;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncg_here = min(NW, ncg - cg0);
  const int rg = NW / ncg_here;
  const int cgl = w % ncg_here, rgi = w / ncg_here;
  const bool act = rgi < rg;
  const int cg = cg0 + cgl;
  const int nq = min(CI, m - cg * CI);
  const double* ap[CI];
#pragma unroll
  for (int q = 0; q < CI; ++q) {
    const int i = min(cg * CI + q, m - 1);
    ap[q] = A + (int64_t)(i / NSD) * N * NSD + (i % NSD);
  }
  double acc[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) acc[k] = 0.0;
  const int64_t r0 = (int64_t)c * BROWS, r1 = min(r0 + BROWS, N);
  if (act) {
    for (int64_t r = r0 + (int64_t)rgi * 32 + lane; r < r1; r += (int64_t)rg * 32) {
      double a[CI], b[NSD];
#pragma unroll
      for (int q = 0; q < CI; ++q) a[q] = (q < nq) ? ap[q][r * NSD] : 0.0;
      load_row<NSD>(B, r, b);
#pragma unroll
      for (int q = 0; q < CI; ++q)
        if (q < nq)
#pragma unroll
          for (int j = 0; j < NSD; ++j) acc[q * NSD + j] = fma(a[q], b[j], acc[q * NSD + j]);
    }
  }
  const double v = reduce_scatter64<32>(acc, lane);  // lane L: entry (L / NSD, L % NSD)
  if (act) red[w][lane] = v;
  __syncthreads();
  if (w < ncg_here) {
    double t = 0.0;
    for (int g = 0; g < rg; ++g) t += red[g * ncg_here + w][lane];
    const int q = lane / NSD, j = lane % NSD, i = cg * CI + q;
    if (q < CI && i < m) out[(int64_t)i * NSD + j] = t;
  }
}

// out[problem][p] = sum over its CTAs of the partials (warp per element)
__global__ void k_breduce(const BProb* __restrict__ probs, const double* partial, int pstride, int ncta_max, int npe,
                          double* out, int ostride) {
  const BProb& P = probs[blockIdx.y];
  if (!P.active) return;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  const double* part = partial + (int64_t)blockIdx.y * ncta_max * pstride;
  for (int p = blockIdx.x * wpb + (threadIdx.x >> 5); p < npe; p += gridDim.x * wpb) {
    double s = 0.0;
    for (int c = lane; c < P.ncta; c += 32) s += part[(int64_t)c * pstride + p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[(int64_t)blockIdx.y * ostride + p] = s;
  }
}

// out_t (=, -=) sum_i A_t[i] C[i][j] for up to 3 (array, out block) pairs;
// A = blocks 0..m/nsd-1 (or a0..) of array asel[t]; C per problem.
struct BLin {
  int asel[3], osel[3], oblk[3];
  int n;
};
// NSD = nsd exactly (no predicated columns: on GB300 every FP64 FMA slot
// counts); a thread reads its whole row of each block (16-byte loads for even
// NSD) before it writes, so out may alias the last block of A.
template <int NSD>
__global__ void __launch_bounds__(BBLK) k_blincomb(const BProb* __restrict__ probs, BLin L, int a0, int m_uniform,
                                                   const int* m_per /* nullable */, const double* C, int cstride,
                                                   int sub, const int* skip, int sstride, int include_inactive) {
  const BProb& P = probs[blockIdx.y];
  if (!P.active && !include_inactive) return;
  if (skip && skip[(int64_t)blockIdx.y * sstride]) return;
  const int m = m_per ? m_per[blockIdx.y] : m_uniform;
  if (m <= 0) return;
  __shared__ double Cs[BMAXM * BMAXS];
  const double* Cp = C + (int64_t)blockIdx.y * cstride;
  for (int i = threadIdx.x; i < m * NSD; i += BBLK) Cs[i] = Cp[i];
  __syncthreads();
  const int64_t N = P.N;
  const int nb = m / NSD;
  for (int64_t r = blockIdx.x * (int64_t)BBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * BBLK) {
    for (int t = 0; t < L.n; ++t) {
      const double* A = barr(P, L.asel[t]) + (int64_t)a0 * N * NSD;
      double acc[NSD];
#pragma unroll
      for (int j = 0; j < NSD; ++j) acc[j] = 0.0;
      for (int b = 0; b < nb; ++b) {
        double x[NSD];
        load_row<NSD>(A + (int64_t)b * N * NSD, r, x);
        const double* cb = &Cs[b * NSD * NSD];
#pragma unroll
        for (int cc = 0; cc < NSD; ++cc)
#pragma unroll
          for (int j = 0; j < NSD; ++j) acc[j] = fma(x[cc], cb[cc * NSD + j], acc[j]);
      }
      double* o = barr(P, L.osel[t]) + (int64_t)L.oblk[t] * N * NSD + r * NSD;
#pragma unroll
      for (int j = 0; j < NSD; ++j) o[j] = sub ? o[j] - acc[j] : acc[j];
    }
  }
}

void launch_blincomb(dim3 grid, cudaStream_t st, int nsd, const BProb* probs, BLin L, int a0, int m,
                     const int* mper, const double* C, int cstride, int sub, const int* skip, int sstride,
                     int include_inactive) {
  switch (nsd) {
#define QP_BLC(NS)                                                                                                \
  case NS:                                                                                                        \
    k_blincomb<NS><<<grid, BBLK, 0, st>>>(probs, L, a0, m, mper, C, cstride, sub, skip, sstride, include_inactive); \
    break;
    QP_BLC(1)
    QP_BLC(2)
    QP_BLC(3)
    QP_BLC(4)
    QP_BLC(5)
    QP_BLC(6)
    QP_BLC(7)
    QP_BLC(8)
#undef QP_BLC
  }
}

// per problem: Cholesky of G (nsd x nsd) -> Rinv (upper); zero pivot -> zero column
__global__ void k_bchol(const BProb* __restrict__ probs, int np, int nsd, const double* G, double* Rinv, int stride) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np || !probs[p].active) return;
  const double* g = G + (int64_t)p * stride;
  double* ri = Rinv + (int64_t)p * stride;
  double R[BMAXS][BMAXS], Ri[BMAXS][BMAXS];
  for (int i = 0; i < nsd; ++i)
    for (int j = 0; j < nsd; ++j) R[i][j] = Ri[i][j] = 0.0;
  for (int j = 0; j < nsd; ++j) {
    double d = g[j * nsd + j];
    for (int k = 0; k < j; ++k) d -= R[k][j] * R[k][j];
    if (!(d > 1e-28 * fabs(g[j * nsd + j])) || !(d > 1e-300)) continue;
    R[j][j] = sqrt(d);
    for (int i = j + 1; i < nsd; ++i) {
      double s = g[j * nsd + i];
      for (int k = 0; k < j; ++k) s -= R[k][j] * R[k][i];
      R[j][i] = s / R[j][j];
    }
  }
  for (int j = nsd - 1; j >= 0; --j) {
    if (R[j][j] == 0.0) continue;
    Ri[j][j] = 1.0 / R[j][j];
    for (int i = j - 1; i >= 0; --i) {
      if (R[i][i] == 0.0) continue;
      double s = 0.0;
      for (int k = i + 1; k <= j; ++k) s += R[i][k] * Ri[k][j];
      Ri[i][j] = -s / R[i][i];
    }
  }
  for (int i = 0; i < nsd; ++i)
    for (int j = 0; j < nsd; ++j) ri[i * nsd + j] = Ri[i][j];
}

// per problem: second Gram-Schmidt pass needed? (column lost > half its norm)
__global__ void k_bneed2(const BProb* __restrict__ probs, int np, int nsd, const double* G0, const double* G1, int* skip,
                         int stride, int sstride) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  int need = 0;
  for (int j = 0; j < nsd; ++j) {
    const double a = G0[(int64_t)p * stride + j * nsd + j], b = G1[(int64_t)p * stride + j * nsd + j];
    if (!(b > 0.25 * a)) need = 1;
  }
  skip[(int64_t)p * sstride] = need ? 0 : 1;
}

// Davidson step on block blk of every active problem (diagonalization_hs2.irp.f:
// 386-395); per-(problem, CTA) squared norms of the first nst columns
struct BStepPar {
  double lambda[BMAXS], s2[BMAXS];
};
__global__ void __launch_bounds__(BBLK) k_bstep(const BProb* __restrict__ probs, const BStepPar* par, int nsd, int blk,
                                                double sz2sz, double* partial, int ncta_max) {
  const BProb& P = probs[blockIdx.y];
  if (!P.active || (int)blockIdx.x >= P.ncta) return;
  __shared__ double red[BMAXS][BBLK / 32];
  const BStepPar pp = par[blockIdx.y];
  const int64_t N = P.N, off = (int64_t)blk * N * nsd;
  double acc[BMAXS];
#pragma unroll
  for (int k = 0; k < BMAXS; ++k) acc[k] = 0.0;
  const int64_t r0 = (int64_t)blockIdx.x * BROWS, r1 = min(r0 + BROWS, N);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += BBLK) {
    const double h = P.hdiag[r];
    for (int k = 0; k < nsd; ++k) {
      const int64_t x = off + r * nsd + k;
      const double u = P.U[x];
      const double v = (pp.lambda[k] * u - P.W[x]) * (1.0 + pp.s2[k] * u - P.S[x] - sz2sz) / fmax(h - pp.lambda[k], 1e-2);
      P.U[x] = v;
      if (k < P.nst) acc[k] = fma(v, v, acc[k]);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < BMAXS; ++k) {
    double s = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < BMAXS) {
    double s = 0.0;
    for (int i = 0; i < BBLK / 32; ++i) s += red[threadIdx.x][i];
    partial[((int64_t)blockIdx.y * ncta_max + blockIdx.x) * BMAXS + threadIdx.x] = s;
  }
}

__global__ void k_bcopy_block(const BProb* __restrict__ probs, int nsd, const int* do_copy) {
  const BProb& P = probs[blockIdx.y];
  if (!do_copy[blockIdx.y]) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N * nsd; i += (int64_t)gridDim.x * blockDim.x)
    P.U[i] = P.R[i];
}

constexpr int SMALL = 8 * BMAXM * BMAXS;  // doubles of per-problem small storage
constexpr int O_H = 0, O_S = 512, O_G = 1024, O_RI = 1536, O_Y = 2048, O_G0 = 2560, O_SKIP = 3072;

template <class T>
void bfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

}  // namespace

struct qpgpu_batch {
  std::vector<qpgpu_ctx*> ctx;
  int np = 0;
  cudaStream_t st = nullptr;
  std::string last_error;
  std::vector<BProb> h;
  BProb* d = nullptr;
  int64_t total_items = 0;
  unsigned long long* d_counter = nullptr;
  int sm_count = 0;  // multiprocessors of the problems' device (set at create)
  int tuned_warps = 0, tuned_bps = 0;  // launch shape of the persistent sigma
  double tune_ms = 0.0;
};

namespace {

int bfail(qpgpu_batch* b, int code, const std::string& msg) {
  b->last_error = msg;
  return code;
}
#define QB_CUDA(b, call)                                                                         \
  do {                                                                                           \
    cudaError_t _e = (call);                                                                     \
    if (_e != cudaSuccess) return bfail((b), QPGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// persistent sigma over block `blk` of every active problem
template <int NST>
void launch_bsigma(qpgpu_batch* B, int prec, int blk, int warps, int bps) {
  cudaMemsetAsync(B->d_counter, 0, sizeof(unsigned long long), B->st);
  const int grid = B->sm_count * bps;
  if (prec == QPGPU_FP32)
    k_bsigma<NST, true><<<grid, warps * 32, 0, B->st>>>(B->d, B->np, B->total_items, blk, B->d_counter);
  else
    k_bsigma<NST, false><<<grid, warps * 32, 0, B->st>>>(B->d, B->np, B->total_items, blk, B->d_counter);
}

void bsigma(qpgpu_batch* B, int nsd, int prec, int blk, int warps, int bps) {
  switch (nsd) {
    case 1: launch_bsigma<1>(B, prec, blk, warps, bps); break;
    case 2: launch_bsigma<2>(B, prec, blk, warps, bps); break;
    case 3: launch_bsigma<3>(B, prec, blk, warps, bps); break;
    case 4: launch_bsigma<4>(B, prec, blk, warps, bps); break;
    case 5: launch_bsigma<5>(B, prec, blk, warps, bps); break;
    case 6: launch_bsigma<6>(B, prec, blk, warps, bps); break;
    case 7: launch_bsigma<7>(B, prec, blk, warps, bps); break;
    default: launch_bsigma<8>(B, prec, blk, warps, bps); break;
  }
  int maxm = 0;
  for (auto& p : B->h) maxm = std::max(maxm, p.n_multi);
  if (maxm > 0) k_bcombine<<<dim3(gsz((int64_t)maxm * nsd), B->np), BBLK, 0, B->st>>>(B->d, nsd, blk);
}

struct BDav {
  qpgpu_batch* B;
  int nsd, itermax, ncta_max;
  double* part = nullptr;   // [np][ncta_max][512]
  double* small = nullptr;  // [np][SMALL]
  BStepPar* step = nullptr;
  int* mper = nullptr;      // [np] basis size of each problem's last Ritz step
  int* copyf = nullptr;     // [np] re-contract flags
  std::vector<void*> owned;
  ~BDav() {
    bfree(part);
    bfree(small);
    bfree(step);
    bfree(mper);
    bfree(copyf);
    for (void* p : owned) cudaFree(p);
  }
};

void bgram(BDav& D, int asel, int a0, int nbA, int bsel, int bb, int out_off, const int* skip) {
  qpgpu_batch* B = D.B;
  const int m = nbA * D.nsd;
  const int ci = 32 / D.nsd;
  const int ncg = (m + ci - 1) / ci;
  const dim3 grid(D.ncta_max, B->np, (ncg + BBLK / 32 - 1) / (BBLK / 32));
  const int ss = SMALL * 2;
  switch (D.nsd) {
#define QP_BG(NS)                                                                                          \
  case NS:                                                                                                 \
    k_bgram<NS><<<grid, BBLK, 0, B->st>>>(B->d, asel, a0, nbA, bsel, bb, D.part, 512, skip, ss, D.ncta_max); \
    break;
    QP_BG(1)
    QP_BG(2)
    QP_BG(3)
    QP_BG(4)
    QP_BG(5)
    QP_BG(6)
    QP_BG(7)
    QP_BG(8)
#undef QP_BG
  }
  k_breduce<<<dim3(gsz((int64_t)m * D.nsd * 32), B->np), BBLK, 0, B->st>>>(B->d, D.part, 512, D.ncta_max, m * D.nsd,
                                                                           D.small + out_off, SMALL);
}

void blin(BDav& D, BLin L, int a0, int m, const int* mper, int coff, int sub, const int* skip, int include_inactive,
          int64_t maxN) {
  qpgpu_batch* B = D.B;
  launch_blincomb(dim3(gsz(maxN), B->np), B->st, D.nsd, B->d, L, a0, m, mper, D.small + coff, SMALL, sub, skip,
                  SMALL * 2, include_inactive);
}

// device part of an iteration before the small eigenproblems: orthonormalise
// block b, sigma on it, new Gram columns into O_H / O_S
void segment_a(BDav& D, int b, int prec, int64_t maxN) {
  qpgpu_batch* B = D.B;
  const int nsd = D.nsd;
  int* skip = (int*)(D.small + O_SKIP);
  if (b > 0) {
    bgram(D, AU, b, 1, AU, b, O_G0, nullptr);
    bgram(D, AU, 0, b, AU, b, O_H, nullptr);
    BLin L{{AU, 0, 0}, {AU, 0, 0}, {b, 0, 0}, 1};
    blin(D, L, 0, b * nsd, nullptr, O_H, 1, nullptr, 0, maxN);
    bgram(D, AU, b, 1, AU, b, O_G, nullptr);
    k_bneed2<<<gsz(B->np, 64), 64, 0, B->st>>>(B->d, B->np, nsd, D.small + O_G0, D.small + O_G, skip, SMALL, SMALL * 2);
    bgram(D, AU, 0, b, AU, b, O_H, skip);
    blin(D, L, 0, b * nsd, nullptr, O_H, 1, skip, 0, maxN);
  }
  for (int pass = 0; pass < 2; ++pass) {
    bgram(D, AU, b, 1, AU, b, O_G, nullptr);
    k_bchol<<<gsz(B->np, 64), 64, 0, B->st>>>(B->d, B->np, nsd, D.small + O_G, D.small + O_RI, SMALL);
    BLin L{{AU, 0, 0}, {AU, 0, 0}, {b, 0, 0}, 1};
    blin(D, L, b, nsd, nullptr, O_RI, 0, nullptr, 0, maxN);
  }
  if (prec == QPGPU_FP32) k_bto_float<<<dim3(gsz(maxN * nsd), B->np), BBLK, 0, B->st>>>(B->d, nsd, b);
  bsigma(B, nsd, prec, b, B->tuned_warps, B->tuned_bps);
  bgram(D, AU, 0, b + 1, AW, b, O_H, nullptr);
  bgram(D, AU, 0, b + 1, AS, b, O_S, nullptr);
}

// device part after them: Ritz vectors into block b+1 and the Davidson step
void segment_b(BDav& D, int b, double sz2sz, int64_t maxN) {
  qpgpu_batch* B = D.B;
  const int nsd = D.nsd;
  BLin L{{AU, AW, AS}, {AU, AW, AS}, {b + 1, b + 1, b + 1}, 3};
  blin(D, L, 0, (b + 1) * nsd, nullptr, O_Y, 0, nullptr, 0, maxN);
  k_bstep<<<dim3(D.ncta_max, B->np), BBLK, 0, B->st>>>(B->d, D.step, nsd, b + 1, sz2sz, D.part, D.ncta_max);
}

struct GraphCache {
  std::vector<cudaGraphExec_t> g;
  ~GraphCache() {
    for (auto e : g)
      if (e) cudaGraphExecDestroy(e);
  }
};

// capture `fn` on the batch stream once and replay it afterwards
template <class F>
int replay(qpgpu_batch* B, cudaGraphExec_t& exec, F fn) {
  if (!exec) {
    cudaGraph_t g = nullptr;
    QB_CUDA(B, cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal));
    fn();
    QB_CUDA(B, cudaStreamEndCapture(B->st, &g));
    QB_CUDA(B, cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
  }
  QB_CUDA(B, cudaGraphLaunch(exec, B->st));
  return 0;
}

}  // namespace

extern "C" {

int qpgpu_batch_create(qpgpu_ctx* const* ctxs, int n, qpgpu_batch** out) {
  if (!ctxs || !out || n < 1 || n > 256) return QPGPU_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!ctxs[i] || !ctxs[i]->have_pairs || ctxs[i]->direct || ctxs[i]->device != ctxs[0]->device)
      return QPGPU_ERR_STATE;
  qpgpu_batch* B = new qpgpu_batch();
  B->ctx.assign(ctxs, ctxs + n);
  B->np = n;
  B->sm_count = ctxs[0]->n_sm;
  if (cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void**)&B->d_counter, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc((void**)&B->d, n * sizeof(BProb)) != cudaSuccess) {
    cudaGetLastError();
    delete B;
    return QPGPU_ERR_CUDA;
  }
  // the fixed-order group reduction of k_bgram uses up to 64 KB of shared memory
  B->h.resize(n);
  int64_t base = 0;
  for (int i = 0; i < n; ++i) {
    qpgpu_ctx* c = ctxs[i];
    BProb& p = B->h[i];
    std::memset(&p, 0, sizeof(BProb));
    p.N = c->N;
    p.active = 1;
    p.rowptr = c->d_rowptr;
    p.colidx = c->d_colidx;
    p.val64 = c->d_val64;
    p.val32 = c->d_val32;
    p.s2ptr = c->d_s2ptr;
    p.s2col = c->d_s2col;
    p.s2val = c->d_s2val;
    p.hdiag = c->d_hdiag;
    p.sdiag = c->d_sdiag;
    p.item_row = c->items.item_row;
    p.item_sub = c->items.item_sub;
    p.row_nitems = c->items.row_nitems;
    p.row_item0 = c->items.row_item0;
    p.multi_rows = c->items.multi_rows;
    p.n_items = c->items.n_items;
    p.n_multi = c->items.n_multi;
    p.item_base = base;
    p.ncta = (int)((c->N + BROWS - 1) / BROWS);
    base += p.n_items;
  }
  B->total_items = base;
  *out = B;
  return QPGPU_OK;
}

int qpgpu_batch_destroy(qpgpu_batch* B) {
  if (!B) return QPGPU_ERR_ARG;
  cudaStreamSynchronize(B->st);
  cudaFree(B->d);
  cudaFree(B->d_counter);
  cudaStreamDestroy(B->st);
  delete B;
  return QPGPU_OK;
}

const char* qpgpu_batch_last_error(qpgpu_batch* B) { return B ? B->last_error.c_str() : "null batch"; }

// Batched Davidson (davidson_diag_hjj_sjj on every problem at once).  u_in[p]:
// host (dim_in[p], n_states_diag) guess vectors of problem p in psi_det order,
// overwritten with the eigenvectors; energies / s2_out: n x n_states_diag;
// n_states[p] <= n_states_diag.  params as for qpgpu_davidson_hs2 (the
// learned preconditioner and the capture are not available in a batch).
int qpgpu_batch_davidson(qpgpu_batch* B, double* const* u_in, const int64_t* dim_in, const int* n_states,
                         double* energies, double* s2_out, const qpgpu_davidson_params* prm,
                         qpgpu_batch_stats* stats) {
  if (!B || !u_in || !dim_in || !n_states || !energies || !s2_out || !prm) return QPGPU_ERR_ARG;
  const int np = B->np, nsd = prm->n_states_diag;
  if (nsd < 1 || nsd > BMAXS || (prm->precision != QPGPU_FP64 && prm->precision != QPGPU_FP32) ||
      prm->preconditioner != 0)
    return bfail(B, QPGPU_ERR_ARG, "bad batch Davidson parameters (n_states_diag <= 8, diagonal step only)");
  int64_t minN = INT64_MAX, maxN = 0;
  for (int p = 0; p < np; ++p) {
    if (n_states[p] < 1 || n_states[p] > nsd || dim_in[p] < B->h[p].N || !u_in[p])
      return bfail(B, QPGPU_ERR_ARG, "bad per-problem arguments");
    minN = std::min(minN, B->h[p].N);
    maxN = std::max(maxN, B->h[p].N);
  }
  if ((int64_t)nsd * 3 > minN) return bfail(B, QPGPU_ERR_ARG, "N_st_diag*3 > sze for a problem of the batch");
  int itermax = std::max(3, (int)std::min<int64_t>(prm->davidson_sze_max, minN / nsd));
  while (itermax * nsd > BMAXM) --itermax;
  const bool mixed = prm->precision == QPGPU_FP32;
  const int max_iter = prm->max_iter > 0 ? prm->max_iter : 1000;
  cudaStream_t st = B->st;
  BDav D;
  D.B = B;
  D.nsd = nsd;
  D.itermax = itermax;
  D.ncta_max = 1;
  for (auto& p : B->h) D.ncta_max = std::max(D.ncta_max, p.ncta);
  // per-problem Davidson storage
  for (int p = 0; p < np; ++p) {
    BProb& P = B->h[p];
    const size_t blk = (size_t)P.N * nsd;
    double *U, *W, *S, *R, *pv, *ps;
    float* u32;
    if (cudaMalloc((void**)&U, blk * itermax * 8) != cudaSuccess ||
        cudaMalloc((void**)&W, blk * itermax * 8) != cudaSuccess ||
        cudaMalloc((void**)&S, blk * itermax * 8) != cudaSuccess || cudaMalloc((void**)&R, blk * 8) != cudaSuccess ||
        cudaMalloc((void**)&u32, blk * 4 + 16) != cudaSuccess ||
        cudaMalloc((void**)&pv, (size_t)P.n_items * nsd * 8 + 16) != cudaSuccess ||
        cudaMalloc((void**)&ps, (size_t)P.n_items * nsd * 8 + 16) != cudaSuccess) {
      cudaGetLastError();
      return bfail(B, QPGPU_ERR_NOMEM, "batch Davidson storage does not fit on the device");
    }
    for (void* x : {(void*)U, (void*)W, (void*)S, (void*)R, (void*)u32, (void*)pv, (void*)ps}) D.owned.push_back(x);
    P.U = U;
    P.W = W;
    P.S = S;
    P.R = R;
    P.u32 = u32;
    P.pv = pv;
    P.ps = ps;
    P.nst = n_states[p];
    P.active = 1;
  }
  QB_CUDA(B, cudaMalloc((void**)&D.part, (size_t)np * D.ncta_max * 512 * 8));
  QB_CUDA(B, cudaMalloc((void**)&D.small, (size_t)np * SMALL * 8));
  QB_CUDA(B, cudaMalloc((void**)&D.step, (size_t)np * sizeof(BStepPar)));
  QB_CUDA(B, cudaMalloc((void**)&D.mper, (size_t)np * sizeof(int)));
  QB_CUDA(B, cudaMalloc((void**)&D.copyf, (size_t)np * sizeof(int)));
  QB_CUDA(B, cudaMemsetAsync(D.small, 0, (size_t)np * SMALL * 8, st));
  QB_CUDA(B, cudaMemcpyAsync(B->d, B->h.data(), np * sizeof(BProb), cudaMemcpyHostToDevice, st));
  // guesses -> block 0 (bilinear order)
  for (int p = 0; p < np; ++p) {
    BProb& P = B->h[p];
    QB_CUDA(B, cudaMemcpy2DAsync(P.R, P.N * 8, u_in[p], dim_in[p] * 8, P.N * 8, nsd, cudaMemcpyHostToDevice, st));
    qp_to_bilinear(P.R, P.N, B->ctx[p]->d_order, P.U, nullptr, nsd, P.N, st);
  }
  QB_CUDA(B, cudaStreamSynchronize(st));
  // autotune the persistent sigma's launch shape once per batch
  if (!B->tuned_warps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    const int warps_c[2] = {4, 8}, bps_c[3] = {2, 4, 8};
    auto t0 = std::chrono::steady_clock::now();
    for (int wi = 0; wi < 2; ++wi)
      for (int bi = 0; bi < 3; ++bi) {
        bsigma(B, nsd, QPGPU_FP64, 0, warps_c[wi], bps_c[bi]);
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2; ++r) bsigma(B, nsd, QPGPU_FP64, 0, warps_c[wi], bps_c[bi]);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          B->tuned_warps = warps_c[wi];
          B->tuned_bps = bps_c[bi];
        }
      }
    B->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    QB_CUDA(B, cudaGetLastError());
  }
  const double Sz0 = 0.5 * (B->ctx[0]->na - B->ctx[0]->nb);
  std::vector<double> sz2sz(np);
  for (int p = 0; p < np; ++p) {
    const double Sz = 0.5 * (B->ctx[p]->na - B->ctx[p]->nb);
    sz2sz[p] = Sz * (Sz - 1.0);
  }
  for (int p = 0; p < np; ++p)
    if (sz2sz[p] != Sz0 * (Sz0 - 1.0))
      return bfail(B, QPGPU_ERR_ARG, "all problems of a batch must have the same S_z");
  const int mmax = itermax * nsd;
  std::vector<std::vector<double>> H(np, std::vector<double>((size_t)mmax * mmax)), S2m = H;
  std::vector<double> hostsmall((size_t)np * 1024), ystage((size_t)np * 512, 0.0), parts((size_t)np * D.ncta_max * BMAXS);
  std::vector<BStepPar> sp(np);
  std::vector<std::vector<double>> lam(np, std::vector<double>(mmax)), s2v = lam;
  std::vector<int> mper(np, 0), copyf(np, 0), conv(np, 0), iters(np, 0);
  std::vector<double> res((size_t)np * BMAXS, 0.0);
  GraphCache ga, gb;
  ga.g.assign(2 * itermax, nullptr);
  gb.g.assign(itermax, nullptr);
  cudaEvent_t t_start, t_end;
  cudaEventCreate(&t_start);
  cudaEventCreate(&t_end);
  cudaEventRecord(t_start, st);
  int n_iter = 0, launches = 0;
  bool all_done = false;
  while (!all_done && n_iter < max_iter) {
    int shift2 = 0;
    for (int iter = 1; iter <= itermax - 1 && !all_done && n_iter < max_iter; ++iter) {
      const int b = iter - 1;
      shift2 = nsd * iter;
      const int prec = (mixed && iter > 1) ? QPGPU_FP32 : QPGPU_FP64;
      int rc = replay(B, ga.g[2 * b + (prec == QPGPU_FP32)], [&] { segment_a(D, b, prec, maxN); });
      if (rc) return rc;
      ++launches;
      ++n_iter;
      QB_CUDA(B, cudaMemcpy2DAsync(hostsmall.data(), 1024 * 8, D.small, SMALL * 8, 1024 * 8, np,
                                   cudaMemcpyDeviceToHost, st));
      QB_CUDA(B, cudaStreamSynchronize(st));
      for (int p = 0; p < np; ++p) {
        if (!B->h[p].active) continue;
        ++iters[p];
        std::vector<double>& h = H[p];
        std::vector<double>& s = S2m[p];
        for (int i = 0; i < shift2; ++i)
          for (int j = 0; j < nsd; ++j) {
            const int col = b * nsd + j;
            if (i > col) continue;
            h[(size_t)i * mmax + col] = h[(size_t)col * mmax + i] = hostsmall[(size_t)p * 1024 + O_H + i * nsd + j];
            s[(size_t)i * mmax + col] = s[(size_t)col * mmax + i] = hostsmall[(size_t)p * 1024 + O_S + i * nsd + j];
          }
        std::vector<double> hs((size_t)shift2 * shift2), ss((size_t)shift2 * shift2), w, y;
        for (int i = 0; i < shift2; ++i)
          for (int j = 0; j < shift2; ++j) {
            hs[(size_t)i * shift2 + j] = h[(size_t)i * mmax + j];
            ss[(size_t)i * shift2 + j] = s[(size_t)i * mmax + j];
          }
        qp_eigh(hs, shift2, w, y);
        for (int k = 0; k < shift2; ++k) {
          double acc = 0.0;
          for (int i = 0; i < shift2; ++i) {
            double t = 0.0;
            for (int j = 0; j < shift2; ++j) t += ss[(size_t)i * shift2 + j] * y[(size_t)j * shift2 + k];
            acc += y[(size_t)i * shift2 + k] * t;
          }
          lam[p][k] = w[k];
          s2v[p][k] = acc + sz2sz[p];
        }
        if (prm->s2_eig) {
          const double ex = Sz0 * (Sz0 + 1.0);
          std::vector<char> ok(shift2);
          for (int k = 0; k < shift2; ++k) ok[k] = std::fabs(s2v[p][k] - ex) < 0.6;
          for (int k = 0; k < shift2; ++k) {
            if (ok[k]) continue;
            for (int l = k + 1; l < shift2; ++l)
              if (ok[l]) {
                for (int i = 0; i < shift2; ++i) std::swap(y[(size_t)i * shift2 + k], y[(size_t)i * shift2 + l]);
                std::swap(s2v[p][k], s2v[p][l]);
                std::swap(lam[p][k], lam[p][l]);
                ok[k] = 1;
                ok[l] = 0;
                break;
              }
          }
        }
        for (int i = 0; i < shift2; ++i)
          for (int j = 0; j < nsd; ++j) ystage[(size_t)p * 512 + i * nsd + j] = y[(size_t)i * shift2 + j];
        for (int k = 0; k < nsd; ++k) {
          sp[p].lambda[k] = lam[p][k];
          sp[p].s2[k] = s2v[p][k];
        }
        mper[p] = shift2;
      }
      QB_CUDA(B, cudaMemcpy2DAsync(D.small + O_Y, SMALL * 8, ystage.data(), 512 * 8, 512 * 8, np,
                                   cudaMemcpyHostToDevice, st));
      QB_CUDA(B, cudaMemcpyAsync(D.step, sp.data(), np * sizeof(BStepPar), cudaMemcpyHostToDevice, st));
      rc = replay(B, gb.g[b], [&] { segment_b(D, b, sz2sz[0], maxN); });
      if (rc) return rc;
      QB_CUDA(B, cudaMemcpyAsync(parts.data(), D.part, parts.size() * 8, cudaMemcpyDeviceToHost, st));
      QB_CUDA(B, cudaStreamSynchronize(st));
      bool changed = false;
      all_done = true;
      for (int p = 0; p < np; ++p) {
        if (!B->h[p].active) continue;
        double mx = 0.0;
        for (int k = 0; k < B->h[p].nst; ++k) {
          double r = 0.0;
          for (int q = 0; q < B->h[p].ncta; ++q) r += parts[((size_t)p * D.ncta_max + q) * BMAXS + k];
          res[(size_t)p * BMAXS + k] = r;
          mx = std::max(mx, r);
        }
        if (mx > 1e8 || !std::isfinite(mx)) return bfail(B, QPGPU_ERR_DAVIDSON, "Davidson failed: residual above 1e8");
        if (mx < prm->threshold && prec == QPGPU_FP64 && (iter >= 2 || mixed)) {
          B->h[p].active = 0;  // frozen; re-contracted at the end of the cycle
          conv[p] = 1;
          copyf[p] = 1;
          changed = true;
        } else {
          all_done = false;
        }
      }
      if (changed) QB_CUDA(B, cudaMemcpyAsync(B->d, B->h.data(), np * sizeof(BProb), cudaMemcpyHostToDevice, st));
    }
    // re-contract (diagonalization_hs2.irp.f:419-420) of the problems still
    // running and of those that converged during this cycle
    for (int p = 0; p < np; ++p)
      if (B->h[p].active) copyf[p] = 1;
    QB_CUDA(B, cudaMemcpyAsync(D.mper, mper.data(), np * sizeof(int), cudaMemcpyHostToDevice, st));
    QB_CUDA(B, cudaMemcpyAsync(D.copyf, copyf.data(), np * sizeof(int), cudaMemcpyHostToDevice, st));
    BLin L{{AU, 0, 0}, {AR, 0, 0}, {0, 0, 0}, 1};
    launch_blincomb(dim3(gsz(maxN), np), st, nsd, B->d, L, 0, shift2, D.mper, D.small + O_Y, SMALL, 0, nullptr, 0, 1);
    k_bcopy_block<<<dim3(gsz(maxN * nsd), np), BBLK, 0, st>>>(B->d, nsd, D.copyf);
    QB_CUDA(B, cudaGetLastError());
    for (int p = 0; p < np; ++p) {
      copyf[p] = 0;
      if (B->h[p].active) std::fill(H[p].begin(), H[p].end(), 0.0), std::fill(S2m[p].begin(), S2m[p].end(), 0.0);
    }
    QB_CUDA(B, cudaMemcpyAsync(D.copyf, copyf.data(), np * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  cudaEventRecord(t_end, st);
  QB_CUDA(B, cudaStreamSynchronize(st));
  float total_ms = 0.f;
  cudaEventElapsedTime(&total_ms, t_start, t_end);
  cudaEventDestroy(t_start);
  cudaEventDestroy(t_end);
  int n_conv = 0;
  for (int p = 0; p < np; ++p) {
    BProb& P = B->h[p];
    qp_from_bilinear(P.U, P.N, B->ctx[p]->d_order, P.R, nsd, P.N, st);
    QB_CUDA(B, cudaMemcpy2DAsync(u_in[p], dim_in[p] * 8, P.R, P.N * 8, P.N * 8, nsd, cudaMemcpyDeviceToHost, st));
    for (int k = 0; k < nsd; ++k) {
      energies[(size_t)p * nsd + k] = lam[p][k];
      s2_out[(size_t)p * nsd + k] = s2v[p][k];
    }
    n_conv += conv[p];
    P.active = 1;
  }
  QB_CUDA(B, cudaStreamSynchronize(st));
  if (stats) {
    stats->n_iter = n_iter;
    stats->n_sigma_launches = launches;
    stats->n_converged = n_conv;
    stats->elapsed_ms = total_ms;
    stats->tune_ms = B->tune_ms;
    stats->tuned_warps = B->tuned_warps;
    stats->tuned_blocks_per_sm = B->tuned_bps;
    if (stats->iters)
      for (int p = 0; p < np; ++p) stats->iters[p] = iters[p];
  }
  return QPGPU_OK;
}

}  // extern "C"
