// Block Davidson on the device: davidson_diag_hjj_sjj
// (src/Davidson/diagonalization_hs2.irp.f:52-444) over the stored-pair sigma.
//
// Vectors live in bilinear order as blocks of N_st_diag columns, each block
// (N_det, N_st_diag) with states fastest (the sigma layout).  Per iteration:
//   orthonormalise the new block against the previous ones      (:216, ortho_qr)
//   W, S = sigma(new block)                                      (:222-226)
//   new Gram columns h(:,new) = U^T W_new, s(:,new) = U^T S_new   (:232-238)
//   small eigenproblem, S^2 of the Ritz vectors, s2_eig filter   (:284-326)
//   Ritz vectors U y, W y, S y                                   (:376-381)
//   Davidson step and squared residual norms                     (:386-395)
// The reference recomputes the whole Gram matrices and QR-factors the whole
// basis every iteration; the columns of earlier blocks do not change within a
// restart cycle, so only the new columns are formed (h and s are read in their
// upper triangle, as dsyev('U') reads them) and the new block is
// orthogonalised by two classical Gram-Schmidt passes and CholQR2.
//
// Mixed precision: with QPGPU_FP32, sigma runs in FP32 (Kahan sums) except on
// the first iteration of each restart cycle, which runs the FP64 sigma on the
// re-contracted Ritz vectors (defect correction).  Convergence is accepted only
// on an FP64 iteration; an FP32 iteration that meets the threshold forces a
// restart, so the reported energies are FP64 ones.  With QPGPU_FF the restart
// sigma is the float-float one (k_sigma_ff, FP64-class accuracy on the FP32
// pipes) and convergence is accepted on those iterations.  In both mixed
// modes the tall-skinny algebra runs on the FP32 pipes: the Gram blocks of
// the Gram-Schmidt passes and projections (k_gram_ff on float-float copies
// of the blocks), the updates, the restart iterations' Ritz vectors and the
// re-contraction in float-float (k_lincomb_ff); the Ritz vectors of
// FP32-sigma iterations in FP32 (k_lincomb32); the step's preconditioner and
// norms in FP32 after an FP64 residual numerator (k_step_mixed).  The small
// factorisations and the eigenproblem stay FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

#include "qpgpu_internal.cuh"
#include "sigma_device.cuh"

// Host eigen-solver for the small projected matrix (stands in for
// lapack_diag/dsyev, LinearAlgebra.irp.f:446-512): eigenvalues ascending,
// eigenvectors in the columns of v (n x n, row-major v[i*n+j] = component i of
// vector j).  Householder reduction to tridiagonal form with the reflections
// accumulated, then the implicit QL iteration with a Wilkinson-type shift on
// the tridiagonal matrix (Bowdler, Martin, Reinsch and Wilkinson, Numer. Math.
// 11 (1968) 293; Golub and Van Loan, Matrix Computations, sec. 8.3): about
// 9 n^3 flops with a fixed iteration count, where a cyclic Jacobi sweep costs
// about 4 n^3 and needs several sweeps.
void qp_eigh(std::vector<double> a, int n, std::vector<double>& w, std::vector<double>& v) {
  w.assign(n, 0.0);
  v.assign((size_t)n * n, 0.0);
  if (n <= 0) return;
  // z holds the eigenvectors as rows (z[j*n+i] = component i of vector j), so
  // that every update below runs along contiguous rows
  std::vector<double> z((size_t)n * n, 0.0), x(n), p(n), q(n), t(n), e(n, 0.0);
  for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  // A <- H_k A H_k zeroes column k below the sub-diagonal; Z <- H_k Z
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // length of the reflected part (rows k+1..n-1)
    double nrm2 = 0.0;
    for (int i = 0; i < m; ++i) {
      x[i] = a[(size_t)(k + 1 + i) * n + k];
      nrm2 += x[i] * x[i];
    }
    const double off2 = nrm2 - x[0] * x[0];
    if (off2 == 0.0) continue;  // already tridiagonal in this column
    double alpha = std::sqrt(nrm2);
    if (x[0] > 0) alpha = -alpha;  // x - alpha e1 without cancellation
    x[0] -= alpha;
    const double beta = 2.0 / (x[0] * x[0] + off2);
    // p = beta A_sub x, K = beta/2 p.x, q = p - K x, A_sub -= x q^T + q x^T
    double px = 0.0;
    for (int i = 0; i < m; ++i) {
      const double* row = &a[(size_t)(k + 1 + i) * n + k + 1];
      double s = 0.0;
      for (int j = 0; j < m; ++j) s += row[j] * x[j];
      p[i] = beta * s;
      px += p[i] * x[i];
    }
    const double K = 0.5 * beta * px;
    for (int i = 0; i < m; ++i) q[i] = p[i] - K * x[i];
    for (int i = 0; i < m; ++i) {
      double* row = &a[(size_t)(k + 1 + i) * n + k + 1];
      const double xi = x[i], qi = q[i];
      for (int j = 0; j < m; ++j) row[j] -= xi * q[j] + qi * x[j];
    }
    a[(size_t)(k + 1) * n + k] = a[(size_t)k * n + k + 1] = alpha;
    for (int i = 1; i < m; ++i) a[(size_t)(k + 1 + i) * n + k] = a[(size_t)k * n + k + 1 + i] = 0.0;
    // rows k+1.. of Z: Z_sub -= beta x (x^T Z_sub)
    for (int c = 0; c < n; ++c) t[c] = 0.0;
    for (int j = 0; j < m; ++j) {
      const double* row = &z[(size_t)(k + 1 + j) * n];
      const double xj = x[j];
      for (int c = 0; c < n; ++c) t[c] += xj * row[c];
    }
    for (int j = 0; j < m; ++j) {
      double* row = &z[(size_t)(k + 1 + j) * n];
      const double bx = beta * x[j];
      for (int c = 0; c < n; ++c) row[c] -= bx * t[c];
    }
  }
  for (int i = 0; i < n; ++i) w[i] = a[(size_t)i * n + i];
  for (int i = 0; i + 1 < n; ++i) e[i] = a[(size_t)(i + 1) * n + i];
  e[n - 1] = 0.0;
  // implicit QL on (w, e); each plane rotation mixes two rows of Z
  const double eps = std::numeric_limits<double>::epsilon();
  for (int l = 0; l < n; ++l) {
    for (int iter = 0; iter < 64; ++iter) {
      int m = l;
      for (; m + 1 < n; ++m)
        if (std::fabs(e[m]) <= eps * (std::fabs(w[m]) + std::fabs(w[m + 1]))) break;
      if (m == l) break;
      double g = (w[l + 1] - w[l]) / (2.0 * e[l]);
      double r = std::fabs(g) < 1e150 ? std::sqrt(g * g + 1.0) : std::fabs(g);
      g = w[m] - w[l] + e[l] / (g + (g >= 0 ? r : -r));
      double sn = 1.0, cs = 1.0, shift = 0.0;
      bool split = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = sn * e[i], b = cs * e[i];
        r = std::sqrt(f * f + g * g);
        e[i + 1] = r;
        if (r == 0.0) {  // the matrix splits at i: deflate and restart the sweep
          w[i + 1] -= shift;
          e[m] = 0.0;
          split = true;
          break;
        }
        sn = f / r;
        cs = g / r;
        g = w[i + 1] - shift;
        r = (w[i] - g) * sn + 2.0 * cs * b;
        shift = sn * r;
        w[i + 1] = g + shift;
        g = cs * r - b;
        double* zi = &z[(size_t)i * n];
        double* zj = &z[(size_t)(i + 1) * n];
        for (int c = 0; c < n; ++c) {
          const double u0 = zi[c], u1 = zj[c];
          zj[c] = sn * u0 + cs * u1;
          zi[c] = cs * u0 - sn * u1;
        }
      }
      if (split) continue;
      w[l] -= shift;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x1, int y1) { return w[x1] < w[y1]; });
  std::vector<double> w2(n);
  for (int j = 0; j < n; ++j) {
    w2[j] = w[ord[j]];
    const double* zr = &z[(size_t)ord[j] * n];
    for (int i = 0; i < n; ++i) v[(size_t)i * n + j] = zr[i];
  }
  w.swap(w2);
}

namespace {

constexpr int DBLK = 256;
constexpr int MAXM = 128;  // basis size N_st_diag * itermax
constexpr int MAXS = 8;    // N_st_diag

inline unsigned gsz(int64_t n, int tpb = DBLK) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (unsigned)g;
}

// hi + lo += x * y for split operands x = xh + xl, y = yh + yl: the product
// of the high parts exactly (rounded value plus its FMA error), the two cross
// terms (the lo * lo term is below 2^-46 of the product), and Knuth's TwoSum
// on the high part of the running sum
__device__ __forceinline__ void ff_mac(float& hi, float& lo, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  float pe = __fmaf_rn(xh, yh, -p);
  pe = __fmaf_rn(xh, yl, pe);
  pe = __fmaf_rn(xl, yh, pe);
  float s, e;
  qpsig::two_sum(hi, p, s, e);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(e, pe));
}

// moves what the low part has gathered into the high part (Dekker's
// Fast2Sum; |lo| <= |hi| up to the rounding of the accumulated errors)
__device__ __forceinline__ void ff_renorm(float& hi, float& lo) {
  const float s = __fadd_rn(hi, lo);
  lo = __fsub_rn(lo, __fsub_rn(s, hi));
  hi = s;
}

// G[i][j] = sum_r A_i[r] B_j[r]: A has m columns (column i is column i % nsd
// of the block i / nsd; blocks strideA apart, rows of nsd values), B is B0
// (nsd columns) or [B0 B1] (2 nsd columns), NBC = the number of B columns.
// GB300 issues two FP64 FMAs per clock per SM, so the kernel only has to keep
// the FP64 pipe fed: a lane owns one row at a time and CI = 32 / NBC columns
// of A, so a row costs CI + NBC loads for CI * NBC FMAs and every FMA is
// useful work (no padded columns).  A warp holds one column group; the eight
// warps of a CTA cover eight column groups, or split the rows when there are
// fewer groups, and gridDim.y passes cover the rest of the columns.  Lanes
// are combined by a reduce-scatter, warps of the same column group through
// shared memory in a fixed order, and one partial per CTA is written, so the
// sums are deterministic.  A non-null `skip` flag that is set makes the
// kernel return at once (the conditional second Gram-Schmidt pass).
template <int NBC>
__global__ void __launch_bounds__(DBLK) k_gram(const double* __restrict__ A, int m, int64_t strideA,
                                               const double* __restrict__ B0, const double* __restrict__ B1, int nsd,
                                               int64_t N, int64_t rows_per_cta, double* partial, const int* skip) {
  constexpr int CI = 32 / NBC;
  if (skip && *skip) return;
  __shared__ double red[DBLK / 32][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncg = (m + CI - 1) / CI;
  const int cg0 = blockIdx.y * (DBLK / 32);
  const int ncg_here = min(DBLK / 32, ncg - cg0);
  const int rg = (DBLK / 32) / ncg_here;  // row groups
  const int cgl = w % ncg_here, rgi = w / ncg_here;
  const bool active = rgi < rg;
  const int cg = cg0 + cgl;
  const int nq = min(CI, m - cg * CI);  // real columns of this group (warp uniform)
  const double* ap[CI];
#pragma unroll
  for (int q = 0; q < CI; ++q) {
    const int i = min(cg * CI + q, m - 1);
    ap[q] = A + (int64_t)(i / nsd) * strideA + (i % nsd);
  }
  double acc[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) acc[k] = 0.0;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(r0 + rows_per_cta, N);
  if (active) {
    for (int64_t r = r0 + (int64_t)rgi * 32 + lane; r < r1; r += (int64_t)rg * 32) {
      double a[CI], b[NBC];
#pragma unroll
      for (int q = 0; q < CI; ++q) a[q] = (q < nq) ? ap[q][r * nsd] : 0.0;
#pragma unroll
      for (int j = 0; j < NBC; ++j) b[j] = (j < nsd) ? B0[r * nsd + j] : B1[r * nsd + j - nsd];
#pragma unroll
      for (int q = 0; q < CI; ++q)
        if (q < nq)
#pragma unroll
          for (int j = 0; j < NBC; ++j) acc[q * NBC + j] = fma(a[q], b[j], acc[q * NBC + j]);
    }
  }
  // lane L ends with entry L = (q, j) = (L / NBC, L % NBC) of the group's tile
  const double v = qpsig::reduce_scatter64<32>(acc, lane);
  if (active) red[w][lane] = v;
  __syncthreads();
  if (w < ncg_here) {
    double t = 0.0;
    for (int g = 0; g < rg; ++g) t += red[g * ncg_here + w][lane];
    const int q = lane / NBC, j = lane % NBC, i = cg * CI + q;
    if (q < CI && i < m) partial[(int64_t)blockIdx.x * m * NBC + (int64_t)i * NBC + j] = t;
  }
}

// out[p] = sum over CTAs of partial[cta][p]: one warp per element, lane l
// adds CTAs l, l+32, ... and the lanes combine in a fixed butterfly order
__global__ void k_reduce_partials(const double* partial, int ncta, int np, double* out, const int* skip) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int p = blockIdx.x * wpb + (threadIdx.x >> 5); p < np; p += gridDim.x * wpb) {
    double s = 0.0;
    for (int c = lane; c < ncta; c += 32) s += partial[(int64_t)c * np + p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[p] = s;
  }
}

// Float-float copies of Davidson blocks for the mixed-precision Gram blocks:
// out[r][j] = split of X0[r][j] (j < nsd) or X1[r][j - nsd] (nx = 2), so a
// row of out holds nx * nsd (hi, lo) pairs.  Every operand of k_gram_ff is
// split once here instead of once per use.
__global__ void k_split_block(const double* __restrict__ X0, const double* __restrict__ X1, int nsd, int nx,
                              int64_t N, float2* __restrict__ out, const int* skip) {
  if (skip && *skip) return;
  // flat over the nsd * N elements of each source block (coalesced loads and
  // stores); the row of element i is i / nsd (32-bit when it fits)
  const int64_t n = N * nsd;
  const bool small = n < (1LL << 31);
  for (int t = 0; t < nx; ++t) {
    const double* x = t ? X1 : X0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      float h, l;
      qpsig::split_ff(x[i], h, l);
      int64_t o = i;
      if (nx > 1) {
        const int64_t r = small ? (int64_t)((unsigned)i / (unsigned)nsd) : i / nsd;
        o = r * (nx * nsd) + t * nsd + (i - r * nsd);
      }
      out[o] = make_float2(h, l);
    }
  }
}

// k_gram in float-float arithmetic on the FP32 pipes (GB300: 64 FP32 FMAs per
// FP64 FMA), for the mixed-precision Davidson's Gram-Schmidt passes and
// projections.  A = m split columns (consecutive split blocks of nsd, block
// stride sA), B = N rows of NBC split values (k_split_block).  The CTA tiling
// over rows and column groups is k_gram's, but each lane owns one entry
// (q, j) = (lane / NBC, lane % NBC) of its warp's CI x NBC tile and runs over
// the rows: tiles of T rows of the CTA's A blocks and of B are staged in
// shared memory by cp.async (double-buffered), and a lane reads one A and one
// B value per row as conflict-free broadcasts.  Each product is ff_mac (about
// 47 bits), the pairs are renormalised every 16 rows, warps of a column group
// and CTAs are combined in FP64 in a fixed order (deterministic sums).
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

struct GramTile {
  int k_lo, nblk;
};
// the split blocks that hold the columns [cg0 * ci, min(m, (cg0 + ncg_here) * ci))
// of gridDim.y slice cgy
__host__ __device__ inline GramTile gram_tile(int m, int nsd, int nbc, int cgy) {
  const int ci = 32 / nbc;
  const int ncg = (m + ci - 1) / ci;
  const int cg0 = cgy * (DBLK / 32);
  const int ncg_here = ncg - cg0 < DBLK / 32 ? ncg - cg0 : DBLK / 32;
  const int c_lo = cg0 * ci, c_hi = m < (cg0 + ncg_here) * ci ? m : (cg0 + ncg_here) * ci;
  GramTile g;
  g.k_lo = c_lo / nsd;
  g.nblk = (c_hi - 1) / nsd - g.k_lo + 1;
  return g;
}
// widest staged row (float2) over the gridDim.y slices, and the row-tile
// height T: two stages in about 72 KB, so three CTAs share an SM
inline int gram_stage_width(int m, int nsd, int nbc) {
  const int ci = 32 / nbc;
  const int ny = ((m + ci - 1) / ci + DBLK / 32 - 1) / (DBLK / 32);
  int w = 0;
  for (int y = 0; y < ny; ++y) w = std::max(w, gram_tile(m, nsd, nbc, y).nblk * nsd + nbc);
  return w;
}
inline int gram_rows_per_stage(int width) {
  const int T = (72 * 1024 / (2 * (int)sizeof(float2) * width)) / 32 * 32;
  return std::max(32, std::min(T, 256));
}

template <int NBC, int NSD>
__global__ void __launch_bounds__(DBLK) k_gram_ff(const float2* __restrict__ A, int m, int64_t sA,
                                                  const float2* __restrict__ B, int64_t N, int64_t rows_per_cta,
                                                  int T, double* partial, const int* skip) {
  constexpr int CI = 32 / NBC;
  if (skip && *skip) return;
  extern __shared__ float2 stage[];
  __shared__ double red[DBLK / 32][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncg = (m + CI - 1) / CI;
  const int cg0 = blockIdx.y * (DBLK / 32);
  const int ncg_here = min(DBLK / 32, ncg - cg0);
  const int rg = (DBLK / 32) / ncg_here;
  const int cgl = w % ncg_here, rgi = w / ncg_here;
  const bool active = rgi < rg;
  const GramTile gt = gram_tile(m, NSD, NBC, blockIdx.y);
  const int wA = gt.nblk * NSD;                 // A float2 per staged row
  const int64_t ssz = (int64_t)T * (wA + NBC);  // float2 per stage
  // this lane's entry
  const int q = lane / NBC, j = lane % NBC;
  const int col = (cg0 + cgl) * CI + q;
  const bool mine = active && q < CI && col < m;
  const int cc = mine ? col : gt.k_lo * NSD;
  const int aoff = (cc / NSD - gt.k_lo) * T * NSD + (cc % NSD);  // within the A part of a stage
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(r0 + rows_per_cta, N);
  auto issue = [&](int64_t r, float2* buf) {
    const int nr = (int)min((int64_t)T, r1 - r);
    for (int kb = 0; kb < gt.nblk; ++kb) {
      const float2* src = A + (int64_t)(gt.k_lo + kb) * sA + r * NSD;
      float2* dst = buf + kb * T * NSD;
      for (int e = threadIdx.x; e < nr * NSD; e += DBLK) cp_async8(dst + e, src + e);
    }
    const float2* src = B + r * NBC;
    float2* dst = buf + T * wA;
    for (int e = threadIdx.x; e < nr * NBC; e += DBLK) cp_async8(dst + e, src + e);
  };
  // a warp takes a contiguous share of each staged tile; two accumulator
  // pairs (alternate rows) give its in-order issue two independent TwoSum
  // chains, and strides are compile-time constants
  float hi = 0.f, lo = 0.f, hi2 = 0.f, lo2 = 0.f;
  if (r0 < r1) issue(r0, stage);
  cp_async_commit();
  int t = 0;
  for (int64_t r = r0; r < r1; r += T, ++t) {
    float2* cur = stage + (t & 1) * ssz;
    if (r + T < r1) issue(r + T, stage + ((t + 1) & 1) * ssz);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    if (mine) {
      const int nr = (int)min((int64_t)T, r1 - r);
      const int share = (nr + rg - 1) / rg;
      const int rb = rgi * share, re = min(nr, rb + share);
      const float2* ap = cur + aoff + rb * NSD;
      const float2* bp = cur + T * wA + j + rb * NBC;
      int rr = rb;
      for (; rr + 16 <= re; rr += 16, ap += 16 * NSD, bp += 16 * NBC) {
#pragma unroll
        for (int k = 0; k < 16; k += 2) {
          const float2 a0 = ap[k * NSD], a1 = ap[(k + 1) * NSD];
          const float2 b0 = bp[k * NBC], b1 = bp[(k + 1) * NBC];
          ff_mac(hi, lo, a0.x, a0.y, b0.x, b0.y);
          ff_mac(hi2, lo2, a1.x, a1.y, b1.x, b1.y);
        }
        ff_renorm(hi, lo);
        ff_renorm(hi2, lo2);
      }
      for (; rr < re; ++rr, ap += NSD, bp += NBC) {
        const float2 a0 = ap[0], b0 = bp[0];
        ff_mac(hi, lo, a0.x, a0.y, b0.x, b0.y);
      }
      ff_renorm(hi, lo);
    }
    __syncthreads();
  }
  if (active) red[w][lane] = ((double)hi + (double)lo) + ((double)hi2 + (double)lo2);
  __syncthreads();
  if (w < ncg_here) {
    double v = 0.0;
    for (int g = 0; g < rg; ++g) v += red[g * ncg_here + w][lane];
    const int i = (cg0 + w) * CI + q;
    if (q < CI && i < m) partial[(int64_t)blockIdx.x * m * NBC + (int64_t)i * NBC + j] = v;
  }
}

// out_t[r][0:nsd] = sum_i A_t[column i][r] C[i][0:nsd] for up to 3 (A, out)
// pairs sharing C (m x nsd, row-major; the m columns are nb consecutive blocks
// of nsd).  A lane owns one row: per block it loads the row's NSD values
// (contiguous; 16-byte loads for even NSD, so a warp reads one contiguous
// span) and does NSD x NSD FMAs against C broadcast from shared memory; the
// next block's values are loaded before the current ones are used.  The sum
// runs over (block, column) in order, so results are deterministic.  out may
// alias a block of A (a lane reads all of its row before writing it).
struct LinComb {
  const double* A[3];
  double* out[3];
  int n;
};
template <int NSD>
__device__ __forceinline__ void load_row(const double* __restrict__ p, double (&x)[NSD]) {
  if constexpr (NSD % 2 == 0) {
#pragma unroll
    for (int c = 0; c < NSD / 2; ++c) {
      const double2 v = reinterpret_cast<const double2*>(p)[c];
      x[2 * c] = v.x;
      x[2 * c + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int c = 0; c < NSD; ++c) x[c] = p[c];
  }
}
template <int NSD>
__global__ void __launch_bounds__(DBLK) k_lincomb(LinComb L, int nb, int64_t N, const double* C, const int* skip) {
  if (skip && *skip) return;
  __shared__ __align__(16) double Cs[MAXM * MAXS];
  for (int i = threadIdx.x; i < nb * NSD * NSD; i += DBLK) Cs[i] = C[i];
  __syncthreads();
  const int64_t sA = N * NSD;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    for (int t = 0; t < L.n; ++t) {
      const double* a = L.A[t] + r * NSD;
      double acc[NSD], x[NSD], xn[NSD];
#pragma unroll
      for (int j = 0; j < NSD; ++j) acc[j] = 0.0;
      load_row<NSD>(a, x);
      for (int b = 0; b < nb; ++b) {
        if (b + 1 < nb) load_row<NSD>(a + (int64_t)(b + 1) * sA, xn);
        const double* cb = Cs + b * NSD * NSD;
#pragma unroll
        for (int c = 0; c < NSD; ++c)
#pragma unroll
          for (int j = 0; j < NSD; ++j) acc[j] = fma(x[c], cb[c * NSD + j], acc[j]);
#pragma unroll
        for (int c = 0; c < NSD; ++c) x[c] = xn[c];
      }
      double* o = L.out[t] + r * NSD;
      if constexpr (NSD % 2 == 0) {
#pragma unroll
        for (int c = 0; c < NSD / 2; ++c) reinterpret_cast<double2*>(o)[c] = make_double2(acc[2 * c], acc[2 * c + 1]);
      } else {
#pragma unroll
        for (int j = 0; j < NSD; ++j) o[j] = acc[j];
      }
    }
  }
}

// k_lincomb in float-float arithmetic on the FP32 pipes (GB300 issues 64
// FP32 FMAs for each FP64 FMA): each product of split operands is formed
// exactly for hi*hi (an FMA gives its rounding error) plus the hi*lo cross
// terms, and the running sum is kept as an unevaluated pair with Knuth's
// TwoSum on the high part.  About 47-bit accuracy; used by the
// mixed-precision Davidson for the Gram-Schmidt / Cholesky-QR updates, the
// Ritz vectors of restart iterations and the re-contraction.  Same row
// ownership, loads and summation order as k_lincomb.
template <int NSD>
__global__ void __launch_bounds__(DBLK) k_lincomb_ff(LinComb L, int nb, int64_t N, const double* C, const int* skip) {
  if (skip && *skip) return;
  __shared__ float2 Cs[MAXM * MAXS];
  for (int i = threadIdx.x; i < nb * NSD * NSD; i += DBLK) {
    float h, l;
    qpsig::split_ff(C[i], h, l);
    Cs[i] = make_float2(h, l);
  }
  __syncthreads();
  const int64_t sA = N * NSD;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    for (int t = 0; t < L.n; ++t) {
      const double* a = L.A[t] + r * NSD;
      float ah[NSD], al[NSD];
      double x[NSD], xn[NSD];
#pragma unroll
      for (int j = 0; j < NSD; ++j) ah[j] = al[j] = 0.f;
      load_row<NSD>(a, x);
      for (int b = 0; b < nb; ++b) {
        if (b + 1 < nb) load_row<NSD>(a + (int64_t)(b + 1) * sA, xn);
        const float2* cb = Cs + b * NSD * NSD;
#pragma unroll
        for (int c = 0; c < NSD; ++c) {
          float xh, xl;
          qpsig::split_ff(x[c], xh, xl);
#pragma unroll
          for (int j = 0; j < NSD; ++j) {
            const float2 cv = cb[c * NSD + j];
            ff_mac(ah[j], al[j], xh, xl, cv.x, cv.y);
          }
        }
#pragma unroll
        for (int c = 0; c < NSD; ++c) x[c] = xn[c];
      }
      double* o = L.out[t] + r * NSD;
#pragma unroll
      for (int j = 0; j < NSD; ++j) o[j] = (double)ah[j] + (double)al[j];
    }
  }
}

// FP64 -> FP32 by truncation and FP32 -> FP64 exactly, with integer
// instructions (GB300's conversions between the two formats issue at the
// FP64 rate).  |x| below 2^-126 gives 0; beyond the float range, or Inf or
// NaN, gives a signed Inf (so a diverging step still reads as non-finite).
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const unsigned sign = h32 & 0x80000000u;
  const int fe = (int)((h32 >> 20) & 0x7ffu) - 896;
  if (fe <= 0) return __uint_as_float(sign);
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned)fe << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
}
__device__ __forceinline__ double f64_from(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 255) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// k_lincomb in FP32 arithmetic (inputs truncated to FP32, outputs widened
// exactly): the Ritz vectors U y, W y, S y of the mixed-precision Davidson on
// the iterations whose W and S come from the FP32 sigma, where they only
// feed the step; restart iterations and the re-contraction use k_lincomb_ff.
template <int NSD>
__global__ void __launch_bounds__(DBLK) k_lincomb32(LinComb L, int nb, int64_t N, const double* C) {
  __shared__ float Cs[MAXM * MAXS];
  for (int i = threadIdx.x; i < nb * NSD * NSD; i += DBLK) Cs[i] = f32_trunc(C[i]);
  __syncthreads();
  const int64_t sA = N * NSD;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    for (int t = 0; t < L.n; ++t) {
      const double* a = L.A[t] + r * NSD;
      float acc[NSD];
      double x[NSD], xn[NSD];
#pragma unroll
      for (int j = 0; j < NSD; ++j) acc[j] = 0.f;
      load_row<NSD>(a, x);
      for (int b = 0; b < nb; ++b) {
        if (b + 1 < nb) load_row<NSD>(a + (int64_t)(b + 1) * sA, xn);
        const float* cb = Cs + b * NSD * NSD;
#pragma unroll
        for (int c = 0; c < NSD; ++c) {
          const float xc = f32_trunc(x[c]);
#pragma unroll
          for (int j = 0; j < NSD; ++j) acc[j] = fmaf(xc, cb[c * NSD + j], acc[j]);
        }
#pragma unroll
        for (int c = 0; c < NSD; ++c) x[c] = xn[c];
      }
      double* o = L.out[t] + r * NSD;
#pragma unroll
      for (int j = 0; j < NSD; ++j) o[j] = f64_from(acc[j]);
    }
  }
}

// Cholesky G = R^T R (n x n, n <= MAXS, in shared memory) and Ri = R^-1
// (upper triangular), by one warp: row j of R is formed by lanes i >= j
// after its pivot, and lane j back-substitutes column j of R^-1.  Every sum
// runs in the order of the one-thread algorithm (k ascending), so the result
// does not depend on the lane layout.  A vanishing pivot (a dependent
// column) gives a zero row of R and a zero column of Ri.
__device__ void chol_inv_warp(const double (*G)[MAXS], double (*R)[MAXS], double (*Ri)[MAXS], int n, int lane) {
  for (int j = 0; j < n; ++j) {
    double dj = G[j][j];
    for (int k = 0; k < j; ++k) dj -= R[k][j] * R[k][j];
    const bool ok = (dj > 1e-28 * fabs(G[j][j])) && (dj > 1e-300);
    const double rjj = ok ? sqrt(dj) : 0.0;
    if (lane < n) {
      double v = 0.0;
      if (lane == j) {
        v = rjj;
      } else if (lane > j && ok) {
        double t = G[j][lane];
        for (int k = 0; k < j; ++k) t -= R[k][j] * R[k][lane];
        v = t / rjj;
      }
      R[j][lane] = v;
    }
    __syncwarp();
  }
  if (lane < n) {
    const int j = lane;
    for (int i = 0; i < n; ++i) Ri[i][j] = 0.0;
    if (R[j][j] != 0.0) {
      Ri[j][j] = 1.0 / R[j][j];
      for (int i = j - 1; i >= 0; --i) {
        if (R[i][i] == 0.0) continue;
        double t = 0.0;
        for (int k = i + 1; k <= j; ++k) t += R[i][k] * Ri[k][j];
        Ri[i][j] = -t / R[i][i];
      }
    }
  }
  __syncwarp();
}

// Rinv = R^-1 for the Cholesky factor of G (nsd x nsd, row-major), one warp
__global__ void k_chol_inv(const double* G, int nsd, double* Rinv) {
  __shared__ double Gs[MAXS][MAXS], R[MAXS][MAXS], Ri[MAXS][MAXS];
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  for (int idx = lane; idx < nsd * nsd; idx += 32) Gs[idx / nsd][idx % nsd] = G[idx];
  __syncwarp();
  chol_inv_warp(Gs, R, Ri, nsd, lane);
  for (int idx = lane; idx < nsd * nsd; idx += 32) Rinv[idx] = Ri[idx / nsd][idx % nsd];
}

// Coefficients of the fused classical Gram-Schmidt + Cholesky-QR update of a
// new block U_b (nsd columns) against the m orthonormal columns before it.
// X = [U_0 .. U_b]^T U_b ((m + nsd) x nsd): C = X[0:m], G0 = X[m:m+nsd].
// G1 = G0 - C^T C is the Gram matrix of U_b - U C.  When every column kept
// more than half of its norm (G1_jj > G0_jj / 4, so G1 carries no
// cancellation) the update is fused with the Cholesky factor G1 = R^T R:
// K = [-C R^-1; R^-1], and U_b <- [U_0 .. U_b] K orthogonalises and
// normalises in one pass.  Otherwise K = [-C; I] (plain Gram-Schmidt) and
// *skip2 = 0 asks for a second pass (mode 1), which always fuses.  Mode 1
// returns at once when *skip2 is set.  A vanishing Cholesky pivot (a
// dependent column) gives a zero column, as in k_chol_inv.
__global__ void k_cgs_coef(const double* X, int m, int nsd, double* K, int* skip2, int mode) {
  if (mode == 1 && *skip2) return;
  __shared__ double G[MAXS][MAXS], R[MAXS][MAXS], Ri[MAXS][MAXS];
  __shared__ int need;
  for (int idx = threadIdx.x; idx < nsd * nsd; idx += blockDim.x) {
    const int i = idx / nsd, j = idx % nsd;
    double g = X[(m + i) * nsd + j];
    for (int k = 0; k < m; ++k) g -= X[k * nsd + i] * X[k * nsd + j];
    G[i][j] = g;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nd = 0;
    if (mode == 0)
      for (int j = 0; j < nsd; ++j)
        if (!(G[j][j] > 0.25 * X[(m + j) * nsd + j])) nd = 1;
    need = nd;
    if (mode == 0) *skip2 = nd ? 0 : 1;
  }
  __syncthreads();
  if (!need && threadIdx.x < 32) chol_inv_warp(G, R, Ri, nsd, threadIdx.x);
  __syncthreads();
  const bool fuse = !need;
  for (int idx = threadIdx.x; idx < (m + nsd) * nsd; idx += blockDim.x) {
    const int i = idx / nsd, j = idx % nsd;
    double v;
    if (i < m) {
      if (fuse) {
        v = 0.0;
        for (int k = 0; k <= j; ++k) v -= X[i * nsd + k] * Ri[k][j];
      } else {
        v = -X[i * nsd + j];
      }
    } else {
      v = fuse ? Ri[i - m][j] : (i - m == j ? 1.0 : 0.0);
    }
    K[idx] = v;
  }
}

struct StepParams {
  double lambda[MAXS];
  double s2[MAXS];
  double sz2sz;
  int nsd, nst;
};

// Davidson step (diagonalization_hs2.irp.f:386-391), in place on the Ritz
// block, and per-CTA partial sums of its squared norms (:395)
__global__ void __launch_bounds__(DBLK) k_step(double* Un, const double* Wn, const double* Sn, const double* hjj,
                                               int64_t N, StepParams p, double* partial) {
  __shared__ double red[MAXS][DBLK / 32];
  double acc[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; ++k) acc[k] = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    const double h = hjj[r];
    for (int k = 0; k < p.nsd; ++k) {
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const double v = (p.lambda[k] * u - Wn[x]) * (1.0 + p.s2[k] * u - Sn[x] - p.sz2sz) /
                       fmax(h - p.lambda[k], 1e-2);
      Un[x] = v;
      if (k < p.nst) acc[k] = fma(v, v, acc[k]);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MAXS; ++k) {
    double s = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < MAXS) {
    double s = 0.0;
    for (int i = 0; i < DBLK / 32; ++i) s += red[threadIdx.x][i];
    partial[(int64_t)blockIdx.x * MAXS + threadIdx.x] = s;
  }
}

// The Davidson step of k_step for the mixed-precision loop: the residual
// numerator lambda u - W is formed by one FP64 FMA (it cancels near
// convergence), then the S^2 factor, the diagonal preconditioner and the
// squared norms run in FP32 -- the accuracy of the FP32 sigma that feeds
// most of these iterations; the step is a search direction and its norm the
// convergence measure, both needed to a few digits.
__global__ void __launch_bounds__(DBLK) k_step_mixed(double* Un, const double* Wn, const double* Sn, const double* hjj,
                                                     int64_t N, StepParams p, double* partial) {
  __shared__ double red[MAXS][DBLK / 32];
  float acc[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; ++k) acc[k] = 0.f;
  const float sz2sz = (float)p.sz2sz;
  float s2f[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; ++k) s2f[k] = (float)p.s2[k];
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    const double h = hjj[r];
#pragma unroll
    for (int k = 0; k < MAXS; ++k) {
      if (k >= p.nsd) break;
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const float num = f32_trunc(fma(p.lambda[k], u, -Wn[x]));
      const float fac = 1.0f + s2f[k] * f32_trunc(u) - f32_trunc(Sn[x]) - sz2sz;
      const float den = fmaxf(f32_trunc(h - p.lambda[k]), 1e-2f);
      const float v = __fdiv_rn(num * fac, den);
      Un[x] = f64_from(v);
      if (k < p.nst) acc[k] = fmaf(v, v, acc[k]);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MAXS; ++k) {
    double s = (double)acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < MAXS) {
    double s = 0.0;
    for (int i = 0; i < DBLK / 32; ++i) s += red[threadIdx.x][i];
    partial[(int64_t)blockIdx.x * MAXS + threadIdx.x] = s;
  }
}

// Features of the target states for the learned step (qp_features), one row
// of QP_MLP_IN floats per (determinant, state); the network is evaluated on
// them by qp_mlp_eval (a spill-free inference kernel) before k_step_mlp.
__global__ void __launch_bounds__(DBLK) k_mlp_features(const double* Un, const double* Wn, const double* Sn,
                                                        const double* hjj, const float4* feat, int64_t N, StepParams p,
                                                        float* X) {
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    const double h = hjj[r];
    const float4 st = feat[r];
    for (int k = 0; k < p.nst; ++k) {
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const double res = p.lambda[k] * u - Wn[x];
      const double d = res * (1.0 + p.s2[k] * u - Sn[x] - p.sz2sz) / fmax(h - p.lambda[k], 1e-2);
      float f[QP_MLP_IN];
      qp_features(st, h - p.lambda[k], u, res, d, f);
      float* o = X + (r * p.nst + k) * QP_MLP_IN;
#pragma unroll
      for (int i = 0; i < QP_MLP_IN; ++i) o[i] = f[i];
    }
  }
}

// Davidson step with the learned preconditioner.  d_k is the reference's
// diagonal correction of Ritz vector k (its squared norm stays the
// convergence measure); g_k = G[r * nst + k] the MLP's per-determinant
// multiplier.
//   replace (extra == 0): state k flagged in mlp_mask takes g_k d_k instead
//     of d_k;
//   extra (extra == 1): the correction slot of the non-target Ritz vector
//     nst + k takes g_k d_k, so the subspace receives both d_k and g_k d_k
//     for a flagged target state k and the Rayleigh-Ritz step weighs them: a
//     poor network costs a little of the block's extra directions instead of
//     the target's own step.
__global__ void __launch_bounds__(DBLK) k_step_mlp(double* Un, const double* Wn, const double* Sn, const double* hjj,
                                                   const float* G, int64_t N, StepParams p, unsigned mlp_mask,
                                                   int extra, double* partial) {
  __shared__ double red[MAXS][DBLK / 32];
  double acc[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; ++k) acc[k] = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    const double h = hjj[r];
    double learned[MAXS];  // g_k d_k of the flagged target states (extra mode)
#pragma unroll
    for (int k = 0; k < MAXS; ++k) {
      learned[k] = 0.0;
      if (k >= p.nsd) continue;
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const double res = p.lambda[k] * u - Wn[x];
      const double d = res * (1.0 + p.s2[k] * u - Sn[x] - p.sz2sz) / fmax(h - p.lambda[k], 1e-2);
      double v = d;
      if (k < p.nst && ((mlp_mask >> k) & 1u)) {
        const double gd = d * (double)G[r * p.nst + k];
        if (extra)
          learned[k] = gd;
        else
          v = gd;
      }
      if (extra && k >= p.nst && ((mlp_mask >> (k - p.nst)) & 1u)) {
#pragma unroll
        for (int q = 0; q < MAXS; ++q)
          if (q == k - p.nst) v = learned[q];
      }
      Un[x] = v;
      if (k < p.nst) acc[k] = fma(d, d, acc[k]);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MAXS; ++k) {
    double s = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < MAXS) {
    double s = 0.0;
    for (int i = 0; i < DBLK / 32; ++i) s += red[threadIdx.x][i];
    partial[(int64_t)blockIdx.x * MAXS + threadIdx.x] = s;
  }
}

// training capture: features, diagonal correction d and Ritz vector c of the
// states k < nst, before the step overwrites the Ritz block
__global__ void k_capture(const double* Un, const double* Wn, const double* Sn, const double* hjj, const float4* feat,
                          int64_t N, StepParams p, int slot0, float* cX, float* cd, float* cc) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
    const double h = hjj[r];
    const float4 st = feat[r];
    for (int k = 0; k < p.nst; ++k) {
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const double res = p.lambda[k] * u - Wn[x];
      const double d = res * (1.0 + p.s2[k] * u - Sn[x] - p.sz2sz) / fmax(h - p.lambda[k], 1e-2);
      const int64_t slot = slot0 + k;
      float f[QP_MLP_IN];
      qp_features(st, h - p.lambda[k], u, res, d, f);
      for (int i = 0; i < QP_MLP_IN; ++i) cX[(slot * N + r) * QP_MLP_IN + i] = f[i];
      cd[slot * N + r] = (float)d;
      cc[slot * N + r] = (float)u;
    }
  }
}

// per-CTA sums over rows for each captured slot (state k = slot % nst of the
// final vectors cf, block 0): mode 0: (cf.c, d.d); mode 1 with dot: (e.e, e.d),
// e = cf - dot c
__global__ void k_capture_sums(const double* cf, int nsd, int nst, const float* cd, const float* cc, int nslot,
                               int64_t N, const double* dot, int mode, double* partial) {
  __shared__ double red[2][DBLK];
  for (int s = 0; s < nslot; ++s) {
    const int k = s % nst;
    double a = 0.0, b = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
      const double c = cc[(int64_t)s * N + r], d = cd[(int64_t)s * N + r], f = cf[r * nsd + k];
      if (mode == 0) {
        a = fma(f, c, a);
        b = fma(d, d, b);
      } else {
        const double e = f - dot[s] * c;
        a = fma(e, e, a);
        b = fma(e, d, b);
      }
    }
    red[0][threadIdx.x] = a;
    red[1][threadIdx.x] = b;
    __syncthreads();
    for (int o = DBLK / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) {
        red[0][threadIdx.x] += red[0][threadIdx.x + o];
        red[1][threadIdx.x] += red[1][threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      partial[((int64_t)blockIdx.x * nslot + s) * 2] = red[0][0];
      partial[((int64_t)blockIdx.x * nslot + s) * 2 + 1] = red[1][0];
    }
    __syncthreads();
  }
}

struct SlotScale {
  double dot, inv_ne, inv_nd, sign;
};

// training samples from the captured slots: target g = (e/|e|)/(d/|d|) aligned
// with d and clipped to [-4, 4], weight N (d/|d|)^2; every `stride`-th row
__global__ void k_capture_samples(const double* cf, int nsd, int nst, const float* cX, const float* cd, const float* cc,
                                  int nslot, int64_t N, const SlotScale* sc, int64_t stride, int64_t per_slot, float* X,
                                  float* G, float* W) {
  const int64_t total = (int64_t)nslot * per_slot;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / per_slot);
    const int64_t r = (t % per_slot) * stride;
    const int k = s % nst;
    const SlotScale q = sc[s];
    const double c = cc[(int64_t)s * N + r], d = cd[(int64_t)s * N + r];
    const double e = cf[r * nsd + k] - q.dot * c;
    const double dn = d * q.inv_nd, en = q.sign * e * q.inv_ne;
    double g = 1.0, w = 0.0;
    if (fabs(dn) > 1e-12) {
      g = fmin(4.0, fmax(-4.0, en / dn));
      w = (double)N * dn * dn;
    }
    for (int i = 0; i < QP_MLP_IN; ++i) X[t * QP_MLP_IN + i] = cX[((int64_t)s * N + r) * QP_MLP_IN + i];
    G[t] = (float)g;
    W[t] = (float)w;
  }
}

__global__ void k_copy(const double* a, double* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

struct Dav {
  qpgpu_ctx* c;
  cudaStream_t st;
  int64_t N;
  int nsd, nst, itermax;
  double *U = nullptr, *W = nullptr, *S = nullptr, *R = nullptr;  // itermax blocks; R: one block
  float* u32 = nullptr;
  double* part = nullptr;  // gram / step partials
  double* small = nullptr;  // device small matrices (MAXM*MAXS x 6)
  float *cX = nullptr, *cd = nullptr, *cc = nullptr;  // training capture
  float *mlpX = nullptr, *mlpG = nullptr;              // learned step: features, multipliers
  float2 *Uf = nullptr, *Bf = nullptr;  // mixed precision: split U blocks, split [W_b S_b]
  int64_t sUf = 0;                       // block stride of Uf (float2)
  int ncta = 0;
  int64_t rows_per_cta = 0;
  // tensor-core Gram blocks (QPGPU_ALGEBRA_TC): biased max exponents of the
  // columns of the finished U blocks, of the current B operand, and the
  // status flag of the bounded tensor-core waits
  bool tc = false;
  int* uexp = nullptr;  // [MAXM]
  int* bexp = nullptr;  // [2 MAXS + 1]: B exponents, then the status flag
  ~Dav() {
    dev_free(U);
    dev_free(W);
    dev_free(S);
    dev_free(R);
    dev_free(u32);
    dev_free(part);
    dev_free(small);
    dev_free(cX);
    dev_free(cd);
    dev_free(cc);
    dev_free(mlpX);
    dev_free(mlpG);
    dev_free(Uf);
    dev_free(Bf);
    dev_free(uexp);
    dev_free(bexp);
  }
  double* blk(double* X, int b) const { return X + (int64_t)b * N * nsd; }
};

// device small-matrix area (doubles)
constexpr int OFF_X = 0;                     // Gram outputs, up to MAXM x 2 MAXS
constexpr int OFF_K = 2 * MAXM * MAXS;       // update coefficients, MAXM x MAXS
constexpr int OFF_Y = 3 * MAXM * MAXS;       // Ritz coefficients y, MAXM x MAXS
constexpr int OFF_G = 4 * MAXM * MAXS;       // nsd x nsd Gram block
constexpr int OFF_RINV = OFF_G + MAXS * MAXS;
constexpr int OFF_FLAG = OFF_RINV + MAXS * MAXS;
constexpr int SMALL_DOUBLES = OFF_FLAG + 8;

// out (m x nbc) = A^T [B0 (B1)] with A = m columns of consecutive blocks
int gram(Dav& d, const double* A, int m, const double* B0, const double* B1, double* out, const int* skip = nullptr) {
  const int nbc = d.nsd * (B1 ? 2 : 1);
  const int ci = 32 / nbc;
  const int ncg = (m + ci - 1) / ci;
  const dim3 grid(d.ncta, (ncg + DBLK / 32 - 1) / (DBLK / 32));
  const int64_t sA = d.N * d.nsd;
#define QP_GRAM_CASE(NB)                                                                      \
  case NB:                                                                                    \
    k_gram<NB><<<grid, DBLK, 0, d.st>>>(A, m, sA, B0, B1, d.nsd, d.N, d.rows_per_cta, d.part, skip); \
    break;
  switch (nbc) {
    QP_GRAM_CASE(1)
    QP_GRAM_CASE(2)
    QP_GRAM_CASE(3)
    QP_GRAM_CASE(4)
    QP_GRAM_CASE(5)
    QP_GRAM_CASE(6)
    QP_GRAM_CASE(7)
    QP_GRAM_CASE(8)
    QP_GRAM_CASE(10)
    QP_GRAM_CASE(12)
    QP_GRAM_CASE(14)
    QP_GRAM_CASE(16)
    default:
      return -1;
  }
#undef QP_GRAM_CASE
  k_reduce_partials<<<gsz((int64_t)m * nbc * 32), DBLK, 0, d.st>>>(d.part, d.ncta, m * nbc, out, skip);
  return 0;
}

// out (m x nbc) = A^T [B0 (B1)] on the tensor cores (FP64-accurate Ozaki
// splitting, ozaki.cu).  The exponents of B0 / B1 are computed here; those
// of A are, by `amode`: TC_BASIS, the cached ones of finished U blocks
// (d.uexp); TC_BASIS_NEW, the same with B0 as A's last block (Gram-Schmidt
// of the new block against the basis that holds it); TC_SELF, A = B0.
enum { TC_BASIS, TC_BASIS_NEW, TC_SELF };
void gram_tc(Dav& d, const double* A, int m, const double* B0, const double* B1, double* out, int amode,
             const int* skip = nullptr) {
  const int nbc = d.nsd * (B1 ? 2 : 1);
  int* eB = d.bexp;
  cudaMemsetAsync(eB, 0, nbc * sizeof(int), d.st);
  qp_col_maxexp(B0, 1, 0, d.nsd, d.nsd, d.N, eB, 0, skip, d.st, d.c->n_sm);
  if (B1) qp_col_maxexp(B1, 1, 0, d.nsd, d.nsd, d.N, eB, d.nsd, skip, d.st, d.c->n_sm);
  const int* eA = amode == TC_SELF ? eB : d.uexp;
  if (amode == TC_BASIS_NEW)
    cudaMemcpyAsync(d.uexp + (m - d.nsd), eB, d.nsd * sizeof(int), cudaMemcpyDeviceToDevice, d.st);
  qp_gram_oz(A, d.N * d.nsd, m, d.nsd, d.nsd, B0, B1, nbc, d.nsd, d.nsd, d.N, eA, eB, d.part, d.c->n_sm, skip,
             d.bexp + 2 * MAXS, d.st);
  qp_oz_reduce(d.part, d.c->n_sm, m * nbc, out, skip, d.st);
}

// lincomb on the tensor cores (FP64-accurate Ozaki splitting, ozaki.cu), one
// (A, out) pair after the other; shapes outside the kernel's range (m > 128)
// take the FP64 pipe
void lincomb(Dav& d, int m, const double* C, const double* A0, double* O0, const double* A1, double* O1,
             const double* A2, double* O2, const int* skip);
void lincomb_tc(Dav& d, int m, const double* C, const double* A0, double* O0, const double* A1 = nullptr,
                double* O1 = nullptr, const double* A2 = nullptr, double* O2 = nullptr, const int* skip = nullptr) {
  const double* A[3] = {A0, A1, A2};
  double* O[3] = {O0, O1, O2};
  for (int t = 0; t < 3 && A[t]; ++t)
    if (qp_lincomb_oz(A[t], d.N * d.nsd, m, d.nsd, C, O[t], d.nsd, d.N, d.c->n_sm, skip, d.bexp + 2 * MAXS, d.st))
      lincomb(d, m, C, A[t], O[t], nullptr, nullptr, nullptr, nullptr, skip);
}

// float-float copy of one block (X1 = nullptr) or of [X0 X1]
void split_block(Dav& d, const double* X0, const double* X1, float2* out, const int* skip = nullptr) {
  const int nx = X1 ? 2 : 1;
  k_split_block<<<std::min<unsigned>(gsz(d.N * d.nsd), d.c->n_sm * 8), DBLK, 0, d.st>>>(X0, X1, d.nsd, nx, d.N, out, skip);
}

// out (m x nbc) = A^T B on split operands: A = m columns of consecutive split
// blocks, B = rows of nbc split values
int gram_ff(Dav& d, const float2* A, int m, const float2* B, int nbc, double* out, const int* skip = nullptr) {
  const int ci = 32 / nbc;
  const int ncg = (m + ci - 1) / ci;
  const dim3 grid(d.ncta, (ncg + DBLK / 32 - 1) / (DBLK / 32));
  const int width = gram_stage_width(m, d.nsd, nbc);
  const int T = gram_rows_per_stage(width);
  const size_t smem = (size_t)2 * T * width * sizeof(float2);
  const bool two = nbc == 2 * d.nsd;
  if (!two && nbc != d.nsd) return -1;
  // opted in at every launch (the attribute belongs to the current device),
  // and for every size: the 48 KB default counts the static red[] too
#define QP_GRAMF_LAUNCH(NB, NS)                                                                        \
  cudaFuncSetAttribute(k_gram_ff<NB, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
  cudaFuncSetAttribute(k_gram_ff<NB, NS>, cudaFuncAttributePreferredSharedMemoryCarveout,              \
                       cudaSharedmemCarveoutMaxShared);                                                \
  k_gram_ff<NB, NS><<<grid, DBLK, smem, d.st>>>(A, m, d.sUf, B, d.N, d.rows_per_cta, T, d.part, skip);
#define QP_GRAMF_CASE(NS)          \
  case NS:                         \
    if (two) {                     \
      QP_GRAMF_LAUNCH(2 * NS, NS)  \
    } else {                       \
      QP_GRAMF_LAUNCH(NS, NS)      \
    }                              \
    break;
  switch (d.nsd) {
    QP_GRAMF_CASE(1)
    QP_GRAMF_CASE(2)
    QP_GRAMF_CASE(3)
    QP_GRAMF_CASE(4)
    QP_GRAMF_CASE(5)
    QP_GRAMF_CASE(6)
    QP_GRAMF_CASE(7)
    QP_GRAMF_CASE(8)
    default:
      return -1;
  }
#undef QP_GRAMF_CASE
#undef QP_GRAMF_LAUNCH
  k_reduce_partials<<<gsz((int64_t)m * nbc * 32), DBLK, 0, d.st>>>(d.part, d.ncta, m * nbc, out, skip);
  return 0;
}

void lincomb(Dav& d, int m, const double* C, const double* A0, double* O0, const double* A1 = nullptr,
             double* O1 = nullptr, const double* A2 = nullptr, double* O2 = nullptr, const int* skip = nullptr) {
  LinComb L{};
  L.A[0] = A0;
  L.out[0] = O0;
  L.n = 1;
  if (A1) {
    L.A[1] = A1;
    L.out[1] = O1;
    L.n = 2;
  }
  if (A2) {
    L.A[2] = A2;
    L.out[2] = O2;
    L.n = 3;
  }
  const int nb = m / d.nsd;
  const unsigned grid = std::min<unsigned>(gsz(d.N), d.c->n_sm * 8);
  switch (d.nsd) {
#define QP_LC_CASE(NS) \
  case NS:             \
    k_lincomb<NS><<<grid, DBLK, 0, d.st>>>(L, nb, d.N, C, skip); \
    break;
    QP_LC_CASE(1)
    QP_LC_CASE(2)
    QP_LC_CASE(3)
    QP_LC_CASE(4)
    QP_LC_CASE(5)
    QP_LC_CASE(6)
    QP_LC_CASE(7)
    QP_LC_CASE(8)
#undef QP_LC_CASE
  }
}

// the same linear combination in float-float arithmetic (mixed precision:
// Ritz vectors, Gram-Schmidt updates, re-contraction)
void lincomb_ff(Dav& d, int m, const double* C, const double* A0, double* O0, const double* A1 = nullptr,
                double* O1 = nullptr, const double* A2 = nullptr, double* O2 = nullptr, const int* skip = nullptr) {
  LinComb L{};
  L.A[0] = A0;
  L.out[0] = O0;
  L.n = 1;
  if (A1) {
    L.A[1] = A1;
    L.out[1] = O1;
    L.n = 2;
  }
  if (A2) {
    L.A[2] = A2;
    L.out[2] = O2;
    L.n = 3;
  }
  const int nb = m / d.nsd;
  const unsigned grid = std::min<unsigned>(gsz(d.N), d.c->n_sm * 8);
  switch (d.nsd) {
#define QP_LCF_CASE(NS) \
  case NS:              \
    k_lincomb_ff<NS><<<grid, DBLK, 0, d.st>>>(L, nb, d.N, C, skip); \
    break;
    QP_LCF_CASE(1)
    QP_LCF_CASE(2)
    QP_LCF_CASE(3)
    QP_LCF_CASE(4)
    QP_LCF_CASE(5)
    QP_LCF_CASE(6)
    QP_LCF_CASE(7)
    QP_LCF_CASE(8)
#undef QP_LCF_CASE
  }
}

// the Ritz-vector combination of three (A, out) pairs in FP32 (k_lincomb32)
void lincomb32(Dav& d, int m, const double* C, const double* A0, double* O0, const double* A1, double* O1,
               const double* A2, double* O2) {
  LinComb L{};
  L.A[0] = A0;
  L.out[0] = O0;
  L.A[1] = A1;
  L.out[1] = O1;
  L.A[2] = A2;
  L.out[2] = O2;
  L.n = 3;
  const int nb = m / d.nsd;
  const unsigned grid = std::min<unsigned>(gsz(d.N), d.c->n_sm * 8);
  switch (d.nsd) {
#define QP_LC32_CASE(NS) \
  case NS:               \
    k_lincomb32<NS><<<grid, DBLK, 0, d.st>>>(L, nb, d.N, C); \
    break;
    QP_LC32_CASE(1)
    QP_LC32_CASE(2)
    QP_LC32_CASE(3)
    QP_LC32_CASE(4)
    QP_LC32_CASE(5)
    QP_LC32_CASE(6)
    QP_LC32_CASE(7)
    QP_LC32_CASE(8)
#undef QP_LC32_CASE
  }
}

// orthonormalise block b against blocks 0..b-1 and within itself: one fused
// Gram-Schmidt + Cholesky-QR pass (k_cgs_coef), a second one when the first
// lost more than half of a column's norm, then a Cholesky-QR pass on the
// block alone (CholQR2).  ff = true: Gram blocks and updates in float-float
// (the small factorisations stay FP64)
void orthonormalise(Dav& d, int b, bool ff) {
  double* Ub = d.blk(d.U, b);
  double* X = d.small + OFF_X;
  double* K = d.small + OFF_K;
  double* G = d.small + OFF_G;
  double* Rinv = d.small + OFF_RINV;
  int* skip2 = (int*)(d.small + OFF_FLAG);
  const int m = b * d.nsd, m1 = m + d.nsd;
  if (d.tc) {  // Gram blocks and updates on the tensor cores (FP64-accurate)
    if (b > 0) {
      gram_tc(d, d.U, m1, Ub, nullptr, X, TC_BASIS_NEW);
      k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 0);
      lincomb_tc(d, m1, K, d.U, Ub);
      gram_tc(d, d.U, m1, Ub, nullptr, X, TC_BASIS_NEW, skip2);
      k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 1);
      lincomb_tc(d, m1, K, d.U, Ub, nullptr, nullptr, nullptr, nullptr, skip2);
    }
    // the nsd x nsd self-Gram and update of Cholesky-QR are too small for
    // the tensor cores' fixed cost: they stay on the FP64 pipe
    for (int pass = (b > 0) ? 1 : 0; pass < 2; ++pass) {
      gram(d, Ub, d.nsd, Ub, nullptr, G);
      k_chol_inv<<<1, 32, 0, d.st>>>(G, d.nsd, Rinv);
      lincomb(d, d.nsd, Rinv, Ub, Ub);
    }
    // the block is final: cache its column exponents for later Grams
    cudaMemsetAsync(d.uexp + m, 0, d.nsd * sizeof(int), d.st);
    qp_col_maxexp(Ub, 1, 0, d.nsd, d.nsd, d.N, d.uexp, m, nullptr, d.st, d.c->n_sm);
    return;
  }
  if (!ff) {
    if (b > 0) {
      gram(d, d.U, m1, Ub, nullptr, X);
      k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 0);
      lincomb(d, m1, K, d.U, Ub);
      gram(d, d.U, m1, Ub, nullptr, X, skip2);
      k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 1);
      lincomb(d, m1, K, d.U, Ub, nullptr, nullptr, nullptr, nullptr, skip2);
    }
    for (int pass = (b > 0) ? 1 : 0; pass < 2; ++pass) {
      gram(d, Ub, d.nsd, Ub, nullptr, G);
      k_chol_inv<<<1, 32, 0, d.st>>>(G, d.nsd, Rinv);
      lincomb(d, d.nsd, Rinv, Ub, Ub);
    }
    return;
  }
  // float-float: the Gram blocks read the split copies Uf (blocks 0..b-1 are
  // split when they are finished; block b is split before each use)
  float2* Ufb = d.Uf + (int64_t)b * d.sUf;
  if (b > 0) {
    split_block(d, Ub, nullptr, Ufb);
    gram_ff(d, d.Uf, m1, Ufb, d.nsd, X);
    k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 0);
    lincomb_ff(d, m1, K, d.U, Ub);
    split_block(d, Ub, nullptr, Ufb, skip2);
    gram_ff(d, d.Uf, m1, Ufb, d.nsd, X, skip2);
    k_cgs_coef<<<1, 128, 0, d.st>>>(X, m, d.nsd, K, skip2, 1);
    lincomb_ff(d, m1, K, d.U, Ub, nullptr, nullptr, nullptr, nullptr, skip2);
  }
  for (int pass = (b > 0) ? 1 : 0; pass < 2; ++pass) {
    split_block(d, Ub, nullptr, Ufb);
    gram_ff(d, Ufb, d.nsd, Ufb, d.nsd, G);
    k_chol_inv<<<1, 32, 0, d.st>>>(G, d.nsd, Rinv);
    lincomb_ff(d, d.nsd, Rinv, Ub, Ub);
  }
  split_block(d, Ub, nullptr, Ufb);
}

// Per-phase stream timeline of one Davidson run (environment QPGPU_PROFILE=1):
// an event closes each phase, and the time between consecutive events is
// charged to the phase that ended, so host work between launches (the small
// eigenproblem) shows up as the gap it leaves on the stream.
struct DavProf {
  enum { OTHER, ORTHO, SIGMA, GRAM, HOST, RITZ, STEP, RESTART, NPH };
  bool on = false;
  cudaStream_t st = nullptr;
  std::vector<std::pair<int, cudaEvent_t>> ev;
  void mark(int phase) {
    if (!on) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    ev.emplace_back(phase, e);
  }
  void report(int n_sigma) {
    if (!on || ev.size() < 2) return;
    static const char* names[NPH] = {"other", "orthonormalise", "sigma", "gram W,S", "host small eig",
                                     "ritz vectors", "step + norms", "restart"};
    double ms[NPH] = {0};
    cudaEventSynchronize(ev.back().second);
    for (size_t i = 1; i < ev.size(); ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[i - 1].second, ev[i].second);
      ms[ev[i].first] += t;
    }
    double tot = 0;
    for (double x : ms) tot += x;
    for (int p = 0; p < NPH; ++p)
      fprintf(stderr, "[qpgpu davidson] %-16s %10.3f ms  %5.1f%%  %8.3f ms/sigma\n", names[p], ms[p],
              100.0 * ms[p] / tot, ms[p] / std::max(1, n_sigma));
    for (auto& e : ev) cudaEventDestroy(e.second);
    ev.clear();
  }
};

}  // namespace

extern "C" int qpgpu_davidson_hs2(qpgpu_ctx* c, double* u_in, int64_t dim_in, double* energies, double* s2_out,
                                  const qpgpu_davidson_params* prm, qpgpu_davidson_trace* trace) {
  if (!c || !u_in || !energies || !s2_out || !prm) return QPGPU_ERR_ARG;
  if (!c->have_pairs) return qpgpu_fail(c, QPGPU_ERR_STATE, "determinants not set");
  const int64_t N = c->N;
  const int nst = prm->n_states, nsd = prm->n_states_diag;
  if (nst < 1 || nsd < nst || nsd > MAXS || dim_in < N || prm->davidson_sze_max < 1 ||
      (prm->precision != QPGPU_FP64 && prm->precision != QPGPU_FP32 && prm->precision != QPGPU_FF))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad Davidson parameters (1 <= n_states <= n_states_diag <= 8)");
  if (prm->algebra != QPGPU_ALGEBRA_FAST && prm->algebra != QPGPU_ALGEBRA_FP64 && prm->algebra != QPGPU_ALGEBRA_TC)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "algebra must be QPGPU_ALGEBRA_FAST, _FP64 or _TC");
  if (prm->dressed && !c->dress.on) return qpgpu_fail(c, QPGPU_ERR_STATE, "dressed Davidson without a dressing");
  if (prm->preconditioner < 0 || prm->preconditioner > 2)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "preconditioner must be 0 (diagonal), 1 (learned) or 2 (learned, extra direction)");
  if ((int64_t)nsd * 3 > N) return qpgpu_fail(c, QPGPU_ERR_ARG, "N_st_diag*3 > sze (diagonalization_hs2.irp.f:110)");
  int itermax = std::max(3, (int)std::min<int64_t>(prm->davidson_sze_max, N / nsd));
  while (itermax * nsd > MAXM) --itermax;
  const bool mixed = prm->precision == QPGPU_FP32 || prm->precision == QPGPU_FF;
  // tall-skinny algebra of the mixed modes on the FP32 pipes (float-float /
  // FP32), or in FP64 like the plain loop (algebra = QPGPU_ALGEBRA_FP64)
  const bool ffalg = mixed && prm->algebra == QPGPU_ALGEBRA_FAST;
  // FP64-accurate Gram blocks on the tensor cores (any precision)
  const bool tcalg = prm->algebra == QPGPU_ALGEBRA_TC;
  const int restart_prec = prm->precision == QPGPU_FF ? QPGPU_FF : QPGPU_FP64;  // defect-correction sigma
  if (mixed && prm->defect_every > 0) itermax = std::max(3, std::min(itermax, prm->defect_every + 1));
  const int max_sigma = prm->max_iter > 0 ? prm->max_iter : 1000;

  std::lock_guard<std::mutex> lk(c->mu);
  Dav d;
  d.c = c;
  d.st = c->stream;
  d.N = N;
  d.nsd = nsd;
  d.nst = nst;
  d.itermax = itermax;
  d.ncta = 2 * c->n_sm;  // two CTAs per SM
  d.tc = tcalg;
  d.rows_per_cta = (N + d.ncta - 1) / d.ncta;
  const size_t blkn = (size_t)N * nsd;
  if (dev_alloc(&d.U, blkn * itermax) != cudaSuccess || dev_alloc(&d.W, blkn * itermax) != cudaSuccess ||
      dev_alloc(&d.S, blkn * itermax) != cudaSuccess || dev_alloc(&d.R, blkn) != cudaSuccess ||
      dev_alloc(&d.u32, (size_t)N * qp_pad_states(nsd)) != cudaSuccess || dev_alloc(&d.part, (size_t)d.ncta * MAXM * 2 * MAXS) != cudaSuccess ||
      dev_alloc(&d.small, (size_t)SMALL_DOUBLES) != cudaSuccess) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "Davidson work arrays do not fit on the device");
  }
  if (tcalg) {
    if (qp_gram_oz_prepare() || dev_alloc(&d.uexp, MAXM) != cudaSuccess ||
        dev_alloc(&d.bexp, 2 * MAXS + 1) != cudaSuccess) {
      cudaGetLastError();
      return qpgpu_fail(c, QPGPU_ERR_NOMEM, "tensor-core Gram work arrays could not be set up");
    }
    QP_CUDA(c, cudaMemsetAsync(d.bexp, 0, (2 * MAXS + 1) * sizeof(int), d.st));
  }
  d.sUf = (int64_t)blkn;
  if (ffalg && (dev_alloc(&d.Uf, blkn * itermax) != cudaSuccess || dev_alloc(&d.Bf, blkn * 2) != cudaSuccess)) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "mixed-precision work arrays do not fit on the device");
  }
  cudaStream_t st = d.st;
  // learned preconditioner and training capture
  const bool use_mlp = prm->preconditioner == 1 || prm->preconditioner == 2;
  if (use_mlp && (!c->mlp.ready || !c->d_detfeat))
    return qpgpu_fail(c, QPGPU_ERR_STATE, "learned preconditioner requested but the MLP is not initialised");
  bool mlp_on[MAXS] = {false};
  int strikes[MAXS] = {0};
  double prev_res[MAXS];
  for (int k = 0; k < MAXS; ++k) prev_res[k] = INFINITY;
  // extra mode: state k's learned correction uses the slot of Ritz vector nst + k
  const int mlp_extra = prm->preconditioner == 2;
  for (int k = 0; k < nst; ++k) mlp_on[k] = use_mlp && (!mlp_extra || nst + k < nsd);
  if (use_mlp && (dev_alloc(&d.mlpX, (size_t)N * nst * QP_MLP_IN) != cudaSuccess ||
                  dev_alloc(&d.mlpG, (size_t)N * nst) != cudaSuccess)) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "learned-step work arrays do not fit on the device");
  }
  int n_fallback = 0;
  const int collect_every = prm->collect_every > 0 ? prm->collect_every : 0;
  const int collect_max = collect_every ? std::max(1, std::min(prm->collect_max > 0 ? prm->collect_max : 8, 64 / nst)) : 0;
  int n_cap = 0, it_global = 0;
  int64_t n_new_samples = 0;
  if (collect_every) {
    if (!c->d_detfeat) return qpgpu_fail(c, QPGPU_ERR_STATE, "no determinant features");
    const size_t nsl = (size_t)collect_max * nst;
    if (cudaMalloc((void**)&d.cX, nsl * N * QP_MLP_IN * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&d.cd, nsl * N * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&d.cc, nsl * N * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return qpgpu_fail(c, QPGPU_ERR_NOMEM, "training capture does not fit on the device");
    }
  }
  cudaEvent_t ev0;
  QP_CUDA(c, cudaEventCreate(&ev0));
  std::vector<cudaEvent_t> evs;
  QP_CUDA(c, cudaEventRecord(ev0, st));
  // guess vectors: u_in(dim_in, nsd) in psi_det order -> block 0, bilinear
  {
    double* hstage = nullptr;
    QP_CUDA(c, cudaMalloc((void**)&hstage, blkn * sizeof(double)));
    QP_CUDA(c, cudaMemcpy2DAsync(hstage, N * sizeof(double), u_in, dim_in * sizeof(double), N * sizeof(double), nsd,
                                 cudaMemcpyHostToDevice, st));
    int* bad = nullptr;
    int hbad = 0;
    const int rcf = qp_numeric_flag(c, st, &bad);
    if (rcf) return rcf;
    qp_to_bilinear(hstage, N, c->d_order, d.U, nullptr, nsd, N, st, bad);
    QP_CUDA(c, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    cudaFree(hstage);
    if (hbad) {
      cudaEventDestroy(ev0);
      return qpgpu_fail(c, QPGPU_ERR_NUMERIC, "the guess vectors hold a NaN or an infinity");
    }
  }
  const double* hjj = prm->dressed ? c->dress.hdress : c->d_hdiag;  // dressed H_jj (:547-549)
  const double Sz = 0.5 * (c->na - c->nb);
  const double sz2sz = Sz * (Sz - 1.0), expected_s2 = Sz * (Sz + 1.0);
  const int mmax = itermax * nsd;
  std::vector<double> h((size_t)mmax * mmax, 0.0), s_((size_t)mmax * mmax, 0.0);
  std::vector<double> hcol((size_t)mmax * nsd), scol((size_t)mmax * nsd), hscol((size_t)mmax * 2 * nsd);
  std::vector<double> lambda(mmax), s2(mmax), y, wv, res(MAXS, 0.0), partial((size_t)d.ncta * MAXS);
  int n_sigma = 0, shift2 = 0, trace_n = 0;
  bool converged = false, failed = false;
  auto record = [&](int prec) {
    if (!trace || trace_n >= trace->cap) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    evs.push_back(e);
    if (trace->sigma_precision) trace->sigma_precision[trace_n] = prec;
    for (int k = 0; k < nst; ++k) {
      if (trace->energies) trace->energies[(size_t)trace_n * nst + k] = lambda[k];
      if (trace->residuals) trace->residuals[(size_t)trace_n * nst + k] = res[k];
    }
    ++trace_n;
  };
  DavProf prof;
  prof.on = c->profile;
  prof.st = st;
  prof.mark(DavProf::OTHER);
  while (!converged && !failed && n_sigma < max_sigma) {
    for (int iter = 1; iter <= itermax - 1; ++iter) {
      const int b = iter - 1;
      const int shift = nsd * b;
      shift2 = nsd * iter;
      orthonormalise(d, b, ffalg);
      prof.mark(DavProf::ORTHO);
      // sigma on block b
      const int prec = (mixed && iter > 1) ? QPGPU_FP32 : restart_prec;
      if (prec == QPGPU_FP32) qp_to_float(d.blk(d.U, b), d.u32, N, nsd, qp_pad_states(nsd), st);
      int rc = (prec == QPGPU_FF)
                   ? qp_sigma_ff(c, &c->items, d.blk(d.W, b), d.blk(d.S, b), d.blk(d.U, b), nsd, st, 0, (int)N, 0, 1)
                   : qp_sigma_launch(c, &c->items, d.blk(d.W, b), d.blk(d.S, b), d.blk(d.U, b), d.u32, nsd, prec, st,
                                     0, (int)N, 0, 1, qp_pad_states(nsd));
      if (!rc && prm->dressed) rc = qp_dress(c, d.blk(d.W, b), d.blk(d.S, b), d.blk(d.U, b), nsd, st);
      if (rc) return rc;
      ++n_sigma;
      prof.mark(DavProf::SIGMA);
      // new Gram columns
      // h(:, new) and s(:, new) in one pass over U: X = U^T [W_b S_b]
      if (ffalg) {
        split_block(d, d.blk(d.W, b), d.blk(d.S, b), d.Bf);
        gram_ff(d, d.Uf, shift2, d.Bf, 2 * nsd, d.small + OFF_X);
      } else if (tcalg) {
        gram_tc(d, d.U, shift2, d.blk(d.W, b), d.blk(d.S, b), d.small + OFF_X, TC_BASIS);
      } else {
        gram(d, d.U, shift2, d.blk(d.W, b), d.blk(d.S, b), d.small + OFF_X);
      }
      QP_CUDA(c, cudaMemcpyAsync(hscol.data(), d.small + OFF_X, (size_t)shift2 * 2 * nsd * sizeof(double),
                                 cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaStreamSynchronize(st));
      for (int i = 0; i < shift2; ++i)
        for (int j = 0; j < nsd; ++j) {
          hcol[(size_t)i * nsd + j] = hscol[(size_t)i * 2 * nsd + j];
          scol[(size_t)i * nsd + j] = hscol[(size_t)i * 2 * nsd + nsd + j];
        }
      prof.mark(DavProf::GRAM);
      for (int i = 0; i < shift2; ++i)
        for (int j = 0; j < nsd; ++j) {
          const int col = shift + j;
          if (i > col) continue;  // upper triangle
          h[(size_t)i * mmax + col] = h[(size_t)col * mmax + i] = hcol[(size_t)i * nsd + j];
          s_[(size_t)i * mmax + col] = s_[(size_t)col * mmax + i] = scol[(size_t)i * nsd + j];
        }
      // small eigenproblem (:284)
      std::vector<double> hs((size_t)shift2 * shift2), ss((size_t)shift2 * shift2);
      for (int i = 0; i < shift2; ++i)
        for (int j = 0; j < shift2; ++j) {
          hs[(size_t)i * shift2 + j] = h[(size_t)i * mmax + j];
          ss[(size_t)i * shift2 + j] = s_[(size_t)i * mmax + j];
        }
      qp_eigh(hs, shift2, wv, y);
      for (int k = 0; k < shift2; ++k) lambda[k] = wv[k];
      // S^2 of the Ritz vectors (:289-301): s2_k = y_k^T s y_k + S_z(S_z-1)
      for (int k = 0; k < shift2; ++k) {
        double acc = 0.0;
        for (int i = 0; i < shift2; ++i) {
          double t = 0.0;
          for (int j = 0; j < shift2; ++j) t += ss[(size_t)i * shift2 + j] * y[(size_t)j * shift2 + k];
          acc += y[(size_t)i * shift2 + k] * t;
        }
        s2[k] = acc + sz2sz;
      }
      // s2_eig filter (:303-326)
      std::vector<char> ok(shift2, 1);
      if (prm->s2_eig)
        for (int k = 0; k < shift2; ++k) ok[k] = std::fabs(s2[k] - expected_s2) < 0.6;
      for (int k = 0; k < shift2; ++k) {
        if (ok[k]) continue;
        for (int l = k + 1; l < shift2; ++l)
          if (ok[l]) {
            for (int i = 0; i < shift2; ++i) std::swap(y[(size_t)i * shift2 + k], y[(size_t)i * shift2 + l]);
            std::swap(s2[k], s2[l]);
            std::swap(lambda[k], lambda[l]);
            ok[k] = 1;
            ok[l] = 0;
            break;
          }
      }
      // state following (:328-370): for target k, order[k] is the row i < nst
      // (the component along the guess / previous Ritz vector i) of largest
      // |y(i,k)| among the rows not taken by an earlier target; the reference
      // then takes Ritz vector order[k] as target k (its row index serves as
      // a column index), with its eigenvalue and S^2
      if (prm->state_following) {
        std::vector<double> ov((size_t)shift2 * shift2);
        for (size_t q = 0; q < ov.size(); ++q) ov[q] = std::fabs(y[q]);
        std::vector<int> order(nst);
        for (int k = 0; k < nst; ++k) {
          double cmax = -1.0;
          for (int i = 0; i < nst; ++i)
            if (ov[(size_t)i * shift2 + k] > cmax) {
              cmax = ov[(size_t)i * shift2 + k];
              order[k] = i;
            }
          for (int i = 0; i < nsd; ++i) ov[(size_t)order[k] * shift2 + i] = -1.0;
        }
        const std::vector<double> y0 = y;
        const std::vector<double> l0(lambda.begin(), lambda.begin() + nst), s0(s2.begin(), s2.begin() + nst);
        for (int k = 0; k < nst; ++k) {
          const int l = order[k];
          if (l == k) continue;
          for (int i = 0; i < shift2; ++i) y[(size_t)i * shift2 + k] = y0[(size_t)i * shift2 + l];
          lambda[k] = l0[l];
          s2[k] = s0[l];
        }
      }
      // Ritz vectors into block b+1 (:376-381); coefficients y(0:shift2, 0:nsd)
      std::vector<double> ycoef((size_t)shift2 * nsd);
      for (int i = 0; i < shift2; ++i)
        for (int j = 0; j < nsd; ++j) ycoef[(size_t)i * nsd + j] = y[(size_t)i * shift2 + j];
      double* ydev = d.small + OFF_Y;
      prof.mark(DavProf::HOST);
      QP_CUDA(c, cudaMemcpyAsync(ydev, ycoef.data(), ycoef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      if ((ffalg || tcalg) && prec == QPGPU_FP32)  // W, S from the FP32 sigma: FP32 Ritz vectors feed the step
        lincomb32(d, shift2, ydev, d.U, d.blk(d.U, iter), d.W, d.blk(d.W, iter), d.S, d.blk(d.S, iter));
      else if (ffalg)  // restart iteration: float-float
        lincomb_ff(d, shift2, ydev, d.U, d.blk(d.U, iter), d.W, d.blk(d.W, iter), d.S, d.blk(d.S, iter));
      else if (tcalg)
        lincomb_tc(d, shift2, ydev, d.U, d.blk(d.U, iter), d.W, d.blk(d.W, iter), d.S, d.blk(d.S, iter));
      else
        lincomb(d, shift2, ydev, d.U, d.blk(d.U, iter), d.W, d.blk(d.W, iter), d.S, d.blk(d.S, iter));
      prof.mark(DavProf::RITZ);
      // Davidson step and residual norms (:386-395)
      StepParams sp{};
      for (int k = 0; k < nsd; ++k) {
        sp.lambda[k] = lambda[k];
        sp.s2[k] = s2[k];
      }
      sp.sz2sz = sz2sz;
      sp.nsd = nsd;
      sp.nst = nst;
      ++it_global;
      if (collect_every && n_cap < collect_max && it_global >= 2 && (it_global - 2) % collect_every == 0) {
        k_capture<<<gsz(N), DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), hjj,
                                           (const float4*)c->d_detfeat, N, sp, n_cap * nst, d.cX, d.cd, d.cc);
        ++n_cap;
      }
      unsigned mask = 0;
      for (int k = 0; k < nst; ++k)
        if (mlp_on[k]) mask |= 1u << k;
      if (mask) {
        k_mlp_features<<<gsz(N), DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), hjj,
                                                (const float4*)c->d_detfeat, N, sp, d.mlpX);
        qp_mlp_eval(c->mlp.params, d.mlpX, d.mlpG, N * nst, st, c->n_sm);
        k_step_mlp<<<d.ncta, DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), hjj, d.mlpG,
                                            N, sp, mask, mlp_extra, d.part);
      }
      else if (ffalg)
        k_step_mixed<<<d.ncta, DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), hjj, N, sp,
                                              d.part);
      else
        k_step<<<d.ncta, DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), hjj, N, sp, d.part);
      QP_CUDA(c, cudaGetLastError());
      QP_CUDA(c, cudaMemcpyAsync(partial.data(), d.part, partial.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
      int tc_status = 0;
      if (tcalg)
        QP_CUDA(c, cudaMemcpyAsync(&tc_status, d.bexp + 2 * MAXS, sizeof(int), cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaStreamSynchronize(st));
      if (tc_status) {
        cudaEventDestroy(ev0);
        return qpgpu_fail(c, QPGPU_ERR_TIMEOUT, "Davidson: a bounded tensor-core wait of the Gram blocks ran out");
      }
      prof.mark(DavProf::STEP);
      double mx = 0.0;
      for (int k = 0; k < nst; ++k) {
        double r = 0.0;
        for (int q = 0; q < d.ncta; ++q) r += partial[(size_t)q * MAXS + k];
        res[k] = r;
        mx = std::max(mx, r);
        if (r > 1e8 || !std::isfinite(r)) failed = true;  // 'Davidson failed' (:404-409)
      }
      // fallback: a state whose residual (the reference's measure, from the
      // diagonal correction) fails to fall by at least 5% after a learned step
      // goes back to the diagonal step for the rest of the run.
      // The first iteration of a restart cycle is not judged: its residual
      // comes from the re-contracted basis (and, in mixed precision, from the
      // cycle's first FP64 sigma), not from the preceding step.
      for (int k = 0; k < nst; ++k) {
        if (mlp_on[k] && iter > 1) {
          strikes[k] = (res[k] > 0.95 * prev_res[k]) ? strikes[k] + 1 : 0;
          if (strikes[k] >= 1) {
            mlp_on[k] = false;
            ++n_fallback;
          }
        }
        prev_res[k] = res[k];
      }
      record(prec);
      if (failed) break;
      // davidson_converged, parameters.irp.f:9-49 ('residual'; not before the 2nd iteration)
      const bool below = std::fabs(mx) < prm->threshold;
      if (below && prec != QPGPU_FP32 && (iter >= 2 || mixed)) {
        converged = true;
        break;
      }
      if (below && prec == QPGPU_FP32) {
        break;  // restart: confirm with an FP64 sigma on the re-contracted vectors
      }
      if (n_sigma >= max_sigma) break;
    }
    // re-contract (:419-420): U(:,0..shift2) y(:,0..nsd) -> block 0
    std::vector<double> ycoef((size_t)shift2 * nsd);
    for (int i = 0; i < shift2; ++i)
      for (int j = 0; j < nsd; ++j) ycoef[(size_t)i * nsd + j] = y[(size_t)i * shift2 + j];
    double* ydev = d.small + OFF_Y;
    QP_CUDA(c, cudaMemcpyAsync(ydev, ycoef.data(), ycoef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (ffalg)
      lincomb_ff(d, shift2, ydev, d.U, d.R);
    else if (tcalg)
      lincomb_tc(d, shift2, ydev, d.U, d.R);
    else
      lincomb(d, shift2, ydev, d.U, d.R);
    k_copy<<<gsz((int64_t)blkn), DBLK, 0, st>>>(d.R, d.U, (int64_t)blkn);
    prof.mark(DavProf::RESTART);
    for (int i = 0; i < mmax; ++i)
      for (int j = 0; j < mmax; ++j) h[(size_t)i * mmax + j] = s_[(size_t)i * mmax + j] = 0.0;
  }
  QP_CUDA(c, cudaGetLastError());
  prof.report(n_sigma);
  // training pairs from the captured iterations, with the final vectors
  if (n_cap > 0 && !failed) {
    const int nslot = n_cap * nst;
    std::vector<double> part((size_t)d.ncta * nslot * 2), dot(nslot, 0.0), nd(nslot, 0.0), ne(nslot, 0.0),
        ed(nslot, 0.0);
    double* dpart = nullptr;
    double* ddot = nullptr;
    SlotScale* dsc = nullptr;
    QP_CUDA(c, cudaMalloc((void**)&dpart, part.size() * sizeof(double)));
    QP_CUDA(c, cudaMalloc((void**)&ddot, nslot * sizeof(double)));
    QP_CUDA(c, cudaMalloc((void**)&dsc, nslot * sizeof(SlotScale)));
    k_capture_sums<<<d.ncta, DBLK, 0, st>>>(d.U, nsd, nst, d.cd, d.cc, nslot, N, nullptr, 0, dpart);
    QP_CUDA(c, cudaMemcpyAsync(part.data(), dpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    for (int q = 0; q < d.ncta; ++q)
      for (int sl = 0; sl < nslot; ++sl) {
        dot[sl] += part[((size_t)q * nslot + sl) * 2];
        nd[sl] += part[((size_t)q * nslot + sl) * 2 + 1];
      }
    QP_CUDA(c, cudaMemcpyAsync(ddot, dot.data(), nslot * sizeof(double), cudaMemcpyHostToDevice, st));
    k_capture_sums<<<d.ncta, DBLK, 0, st>>>(d.U, nsd, nst, d.cd, d.cc, nslot, N, ddot, 1, dpart);
    QP_CUDA(c, cudaMemcpyAsync(part.data(), dpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    for (int q = 0; q < d.ncta; ++q)
      for (int sl = 0; sl < nslot; ++sl) {
        ne[sl] += part[((size_t)q * nslot + sl) * 2];
        ed[sl] += part[((size_t)q * nslot + sl) * 2 + 1];
      }
    std::vector<SlotScale> sc(nslot);
    for (int sl = 0; sl < nslot; ++sl) {
      const bool ok = ne[sl] > 1e-30 && nd[sl] > 1e-300;
      sc[sl].dot = dot[sl];
      sc[sl].inv_ne = ok ? 1.0 / std::sqrt(ne[sl]) : 0.0;
      sc[sl].inv_nd = ok ? 1.0 / std::sqrt(nd[sl]) : 0.0;
      sc[sl].sign = ed[sl] >= 0 ? 1.0 : -1.0;
    }
    QP_CUDA(c, cudaMemcpyAsync(dsc, sc.data(), nslot * sizeof(SlotScale), cudaMemcpyHostToDevice, st));
    const int64_t per_cap = 32768;
    const int64_t stride = std::max<int64_t>(1, (N + per_cap - 1) / per_cap);
    const int64_t per_slot = (N + stride - 1) / stride;
    const int64_t total = per_slot * nslot;
    float *X = nullptr, *Gt = nullptr, *Wt = nullptr;
    QP_CUDA(c, cudaMalloc((void**)&X, total * QP_MLP_IN * sizeof(float)));
    QP_CUDA(c, cudaMalloc((void**)&Gt, total * sizeof(float)));
    QP_CUDA(c, cudaMalloc((void**)&Wt, total * sizeof(float)));
    k_capture_samples<<<gsz(total), DBLK, 0, st>>>(d.U, nsd, nst, d.cX, d.cd, d.cc, nslot, N, dsc, stride, per_slot, X,
                                                   Gt, Wt);
    int rc2 = qp_mlp_append(c, X, Gt, Wt, total, true);
    cudaFree(X);
    cudaFree(Gt);
    cudaFree(Wt);
    cudaFree(dpart);
    cudaFree(ddot);
    cudaFree(dsc);
    if (rc2) return rc2;
    n_new_samples = total;
  }
  // final vectors (block 0 after re-contraction) back to psi_det order
  {
    double* hstage = nullptr;
    QP_CUDA(c, cudaMalloc((void**)&hstage, blkn * sizeof(double)));
    qp_from_bilinear(d.U, N, c->d_order, hstage, nsd, N, st);
    QP_CUDA(c, cudaMemcpy2DAsync(u_in, dim_in * sizeof(double), hstage, N * sizeof(double), N * sizeof(double), nsd,
                                 cudaMemcpyDeviceToHost, st));
    QP_CUDA(c, cudaStreamSynchronize(st));
    cudaFree(hstage);
  }
  for (int k = 0; k < nsd; ++k) {
    energies[k] = lambda[k];
    s2_out[k] = s2[k];
  }
  if (trace) {
    trace->n = trace_n;
    for (int i = 0; i < trace_n; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev0, evs[i]);
      if (trace->elapsed_ms) trace->elapsed_ms[i] = ms;
      cudaEventDestroy(evs[i]);
    }
    trace->n_sigma = n_sigma;
    trace->converged = converged ? 1 : 0;
    trace->n_fallback = n_fallback;
    trace->n_samples = n_new_samples;
  }
  cudaEventDestroy(ev0);
  if (failed) return qpgpu_fail(c, QPGPU_ERR_DAVIDSON, "Davidson failed: residual above 1e8");
  return n_sigma;
}
