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
// restart, so the reported energies and residuals are FP64 ones.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "qpgpu_internal.cuh"

// Host cyclic Jacobi eigen-solver for the small projected matrix (stands in
// for lapack_diag/dsyev, LinearAlgebra.irp.f:446-512): eigenvalues ascending,
// eigenvectors in the columns of v (n x n, row-major v[i*n+j] = component i of
// vector j).
void qp_jacobi(std::vector<double> a, int n, std::vector<double>& w, std::vector<double>& v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double x = a[(size_t)i * n + j] * a[(size_t)i * n + j];
        tot += x;
        if (i != j) off += x;
      }
    if (off == 0.0 || off <= 1e-32 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - s * vkq;
          v[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int x, int y) { return a[(size_t)x * n + x] < a[(size_t)y * n + y]; });
  std::vector<double> v2((size_t)n * n);
  w.resize(n);
  for (int j = 0; j < n; ++j) {
    w[j] = a[(size_t)ord[j] * n + ord[j]];
    for (int i = 0; i < n; ++i) v2[(size_t)i * n + j] = v[(size_t)i * n + ord[j]];
  }
  v.swap(v2);
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

// G[i][j] = sum_r A_i[r] B_j[r] for the m columns of A (stacked blocks of nsd
// columns, block stride N*nsd) and the nsd columns of B.  Rows are staged in
// shared memory; a thread owns CI consecutive columns of A for every j (a
// CI x nsd register tile: CI + nsd shared reads per CI*nsd FMAs) over the rows
// of its row group, and the row groups are added in a fixed order.  One
// partial per CTA.  A non-null `skip` flag that is set makes the kernel write
// zeros (the conditional second Gram-Schmidt pass).
constexpr int GTR = 32;
template <int CI>
__global__ void __launch_bounds__(DBLK) k_gram(const double* A, int m, const double* B, int nsd, int64_t N,
                                               int64_t rows_per_cta, double* partial, const int* skip) {
  extern __shared__ double sm[];
  double* As = sm;            // [GTR][m]
  double* Bs = sm + GTR * m;  // [GTR][nsd]
  const int np = m * nsd;
  const int ncol = m / CI;                       // column groups
  const int groups = min(DBLK / ncol, GTR);      // row groups
  if (skip && *skip) {
    for (int p = threadIdx.x; p < np; p += DBLK) partial[(int64_t)blockIdx.x * np + p] = 0.0;
    return;
  }
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(r0 + rows_per_cta, N);
  const int ci = threadIdx.x % ncol, g = threadIdx.x / ncol;
  const bool active = g < groups;
  double acc[CI][MAXS];
#pragma unroll
  for (int a = 0; a < CI; ++a)
#pragma unroll
    for (int j = 0; j < MAXS; ++j) acc[a][j] = 0.0;
  for (int64_t t0 = r0; t0 < r1; t0 += GTR) {
    const int tr = (int)min((int64_t)GTR, r1 - t0);
    __syncthreads();
    const int nb = m / nsd;
    for (int idx = threadIdx.x; idx < nb * tr * nsd; idx += DBLK) {
      const int b = idx / (tr * nsd), rem = idx % (tr * nsd), r = rem / nsd, c = rem % nsd;
      As[r * m + b * nsd + c] = A[(int64_t)b * N * nsd + (t0 + r) * nsd + c];
    }
    for (int idx = threadIdx.x; idx < tr * nsd; idx += DBLK) Bs[idx] = B[t0 * nsd + idx];
    __syncthreads();
    if (active) {
      for (int r = g; r < tr; r += groups) {
        double a[CI];
#pragma unroll
        for (int q = 0; q < CI; ++q) a[q] = As[r * m + ci * CI + q];
        const double* brow = &Bs[r * nsd];
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
          if (j < nsd) {
            const double bv = brow[j];
#pragma unroll
            for (int q = 0; q < CI; ++q) acc[q][j] = fma(a[q], bv, acc[q][j]);
          }
        }
      }
    }
  }
  __syncthreads();
  // fixed-order sum over row groups through shared memory (reuses the tiles)
  double* red = sm;  // [groups][m][nsd]
  if (active)
#pragma unroll
    for (int q = 0; q < CI; ++q)
      for (int j = 0; j < nsd; ++j) red[((size_t)g * m + ci * CI + q) * nsd + j] = acc[q][j];
  __syncthreads();
  for (int p = threadIdx.x; p < np; p += DBLK) {
    double s = 0.0;
    for (int q = 0; q < groups; ++q) s += red[(size_t)q * np + p];
    partial[(int64_t)blockIdx.x * np + p] = s;
  }
}

// out[p] = sum over CTAs of partial[cta][p]: one warp per element, lane l
// adds CTAs l, l+32, ... and the lanes combine in a fixed butterfly order
__global__ void k_reduce_partials(const double* partial, int ncta, int np, double* out) {
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

// out_k[r][j] (=, -=) sum_i A_k[i-th column][r] C[i][j], for up to 3 (A, out)
// pairs sharing C (m x nsd, row-major).  Each thread owns LR rows (LR*256
// apart, so a warp's loads stay contiguous) and keeps LR x nsd accumulators:
// one shared-memory read of C serves LR FMAs.  out may alias A when m == nsd
// (a thread reads all its rows before writing them).
constexpr int LR = 4;
struct LinComb {
  const double* A[3];
  double* out[3];
  int n;
};
__global__ void __launch_bounds__(DBLK) k_lincomb(LinComb L, int m, int nsd, int64_t N, const double* C, int sub,
                                                  const int* skip) {
  if (skip && *skip) return;
  __shared__ __align__(16) double Cs[MAXM * MAXS];
  for (int i = threadIdx.x; i < m * nsd; i += DBLK) Cs[i] = C[i];
  __syncthreads();
  const int nb = m / nsd;
  const int64_t span = (int64_t)DBLK * LR;
  for (int64_t base = (int64_t)blockIdx.x * span; base < N; base += (int64_t)gridDim.x * span) {
    int64_t rr[LR];
    bool ok[LR];
#pragma unroll
    for (int q = 0; q < LR; ++q) {
      rr[q] = base + threadIdx.x + (int64_t)q * DBLK;
      ok[q] = rr[q] < N;
    }
    for (int t = 0; t < L.n; ++t) {
      double acc[LR][MAXS];
#pragma unroll
      for (int q = 0; q < LR; ++q)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) acc[q][j] = 0.0;
      for (int b = 0; b < nb; ++b) {
        const double* ab = L.A[t] + (int64_t)b * N * nsd;
        for (int c = 0; c < nsd; ++c) {
          double x[LR];
#pragma unroll
          for (int q = 0; q < LR; ++q) x[q] = ok[q] ? ab[rr[q] * nsd + c] : 0.0;
          const double* crow = &Cs[(b * nsd + c) * nsd];
#pragma unroll
          for (int j = 0; j < MAXS; ++j) {
            if (j < nsd) {
              const double cv = crow[j];
#pragma unroll
              for (int q = 0; q < LR; ++q) acc[q][j] = fma(x[q], cv, acc[q][j]);
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < LR; ++q) {
        if (!ok[q]) continue;
        double* o = L.out[t] + rr[q] * nsd;
#pragma unroll
        for (int j = 0; j < MAXS; ++j)
          if (j < nsd) o[j] = sub ? o[j] - acc[q][j] : acc[q][j];
      }
    }
  }
}

// Cholesky G = R^T R (nsd x nsd) and Rinv = R^-1 (row-major, upper), one
// thread.  A vanishing pivot (dependent column) gives a zero column.
__global__ void k_chol_inv(const double* G, int nsd, double* Rinv) {
  if (threadIdx.x || blockIdx.x) return;
  double R[MAXS][MAXS], Ri[MAXS][MAXS];
  for (int i = 0; i < nsd; ++i)
    for (int j = 0; j < nsd; ++j) R[i][j] = Ri[i][j] = 0.0;
  for (int j = 0; j < nsd; ++j) {
    double d = G[j * nsd + j];
    for (int k = 0; k < j; ++k) d -= R[k][j] * R[k][j];
    const double scale = fabs(G[j * nsd + j]);
    if (!(d > 1e-28 * scale) || !(d > 1e-300)) {
      for (int k = 0; k < nsd; ++k) R[j][k] = 0.0;
      R[j][j] = 0.0;
      continue;
    }
    R[j][j] = sqrt(d);
    for (int i = j + 1; i < nsd; ++i) {
      double s = G[j * nsd + i];
      for (int k = 0; k < j; ++k) s -= R[k][j] * R[k][i];
      R[j][i] = s / R[j][j];
    }
  }
  // back substitution: Ri = R^-1 (upper triangular); zero pivot -> zero column
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
    for (int j = 0; j < nsd; ++j) Rinv[i * nsd + j] = Ri[i][j];
}

// second Gram-Schmidt pass needed?  Yes when a column lost more than half of
// its norm in the first pass (G0 before, G1 after; diagonals).
__global__ void k_need_second_pass(const double* G0, const double* G1, int nsd, int* skip) {
  if (threadIdx.x || blockIdx.x) return;
  int need = 0;
  for (int j = 0; j < nsd; ++j) {
    const double a = G0[j * nsd + j], b = G1[j * nsd + j];
    if (!(b > 0.25 * a)) need = 1;
  }
  *skip = need ? 0 : 1;
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

// Davidson step with the learned preconditioner: the reference's diagonal
// correction d (whose squared norm stays the convergence measure) is scaled
// per determinant by the MLP's multiplier g for the states flagged in
// p.mlp_mask; other states take d unchanged.
__global__ void __launch_bounds__(DBLK) k_step_mlp(double* Un, const double* Wn, const double* Sn, const double* hjj,
                                                   const float4* feat, const float* P, int64_t N, StepParams p,
                                                   unsigned mlp_mask, double* partial) {
  __shared__ float Ps[QP_MLP_NPARAM];
  __shared__ double red[MAXS][DBLK / 32];
  for (int i = threadIdx.x; i < QP_MLP_NPARAM; i += DBLK) Ps[i] = P[i];
  __syncthreads();
  double acc[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; ++k) acc[k] = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)DBLK + threadIdx.x; r < N; r += (int64_t)gridDim.x * DBLK) {
    const double h = hjj[r];
    const float4 st = feat[r];
    for (int k = 0; k < p.nsd; ++k) {
      const int64_t x = r * p.nsd + k;
      const double u = Un[x];
      const double res = p.lambda[k] * u - Wn[x];
      const double d = res * (1.0 + p.s2[k] * u - Sn[x] - p.sz2sz) / fmax(h - p.lambda[k], 1e-2);
      double v = d;
      if ((mlp_mask >> k) & 1u) {
        float f[QP_MLP_IN];
        qp_features(st, h - p.lambda[k], u, res, d, f);
        v = d * (double)qp_mlp_forward(Ps, f);
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
  int ncta = 0;
  int64_t rows_per_cta = 0;
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
  }
  double* blk(double* X, int b) const { return X + (int64_t)b * N * nsd; }
};

int gram(Dav& d, const double* A, int m, const double* B, double* out_dev, const int* skip = nullptr) {
  const int ci = (m % 4 == 0) ? 4 : (m % 2 == 0) ? 2 : 1;
  const int groups = std::min(DBLK / (m / ci), GTR);
  const size_t shm = std::max((size_t)GTR * (m + d.nsd), (size_t)groups * m * d.nsd) * sizeof(double);
  static bool attr_set = false;  // shared memory above 48 KB needs an opt-in (at most 64 KB here)
  if (!attr_set) {
    cudaFuncSetAttribute(k_gram<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    cudaFuncSetAttribute(k_gram<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    cudaFuncSetAttribute(k_gram<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    attr_set = true;
  }
  if (ci == 4)
    k_gram<4><<<d.ncta, DBLK, shm, d.st>>>(A, m, B, d.nsd, d.N, d.rows_per_cta, d.part, skip);
  else if (ci == 2)
    k_gram<2><<<d.ncta, DBLK, shm, d.st>>>(A, m, B, d.nsd, d.N, d.rows_per_cta, d.part, skip);
  else
    k_gram<1><<<d.ncta, DBLK, shm, d.st>>>(A, m, B, d.nsd, d.N, d.rows_per_cta, d.part, skip);
  k_reduce_partials<<<gsz((int64_t)m * d.nsd * 32), DBLK, 0, d.st>>>(d.part, d.ncta, m * d.nsd, out_dev);
  return 0;
}

void lincomb(Dav& d, int m, const double* C, int sub, const double* A0, double* O0, const double* A1 = nullptr,
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
  k_lincomb<<<gsz((d.N + LR - 1) / LR), DBLK, 0, d.st>>>(L, m, d.nsd, d.N, C, sub, skip);
}

// orthonormalise block b against blocks 0..b-1 (classical Gram-Schmidt, a
// second pass when the first lost more than half of a column's norm) and
// within itself (CholQR2)
void orthonormalise(Dav& d, int b) {
  double* Ub = d.blk(d.U, b);
  double* cbuf = d.small;  // m x nsd
  double* G = d.small + MAXM * MAXS;
  double* Rinv = d.small + 2 * MAXM * MAXS;
  double* G0 = d.small + 4 * MAXM * MAXS;
  int* skip = (int*)(d.small + 5 * MAXM * MAXS);
  if (b > 0) {
    gram(d, Ub, d.nsd, Ub, G0);
    gram(d, d.U, b * d.nsd, Ub, cbuf);
    lincomb(d, b * d.nsd, cbuf, 1, d.U, Ub);
    gram(d, Ub, d.nsd, Ub, G);
    k_need_second_pass<<<1, 1, 0, d.st>>>(G0, G, d.nsd, skip);
    gram(d, d.U, b * d.nsd, Ub, cbuf, skip);
    lincomb(d, b * d.nsd, cbuf, 1, d.U, Ub, nullptr, nullptr, nullptr, nullptr, skip);
  }
  for (int pass = 0; pass < 2; ++pass) {
    gram(d, Ub, d.nsd, Ub, G);
    k_chol_inv<<<1, 1, 0, d.st>>>(G, d.nsd, Rinv);
    lincomb(d, d.nsd, Rinv, 0, Ub, Ub);
  }
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
      (prm->precision != QPGPU_FP64 && prm->precision != QPGPU_FP32))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad Davidson parameters (1 <= n_states <= n_states_diag <= 8)");
  if ((int64_t)nsd * 3 > N) return qpgpu_fail(c, QPGPU_ERR_ARG, "N_st_diag*3 > sze (diagonalization_hs2.irp.f:110)");
  int itermax = std::max(3, (int)std::min<int64_t>(prm->davidson_sze_max, N / nsd));
  while (itermax * nsd > MAXM) --itermax;
  const bool mixed = prm->precision == QPGPU_FP32;
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
  d.ncta = 2 * 152;
  d.rows_per_cta = (N + d.ncta - 1) / d.ncta;
  const size_t blkn = (size_t)N * nsd;
  if (dev_alloc(&d.U, blkn * itermax) != cudaSuccess || dev_alloc(&d.W, blkn * itermax) != cudaSuccess ||
      dev_alloc(&d.S, blkn * itermax) != cudaSuccess || dev_alloc(&d.R, blkn) != cudaSuccess ||
      dev_alloc(&d.u32, blkn) != cudaSuccess || dev_alloc(&d.part, (size_t)d.ncta * MAXM * MAXS) != cudaSuccess ||
      dev_alloc(&d.small, (size_t)6 * MAXM * MAXS) != cudaSuccess) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "Davidson work arrays do not fit on the device");
  }
  cudaStream_t st = d.st;
  // learned preconditioner and training capture
  const bool use_mlp = prm->preconditioner == 1;
  if (use_mlp && (!c->mlp.ready || !c->d_detfeat))
    return qpgpu_fail(c, QPGPU_ERR_STATE, "learned preconditioner requested but the MLP is not initialised");
  bool mlp_on[MAXS] = {false};
  int strikes[MAXS] = {0};
  double prev_res[MAXS];
  for (int k = 0; k < MAXS; ++k) prev_res[k] = INFINITY;
  for (int k = 0; k < nst; ++k) mlp_on[k] = use_mlp;
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
    qp_to_bilinear(hstage, N, c->d_order, d.U, nullptr, nsd, N, st);
    QP_CUDA(c, cudaStreamSynchronize(st));
    cudaFree(hstage);
  }
  const double Sz = 0.5 * (c->na - c->nb);
  const double sz2sz = Sz * (Sz - 1.0), expected_s2 = Sz * (Sz + 1.0);
  const int mmax = itermax * nsd;
  std::vector<double> h((size_t)mmax * mmax, 0.0), s_((size_t)mmax * mmax, 0.0);
  std::vector<double> hcol((size_t)mmax * nsd), scol((size_t)mmax * nsd);
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
      orthonormalise(d, b);
      prof.mark(DavProf::ORTHO);
      // sigma on block b
      const int prec = (mixed && iter > 1) ? QPGPU_FP32 : QPGPU_FP64;
      if (prec == QPGPU_FP32) qp_to_float(d.blk(d.U, b), d.u32, (int64_t)blkn, st);
      int rc = qp_sigma_launch(c, &c->items, d.blk(d.W, b), d.blk(d.S, b), d.blk(d.U, b), d.u32, nsd, prec, st, 0,
                               (int)N, 0, 1);
      if (rc) return rc;
      ++n_sigma;
      prof.mark(DavProf::SIGMA);
      // new Gram columns
      gram(d, d.U, shift2, d.blk(d.W, b), d.small);
      gram(d, d.U, shift2, d.blk(d.S, b), d.small + MAXM * MAXS);
      QP_CUDA(c, cudaMemcpyAsync(hcol.data(), d.small, (size_t)shift2 * nsd * sizeof(double), cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaMemcpyAsync(scol.data(), d.small + MAXM * MAXS, (size_t)shift2 * nsd * sizeof(double),
                                 cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaStreamSynchronize(st));
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
      qp_jacobi(hs, shift2, wv, y);
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
      // Ritz vectors into block b+1 (:376-381); coefficients y(0:shift2, 0:nsd)
      std::vector<double> ycoef((size_t)shift2 * nsd);
      for (int i = 0; i < shift2; ++i)
        for (int j = 0; j < nsd; ++j) ycoef[(size_t)i * nsd + j] = y[(size_t)i * shift2 + j];
      double* ydev = d.small + 3 * MAXM * MAXS;
      prof.mark(DavProf::HOST);
      QP_CUDA(c, cudaMemcpyAsync(ydev, ycoef.data(), ycoef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      lincomb(d, shift2, ydev, 0, d.U, d.blk(d.U, iter), d.W, d.blk(d.W, iter), d.S, d.blk(d.S, iter));
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
        k_capture<<<gsz(N), DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), c->d_hdiag,
                                           (const float4*)c->d_detfeat, N, sp, n_cap * nst, d.cX, d.cd, d.cc);
        ++n_cap;
      }
      unsigned mask = 0;
      for (int k = 0; k < nst; ++k)
        if (mlp_on[k]) mask |= 1u << k;
      if (mask)
        k_step_mlp<<<d.ncta, DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), c->d_hdiag,
                                            (const float4*)c->d_detfeat, c->mlp.params, N, sp, mask, d.part);
      else
        k_step<<<d.ncta, DBLK, 0, st>>>(d.blk(d.U, iter), d.blk(d.W, iter), d.blk(d.S, iter), c->d_hdiag, N, sp, d.part);
      QP_CUDA(c, cudaGetLastError());
      QP_CUDA(c, cudaMemcpyAsync(partial.data(), d.part, partial.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
      QP_CUDA(c, cudaStreamSynchronize(st));
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
      // diagonal correction) fell by less than 5% in two consecutive learned
      // steps goes back to the diagonal step for the rest of the run
      for (int k = 0; k < nst; ++k) {
        if (mlp_on[k]) {
          strikes[k] = (res[k] > 0.95 * prev_res[k]) ? strikes[k] + 1 : 0;
          if (strikes[k] >= 2) {
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
      if (below && prec == QPGPU_FP64 && (iter >= 2 || mixed)) {
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
    double* ydev = d.small + 3 * MAXM * MAXS;
    QP_CUDA(c, cudaMemcpyAsync(ydev, ycoef.data(), ycoef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    lincomb(d, shift2, ydev, 0, d.U, d.R);
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
