// Sigma application v = H u, s = S^2 u over the stored connected pairs.
//
// The reference computes every matrix element again at each call
// (src/Davidson/u0Hu0.irp.f:177-444); here they are built once per
// determinant set and sigma is a row-owner gather: each row is owned by one
// warp (rows longer than CHUNK pairs are split over several warps whose
// partial sums are added in a fixed order), so there are no atomics and the
// result is deterministic.  u is laid out (N_det, N_st) with states fastest,
// as u_t(N_st, N_det) in the reference (:27-41), so the N_st coefficients of a
// connected determinant J are one contiguous load.
#include <algorithm>
#include <cstdio>

#include "qpgpu_internal.cuh"
#include "sigma_device.cuh"

namespace {

constexpr int SBLK = 256;

struct SigArgs {
  int64_t N;
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
  int64_t n_items;
  const double* u;   // (N, NST) FP64
  const float* u32;  // (N, u32_ld) FP32 (precision FP32): rows u32_ld floats apart
  int u32_ld;
  const float* u32lo;   // precision FF: low parts of u, same layout as u32 (the high parts)
  const float* val32lo; // precision FF: low parts of the stored elements (val32 = high parts)
  double* v;
  double* s;
  double* pv;  // partial sums (n_items, NST)
  double* ps;
  int row_lo, row_hi;  // rows [row_lo, row_hi) are written (range variant)
  int row_step, row_first;
};

__device__ __forceinline__ bool row_selected(const SigArgs& a, int k) {
  if (k < a.row_lo || k >= a.row_hi) return false;
  return ((k - a.row_first) % a.row_step) == 0;
}

using namespace qpsig;

// write the reduced state sums (lane L holds state L >> shift) and the diagonal
template <int NST>
__device__ __forceinline__ void store_row(const SigArgs& a, int64_t it, int k, int lane, double hv, double sv,
                                          bool has_s2) {
  constexpr int SH = 5 - Pow2<NST>::lg;
  const int st = lane >> SH;
  const bool owner = (lane & ((1 << SH) - 1)) == 0 && st < NST;
  if (!owner) return;
  if (a.row_nitems[k] == 1) {
    const double uk = a.u[(int64_t)k * NST + st];
    a.v[(int64_t)k * NST + st] = hv + a.hdiag[k] * uk;
    a.s[(int64_t)k * NST + st] = (has_s2 ? sv : 0.0) + a.sdiag[k] * uk;
  } else {
    a.pv[it * NST + st] = hv;
    a.ps[it * NST + st] = has_s2 ? sv : 0.0;
  }
}



constexpr int UNR = 2;    // FP64 sigma: pairs per lane per loop trip (FP64-pipe bound)
constexpr int UNR32 = 4;  // FP32 sigma: more independent loads in flight (latency bound)

template <int NST>
__global__ void __launch_bounds__(SBLK) k_sigma64(SigArgs a) {
  constexpr int NP = Pow2<NST>::v;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * SBLK + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * SBLK) >> 5;
  for (int64_t it = warp; it < a.n_items; it += nwarp) {
    const int k = a.item_row[it];
    if (!row_selected(a, k)) continue;
    const int j = a.item_sub[it];
    const int64_t rb = a.rowptr[k], re = a.rowptr[k + 1];
    const int64_t beg = rb + (int64_t)j * QP_SIGMA_CHUNK;
    const int64_t end = min(beg + (int64_t)QP_SIGMA_CHUNK, re);
    double acc[NP];
#pragma unroll
    for (int st = 0; st < NP; ++st) acc[st] = 0.0;
    for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * UNR) {
      int col[UNR];
      double hv[UNR];
#pragma unroll
      for (int q = 0; q < UNR; ++q) {
        const int64_t e = e0 + 32 * q;
        col[q] = e < end ? __ldg(&a.colidx[e]) : k;
        hv[q] = e < end ? __ldg(&a.val64[e]) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < UNR; ++q) {
        double x[NST];
        load_row<NST>(a.u, col[q], x);
#pragma unroll
        for (int st = 0; st < NST; ++st) acc[st] = fma(hv[q], x[st], acc[st]);
      }
    }
    const double hsum = reduce_scatter64<NP>(acc, lane);
    double ssum = 0.0;
    const int64_t sb = a.s2ptr[k], se = a.s2ptr[k + 1];
    const bool has_s2 = (j == 0) && (se > sb);
    if (has_s2) {
      double sacc[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) sacc[st] = 0.0;
      for (int64_t e = sb + lane; e < se; e += 32) {
        const double sv = (double)__ldg(&a.s2val[e]);
        double x[NST];
        load_row<NST>(a.u, __ldg(&a.s2col[e]), x);
#pragma unroll
        for (int st = 0; st < NST; ++st) sacc[st] = fma(sv, x[st], sacc[st]);
      }
      ssum = reduce_scatter64<NP>(sacc, lane);
    }
    store_row<NST>(a, it, k, lane, hsum, ssum, has_s2);
  }
}

// (column, value) pairs of one trip: lane's pairs e0, e0+32, ...; past the
// end of the chunk the row's own column with value 0 (a harmless gather)
__device__ __forceinline__ void load_trip32(const SigArgs& a, int64_t e0, int64_t end, int k, int (&col)[UNR32],
                                            float (&hv)[UNR32]) {
#pragma unroll
  for (int q = 0; q < UNR32; ++q) {
    const int64_t e = e0 + 32 * q;
    col[q] = e < end ? __ldg(&a.colidx[e]) : k;
    hv[q] = e < end ? __ldg(&a.val32[e]) : 0.f;
  }
}

// Kahan-compensated sum += hv * u32[col] for the trip's pairs
template <int NST, int NP, int LD, bool V8>
__device__ __forceinline__ void accumulate32(const SigArgs& a, const int (&col)[UNR32], const float (&hv)[UNR32],
                                             float (&sum)[NP], float (&cmp)[NP]) {
#pragma unroll
  for (int q = 0; q < UNR32; ++q) {
    float x[NST];
    load_row_ld<NST, LD, V8>(a.u32, col[q], x);
#pragma unroll
    for (int st = 0; st < NST; ++st) {
      const float y = __fmaf_rn(hv[q], x[st], -cmp[st]);
      const float t = __fadd_rn(sum[st], y);
      cmp[st] = __fsub_rn(__fsub_rn(t, sum[st]), y);
      sum[st] = t;
    }
  }
}

// FP32 matrix elements x FP32 coefficients with Kahan-compensated lane sums;
// lanes are combined as float-float pairs, and only the owner lane of each
// state converts to FP64 and adds the FP64 diagonal term.
//
// The kernel is bound by load latency (each coefficient gather waits on its
// column index).  With PIPE the next trip's (column, value) pairs are loaded
// one trip ahead of the current trip's gathers, at the price of registers,
// hence occupancy; which launch shape hides the latency best depends on the
// row lengths, so it is chosen by timing (tune_sigma32).  Every shape gives
// bit-identical sums: each lane sees the same pairs in the same order.
template <int NST, bool PIPE, int BS, int LD, bool V8>
__global__ void __launch_bounds__(BS) k_sigma32(SigArgs a) {
  constexpr int NP = Pow2<NST>::v;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * BS + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * BS) >> 5;
  for (int64_t it = warp; it < a.n_items; it += nwarp) {
    const int k = a.item_row[it];
    if (!row_selected(a, k)) continue;
    const int j = a.item_sub[it];
    const int64_t rb = a.rowptr[k], re = a.rowptr[k + 1];
    const int64_t beg = rb + (int64_t)j * QP_SIGMA_CHUNK;
    const int64_t end = min(beg + (int64_t)QP_SIGMA_CHUNK, re);
    float sum[NP], cmp[NP];
#pragma unroll
    for (int st = 0; st < NP; ++st) sum[st] = cmp[st] = 0.f;
    int col[UNR32];
    float hv[UNR32];
    if (PIPE) load_trip32(a, beg + lane, end, k, col, hv);
    for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * UNR32) {
      if (PIPE) {
        int ncol[UNR32];
        float nhv[UNR32];
        load_trip32(a, e0 + 32 * UNR32, end, k, ncol, nhv);
        accumulate32<NST, NP, LD, V8>(a, col, hv, sum, cmp);
#pragma unroll
        for (int q = 0; q < UNR32; ++q) {
          col[q] = ncol[q];
          hv[q] = nhv[q];
        }
        continue;
      }
      load_trip32(a, e0, end, k, col, hv);
#pragma unroll
      for (int q = 0; q < UNR32; ++q) {
        float x[NST];
        load_row_ld<NST, LD, V8>(a.u32, col[q], x);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          const float y = __fmaf_rn(hv[q], x[st], -cmp[st]);
          const float t = __fadd_rn(sum[st], y);
          cmp[st] = __fsub_rn(__fsub_rn(t, sum[st]), y);
          sum[st] = t;
        }
      }
    }
    // Kahan state (sum, -cmp) is a float-float value
#pragma unroll
    for (int st = 0; st < NP; ++st) cmp[st] = -cmp[st];
    float rh, rl;
    reduce_scatter_ff<NP>(sum, cmp, lane, rh, rl);
    const double hsum = (double)rh + (double)rl;
    double ssum = 0.0;
    const int64_t sb = a.s2ptr[k], se = a.s2ptr[k + 1];
    const bool has_s2 = (j == 0) && (se > sb);
    if (has_s2) {
      float sh[NP], sl[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) sh[st] = sl[st] = 0.f;
      for (int64_t e = sb + lane; e < se; e += 32) {
        const float sv = __ldg(&a.s2val[e]);  // +-1: products are exact
        float x[NST];
        load_row_ld<NST, LD, V8>(a.u32, __ldg(&a.s2col[e]), x);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          float s, err;
          two_sum(sh[st], sv * x[st], s, err);
          sh[st] = s;
          sl[st] = __fadd_rn(sl[st], err);
        }
      }
      float qh, ql;
      reduce_scatter_ff<NP>(sh, sl, lane, qh, ql);
      ssum = (double)qh + (double)ql;
    }
    store_row<NST>(a, it, k, lane, hsum, ssum, has_s2);
  }
}

// rows split over several items: add the partials in item order
__global__ void k_sigma_combine(SigArgs a, const int* multi_rows, const int* row_item0, int n_multi, int nst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n_multi * nst;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = multi_rows[t / nst];
    const int st = (int)(t % nst);
    if (!row_selected(a, k)) continue;
    const int i0 = row_item0[k], ni = a.row_nitems[k];
    double av = 0.0, as = 0.0;
    for (int i = 0; i < ni; ++i) {
      av += a.pv[(int64_t)(i0 + i) * nst + st];
      as += a.ps[(int64_t)(i0 + i) * nst + st];
    }
    const double uk = a.u[(int64_t)k * nst + st];
    a.v[(int64_t)k * nst + st] = av + a.hdiag[k] * uk;
    a.s[(int64_t)k * nst + st] = as + a.sdiag[k] * uk;
  }
}

// ---- work items -----------------------------------------------------------
__global__ void k_row_nitems(const int64_t* rowptr, int* nit, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t nnz = rowptr[k + 1] - rowptr[k];
    nit[k] = (int)max((int64_t)1, (nnz + QP_SIGMA_CHUNK - 1) / QP_SIGMA_CHUNK);
  }
}

__global__ void k_fill_items(const int* nit, const int* item0, int* item_row, int* item_sub, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x)
    for (int j = 0; j < nit[k]; ++j) {
      item_row[item0[k] + j] = (int)k;
      item_sub[item0[k] + j] = j;
    }
}

// bad (optional): set to 1 when an input coefficient is NaN or infinite
template <class T>
__global__ void k_to_bilinear(const T* u0, int64_t ld, const int* order, double* ut, float* ut32, int nst,
                              int64_t N, int* bad) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * nst; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / nst;
    const int st = (int)(t % nst);
    const double x = (double)u0[(int64_t)st * ld + order[p]];
    if (bad && !isfinite(x)) *bad = 1;
    if (ut) ut[t] = x;
    if (ut32) ut32[t] = (float)x;
  }
}

__global__ void k_nonfinite(const double* x, int64_t n, int* bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(x[i])) *bad = 1;
}

__global__ void k_from_bilinear(const double* vt, int64_t ld, const int* order, double* v0, int nst, int64_t N) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * nst; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / nst;
    const int st = (int)(t % nst);
    v0[(int64_t)st * ld + order[p]] = vt[t];
  }
}

// y (N rows of ld floats) <- x (N rows of nst doubles)
// lo = val64 - val32 rounded to FP32 (the low parts of the stored elements)
__global__ void k_lo_parts(const double* v64, const float* v32, float* lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    lo[i] = (float)(v64[i] - (double)v32[i]);
}

// (hi, lo) rows of ld floats <- x (N rows of nst doubles), integer split
__global__ void k_split_rows(const double* x, float* hi, float* lo, int64_t N, int nst, int ld) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * nst; i += (int64_t)gridDim.x * blockDim.x) {
    float h, l;
    split_ff(x[i], h, l);
    const int64_t o = (i / nst) * ld + i % nst;
    hi[o] = h;
    lo[o] = l;
  }
}

__global__ void k_to_float(const double* x, float* y, int64_t N, int nst, int ld) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * nst; i += (int64_t)gridDim.x * blockDim.x)
    y[(i / nst) * ld + i % nst] = (float)x[i];
}

inline unsigned gsz(int64_t n, int tpb) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 32) g = 65535LL * 32;
  return (unsigned)g;
}

// FP32 launch shapes tried by the tuner: kernel variant, CTA size and grid
// policy (0: one warp per work item; n: a persistent grid of n CTAs per SM)
struct Sig32Shape {
  bool pipe;
  int bs, ctas_per_sm;
};
constexpr Sig32Shape kSig32Shapes[] = {{false, 256, 0}, {false, 128, 0}, {false, 64, 0}, {true, 256, 0}};
constexpr int kNSig32Shapes = sizeof(kSig32Shapes) / sizeof(kSig32Shapes[0]);

template <int NST, int LD, bool V8>
void launch_sigma32_ld(const SigArgs& a, int variant, cudaStream_t st, int n_sm) {
  const Sig32Shape sh = kSig32Shapes[variant];
  int64_t g = (a.n_items * 32 + sh.bs - 1) / sh.bs;
  if (sh.ctas_per_sm) g = std::min<int64_t>(g, (int64_t)sh.ctas_per_sm * n_sm);
  g = std::max<int64_t>(1, std::min<int64_t>(g, 65535LL * 32));
  const unsigned grid = (unsigned)g;
  switch (variant) {
    case 1: k_sigma32<NST, false, 128, LD, V8><<<grid, 128, 0, st>>>(a); break;
    case 2: k_sigma32<NST, false, 64, LD, V8><<<grid, 64, 0, st>>>(a); break;
    case 3: k_sigma32<NST, true, 256, LD, V8><<<grid, 256, 0, st>>>(a); break;
    default: k_sigma32<NST, false, 256, LD, V8><<<grid, 256, 0, st>>>(a); break;
  }
}

// dense rows (u32_ld == NST) or rows padded to 4 / 8 floats; rows of 8 floats
// on a 32-byte aligned array are read with one 256-bit load each
template <int NST>
void launch_sigma32(const SigArgs& a, int variant, cudaStream_t st, int n_sm) {
  constexpr int P = Pow2<NST>::v;
  const bool a32 = ((uintptr_t)a.u32 & 31) == 0;
  if constexpr (P == 8) {
    if (a.u32_ld == 8 && a32) {
      launch_sigma32_ld<NST, 8, true>(a, variant, st, n_sm);
      return;
    }
    if constexpr (NST == 8) {
      k_sigma32<8, false, 256, 8, false><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(
                                               (a.n_items * 32 + 255) / 256, 65535LL * 32)),
                                           256, 0, st>>>(a);
      return;
    }
  }
  if constexpr (P != NST && P == 4) {
    if (a.u32_ld == 4) {
      launch_sigma32_ld<NST, 4, false>(a, variant, st, n_sm);
      return;
    }
  }
  if constexpr (NST != 8) launch_sigma32_ld<NST, NST, false>(a, variant, st, n_sm);
}

// Float-float sigma: elements h = vh + vl and coefficients u = uh + ul as
// FP32 pairs (rows padded to LD floats, 32-byte aligned; LD = 8 uses one
// 256-bit load per part).  Per pair and state the product is formed exactly
// for vh*uh (FMA gives its rounding error) plus the cross terms, and each
// lane keeps its sum as an unevaluated float pair updated with Knuth's
// TwoSum; lanes are combined with reduce_scatter_ff.  About 1e-13 relative,
// FP32 pipes only, except the FP64 diagonal term of the owner lanes.
template <int NST, int LD>
__global__ void __launch_bounds__(128) k_sigma_ff(SigArgs a) {
  constexpr int NP = Pow2<NST>::v;
  constexpr int UNRF = 2;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * 128 + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * 128) >> 5;
  for (int64_t it = warp; it < a.n_items; it += nwarp) {
    const int k = a.item_row[it];
    if (!row_selected(a, k)) continue;
    const int j = a.item_sub[it];
    const int64_t rb = a.rowptr[k], re = a.rowptr[k + 1];
    const int64_t beg = rb + (int64_t)j * QP_SIGMA_CHUNK;
    const int64_t end = min(beg + (int64_t)QP_SIGMA_CHUNK, re);
    float ah[NP], al[NP];
#pragma unroll
    for (int st = 0; st < NP; ++st) ah[st] = al[st] = 0.f;
    for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * UNRF) {
      int col[UNRF];
      float vh[UNRF], vl[UNRF];
#pragma unroll
      for (int q = 0; q < UNRF; ++q) {
        const int64_t e = e0 + 32 * q;
        col[q] = e < end ? __ldg(&a.colidx[e]) : k;
        vh[q] = e < end ? __ldg(&a.val32[e]) : 0.f;
        vl[q] = e < end ? __ldg(&a.val32lo[e]) : 0.f;
      }
#pragma unroll
      for (int q = 0; q < UNRF; ++q) {
        float xh[NST], xl[NST];
        load_row_ld<NST, LD, LD == 8>(a.u32, col[q], xh);
        load_row_ld<NST, LD, LD == 8>(a.u32lo, col[q], xl);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          const float p = __fmul_rn(vh[q], xh[st]);
          float pe = __fmaf_rn(vh[q], xh[st], -p);
          pe = __fmaf_rn(vh[q], xl[st], pe);
          pe = __fmaf_rn(vl[q], xh[st], pe);
          float t, err;
          two_sum(ah[st], p, t, err);
          ah[st] = t;
          al[st] = __fadd_rn(al[st], __fadd_rn(err, pe));
        }
      }
    }
    float rh, rl;
    reduce_scatter_ff<NP>(ah, al, lane, rh, rl);
    const double hsum = (double)rh + (double)rl;
    double ssum = 0.0;
    const int64_t sb = a.s2ptr[k], se = a.s2ptr[k + 1];
    const bool has_s2 = (j == 0) && (se > sb);
    if (has_s2) {
      float sh[NP], sl[NP];
#pragma unroll
      for (int st = 0; st < NP; ++st) sh[st] = sl[st] = 0.f;
      for (int64_t e = sb + lane; e < se; e += 32) {
        const float sv = __ldg(&a.s2val[e]);  // +-1: the products are exact
        const int cj = __ldg(&a.s2col[e]);
        float xh[NST], xl[NST];
        load_row_ld<NST, LD, LD == 8>(a.u32, cj, xh);
        load_row_ld<NST, LD, LD == 8>(a.u32lo, cj, xl);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          float t, err;
          two_sum(sh[st], sv * xh[st], t, err);
          sh[st] = t;
          sl[st] = __fadd_rn(sl[st], __fadd_rn(err, sv * xl[st]));
        }
      }
      float qh, ql;
      reduce_scatter_ff<NP>(sh, sl, lane, qh, ql);
      ssum = (double)qh + (double)ql;
    }
    store_row<NST>(a, it, k, lane, hsum, ssum, has_s2);
  }
}

template <int NST>
void launch_sigma(const SigArgs& a, int precision, unsigned grid, cudaStream_t st, int n_sm, int variant) {
  constexpr int P = Pow2<NST>::v;
  if (precision == QPGPU_FF) {
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((a.n_items * 32 + 127) / 128, 65535LL * 32));
    k_sigma_ff<NST, P><<<g, 128, 0, st>>>(a);
  } else if (precision == QPGPU_FP32)
    launch_sigma32<NST>(a, variant < 0 ? 0 : variant, st, n_sm);
  else
    k_sigma64<NST><<<grid, SBLK, 0, st>>>(a);
}

void launch_any(const SigArgs& a, int nst, int precision, unsigned grid, cudaStream_t st, int n_sm, int variant) {
  switch (nst) {
    case 1: launch_sigma<1>(a, precision, grid, st, n_sm, variant); break;
    case 2: launch_sigma<2>(a, precision, grid, st, n_sm, variant); break;
    case 3: launch_sigma<3>(a, precision, grid, st, n_sm, variant); break;
    case 4: launch_sigma<4>(a, precision, grid, st, n_sm, variant); break;
    case 5: launch_sigma<5>(a, precision, grid, st, n_sm, variant); break;
    case 6: launch_sigma<6>(a, precision, grid, st, n_sm, variant); break;
    case 7: launch_sigma<7>(a, precision, grid, st, n_sm, variant); break;
    default: launch_sigma<8>(a, precision, grid, st, n_sm, variant); break;
  }
}

// Times every FP32 launch shape on this determinant set (two launches each,
// the second timed with events on the caller's stream) and keeps the fastest
// for n_st.  Runs once per determinant set and n_st, on the first FP32 call;
// the outputs it writes are those of the call itself.
int tune_sigma32(qpgpu_ctx* c, SigmaItems* it, const SigArgs& a, int nst, cudaStream_t st, int slot) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return qpgpu_fail(c, QPGPU_ERR_CUDA, "cudaEventCreate failed while tuning the FP32 sigma");
  }
  int best = 0;
  float best_ms = 1e30f;
  for (int v = 0; v < kNSig32Shapes; ++v) {
    launch_any(a, nst, QPGPU_FP32, 1, st, c->n_sm, v);
    cudaEventRecord(e0, st);
    launch_any(a, nst, QPGPU_FP32, 1, st, c->n_sm, v);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (c->profile) fprintf(stderr, "[qpgpu] sigma32 n_st=%d row=%d floats shape %d: %.3f ms\n", nst, a.u32_ld, v, ms);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QP_CUDA(c, cudaGetLastError());
  it->sig32_variant[slot] = best;
  return 0;
}

}  // namespace

// Work items of the sigma kernels (one per chunk of a row), built after the pairs.
int qp_build_sigma_items(qpgpu_ctx* c, SigmaItems* it) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  it->free_all();
  QP_CUDA(c, dev_alloc(&it->row_nitems, N + 1));
  QP_CUDA(c, dev_alloc(&it->row_item0, N + 1));
  k_row_nitems<<<gsz(N, 256), 256, 0, st>>>(c->d_rowptr, it->row_nitems, N);
  QP_CUDA(c, cudaMemsetAsync(it->row_nitems + N, 0, sizeof(int), st));
  std::vector<int> nit(N);
  QP_CUDA(c, cudaMemcpyAsync(nit.data(), it->row_nitems, N * sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  std::vector<int> item0(N + 1);
  std::vector<int> multi;
  int64_t acc = 0;
  for (int64_t k = 0; k < N; ++k) {
    item0[k] = (int)acc;
    acc += nit[k];
    if (nit[k] > 1) multi.push_back((int)k);
  }
  item0[N] = (int)acc;
  it->n_items = acc;
  it->n_multi = (int)multi.size();
  QP_CUDA(c, cudaMemcpyAsync(it->row_item0, item0.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, dev_alloc(&it->item_row, acc));
  QP_CUDA(c, dev_alloc(&it->item_sub, acc));
  QP_CUDA(c, dev_alloc(&it->multi_rows, multi.size() + 1));
  if (!multi.empty())
    QP_CUDA(c, cudaMemcpyAsync(it->multi_rows, multi.data(), multi.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  k_fill_items<<<gsz(N, 256), 256, 0, st>>>(it->row_nitems, it->row_item0, it->item_row, it->item_sub, N);
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaStreamSynchronize(st));
  return 0;
}

// Partial-sum buffers sized for nst states.
static int ensure_partials(qpgpu_ctx* c, SigmaItems* it, int nst) {
  const size_t need = (size_t)it->n_items * nst;
  if (it->partial_cap >= need) return 0;
  dev_free(it->pv);
  dev_free(it->ps);
  it->pv = it->ps = nullptr;
  it->partial_cap = 0;
  QP_CUDA(c, dev_alloc(&it->pv, need));
  QP_CUDA(c, dev_alloc(&it->ps, need));
  it->partial_cap = need;
  return 0;
}

int qp_sigma_launch(qpgpu_ctx* c, SigmaItems* it, double* v, double* s, const double* u, const float* u32, int nst,
                    int precision, cudaStream_t st, int row_lo, int row_hi, int row_first, int row_step,
                    int u32_ld, const float* u32lo) {
  if (nst < 1 || nst > 8) return qpgpu_fail(c, QPGPU_ERR_ARG, "n_st must be in 1..8 per sigma block");
  if (c->direct) return qp_sigma_direct(c, v, s, u, nst, st, row_lo, row_hi, row_first, row_step);
  if (u32_ld <= 0) u32_ld = nst;
  if (u32_ld != nst && !(u32_ld == qp_pad_states(nst) && (((uintptr_t)u32) & 31) == 0))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "FP32 rows must be n_st floats apart, or padded to 4/8 and 32-byte aligned");
  if (precision == QPGPU_FP32 && !u32) return qpgpu_fail(c, QPGPU_ERR_ARG, "FP32 sigma needs u_t32");
  int rc = ensure_partials(c, it, nst);
  if (rc) return rc;
  SigArgs a{};
  a.N = c->N;
  a.rowptr = c->d_rowptr;
  a.colidx = c->d_colidx;
  a.val64 = c->d_val64;
  a.val32 = c->d_val32;
  a.s2ptr = c->d_s2ptr;
  a.s2col = c->d_s2col;
  a.s2val = c->d_s2val;
  a.hdiag = c->d_hdiag;
  a.sdiag = c->d_sdiag;
  a.item_row = it->item_row;
  a.item_sub = it->item_sub;
  a.row_nitems = it->row_nitems;
  a.n_items = it->n_items;
  a.u = u;
  a.u32 = u32;
  a.u32_ld = u32_ld;
  a.u32lo = u32lo;
  a.val32lo = c->d_val32lo;
  if (precision == QPGPU_FF && (!u32lo || !c->d_val32lo || u32_ld != qp_pad_states(nst)))
    return qpgpu_fail(c, QPGPU_ERR_STATE, "float-float sigma needs split coefficients and elements");
  a.v = v;
  a.s = s;
  a.pv = it->pv;
  a.ps = it->ps;
  a.row_lo = row_lo;
  a.row_hi = row_hi;
  a.row_first = row_first;
  a.row_step = row_step;
  const unsigned grid = gsz(it->n_items * 32, SBLK);
  const int slot = nst + (u32_ld != nst ? 9 : 0);
  if (precision == QPGPU_FP32 && it->sig32_variant[slot] < 0) {
    rc = tune_sigma32(c, it, a, nst, st, slot);
    if (rc) return rc;
  }
  launch_any(a, nst, precision, grid, st, c->n_sm, it->sig32_variant[slot]);
  if (it->n_multi > 0)
    k_sigma_combine<<<gsz((int64_t)it->n_multi * nst, 256), 256, 0, st>>>(a, it->multi_rows, it->row_item0,
                                                                         it->n_multi, nst);
  QP_CUDA(c, cudaGetLastError());
  return 0;
}

void qp_to_bilinear(const double* u0, int64_t ld, const int* order, double* ut, float* ut32, int nst, int64_t N,
                    cudaStream_t st, int* bad) {
  k_to_bilinear<double><<<gsz(N * nst, 256), 256, 0, st>>>(u0, ld, order, ut, ut32, nst, N, bad);
}

void qp_flag_nonfinite(const double* x, int64_t n, int* bad, cudaStream_t st) {
  k_nonfinite<<<gsz(n, 256), 256, 0, st>>>(x, n, bad);
}

void qp_from_bilinear(const double* vt, int64_t ld, const int* order, double* v0, int nst, int64_t N,
                      cudaStream_t st) {
  k_from_bilinear<<<gsz(N * nst, 256), 256, 0, st>>>(vt, ld, order, v0, nst, N);
}

int qp_sigma_ff(qpgpu_ctx* c, SigmaItems* it, double* v, double* s, const double* u, int nst, cudaStream_t st,
                int row_lo, int row_hi, int row_first, int row_step) {
  if (nst < 1 || nst > 8) return qpgpu_fail(c, QPGPU_ERR_ARG, "n_st must be in 1..8 per sigma block");
  if (c->direct) return qp_sigma_direct(c, v, s, u, nst, st, row_lo, row_hi, row_first, row_step);
  const int64_t N = c->N;
  if (!c->d_val32lo) {  // once per determinant set
    QP_CUDA(c, dev_alloc(&c->d_val32lo, c->P));
    k_lo_parts<<<gsz(c->P, 256), 256, 0, st>>>(c->d_val64, c->d_val32, c->d_val32lo, c->P);
  }
  const int ld = qp_pad_states(nst);
  const size_t half = ((size_t)N * ld + 63) / 64 * 64;  // keeps lo 256-byte aligned
  if (c->ffu_floats < 2 * half) {
    dev_free(c->d_ffu);
    c->d_ffu = nullptr;
    c->ffu_floats = 0;
    QP_CUDA(c, dev_alloc(&c->d_ffu, 2 * half));
    c->ffu_floats = 2 * half;
  }
  float* hi = c->d_ffu;
  float* lo = c->d_ffu + half;
  k_split_rows<<<gsz(N * nst, 256), 256, 0, st>>>(u, hi, lo, N, nst, ld);
  return qp_sigma_launch(c, it, v, s, u, hi, nst, QPGPU_FF, st, row_lo, row_hi, row_first, row_step, ld, lo);
}

void qp_to_float(const double* x, float* y, int64_t N, int nst, int ld, cudaStream_t st) {
  k_to_float<<<gsz(N * nst, 256), 256, 0, st>>>(x, y, N, nst, ld);
}

// ---------------------------------------------------------------------------
// Sigma without device allocation.
//
// qpgpu_sigma_bilinear keeps its per-chunk partial sums (rows whose pairs span
// several work chunks) in a buffer that it grows with cudaMalloc on first use.
// Some callers cannot let a library call cudaMalloc: a host code whose device
// memory is owned by its own pool allocator (cudaMalloc fails or fragments the
// pool), or a worker that overlaps sigma with copies and communication on
// other streams, where cudaMalloc/cudaFree would synchronise the device.  For
// them the scratch lives in a fixed device array below, of
// QP_NOALLOC_SLOTS doubles for each of the two sums (8 MiB in total), which
// every GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------
#define QP_NOALLOC_SLOTS (1 << 19)
static __device__ __align__(256) double g_noalloc_partials[2 * QP_NOALLOC_SLOTS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};  // device address of the array, per device
}  // namespace

extern "C" int qpgpu_sigma_bilinear_noalloc(qpgpu_ctx* c, double* v_t, double* s_t, const double* u_t,
                                            const float* u_t32, int n_st, int precision, void* stream) {
  if (!c) return QPGPU_ERR_ARG;
  if (!c->have_ints || !c->have_pairs) return qpgpu_fail(c, QPGPU_ERR_STATE, "determinants not set");
  if (c->direct) return qpgpu_fail(c, QPGPU_ERR_STATE, "the no-alloc sigma needs stored pairs (direct sigma set)");
  if (!v_t || !s_t || !u_t || n_st < 1 || n_st > 8 || (precision != QPGPU_FP64 && precision != QPGPU_FP32) ||
      (precision == QPGPU_FP32 && !u_t32))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad sigma arguments (n_st must be 1..8)");
  if (((uintptr_t)u_t & 15) || (u_t32 && ((uintptr_t)u_t32 & 15)))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "u_t and u_t32 must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(c->mu);
  const SigmaItems* it = &c->items;
  if (it->n_items * (int64_t)n_st > (int64_t)QP_NOALLOC_SLOTS)
    return qpgpu_fail(c, QPGPU_ERR_ARG,
                      "no-alloc sigma: work chunks x n_st exceeds the fixed scratch of 524288 slots");
  // device address of the scratch array on this context's device, looked up
  // once per device (in host code the array's name is not a device address)
  if (c->device < 0 || c->device >= kMaxDevices) return qpgpu_fail(c, QPGPU_ERR_ARG, "device ordinal too large");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[c->device]) {
      int cur = -1;
      if (cudaGetDevice(&cur) != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, "cudaGetDevice failed");
      if (cur != c->device && cudaSetDevice(c->device) != cudaSuccess)
        return qpgpu_fail(c, QPGPU_ERR_CUDA, "cudaSetDevice failed");
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (cur != c->device) cudaSetDevice(cur);
      if (e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, "cudaGetSymbolAddress of the sigma scratch failed");
      g_noalloc_ptr[c->device] = (double*)p;
    }
    scratch = g_noalloc_ptr[c->device];
  }
  SigArgs a{};
  a.N = c->N;
  a.rowptr = c->d_rowptr;
  a.colidx = c->d_colidx;
  a.val64 = c->d_val64;
  a.val32 = c->d_val32;
  a.s2ptr = c->d_s2ptr;
  a.s2col = c->d_s2col;
  a.s2val = c->d_s2val;
  a.hdiag = c->d_hdiag;
  a.sdiag = c->d_sdiag;
  a.item_row = it->item_row;
  a.item_sub = it->item_sub;
  a.row_nitems = it->row_nitems;
  a.n_items = it->n_items;
  a.u = u_t;
  a.u32 = u_t32;
  a.u32_ld = n_st;
  a.v = v_t;
  a.s = s_t;
  a.pv = scratch;  // every slot read by k_sigma_combine is written earlier in the same call
  a.ps = scratch + QP_NOALLOC_SLOTS;
  a.row_lo = 0;
  a.row_hi = (int)c->N;
  a.row_first = 0;
  a.row_step = 1;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const unsigned grid = gsz(it->n_items * 32, SBLK);
  launch_any(a, n_st, precision, grid, st, c->n_sm, it->sig32_variant[n_st]);
  if (it->n_multi > 0)
    k_sigma_combine<<<gsz((int64_t)it->n_multi * n_st, 256), 256, 0, st>>>(a, it->multi_rows, it->row_item0,
                                                                          it->n_multi, n_st);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, cudaGetErrorString(e));
  return QPGPU_OK;
}
