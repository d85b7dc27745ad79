// Device helpers shared by the sigma kernels (single problem and batched).
#pragma once

#include "qpgpu_internal.cuh"

namespace qpsig {

// ---- cross-lane reductions ---------------------------------------------
// Reduce-scatter of NSTP per-lane partial sums over the 32 lanes of a warp:
// each round halves the values a lane keeps (exchanging the other half with
// its partner), then plain butterflies finish.  A lane performs
// log2(NSTP) + ... = 5 + NSTP - 1 - log2(NSTP) additions instead of 5 * NSTP,
// which matters on GB300 where FP64 issue is scarce.  On return acc[0] of lane
// L holds the full sum of state (L >> (5 - log2 NSTP)).  The order of the
// additions is fixed, so results are deterministic.
template <int NSTP>
__device__ __forceinline__ double reduce_scatter64(double (&acc)[NSTP], int lane) {
  int off = 16;
#pragma unroll
  for (int m = NSTP; m > 1; m >>= 1, off >>= 1) {
    const bool up = lane & off;
#pragma unroll
    for (int i = 0; i < m / 2; ++i) {
      const double send = up ? acc[i] : acc[i + m / 2];
      const double keep = up ? acc[i + m / 2] : acc[i];
      acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  double x = acc[0];
#pragma unroll
  for (; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  return x;
}

// Float-float (hi + lo) form of a double, built with integer and FP32
// instructions only: hi keeps the top 24 bits of the significand
// (truncated), lo the next 23 (the last 6 bits, below 2^-46 |x|, are
// dropped), so hi + lo carries about 47 significant bits.  |x| below 2^-126
// gives (0, 0) and below 2^-80 lo = 0, absolute errors far below anything a
// Davidson vector resolves.  Finite |x| < 2^127 is assumed (normalised CI
// vectors and their sigma).
__device__ __forceinline__ void split_ff(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const unsigned sign = h32 & 0x80000000u;
  const int e = (int)((h32 >> 20) & 0x7ffu);
  const int fe = e - 896;  // float biased exponent of hi (e - 1023 + 127)
  if (fe <= 0) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((unsigned)fe << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
  const int se = e - 942;  // biased exponent of 2^(e - 1069)
  if (se <= 0) {
    lo = 0.f;
    return;
  }
  const float r = __fsub_rn(__uint_as_float(0x4B000000u | ((l32 & 0x1fffffffu) >> 6)), 8388608.0f);
  lo = __fmul_rn(r, __uint_as_float((unsigned)se << 23));
  if (sign) lo = -lo;
}

// error-free sum of two floats (Knuth TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// float-float (hi, lo) version of reduce_scatter64, all arithmetic in FP32
template <int NSTP>
__device__ __forceinline__ void reduce_scatter_ff(float (&hi)[NSTP], float (&lo)[NSTP], int lane, float& rh,
                                                  float& rl) {
  int off = 16;
#pragma unroll
  for (int m = NSTP; m > 1; m >>= 1, off >>= 1) {
    const bool up = lane & off;
#pragma unroll
    for (int i = 0; i < m / 2; ++i) {
      const float sh = up ? hi[i] : hi[i + m / 2], sl = up ? lo[i] : lo[i + m / 2];
      const float kh = up ? hi[i + m / 2] : hi[i], kl = up ? lo[i + m / 2] : lo[i];
      const float oh = __shfl_xor_sync(0xffffffffu, sh, off), ol = __shfl_xor_sync(0xffffffffu, sl, off);
      float s, e;
      two_sum(kh, oh, s, e);
      const float l = __fadd_rn(__fadd_rn(kl, ol), e);
      hi[i] = __fadd_rn(s, l);
      lo[i] = __fsub_rn(l, __fsub_rn(hi[i], s));
    }
  }
  float h = hi[0], l = lo[0];
#pragma unroll
  for (; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, off), ol = __shfl_xor_sync(0xffffffffu, l, off);
    float s, e;
    two_sum(h, oh, s, e);
    const float t = __fadd_rn(__fadd_rn(l, ol), e);
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
  }
  rh = h;
  rl = l;
}

template <int NST>
struct Pow2 {
  static constexpr int v = NST <= 1 ? 1 : NST <= 2 ? 2 : NST <= 4 ? 4 : 8;
  static constexpr int lg = NST <= 1 ? 0 : NST <= 2 ? 1 : NST <= 4 ? 2 : 3;
};

// coefficient row of determinant `col`: vector loads where the layout allows
template <int NST>
__device__ __forceinline__ void load_row(const double* u, int64_t col, double (&x)[NST]) {
  const double* p = u + col * NST;
  if constexpr (NST % 2 == 0) {
#pragma unroll
    for (int i = 0; i < NST; i += 2) {
      const double2 t = __ldg(reinterpret_cast<const double2*>(p + i));
      x[i] = t.x;
      x[i + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < NST; ++i) x[i] = __ldg(p + i);
  }
}

template <int NST>
__device__ __forceinline__ void load_row(const float* u, int64_t col, float (&x)[NST]) {
  const float* p = u + col * NST;
  if constexpr (NST % 4 == 0) {
#pragma unroll
    for (int i = 0; i < NST; i += 4) {
      const float4 t = __ldg(reinterpret_cast<const float4*>(p + i));
      x[i] = t.x;
      x[i + 1] = t.y;
      x[i + 2] = t.z;
      x[i + 3] = t.w;
    }
  } else if constexpr (NST % 2 == 0) {
#pragma unroll
    for (int i = 0; i < NST; i += 2) {
      const float2 t = __ldg(reinterpret_cast<const float2*>(p + i));
      x[i] = t.x;
      x[i + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < NST; ++i) x[i] = __ldg(p + i);
  }
}

// FP32 coefficients of row col from a layout whose rows are LD floats apart
// (LD = NST, or NST padded to 4 or 8 so that a row sits in one 32-byte
// sector: 16-byte loads, then an 8-byte and a 4-byte load for the rest)
template <int NST, int LD, bool V8 = false>
__device__ __forceinline__ void load_row_ld(const float* u, int64_t col, float (&x)[NST]) {
  const float* p = u + col * LD;
  if constexpr (LD == 8 && V8) {
    // one 32-byte load (sm_100+ 256-bit vector load; p is 32-byte aligned):
    // a single L2 request per row instead of two
    float t[8];
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(t[0]), "=f"(t[1]), "=f"(t[2]), "=f"(t[3]), "=f"(t[4]), "=f"(t[5]), "=f"(t[6]), "=f"(t[7])
        : "l"(p));
#pragma unroll
    for (int i = 0; i < NST; ++i) x[i] = t[i];
  } else if constexpr (LD % 4 == 0) {
    constexpr int N4 = NST / 4, R = NST % 4;
#pragma unroll
    for (int i = 0; i < N4; ++i) {
      const float4 t = __ldg(reinterpret_cast<const float4*>(p) + i);
      x[4 * i] = t.x;
      x[4 * i + 1] = t.y;
      x[4 * i + 2] = t.z;
      x[4 * i + 3] = t.w;
    }
    if constexpr (R >= 2) {
      const float2 t = __ldg(reinterpret_cast<const float2*>(p + 4 * N4));
      x[4 * N4] = t.x;
      x[4 * N4 + 1] = t.y;
    }
    if constexpr (R % 2 == 1) x[NST - 1] = __ldg(p + NST - 1);
  } else {
    load_row<NST>(u, col, x);
  }
}


}  // namespace qpsig
