// FP64-accurate tall-skinny Gram blocks X = A^T B on the tensor cores
// (tcgen05, sm_103a) by error-free splitting of the FP64 operands into BF16
// digit planes (the Ozaki scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59 (2012)
// 95-118), with exact integer accumulation of the digit products and FP64
// combination of the per-CTA results.
//
// Splitting.  Column c of an operand gets the exponent E_c with |x| < 2^E_c
// for every element (k_col_maxexp).  An element is rounded to the 56-bit
// fixed-point integer F = round(|x| 2^(56 - E_c)) and written in balanced
// base 128, F = sum_p d_p 2^(49 - 7p) with d_1..d_7 in [-64, 63] and d_0 in
// [0, 128], every digit times the sign of x: integers exact in BF16.  The
// digits are those of F + 64 (1 + 2^7 + ... + 2^49) less 64 each, so they
// come out of independent shifts and masks, with no carry chain.
// Balanced digits make both the rounding and the dropped low-order products
// zero-mean, so they do not pile up in sums of squares (Gram diagonals).
//
// Products.  For digit planes p of A and q of B, tcgen05.mma (kind::f16,
// BF16 x BF16 -> FP32, M = 128 columns of A, N = 16 columns of B, K = rows)
// forms sum_r d_p(a_ri) d_q(b_rj) exactly: a product is at most 2^14 (both
// leading digits) or 2^13, and a level L = p + q over 128 rows stays below
// 2^23, so the FP32 accumulator of each level holds an exact integer.
// Levels L = 0..7 are kept (a dropped product is below 2^-56 of
// max|a| max|b|, like the rounding of the splitting).  Every 128 rows (a
// window) the eight level accumulators are read from tensor memory and added,
// as integers, to two int64 fixed-point sums per entry (levels 0-3 and 4-7),
// so nothing is rounded until the CTA's rows are done; then each CTA's entry
// becomes an FP64 value and the CTAs are summed in FP64 in a fixed order.
//
// Pipeline (one CTA per SM over a contiguous block of rows, chunks of 32
// rows), one role per warp:
//  * warp 13 streams the raw FP64 rows of each chunk into a ring of raw
//    stages (cp.async.bulk per operand block, completing on rawfull[r]; a
//    block whose rows are strided or unaligned is copied by the warp's lanes);
//  * warps 0-7 cut the chunk into digit planes (stores of 2, 4 or 8 rows of
//    one column), free the raw stage (rawempty[r]) and fill digit stage s
//    (full[s]);
//  * warp 12 issues the chunk's 16 MMAs once full[s] completes and commits
//    them to empty[s] and, at the end of a window, to accf[b]; the windows
//    rotate over four tensor-memory accumulator buffers b;
//  * warps 8-11, whose lane quarters cover the 128 accumulator rows, add a
//    finished window to their int64 sums and arrive on acce[b], so that the
//    integer work never holds up the splitting.
// A plane p of A meets B planes 0..7-p only (levels p..7), so its MMA has
// N = (8 - p) 16 and writes the accumulator from level p on.
// Every mbarrier wait is bounded and gives up early once another warp has set
// the CTA's error flag; the warps then leave their loops, the kernel waits
// (bounded) for its bulk copies and MMAs, frees its tensor memory and sets
// *status.
#include <algorithm>

#include "qpgpu_internal.cuh"

namespace {

constexpr int OZ_SPLIT = 256;                // splitting threads (warps 0-7)
constexpr int OZ_FLUSH_WARP = 8;             // warps 8-11 flush the accumulators
constexpr int OZ_MMA_WARP = 12;              // issues the MMAs, owns the tensor memory
constexpr int OZ_LOAD_WARP = 13;             // streams the raw rows
constexpr int OZ_THREADS = 14 * 32;
constexpr int OZ_M = 128;                    // MMA M: columns of A (padded)
constexpr int OZ_N = 16;                     // columns of B (padded)
constexpr int OZ_KC = 32;                    // rows per chunk (MMA K = 2 x 16)
constexpr int OZ_DIG = 8;                    // digit planes per operand
constexpr int OZ_LEVELS = 8;                 // levels p + q = 0..7 kept
constexpr int OZ_WINDOW = 4;                 // chunks per accumulator window (128 rows)
constexpr int OZ_NBUF = 4;                   // accumulator buffers
constexpr int OZ_A_TILE = OZ_M * OZ_KC * 2;  // bytes of one A digit plane
constexpr int OZ_B_TILE = OZ_N * OZ_KC * 2;
// a digit stage: the 8 A planes, then the 8 B planes, so that B planes
// 0..n-1 form one K-major operand of 16 n rows
constexpr int OZ_STAGE = OZ_DIG * OZ_A_TILE + OZ_DIG * OZ_B_TILE;
constexpr int OZ_TAB = 6144;  // alignment, exponents, block tables, barriers
constexpr int OZ_SMEM_MAX = 232448;
constexpr int OZ_MAXRAW = 8;  // raw stages at most
constexpr int OZ_MAXBLK = OZ_M + 2;  // operand blocks: at most one per column of A, two of B

constexpr int OZ_ACC_COLS = OZ_LEVELS * OZ_N;     // 128 tensor-memory columns per buffer
constexpr int OZ_TMEM_COLS = OZ_NBUF * OZ_ACC_COLS;  // 512: the whole tensor memory of the SM
constexpr long long OZ_WAIT_LIMIT = 1LL << 25;

// barrier slots
constexpr int OZ_B_FULL = 0, OZ_B_EMPTY = 2, OZ_B_ACCF = 4, OZ_B_ACCE = OZ_B_ACCF + OZ_NBUF,
              OZ_B_RAWF = OZ_B_ACCE + OZ_NBUF, OZ_B_RAWE = OZ_B_RAWF + OZ_MAXRAW, OZ_NBARS = OZ_B_RAWE + OZ_MAXRAW;

struct OzArgs {
  const double* A;  // blocks of nsdA columns, rows ldA values apart, blocks sA apart
  int64_t sA;
  int m, nsdA, ldA;
  const double* B0;  // nsdB columns, rows ldB apart
  const double* B1;  // optional second block (columns nsdB..2 nsdB-1)
  int nbc, nsdB, ldB;
  int64_t N, rows_per_cta;
  const int* eA;  // biased max exponent of each column of A (k_col_maxexp)
  const int* eB;
  double* partial;  // [cta][m][nbc]
  const int* skip;
  int* status;
  int nraw;        // raw stages in the ring
  int raw_stride;  // doubles per raw stage
  int rpt;         // rows per splitting task: 2, 4 or 8
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) in a K-major tile of 8 x 16-byte core
// matrices, core (row / 8, k / 8) at ((row / 8) * (KC / 8) + k / 8) * 128:
// the start of K step t is + t * 256, the K-direction stride (LBO) 128 bytes,
// the row-group stride (SBO) (KC / 8) * 128 = 512 bytes
__device__ __forceinline__ int kmaj(int row, int k) {
  return (((row >> 3) * (OZ_KC / 8)) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// tcgen05 shared-memory matrix descriptor: start, LBO, SBO (bytes >> 4),
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__device__ __forceinline__ uint32_t oz_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(OZ_M >> 4) << 24);
}

// 64 in every base-128 digit position of a 56-bit integer
constexpr unsigned long long OZ_H = 64ull * ((1ull << 49) | (1ull << 42) | (1ull << 35) | (1ull << 28) |
                                             (1ull << 21) | (1ull << 14) | (1ull << 7) | 1ull);

// the 8 balanced digits of x against the column's biased max exponent eb
// (|x| < 2^(eb - 1022)), as FP32 values (exact small integers, so their top
// 16 bits are their BF16 bits).  F = round(|x| 2^(56 - E)), E = eb - 1022,
// is the 53-bit significand M = m53 2^3 rounded-shifted right by eb - ex
// (<= 2^56).  With G = F + OZ_H, the plain base-128 digits g_p of G less 64
// are a balanced expansion of F: F = sum_p (g_p - 64) 2^(49 - 7p), d_0 in
// [0, 128] and d_1..d_7 in [-64, 63].  No digit waits on another: each is a
// shift, a mask with the 2^23 exponent bits, and one exact FMA that removes
// 2^23 + 64 and applies the sign of x.
__device__ __forceinline__ void oz_digits(double x, int eb, float (&d)[OZ_DIG]) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t bh = (uint32_t)(b >> 32);
  const int ex = (int)((bh >> 20) & 0x7FF);
  const int k = max(eb - ex, 0);
  unsigned long long F = 0;
  if (ex != 0 && k < 57) {
    const unsigned long long M = ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 3;
    F = k == 0 ? M : (M + (1ull << (k - 1))) >> k;
  }
  const unsigned long long G = F + OZ_H;
  const uint32_t gl = (uint32_t)G, gh = (uint32_t)(G >> 32);
  const uint32_t sbit = bh & 0x80000000u;
  const float sg = __uint_as_float(sbit | 0x3F800000u);   // +-1
  const float sc = __uint_as_float(sbit | 0x4B000040u);   // +-(2^23 + 64)
  const uint32_t g[OZ_DIG] = {gh >> 17, gh >> 10, gh >> 3, __funnelshift_r(gl, gh, 28), gl >> 21, gl >> 14, gl >> 7, gl};
#pragma unroll
  for (int p = 0; p < OZ_DIG; ++p)
    d[p] = __fmaf_rn(sg, __uint_as_float(0x4B000000u | (g[p] & (p == 0 ? 0xFFu : 0x7Fu))), -sc);
}

// BF16 bits of two exact small-integer FP32 values, packed (lo, hi)
__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait for the completion of phase `parity` of an mbarrier; gives up
// early once the CTA's error flag is set
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const int* sflag) {
  for (long long it = 0; it < OZ_WAIT_LIMIT; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255) == 255 && *(volatile const int*)sflag) return false;
  }
  return false;
}

// bounded wait that ignores the error flag: for the drains before exit
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < OZ_WAIT_LIMIT; ++it)
    if (mbar_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// level L of accumulator buffer `buf` (this warp's 32 lanes, 16 columns),
// exact integers below 2^23, shifted by sh into acc
__device__ __forceinline__ void oz_flush1(uint32_t taddr, int sh, long long (&acc)[OZ_N]) {
  uint32_t v[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < OZ_N; ++j) acc[j] += (long long)__float2int_rn(__uint_as_float(v[j])) << sh;
}

// digit planes of one chunk: task (column, group of RPT rows) writes RPT
// rows of one column into each of the 8 planes of stage (sa, sb)
template <int RPT>
__device__ __forceinline__ void oz_split(const double* rsrc, uint8_t* sa, uint8_t* sb, int m, int rw, int nrow,
                                         const int* coff, const int* cw, const int* sE, int tid) {
  const int ntask = rw * (OZ_KC / RPT);
  for (int t = tid; t < ntask; t += OZ_SPLIT) {
    const int grp = t / rw, col = t - grp * rw;
    const bool isA = col < m;
    const int cc = isA ? col : col - m;
    const int eb = sE[isA ? cc : OZ_M + cc];
    const int wcol = cw[col], k0 = RPT * grp;
    const double* xs = rsrc + coff[col] + k0 * wcol;
    uint32_t pk[OZ_DIG][RPT / 2];
#pragma unroll
    for (int k = 0; k < RPT; k += 2) {
      float d0[OZ_DIG], d1[OZ_DIG];
      oz_digits(k0 + k < nrow ? xs[k * wcol] : 0.0, eb, d0);
      oz_digits(k0 + k + 1 < nrow ? xs[(k + 1) * wcol] : 0.0, eb, d1);
#pragma unroll
      for (int p = 0; p < OZ_DIG; ++p) pk[p][k >> 1] = bf16x2(d0[p], d1[p]);
    }
    uint8_t* dst = (isA ? sa : sb) + kmaj(cc, k0);
    const int tile = isA ? OZ_A_TILE : OZ_B_TILE;
#pragma unroll
    for (int p = 0; p < OZ_DIG; ++p) {
      if constexpr (RPT == 8)
        *reinterpret_cast<uint4*>(dst + p * tile) = make_uint4(pk[p][0], pk[p][1], pk[p][2], pk[p][3]);
      else if constexpr (RPT == 4)
        *reinterpret_cast<uint2*>(dst + p * tile) = make_uint2(pk[p][0], pk[p][1]);
      else
        *reinterpret_cast<uint32_t*>(dst + p * tile) = pk[p][0];
    }
  }
}

__global__ void __launch_bounds__(OZ_THREADS, 1) k_gram_oz(OzArgs g) {
  if (g.skip && *g.skip) return;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sbase = (uint8_t*)(((uintptr_t)smem + 1023) & ~(uintptr_t)1023);
  uint8_t* tiles = sbase;                                 // digit stage s: A planes, then B planes
  double* raw = (double*)(sbase + 2 * OZ_STAGE);          // nraw stages, operand blocks of [OZ_KC][width]
  const double** bsrc = (const double**)(sbase + 2 * OZ_STAGE + (size_t)g.nraw * g.raw_stride * 8);  // block bases
  int* bw = (int*)(bsrc + OZ_MAXBLK);                     // [OZ_MAXBLK] block widths
  int* bld = bw + OZ_MAXBLK;                              // [OZ_MAXBLK] row strides
  int* boff = bld + OZ_MAXBLK;                            // [OZ_MAXBLK] raw-stage offsets (doubles)
  int* coff = boff + OZ_MAXBLK;                           // [OZ_M + OZ_N] raw offset of each column
  int* cw = coff + OZ_M + OZ_N;                           // [OZ_M + OZ_N] width of its block
  int* sE = cw + OZ_M + OZ_N;                             // [OZ_M] A, [OZ_N] B exponents
  uint64_t* bars = (uint64_t*)(((uintptr_t)(sE + OZ_M + OZ_N) + 7) & ~(uintptr_t)7);
  uint32_t* tmem_slot = (uint32_t*)(bars + OZ_NBARS);
  int* sflag = (int*)(tmem_slot + 1);                     // error flag of the CTA
  int* snblk = sflag + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = g.m, nbc = g.nbc, rw = m + nbc;
  const uint32_t bar0 = smem_u32(bars);
  auto BAR = [&](int slot, int i) { return bar0 + 8u * (uint32_t)(slot + i); };

  for (int i = tid; i < 2 * OZ_STAGE / 16; i += OZ_THREADS) reinterpret_cast<uint4*>(tiles)[i] = make_uint4(0, 0, 0, 0);
  for (int i = tid; i < OZ_M; i += OZ_THREADS) sE[i] = i < m ? g.eA[i] : 0;
  for (int j = tid; j < OZ_N; j += OZ_THREADS) sE[OZ_M + j] = j < nbc ? g.eB[j] : 0;
  if (warp == OZ_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(BAR(OZ_B_FULL, s)), "r"(OZ_SPLIT / 32));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(BAR(OZ_B_EMPTY, s)));
    }
    for (int b = 0; b < OZ_NBUF; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(BAR(OZ_B_ACCF, b)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(BAR(OZ_B_ACCE, b)));
    }
    for (int r = 0; r < OZ_MAXRAW; ++r) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(BAR(OZ_B_RAWF, r)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(BAR(OZ_B_RAWE, r)), "r"(OZ_SPLIT / 32));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
    *sflag = 0;
    // operand blocks: A in blocks of nsdA columns, then B0 and B1; each is
    // staged as [OZ_KC][width] at boff, its column c at coff[c] + row * width
    int nb = 0, col = 0, off = 0;
    for (int c0 = 0; c0 < m; c0 += g.nsdA, ++nb) {
      const int w = min(g.nsdA, m - c0);
      bsrc[nb] = g.A + (int64_t)(c0 / g.nsdA) * g.sA;
      bw[nb] = w;
      bld[nb] = g.ldA;
      boff[nb] = off;
      for (int j = 0; j < w; ++j, ++col) {
        coff[col] = off + j;
        cw[col] = w;
      }
      off += OZ_KC * w;
    }
    for (int c0 = 0; c0 < nbc; c0 += g.nsdB, ++nb) {
      const int w = min(g.nsdB, nbc - c0);
      bsrc[nb] = c0 == 0 ? g.B0 : g.B1;
      bw[nb] = w;
      bld[nb] = g.ldB;
      boff[nb] = off;
      for (int j = 0; j < w; ++j, ++col) {
        coff[col] = off + j;
        cw[col] = w;
      }
      off += OZ_KC * w;
    }
    *snblk = nb;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int64_t r0 = (int64_t)blockIdx.x * g.rows_per_cta;
  const int64_t r1 = min(r0 + g.rows_per_cta, g.N);
  const int nchunks = r1 > r0 ? (int)((r1 - r0 + OZ_KC - 1) / OZ_KC) : 0;
  const int nwin = (nchunks + OZ_WINDOW - 1) / OZ_WINDOW;
  const int nraw = g.nraw;
  long long hi[OZ_N], lo[OZ_N];  // fixed-point sums of this thread's A column (flush warps)
#pragma unroll
  for (int j = 0; j < OZ_N; ++j) hi[j] = lo[j] = 0;

  if (warp < OZ_SPLIT / 32) {
    // ---- splitting warps -------------------------------------------------
    for (int c = 0; c < nchunks; ++c) {
      const int s = c & 1, rs = c % nraw;
      // chunk c's raw rows have landed; the MMAs of chunk c - 2 are done with digit stage s
      bool ok = mbar_wait(BAR(OZ_B_RAWF, rs), (uint32_t)(c / nraw) & 1u, sflag);
      if (ok && c >= 2) ok = mbar_wait(BAR(OZ_B_EMPTY, s), (uint32_t)((c >> 1) - 1) & 1u, sflag);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(sflag, 1);
        break;
      }
      uint8_t* sa = tiles + s * OZ_STAGE;
      uint8_t* sb = sa + OZ_DIG * OZ_A_TILE;
      const double* rsrc = raw + (size_t)rs * g.raw_stride;
      const int nrow = (int)min((int64_t)OZ_KC, r1 - (r0 + (int64_t)c * OZ_KC));
      if (g.rpt == 8)
        oz_split<8>(rsrc, sa, sb, m, rw, nrow, coff, cw, sE, tid);
      else if (g.rpt == 4)
        oz_split<4>(rsrc, sa, sb, m, rw, nrow, coff, cw, sE, tid);
      else
        oz_split<2>(rsrc, sa, sb, m, rw, nrow, coff, cw, sE, tid);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(BAR(OZ_B_RAWE, rs));
        mbar_arrive(BAR(OZ_B_FULL, s));
      }
    }
  } else if (warp < OZ_MMA_WARP) {
    // ---- flush warps: lane quarter q = warp % 4 holds rows 32 q .. 32 q + 31
    const uint32_t lrow = (uint32_t)((warp & 3) * 32) << 16;
    for (int w = 0; w < nwin; ++w) {
      const int buf = w % OZ_NBUF;
      const bool ok = mbar_wait(BAR(OZ_B_ACCF, buf), (uint32_t)(w / OZ_NBUF) & 1u, sflag);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(sflag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ta = tmem + lrow + (uint32_t)(buf * OZ_ACC_COLS);
#pragma unroll
      for (int L = 0; L < OZ_LEVELS / 2; ++L) oz_flush1(ta + L * OZ_N, 7 * (3 - L), hi);
#pragma unroll
      for (int L = OZ_LEVELS / 2; L < OZ_LEVELS; ++L) oz_flush1(ta + L * OZ_N, 7 * (7 - L), lo);
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(BAR(OZ_B_ACCE, buf));
    }
  } else if (warp == OZ_MMA_WARP) {
    // ---- MMA warp: lane 0 issues, the warp stays converged ----------------
    uint32_t last_bar = 0, last_par = 0;  // the latest commit: its completion covers every MMA
    for (int c = 0; c < nchunks; ++c) {
      const int s = c & 1, w = c / OZ_WINDOW, buf = w % OZ_NBUF;
      bool ok = true;
      if (lane == 0) {
        // accumulator buffer flushed (window w - 4), digit stage s full
        if (c % OZ_WINDOW == 0 && w >= OZ_NBUF)
          ok = mbar_wait(BAR(OZ_B_ACCE, buf), (uint32_t)(w / OZ_NBUF - 1) & 1u, sflag);
        if (ok) ok = mbar_wait(BAR(OZ_B_FULL, s), (uint32_t)(c >> 1) & 1u, sflag);
        if (ok) {
          asm volatile("tcgen05.fence::after_thread_sync;");
          const bool first = (c % OZ_WINDOW) == 0;
          const uint32_t a0 = smem_u32(tiles + s * OZ_STAGE);
          const uint32_t b0 = a0 + OZ_DIG * OZ_A_TILE;  // B planes 0..7
#pragma unroll
          for (int p = 0; p < OZ_DIG; ++p)
#pragma unroll
            for (int kt = 0; kt < OZ_KC / 16; ++kt) {
              // levels L = p..7 of A plane p against B planes 0..7-p; the
              // first product of a window overwrites the accumulator
              const uint32_t acc = (first && p == 0 && kt == 0) ? 0u : 1u;
              asm volatile(
                  "{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n}" ::"r"(
                      tmem + (uint32_t)(buf * OZ_ACC_COLS + p * OZ_N)),
                  "l"(sdesc(a0 + p * OZ_A_TILE + kt * 256)), "l"(sdesc(b0 + kt * 256)),
                  "r"(oz_idesc((OZ_LEVELS - p) * OZ_N)), "r"(acc));
            }
          mma_commit(BAR(OZ_B_EMPTY, s));
          last_bar = BAR(OZ_B_EMPTY, s);
          last_par = (uint32_t)(c >> 1) & 1u;
          if (c % OZ_WINDOW == OZ_WINDOW - 1 || c == nchunks - 1) mma_commit(BAR(OZ_B_ACCF, buf));
        } else {
          atomicExch(sflag, 1);
        }
      }
      if (!__shfl_sync(0xffffffffu, (int)ok, 0)) break;
    }
    // before the tensor memory is freed, every MMA issued must have completed
    if (lane == 0 && last_bar != 0 && !mbar_drain(last_bar, last_par)) atomicExch(sflag, 1);
    __syncwarp();
  } else if (warp == OZ_LOAD_WARP) {
    // ---- load warp: raw rows of chunk cc into raw stage cc % nraw ---------
    // A block whose rows are contiguous (row stride = width) and 16-byte
    // aligned comes in with one bulk copy; any other block is copied by the
    // lanes.  Rows past r1 are not copied: the split reads them as zeros.
    const int nblk = *snblk;
    int issued = 0;
    for (int cc = 0; cc < nchunks; ++cc) {
      const int rs = cc % nraw;
      const bool ok = cc < nraw || mbar_wait(BAR(OZ_B_RAWE, rs), (uint32_t)(cc / nraw - 1) & 1u, sflag);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(sflag, 1);
        break;
      }
      double* dst0 = raw + (size_t)rs * g.raw_stride;
      const int64_t rb = r0 + (int64_t)cc * OZ_KC;
      const int nrow = (int)min((int64_t)OZ_KC, r1 - rb);
      uint32_t bytes = 0;
      for (int k = 0; k < nblk; ++k) {
        const uint32_t nb = (uint32_t)(nrow * bw[k] * 8);
        const double* src = bsrc[k] + rb * bld[k];
        if (bld[k] == bw[k] && ((uintptr_t)src & 15) == 0 && (nb & 15) == 0) {
          bytes += nb;
        } else {
          for (int t = lane; t < nrow * bw[k]; t += 32) {
            const int rr = t / bw[k], j = t - rr * bw[k];
            dst0[boff[k] + t] = src[(int64_t)rr * bld[k] + j];
          }
        }
      }
      __syncwarp();
      if (lane == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(BAR(OZ_B_RAWF, rs)), "r"(bytes)
                     : "memory");
        for (int k = 0; k < nblk; ++k) {
          const uint32_t nb = (uint32_t)(nrow * bw[k] * 8);
          const double* src = bsrc[k] + rb * bld[k];
          if (bld[k] == bw[k] && ((uintptr_t)src & 15) == 0 && (nb & 15) == 0 && nb > 0)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(dst0 + boff[k])),
                "l"(src), "r"(nb), "r"(BAR(OZ_B_RAWF, rs))
                : "memory");
        }
      }
      issued = cc + 1;
    }
    // the copies still in flight land before the CTA may exit
    if (lane == 0)
      for (int cc = max(0, issued - nraw); cc < issued; ++cc)
        if (!mbar_drain(BAR(OZ_B_RAWF, cc % nraw), (uint32_t)(cc / nraw) & 1u)) atomicExch(sflag, 1);
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const bool ok = *(volatile int*)sflag == 0;
  if (!ok && tid == 0) atomicExch(g.status, 1);
  if (warp >= OZ_FLUSH_WARP && warp < OZ_MMA_WARP) {
    const int i = (warp & 3) * 32 + lane;
    if (i < m)
#pragma unroll
      for (int j = 0; j < OZ_N; ++j)
        if (j < nbc) {
          const int e = (sE[i] - 1022) + (sE[OZ_M + j] - 1022);
          const double v = ldexp((double)hi[j], e - 35) + ldexp((double)lo[j], e - 63);
          g.partial[((int64_t)blockIdx.x * m + i) * nbc + j] = ok ? v : 0.0;
        }
  }
  if (warp == OZ_MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS));
}


// ---- linear combinations O = [A_0 .. A_nb-1] C on the tensor cores --------
//
// O(r, j) = sum_i A(r, i) C(i, j): the Davidson updates (Gram-Schmidt and
// Cholesky-QR, Ritz vectors, re-contraction).  A is nb blocks of nsd columns
// (rows nsd doubles apart, blocks sA apart), C is (m x nsd) row-major
// (m = nb nsd), O has rows ldO doubles apart and may be the last block of A.
// The contraction runs over i, so each row r of A gets its own exponent
// (the largest over its m values) and C one per column j; the digits and
// levels are those of k_gram_oz, and a level of one entry sums at most
// m <= 128 products, below 2^23.  One CTA per SM walks tiles of 128 rows:
// the tile's rows are loaded into shared memory, its row exponents formed,
// then each K step of 16 columns is cut into the 8 A digit planes (two
// stages, so that the split of step c + 1 overlaps the MMAs of step c) and
// one thread issues its 8 MMAs (M = 128 rows, N = (8 - p) 16, K = 16) into
// the tile's accumulator; when the tile's MMAs are done, warps 0-3 read the
// 8 levels of their rows and write O in FP64.  The digit planes of C are
// built once per CTA.  Waits are bounded as in k_gram_oz.
constexpr int LC_THREADS = 512;             // 16 warps: 4 threads per row of a tile
constexpr int LC_RQ = LC_THREADS / 128;      // threads per row
constexpr int LC_TM = 128;                       // rows per tile (MMA M)
constexpr int LC_KS = 16;                        // K step (columns of A)
constexpr int LC_APLANE = LC_TM * LC_KS * 2;     // 4 KB: one A digit plane of one K step
constexpr int LC_ASTAGE = OZ_DIG * LC_APLANE;    // 32 KB
constexpr int LC_BCHUNK = OZ_DIG * OZ_N * LC_KS * 2;  // 4 KB: the 8 C planes of one K step
constexpr int LC_MAXM = 128;
constexpr int LC_TMEM_COLS = OZ_LEVELS * OZ_N;   // 128

struct LcArgs {
  const double* A;
  int64_t sA;
  int m, nsd;
  const double* C;  // (m, nsd) row-major
  double* O;
  int64_t ldO;
  int64_t N, rows_per_cta;
  int row_stride;  // doubles per staged row in shared memory
  const int* skip;
  int* status;
};

// byte offset of (row, k) in a K-major tile of 8 x 16-byte core matrices
// with K = 16: row-group stride (SBO) 256 bytes, K-direction stride (LBO) 128
__device__ __forceinline__ int kmaj16(int row, int k) {
  return (((row >> 3) * 2) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ uint64_t sdesc16(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__device__ __forceinline__ int biased_exp(double x) {
  return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FF);
}

__global__ void __launch_bounds__(LC_THREADS, 1) k_lincomb_oz(LcArgs g) {
  if (g.skip && *g.skip) return;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sbase = (uint8_t*)(((uintptr_t)smem + 1023) & ~(uintptr_t)1023);
  uint8_t* adig = sbase;                                  // 2 stages of 8 A planes
  uint8_t* bdig = sbase + 2 * LC_ASTAGE;                  // nks x 8 C planes
  const int m = g.m, nsd = g.nsd, nb = m / nsd;
  const int nks = (m + LC_KS - 1) / LC_KS;
  const int rs = g.row_stride;                            // doubles per staged row (nsd, or nsd + 1: odd)
  double* raw = (double*)(bdig + (size_t)nks * LC_BCHUNK);  // [block][128 rows][rs]
  int* eb = (int*)(raw + (size_t)nb * LC_TM * rs);        // [128] row exponents
  int* ej = eb + LC_TM;                                    // [16] column exponents of C
  // [LC_RQ][128] partial row exponents: in digit stage 1, idle at the start
  // of a tile (the previous tile's MMAs are done, its flush used stage 0)
  int* eh = (int*)(adig + LC_ASTAGE);
  uint64_t* bars = (uint64_t*)(((uintptr_t)(ej + OZ_N) + 7) & ~(uintptr_t)7);  // stage[2], tile
  uint32_t* tmem_slot = (uint32_t*)(bars + 3);
  int* sflag = (int*)(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t bar0 = smem_u32(bars);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(LC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int b = 0; b < 3; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u * b));
    asm volatile("fence.mbarrier_init.release.cluster;");
    *sflag = 0;
  }
  // C: column exponents, then its digit planes (rows j of plane q at q 16 + j)
  for (int x = tid; x < nks * LC_BCHUNK / 16; x += LC_THREADS) reinterpret_cast<uint4*>(bdig)[x] = make_uint4(0, 0, 0, 0);
  if (tid < OZ_N) {
    int e = 0;
    if (tid < nsd)
      for (int i = 0; i < m; ++i) e = max(e, biased_exp(g.C[(int64_t)i * nsd + tid]));
    ej[tid] = e;
  }
  __syncthreads();
  for (int x = tid; x < m * nsd; x += LC_THREADS) {
    const int i = x / nsd, j = x - i * nsd;
    float d[OZ_DIG];
    oz_digits(g.C[x], ej[j], d);
    uint8_t* base = bdig + (size_t)(i / LC_KS) * LC_BCHUNK;
    const int k = i % LC_KS;
#pragma unroll
    for (int q = 0; q < OZ_DIG; ++q)
      *reinterpret_cast<uint16_t*>(base + kmaj16(q * OZ_N + j, k)) = (uint16_t)(__float_as_uint(d[q]) >> 16);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int64_t r0 = (int64_t)blockIdx.x * g.rows_per_cta;
  const int64_t r1 = min(r0 + g.rows_per_cta, g.N);
  const int ntile = r1 > r0 ? (int)((r1 - r0 + LC_TM - 1) / LC_TM) : 0;
  int gstep = 0;            // K steps issued so far (stage = gstep & 1)
  bool ok = true;
  uint32_t last_bar = 0, last_par = 0;
  // tile tt's rows into the padded staging rows with asynchronous 8-byte
  // copies: thread (row r, quarter h) copies blocks h, h + 4, ... of its row
  auto issue_rows = [&](int tt) {
    const int64_t Rt = r0 + (int64_t)tt * LC_TM;
    const int nrt = (int)min((int64_t)LC_TM, r1 - Rt);
    const int r = tid & (LC_TM - 1), h = tid >> 7;
    if (r < nrt)
      for (int b = h; b < nb; b += LC_RQ) {
        const double* src = g.A + (int64_t)b * g.sA + (Rt + r) * nsd;
        const uint32_t dst = smem_u32(raw + ((size_t)b * LC_TM + r) * rs);
        for (int c = 0; c < nsd; ++c)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst + 8u * c), "l"(src + c) : "memory");
      }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  if (ntile > 0) issue_rows(0);
  for (int t = 0; t < ntile && ok; ++t) {
    const int64_t R = r0 + (int64_t)t * LC_TM;
    const int nr = (int)min((int64_t)LC_TM, r1 - R);
    // this tile's rows have landed: their largest exponents
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    {
      const int r = tid & (LC_TM - 1), h = tid >> 7;
      int e = 0;
      if (r < nr)
        for (int b = h; b < nb; b += LC_RQ) {
          const double* row = raw + ((size_t)b * LC_TM + r) * rs;
          for (int c = 0; c < nsd; ++c) e = max(e, biased_exp(row[c]));
        }
      eh[h * LC_TM + r] = e;
    }
    __syncthreads();
    if (tid < LC_TM) eb[tid] = max(max(eh[tid], eh[LC_TM + tid]), max(eh[2 * LC_TM + tid], eh[3 * LC_TM + tid]));
    __syncthreads();
    for (int c = 0; c < nks; ++c, ++gstep) {
      const int s = gstep & 1;
      // the MMAs of step gstep - 2 are done with stage s
      if (gstep >= 2 && !mbar_wait(bar0 + 8u * s, (uint32_t)((gstep >> 1) - 1) & 1u, sflag)) ok = false;
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      uint8_t* sa = adig + s * LC_ASTAGE;
      {
        // thread: row r, 4 consecutive K of the step (half a 16-byte core row per plane)
        const int r = tid & (LC_TM - 1), k0 = (tid >> 7) * 4;
        const int er = eb[r];
        // column i of A is (block bi, column si) of the staged rows
        const int ibeg = c * LC_KS + k0;
        int bi = ibeg / nsd, si = ibeg - bi * nsd;
        double xv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          xv[k] = (r < nr && ibeg + k < m) ? raw[((size_t)bi * LC_TM + r) * rs + si] : 0.0;
          if (++si == nsd) {
            si = 0;
            ++bi;
          }
        }
        uint32_t pk[OZ_DIG][2];
#pragma unroll
        for (int k = 0; k < 4; k += 2) {
          float d0[OZ_DIG], d1[OZ_DIG];
          oz_digits(xv[k], er, d0);
          oz_digits(xv[k + 1], er, d1);
#pragma unroll
          for (int p = 0; p < OZ_DIG; ++p) pk[p][k >> 1] = bf16x2(d0[p], d1[p]);
        }
#pragma unroll
        for (int p = 0; p < OZ_DIG; ++p)
          *reinterpret_cast<uint2*>(sa + p * LC_APLANE + kmaj16(r, k0)) = make_uint2(pk[p][0], pk[p][1]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(bdig + (size_t)c * LC_BCHUNK);
#pragma unroll
        for (int p = 0; p < OZ_DIG; ++p) {
          const uint32_t acc = (c == 0 && p == 0) ? 0u : 1u;
          asm volatile(
              "{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n}" ::"r"(tmem + (uint32_t)(p * OZ_N)),
              "l"(sdesc16(a0 + p * LC_APLANE)), "l"(sdesc16(b0)), "r"(oz_idesc((OZ_LEVELS - p) * OZ_N)), "r"(acc));
        }
        mma_commit(bar0 + 8u * s);
        last_bar = bar0 + 8u * s;
        last_par = (uint32_t)(gstep >> 1) & 1u;
      }
    }
    if (!ok) break;
    // every split of this tile is done, so the staging rows are free: the
    // next tile's copies fly during this tile's MMA tail and flush
    if (t + 1 < ntile) issue_rows(t + 1);
    // the tile's MMAs are done: warps 0-3 write its rows
    if (tid == 0) mma_commit(bar0 + 16u);
    if (!mbar_wait(bar0 + 16u, (uint32_t)t & 1u, sflag)) ok = false;
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    {
      // warps w and w + 4 share lane quarter w % 4 (rows 32 (w % 4) ..):
      // warp w sums levels 0-3, warp w + 4 levels 4-7; both halves meet in
      // shared memory (the digit stages are free now)
      long long acc[OZ_N];
#pragma unroll
      for (int j = 0; j < OZ_N; ++j) acc[j] = 0;
      const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16);
      if (warp < 4) {
#pragma unroll
        for (int L = 0; L < OZ_LEVELS / 2; ++L) oz_flush1(ta + L * OZ_N, 7 * (3 - L), acc);
      } else if (warp < 8) {
#pragma unroll
        for (int L = OZ_LEVELS / 2; L < OZ_LEVELS; ++L) oz_flush1(ta + L * OZ_N, 7 * (7 - L), acc);
      }
      long long* lo_s = reinterpret_cast<long long*>(adig);  // [128 rows][17]: odd stride, no bank conflicts
      const int r = tid & (LC_TM - 1);
      if (warp >= 4 && warp < 8)
#pragma unroll
        for (int j = 0; j < OZ_N; ++j) lo_s[r * (OZ_N + 1) + j] = acc[j];
      __syncthreads();
      if (warp < 4 && r < nr) {
        double* o = g.O + (R + r) * g.ldO;
#pragma unroll
        for (int j = 0; j < OZ_N; ++j)
          if (j < nsd) {
            const int e = (eb[r] - 1022) + (ej[j] - 1022);
            const double h = (double)acc[j], l = (double)lo_s[r * (OZ_N + 1) + j];
            double v;
            if (e - 63 >= -1022 && e - 35 <= 1023)  // both scales are normal powers of two: exact products
              v = h * __longlong_as_double((long long)(e - 35 + 1023) << 52) +
                  l * __longlong_as_double((long long)(e - 63 + 1023) << 52);
            else
              v = ldexp(h, e - 35) + ldexp(l, e - 63);
            o[j] = v;
          }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
  }
  // no copy or MMA may be in flight when the CTA exits / frees its tensor memory
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (tid == 0 && last_bar != 0 && !mbar_drain(last_bar, last_par)) atomicExch(sflag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (tid == 0 && (!ok || *(volatile int*)sflag)) atomicExch(g.status, 1);
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(LC_TMEM_COLS));
}

// biased max exponent of each column (nsd <= 256 columns per block, rows ld
// values apart, nblk blocks sX apart) into E[col0 + block * nsd + s]
// (atomicMax; E must be zeroed first).  Thread t of a CTA keeps column
// t % nsd of the CTA's rows t / nsd, + rows per pass, ...: consecutive
// threads read consecutive values of a row.  Order-independent, hence
// deterministic.
__global__ void __launch_bounds__(256) k_col_maxexp(const double* X, int nblk, int64_t sX, int nsd, int ld, int64_t N,
                                                    int* E, int col0, const int* skip) {
  if (skip && *skip) return;
  __shared__ int smax[256];
  const int rpp = blockDim.x / nsd;  // rows per pass of one CTA
  const int c = threadIdx.x % nsd, rl = threadIdx.x / nsd;
  const int64_t rstep = (int64_t)gridDim.x * rpp;
  for (int b = 0; b < nblk; ++b) {
    const double* x = X + (int64_t)b * sX;
    for (int i = threadIdx.x; i < nsd; i += blockDim.x) smax[i] = 0;
    __syncthreads();
    int mx = 0;
    if (rl < rpp) {
#pragma unroll 4
      for (int64_t r = (int64_t)blockIdx.x * rpp + rl; r < N; r += rstep)
        mx = max(mx, (int)(((unsigned long long)__double_as_longlong(x[r * ld + c]) >> 52) & 0x7FF));
      if (mx > 0) atomicMax(&smax[c], mx);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nsd; i += blockDim.x)
      if (smax[i] > 0) atomicMax(&E[col0 + b * nsd + i], smax[i]);
    __syncthreads();
  }
}

// out[p] = sum over CTAs c = 0, 1, ... of partial[c][p], in that order
__global__ void k_oz_reduce(const double* partial, int ncta, int np, double* out, const int* skip) {
  if (skip && *skip) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < ncta; ++c) s += partial[(int64_t)c * np + p];
    out[p] = s;
  }
}

}  // namespace

void qp_oz_reduce(const double* partial, int ncta, int np, double* out, const int* skip, cudaStream_t st) {
  k_oz_reduce<<<(np + 127) / 128, 128, 0, st>>>(partial, ncta, np, out, skip);
}

// Opt-in shared memory of k_gram_oz on the current device (once per device).
int qp_gram_oz_prepare() {
  static int done[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  if (cudaFuncSetAttribute(k_gram_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_MAX) != cudaSuccess)
    return -1;
  done[dev] = 1;
  return 0;
}

void qp_col_maxexp(const double* X, int nblk, int64_t sX, int nsd, int ld, int64_t N, int* E, int col0,
                   const int* skip, cudaStream_t st, int n_sm) {
  k_col_maxexp<<<4 * n_sm, 256, 0, st>>>(X, nblk, sX, nsd, ld, N, E, col0, skip);
}

// X (m x nbc, row-major) = A^T [B0 B1] per CTA into partial[cta][m][nbc];
// A: m columns in blocks of nsdA (rows ldA apart, blocks sA apart); B0 (and
// B1): nsdB columns each, rows ldB apart; m <= 128, nbc <= 16.  Exponents eA
// (m), eB (nbc) from qp_col_maxexp.
void qp_gram_oz(const double* A, int64_t sA, int m, int nsdA, int ldA, const double* B0, const double* B1, int nbc,
                int nsdB, int ldB, int64_t N, const int* eA, const int* eB, double* partial, int ncta,
                const int* skip, int* status, cudaStream_t st) {
  OzArgs g;
  g.A = A;
  g.sA = sA;
  g.m = m;
  g.nsdA = nsdA;
  g.ldA = ldA;
  g.B0 = B0;
  g.B1 = B1;
  g.nbc = nbc;
  g.nsdB = nsdB;
  g.ldB = ldB;
  g.N = N;
  int64_t rpc = (N + ncta - 1) / ncta;
  rpc = (rpc + OZ_KC - 1) / OZ_KC * OZ_KC;
  g.rows_per_cta = rpc;
  g.eA = eA;
  g.eB = eB;
  g.partial = partial;
  g.skip = skip;
  g.status = status;
  // raw stages of OZ_KC rows of the m + nbc columns (256-byte aligned): as
  // many as fit beside the digit stages, up to OZ_MAXRAW
  const int rw = m + nbc;
  g.raw_stride = (OZ_KC * rw + 31) / 32 * 32;
  g.nraw = std::max(1, std::min(OZ_MAXRAW, (OZ_SMEM_MAX - 2 * OZ_STAGE - OZ_TAB) / (g.raw_stride * 8)));
  const int smem = 2 * OZ_STAGE + g.nraw * g.raw_stride * 8 + OZ_TAB;
  // rows per splitting task: the fewest rows per thread on the longest
  // thread's path (more, narrower stores only where that gains)
  int best = 1 << 30;
  g.rpt = 8;
  for (int r : {8, 4, 2}) {
    const int ntask = rw * (OZ_KC / r);
    const int cost = (ntask + OZ_SPLIT - 1) / OZ_SPLIT * r * 4 + (8 / r);
    if (cost < best) {
      best = cost;
      g.rpt = r;
    }
  }
  k_gram_oz<<<ncta, OZ_THREADS, smem, st>>>(g);
}


// Opt-in shared memory of k_lincomb_oz (once per device).
static int lincomb_oz_prepare() {
  static int done[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  if (cudaFuncSetAttribute(k_lincomb_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_MAX) != cudaSuccess)
    return -1;
  done[dev] = 1;
  return 0;
}

// O = [A_0 .. A_nb-1] C on the tensor cores (FP64-accurate); m = nb nsd <=
// 128, nsd <= 16.  Returns -1 when the shapes are outside the kernel's range
// (the caller keeps its FP64 path), else 0.
int qp_lincomb_oz(const double* A, int64_t sA, int m, int nsd, const double* C, double* O, int64_t ldO, int64_t N,
                  int ncta, const int* skip, int* status, cudaStream_t st) {
  if (m < 1 || m > LC_MAXM || nsd < 1 || nsd > OZ_N || m % nsd) return -1;
  if (lincomb_oz_prepare()) return -1;
  const int nks = (m + LC_KS - 1) / LC_KS;
  const int nb = m / nsd;
  // staged rows of an odd number of doubles (no shared-memory bank
  // conflicts between consecutive rows) when they fit, else unpadded
  auto need = [&](int rsd) {
    return 1024 + 2 * (size_t)LC_ASTAGE + (size_t)nks * LC_BCHUNK + (size_t)nb * LC_TM * rsd * 8 +
           (LC_TM + OZ_N) * 4 + 64;
  };
  int rsd = (nsd & 1) ? nsd : nsd + 1;
  if (need(rsd) > (size_t)OZ_SMEM_MAX) rsd = nsd;
  const size_t smem = need(rsd);
  if (smem > (size_t)OZ_SMEM_MAX) return -1;
  LcArgs g;
  g.A = A;
  g.sA = sA;
  g.m = m;
  g.nsd = nsd;
  g.C = C;
  g.O = O;
  g.ldO = ldO;
  g.N = N;
  int64_t rpc = (N + ncta - 1) / ncta;
  rpc = (rpc + LC_TM - 1) / LC_TM * LC_TM;
  g.rows_per_cta = rpc;
  g.row_stride = rsd;
  g.skip = skip;
  g.status = status;
  k_lincomb_oz<<<ncta, LC_THREADS, smem, st>>>(g);
  return 0;
}

extern "C" int qpgpu_gram_tc(qpgpu_ctx* c, const double* A, int64_t lda, int m, const double* B, int64_t ldb, int n,
                             int64_t N, double* X, void* stream) {
  if (!c) return QPGPU_ERR_ARG;
  if (!A || !B || !X || m < 1 || m > 128 || n < 1 || n > 16 || N < 1 || lda < m || ldb < n || lda > (1 << 30) ||
      ldb > (1 << 30))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "gram_tc: need 1 <= m <= 128, 1 <= n <= 16, N >= 1, lda >= m, ldb >= n");
  std::lock_guard<std::mutex> lk(c->mu);
  if (qp_gram_oz_prepare()) return qpgpu_fail(c, QPGPU_ERR_CUDA, "gram_tc: shared-memory opt-in failed");
  const int ncta = c->n_sm;
  const size_t need = (size_t)ncta * m * n * sizeof(double) + (size_t)(m + n + 8) * sizeof(int) + 256;
  if (c->tc_scratch_bytes < need) {
    dev_free(c->d_tc_scratch);
    c->d_tc_scratch = nullptr;
    c->tc_scratch_bytes = 0;
    QP_CUDA(c, cudaMalloc(&c->d_tc_scratch, need));
    c->tc_scratch_bytes = need;
  }
  double* part = (double*)c->d_tc_scratch;
  int* E = (int*)(part + (size_t)ncta * m * n);
  int* status = E + m + n;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  QP_CUDA(c, cudaMemsetAsync(E, 0, (m + n + 1) * sizeof(int), st));
  qp_col_maxexp(A, 1, 0, m, (int)lda, N, E, 0, nullptr, st, c->n_sm);
  qp_col_maxexp(B, 1, 0, n, (int)ldb, N, E + m, 0, nullptr, st, c->n_sm);
  qp_gram_oz(A, 0, m, m, (int)lda, B, nullptr, n, n, (int)ldb, N, E, E + m, part, ncta, nullptr, status, st);
  qp_oz_reduce(part, ncta, m * n, X, nullptr, st);
  int hs = 0;
  QP_CUDA(c, cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  if (hs) return qpgpu_fail(c, QPGPU_ERR_TIMEOUT, "gram_tc: a bounded tensor-core wait ran out");
  return QPGPU_OK;
}

extern "C" int qpgpu_lincomb_tc(qpgpu_ctx* c, const double* A, int64_t sA, int m, int nsd, const double* C, double* O,
                                int64_t ldO, int64_t N, void* stream) {
  if (!c) return QPGPU_ERR_ARG;
  if (!A || !C || !O || m < 1 || m > LC_MAXM || nsd < 1 || nsd > OZ_N || m % nsd || N < 1 || ldO < nsd ||
      (m > nsd && sA < N * nsd))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "lincomb_tc: need m = nb nsd <= 128, nsd <= 16, N >= 1, ldO >= nsd, sA >= N nsd");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->d_tc_scratch || c->tc_scratch_bytes < sizeof(int)) {
    dev_free(c->d_tc_scratch);
    c->d_tc_scratch = nullptr;
    c->tc_scratch_bytes = 0;
    QP_CUDA(c, cudaMalloc(&c->d_tc_scratch, 256));
    c->tc_scratch_bytes = 256;
  }
  int* status = (int*)c->d_tc_scratch;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  QP_CUDA(c, cudaMemsetAsync(status, 0, sizeof(int), st));
  if (qp_lincomb_oz(A, sA, m, nsd, C, O, ldO, N, c->n_sm, nullptr, status, st))
    return qpgpu_fail(c, QPGPU_ERR_CUDA, "lincomb_tc: shared-memory opt-in failed");
  QP_CUDA(c, cudaGetLastError());
  int hs = 0;
  QP_CUDA(c, cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  if (hs) return qpgpu_fail(c, QPGPU_ERR_TIMEOUT, "lincomb_tc: a bounded tensor-core wait ran out");
  return QPGPU_OK;
}
