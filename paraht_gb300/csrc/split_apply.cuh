// split_apply.cuh -- split-precision (emulated FP64) application of compact-WY op lists on the
// BF16 tensor cores.
//
// Every bulk update of the reduction is an ordered list of ops  C <- C - (C V) (T V^T)  applied
// to row strips of a matrix (a left op  C <- C - V T^T V^T C  on column-major C is the same op on
// C^T, so one kernel serves both, with the strides of C as parameters).  Here each op's two
// products are computed on the tensor cores from FP64 operands split into 8-bit digits:
//
//   x = 2^e * sum_{t=0}^{6} d_t 2^{-8(t+1)},  d_t integers in [-255, 255],
//
// with one power-of-two scale e per row of the left factor and per column of the right factor
// (fixed-point slicing, the Ozaki scheme; digits rounded to nearest, the leading one may reach
// 256).  A digit is exact in BF16, a digit product is exact in FP32 and so is every sum of them
// that the MMA forms for one level l = t+u over an inner chunk of 32 (|sum| < 2^24); the 34
// products with t+u <= 7 give each result as accurately as an FP64 dot product (about 2^-52 of
// row scale x column scale; the omitted levels are below 2^-64).  The levels are recombined exactly in int64 and turned
// into one FP64 value; C is updated in FP64.  The small operands (V's digits, W = T V^T and
// its digits) are prepared once per op by k_split_prep.
//
// Restrictions of this kernel: k <= 16 reflectors per op and an inner dimension len <= 64;
// the driver falls back to the FP64 kernels (wy_apply.cuh) otherwise.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "launch_count.h"
#include "paraht_internal.cuh"
#include "wy_apply.cuh"

namespace pht {

constexpr int kSpD = 7;         // digits per operand
constexpr int kSpLevels = 8;     // levels 0..7 kept (t+u <= 7)
constexpr int kSpMaxK = 16;      // reflectors per op
constexpr int kSpMaxLen = 64;    // inner dimension of the first product
constexpr int kSpRS = 64;        // rows of C per CTA (4 warps x 16)
constexpr int kSpThreads = 128;
constexpr int kSpLenPad = kSpMaxLen + 8;  // bf16 row pitch of len-indexed tiles (bank-conflict free)
constexpr int kSpKPad = kSpMaxK + 8;      // bf16 row pitch of k-indexed tiles

// Per-op prepared operands (global workspace, one slot per op of a launch).
struct SplitOpData {
  __nv_bfloat16 vd[kSpD][kSpMaxK][kSpLenPad];  // digits of V, [digit][m][c]  (B operand of C V)
  __nv_bfloat16 wd[kSpD][kSpMaxLen][kSpKPad];  // digits of W = T V^T, [digit][c][m] (B operand of X W)
  int fv[kSpMaxK];                             // column scales of V
  int fw[kSpMaxLen];                           // column scales of W
};

// Integer bit-pattern helpers.  On GB300 every FP64 instruction (including compare, min/max
// and conversions) issues at 1/64 of the FP32 rate, so the split path does its bookkeeping on
// the integer pipe: |x| and max|x| on the bit patterns (non-negative doubles order like their
// patterns), exponents from the exponent field, and exact int <-> float conversions by hand.
PHT_DEV uint64_t abs_bits(double x) { return (uint64_t)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull; }

// Exponent e with |x| < 2^e for the largest |x|, from its bit pattern (0 -> -1000).
PHT_DEV int scale_exp_bits(uint64_t amax_bits) {
  const int ex = (int)(amax_bits >> 52);
  return ex == 0 ? -1000 : ex - 1022;  // |x| = 1.m 2^(ex-1023) < 2^(ex-1022)
}
PHT_DEV int scale_exp(double amax) { return scale_exp_bits(abs_bits(amax)); }

// An FP32 value holding an exact integer |v| < 2^24 -> int (integer pipe only).
PHT_DEV int f32_exact_int(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t mag = b & 0x7FFFFFFFu;
  const int ex = (int)(mag >> 23);
  int v = 0;
  if (ex >= 127) v = (int)(((mag & 0x7FFFFFu) | 0x800000u) >> (150 - ex));  // 1 <= |f| < 2^24
  return (b >> 31) ? -v : v;
}

// double(N) * 2^s for |N| < 2^53 (exact), built on the integer pipe; 0 for N = 0.
PHT_DEV double ll_to_double_scaled(long long N, int s) {
  if (N == 0) return 0.0;
  const uint64_t sign = (uint64_t)N & 0x8000000000000000ull;
  const uint64_t a = (uint64_t)(N < 0 ? -N : N);
  const int msb = 63 - __clzll((long long)a);  // <= 52
  const uint64_t mant = (a << (52 - msb)) & 0xFFFFFFFFFFFFFull;
  const long long ex = (long long)msb + 1023 + s;
  if (ex <= 0) return 0.0;  // below the normal range: negligible at the scales used here
  return __longlong_as_double((long long)(sign | ((uint64_t)ex << 52) | mant));
}

// 8-bit digit t (0..6) of |x| * 2^{-e}, as a signed BF16 bit pattern (the leading digit, t = 0,
// is not masked: rounding may carry it to 256).
PHT_DEV uint16_t digit_bf16(uint64_t F, int t, bool neg) {
  const uint32_t d = t == 0 ? (uint32_t)(F >> 48) : (uint32_t)(F >> (48 - 8 * t)) & 0xFFu;
  // exact float of d (d < 2^23): OR into 2^23 and subtract 2^23; d <= 255 has at most 8
  // significant bits so the upper 16 bits of the float are exactly its BF16 value
  const float f = __int_as_float(0x4B000000 | d) - 8388608.0f;
  uint32_t b = (uint32_t)__float_as_int(f) >> 16;
  if (neg && d) b |= 0x8000u;
  return (uint16_t)b;
}

// |x| * 2^(56 - e) rounded to the nearest integer (|x| < 2^e): 56 fractional bits hold the
// 7 digits.
PHT_DEV uint64_t fixed56(double x, int e) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);  // sign handled by the caller (bit 63)
  if (ex == 0 || e <= -1000) return 0;  // zero (and denormals, far below any scale used here)
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int s = ex - 1018 - e;  // |x| = m 2^(ex-1075);  F57 = m 2^(ex-1075+57-e), one extra bit
  uint64_t f57;
  if (s >= 0)
    f57 = m << s;  // s <= 4 since |x| < 2^e
  else if (s <= -64)
    f57 = 0;
  else
    f57 = m >> (-s);
  return (f57 + 1) >> 1;
}

PHT_DEV double pow2(int s) {  // 2^s for -1022 <= s <= 1023
  return __longlong_as_double((long long)(s + 1023) << 52);
}

// Exact recombination of the 8 level sums (FP32 values that are exact integers):
//   sum_l 2^{-8l} a_l = 2^{-24} Nh + 2^{-56} Nl,  Nh = a0 2^24 + a1 2^16 + a2 2^8 + a3,
//   Nl = a4 2^24 + a5 2^16 + a6 2^8 + a7  (int64, added into the running sums; both stay below
//   2^53 and convert to double exactly).
// Level sums are exact while |a_l| < 2^24: at most 7 digit pairs x 32 inner terms x 256*255.
PHT_DEV void add_levels(const float* a, long long& Nh, long long& Nl) {
  const long long n0 = f32_exact_int(a[0]), n1 = f32_exact_int(a[1]), n2 = f32_exact_int(a[2]),
                  n3 = f32_exact_int(a[3]);
  const long long n4 = f32_exact_int(a[4]), n5 = f32_exact_int(a[5]), n6 = f32_exact_int(a[6]),
                  n7 = f32_exact_int(a[7]);
  Nh += (n0 << 24) + (n1 << 16) + (n2 << 8) + n3;
  Nl += (n4 << 24) + (n5 << 16) + (n6 << 8) + n7;
}

PHT_DEV void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------------------------------------
// Preparation: one CTA per op.  V digits (per column m), W = T V^T (FP64, k x len), W digits
// (per column c).  Columns/rows beyond (len, k) are zero.
// ------------------------------------------------------------------------------------------
template <class Geo>
__global__ void __launch_bounds__(128) k_split_prep(Geo g, SplitOpData* out) {
  __shared__ double Ws[kSpMaxK][kSpMaxLen + 1];
  const int slot = blockIdx.x;
  const WYOp op = g.op(g.slot_op(slot));
  SplitOpData* D = out + slot;
  const int t = threadIdx.x;
  const int len = (op.len > 0 && op.k > 0) ? op.len : 0, k = (op.len > 0) ? op.k : 0;
  // V digits, column scale over the column's len entries
  for (int m = t; m < kSpMaxK; m += blockDim.x) {
    uint64_t amax = 0;
    for (int c = 0; c < len && m < k; ++c) amax = max(amax, abs_bits(op.V[(size_t)m * op.ldv + c]));
    const int e = scale_exp_bits(amax);
    D->fv[m] = e;
    for (int c = 0; c < kSpMaxLen; ++c) {
      const double x = (m < k && c < len) ? op.V[(size_t)m * op.ldv + c] : 0.0;
      const uint64_t F = fixed56(x, e);
      const bool neg = __double_as_longlong(x) < 0;
      for (int d = 0; d < kSpD; ++d) {
        const uint16_t b = digit_bf16(F, d, neg);
        D->vd[d][m][c] = __ushort_as_bfloat16(b);
      }
    }
  }
  // W = T V^T :  W[m][c] = sum_l T[l][m]^T ... = sum_l T[m][l] V[c][l]
  for (int e = t; e < kSpMaxK * kSpMaxLen; e += blockDim.x) {
    const int m = e % kSpMaxK, c = e / kSpMaxK;
    double s = 0.0;
    if (m < k && c < len)
      for (int l = 0; l < k; ++l) s = fma(op.T[m + (size_t)l * op.ldt], op.V[c + (size_t)l * op.ldv], s);
    Ws[m][c] = s;
  }
  __syncthreads();
  for (int c = t; c < kSpMaxLen; c += blockDim.x) {
    uint64_t amax = 0;
    for (int m = 0; m < kSpMaxK; ++m) amax = max(amax, abs_bits(Ws[m][c]));
    const int e = scale_exp_bits(amax);
    D->fw[c] = e;
    for (int m = 0; m < kSpMaxK; ++m) {
      const double x = Ws[m][c];
      const uint64_t F = fixed56(x, e);
      const bool neg = __double_as_longlong(x) < 0;
      for (int d = 0; d < kSpD; ++d) D->wd[d][c][m] = __ushort_as_bfloat16(digit_bf16(F, d, neg));
    }
    for (int m = kSpMaxK; m < kSpKPad; ++m)
      for (int d = 0; d < kSpD; ++d) D->wd[d][c][m] = __ushort_as_bfloat16(0);
  }
}

// ------------------------------------------------------------------------------------------
// Application: one CTA per strip of kSpRS rows of the (possibly transposed) matrix C, addressed
// as C[row * rs + col * cs].  For every op of the list that touches the strip:
//   X = C_sub V (RS x k), X <- digits, C_sub -= X W.
// ------------------------------------------------------------------------------------------
struct SplitSmem {
  double c[kSpRS][kSpMaxLen + 1];                // C tile (FP64)
  __nv_bfloat16 cd[kSpD][kSpRS][kSpLenPad];      // digits of the C tile
  __nv_bfloat16 vd[kSpD][kSpMaxK][kSpLenPad];    // digits of V
  __nv_bfloat16 wd[kSpD][kSpMaxLen][kSpKPad];    // digits of W
  __nv_bfloat16 xd[kSpD][kSpRS][kSpKPad];        // digits of X
  int erow[kSpRS];                               // row scales of C
  int xrow[kSpRS];                               // row scales of X
  int fv[kSpMaxK];
  int fw[kSpMaxLen];
};

template <class Geo>
__global__ void __launch_bounds__(kSpThreads) k_split_apply(double* __restrict__ C, long long rs, long long cs,
                                                           int row0, int row1, Geo g,
                                                           const SplitOpData* __restrict__ prep) {
  extern __shared__ __align__(16) unsigned char smraw[];
  SplitSmem& S = *reinterpret_cast<SplitSmem*>(smraw);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int gq = lane >> 2, tq = lane & 3;  // mma groupID, thread-in-group
  const int rbeg = row0 + blockIdx.x * kSpRS;
  if (rbeg > row1) return;
  const int rend = min(row1, rbeg + kSpRS - 1);
  const int nops = g.count();
  for (int o = 0; o < nops; ++o) {
    const WYOp op = g.op(o);
    const int ra = max(rbeg, op.lo), rb = min(rend, op.hi);
    if (ra > rb || op.k <= 0 || op.len <= 0) continue;
    const int h = rb - ra + 1, len = op.len;
    __syncthreads();
    // ---- load C tile (zero padded) and the op's prepared digits ----
    for (int e = t; e < kSpRS * kSpMaxLen; e += blockDim.x) {
      int rr, cc;
      if (cs == 1) {  // columns of the tile contiguous in memory
        cc = e % kSpMaxLen;
        rr = e / kSpMaxLen;
      } else {
        rr = e % kSpRS;
        cc = e / kSpRS;
      }
      S.c[rr][cc] = (rr < h && cc < len) ? C[(long long)(ra + rr) * rs + (long long)(op.start + cc) * cs] : 0.0;
    }
    if (op.k == 1) {
      // single reflector (c <- c - tau (c.v) v^T): FP64 in place, two threads per row
      __syncthreads();
      const int rr = t >> 1, half = t & 1;
      const double tau = op.T[0];
      double sdot = 0.0;
      for (int cc = half; cc < len; cc += 2) sdot = fma(S.c[rr][cc], op.V[cc], sdot);
      sdot += __shfl_xor_sync(0xffffffffu, sdot, 1);
      sdot *= tau;
      for (int cc = half; cc < len; cc += 2) S.c[rr][cc] = fma(-sdot, op.V[cc], S.c[rr][cc]);
    } else {
    const SplitOpData* P = prep + g.op_slot(o);
    {
      const uint4* src = reinterpret_cast<const uint4*>(P->vd);
      uint4* dst = reinterpret_cast<uint4*>(S.vd);
      for (int e = t; e < (int)(sizeof(S.vd) / 16); e += blockDim.x) dst[e] = src[e];
      const uint4* src2 = reinterpret_cast<const uint4*>(P->wd);
      uint4* dst2 = reinterpret_cast<uint4*>(S.wd);
      for (int e = t; e < (int)(sizeof(S.wd) / 16); e += blockDim.x) dst2[e] = src2[e];
      for (int e = t; e < kSpMaxK; e += blockDim.x) S.fv[e] = P->fv[e];
      for (int e = t; e < kSpMaxLen; e += blockDim.x) S.fw[e] = P->fw[e];
    }
    __syncthreads();
    // ---- row scales of C and its digits (2 threads per row) ----
    {
      const int rr = t >> 1, half = t & 1;
      uint64_t amax = 0;
      for (int cc = half; cc < kSpMaxLen; cc += 2) amax = max(amax, abs_bits(S.c[rr][cc]));
      const uint64_t other = (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 1);
      amax = max(amax, other);
      const int e = scale_exp_bits(amax);
      if (half == 0) S.erow[rr] = e;
      for (int cc = half; cc < kSpMaxLen; cc += 2) {
        const double x = S.c[rr][cc];
        const uint64_t F = fixed56(x, e);
        const bool neg = __double_as_longlong(x) < 0;
#pragma unroll
        for (int d = 0; d < kSpD; ++d) S.cd[d][rr][cc] = __ushort_as_bfloat16(digit_bf16(F, d, neg));
      }
    }
    __syncthreads();
    const int m0 = warp * 16;  // this warp's 16 rows
    // ---- X = C V : levels acc[level][ntile(2)][4], summed exactly in int64 per 32-column chunk ----
    long long xh[2][2][2], xl[2][2][2];  // [hh][nt][j]
#pragma unroll
    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) xh[hh][nt][j] = xl[hh][nt][j] = 0;
    for (int kc = 0; kc < len; kc += 32) {
    float acc[kSpLevels][2][4];
#pragma unroll
    for (int l = 0; l < kSpLevels; ++l)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[l][nt][q] = 0.f;
    const int kend = min(len, kc + 32);
    for (int k0 = kc; k0 < kend; k0 += 16) {
#pragma unroll
      for (int ta = 0; ta < kSpD; ++ta) {
        const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&S.cd[ta][m0 + gq][k0 + 2 * tq]);
        const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&S.cd[ta][m0 + gq + 8][k0 + 2 * tq]);
        const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&S.cd[ta][m0 + gq][k0 + 2 * tq + 8]);
        const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&S.cd[ta][m0 + gq + 8][k0 + 2 * tq + 8]);
#pragma unroll
        for (int ub = 0; ub < kSpD; ++ub) {
          if (ta + ub >= kSpLevels) continue;
#pragma unroll
          for (int nt = 0; nt < 2; ++nt) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&S.vd[ub][nt * 8 + gq][k0 + 2 * tq]);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&S.vd[ub][nt * 8 + gq][k0 + 2 * tq + 8]);
            mma_bf16(acc[ta + ub][nt], a0, a1, a2, a3, b0, b1);
          }
        }
      }
    }
    // element (row m0+gq+8*hh, col nt*8+2*tq+j) <- acc[.][nt][2*hh+j]
#pragma unroll
    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          float lv[kSpLevels];
#pragma unroll
          for (int l = 0; l < kSpLevels; ++l) lv[l] = acc[l][nt][2 * hh + j];
          add_levels(lv, xh[hh][nt][j], xl[hh][nt][j]);
        }
    }
    // ---- X (FP64) = (Nh 2^-24 + Nl 2^-56) 2^(er + fv - 16); X row scales; X digits ----
    double xv[2][2][2];  // [hh][nt][j]
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int rr = m0 + gq + 8 * hh;
      const int er = S.erow[rr];
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int m = nt * 8 + 2 * tq + j;
          const int sc = er + S.fv[m] - 16;
          // hi + lo in one rounding: lo is exact and far below hi's ulp except when hi is 0
          xv[hh][nt][j] = (er <= -1000 || S.fv[m] <= -1000)
                              ? 0.0
                              : ll_to_double_scaled(xh[hh][nt][j], sc - 24) + ll_to_double_scaled(xl[hh][nt][j], sc - 56);
        }
    }
    // row max of X over its 16 columns (4 lanes of a group share the row)
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      uint64_t amax = max(max(abs_bits(xv[hh][0][0]), abs_bits(xv[hh][0][1])),
                          max(abs_bits(xv[hh][1][0]), abs_bits(xv[hh][1][1])));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 1));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 2));
      const int e = scale_exp_bits(amax);
      const int rr = m0 + gq + 8 * hh;
      if (tq == 0) S.xrow[rr] = e;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int m = nt * 8 + 2 * tq + j;
          const double x = xv[hh][nt][j];
          const uint64_t F = fixed56(x, e);
          const bool neg = __double_as_longlong(x) < 0;
#pragma unroll
          for (int d = 0; d < kSpD; ++d) S.xd[d][rr][m] = __ushort_as_bfloat16(digit_bf16(F, d, neg));
        }
    }
    __syncwarp();
    // ---- C_sub -= X W, 16 columns (2 n-tiles) at a time ----
    for (int c0 = 0; c0 < len; c0 += 16) {
      float a2c[kSpLevels][2][4];
#pragma unroll
      for (int l = 0; l < kSpLevels; ++l)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) a2c[l][nt][q] = 0.f;
#pragma unroll
      for (int ta = 0; ta < kSpD; ++ta) {
        const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&S.xd[ta][m0 + gq][2 * tq]);
        const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&S.xd[ta][m0 + gq + 8][2 * tq]);
        const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&S.xd[ta][m0 + gq][2 * tq + 8]);
        const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&S.xd[ta][m0 + gq + 8][2 * tq + 8]);
#pragma unroll
        for (int ub = 0; ub < kSpD; ++ub) {
          if (ta + ub >= kSpLevels) continue;
#pragma unroll
          for (int nt = 0; nt < 2; ++nt) {
            const int n0 = c0 + nt * 8;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&S.wd[ub][n0 + gq][2 * tq]);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&S.wd[ub][n0 + gq][2 * tq + 8]);
            mma_bf16(a2c[ta + ub][nt], a0, a1, a2, a3, b0, b1);
          }
        }
      }
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int rr = m0 + gq + 8 * hh;
        const int er = S.xrow[rr];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int cc = c0 + nt * 8 + 2 * tq + j;
            if (cc >= len || er <= -1000 || S.fw[cc] <= -1000) continue;
            float lv[kSpLevels];
#pragma unroll
            for (int l = 0; l < kSpLevels; ++l) lv[l] = a2c[l][nt][2 * hh + j];
            long long nh = 0, nl = 0;
            add_levels(lv, nh, nl);
            const int sc = er + S.fw[cc] - 16;
            S.c[rr][cc] -= ll_to_double_scaled(nh, sc - 24) + ll_to_double_scaled(nl, sc - 56);
          }
      }
    }
    }  // compact-WY op
    __syncthreads();
    // ---- store the tile ----
    for (int e = t; e < kSpRS * kSpMaxLen; e += blockDim.x) {
      int rr, cc;
      if (cs == 1) {
        cc = e % kSpMaxLen;
        rr = e / kSpMaxLen;
      } else {
        rr = e % kSpRS;
        cc = e / kSpRS;
      }
      if (rr < h && cc < len) C[(long long)(ra + rr) * rs + (long long)(op.start + cc) * cs] = S.c[rr][cc];
    }
  }
}

inline size_t split_apply_smem() { return sizeof(SplitSmem); }

// Whether every op of a list fits this kernel (checked by the caller from the parameters).
inline bool split_fits(int k_max, int len_max) { return k_max <= kSpMaxK && len_max <= kSpMaxLen; }

// Prepares the op list's compact-WY ops (nops slots of `prep`, Geo::slot_op) and applies it to rows [row0, row1] of C viewed
// with strides (rs, cs).
template <class Geo>
inline void launch_split_apply(double* C, long long rs, long long cs, int row0, int row1, const Geo& g, int nops,
                               SplitOpData* prep, cudaStream_t s) {
  if (row1 < row0 || nops <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_split_apply<Geo>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)split_apply_smem());
    attr = true;
  }
  count_launch(2);
  k_split_prep<Geo><<<nops, 128, 0, s>>>(g, prep);
  const int nblk = (row1 - row0 + 1 + kSpRS - 1) / kSpRS;
  k_split_apply<Geo><<<nblk, kSpThreads, split_apply_smem(), s>>>(C, rs, cs, row0, row1, g, prep);
}

// FP64 or split-precision application of an op list, chosen per launch site.
// Left ops act on column strips of X; they are right ops on X^T (rows = columns of X).
template <class Geo>
inline void apply_left_any(void* split_slots, double* X, int ldx, int col0, int col1, const Geo& g, int nops,
                           cudaStream_t s) {
  if (split_slots)
    launch_split_apply(X, (long long)ldx, 1LL, col0, col1, g, nops, (SplitOpData*)split_slots, s);
  else
    launch_apply_left(X, ldx, col0, col1, g, s);
}
template <class Geo>
inline void apply_right_any(void* split_slots, double* X, int ldx, int row0, int row1, const Geo& g, int nops,
                            cudaStream_t s) {
  if (split_slots)
    launch_split_apply(X, 1LL, (long long)ldx, row0, row1, g, nops, (SplitOpData*)split_slots, s);
  else
    launch_apply_right(X, ldx, row0, row1, g, s);
}

}  // namespace pht
