// wy_stream.cuh -- split-precision (emulated FP64) application of a whole compact-WY op list to
// row strips that stay on chip for the length of the list.
//
// Every bulk update of the reduction is an ordered list of ops  C <- C - (C V) T V^T  on a
// strip view of a matrix (left ops act on C^T, see split_fits / apply_*_any).  Consecutive ops
// of a list overlap in their column spans, so one CTA keeps the rows of its strip resident in
// shared memory for the whole list, fetching each column the first time an op needs it and
// writing it back when it leaves the window or the list ends.
//
// Number format.  A resident row is held in fixed point, int64 values v with x = v 2^(e-62) for
// a per-row scale e, set 5 bits above the largest magnitude loaded (|v| < 2^57) and raised (all
// resident values shifted) when a larger value is loaded.  Each op is orthogonal on its span, so
// its results are bounded by the 2-norm of its inputs, at most 8 (= sqrt(64)) times their
// largest value; before every op a row whose largest value among the op's columns has reached
// 2^58 is shifted down to below 2^57, so no value ever reaches 2^62.  The spacing 2^(e-62) is
// 2^-56 of the row's largest loaded element, finer than FP64's 2^-53 at that magnitude.
//
// Products.  Each op is two exact digit products on the tensor cores (mma.sync m16n8k16,
// FP16 inputs, FP32 accumulation), X = C V and C -= X W with W = T V^T formed once per op, or
// three, X = C V, Y = X T, C -= Y V^T, for lists that mask Y (below).  Operands are split into
// 8 digits of 7 bits (x = 2^e sum_t d_t 2^{-7(t+1)}, |d_t| <= 128, one power-of-two scale per
// row of the left and per column of the right factor, the Ozaki scheme); the 43 digit pairs
// with t+u <= 8 are accumulated per level l = t+u exactly in FP32 over at most 32 inner terms
// (|a_l| < 2^22), in accumulators biased by 1.5 2^23 so that each level is read off the FP32
// bit pattern with one integer subtraction, and recombined exactly in int64/int128.  The
// omitted levels (t+u >= 9) are below 2^-60 of row scale x column scale per inner term, so an
// element much smaller than its row's largest still gets about FP64 accuracy.  X and Y are rounded to 56-bit digits before the next product; C's
// correction is added in integer arithmetic.  There is no FP64 instruction in the op loop
// (on GB300 each FP64 warp instruction occupies a scheduler's FP64 pipe for about 64 cycles).
// The digits of C, X and Y are formed in registers, directly in the MMA fragment layout.
//
// Reflector masks.  An op may apply a different contiguous subset [a, b] of its k reflectors to
// each row (the staircase single reflectors of stage 2, src/rht2ht.f90:1644-1661, 1818-1844,
// 1894-1920): for a forward T, H_a ... H_b = I - V_{a:b} T_{a:b,a:b} V_{a:b}^T, which is
// obtained by zeroing X outside [a, b] and Y outside [a, b].  Geo::range supplies [a, b].  When
// every range ends at the last reflector (b = k-1) zeroing X suffices (T is upper triangular, so
// Y vanishes before a), and the two-product form applies; Geo::masks_y selects the three-product
// form.
//
// One-product forms.  Lists whose ops all apply every reflector to every row take C -= C M with
// M = V T V^T (formed once per op, span <= 32); the dense ops of the Givens stage 2 (V = I,
// M = I - G, an accumulated block of rotations) take the same form, up to 48 wide in lists of
// their own (WsOpMW operands; the level sums are taken out after 32 inner terms).
//
// Limits: k <= 16 reflectors, span len <= 64 per op; dense ops len <= 48.
#pragma once
#include <cuda_fp16.h>
#include <stddef.h>
#include <stdint.h>

#include <type_traits>

#include "launch_count.h"
#include "paraht_internal.cuh"

namespace pht {

constexpr int kWsD = 8;            // digits per operand (7 bits each)
constexpr int kWsLv = 9;           // levels kept (t + u <= 8)
constexpr int kWsK = 16;           // reflectors per op
constexpr int kWsLen = 64;         // span per op
constexpr int kWsWarps = 4;        // 16 strip rows per warp
constexpr int kWsRows = 16 * kWsWarps;
constexpr int kWsThreads = 32 * kWsWarps;
constexpr int kWsCW = 64;          // resident column slots per row (slot = column mod kWsCW)
constexpr int kWsPL = kWsLen + 8;  // fp16 pitch of len-indexed digit rows (conflict-free)
constexpr int kWsPK = kWsK + 8;    // fp16 pitch of k-indexed digit rows
constexpr int kWsMM = 32;          // largest span with the one-product form C -= C M
constexpr int kWsPM = kWsMM + 8;   // fp16 pitch of M's digit rows
constexpr int kWsMW = 48;          // largest dense op of the wide one-product form
constexpr int kWsPMW = kWsMW + 8;  // fp16 pitch of its digit rows
constexpr int kWsHead = 5;         // headroom bits of the row scale at load time
constexpr int kWsGuard = 57;       // a row is shifted down before an op when a value passes 2^57
constexpr int kWsNoScale = -2000;  // row scale not set yet (no nonzero value loaded)

// Operand digits of one op, prepared once per op (k_ws_prep) and copied to shared memory.  In the
// two-product form vt/fvt hold W = T V^T by columns of W and td is unused; mt/fm (lists without
// Y masks, len <= kWsMM) hold M = V W.
struct WsOpDigits {
  // C -= C M, M = V T V^T (len <= kWsMM): the whole op as one product (first: copied alone)
  uint16_t mt[kWsD][kWsMM][kWsPM];   // M   [c_out][c_in]: B operand of C M
  int fm[kWsMM];                     // scale of column c_out of M
  uint16_t vd[kWsD][kWsK][kWsPL];    // V   [m][c]: B operand of C V (FP16 bit patterns)
  uint16_t td[kWsD][kWsK][kWsPK];    // T   [m][l]: B operand of X T
  uint16_t vt[kWsD][kWsLen][kWsPK];  // V^T [c][m]: B operand of Y V^T
  int fv[kWsK];                           // scale of column m of V
  int ft[kWsK];                           // scale of column m of T
  int fvt[kWsLen];                        // scale of row c of V
};

// Operands of a dense op of a wide list (Geo::wide_dense(): every op dense, len <= kWsMW), written
// over the op's WsOpDigits slot.
struct WsOpMW {
  uint16_t mt[kWsD][kWsMW][kWsPMW];  // M [c_out][c_in]
  int fm[kWsMW];                     // scale of column c_out of M
};
static_assert(sizeof(WsOpMW) <= sizeof(WsOpDigits), "a wide op fits its slot");
static_assert(sizeof(WsOpMW) % 16 == 0, "copied in 16-byte words");

// ------------------------------------------------------------------------------------------
// Integer helpers (no FP64 pipe)
// ------------------------------------------------------------------------------------------
typedef unsigned __int128 u128;

PHT_DEV uint64_t ws_abs_bits(double x) { return (uint64_t)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull; }

// e with |x| < 2^e for the largest |x| given by its bit pattern (0 -> kWsNoScale)
PHT_DEV int ws_exp_bits(uint64_t amax_bits) {
  const int ex = (int)(amax_bits >> 52);
  return ex == 0 ? kWsNoScale : ex - 1022;
}

PHT_DEV int ws_bitlen(u128 a) {
  const uint64_t hi = (uint64_t)(a >> 64), lo = (uint64_t)a;
  if (hi) return 128 - __clzll((long long)hi);
  return lo ? 64 - __clzll((long long)lo) : 0;
}

// round(a 2^s) (round half up), for results below 2^64
PHT_DEV uint64_t ws_scale_u(u128 a, int s) {
  if (s >= 0) return s >= 64 ? 0 : (uint64_t)(a << s);
  if (s <= -128) return 0;
  return (uint64_t)((a + ((u128)1 << (-s - 1))) >> (-s));
}

// FP64 x -> round(x 2^(62-e)) as int64 (|x| < 2^e), integer operations only
PHT_DEV long long ws_to_fixed(double x, int e) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0 || e == kWsNoScale) return 0;  // zero (and denormals, far below any row scale)
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  // x = m 2^(ex-1075);  v = m 2^(ex-1075+62-e)
  const uint64_t v = ws_scale_u((u128)m, ex - 1013 - e);
  return (b >> 63) ? -(long long)v : (long long)v;
}

// int64 v -> FP64 of v 2^(e-62), rounded to nearest (ties away), integer operations only
PHT_DEV double ws_from_fixed(long long v, int e) {
  if (v == 0 || e == kWsNoScale) return 0.0;
  const uint64_t sign = (uint64_t)v & 0x8000000000000000ull;
  uint64_t a = (uint64_t)(v < 0 ? -v : v);
  int msb = 63 - __clzll((long long)a);  // value = a 2^(e-62), a in [2^msb, 2^(msb+1))
  uint64_t mant;
  if (msb > 52) {
    const int sh = msb - 52;
    mant = (a + (1ull << (sh - 1))) >> sh;
    if (mant >> 53) {  // rounding carried into a new bit
      mant >>= 1;
      ++msb;
    }
  } else {
    mant = a << (52 - msb);
  }
  const long long ex = (long long)msb + e - 62 + 1023;
  if (ex <= 0) return 0.0;  // below the normal range
  return __longlong_as_double((long long)(sign | ((uint64_t)ex << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// digit t (0..7) of a 56-bit rounded magnitude F: t = 0 takes bits 49..56 (rounding may carry
// it to 128), t >= 1 bits 49-7t .. 55-7t
PHT_DEV uint32_t ws_dig(uint64_t F, int t) {
  return t == 0 ? (uint32_t)(F >> 49) : (uint32_t)(F >> (49 - 7 * t)) & 0x7Fu;
}
// FP16 bit patterns of two digits (d <= 128) with signs: 1024 + d is exact in FP16 (0x6400 | d),
// one packed subtraction of 1024 leaves d exactly
PHT_DEV uint32_t ws_h2(uint32_t dlo, uint32_t dhi, bool nlo, bool nhi) {
  uint32_t v = dlo | (dhi << 16) | 0x64006400u;
  __half2 h = *reinterpret_cast<__half2*>(&v);
  h = __hsub2(h, __halves2half2(__ushort_as_half((unsigned short)0x6400), __ushort_as_half((unsigned short)0x6400)));
  const uint32_t r = *reinterpret_cast<uint32_t*>(&h);
  return r ^ ((nlo ? 0x8000u : 0u) | (nhi ? 0x80000000u : 0u));
}
PHT_DEV uint16_t ws_h1(uint32_t d, bool neg) { return (uint16_t)ws_h2(d, 0, neg, false); }

// Level accumulators start at 1.5 2^23: while |a_l| < 2^22 every partial sum is an exact
// integer in [2^22, 2^24) and the FP32 bit pattern is a_l + 0x4B400000.
constexpr float kWsMagic = 12582912.0f;
PHT_DEV int ws_lv(float f) { return __float_as_int(f) - 0x4B400000; }

// sum_l a_l 2^{-7l} = 2^{-21} Nh + 2^{-56} Nl (levels 0-3 in Nh, 4-8 in Nl), accumulated exactly;
// a_l read from the biased accumulators (|a_l| <= 8 pairs x 32 terms x 128 x 127 < 2^22)
PHT_DEV void ws_add_levels(const float* a, long long& Nh, long long& Nl) {
  Nh += ((long long)ws_lv(a[0]) << 21) + ((long long)ws_lv(a[1]) << 14) + ((long long)ws_lv(a[2]) << 7) + ws_lv(a[3]);
  Nl += ((long long)ws_lv(a[4]) << 28) + ((long long)ws_lv(a[5]) << 21) + ((long long)ws_lv(a[6]) << 14) +
        ((long long)ws_lv(a[7]) << 7) + ws_lv(a[8]);
}

// (Nh 2^35 + Nl) as a signed 128-bit integer: the product is 2^(e_left + e_right - 70) times it
PHT_DEV __int128 ws_join(long long Nh, long long Nl) { return ((__int128)Nh << 35) + (__int128)Nl; }

PHT_DEV void ws_mma(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

PHT_DEV uint32_t ws_ld32(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// ------------------------------------------------------------------------------------------
// Preparation: one CTA (128 threads) per op slot.  V and T are staged in shared memory; digits
// (rounded, 8 x 7 bits) of V by columns, of W = T V^T (two-product form) or of V^T and T by
// columns; entries beyond (len, k) are zero.
// ------------------------------------------------------------------------------------------
PHT_DEV void ws_put_digits(uint16_t* dst, int stride, double x, int e) {  // dst[d * stride]
  const long long v = ws_to_fixed(x, e);
  const uint64_t F56 = ((uint64_t)(v < 0 ? -v : v) + 32) >> 6;
  const bool neg = __double_as_longlong(x) < 0;
#pragma unroll
  for (int d = 0; d < kWsD; ++d) dst[(size_t)d * stride] = ws_h1(ws_dig(F56, d), neg);
}

template <class Geo>
__global__ void __launch_bounds__(128) k_ws_prep(Geo g, WsOpDigits* out) {
  __shared__ double Vs[kWsLen][kWsK + 1];  // V[c][m]
  __shared__ double Tsh[kWsK][kWsK + 1];   // T[l][m]
  __shared__ double Wsh[kWsK][kWsLen + 1]; // W[m][c] (two-product form)
  __shared__ double Msh[kWsMW][kWsMW + 1]; // M[c_in][c_out] = V W (one-product forms)
  __shared__ int sc[kWsLen];
  __shared__ int scv[kWsK];  // V's column scales (sc is reused for M's and W's columns)
  const int slot = blockIdx.x;
  const WYOp op = g.op(g.slot_op(slot));
  WsOpDigits* D = out + slot;
  const int t = threadIdx.x;
  const bool live = op.len > 0 && op.k > 0;
  const int len = live ? op.len : 0, k = live ? op.k : 0;
  const bool two = !g.masks_y();
  if (op.dense) {
    // C -= C M with M = T = I - G given explicitly (one-product forms only): width kWsMM, or
    // kWsMW in the WsOpMW layout for a wide list
    const bool wide = g.wide_dense();
    const int mw = wide ? kWsMW : kWsMM, pm = wide ? kWsPMW : kWsPM;
    uint16_t* mt = wide ? &reinterpret_cast<WsOpMW*>(D)->mt[0][0][0] : &D->mt[0][0][0];
    int* fm = wide ? reinterpret_cast<WsOpMW*>(D)->fm : D->fm;
    for (int e = t; e < mw * mw; e += 128) {
      const int ci = e % mw, co = e / mw;
      Msh[ci][co] = (ci < len && co < len) ? op.T[ci + (size_t)co * op.ldt] : 0.0;
    }
    __syncthreads();
    for (int co0 = 0; co0 < mw; co0 += 32) {  // scales of M's columns: 4 lanes per column
      const int co = co0 + (t >> 2), part = t & 3;
      uint64_t amax = 0;
      if (co < mw)
        for (int c = part; c < mw; c += 4) amax = max(amax, ws_abs_bits(Msh[c][co]));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 1));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 2));
      if (part == 0 && co < mw) {
        fm[co] = ws_exp_bits(amax);
        sc[co] = ws_exp_bits(amax);
      }
    }
    __syncthreads();
    for (int e = t; e < mw * pm; e += 128) {
      const int co = e / pm, ci2 = e % pm;
      ws_put_digits(mt + (size_t)co * pm + ci2, mw * pm, ci2 < mw ? Msh[ci2][co] : 0.0, sc[co]);
    }
    return;
  }
  for (int e = t; e < kWsLen * kWsK; e += 128) {
    const int c = e % kWsLen, m = e / kWsLen;
    Vs[c][m] = (c < len && m < k) ? op.V[c + (size_t)m * op.ldv] : 0.0;
  }
  for (int e = t; e < kWsK * kWsK; e += 128) {
    const int l = e % kWsK, m = e / kWsK;
    Tsh[l][m] = (l < k && m < k) ? op.T[l + (size_t)m * op.ldt] : 0.0;
  }
  __syncthreads();
  // scales of V's columns: 8 lanes per column
  {
    const int m = t >> 3, part = t & 7;
    uint64_t amax = 0;
    for (int c = part; c < kWsLen; c += 8) amax = max(amax, ws_abs_bits(Vs[c][m]));
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, o));
    if (part == 0) {
      D->fv[m] = ws_exp_bits(amax);
      scv[m] = ws_exp_bits(amax);
    }
  }
  // T's columns (three-product form); W = T V^T, eight independent sums per thread
  if (!two && t < kWsK) {
    uint64_t amax = 0;
    for (int l = 0; l < kWsK; ++l) amax = max(amax, ws_abs_bits(Tsh[l][t]));
    D->ft[t] = ws_exp_bits(amax);
  }
  if (two) {
    const int m = t & 15, c0 = t >> 4;  // columns c0, c0+8, ..., c0+56
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int l = 0; l < kWsK; ++l) {
      const double tl = Tsh[m][l];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fma(tl, Vs[c0 + 8 * q][l], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) Wsh[m][c0 + 8 * q] = acc[q];
  }
  __syncthreads();
  const bool one = two && len <= kWsMM;
  if (one) {  // M = V W, eight independent sums per thread
    const int ci = t & 31, co0 = t >> 5;  // columns co0, co0+4, ..., co0+28
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int m = 0; m < kWsK; ++m) {
      const double v = Vs[ci][m];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fma(v, Wsh[m][co0 + 4 * q], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) Msh[ci][co0 + 4 * q] = acc[q];
    __syncthreads();
    {  // scales of M's columns: 4 lanes per column
      const int co = t >> 2, part = t & 3;
      uint64_t amax = 0;
      for (int c = part; c < kWsMM; c += 4) amax = max(amax, ws_abs_bits(Msh[c][co]));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 1));
      amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 2));
      if (part == 0) {
        D->fm[co] = ws_exp_bits(amax);
        sc[co] = ws_exp_bits(amax);
      }
    }
    __syncthreads();
    for (int e = t; e < kWsMM * kWsPM; e += 128) {
      const int co = e / kWsPM, ci2 = e % kWsPM;
      ws_put_digits(&D->mt[0][co][ci2], kWsMM * kWsPM, ci2 < kWsMM ? Msh[ci2][co] : 0.0, sc[co]);
    }
    __syncthreads();  // sc is reused below
  }
  // V digits [m][c]
  for (int e = t; e < kWsK * kWsPL; e += 128) {
    const int m = e / kWsPL, c = e % kWsPL;
    ws_put_digits(&D->vd[0][m][c], kWsK * kWsPL, c < kWsLen ? Vs[c][m] : 0.0, scv[m]);
  }
  __syncthreads();  // sc is reused below
  // right factor of the last product by columns c: W (two-product form) or V^T
  {
    const int c = t >> 1, half = t & 1;
    uint64_t amax = 0;
    for (int m = half; m < kWsK; m += 2) amax = max(amax, ws_abs_bits(two ? Wsh[m][c] : Vs[c][m]));
    amax = max(amax, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)amax, 1));
    if (half == 0) {
      D->fvt[c] = ws_exp_bits(amax);
      sc[c] = ws_exp_bits(amax);
    }
  }
  __syncthreads();
  for (int e = t; e < kWsLen * kWsPK; e += 128) {
    const int c = e / kWsPK, m = e % kWsPK;
    const double x = m < kWsK ? (two ? Wsh[m][c] : Vs[c][m]) : 0.0;
    ws_put_digits(&D->vt[0][c][m], kWsLen * kWsPK, x, sc[c]);
  }
  if (!two) {
    for (int e = t; e < kWsK * kWsPK; e += 128) {
      const int m = e / kWsPK, l = e % kWsPK;
      uint64_t amax = 0;
      for (int q = 0; q < kWsK; ++q) amax = max(amax, ws_abs_bits(Tsh[q][m]));
      ws_put_digits(&D->td[0][m][l], kWsK * kWsPK, l < kWsK ? Tsh[l][m] : 0.0, ws_exp_bits(amax));
    }
  }
}

// ------------------------------------------------------------------------------------------
// Application.
// ------------------------------------------------------------------------------------------
struct WsWarp {                                // per-warp bookkeeping (16 rows)
  int tag[kWsCW];                              // column held by each slot (-1: none)
  int newc[kWsLen];                            // op-relative columns loaded for the current op
  int rmax[16];                                // largest exponent among a row's loaded values
};
// The one-product operands alone (the leading members of WsOpDigits).
struct WsOpM {
  uint16_t mt[kWsD][kWsMM][kWsPM];
  int fm[kWsMM];
};
static_assert(sizeof(WsOpM) == offsetof(WsOpDigits, vd), "WsOpM is the prefix of WsOpDigits");
// List forms: 0 general (each op in the one-, two- or three-product form it allows); 1 every op
// takes the one-product form (full reflector ranges, len <= kWsMM), so only M's digits are
// staged: 57 KB instead of 104 KB, three CTAs per SM; 2 every op is a dense op of a wide list
// (len <= kWsMW, WsOpMW operands): 80 KB, two CTAs per SM.
template <int kForm>
struct WsSmemT {
  typename std::conditional<kForm == 0, WsOpDigits,
                            typename std::conditional<kForm == 1, WsOpM, WsOpMW>::type>::type op;  // the current op
  long long win[kWsRows][kWsCW + 1];           // resident values (fixed point)
  unsigned long long dirty[kWsRows];           // slots modified since loaded (one bit per slot)
  int escale[kWsRows];                         // row scales
  WsWarp w[kWsWarps];
};
static_assert(kWsCW == 64, "dirty masks hold one bit per slot");

template <int kForm>
inline size_t ws_smem_bytes() { return sizeof(WsSmemT<kForm>); }

// round(a 2^s), a < 2^62, 64-bit only
PHT_DEV uint64_t ws_scale64(uint64_t a, int s) {
  if (s >= 0) return s >= 64 ? 0 : a << s;
  if (s <= -64) return 0;
  return (a + (1ull << (-s - 1))) >> (-s);
}

// Digits (8 x 7 bits, rounded) of eight values, packed as the A fragments of one m16n8k16 step:
// F[i] are 56-bit magnitudes in the fragment order (row gq: k, k+1 | row gq+8: k, k+1 | row gq:
// k+8, k+9 | row gq+8: k+8, k+9), neg their signs.
PHT_DEV void ws_afrag(const uint64_t* F, const bool* neg, uint32_t (*af)[4]) {
#pragma unroll
  for (int t = 0; t < kWsD; ++t)
#pragma unroll
    for (int q = 0; q < 4; ++q)
      af[t][q] = ws_h2(ws_dig(F[2 * q], t), ws_dig(F[2 * q + 1], t), neg[2 * q], neg[2 * q + 1]);
}

// acc[l][nt][*] += sum over digit pairs (t + u = l) of A_t B_u for one 16-deep step; B from a
// [digit][n][k] array with pitch P (fp16), n-tiles at n0 and n0 + 8, k at k0.
template <int P>
PHT_DEV void ws_mma_step(float (*acc)[2][4], const uint32_t (*af)[4], const uint16_t* B, int dstride, int n0,
                         int k0, int gq, int tq) {
  // right digit outer: each B fragment is loaded once and used by every left digit ta <= 7-ub
#pragma unroll
  for (int ub = 0; ub < kWsD; ++ub) {
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      const uint16_t* row = B + (size_t)ub * dstride + (size_t)(n0 + nt * 8 + gq) * P + k0 + 2 * tq;
      const uint32_t b0 = ws_ld32(row), b1 = ws_ld32(row + 8);
#pragma unroll
      for (int ta = 0; ta < kWsD; ++ta) {
        if (ta + ub >= kWsLv) continue;
        ws_mma(acc[ta + ub][nt], af[ta][0], af[ta][1], af[ta][2], af[ta][3], b0, b1);
      }
    }
  }
}

PHT_DEV void ws_zero_acc(float (*acc)[2][4]) {
#pragma unroll
  for (int l = 0; l < kWsLv; ++l)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[l][nt][q] = kWsMagic;
}

// Accumulator element e (0..7 = [hh][nt][j] as hh*4 + nt*2 + j) of a [level][nt][4] set -> its
// exact (Nh, Nl) contribution.
PHT_DEV void ws_levels_of(const float (*acc)[2][4], int hh, int nt, int j, long long& Nh, long long& Nl) {
  float lv[kWsLv];
#pragma unroll
  for (int l = 0; l < kWsLv; ++l) lv[l] = acc[l][nt][2 * hh + j];
  ws_add_levels(lv, Nh, Nl);
}

// A 16 x 16 product held as exact (S, E) pairs (value S 2^E) in accumulator layout -> masked,
// row-normalised digits packed as A fragments of the next product (columns m are its k).
// Returns in emax[hh] the row exponent (|value| < 2^emax; kWsNoScale: zero row).
PHT_DEV void ws_to_afrag(__int128 (*xs)[2][2], const int (*xe)[2][2], int* emax, uint32_t (*af)[4]) {
  uint64_t F[8];
  bool neg[8];
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    int em = kWsNoScale;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const __int128 v = xs[hh][nt][j];
        if (v != 0) em = max(em, ws_bitlen((u128)(v < 0 ? -v : v)) + xe[hh][nt][j]);
      }
    em = max(em, __shfl_xor_sync(0xffffffffu, em, 1));
    em = max(em, __shfl_xor_sync(0xffffffffu, em, 2));
    emax[hh] = em;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const __int128 v = xs[hh][nt][j];
        const int i = nt * 4 + hh * 2 + j;  // fragment order: a0 (hh0,nt0) a1 (hh1,nt0) a2 (hh0,nt1) a3 (hh1,nt1)
        neg[i] = v < 0;
        F[i] = (v == 0) ? 0 : ws_scale_u((u128)(neg[i] ? -v : v), xe[hh][nt][j] + 56 - em);
      }
  }
  ws_afrag(F, neg, af);
}

template <class Geo, int kForm>
__global__ void __launch_bounds__(kWsThreads, kForm == 1 ? 3 : 2)
    k_ws_apply(double* __restrict__ C, long long rs, long long cs, int row0, int row1, Geo g,
               const WsOpDigits* __restrict__ prep, unsigned long long* __restrict__ flops) {
  extern __shared__ __align__(16) unsigned char ws_raw[];
  constexpr bool kOne = kForm != 0;  // every op of the list is one product C -= C M
  WsSmemT<kForm>& S = *reinterpret_cast<WsSmemT<kForm>*>(ws_raw);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const int rbeg = row0 + blockIdx.x * kWsRows;
  if (rbeg > row1) return;
  const int rend = min(row1, rbeg + kWsRows - 1);
  WsWarp& W = S.w[warp];
  const int wr0 = warp * 16;                            // CTA-local first row of this warp
  const int grow0 = rbeg + wr0;                         // its strip row
  const int nrows = max(0, min(16, rend - grow0 + 1));  // rows of this warp inside the strip
  for (int i = lane; i < kWsCW; i += 32) W.tag[i] = -1;
  if (lane < 16) {
    S.escale[wr0 + lane] = kWsNoScale;
    S.dirty[wr0 + lane] = 0ull;
  }
  __syncwarp();
  const int nops = g.count();
  const bool ymask = g.masks_y();
  const int rA = wr0 + gq, rB = wr0 + gq + 8;  // CTA-local rows of this lane's fragments
  for (int o = 0; o < nops; ++o) {
    const WYOp op = g.op(o);
    const int ra = max(rbeg, op.lo), rb = min(rend, op.hi);
    if (ra > rb || op.k <= 0 || op.len <= 0) continue;  // CTA-uniform
    const int len = op.len, k = op.k;
    // ---- reflector ranges of this lane's rows; which product form each warp takes ----
    int ra0 = 1, rb0 = 0, ra1 = 1, rb1 = 0;
    {
      const int r0 = grow0 + gq, r1 = grow0 + gq + 8;
      if (gq < nrows && r0 >= op.lo && r0 <= op.hi) g.range(o, op, r0, ra0, rb0);
      if (gq + 8 < nrows && r1 >= op.lo && r1 <= op.hi) g.range(o, op, r1, ra1, rb1);
    }
    const bool on0 = ra0 <= rb0, on1 = ra1 <= rb1;
    const bool wact = __any_sync(0xffffffffu, on0 || on1);
    const bool full = (!on0 || (ra0 == 0 && rb0 == k - 1)) && (!on1 || (ra1 == 0 && rb1 == k - 1));
    // C -= C M; a kOne list guarantees it (checked on the host)
    const bool wone = kOne || (!ymask && len <= kWsMM && __all_sync(0xffffffffu, full));
    // the previous op's digits are no longer read; copy only the parts some warp needs
    const int need_rest = kOne ? 0 : __syncthreads_or(wact && !wone);
    if (kOne) __syncthreads();
    {
      const size_t bytes = kForm == 2 ? sizeof(WsOpMW) : need_rest ? sizeof(WsOpDigits) : offsetof(WsOpDigits, vd);
      const uint4* src = reinterpret_cast<const uint4*>(prep + g.op_slot(o));
      uint4* dst = reinterpret_cast<uint4*>(&S.op);
      for (int e = t; e < (int)(bytes / 16); e += kWsThreads) dst[e] = src[e];
    }
    __syncthreads();
    if (!wact) continue;  // warp-uniform
    // ---- make the op's columns resident: new columns by ballot (two per lane) ----
    int nn;
    {
      const int c0 = lane, c1 = lane + 32;
      const bool n0 = c0 < len && W.tag[(op.start + c0) & (kWsCW - 1)] != op.start + c0;
      const bool n1 = c1 < len && W.tag[(op.start + c1) & (kWsCW - 1)] != op.start + c1;
      const uint32_t m0 = __ballot_sync(0xffffffffu, n0), m1 = __ballot_sync(0xffffffffu, n1);
      const uint32_t below = (1u << lane) - 1u;
      if (n0) W.newc[__popc(m0 & below)] = c0;
      if (n1) W.newc[__popc(m0) + __popc(m1 & below)] = c1;
      nn = __popc(m0) + __popc(m1);
    }
    if (lane < 16) W.rmax[lane] = kWsNoScale;
    __syncwarp();
    // evict (write back the old column of the slot for dirty rows), load raw FP64 bits and note
    // each row's largest exponent; lanes run along the contiguous direction of the matrix
    for (int e = lane; e < nn * 16; e += 32) {
      const int i = (cs == 1) ? e % nn : e >> 4, rl = (cs == 1) ? e / nn : e & 15;
      const int col = op.start + W.newc[i], sl = col & (kWsCW - 1), rr = wr0 + rl;
      const int old = W.tag[sl];
      long long raw = 0;
      if (rl < nrows) {
        if (old >= 0 && ((S.dirty[rr] >> sl) & 1ull))
          C[(long long)(grow0 + rl) * rs + (long long)old * cs] = ws_from_fixed(S.win[rr][sl], S.escale[rr]);
        raw = __double_as_longlong(__ldcg(&C[(long long)(grow0 + rl) * rs + (long long)col * cs]));
        const int ex = ws_exp_bits((uint64_t)raw & 0x7FFFFFFFFFFFFFFFull);
        if (ex != kWsNoScale) atomicMax(&W.rmax[rl], ex);
      }
      S.win[rr][sl] = raw;
    }
    __syncwarp();
    uint64_t newmask = 0;  // slots that now hold raw bits
    for (int i = 0; i < nn; ++i) newmask |= 1ull << ((op.start + W.newc[i]) & (kWsCW - 1));
    for (int i = lane; i < nn; i += 32) W.tag[(op.start + W.newc[i]) & (kWsCW - 1)] = op.start + W.newc[i];
    if (lane < 16) S.dirty[wr0 + lane] &= ~newmask;  // freshly loaded entries are clean
    if (lane < nrows) {  // raise a row's scale when a loaded value needs it (rare)
      const int rr = wr0 + lane, ex = W.rmax[lane];
      const int e = S.escale[rr];
      if (ex != kWsNoScale && (e == kWsNoScale || ex + kWsHead > e)) {
        const int enew = ex + kWsHead;
        if (e != kWsNoScale) {
          const int sh = enew - e;
          for (int q = 0; q < kWsCW; ++q) {
            if (W.tag[q] < 0 || ((newmask >> q) & 1ull)) continue;
            const long long v = S.win[rr][q];
            const uint64_t s2 = ws_scale64((uint64_t)(v < 0 ? -v : v), -sh);
            S.win[rr][q] = v < 0 ? -(long long)s2 : (long long)s2;
          }
        }
        S.escale[rr] = enew;
      }
    }
    __syncwarp();
    for (int e = lane; e < nn * 16; e += 32) {  // convert the loaded values
      const int i = (cs == 1) ? e % nn : e >> 4, rl = (cs == 1) ? e / nn : e & 15;
      const int sl = (op.start + W.newc[i]) & (kWsCW - 1), rr = wr0 + rl;
      if (rl < nrows) S.win[rr][sl] = ws_to_fixed(__longlong_as_double(S.win[rr][sl]), S.escale[rr]);
    }
    __syncwarp();
    if (flops) {  // algorithmic work (4 len k, or 2 len^2 for a dense op) FP64-equivalent flops per active row
      const int act = __popc(__ballot_sync(0xffffffffu, tq == 0 && on0)) + __popc(__ballot_sync(0xffffffffu, tq == 0 && on1));
      if (lane == 0) atomicAdd(flops, (unsigned long long)act * op_row_flops(op));
    }
    // Only the entries an op modifies are written back: rows of a resident window that an op
    // does not touch may be updated concurrently by other kernels on other streams (the next
    // group's chase and lookahead), whose results a stale copy must not overwrite.
    if (tq == 0) {  // the op's slots become dirty on the active rows
      const unsigned long long span = len >= 64 ? ~0ull : ((1ull << len) - 1ull);
      const int sh = op.start & (kWsCW - 1);
      const unsigned long long opmask = sh ? ((span << sh) | (span >> (64 - sh))) : span;
      if (on0) S.dirty[rA] |= opmask;
      if (on1) S.dirty[rB] |= opmask;
    }
    // ---- bit length of each row's largest value in the op's columns (4 lanes per row pair) ----
    const int lenp = (len + 15) & ~15;
    int blA, blB;
    {
      uint64_t mA = 0, mB = 0;
      for (int k0 = 0; k0 < lenp; k0 += 16)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int cc = k0 + 2 * tq + (q & 1) + 8 * (q >> 1);
          if (cc < len) {
            const int sl = (op.start + cc) & (kWsCW - 1);
            const long long va = S.win[rA][sl], vb = S.win[rB][sl];
            mA = max(mA, (uint64_t)(va < 0 ? -va : va));
            mB = max(mB, (uint64_t)(vb < 0 ? -vb : vb));
          }
        }
      mA = max(mA, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)mA, 1));
      mA = max(mA, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)mA, 2));
      mB = max(mB, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)mB, 1));
      mB = max(mB, (uint64_t)__shfl_xor_sync(0xffffffffu, (long long)mB, 2));
      // growth guard: shift a row down (raise its scale) when its largest value among the op's
      // columns has more than kWsGuard bits, so that the op's results stay below 2^62
      int shA = 0, shB = 0;
      if (mA >> kWsGuard) shA = (64 - __clzll((long long)mA)) - kWsGuard;
      if (mB >> kWsGuard) shB = (64 - __clzll((long long)mB)) - kWsGuard;
      if (__any_sync(0xffffffffu, shA || shB)) {
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int sh = hh ? shB : shA, rr = hh ? rB : rA;
          const int rowl = gq + 8 * hh;
          if (!sh || rowl >= nrows) continue;
          for (int q = tq; q < kWsCW; q += 4) {
            if (W.tag[q] < 0) continue;
            const long long v = S.win[rr][q];
            const uint64_t a = ws_scale64((uint64_t)(v < 0 ? -v : v), -sh);
            S.win[rr][q] = v < 0 ? -(long long)a : (long long)a;
          }
        }
        __syncwarp();
        if (tq == 0) {
          if (shA && gq < nrows) S.escale[rA] += shA;
          if (shB && gq + 8 < nrows) S.escale[rB] += shB;
        }
        __syncwarp();
        mA = ws_scale64(mA, -shA);
        mB = ws_scale64(mB, -shB);
      }
      blA = mA ? 64 - __clzll((long long)mA) : 0;
      blB = mB ? 64 - __clzll((long long)mB) : 0;
    }
    // digit scales of C's rows (|x| < 2^erow) and their fixed-point scales
    const int efix0 = gq < nrows ? S.escale[rA] : kWsNoScale;
    const int efix1 = gq + 8 < nrows ? S.escale[rB] : kWsNoScale;
    const int erow0 = (efix0 != kWsNoScale && blA > 0) ? efix0 - 62 + blA : kWsNoScale;
    const int erow1 = (efix1 != kWsNoScale && blB > 0) ? efix1 - 62 + blB : kWsNoScale;
    // A fragments of C for one 16-column step at k0
    auto cfrag = [&](int k0, uint32_t (*af)[4]) {
      uint64_t F[8];
      bool neg[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {  // fragment order: (A,k) (A,k+1) (B,k) (B,k+1) (A,k+8) ...
        const int rowB = (i >> 1) & 1, cc = k0 + 2 * tq + (i & 1) + 8 * (i >> 2);
        long long v = 0;
        if (cc < len) v = S.win[rowB ? rB : rA][(op.start + cc) & (kWsCW - 1)];
        neg[i] = v < 0;
        F[i] = ws_scale64((uint64_t)(neg[i] ? -v : v), 56 - (rowB ? blB : blA));
      }
      ws_afrag(F, neg, af);
    };
    // C -= (correction levels in acc), columns c0 + nt*8 + 2tq + j; right-factor column scales fr,
    // left digit scale zrow[hh]
    auto correct = [&](const float (*acc)[2][4], int c0, const int* fr, const int* zrow, bool act0, bool act1) {
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        if (!(hh ? act1 : act0)) continue;
        const int rr = hh ? rB : rA;
        const int er = hh ? efix1 : efix0, zr = zrow[hh];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int cc = c0 + nt * 8 + 2 * tq + j;
            if (cc >= len) continue;
            const int fc = fr[cc];
            if (fc == kWsNoScale) continue;
            long long nh = 0, nl = 0;
            ws_levels_of(acc, hh, nt, j, nh, nl);
            if ((nh | nl) == 0) continue;
            // correction in the row's fixed point: (nh 2^35 + nl) 2^sh, sh = zr + fc - 70 + 62 - er
            const int sh = zr + fc - 8 - er;
            const long long ah = nh < 0 ? -nh : nh, al = nl < 0 ? -nl : nl;
            const long long dh = (long long)ws_scale64((uint64_t)ah, sh + 35);
            const long long dl = (long long)ws_scale64((uint64_t)al, sh);
            S.win[rr][(op.start + cc) & (kWsCW - 1)] -= (nh < 0 ? -dh : dh) + (nl < 0 ? -dl : dl);
          }
      }
    };
    if constexpr (kForm == 2) {
      // ---- wide dense op, C -= C M with len <= 48: three k-steps.  The FP32 level sums are exact
      // for at most 32 terms, so the first two k-steps' levels are taken out before the third;
      // C's third k-step fragments are rebuilt per 16-column group from columns 32..47, which
      // only the last group's correction (after its products) modifies ----
      uint32_t af0[kWsD][4], af1[kWsD][4];
      cfrag(0, af0);
      if (lenp > 16) cfrag(16, af1);
      const bool act0 = on0 && erow0 != kWsNoScale, act1 = on1 && erow1 != kWsNoScale;
      for (int c0 = 0; c0 < lenp; c0 += 16) {
        long long nh[2][2][2], nl[2][2][2];  // [hh][nt][j]
        {
          float acc[kWsLv][2][4];
          ws_zero_acc(acc);
          ws_mma_step<kWsPMW>(acc, af0, &S.op.mt[0][0][0], kWsMW * kWsPMW, c0, 0, gq, tq);
          if (lenp > 16) ws_mma_step<kWsPMW>(acc, af1, &S.op.mt[0][0][0], kWsMW * kWsPMW, c0, 16, gq, tq);
#pragma unroll
          for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
              for (int j = 0; j < 2; ++j) {
                nh[hh][nt][j] = nl[hh][nt][j] = 0;
                ws_levels_of(acc, hh, nt, j, nh[hh][nt][j], nl[hh][nt][j]);
              }
        }
        if (lenp > 32) {
          uint32_t af2[kWsD][4];
          cfrag(32, af2);
          float acc[kWsLv][2][4];
          ws_zero_acc(acc);
          ws_mma_step<kWsPMW>(acc, af2, &S.op.mt[0][0][0], kWsMW * kWsPMW, c0, 32, gq, tq);
#pragma unroll
          for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
              for (int j = 0; j < 2; ++j) ws_levels_of(acc, hh, nt, j, nh[hh][nt][j], nl[hh][nt][j]);
        }
        // C -= the summed levels, as in correct() with the right factor's column scales fm
        const int zrow[2] = {erow0, erow1};
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          if (!(hh ? act1 : act0)) continue;
          const int rr = hh ? rB : rA;
          const int er = hh ? efix1 : efix0, zr = zrow[hh];
#pragma unroll
          for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int cc = c0 + nt * 8 + 2 * tq + j;
              if (cc >= len) continue;
              const int fc = S.op.fm[cc];
              if (fc == kWsNoScale) continue;
              const long long h = nh[hh][nt][j], l = nl[hh][nt][j];
              if ((h | l) == 0) continue;
              const int sh = zr + fc - 8 - er;
              const long long ah = h < 0 ? -h : h, al = l < 0 ? -l : l;
              const long long dh = (long long)ws_scale64((uint64_t)ah, sh + 35);
              const long long dl = (long long)ws_scale64((uint64_t)al, sh);
              S.win[rr][(op.start + cc) & (kWsCW - 1)] -= (h < 0 ? -dh : dh) + (l < 0 ? -dl : dl);
            }
        }
      }
      __syncwarp();
      continue;
    }
    if (wone) {
      // ---- one product: C -= C M (len <= 32: two k-steps, two 16-column groups) ----
      uint32_t af0[kWsD][4], af1[kWsD][4];
      cfrag(0, af0);
      if (lenp > 16) cfrag(16, af1);
      const int zrow[2] = {erow0, erow1};
      for (int c0 = 0; c0 < lenp; c0 += 16) {
        float acc[kWsLv][2][4];
        ws_zero_acc(acc);
        ws_mma_step<kWsPM>(acc, af0, &S.op.mt[0][0][0], kWsMM * kWsPM, c0, 0, gq, tq);
        if (lenp > 16) ws_mma_step<kWsPM>(acc, af1, &S.op.mt[0][0][0], kWsMM * kWsPM, c0, 16, gq, tq);
        correct(acc, c0, S.op.fm, zrow, on0 && erow0 != kWsNoScale, on1 && erow1 != kWsNoScale);
      }
      __syncwarp();
      continue;
    }
    if constexpr (!kOne) {
    // ---- X = C V (16 x k), exact levels per 32-column chunk ----
    long long xh[2][2][2], xl[2][2][2];  // [hh][nt][j]
#pragma unroll
    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) xh[hh][nt][j] = xl[hh][nt][j] = 0;
    for (int kc = 0; kc < lenp; kc += 32) {
      float acc[kWsLv][2][4];
      ws_zero_acc(acc);
      for (int k0 = kc; k0 < min(lenp, kc + 32); k0 += 16) {
        uint32_t af[kWsD][4];
        cfrag(k0, af);
        ws_mma_step<kWsPL>(acc, af, &S.op.vd[0][0][0], kWsK * kWsPL, 0, k0, gq, tq);
      }
#pragma unroll
      for (int hh = 0; hh < 2; ++hh)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int j = 0; j < 2; ++j) ws_levels_of(acc, hh, nt, j, xh[hh][nt][j], xl[hh][nt][j]);
    }
    // ---- X = S 2^E, E = erow + fv_m - 70 (masked); its digits as A fragments ----
    __int128 xs[2][2][2];
    int xe[2][2][2];
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int er = hh ? erow1 : erow0;
      const int a = hh ? ra1 : ra0, b = hh ? rb1 : rb0;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int m = nt * 8 + 2 * tq + j;
          const int fvm = S.op.fv[m];
          const bool on = m >= a && m <= b && m < k && er != kWsNoScale && fvm != kWsNoScale;
          xs[hh][nt][j] = on ? ws_join(xh[hh][nt][j], xl[hh][nt][j]) : (__int128)0;
          xe[hh][nt][j] = on ? er + fvm - 70 : 0;
        }
    }
    int zrow[2];
    uint32_t zf[kWsD][4];
    ws_to_afrag(xs, xe, zrow, zf);
    if (ymask) {  // Y = X T (16 x k), masked, as the left factor of Y V^T
      float acc[kWsLv][2][4];
      ws_zero_acc(acc);
      ws_mma_step<kWsPK>(acc, zf, &S.op.td[0][0][0], kWsK * kWsPK, 0, 0, gq, tq);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int a = hh ? ra1 : ra0, b = hh ? rb1 : rb0, xr = zrow[hh];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int m = nt * 8 + 2 * tq + j;
            const int ftm = S.op.ft[m];
            long long yh = 0, yl = 0;
            ws_levels_of(acc, hh, nt, j, yh, yl);
            const bool on = m >= a && m <= b && m < k && xr != kWsNoScale && ftm != kWsNoScale;
            xs[hh][nt][j] = on ? ws_join(yh, yl) : (__int128)0;
            xe[hh][nt][j] = on ? xr + ftm - 70 : 0;
          }
      }
      ws_to_afrag(xs, xe, zrow, zf);
    }
    // ---- C -= Z R (Z = X with R = W, or Z = Y with R = V^T), 16 columns at a time ----
    const bool act0 = on0 && zrow[0] != kWsNoScale, act1 = on1 && zrow[1] != kWsNoScale;
    for (int c0 = 0; c0 < lenp; c0 += 16) {
      float acc[kWsLv][2][4];
      ws_zero_acc(acc);
      ws_mma_step<kWsPK>(acc, zf, &S.op.vt[0][0][0], kWsLen * kWsPK, c0, 0, gq, tq);
      correct(acc, c0, S.op.fvt, zrow, act0, act1);
    }
    __syncwarp();
    }  // !kOne
  }
  // ---- write back every modified resident value ----
  __syncwarp();
  for (int e = lane; e < kWsCW * 16; e += 32) {
    const int sl = (cs == 1) ? e % kWsCW : e >> 4, rl = (cs == 1) ? e / kWsCW : e & 15;
    const int col = W.tag[sl], rr = wr0 + rl;
    if (col >= 0 && rl < nrows && ((S.dirty[rr] >> sl) & 1ull))
      C[(long long)(grow0 + rl) * rs + (long long)col * cs] = ws_from_fixed(S.win[rr][sl], S.escale[rr]);
  }
}

inline bool ws_fits(int k_max, int len_max) { return k_max <= kWsK && len_max <= kWsLen; }

// Prepares the op list (nslots prep slots, Geo::slot_op; skipped when prepare is false) and
// applies it to strip rows [row0, row1] of C viewed with strides (rs, cs).
template <class Geo, int kForm>
inline void ws_set_smem_attr() {
  static std::atomic<unsigned long long> done{0};
  smem_once((const void*)k_ws_apply<Geo, kForm>, ws_smem_bytes<kForm>(), done);
}

template <class Geo>
inline void launch_ws_apply(double* C, long long rs, long long cs, int row0, int row1, const Geo& g, int nslots,
                            WsOpDigits* prep, cudaStream_t s, bool prepare = true) {
  if (row1 < row0 || nslots <= 0) return;
  const int form = g.wide_dense() ? 2 : g.one_product_only() ? 1 : 0;
  if (form == 2)
    ws_set_smem_attr<Geo, 2>();
  else if (form == 1)
    ws_set_smem_attr<Geo, 1>();
  else
    ws_set_smem_attr<Geo, 0>();
  if (prepare) {
    count_launch();
    k_ws_prep<Geo><<<nslots, 128, 0, s>>>(g, prep);
  }
  count_launch();
  const int nblk = (row1 - row0 + 1 + kWsRows - 1) / kWsRows;
  KernelClock* kc = tl_kclock;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool timed = kc && kc->pair(Geo::kSite, &e0, &e1);
  if (timed) cudaEventRecord(e0, s);
  unsigned long long* fl = timed ? kc->dflops + Geo::kSite : nullptr;
  if (form == 2)
    k_ws_apply<Geo, 2><<<nblk, kWsThreads, ws_smem_bytes<2>(), s>>>(C, rs, cs, row0, row1, g, prep, fl);
  else if (form == 1)
    k_ws_apply<Geo, 1><<<nblk, kWsThreads, ws_smem_bytes<1>(), s>>>(C, rs, cs, row0, row1, g, prep, fl);
  else
    k_ws_apply<Geo, 0><<<nblk, kWsThreads, ws_smem_bytes<0>(), s>>>(C, rs, cs, row0, row1, g, prep, fl);
  if (timed) cudaEventRecord(e1, s);
}

}  // namespace pht
