// stage2_geom.cuh -- stage-2 op lists (lookahead and delayed bulk updates of one sweep group,
// src/rht2ht.f90:1630-2024) and the TV formation, shared by the single-pencil driver (stage2.cu)
// and the persistent batched kernel (batched.cu).
#pragma once
#include "paraht_internal.cuh"
#include "s2_common.cuh"

namespace pht {

enum S2Kind {
  kLaRight = 0,   // lookahead, right single reflectors (rht2ht.f90:1644-1661, 1710-1728)
  kLaLeftB = 1,   // lookahead, left WY on B (1669-1684)
  kLaLeftA = 2,   // lookahead, left WY on A (1737-1765)
  kUpRight = 3,   // bulk right: staircase single reflectors + WY (1818-1844, 1894-1920)
  kUpLeft = 4,    // bulk left WY on A and B (1852-1866, 1928-1951)
  kUpQ = 5,       // Q accumulation (1976-1986)
  kUpZ = 6,       // Z accumulation (2009-2018)
};

struct GeoS2 {
  S2Store S;
  int n, J, r, nq, nblocks, kind;  // J = jblock (1-based)
  // blk = 1: one op per block also for kLaRight / kUpRight, whose single reflectors act on a
  // staircase of rows; range() gives each row its contiguous subset of the block's reflectors
  // (the split-precision kernel, wy_stream.cuh).  blk = 0: the reference's op sequence with
  // the single reflectors as separate ops (FP64 kernels).
  int blk = 0;
  __host__ __device__ bool per_refl() const { return !blk && (kind == kLaRight || kind == kUpRight); }
  __host__ __device__ int count() const { return per_refl() ? nblocks * nq : nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  // Whether some row stops before the block's last reflector (the lookahead staircase): the
  // split kernel then forms Y = X T and masks it (wy_stream.cuh).
  PHT_DEV bool masks_y() const { return blk && kind == kLaRight; }
  // Whether every op of the list applies all its reflectors to every row over a span of at most
  // 32 columns (the split kernel's one-product form C -= C M): the left lists and Q, Z.
  __host__ __device__ bool one_product_only() const {
    const bool full = kind == kUpQ || kind == kUpZ || kind == kUpLeft || kind == kLaLeftA || kind == kLaLeftB;
    return full && r + nq <= 32;
  }
  __host__ __device__ bool wide_dense() const { return false; }
  static constexpr int kSite = 1;  // stage-2 op list (kernel statistics)
  // Reflectors [a, b] (0-based) of op o applied to strip row `row` (0-based, lo <= row <= hi).
  PHT_DEV void range(int o, const WYOp& w, int row, int& a, int& b) const {
    a = 0;
    b = w.k - 1;
    if (!blk || (kind != kUpRight && kind != kLaRight)) return;
    const int ib = nblocks - o;
    const int base = J + 1 + (ib - 1) * r;
    const int R1 = row + 1, D = base - R1;  // 1-based row, distance to the block's first row
    if (kind == kUpRight) {
      // rows 1 .. istart-1: the whole block (rht2ht.f90:1894-1920); rows istart ..: the single
      // reflectors ic = 2..nq with row < istart2(ic) = base - (2nq-ic) r (:1818-1844)
      const int istart = max(J + 1, base - (2 * nq - 1) * r);
      if (R1 <= istart - 1) return;
      if (D < 1) {
        a = 1;
        b = 0;
        return;
      }
      a = max(2, 2 * nq - (D - 1) / r) - 1;
      return;
    }
    // lookahead (:1644-1661, 1710-1728): reflector ic on rows [istart(ic), istart2(ic)),
    // istart(ic) = max(J+1, base - (2nq-ic) r), istart2(ic) = max(J+1, base - (nq-ic) r)
    if (R1 < J + 1 || D < 1) {
      a = 1;
      b = 0;
      return;
    }
    const int cd = (D + r - 1) / r;
    a = max(1, nq - cd + 1) - 1;
    b = min(w.k, 2 * nq - cd) - 1;
  }
  PHT_DEV WYOp single(int ic, int ib, int rlo1, int rhi1) const {  // 1-based inclusive rows
    const int jb = J + (ib - 1) * r;
    WYOp w;
    w.start = jb + ic - 1;
    w.len = min(r, n - jb - ic + 1);
    w.k = w.len >= 1 ? 1 : 0;
    w.lo = rlo1 - 1;
    w.hi = rhi1 - 1;
    w.V = S.V + S.ui(ic, ic, ib);
    w.ldv = S.ldu;
    w.T = S.tauV + S.ti(ic, ib);
    w.ldt = 1;
    return w;
  }
  PHT_DEV WYOp op(int o) const {
    WYOp w;
    if (blk && (kind == kLaRight || kind == kUpRight)) {  // the block's compact WY, row staircase
      const int ib = nblocks - o;
      const int jb = J + (ib - 1) * r, base = J + 1 + (ib - 1) * r;
      w.start = jb;
      w.len = min(n - jb, r + nq);
      w.k = min(nq, w.len);
      w.V = S.V + S.ui(1, 1, ib);
      w.ldv = S.ldu;
      w.T = S.TV + S.tt(ib);
      w.ldt = nq;
      if (kind == kUpRight) {
        w.lo = 0;
        w.hi = max(max(J + 1, base - (2 * nq - 1) * r) - 2, max(J + 1, base - nq * r) - 2);
      } else {
        w.lo = max(J + 1, base - (2 * nq - 1) * r) - 1;
        w.hi = base - 2;
      }
      return w;
    }
    if (kind == kLaRight || kind == kUpRight) {
      const int ib = nblocks - o / nq, sub = o % nq;
      const int base = J + 1 + (ib - 1) * r;
      if (kind == kLaRight) {
        const int ic = sub + 1;
        const int istart = max(J + 1, base - nq * r - (nq - ic) * r);
        const int istart2 = max(J + 1, base - (nq - ic) * r);
        return single(ic, ib, istart, istart2 - 1);
      }
      const int istart = max(J + 1, base - (2 * nq - 1) * r);
      if (sub < nq - 1) {
        const int ic = sub + 2;
        const int istart2 = max(J + 1, base - (2 * nq - ic) * r);
        return single(ic, ib, istart, istart2 - 1);
      }
      const int jb = J + (ib - 1) * r;
      w.start = jb;
      w.len = min(n - jb, r + nq);
      w.k = min(nq, w.len);
      w.lo = 0;
      w.hi = istart - 2;
      w.V = S.V + S.ui(1, 1, ib);
      w.ldv = S.ldu;
      w.T = S.TV + S.tt(ib);
      w.ldt = nq;
      return w;
    }
    const int ib = nblocks - o;
    const int jb = J + (ib - 1) * r;
    w.start = jb;
    w.len = min(n - jb, kind == kUpQ ? r + nq - 1 : r + nq);
    w.k = min(nq, w.len);
    w.ldv = S.ldu;
    w.ldt = nq;
    if (kind == kUpZ) {
      w.V = S.V + S.ui(1, 1, ib);
      w.T = S.TV + S.tt(ib);
    } else {
      w.V = S.U + S.ui(1, 1, ib);
      w.T = S.TU + S.tt(ib);
    }
    const int istop2 = min(n, J + (ib - 1) * r + r + nq + r * nq - 1);
    switch (kind) {
      case kLaLeftB: {
        const int istop = min(n, J + (ib - 1) * r + r + nq - 1);
        w.lo = istop;
        w.hi = istop2 - 1;
        break;
      }
      case kLaLeftA: {
        const int istop = (ib == 1) ? min(n, J + nq - 1) : min(n, J + 1 + (ib - 2) * r + nq - 1);
        w.lo = istop;
        w.hi = istop2 - 1;
        break;
      }
      case kUpLeft:
        w.lo = istop2;
        w.hi = n - 1;
        break;
      default:  // Q, Z: all rows
        w.lo = 0;
        w.hi = n - 1;
        break;
    }
    return w;
  }
};

// TV of block ib (rht2ht.f90:1599-1610; TU is built by the chase itself): one CTA, shared
// memory 2 nq^2 doubles at smt.
static __device__ void s2_form_t_body(int n, int J, int r, int nq, int ib, const S2Store& S, double* smt) {
  double* G = smt;             // nq*nq
  double* Ts = smt + nq * nq;  // nq*nq
  const bool isV = true;  // TU is built by the chase itself (stage2_chase.cu)
  const double* Vb = (isV ? S.V : S.U) + S.ui(1, 1, ib);
  const double* tau = (isV ? S.tauV : S.tauU) + S.ti(1, ib);
  double* T = (isV ? S.TV : S.TU) + S.tt(ib);
  const int jb = J + (ib - 1) * r;
  const int rows = min(n - jb, r + nq);
  const int k = min(nq, rows);
  const int t = threadIdx.x;
  for (int e = t; e < nq * nq; e += blockDim.x) {
    const int q = e % nq, m = e / nq;
    double s = 0.0;
    if (q < m && m < k)
      for (int i = 0; i < rows; ++i) s = fma(Vb[i + (size_t)q * S.ldu], Vb[i + (size_t)m * S.ldu], s);
    G[q + m * nq] = s;
  }
  for (int e = t; e < nq * nq; e += blockDim.x) Ts[e] = 0.0;
  __syncthreads();
  for (int m = 0; m < k; ++m) {
    if (t < m) {
      double s = 0.0;
      for (int q = t; q < m; ++q) s = fma(Ts[t + q * nq], G[q + m * nq], s);
      Ts[t + m * nq] = -tau[m] * s;
    }
    if (t == m) Ts[m + m * nq] = tau[m];
    __syncthreads();
  }
  for (int e = t; e < nq * nq; e += blockDim.x) T[e] = Ts[e];
}

}  // namespace pht
