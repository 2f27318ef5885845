// stage2.cu -- stage 2 of the HT reduction on the GPU: (A r-Hessenberg, B triangular) ->
// (A Hessenberg, B triangular), accumulating Q and Z.
//
// Follows src/rht2ht.f90:1346-2051 (rht2ht_householder).  For each group of nq columns
// starting at jblock (rht2ht.f90:1417):
//   1. s2_launch_chase (stage2_chase.cu): the band-only bulge chase of the group's nq columns
//      (rht2ht.f90:1433-1596), pipelined across CTAs, producing nq left reflectors U(:,ic,ib) and
//      nq right reflectors V(:,ic,ib) per block ib.
//   2. k_s2_form_t: TU, TV for every block (dlarft 'F','C', rht2ht.f90:1599-1610).
//   3. lookahead updates of B and A (rht2ht.f90:1630-1772) and the delayed bulk updates of B, A,
//      Q and Z (rht2ht.f90:1803-2024), each an ordered compact-WY op list (wy_apply.cuh) whose
//      row/column ranges are the reference's staircase (istart/istart2/istop/istop2).
// As in the reference's task graph, the generation of group k+1 overlaps the bulk updates of
// group k (side stream, double-buffered reflectors, rht2ht.f90:1786-1797), and the lookahead of
// group k+1 waits for the bulk updates of group k (the A(2,2)/B(2,2) dependency tokens).
#include <algorithm>

#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "s2_common.cuh"
#include "split_apply.cuh"
#include "wy_apply.cuh"

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
  PHT_DEV bool per_refl() const { return !blk && (kind == kLaRight || kind == kUpRight); }
  PHT_DEV int count() const { return per_refl() ? nblocks * nq : nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  // Whether some row stops before the block's last reflector (the lookahead staircase): the
  // split kernel then forms Y = X T and masks it (wy_stream.cuh).
  PHT_DEV bool masks_y() const { return blk && kind == kLaRight; }
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

// TU / TV of every block (rht2ht.f90:1599-1610): one CTA per block and per factor.
__global__ void k_s2_form_t(int n, int J, int r, int nq, int nblocks, S2Store S) {
  extern __shared__ double smt[];
  double* G = smt;             // nq*nq
  double* Ts = smt + nq * nq;  // nq*nq
  const int ib = blockIdx.x + 1;
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

// ------------------------------------------------------------------------------------------
// Host driver
// ------------------------------------------------------------------------------------------

static int s2_nblk0(int n, int r) { return std::max(1, (n - 1 + r - 1) / r) + 2; }

size_t s2_workspace_bytes(int n, int r, int nq) {
  const size_t nb0 = s2_nblk0(n, r);
  const size_t ldu = r + nq;
  return 2 * sizeof(double) * (2 * ldu * nq * nb0 + 2 * (size_t)nq * nq * nb0 + 2 * (size_t)nq * nb0) +
         sizeof(int) * (nq + 2) + 4096;
}

int s2_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r, int nq,
           PhaseTimer* timer) {
  if (n < 3) return 0;  // rht2ht.f90:1417: empty loop
  const int nb0 = s2_nblk0(n, r);
  const int ldu = r + nq;
  char* ws = (char*)ctx.workspace(s2_workspace_bytes(n, r, nq));
  if (!ws) return PARAHT_ERR_ALLOC;
  // Two reflector sets (the reference's U/V and U2/V2 copies, rht2ht.f90:1786-1797) used
  // alternately, plus the chase's progress words.
  S2Store S[2];
  double* d = (double*)ws;
  for (int k = 0; k < 2; ++k) {
    S[k].ldu = ldu;
    S[k].nq = nq;
    S[k].U = d;
    S[k].V = S[k].U + (size_t)ldu * nq * nb0;
    S[k].TU = S[k].V + (size_t)ldu * nq * nb0;
    S[k].TV = S[k].TU + (size_t)nq * nq * nb0;
    S[k].tauU = S[k].TV + (size_t)nq * nq * nb0;
    S[k].tauV = S[k].tauU + (size_t)nq * nb0;
    d = S[k].tauV + (size_t)nq * nb0;
  }
  ChaseSync sync;
  sync.prog = (int*)d;
  sync.ticket = sync.prog + (nq + 1);
  sync.status = ctx.dstatus;
  // Generation + lookahead on the main stream, delayed bulk updates on the side stream
  // (the reference's priority-100 / priority-1 tasks).  With time_components everything runs
  // on the main stream so the phases can be timed separately (the reference inserts taskwaits).
  cudaStream_t sg = ctx.stream;
  cudaStream_t su = (timer || ctx.sequential_chase) ? ctx.stream : ctx.side;
  if (su != sg) {
    cudaEventRecord(ctx.ev_a, sg);
    cudaStreamWaitEvent(su, ctx.ev_a, 0);
  }
  // split-precision lookahead and bulk updates where the op shapes fit (k = nq reflectors,
  // r+nq long).  Operand regions (one per op list; lists applied to both A and B share one):
  // 0 bulk right, 1 bulk left, 2 Q, 3 Z (side stream), 4 lookahead right, 5 lookahead left
  // (main stream)
  const bool sp = ctx.split && split_fits(nq, r + nq);
  void* reg[6] = {};
  if (sp)
    for (int i = 0; i < 6; ++i) {
      reg[i] = ctx.split_region(i, nb0, sizeof(SplitOpData));
      if (!reg[i]) return PARAHT_ERR_ALLOC;
    }
  int k = 0;
  for (int J = 1; J <= n - 2; J += nq, ++k) {  // rht2ht.f90:1417
    const int nblocks = (n - J + r - 1) / r;
    const int nz = std::min(nb0, nblocks + 2);
    const S2Store& St = S[k & 1];
    if (timer) timer->mark(sg, 0);
    cudaMemsetAsync(St.U, 0, sizeof(double) * (size_t)ldu * nq * nz, sg);
    cudaMemsetAsync(St.V, 0, sizeof(double) * (size_t)ldu * nq * nz, sg);
    cudaMemsetAsync(St.tauU, 0, sizeof(double) * (size_t)nq * nz, sg);
    cudaMemsetAsync(St.tauV, 0, sizeof(double) * (size_t)nq * nz, sg);
    cudaMemsetAsync(St.TU, 0, sizeof(double) * (size_t)nq * nq * nz, sg);
    s2_launch_chase(sg, A, lda, B, ldb, n, J, r, nq, St, sync, ctx.sequential_chase, ctx.spin_limit);
    count_launch();
    k_s2_form_t<<<dim3(nblocks, 1), 128, sizeof(double) * 2 * nq * nq, sg>>>(n, J, r, nq, nblocks, St);
    if (timer) timer->mark(sg, 1);
    if (k > 0 && su != sg) cudaStreamWaitEvent(sg, ctx.ev_b, 0);  // lookahead k after bulk k-1
    GeoS2 g{St, n, J, r, nq, nblocks, kLaRight};
    g.blk = sp ? 1 : 0;  // split kernel: one op per block, row staircase through range()
    apply_right_any(reg[4], B, ldb, J, n - 1, g, nblocks, sg);  // rows >= istart >= jblock+1
    apply_right_any(reg[4], A, lda, J, n - 1, g, nblocks, sg, false);
    g.kind = kLaLeftB;
    apply_left_any(reg[5], B, ldb, J, n - 1, g, nblocks, sg);
    g.kind = kLaLeftA;
    apply_left_any(reg[5], A, lda, J, n - 1, g, nblocks, sg, false);
    if (timer) timer->mark(sg, 2);
    if (su != sg) {
      cudaEventRecord(ctx.ev_a, sg);
      cudaStreamWaitEvent(su, ctx.ev_a, 0);
    }
    // bulk updates; in the right update a row can lie in block ib's compact-WY range and in
    // block ib-1's staircase range, so singles and blocks form one ordered list
    g.kind = kUpRight;
    apply_right_any(reg[0], B, ldb, 0, n - 1, g, nblocks, su);
    apply_right_any(reg[0], A, lda, 0, n - 1, g, nblocks, su, false);
    g.kind = kUpLeft;
    apply_left_any(reg[1], B, ldb, J, n - 1, g, nblocks, su);
    apply_left_any(reg[1], A, lda, J, n - 1, g, nblocks, su, false);
    g.kind = kUpQ;
    apply_right_any(reg[2], Q, ldq, 0, n - 1, g, nblocks, su);
    g.kind = kUpZ;
    apply_right_any(reg[3], Z, ldz, 0, n - 1, g, nblocks, su);
    if (su != sg) cudaEventRecord(ctx.ev_b, su);
  }
  if (su != sg) cudaStreamWaitEvent(sg, ctx.ev_b, 0);
  if (timer) timer->mark(sg, -1);
  return 0;
}

}  // namespace pht
