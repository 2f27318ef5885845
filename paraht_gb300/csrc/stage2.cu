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
  PHT_DEV int count() const {
    switch (kind) {
      case kLaRight:
      case kUpRight:
        return nblocks * nq;
      default:
        return nblocks;
    }
  }
  // Split-precision preparation slots: only the compact-WY ops (kUpRight: the last op of each
  // block; single reflectors are applied in FP64 by the split kernel and need no slot).
  PHT_DEV int slot_op(int s) const { return kind == kUpRight ? s * nq + nq - 1 : s; }
  PHT_DEV int op_slot(int o) const { return kind == kUpRight ? o / nq : o; }
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
  // split-precision bulk updates where the op shapes fit (k = nq reflectors, r+nq long);
  // regions: 0 B right, 1 A right, 2 B left, 3 A left, 4 Q, 5 Z
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
    launch_apply_right(B, ldb, J, n - 1, g, sg);  // rows >= istart >= jblock+1
    launch_apply_right(A, lda, J, n - 1, g, sg);
    g.kind = kLaLeftB;
    launch_apply_left(B, ldb, J, n - 1, g, sg);
    g.kind = kLaLeftA;
    launch_apply_left(A, lda, J, n - 1, g, sg);
    if (timer) timer->mark(sg, 2);
    if (su != sg) {
      cudaEventRecord(ctx.ev_a, sg);
      cudaStreamWaitEvent(su, ctx.ev_a, 0);
    }
    // bulk updates; in the right update a row can lie in block ib's compact-WY range and in
    // block ib-1's staircase range, so singles and blocks form one ordered list
    g.kind = kUpRight;
    apply_right_any(reg[0], B, ldb, 0, n - 1, g, nblocks, su);
    apply_right_any(reg[1], A, lda, 0, n - 1, g, nblocks, su);
    g.kind = kUpLeft;
    apply_left_any(reg[2], B, ldb, J, n - 1, g, nblocks, su);
    apply_left_any(reg[3], A, lda, J, n - 1, g, nblocks, su);
    g.kind = kUpQ;
    apply_right_any(reg[4], Q, ldq, 0, n - 1, g, nblocks, su);
    g.kind = kUpZ;
    apply_right_any(reg[5], Z, ldz, 0, n - 1, g, nblocks, su);
    if (su != sg) cudaEventRecord(ctx.ev_b, su);
  }
  if (su != sg) cudaStreamWaitEvent(sg, ctx.ev_b, 0);
  if (timer) timer->mark(sg, -1);
  return 0;
}

}  // namespace pht
