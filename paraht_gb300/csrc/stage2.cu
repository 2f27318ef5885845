// stage2.cu -- stage 2 of the HT reduction on the GPU: (A r-Hessenberg, B triangular) ->
// (A Hessenberg, B triangular), accumulating Q and Z.
//
// Follows src/rht2ht.f90:1346-2051 (rht2ht_householder).  For each group of nq columns
// starting at jblock (rht2ht.f90:1417):
//   1. s2_launch_chase (stage2_chase.cu): the band-only bulge chase of the group's nq columns
//      (rht2ht.f90:1433-1596), pipelined across CTAs, producing nq left reflectors U(:,ic,ib) and
//      nq right reflectors V(:,ic,ib) per block ib.
//   2. k_s2_form_t: TV for every block (dlarft 'F','C', rht2ht.f90:1599-1610; TU is built by the
//      chase itself as the sweeps generate its columns).
//   3. lookahead updates of B and A (rht2ht.f90:1630-1772) and the delayed bulk updates of B, A,
//      Q and Z (rht2ht.f90:1803-2024), each an ordered compact-WY op list (GeoS2 in
//      stage2_geom.cuh; FP64 kernels in wy_apply.cuh, split precision in wy_stream.cuh) whose
//      row/column ranges are the reference's staircase (istart/istart2/istop/istop2).
// As in the reference's task graph, the generation of group k+1 overlaps the bulk updates of
// group k (side stream, double-buffered reflectors, rht2ht.f90:1786-1797), and the lookahead of
// group k+1 waits for the bulk updates of group k (the A(2,2)/B(2,2) dependency tokens).
#include <algorithm>

#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "s2_common.cuh"
#include "split_apply.cuh"
#include "stage2_geom.cuh"
#include "wy_apply.cuh"

namespace pht {

// TV of every block of a group: one CTA per block.
__global__ void k_s2_form_t(int n, int J, int r, int nq, int nblocks, S2Store S) {
  extern __shared__ double smt[];
  s2_form_t_body(n, J, r, nq, blockIdx.x + 1, S, smt);
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
  const bool one_bulk = (timer && timer->serial) || ctx.sequential_chase;
  cudaStream_t su = one_bulk ? ctx.stream : ctx.side;
  cudaStream_t sa = one_bulk ? su : ctx.side2, sq = one_bulk ? su : ctx.side3, sz = one_bulk ? su : ctx.side4;
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
    if (k >= 2 && su != sg) {  // the Q and Z lists of group k-2 read this store
      if (timer) timer->mark(sg, 2);
      cudaStreamWaitEvent(sg, ctx.ev_s2[2 + 2 * (k & 1)], 0);
      cudaStreamWaitEvent(sg, ctx.ev_s2[3 + 2 * (k & 1)], 0);
    }
    if (timer) timer->mark(sg, 0);
    cudaMemsetAsync(St.U, 0, sizeof(double) * (size_t)ldu * nq * nz, sg);
    cudaMemsetAsync(St.V, 0, sizeof(double) * (size_t)ldu * nq * nz, sg);
    cudaMemsetAsync(St.tauU, 0, sizeof(double) * (size_t)nq * nz, sg);
    cudaMemsetAsync(St.tauV, 0, sizeof(double) * (size_t)nq * nz, sg);
    cudaMemsetAsync(St.TU, 0, sizeof(double) * (size_t)nq * nq * nz, sg);
    s2_launch_chase(sg, A, lda, B, ldb, n, J, r, nq, St, sync, ctx.sequential_chase, ctx.spin_limit);
    count_launch();
    k_s2_form_t<<<dim3(nblocks, 1), 128, sizeof(double) * 2 * nq * nq, sg>>>(n, J, r, nq, nblocks, St);
    if (k > 0 && su != sg) {  // lookahead k after the A and B lists of group k-1
      if (timer) timer->mark(sg, 2);
      cudaStreamWaitEvent(sg, ctx.ev_b, 0);
    }
    if (timer) timer->mark(sg, 1);
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
    // block ib-1's staircase range, so singles and blocks form one ordered list.  The four
    // matrices are independent: B's right-then-left lists on su, A's on sa, Q's on sq, Z's on sz
    // (one stream when the phases are timed or the schedule is sequential); each matrix keeps
    // the reference's order of its own lists (rht2ht.f90:1803-2024).
    GeoS2 gr = g, gl = g, gq = g, gz = g;
    gr.kind = kUpRight;
    gl.kind = kUpLeft;
    gq.kind = kUpQ;
    gz.kind = kUpZ;
    prepare_any(reg[0], gr, nblocks, su);
    prepare_any(reg[1], gl, nblocks, su);
    if (su != sa) {
      cudaEventRecord(ctx.ev_s2[0], su);  // operands of the right and left lists ready
      cudaStreamWaitEvent(sa, ctx.ev_s2[0], 0);
      cudaStreamWaitEvent(sq, ctx.ev_a, 0);  // the chase and lookahead of this group are done
      cudaStreamWaitEvent(sz, ctx.ev_a, 0);
    }
    apply_right_side(reg[0], B, ldb, 0, n - 1, gr, nblocks, su, false);
    apply_left_side(reg[1], B, ldb, J, n - 1, gl, nblocks, su, false);
    apply_right_side(reg[0], A, lda, 0, n - 1, gr, nblocks, sa, false);
    apply_left_side(reg[1], A, lda, J, n - 1, gl, nblocks, sa, false);
    apply_right_side(reg[2], Q, ldq, 0, n - 1, gq, nblocks, sq);
    apply_right_side(reg[3], Z, ldz, 0, n - 1, gz, nblocks, sz);
    if (su != sa) {  // A joins B (the next lookahead's dependency); Q and Z run on
      cudaEventRecord(ctx.ev_s2[1], sa);
      cudaStreamWaitEvent(su, ctx.ev_s2[1], 0);
      cudaEventRecord(ctx.ev_s2[2 + 2 * (k & 1)], sq);
      cudaEventRecord(ctx.ev_s2[3 + 2 * (k & 1)], sz);
    }
    if (su != sg) cudaEventRecord(ctx.ev_b, su);
  }
  if (su != sg) {  // join; the Q and Z streams run in order, so their last group's events suffice
    if (timer) timer->mark(sg, 2);
    cudaStreamWaitEvent(sg, ctx.ev_b, 0);
    if (k > 0) {
      cudaStreamWaitEvent(sg, ctx.ev_s2[2 + 2 * ((k - 1) & 1)], 0);
      cudaStreamWaitEvent(sg, ctx.ev_s2[3 + 2 * ((k - 1) & 1)], 0);
    }
  }
  if (timer) timer->mark(sg, -1);
  return 0;
}

}  // namespace pht
