// stage2g.cu -- stage 2 with Givens rotations (src/rht2ht.f90:696-1344, rht2ht_givens):
// (A r-Hessenberg, B triangular) -> (A Hessenberg, B triangular), accumulating Q and Z.
//
// For each group of nq columns starting at jblock = J (:766):
//   1. k_s2g_init: U(ib) = V(ib) = I, CV = 1, SV = 0 for the group's blocks;
//   2. s2g_launch_chase (stage2g_chase.cu): the band-only chase with rotations (:776-960), which
//      also accumulates every block's rotations into U(ib), V(ib) (:970-1003);
//   3. k_s2g_form: the dense ops' factors I - U(ib), I - V(ib);
//   4. lookahead of B then A (:1008-1131): the right rotations on the staircase of rows above each
//      block (k_s2g_stair) and U(ib)^T on the columns the next group needs (dense op lists);
//   5. delayed updates (:1173-1366), four independent chains as in the Householder stage 2:
//      B and A each: V(ib) on rows 1..istart-1 (dense right list), the staircase rotations of rows
//      istart.. (k_s2g_stair), U(ib)^T on columns istop+1..n (dense left list); Q U(ib); Z V(ib).
// For a given row the right list's blocks all precede its staircase blocks in the reference's
// order (istart(ib) grows with ib, and blocks run from nblocks down to 1), so running the whole
// list before the staircase kernel keeps every row's order.  Dense ops run through the FP64
// op-list kernels, or the split-precision kernel's one-product form when r + nq <= 32.
// Supported: r <= 32 (one warp holds a block column), r + nq <= 64.
#include <algorithm>

#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "split_apply.cuh"
#include "stage2g_common.cuh"
#include "wy_apply.cuh"

namespace pht {

// U(ib) = V(ib) = I and CV = 1, SV = 0 for blocks 1..nblocks: one CTA per block.
__global__ void k_s2g_init(S2GStore S) {
  const int ib = blockIdx.x + 1, ldu = S.ldu;
  double* U = S.U + S.gi(1, 1, ib);
  double* V = S.V + S.gi(1, 1, ib);
  for (int e = threadIdx.x; e < ldu * ldu; e += blockDim.x) {
    const double v = (e % ldu == e / ldu) ? 1.0 : 0.0;
    U[e] = v;
    V[e] = v;
  }
  double* C = S.CV + S.ri(1, 1, ib);
  double* Sn = S.SV + S.ri(1, 1, ib);
  for (int e = threadIdx.x; e < ldu * S.nq; e += blockDim.x) {
    C[e] = 1.0;
    Sn[e] = 0.0;
  }
}

// MU = I - U(ib), MV = I - V(ib): one CTA per block.
__global__ void k_s2g_form(S2GStore S) {
  const int ib = blockIdx.x + 1, ldu = S.ldu;
  const size_t o = S.gi(1, 1, ib);
  for (int e = threadIdx.x; e < ldu * ldu; e += blockDim.x) {
    const double d = (e % ldu == e / ldu) ? 1.0 : 0.0;
    S.MU[o + e] = d - S.U[o + e];
    S.MV[o + e] = d - S.V[o + e];
  }
}

// Right rotations of the group on the staircase of rows above the blocks, one row per thread
// (1-based row R = J + 1 + global thread index).  mode 0, the lookahead (:1018-1029,
// :1074-1087): sweep ic's rotations of block ib on rows [max(J+1, b - (2nq-ic) r),
// max(J+1, b - (nq-ic) r)); mode 1, the delayed update (:1246-1257, :1289-1296): rows
// [max(J+1, b - (2nq-1) r), max(J+1, b - (2nq-ic) r)), with b = J + 1 + (ib-1) r.  Blocks run
// from the last to the first, rotations ig = r-1 .. 1 (only those the chase generated; the
// others are the identity) on columns (jb+ic+ig-1, jb+ic+ig), jb = J + (ib-1) r, never beyond
// column n.  Each thread stages the r+nq-1 columns a block touches in shared memory.
__global__ void __launch_bounds__(128) k_s2g_stair(double* __restrict__ X, int ldx, int n, int J, int r, int nq,
                                                   int nblocks, S2GStore S, int mode) {
  extern __shared__ double stw[];
  const int w = r + nq;  // row slice: columns jb+1 .. jb+r+nq-1 at w[0 .. r+nq-2]
  double* row = stw + (size_t)threadIdx.x * (w + 1);
  const int R = J + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (R > n) return;
  const int q = (R - J - 1) / r;
  const int ib_hi = min(nblocks, q + 2 * nq + 1), ib_lo = max(1, q + 1);
  for (int ib = ib_hi; ib >= ib_lo; --ib) {
    const int b = J + 1 + (ib - 1) * r, jb = J + (ib - 1) * r;
    // which sweeps' rotations reach this row
    int ic_lo = nq + 1, ic_hi = 0;
    for (int ic = 1; ic <= nq; ++ic) {
      int lo, hi;
      if (mode == 0) {
        lo = max(J + 1, b - (2 * nq - ic) * r);
        hi = max(J + 1, b - (nq - ic) * r);
      } else {
        lo = max(J + 1, b - (2 * nq - 1) * r);
        hi = max(J + 1, b - (2 * nq - ic) * r);
      }
      if (R >= lo && R < hi) {
        ic_lo = min(ic_lo, ic);
        ic_hi = ic;
      }
    }
    if (ic_hi == 0) continue;
    const int ncol = min(n, jb + r + nq - 1) - jb;  // columns jb+1 .. jb+ncol
    for (int j = 0; j < ncol; ++j) row[j] = X[(size_t)(R - 1) + (size_t)(jb + j) * ldx];
    for (int ic = ic_lo; ic <= ic_hi; ++ic) {
      int lo, hi;
      if (mode == 0) {
        lo = max(J + 1, b - (2 * nq - ic) * r);
        hi = max(J + 1, b - (nq - ic) * r);
      } else {
        lo = max(J + 1, b - (2 * nq - 1) * r);
        hi = max(J + 1, b - (2 * nq - ic) * r);
      }
      if (R < lo || R >= hi) continue;
      // rotation ig on (x = column jb+ic+ig, y = column jb+ic+ig-1) = row[ic+ig-1], row[ic+ig-2]
      const int igmax = min(r - 1, n - jb - ic);
      if (igmax < 1) continue;
      double carry = row[ic + igmax - 1];
      for (int ig = igmax; ig >= 1; --ig) {
        const double c = S.CV[S.ri(ic + ig - 1, ic, ib)], sn = S.SV[S.ri(ic + ig - 1, ic, ib)];
        const double yv = row[ic + ig - 2];
        row[ic + ig - 1] = fma(c, carry, sn * yv);
        carry = fma(c, yv, -sn * carry);
      }
      row[ic - 1] = carry;
    }
    for (int j = 0; j < ncol; ++j) X[(size_t)(R - 1) + (size_t)(jb + j) * ldx] = row[j];
  }
}

static void launch_stair(cudaStream_t s, double* X, int ldx, int n, int J, int r, int nq, int nblocks,
                         const S2GStore& S, int mode) {
  const int rows = n - J;
  if (rows <= 0) return;
  count_launch();
  const size_t smem = sizeof(double) * 128 * (size_t)(r + nq + 1);
  k_s2g_stair<<<(rows + 127) / 128, 128, smem, s>>>(X, ldx, n, J, r, nq, nblocks, S, mode);
}

static int s2g_nblk0(int n, int r) { return std::max(1, (n - 1 + r - 1) / r) + 2; }

size_t s2g_workspace_bytes(int n, int r, int nq) {
  const size_t nb0 = s2g_nblk0(n, r), ldu = r + nq;
  return sizeof(double) * (2 * (4 * ldu * ldu * nb0 + 2 * ldu * nq * nb0) + ldu * ldu) + sizeof(int) * (nq + 2) +
         4096;
}

bool s2g_supported(int r, int nq) { return r <= 32 && r + nq <= 64; }

int s2g_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r, int nq,
            PhaseTimer* timer) {
  if (n < 3) return 0;  // rht2ht.f90:766: empty loop
  if (!s2g_supported(r, nq)) return PARAHT_ERR_NOT_SUPPORTED;
  const int nb0 = s2g_nblk0(n, r), ldu = r + nq;
  char* ws = (char*)ctx.workspace(s2g_workspace_bytes(n, r, nq));
  if (!ws) return PARAHT_ERR_ALLOC;
  double* d = (double*)ws;
  double* ident = d;
  d += (size_t)ldu * ldu;
  S2GStore S[2];
  for (int k = 0; k < 2; ++k) {
    S[k].ldu = ldu;
    S[k].nq = nq;
    S[k].I = ident;
    S[k].U = d;
    S[k].V = S[k].U + (size_t)ldu * ldu * nb0;
    S[k].MU = S[k].V + (size_t)ldu * ldu * nb0;
    S[k].MV = S[k].MU + (size_t)ldu * ldu * nb0;
    S[k].CV = S[k].MV + (size_t)ldu * ldu * nb0;
    S[k].SV = S[k].CV + (size_t)ldu * nq * nb0;
    d = S[k].SV + (size_t)ldu * nq * nb0;
  }
  ChaseSync sync;
  sync.prog = (int*)d;
  sync.ticket = sync.prog + (nq + 1);
  sync.status = ctx.dstatus;
  cudaStream_t sg = ctx.stream;
  const bool one_bulk = (timer && timer->serial) || ctx.sequential_chase;
  cudaStream_t su = one_bulk ? sg : ctx.side, sa = one_bulk ? sg : ctx.side2, sq = one_bulk ? sg : ctx.side3,
               sz = one_bulk ? sg : ctx.side4;
  set_identity(sg, ldu, ident, ldu);
  if (su != sg) {
    cudaEventRecord(ctx.ev_a, sg);
    cudaStreamWaitEvent(su, ctx.ev_a, 0);
  }
  // split-precision dense ops (one-product forms) when r + nq <= 48; operand regions: 0 bulk
  // right, 1 bulk left (both shared by A and B), 2 Q, 3 Z, 4 lookahead left B, 5 lookahead left A
  const bool sp = ctx.split && r + nq <= kWsMW;
  void* reg[6] = {};
  if (sp)
    for (int i = 0; i < 6; ++i) {
      reg[i] = ctx.split_region(i, nb0, sizeof(SplitOpData));
      if (!reg[i]) return PARAHT_ERR_ALLOC;
    }
  const size_t stair_smem = sizeof(double) * 128 * (size_t)(ldu + 1);
  if (stair_smem > 48 * 1024)
    if (const int rc = smem_at_least((const void*)k_s2g_stair, stair_smem)) return rc;
  int k = 0;
  for (int J = 1; J <= n - 2; J += nq, ++k) {
    const int nblocks = (n - J + r - 1) / r;
    const S2GStore& St = S[k & 1];
    if (k >= 2 && su != sg) {  // the Q and Z lists of group k-2 read this store
      if (timer) timer->mark(sg, 2);
      cudaStreamWaitEvent(sg, ctx.ev_s2[2 + 2 * (k & 1)], 0);
      cudaStreamWaitEvent(sg, ctx.ev_s2[3 + 2 * (k & 1)], 0);
    }
    if (timer) timer->mark(sg, 0);
    count_launch();
    k_s2g_init<<<nblocks, 256, 0, sg>>>(St);
    s2g_launch_chase(sg, A, lda, B, ldb, n, J, r, nq, St, sync, ctx.sequential_chase, ctx.spin_limit);
    count_launch();
    k_s2g_form<<<nblocks, 256, 0, sg>>>(St);
    if (k > 0 && su != sg) {  // lookahead k after the A and B lists of group k-1
      if (timer) timer->mark(sg, 2);
      cudaStreamWaitEvent(sg, ctx.ev_b, 0);
    }
    if (timer) timer->mark(sg, 1);
    GeoS2G g{St, n, J, r, nq, nblocks, kGLaLeftB};
    launch_stair(sg, B, ldb, n, J, r, nq, nblocks, St, 0);
    apply_left_any(reg[4], B, ldb, J, n - 1, g, nblocks, sg);
    g.kind = kGLaLeftA;
    launch_stair(sg, A, lda, n, J, r, nq, nblocks, St, 0);
    apply_left_any(reg[5], A, lda, J, n - 1, g, nblocks, sg);
    if (timer) timer->mark(sg, 2);
    if (su != sg) {
      cudaEventRecord(ctx.ev_a, sg);
      cudaStreamWaitEvent(su, ctx.ev_a, 0);
    }
    GeoS2G gr = g, gl = g, gq = g, gz = g;
    gr.kind = kGUpRight;
    gl.kind = kGUpLeft;
    gq.kind = kGUpQ;
    gz.kind = kGUpZ;
    prepare_any(reg[0], gr, nblocks, su);
    prepare_any(reg[1], gl, nblocks, su);
    if (su != sa) {
      cudaEventRecord(ctx.ev_s2[0], su);
      cudaStreamWaitEvent(sa, ctx.ev_s2[0], 0);
      cudaStreamWaitEvent(sq, ctx.ev_a, 0);
      cudaStreamWaitEvent(sz, ctx.ev_a, 0);
    }
    apply_right_side(reg[0], B, ldb, 0, n - 1, gr, nblocks, su, false);
    launch_stair(su, B, ldb, n, J, r, nq, nblocks, St, 1);
    apply_left_side(reg[1], B, ldb, J, n - 1, gl, nblocks, su, false);
    apply_right_side(reg[0], A, lda, 0, n - 1, gr, nblocks, sa, false);
    launch_stair(sa, A, lda, n, J, r, nq, nblocks, St, 1);
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
