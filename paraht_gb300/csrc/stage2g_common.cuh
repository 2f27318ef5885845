// stage2g_common.cuh -- storage, rotation arithmetic and op lists of the Givens stage 2
// (src/rht2ht.f90:696-1344, rht2ht_givens), shared by its chase kernel (stage2g_chase.cu) and
// its driver (stage2g.cu).
//
// The sweep group of nq columns at jblock = J chases its bulges with Givens rotations: nb-1
// rotations from the left reduce a column of A (DLARTG from the bottom), and nb-1 rotations
// from the right remove the one subdiagonal they leave in B, so no RQ factorisation is needed.
// The rotations of block ib of the group are accumulated into (r+nq) x (r+nq) orthogonal
// matrices U(ib) (left) and V(ib) (right) (src/rht2ht.f90:970-1003); here the chase
// accumulates them itself as the sweeps pass each block.  The lookahead and delayed updates
// are then dense products with U(ib), V(ib) (the reference's dgemm calls) plus, on a staircase
// of rows, the individual right rotations (kept as (c, s) in CV, SV).
#pragma once
#include <cuda_runtime.h>

#include "paraht_internal.cuh"
#include "s2_common.cuh"

namespace pht {

// One reflector set of a Givens sweep group (two are used alternately).  Helpers take the
// reference's 1-based indices: U(i, j, ib), CV(i, ic, ib).
struct S2GStore {
  double *U, *V;    // ldu x ldu x nblk: accumulated left / right rotations of each block
  double *MU, *MV;  // ldu x ldu x nblk: I - U, I - V (the dense ops' T factors)
  double *CV, *SV;  // ldu x nq x nblk: right rotations (c, s) of rotation ig of sweep ic at row ic+ig-1
  const double* I;  // ldu x ldu identity (the dense ops' V factor)
  int ldu, nq;
  PHT_DEV __host__ size_t gi(int i, int j, int ib) const {
    return (size_t)(i - 1) + (size_t)(j - 1) * ldu + (size_t)(ib - 1) * ldu * ldu;
  }
  PHT_DEV __host__ size_t ri(int i, int ic, int ib) const {
    return (size_t)(i - 1) + (size_t)(ic - 1) * ldu + (size_t)(ib - 1) * ldu * nq;
  }
};

// Rotation with LAPACK DLARTG's conventions (c >= 0, r carries the sign of f, s = g / r;
// g = 0: c = 1, s = 0, r = f; f = 0: c = 0, s = sign(g), r = |g|), computed with one reciprocal
// square root instead of DLARTG's square root and division (every dependent FP64 instruction
// costs about 64 cycles on GB300; the results agree to a few ulps).  Inputs are scaled when
// f^2 + g^2 would leave the normal range.
PHT_DEV void givens(double f, double g, double& c, double& s, double& r) {
  if (g == 0.0) {
    c = 1.0;
    s = 0.0;
    r = f;
    return;
  }
  if (f == 0.0) {
    c = 0.0;
    s = copysign(1.0, g);
    r = fabs(g);
    return;
  }
  const double af = fabs(f), ag = fabs(g);
  const double big = fmax(af, ag);
  if (big > 1e150 || big < 1e-150) {
    const double u = big;
    const double fs = f / u, gs = g / u;
    const double t = fma(fs, fs, gs * gs);
    const double ri = rsqrt(t);
    c = fabs(fs) * ri;
    r = copysign(t * ri * u, f);
    s = gs * copysign(ri, f);
    return;
  }
  const double t = fma(f, f, g * g);
  const double ri = rsqrt(t);
  c = af * ri;
  r = copysign(t * ri, f);
  s = g * copysign(ri, f);
}

enum S2GKind {
  kGLaLeftB = 0,  // lookahead, U(ib)^T on B rows of block ib, columns istop+1..istop2 (:1035-1045)
  kGLaLeftA = 1,  // lookahead, U(ib)^T on A (:1094-1124)
  kGUpRight = 2,  // delayed right update, rows 1..istart-1 times V(ib) (:1258-1259, :1300-1301)
  kGUpLeft = 3,   // delayed left update, U(ib)^T on columns istop+1..n (:1267-1276, :1306-1331)
  kGUpQ = 4,      // Q(:, block) <- Q(:, block) U(ib) (:1345-1348)
  kGUpZ = 5,      // Z(:, block) <- Z(:, block) V(ib) (:1360-1363)
};

// Dense op lists of a Givens group: one op per block, blocks in the reference's order
// (ib = nblocks .. 1).  Op o applies G = U(ib) or V(ib) as C <- C G / C <- G^T C, stored as
// V = I, T = I - G (WYOp::dense).  The block's rows/columns are base+1 .. base+len (1-based,
// base = J + (ib-1) r, len = min(n - base, r + nq)), the same for A and B in every list.
struct GeoS2G {
  S2GStore S;
  int n, J, r, nq, nblocks, kind;
  __host__ __device__ int count() const { return nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  static constexpr int kSite = 1;  // stage-2 op list (kernel statistics)
  PHT_DEV bool masks_y() const { return false; }
  // every op is a full product C -= C (I - G): the split kernel's one-product form when it fits
  // 32 columns, its wide dense form up to 48
  __host__ __device__ bool one_product_only() const { return r + nq <= 32; }
  __host__ __device__ bool wide_dense() const { return r + nq > 32; }
  PHT_DEV void range(int, const WYOp& w, int, int& a, int& b) const {
    a = 0;
    b = w.k - 1;
  }
  PHT_DEV WYOp op(int o) const {
    const int ib = nblocks - o;
    const int base = J + (ib - 1) * r;
    WYOp w;
    w.start = base;
    w.len = max(0, min(n - base, r + nq));
    w.k = w.len;
    w.dense = 1;
    w.V = S.I;
    w.ldv = S.ldu;
    w.ldt = S.ldu;
    const bool right = kind == kGUpRight || kind == kGUpZ;
    w.T = (right ? S.MV : S.MU) + S.gi(1, 1, ib);
    const int istop2 = min(n, base + r + nq + r * nq - 1);
    switch (kind) {
      case kGLaLeftB:
        w.lo = min(n, base + r + nq - 1);
        w.hi = istop2 - 1;
        break;
      case kGLaLeftA:
        w.lo = (ib == 1) ? min(n, J + nq - 1) : min(n, base - r + nq);
        w.hi = istop2 - 1;
        break;
      case kGUpRight: {
        const int istart = max(J + 1, base + 1 - (2 * nq - 1) * r);
        w.lo = 0;
        w.hi = istart - 2;
        break;
      }
      case kGUpLeft:
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

// Bulge chase of one Givens group (stage2g_chase.cu): nq sweeps, pipelined across CTAs
// (sequential != 0: one CTA, sweeps in order).  Rotations are accumulated into S.U, S.V (which
// must hold the identity for blocks 1..nblocks) and the right rotations stored in S.CV, S.SV.
void s2g_launch_chase(cudaStream_t st, double* A, int lda, double* B, int ldb, int n, int J, int r, int nq,
                      const S2GStore& S, const ChaseSync& sync, int sequential, long long spin_limit);

}  // namespace pht
