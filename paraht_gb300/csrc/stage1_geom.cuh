// stage1_geom.cuh -- stage-1 panel geometry and its compact-WY op lists (src/ab2rht.f90:71-99).
#pragma once
#include "paraht_internal.cuh"

namespace pht {

// ------------------------------------------------------------------------------------------
// Panel geometry (0-based).  Block o (o = 0 .. nblocks-1) is the o-th block from the bottom.
// ------------------------------------------------------------------------------------------
struct S1Panel {
  int n, nb, p, jb0;  // jb0: first panel column (0-based)
  int nblocks, ibtop0, stride, L;
  PHT_DEV __host__ int ib(int o) const { return ibtop0 - o * stride; }
  PHT_DEV __host__ int ib2(int o) const { return min(n - 1, ib(o) + L - 1); }
  PHT_DEV __host__ int nb2(int o) const { return ib2(o) - ib(o) + 1; }
};

__host__ __device__ inline S1Panel make_panel(int n, int nb, int p, int jb0) {
  S1Panel g;
  g.n = n;
  g.nb = nb;
  g.p = p;
  g.jb0 = jb0;
  const int m = n - nb - jb0;  // rows jb0+nb .. n-1  (ab2rht.f90:74: n-nb-jb+1 with 1-based jb)
  g.stride = (p - 1) * nb;
  g.nblocks = (m + g.stride - 1) / g.stride;
  g.L = p * nb;
  g.ibtop0 = jb0 + nb + (g.nblocks - 1) * g.stride;
  return g;
}

// Left ops of the panel on B (columns >= ib) or A (columns >= jb+nb): dlarfb('L','T','F','C').
struct GeoS1Left {
  S1Panel P;
  const double* VL;
  const double* TL;
  int onA;
  __host__ __device__ int count() const { return P.nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  static constexpr int kSite = 0;  // stage-1 op list (kernel statistics)
  PHT_DEV bool masks_y() const { return false; }
  // every op applies all its reflectors to every row; one product C -= C M when spans are <= 32
  __host__ __device__ bool one_product_only() const { return P.L <= 32; }
  __host__ __device__ bool wide_dense() const { return false; }
  PHT_DEV void range(int, const WYOp& w, int, int& a, int& b) const {
    a = 0;
    b = w.k - 1;
  }
  PHT_DEV WYOp op(int o) const {
    WYOp w;
    w.start = P.ib(o);
    w.len = P.nb2(o);
    w.k = min(P.nb, w.len);
    w.lo = onA ? P.jb0 + P.nb : P.ib(o);
    w.hi = P.n - 1;
    w.V = VL + (size_t)o * P.L * P.nb;
    w.ldv = P.L;
    w.T = TL + (size_t)o * P.nb * P.nb;
    w.ldt = P.nb;
    return w;
  }
};

// Right ops of the panel's left reflectors on Q: Q(:, ib:ib2) <- Q H (ab2rht.f90:241).
struct GeoS1Q {
  S1Panel P;
  const double* VL;
  const double* TL;
  __host__ __device__ int count() const { return P.nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  static constexpr int kSite = 0;  // stage-1 op list (kernel statistics)
  PHT_DEV bool masks_y() const { return false; }
  // every op applies all its reflectors to every row; one product C -= C M when spans are <= 32
  __host__ __device__ bool one_product_only() const { return P.L <= 32; }
  __host__ __device__ bool wide_dense() const { return false; }
  PHT_DEV void range(int, const WYOp& w, int, int& a, int& b) const {
    a = 0;
    b = w.k - 1;
  }
  PHT_DEV WYOp op(int o) const {
    WYOp w;
    w.start = P.ib(o);
    w.len = P.nb2(o);
    w.k = min(P.nb, w.len);
    w.lo = 0;
    w.hi = P.n - 1;
    w.V = VL + (size_t)o * P.L * P.nb;
    w.ldv = P.L;
    w.T = TL + (size_t)o * P.nb * P.nb;
    w.ldt = P.nb;
    return w;
  }
};

// Right reflectors (stored transposed in VRc) on A, Z (all rows) or on B (rows up to ib2 of a
// single block, bl_only >= 0).
struct GeoS1Right {
  S1Panel P;
  const double* VRc;
  const double* TR;
  int bl_only;  // -1: all blocks, all rows; else only block bl_only, rows [row_lo, row_hi]
  int row_lo = 0, row_hi = -1;
  __host__ __device__ int count() const { return bl_only >= 0 ? 1 : P.nblocks; }
  PHT_DEV int slot_op(int s) const { return s; }
  PHT_DEV int op_slot(int o) const { return o; }
  static constexpr int kSite = 0;  // stage-1 op list (kernel statistics)
  PHT_DEV bool masks_y() const { return false; }
  // every op applies all its reflectors to every row; one product C -= C M when spans are <= 32
  __host__ __device__ bool one_product_only() const { return P.L <= 32; }
  __host__ __device__ bool wide_dense() const { return false; }
  PHT_DEV void range(int, const WYOp& w, int, int& a, int& b) const {
    a = 0;
    b = w.k - 1;
  }
  PHT_DEV WYOp op(int i) const {
    const int o = bl_only >= 0 ? bl_only : i;
    WYOp w;
    w.start = P.ib(o);
    w.len = P.nb2(o);
    w.k = (w.len > P.nb) ? P.nb : w.len;
    w.lo = bl_only >= 0 ? row_lo : 0;
    w.hi = bl_only >= 0 ? row_hi : P.n - 1;
    w.V = VRc + (size_t)o * P.L * P.nb;
    w.ldv = P.L;
    w.T = TR + (size_t)o * P.nb * P.nb;
    w.ldt = P.nb;
    return w;
  }
};

}  // namespace pht
