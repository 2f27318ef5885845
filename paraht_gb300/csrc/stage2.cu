// stage2.cu -- stage 2 of the HT reduction on the GPU: (A r-Hessenberg, B triangular) ->
// (A Hessenberg, B triangular), accumulating Q and Z.
//
// Follows src/rht2ht.f90:1346-2051 (rht2ht_householder).  For each group of nq columns
// starting at jblock (rht2ht.f90:1417):
//   1. k_s2_generate: the band-only bulge chase of the group's nq columns (rht2ht.f90:1433-1596),
//      producing nq left reflectors U(:,ic,ib) and nq right reflectors V(:,ic,ib) per block ib.
//   2. k_s2_form_t: TU, TV for every block (dlarft 'F','C', rht2ht.f90:1599-1610).
//   3. lookahead updates of B and A (rht2ht.f90:1630-1772) and the delayed bulk updates of B, A,
//      Q and Z (rht2ht.f90:1803-2024), each an ordered compact-WY op list (wy_apply.cuh) whose
//      row/column ranges are the reference's staircase (istart/istart2/istop/istop2).
// The reference double-buffers the reflectors (rht2ht.f90:1786-1797) so that the next
// generation overlaps the bulk updates; here the stream order already serialises them.
#include <algorithm>

#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "wy_apply.cuh"

namespace pht {

// ------------------------------------------------------------------------------------------
// Reflector storage for one group: U, V (ldu = r+nq) x nq x nblk, TU, TV nq x nq x nblk,
// tauU, tauV nq x nblk.  Helpers take the reference's 1-based (i, ic, ib).
// ------------------------------------------------------------------------------------------
struct S2Store {
  double *U, *V, *TU, *TV, *tauU, *tauV;
  int ldu, nq;
  PHT_DEV __host__ size_t ui(int i, int ic, int ib) const {
    return (size_t)(i - 1) + (size_t)(ic - 1) * ldu + (size_t)(ib - 1) * ldu * nq;
  }
  PHT_DEV __host__ size_t ti(int ic, int ib) const { return (size_t)(ic - 1) + (size_t)(ib - 1) * nq; }
  PHT_DEV __host__ size_t tt(int ib) const { return (size_t)(ib - 1) * nq * nq; }
};

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

// ------------------------------------------------------------------------------------------
// CTA-cooperative level-2 helpers on global memory (all threads call them; they end with a
// __syncthreads so the result is visible to the whole CTA).
// ------------------------------------------------------------------------------------------
struct Smem2 {
  double* red;  // 32
  double* Bc;   // r x r (ld r)
  double* q;    // r
  double* tau;  // r
  double* sc;   // scalars
};

// c <- (I - tau v v^T) c for one column c (length m, contiguous): dlarf('L', m, 1, ...).
__device__ void cta_larf_col(int m, const double* v, double tau, double* c, Smem2& s) {
  if (m <= 0 || tau == 0.0) return;
  double p = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) p = fma(v[i], c[i], p);
  const double w = block_sum(p, s.red);
  const double tw = tau * w;
  for (int i = threadIdx.x; i < m; i += blockDim.x) c[i] = fma(-tw, v[i], c[i]);
  __syncthreads();
}

// C (m x nc, ld ldc) <- (I - tau v v^T) C: dlarf('L', m, nc, ...).  One warp per column.
__device__ void cta_larf_left(int m, int nc, const double* v, double tau, double* C, int ldc) {
  if (m <= 0 || nc <= 0 || tau == 0.0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < nc; j += nw) {
    double* c = C + (size_t)j * ldc;
    double p = 0.0;
    for (int i = lane; i < m; i += 32) p = fma(v[i], c[i], p);
    const double tw = tau * warp_sum(p);
    for (int i = lane; i < m; i += 32) c[i] = fma(-tw, v[i], c[i]);
  }
  __syncthreads();
}

// C (mr x nc, ld ldc) <- C (I - tau v v^T): dlarf('R', mr, nc, ...).  One thread per row.
__device__ void cta_larf_right(int mr, int nc, const double* v, double tau, double* C, int ldc) {
  if (mr <= 0 || nc <= 0 || tau == 0.0) return;
  for (int i = threadIdx.x; i < mr; i += blockDim.x) {
    double a0 = 0, a1 = 0;
    int j = 0;
    for (; j + 1 < nc; j += 2) {
      a0 = fma(C[i + (size_t)j * ldc], v[j], a0);
      a1 = fma(C[i + (size_t)(j + 1) * ldc], v[j + 1], a1);
    }
    if (j < nc) a0 = fma(C[i + (size_t)j * ldc], v[j], a0);
    const double tw = tau * (a0 + a1);
    for (j = 0; j < nc; ++j) C[i + (size_t)j * ldc] = fma(-tw, v[j], C[i + (size_t)j * ldc]);
  }
  __syncthreads();
}

// DLARFG on (alpha, x[0..m-2] with stride incx); writes beta to *alpha, scales x, returns tau.
__device__ double cta_larfg(int m, double* alpha, double* x, int incx, Smem2& s) {
  if (m <= 1) {
    __syncthreads();
    return 0.0;
  }
  double p = 0.0;
  for (int i = threadIdx.x; i < m - 1; i += blockDim.x) p = fma(x[(size_t)i * incx], x[(size_t)i * incx], p);
  const double ss = block_sum(p, s.red);
  const Reflector h = make_reflector(*alpha, ss);
  __syncthreads();
  for (int i = threadIdx.x; i < m - 1; i += blockDim.x) x[(size_t)i * incx] *= h.scal;
  if (threadIdx.x == 0) *alpha = h.beta;
  __syncthreads();
  return h.tau;
}

// "Opposite" reflector of rht2ht.f90:1499-1508: RQ of the nb x nb block Bc (dgerq2), first row
// of the orthogonal factor (dorgr2 row 1), then DLARFG on that row.  Returns tauV and leaves
// the reflector tail (entries 2..nb) in s.q[1..nb-1].
__device__ double opposite_reflector(int nb, int r, Smem2& s) {
  double* Bc = s.Bc;
  const int t = threadIdx.x;
  for (int i = nb - 1; i >= 0; --i) {  // dgerq2: rows bottom to top
    double p = 0.0;
    for (int c = t; c < i; c += blockDim.x) p = fma(Bc[i + c * r], Bc[i + c * r], p);
    const double ss = block_sum(p, s.red);
    const Reflector h = make_reflector(Bc[i + i * r], ss);
    __syncthreads();
    for (int c = t; c < i; c += blockDim.x) Bc[i + c * r] *= h.scal;
    __syncthreads();
    if (h.tau != 0.0) {
      for (int rho = t; rho < i; rho += blockDim.x) {
        double w = Bc[rho + i * r];
        for (int c = 0; c < i; ++c) w = fma(Bc[rho + c * r], Bc[i + c * r], w);
        const double tw = h.tau * w;
        for (int c = 0; c < i; ++c) Bc[rho + c * r] = fma(-tw, Bc[i + c * r], Bc[rho + c * r]);
        Bc[rho + i * r] -= tw;
      }
    }
    __syncthreads();
    if (t == 0) {
      Bc[i + i * r] = h.beta;
      s.tau[i] = h.tau;
    }
    __syncthreads();
  }
  // q = e1^T H(1) H(2) ... H(nb)   (row 1 of dorgr2's Q)
  for (int c = t; c < nb; c += blockDim.x) s.q[c] = (c == 0) ? 1.0 : 0.0;
  __syncthreads();
  for (int i = 0; i < nb; ++i) {
    const double ti = s.tau[i];
    if (ti != 0.0) {
      // w = q . v_i (v_i = [Bc(i, 0:i-1), 1])
      double p = 0.0;
      for (int c = t; c <= i; c += blockDim.x) p = fma(s.q[c], (c == i) ? 1.0 : Bc[i + c * r], p);
      const double w = block_sum(p, s.red);
      const double tw = ti * w;
      for (int c = t; c <= i; c += blockDim.x) s.q[c] = fma(-tw, (c == i) ? 1.0 : Bc[i + c * r], s.q[c]);
      __syncthreads();
    }
  }
  // DLARFG on the first row: alpha = q[0], x = q[1..nb-1]
  return cta_larfg(nb, &s.q[0], &s.q[1], 1, s);
}

constexpr int kS2GenThreads = 256;

// One CTA: the generation loop of rht2ht.f90:1450-1596 for group jblock = J (1-based).
__global__ void __launch_bounds__(kS2GenThreads) k_s2_generate(double* __restrict__ A, int lda,
                                                                double* __restrict__ B, int ldb, int n, int J, int r,
                                                                int nq, S2Store S) {
  extern __shared__ double sm[];
  Smem2 s;
  s.red = sm;
  s.Bc = sm + 32;
  s.q = s.Bc + r * r;
  s.tau = s.q + r;
  s.sc = s.tau + r;
#define A1(i, j) A[(size_t)((i)-1) + (size_t)((j)-1) * lda]
#define B1(i, j) B[(size_t)((i)-1) + (size_t)((j)-1) * ldb]
  const int t = threadIdx.x;
  for (int ic = 1; ic <= nq; ++ic) {
    const int jc = J + ic - 1;
    int nb = min(r, n - jc);
    int istart = J + 1;
    // delayed left reflectors of this group on B(J+i.., jc+r) and A(J+i.., jc) (:1466-1482)
    if (jc + r <= n)
      for (int i = 1; i <= ic - 1; ++i) cta_larf_col(r, S.U + S.ui(i, i, 1), S.tauU[S.ti(i, 1)], &B1(J + i, jc + r), s);
    for (int i = 1; i <= ic - 1; ++i)
      if (jc <= n)
        cta_larf_col(min(r, n - J - i + 1), S.U + S.ui(i, i, 1), S.tauU[S.ti(i, 1)], &A1(J + i, jc), s);
    if (nb < 2) continue;
    {
      // left reflector on A(jc+1:jc+nb, jc) (:1487-1496)
      const double tu = cta_larfg(nb, &A1(jc + 1, jc), &A1(jc + 2, jc), 1, s);
      double* u = S.U + S.ui(ic, ic, 1);
      for (int i = 2 + t; i <= nb; i += blockDim.x) {
        u[i - 1] = A1(jc + i, jc);
        A1(jc + i, jc) = 0.0;
      }
      if (t == 0) {
        u[0] = 1.0;
        S.tauU[S.ti(ic, 1)] = tu;
      }
      __syncthreads();
      cta_larf_left(nb, nb, u, tu, &B1(jc + 1, jc + 1), ldb);
      // opposite reflector from the RQ of the B block (:1499-1508)
      for (int e = t; e < nb * nb; e += blockDim.x) s.Bc[(e % nb) + (e / nb) * r] = B1(jc + 1 + e % nb, jc + 1 + e / nb);
      __syncthreads();
      const double tv = opposite_reflector(nb, r, s);
      double* v = S.V + S.ui(ic, ic, 1);
      for (int i = 2 + t; i <= nb; i += blockDim.x) v[i - 1] = s.q[i - 1];
      if (t == 0) {
        v[0] = 1.0;
        S.tauV[S.ti(ic, 1)] = tv;
      }
      __syncthreads();
      cta_larf_right(min(n, jc + r + nb) - jc, nb, v, tv, &A1(jc + 1, jc + 1), lda);  // :1510
      cta_larf_right(nb, nb, v, tv, &B1(jc + 1, jc + 1), ldb);                          // :1513
      for (int i = 2 + t; i <= nb; i += blockDim.x) B1(jc + i, jc + 1) = 0.0;
      __syncthreads();
      cta_larf_right(jc - istart + 1, nb, v, tv, &A1(istart, jc + 1), lda);  // :1518
      cta_larf_right(jc - istart + 1, nb, v, tv, &B1(istart, jc + 1), ldb);  // :1520
    }
    // chase the bulge down (:1528-1594)
    for (int jb = jc + 1; jb <= n; jb += r) {
      const int ib = (jb - (jc + 1)) / r + 2;
      nb = min(r, n - jb - r + 1);
      istart = max(J + 1, J + 1 + (ib - 1) * r - (nq - ic) * r);
      if (jb + r + r - 1 <= n)
        for (int i = 1; i <= ic - 1; ++i)
          cta_larf_col(r, S.U + S.ui(i, i, ib), S.tauU[S.ti(i, ib)], &B1(jb + r - ic + i, jb + r + r - 1), s);
      for (int i = 1; i <= ic - 1; ++i)
        if (jb + r - ic + i <= n)
          cta_larf_col(min(r, n - (jb + r - ic + i) + 1), S.U + S.ui(i, i, ib), S.tauU[S.ti(i, ib)],
                       &A1(jb + r - ic + i, jb), s);
      if (nb < 2) continue;
      const double tu = cta_larfg(nb, &A1(jb + r, jb), &A1(jb + r + 1, jb), 1, s);
      double* u = S.U + S.ui(ic, ic, ib);
      for (int i = 1 + t; i <= nb - 1; i += blockDim.x) {
        u[i] = A1(jb + r + i, jb);
        A1(jb + r + i, jb) = 0.0;
      }
      if (t == 0) {
        u[0] = 1.0;
        S.tauU[S.ti(ic, ib)] = tu;
      }
      __syncthreads();
      cta_larf_left(nb, nb, u, tu, &B1(jb + r, jb + r), ldb);  // :1566
      for (int e = t; e < nb * nb; e += blockDim.x) s.Bc[(e % nb) + (e / nb) * r] = B1(jb + r + e % nb, jb + r + e / nb);
      __syncthreads();
      const double tv = opposite_reflector(nb, r, s);
      double* v = S.V + S.ui(ic, ic, ib);
      for (int i = 2 + t; i <= nb; i += blockDim.x) v[i - 1] = s.q[i - 1];
      if (t == 0) {
        v[0] = 1.0;
        S.tauV[S.ti(ic, ib)] = tv;
      }
      __syncthreads();
      cta_larf_right(min(n, jb + 2 * r + nb - 1) - jb - r + 1, nb, v, tv, &A1(jb + r, jb + r), lda);  // :1581
      cta_larf_right(nb, nb, v, tv, &B1(jb + r, jb + r), ldb);                                        // :1584
      for (int i = 1 + t; i <= nb - 1; i += blockDim.x) B1(jb + r + i, jb + r) = 0.0;
      __syncthreads();
      cta_larf_right(jb + r - istart, nb, v, tv, &A1(istart, jb + r), lda);  // :1589
      cta_larf_right(jb + r - istart, nb, v, tv, &B1(istart, jb + r), ldb);  // :1591
    }
  }
#undef A1
#undef B1
}

// TU / TV of every block (rht2ht.f90:1599-1610): one CTA per block and per factor.
__global__ void k_s2_form_t(int n, int J, int r, int nq, int nblocks, S2Store S) {
  extern __shared__ double smt[];
  double* G = smt;             // nq*nq
  double* Ts = smt + nq * nq;  // nq*nq
  const int ib = blockIdx.x + 1;
  const bool isV = blockIdx.y == 1;
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
  return sizeof(double) * (2 * ldu * nq * nb0 + 2 * (size_t)nq * nq * nb0 + 2 * (size_t)nq * nb0) + 4096;
}

int s2_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r, int nq,
           PhaseTimer* timer) {
  if (n < 3) return 0;  // rht2ht.f90:1417: empty loop
  cudaStream_t st = ctx.stream;
  const int nb0 = s2_nblk0(n, r);
  const int ldu = r + nq;
  double* ws = (double*)ctx.workspace(s2_workspace_bytes(n, r, nq));
  if (!ws) return PARAHT_ERR_ALLOC;
  S2Store S;
  S.ldu = ldu;
  S.nq = nq;
  S.U = ws;
  S.V = S.U + (size_t)ldu * nq * nb0;
  S.TU = S.V + (size_t)ldu * nq * nb0;
  S.TV = S.TU + (size_t)nq * nq * nb0;
  S.tauU = S.TV + (size_t)nq * nq * nb0;
  S.tauV = S.tauU + (size_t)nq * nb0;
  const size_t gen_smem = sizeof(double) * (32 + (size_t)r * r + 2 * r + 8);
  for (int J = 1; J <= n - 2; J += nq) {  // rht2ht.f90:1417
    const int nblocks = (n - J + r - 1) / r;
    const int nz = std::min(nb0, nblocks + 2);
    if (timer) timer->mark(st, 0);
    cudaMemsetAsync(S.U, 0, sizeof(double) * (size_t)ldu * nq * nz, st);
    cudaMemsetAsync(S.V, 0, sizeof(double) * (size_t)ldu * nq * nz, st);
    cudaMemsetAsync(S.tauU, 0, sizeof(double) * (size_t)nq * nz, st);
    cudaMemsetAsync(S.tauV, 0, sizeof(double) * (size_t)nq * nz, st);
    k_s2_generate<<<1, kS2GenThreads, gen_smem, st>>>(A, lda, B, ldb, n, J, r, nq, S);
    k_s2_form_t<<<dim3(nblocks, 2), 128, sizeof(double) * 2 * nq * nq, st>>>(n, J, r, nq, nblocks, S);
    if (timer) timer->mark(st, 1);
    const GeoS2 base{S, n, J, r, nq, nblocks, 0};
    GeoS2 g = base;
    g.kind = kLaRight;
    launch_apply_right(B, ldb, 0, n - 1, g, st);
    launch_apply_right(A, lda, 0, n - 1, g, st);
    g.kind = kLaLeftB;
    launch_apply_left(B, ldb, 0, n - 1, g, st);
    g.kind = kLaLeftA;
    launch_apply_left(A, lda, 0, n - 1, g, st);
    if (timer) timer->mark(st, 2);
    g.kind = kUpRight;
    launch_apply_right(B, ldb, 0, n - 1, g, st);
    launch_apply_right(A, lda, 0, n - 1, g, st);
    g.kind = kUpLeft;
    launch_apply_left(B, ldb, 0, n - 1, g, st);
    launch_apply_left(A, lda, 0, n - 1, g, st);
    g.kind = kUpQ;
    launch_apply_right(Q, ldq, 0, n - 1, g, st);
    g.kind = kUpZ;
    launch_apply_right(Z, ldz, 0, n - 1, g, st);
  }
  if (timer) timer->mark(st, -1);
  return 0;
}

}  // namespace pht
