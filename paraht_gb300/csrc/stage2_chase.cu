// stage2_chase.cu -- the band-only bulge chase of one stage-2 sweep group, pipelined across CTAs.
//
// Restates the generation loop of src/rht2ht.f90:1450-1596.  Sweep ic (column jc = J+ic-1)
// takes steps ib = 1 (the column itself) and ib = 2, 3, ... (chasing the bulge down by r).
// The reference runs the nq sweeps of a group one after the other.  Here each sweep gets its
// own CTA and starts as soon as the sweep before it is two steps ahead: step ib of sweep ic
// touches columns [jb, jb+2r-1] (jb its reduced column) and reads the left reflectors U(i,ib),
// i < ic; step ib+2 of sweep ic-1 is the last step of that sweep whose footprint intersects
// (the window row jb+2r of column jb+r), and steps >= ib+3 of sweep ic-1 touch only columns
// >= jb+3r-1.  Waiting for "sweep ic-1 has finished step ib+2" therefore reproduces the
// reference's order on every matrix entry, so the pipelined schedule performs exactly the
// sequential arithmetic (the sequential mode, one CTA running the sweeps in order, must give
// bitwise identical results).
//
// Synchronisation: per-sweep progress words in global memory (st.release / ld.acquire at GPU
// scope), a ticket so that sweep ic-1 always starts before sweep ic (no deadlock even when not
// all CTAs are resident), and bounded waits: a wait that exceeds spin_limit polls sets
// status = PARAHT_ERR_TIMEOUT and the CTA returns; waiters also give up as soon as status is set.
// This file is compiled with -Xptxas -dlcm=cg so that global loads bypass L1 and observe the
// other CTAs' writes after the acquire.
#include "../../include/paraht.h"
#include "launch_count.h"
#include "paraht_internal.cuh"
#include "s2_common.cuh"

namespace pht {

struct Smem2 {
  double* red;  // 32
  double* Bc;   // r x r (ld r)
  double* q;    // r
  double* tau;  // r
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
// of the orthogonal factor (row 1 of dorgr2's Q = H(1)...H(nb)), then DLARFG on that row.
// Returns tauV; the reflector tail (entries 2..nb) is left in s.q[1..nb-1].
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
  for (int c = t; c < nb; c += blockDim.x) s.q[c] = (c == 0) ? 1.0 : 0.0;
  __syncthreads();
  for (int i = 0; i < nb; ++i) {
    const double ti = s.tau[i];
    if (ti != 0.0) {
      double p = 0.0;
      for (int c = t; c <= i; c += blockDim.x) p = fma(s.q[c], (c == i) ? 1.0 : Bc[i + c * r], p);
      const double w = block_sum(p, s.red);
      const double tw = ti * w;
      for (int c = t; c <= i; c += blockDim.x) s.q[c] = fma(-tw, (c == i) ? 1.0 : Bc[i + c * r], s.q[c]);
      __syncthreads();
    }
  }
  return cta_larfg(nb, &s.q[0], &s.q[1], 1, s);
}

PHT_DEV int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
PHT_DEV void st_release(int* p, int v) { asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory"); }

// Last step index of sweep ic (1 = only the column step).
PHT_DEV int last_step(int n, int J, int r, int ic) {
  const int jc = J + ic - 1;
  const int nb = min(r, n - jc);
  if (nb < 2) return 1;
  return (n - jc - 1) / r + 2;
}

struct ChaseArgs {
  double* A;
  int lda;
  double* B;
  int ldb;
  int n, J, r, nq;
  S2Store S;
  ChaseSync sync;
  long long spin_limit;
  int pipelined;
};

// Waits until sweep ic-1 has completed step `need`; returns false if the wait was abandoned.
__device__ bool wait_prev(const ChaseArgs& a, int ic, int need, int* abort_flag) {
  if (!a.pipelined || ic <= 1) return true;
  if (threadIdx.x == 0) {
    long long it = 0;
    int ok = 1;
    while (ld_acquire(&a.sync.prog[ic - 1]) < need) {
      if (ld_acquire(a.sync.status) != 0) {
        ok = 0;
        break;
      }
      if (++it > a.spin_limit) {
        atomicCAS(a.sync.status, 0, PARAHT_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(128);
    }
    *abort_flag = !ok;
  }
  __syncthreads();
  return !*abort_flag;
}

__device__ void publish(const ChaseArgs& a, int ic, int step) {
  if (!a.pipelined) return;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release(&a.sync.prog[ic], step);
}

// One sweep: rht2ht.f90:1452-1594 for column jc = J + ic - 1.
__device__ void run_sweep(const ChaseArgs& a, int ic, Smem2& s, int* abort_flag) {
  double* A = a.A;
  double* B = a.B;
  const int lda = a.lda, ldb = a.ldb, n = a.n, J = a.J, r = a.r, nq = a.nq;
  const S2Store& S = a.S;
#define A1(i, j) A[(size_t)((i)-1) + (size_t)((j)-1) * lda]
#define B1(i, j) B[(size_t)((i)-1) + (size_t)((j)-1) * ldb]
  const int t = threadIdx.x;
  const int last_prev = (ic > 1) ? last_step(n, J, r, ic - 1) : 0;
  const int jc = J + ic - 1;
  int nb = min(r, n - jc);
  int istart = J + 1;
  if (!wait_prev(a, ic, min(1 + 2, last_prev), abort_flag)) return;
  // delayed left reflectors of this group on B(J+i.., jc+r) and A(J+i.., jc) (:1466-1482)
  if (jc + r <= n)
    for (int i = 1; i <= ic - 1; ++i) cta_larf_col(r, S.U + S.ui(i, i, 1), S.tauU[S.ti(i, 1)], &B1(J + i, jc + r), s);
  for (int i = 1; i <= ic - 1; ++i)
    if (jc <= n) cta_larf_col(min(r, n - J - i + 1), S.U + S.ui(i, i, 1), S.tauU[S.ti(i, 1)], &A1(J + i, jc), s);
  if (nb >= 2) {
    const double tu = cta_larfg(nb, &A1(jc + 1, jc), &A1(jc + 2, jc), 1, s);  // :1487
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
    cta_larf_left(nb, nb, u, tu, &B1(jc + 1, jc + 1), ldb);  // :1495
    for (int e = t; e < nb * nb; e += blockDim.x) s.Bc[(e % nb) + (e / nb) * r] = B1(jc + 1 + e % nb, jc + 1 + e / nb);
    __syncthreads();
    const double tv = opposite_reflector(nb, r, s);  // :1499-1508
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
  publish(a, ic, 1);
  if (nb < 2) return;  // :1484 skips the chase
  for (int jb = jc + 1; jb <= n; jb += r) {  // :1528
    const int ib = (jb - (jc + 1)) / r + 2;
    if (!wait_prev(a, ic, min(ib + 2, last_prev), abort_flag)) return;
    nb = min(r, n - jb - r + 1);
    istart = max(J + 1, J + 1 + (ib - 1) * r - (nq - ic) * r);
    if (jb + r + r - 1 <= n)  // :1539-1544
      for (int i = 1; i <= ic - 1; ++i)
        cta_larf_col(r, S.U + S.ui(i, i, ib), S.tauU[S.ti(i, ib)], &B1(jb + r - ic + i, jb + r + r - 1), s);
    for (int i = 1; i <= ic - 1; ++i)  // :1550-1553
      if (jb + r - ic + i <= n)
        cta_larf_col(min(r, n - (jb + r - ic + i) + 1), S.U + S.ui(i, i, ib), S.tauU[S.ti(i, ib)],
                     &A1(jb + r - ic + i, jb), s);
    if (nb >= 2) {
      const double tu = cta_larfg(nb, &A1(jb + r, jb), &A1(jb + r + 1, jb), 1, s);  // :1558
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
      for (int e = t; e < nb * nb; e += blockDim.x)
        s.Bc[(e % nb) + (e / nb) * r] = B1(jb + r + e % nb, jb + r + e / nb);
      __syncthreads();
      const double tv = opposite_reflector(nb, r, s);  // :1570-1579
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
    publish(a, ic, ib);
  }
#undef A1
#undef B1
}

constexpr int kChaseThreads = 256;

__global__ void __launch_bounds__(kChaseThreads) k_s2_chase(ChaseArgs a) {
  extern __shared__ double sm[];
  __shared__ int s_ic, s_abort;
  Smem2 s;
  s.red = sm;
  s.Bc = sm + 32;
  s.q = s.Bc + a.r * a.r;
  s.tau = s.q + a.r;
  if (threadIdx.x == 0) s_abort = 0;
  if (!a.pipelined) {
    __syncthreads();
    for (int ic = 1; ic <= a.nq; ++ic) run_sweep(a, ic, s, &s_abort);
    return;
  }
  if (threadIdx.x == 0) s_ic = atomicAdd(a.sync.ticket, 1) + 1;
  __syncthreads();
  run_sweep(a, s_ic, s, &s_abort);
}

void s2_launch_chase(cudaStream_t st, double* A, int lda, double* B, int ldb, int n, int J, int r, int nq,
                     const S2Store& S, const ChaseSync& sync, int sequential, long long spin_limit) {
  ChaseArgs a;
  a.A = A;
  a.lda = lda;
  a.B = B;
  a.ldb = ldb;
  a.n = n;
  a.J = J;
  a.r = r;
  a.nq = nq;
  a.S = S;
  a.sync = sync;
  a.spin_limit = spin_limit;
  a.pipelined = sequential ? 0 : 1;
  const size_t smem = sizeof(double) * (32 + (size_t)r * r + 2 * r + 8);
  if (a.pipelined) {
    cudaMemsetAsync(sync.prog, 0, sizeof(int) * (nq + 1), st);
    cudaMemsetAsync(sync.ticket, 0, sizeof(int), st);
  }
  count_launch();
  k_s2_chase<<<a.pipelined ? nq : 1, kChaseThreads, smem, st>>>(a);
}

}  // namespace pht
