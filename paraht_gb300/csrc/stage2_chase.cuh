// stage2_chase.cuh -- device code of the band-only bulge chase of one stage-2 sweep group, pipelined across CTAs.
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
// sequential arithmetic (the sequential mode, one CTA running the sweeps in order, gives
// bitwise identical results).
//
// Latency: a dependent FP64 instruction costs about 64 cycles on GB300, so every step keeps
// its small problems in registers/shared memory, uses warp shuffles (groups of 4 lanes per
// row or column) instead of CTA-wide reductions, and
//  * applies the delayed left reflectors U(1..ic-1, ib) to an entering column as one compact-WY
//    block (c <- c - U T^T U^T c; the reference applies them one by one, rht2ht.f90:1466-1482,
//    :1539-1553 -- same product, other rounding).  The forward triangular factor TU of every
//    block is built column by column as the sweeps generate its reflectors: sweep ic adds
//    column ic of TU(:,:,ib) right after generating U(ic, ib) (the result is dlarft's TU,
//    rht2ht.f90:1599-1603);
//  * fuses the four right-reflector updates of a step (A and B windows, rows above) into one
//    pass over independent rows;
//  * runs eight warps per sweep so that the FP64 updates of a step (rows above the window in
//    particular) are spread over all four schedulers of the SM.
//
// Synchronisation: per-sweep progress words in global memory (st.release / ld.acquire at GPU
// scope), a ticket so that sweep ic-1 always starts before sweep ic (no deadlock even when not
// all CTAs are resident), and bounded waits: a wait that exceeds spin_limit polls sets
// status = PARAHT_ERR_TIMEOUT and the CTA returns; waiters also give up as soon as status is set.
// The pipelined kernel's translation unit is compiled with -Xptxas -dlcm=cg so that global loads
// bypass L1 and observe the other CTAs' writes after the acquire.  The sequential mode (one CTA)
// needs neither.
//
// The kernel of the single-pencil path is in stage2_chase.cu; the persistent batched kernel
// (batched.cu) runs the same sweeps in the sequential mode.
#pragma once
#include "../../include/paraht.h"
#include "paraht_internal.cuh"
#include "s2_common.cuh"

namespace pht {

template <int G>
PHT_DEV double gsum(double v) {
#pragma unroll
  for (int o = 1; o < G; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
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

// Shared memory of one sweep CTA (r <= 64, nq <= 64).
struct Sm {
  double* Bc;   // r x r (ld r+1): the RQ'd B block
  double* y;    // nq       : U^T c / T^T y
  double* z;    // nq
  double* d;    // r        : per-row dot products
  double* q;    // r        : first row of the RQ orthogonal factor
  double* tau;  // r
  double* sc;   // 8 scalars
  double* red;  // 32
  int* abort_flag;
  int ldr;      // leading dimension of Bc (r + 1)
};

constexpr int kChaseMaxThreads = 256;

// Waits until sweep ic-1 has completed step `need`; returns false if the wait was abandoned.
static __device__ bool wait_prev(const ChaseArgs& a, int ic, int need, int* abort_flag) {
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
      __nanosleep(64);
    }
    *abort_flag = !ok;
  }
  __syncthreads();
  return !*abort_flag;
}

static __device__ void publish(const ChaseArgs& a, int ic, int step) {
  if (!a.pipelined) return;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release(&a.sync.prog[ic], step);
}

// c <- H_{m}...H_1 c = c - U T^T U^T c for the first m reflectors of block `ib` (forward
// T = TU(:,:,ib), reflector i stored at U(i:, i, ib), column frame: row f+i-1 of the block is
// entry i-1 of U's column).  c points at the matrix entry of block row 1 (row jb_blk+1);
// `len` limits the rows that exist (n).  All threads participate.
static __device__ void apply_delayed_left(const S2Store& S, int ib, int m, double* c, int len, Sm& s) {
  if (m <= 0 || len <= 0) return;
  const int t = threadIdx.x, nt = blockDim.x;
  const double* U = S.U + S.ui(1, 1, ib);
  const double* T = S.TU + S.tt(ib);
  const int ldu = S.ldu, nq = S.nq;
  // y_j = u_j . c  (u_j nonzero on frame rows j .. j+r-1), 4 lanes per j; uniform loop bounds
  // so that every lane takes part in the shuffles
  for (int base = 0; base < m; base += nt / 4) {
    const int j = base + t / 4, part = t % 4;
    double acc = 0.0;
    if (j < m) {
      const int hi = min(len, ldu);  // frame rows of the block: 0 .. ldu-1
      for (int i = j + part; i < hi; i += 4) acc = fma(U[i + (size_t)j * ldu], c[i], acc);
    }
    acc = gsum<4>(acc);
    if (part == 0 && j < m) s.y[j] = acc;
  }
  __syncthreads();
  // z = T^T y :  z_j = sum_{l<=j} T[l][j] y_l
  for (int j = t; j < m; j += nt) {
    double acc = 0.0;
    for (int l = 0; l <= j; ++l) acc = fma(T[l + (size_t)j * nq], s.y[l], acc);
    s.z[j] = acc;
  }
  __syncthreads();
  // c -= U z  (row i gets contributions from reflectors j with j <= i < j + r)
  for (int i = t; i < len; i += nt) {
    double acc = 0.0;
    const int jlo = max(0, i - S.ldu + 1), jhi = min(m - 1, i);
    for (int j = jlo; j <= jhi; ++j) acc = fma(U[i + (size_t)j * ldu], s.z[j], acc);
    c[i] -= acc;
  }
  __syncthreads();
}

// Column ic of the forward T of block ib: T[0:ic-1, ic-1] = -tau * T_prev (U_prev^T u_ic),
// T[ic-1][ic-1] = tau (dlarft 'F','C').  u_ic = U(:, ic, ib) (already stored).
static __device__ void add_t_column(const S2Store& S, int ib, int ic, double tau, int len, Sm& s) {
  const int t = threadIdx.x, nt = blockDim.x;
  const double* U = S.U + S.ui(1, 1, ib);
  double* T = S.TU + S.tt(ib);
  const int ldu = S.ldu, nq = S.nq, m = ic - 1;
  const double* u = U + (size_t)m * ldu;
  for (int base = 0; base < m; base += nt / 4) {  // y_j = u_j . u_m, j < m
    const int j = base + t / 4, part = t % 4;
    double acc = 0.0;
    if (j < m) {
      const int hi = min(len, ldu);  // frame rows of the block: 0 .. ldu-1
      for (int i = m + part; i < hi; i += 4) acc = fma(U[i + (size_t)j * ldu], u[i], acc);
    }
    acc = gsum<4>(acc);
    if (part == 0 && j < m) s.y[j] = acc;
  }
  __syncthreads();
  for (int l = t; l < m; l += nt) {
    double acc = 0.0;
    for (int q = l; q < m; ++q) acc = fma(T[l + (size_t)q * nq], s.y[q], acc);
    T[l + (size_t)m * nq] = -tau * acc;
  }
  if (t == 0) T[m + (size_t)m * nq] = tau;
  for (int l = m + 1 + t; l < nq; l += nt) T[l + (size_t)m * nq] = 0.0;
  __syncthreads();
}

// DLARFG on the contiguous column x[0..m-1] (alpha = x[0]); 4-lane groups across the CTA.
// Writes beta to x[0], the scaled tail to x[1..], returns tau (same value in every thread).
static __device__ double larfg_col(int m, double* x, Sm& s) {
  if (m <= 1) {
    __syncthreads();
    return 0.0;
  }
  const int t = threadIdx.x, nt = blockDim.x;
  double p = 0.0;
  for (int i = 1 + t; i < m; i += nt) p = fma(x[i], x[i], p);
  p = gsum<32>(p);
  const int w = t >> 5, lane = t & 31;
  if (lane == 0) s.red[w] = p;
  __syncthreads();
  double ss = 0.0;
  for (int k = 0; k < (nt >> 5); ++k) ss += s.red[k];
  const Reflector h = make_reflector(x[0], ss);
  __syncthreads();
  for (int i = 1 + t; i < m; i += nt) x[i] *= h.scal;
  if (t == 0) x[0] = h.beta;
  __syncthreads();
  return h.tau;
}

// Up to four row ranges updated by the same right reflector (dlarf 'R'): 4 lanes per row.
struct RightJob {
  double* C;
  int ld, rows;
};
static __device__ void larf_right4(const RightJob* jobs, int njobs, int nc, const double* v, double tau) {
  if (nc <= 0 || tau == 0.0) {
    __syncthreads();
    return;
  }
  const int t = threadIdx.x, nt = blockDim.x;
  int total = 0;
  for (int k = 0; k < njobs; ++k) total += max(0, jobs[k].rows);
  for (int base = 0; base < total; base += nt / 4) {
    int e = base + t / 4;
    const int part = t % 4;
    double* C = nullptr;
    int ld = 0;
    bool valid = e < total;
    if (valid) {
      for (int k = 0; k < njobs; ++k) {
        const int rk = max(0, jobs[k].rows);
        if (e < rk) {
          C = jobs[k].C + e;
          ld = jobs[k].ld;
          break;
        }
        e -= rk;
      }
    }
    double acc = 0.0;
    if (valid)
      for (int j = part; j < nc; j += 4) acc = fma(C[(size_t)j * ld], v[j], acc);
    acc = gsum<4>(acc);
    if (valid) {
      const double tw = tau * acc;
      for (int j = part; j < nc; j += 4) C[(size_t)j * ld] = fma(-tw, v[j], C[(size_t)j * ld]);
    }
  }
  __syncthreads();
}

// "Opposite" reflector of rht2ht.f90:1499-1508: RQ (dgerq2) of the nb x nb block in s.Bc,
// first row q of the orthogonal factor (row 1 of dorgr2's H(1)...H(nb)), DLARFG on q.
// Returns tauV; the reflector tail (entries 2..nb) is left in s.q[1..nb-1].
static __device__ double opposite_reflector(int nb, int ldb, Sm& s) {
  double* Bc = s.Bc;
  const int t = threadIdx.x;
  const int rho = t / 4, part = t % 4;  // 4 lanes per row; nt/4 >= r rows
  for (int i = nb - 1; i >= 0; --i) {
    double acc = 0.0;
    if (rho <= i)
      for (int c = part; c < i; c += 4) acc = fma(Bc[rho + c * ldb], Bc[i + c * ldb], acc);
    acc = gsum<4>(acc);
    if (part == 0 && rho <= i) s.d[rho] = acc;
    if (rho == i && part == 0) {
      const Reflector h = make_reflector(Bc[i + i * ldb], acc);
      s.sc[0] = h.tau;
      s.sc[1] = h.scal;
      s.sc[2] = h.beta;
    }
    __syncthreads();
    const double ti = s.sc[0], scal = s.sc[1], beta = s.sc[2];
    if (rho < i && ti != 0.0) {
      const double w = Bc[rho + i * ldb] + scal * s.d[rho];
      const double tw = ti * w, tws = tw * scal;
      for (int c = part; c < i; c += 4) Bc[rho + c * ldb] = fma(-tws, Bc[i + c * ldb], Bc[rho + c * ldb]);
      if (part == 0) Bc[rho + i * ldb] -= tw;
    }
    __syncthreads();
    if (rho == i) {
      for (int c = part; c < i; c += 4) Bc[i + c * ldb] *= scal;
      if (part == 0) {
        Bc[i + i * ldb] = beta;
        s.tau[i] = ti;
      }
    }
  }
  __syncthreads();
  // q = e1^T H(1) H(2) ... H(nb): one warp, lane c holds q[c] (nb <= 64 -> 2 per lane)
  if (t < 32) {
    double q0 = (t == 0) ? 1.0 : 0.0, q1 = 0.0;  // q[t], q[t+32]
    for (int i = 0; i < nb; ++i) {
      const double ti = s.tau[i];
      if (ti == 0.0) continue;
      // v_i = [Bc(i, 0:i-1), 1, 0...]
      const double v0 = (t < i) ? Bc[i + t * ldb] : (t == i ? 1.0 : 0.0);
      const double v1 = (t + 32 < i) ? Bc[i + (t + 32) * ldb] : (t + 32 == i ? 1.0 : 0.0);
      const double w = gsum<32>(fma(q0, v0, q1 * v1));
      const double tw = ti * w;
      q0 = fma(-tw, v0, q0);
      q1 = fma(-tw, v1, q1);
    }
    if (t < nb) s.q[t] = q0;
    if (t + 32 < nb) s.q[t + 32] = q1;
  }
  __syncthreads();
  return larfg_col(nb, s.q, s);
}

// C (m x nc, ld ldc) <- (I - tau v v^T) C (dlarf 'L') by the threads t >= t0 only (t0 a multiple
// of 32), 4 lanes per column, without a barrier.
static __device__ void larf_left_part(int m, int nc, const double* v, double tau, double* C, int ldc, int t0) {
  const int t = (int)threadIdx.x - t0, nt = (int)blockDim.x - t0;
  if (t < 0 || m <= 0 || nc <= 0 || tau == 0.0) return;
  for (int base = 0; base < nc; base += nt / 4) {
    const int j = base + t / 4, part = t % 4;
    double acc = 0.0;
    if (j < nc)
      for (int i = part; i < m; i += 4) acc = fma(v[i], C[i + (size_t)j * ldc], acc);
    acc = gsum<4>(acc);
    if (j < nc) {
      const double tw = tau * acc;
      for (int i = part; i < m; i += 4) C[i + (size_t)j * ldc] = fma(-tw, v[i], C[i + (size_t)j * ldc]);
    }
  }
}

// The B block at Bblk (nb x nb) <- H_u Bblk (rht2ht.f90:1495 / :1566) and the opposite reflector
// of the product (:1499-1508 / :1570-1579).  Returns tau_v; the reflector tail is in s.q[1..nb-1].
// (The block is a general matrix here: the sweeps of a group leave fill below its diagonal that
// later sweeps remove, so the first row of its RQ factor needs the full factorisation.)
static __device__ double left_and_opposite(int nb, const double* u, double tu, double* Bblk, int ldb, Sm& s) {
  const int t = threadIdx.x, ldr = s.ldr;
  larf_left_part(nb, nb, u, tu, Bblk, ldb, 0);
  __syncthreads();
  for (int e = t; e < nb * nb; e += blockDim.x) s.Bc[(e % nb) + (e / nb) * ldr] = Bblk[(e % nb) + (size_t)(e / nb) * ldb];
  __syncthreads();
  return opposite_reflector(nb, ldr, s);
}

// One sweep: rht2ht.f90:1452-1594 for column jc = J + ic - 1.
static __device__ void run_sweep(const ChaseArgs& a, int ic, Sm& s) {
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
  if (!wait_prev(a, ic, min(1 + 2, last_prev), s.abort_flag)) return;
  // delayed left reflectors U(1..ic-1, 1) on B(J+1.., jc+r) and A(J+1.., jc) (:1466-1482)
  if (jc + r <= n) apply_delayed_left(S, 1, ic - 1, &B1(J + 1, jc + r), min(n - J, r + ic - 2), s);
  if (jc <= n) apply_delayed_left(S, 1, ic - 1, &A1(J + 1, jc), min(n - J, r + ic - 2), s);
  if (nb >= 2) {
    const double tu = larfg_col(nb, &A1(jc + 1, jc), s);  // :1487
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
    add_t_column(S, 1, ic, tu, min(n - J, r + nq), s);
    const double tv = left_and_opposite(nb, u, tu, &B1(jc + 1, jc + 1), ldb, s);  // :1495-1508
    double* v = S.V + S.ui(ic, ic, 1);
    for (int i = 2 + t; i <= nb; i += blockDim.x) v[i - 1] = s.q[i - 1];
    if (t == 0) {
      v[0] = 1.0;
      S.tauV[S.ti(ic, 1)] = tv;
    }
    __syncthreads();
    {
      // :1510, :1513, :1518, :1520 -- one reflector, four row ranges
      RightJob jobs[4] = {{&A1(jc + 1, jc + 1), lda, min(n, jc + r + nb) - jc},
                          {&B1(jc + 1, jc + 1), ldb, nb},
                          {&A1(istart, jc + 1), lda, jc - istart + 1},
                          {&B1(istart, jc + 1), ldb, jc - istart + 1}};
      larf_right4(jobs, 4, nb, v, tv);
    }
    for (int i = 2 + t; i <= nb; i += blockDim.x) B1(jc + i, jc + 1) = 0.0;
    __syncthreads();
  } else if (ic <= nq) {
    // no reflector in this column: keep TU's column ic consistent (tau = 0)
    add_t_column(S, 1, ic, 0.0, min(n - J, r + nq), s);
  }
  publish(a, ic, 1);
  if (nb < 2) return;  // :1484 skips the chase
  for (int jb = jc + 1; jb <= n; jb += r) {  // :1528
    const int ib = (jb - (jc + 1)) / r + 2;
    if (!wait_prev(a, ic, min(ib + 2, last_prev), s.abort_flag)) return;
    nb = min(r, n - jb - r + 1);
    istart = max(J + 1, J + 1 + (ib - 1) * r - (nq - ic) * r);
    const int jbb = J + (ib - 1) * r;  // block frame: reflector i of block ib starts at row jbb+i
    if (jb + r + r - 1 <= n)           // :1539-1544
      apply_delayed_left(S, ib, ic - 1, &B1(jbb + 1, jb + r + r - 1), min(n - jbb, r + ic - 2), s);
    if (jb + r - ic + 1 <= n)  // :1550-1553
      apply_delayed_left(S, ib, ic - 1, &A1(jbb + 1, jb), min(n - jbb, r + ic - 2), s);
    if (nb >= 2) {
      const double tu = larfg_col(nb, &A1(jb + r, jb), s);  // :1558
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
      add_t_column(S, ib, ic, tu, min(n - jbb, r + nq), s);
      const double tv = left_and_opposite(nb, u, tu, &B1(jb + r, jb + r), ldb, s);  // :1566-1579
      double* v = S.V + S.ui(ic, ic, ib);
      for (int i = 2 + t; i <= nb; i += blockDim.x) v[i - 1] = s.q[i - 1];
      if (t == 0) {
        v[0] = 1.0;
        S.tauV[S.ti(ic, ib)] = tv;
      }
      __syncthreads();
      {
        // :1581, :1584, :1589, :1591
        RightJob jobs[4] = {{&A1(jb + r, jb + r), lda, min(n, jb + 2 * r + nb - 1) - jb - r + 1},
                            {&B1(jb + r, jb + r), ldb, nb},
                            {&A1(istart, jb + r), lda, jb + r - istart},
                            {&B1(istart, jb + r), ldb, jb + r - istart}};
        larf_right4(jobs, 4, nb, v, tv);
      }
      for (int i = 1 + t; i <= nb - 1; i += blockDim.x) B1(jb + r + i, jb + r) = 0.0;
      __syncthreads();
    } else if (jbb < n) {
      add_t_column(S, ib, ic, 0.0, min(n - jbb, r + nq), s);
    }
    publish(a, ic, ib);
  }
#undef A1
#undef B1
}

// Carves the chase's shared memory (chase_smem_bytes) for an r x r block and nq sweeps.
PHT_DEV Sm chase_sm(double* sm, int r, int nq, int* abort_flag) {
  Sm s;
  s.Bc = sm;
  s.y = s.Bc + (size_t)r * (r + 1);
  s.z = s.y + nq;
  s.d = s.z + nq;
  s.q = s.d + r;
  s.tau = s.q + r;
  s.sc = s.tau + r;
  s.red = s.sc + 8;
  s.abort_flag = abort_flag;
  s.ldr = r + 1;
  return s;
}
inline size_t chase_smem_bytes(int r, int nq) {
  return sizeof(double) * ((size_t)r * (r + 1) + 2 * (size_t)nq + 3 * (size_t)r + 8 + 32);
}

}  // namespace pht
