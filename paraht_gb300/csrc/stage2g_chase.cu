// stage2g_chase.cu -- bulge chase of one Givens stage-2 sweep group (src/rht2ht.f90:776-960),
// one CTA per sweep, pipelined like the Householder chase: sweep ic starts step ib once sweep
// ic-1 has finished step ib+2.  A Givens step touches exactly the entries the Householder step
// of the same (ic, ib) touches (columns [jb, jb+2r-1] and the rows above, src/rht2ht.f90:879-957
// has the index structure of :1528-1594), so the same two-step lag reproduces the reference's
// order on every matrix entry; the sequential mode (one CTA, sweeps in order) is the
// reference's schedule.
//
// Step ib of sweep ic (1-based; base = J + (ib-1) r is the block frame, p0 = base + ic the first
// row of the reduced segment, cA the column reduced):
//  1. the left rotations of sweeps 1..ic-1 at block ib, applied to the entering column of B
//     (p0 + r - 1) and to column cA of A (:806-828, :892-914).  The reference applies them one
//     by one; here every sweep multiplies its rotations into U(ib) as it passes the block
//     (:970-984 done on the fly), so the delayed application is c <- U(ib)^T c, one
//     (r+nq)-long matrix-vector product (same product, other rounding);
//  2. nb-1 rotations from the bottom reduce A(p0:p0+nb-1, cA) to (r, 0, ..., 0) (:833-838).
//     Rotation k combines element k with the result r_{k+1} of the rotations below it, so
//     |r_k| is the norm of elements k..nb-1: one warp forms all of them from a suffix sum of
//     squares (DLARTG's signs: c >= 0, r_k has the sign of element k) instead of a chain of
//     nb-1 dependent DLARTG calls;
//  3. the left rotations applied to the nb x nb block of B (:840-843), one column per lane;
//  4. nb-1 rotations from the right remove the subdiagonal they leave in B, bottom to top
//     (:846-854): a dependent chain (each rotation changes the next diagonal entry), one warp,
//     one row per lane, the block in shared memory;
//  5. the right rotations applied to the A window and to the rows above of A and B
//     (:856-870, :942-956), one row per thread;
//  6. the step's rotations multiplied into U(ib) and V(ib) (:970-1003) and the right ones stored
//     as (c, s) for the staircase updates.
// Within a step, warp 0 forms the rotations (2-4) and publishes each one through a flag in shared
// memory as it is formed; the other warps apply them meanwhile (5-6), waiting (bounded) for each
// rotation in the order the chain forms them.  Synchronisation between sweeps (progress words,
// ticket, bounded waits) is that of the Householder chase.
// Compiled with -Xptxas -dlcm=cg so that global loads bypass L1 and observe the other CTAs'
// writes after the acquire.
#include "../../include/paraht.h"
#include "launch_count.h"
#include "stage2_chase.cuh"
#include "stage2g_common.cuh"

namespace pht {

constexpr int kGChaseThreads = 256;
// R: the largest band the instantiation takes (16 or 32; a block column fits one warp, and a row
// of a block is held in R registers)

struct GChaseArgs {
  double* A;
  int lda;
  double* B;
  int ldb;
  int n, J, r, nq;
  S2GStore S;
  ChaseSync sync;
  long long spin_limit;
  int pipelined;
};

// Shared memory of one sweep CTA (r <= 32, r + nq <= 64).
struct GSm {
  double* Bc;   // r x (r+1): the B block, row-major (row i at Bc + i*ldr)
  double* cu;   // r: left rotations of the current step (index ig = 1..nb-1)
  double* su;   // r
  double* cv;   // r: right rotations
  double* sv;   // r
  double* vec;  // 2 ldu: columns of the delayed left application
  int* abort_flag;
  int* rflag;   // rflag[ig] = the step's tick once right rotation ig is in cv, sv; rflag[0]: cu, su
  int ldr;
};

// Waits until flag == tick (a value warp 0 stores after publishing the data it guards), at most
// spin_limit polls; on timeout the chase's status word reports PARAHT_ERR_TIMEOUT and the wait
// returns false.  Every lane of the calling warp waits for the same flag.
static __device__ bool g_wait_flag(const int* flag, int tick, const GChaseArgs& a) {
  long long it = 0;
  while (*(volatile const int*)flag != tick) {
    if (++it > a.spin_limit) {
      atomicCAS(a.sync.status, 0, PARAHT_ERR_TIMEOUT);
      return false;
    }
  }
  __threadfence_block();
  return true;
}

constexpr int kGFlags = 33;  // rflag entries (r <= 32, plus the left rotations')
inline size_t g_chase_smem_bytes(int r, int nq) {
  return sizeof(double) * ((size_t)r * (r + 1) + 4 * (size_t)r + 2 * (size_t)(r + nq)) + sizeof(int) * kGFlags;
}

static __device__ bool g_wait(const GChaseArgs& a, int ic, int need, int* abort_flag) {
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

static __device__ void g_publish(const GChaseArgs& a, int ic, int step) {
  if (!a.pipelined) return;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release(&a.sync.prog[ic], step);
}

// col1, col2 (either may be null) point at row base+1 of a column; rows base+1 .. base+m:
// c <- U(ib)^T c.  All threads take part.
static __device__ void g_delayed_left(const S2GStore& S, int ib, int m, double* col1, double* col2, GSm& s) {
  const int t = threadIdx.x, nt = blockDim.x, ldu = S.ldu;
  for (int e = t; e < 2 * ldu; e += nt) {
    const int w = e / ldu, i = e % ldu;
    const double* col = w ? col2 : col1;
    s.vec[e] = (col && i < m) ? col[i] : 0.0;
  }
  __syncthreads();
  const double* U = S.U + S.gi(1, 1, ib);
  for (int b0 = 0; b0 < 2 * ldu; b0 += nt / 4) {  // uniform trip count: every lane takes part in gsum
    const int o = b0 + t / 4, part = t % 4;
    const int w = o / ldu, i = o % ldu;
    double* col = (o < 2 * ldu) ? (w ? col2 : col1) : nullptr;
    const bool live = col && i < m;
    double acc = 0.0;
    if (live)
      for (int j = part; j < m; j += 4) acc = fma(U[j + (size_t)i * ldu], s.vec[w * ldu + j], acc);
    acc = gsum<4>(acc);
    if (live && part == 0) col[i] = acc;
  }
  __syncthreads();
}

// G <- G * (the step's rotations ig = nb-1 .. 1) for the ldu rows of G, one lane per row: the
// left rotations as drot(U(:, ic-1+ig), U(:, ic+ig)) (:975-980), the right ones as
// drot(V(:, ic+ig), V(:, ic+ig-1)) (:990-995).  The step touches columns ic-1 .. ic+nb-2
// (0-based), held in registers (w[j] = column ic-1+j).
template <int R, bool kLeft>
static __device__ __noinline__ void g_accumulate(double* G, int ldu, int ic, int nb, const double* cs,
                                                 const double* sns, int lane, const int* rflag = nullptr,
                                                 int tick = 0, const GChaseArgs* a = nullptr) {
  for (int row = lane; row < ldu; row += 32) {
    double* Gr = G + row + (size_t)(ic - 1) * ldu;
    double w[R];
#pragma unroll
    for (int j = 0; j < R; ++j) w[j] = j < nb ? Gr[(size_t)j * ldu] : 0.0;
    double carry = w[R - 1];
    int ready = R;  // rotations ig >= ready are known to be published
#pragma unroll
    for (int ig = R - 1; ig >= 1; --ig) {
      if (ig > nb - 1) {
        carry = w[ig - 1];
        continue;
      }
      if (rflag && ig < ready) {  // the rotation chain publishes ig = nb-1 .. 1 in this order
        g_wait_flag(rflag + ig, tick, *a);
        ready = ig;
      }
      const double c = cs[ig], sn = sns[ig];
      const double v = w[ig - 1];
      if (kLeft) {  // x = column ic-2+ig, y = ic-1+ig
        w[ig] = fma(c, carry, -sn * v);
        carry = fma(c, v, sn * carry);
      } else {  // x = column ic-1+ig, y = ic-2+ig
        w[ig] = fma(c, carry, sn * v);
        carry = fma(c, v, -sn * carry);
      }
    }
    w[0] = carry;
#pragma unroll
    for (int j = 0; j < R; ++j)
      if (j < nb) Gr[(size_t)j * ldu] = w[j];
  }
}

// Right rotations of the step (cv, sv) on `rows` rows of X starting at `row0` (one row per thread
// t0 + k * stride), columns p0 .. p0+nb-1 held in R registers per row.
template <int R>
static __device__ __noinline__ void g_rows_right(double* X, int ld, int row0, int rows, int p0, int nb, const double* cv,
                                                 const double* sv, int t0, int stride, const int* rflag, int tick,
                                                 const GChaseArgs& a, int& ready) {
  // ready: rotations ig >= ready are known to be published (ig = nb-1 .. 1 in this order)
  for (int e = t0; e < rows; e += stride) {
    double* row = X + (size_t)(row0 + e - 1) + (size_t)(p0 - 1) * ld;
    double v[R];
#pragma unroll
    for (int j = 0; j < R; ++j) v[j] = j < nb ? row[(size_t)j * ld] : 0.0;
    double carry = v[R - 1];
#pragma unroll
    for (int ig = R - 1; ig >= 1; --ig) {
      if (ig > nb - 1) {
        carry = v[ig - 1];
        continue;
      }
      if (ig < ready) {
        g_wait_flag(rflag + ig, tick, a);
        ready = ig;
      }
      const double c = cv[ig], sn = sv[ig];
      const double yv = v[ig - 1];
      v[ig] = fma(c, carry, sn * yv);
      carry = fma(c, yv, -sn * carry);
    }
    v[0] = carry;
#pragma unroll
    for (int j = 0; j < R; ++j)
      if (j < nb) row[(size_t)j * ld] = v[j];
  }
}

// One sweep: src/rht2ht.f90:788-957 for column jc = J + ic - 1.
template <int R>
static __device__ void g_run_sweep(const GChaseArgs& a, int ic, GSm& s) {
  double* A = a.A;
  double* B = a.B;
  const int lda = a.lda, ldb = a.ldb, n = a.n, J = a.J, r = a.r, nq = a.nq;
  const S2GStore& S = a.S;
  const int ldu = S.ldu, ldr = s.ldr;
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31;
#define A1(i, j) A[(size_t)((i)-1) + (size_t)((j)-1) * lda]
#define B1(i, j) B[(size_t)((i)-1) + (size_t)((j)-1) * ldb]
  const int last_prev = (ic > 1) ? last_step(n, J, r, ic - 1) : 0;
  const int jc = J + ic - 1;
  for (int ib = 1;; ++ib) {
    int p0, cA, nb, istart;
    if (ib == 1) {
      p0 = jc + 1;
      cA = jc;
      nb = min(r, n - jc);
      istart = J + 1;
    } else {
      const int jb = jc + 1 + (ib - 2) * r;  // :879
      if (jb > n) break;
      p0 = jb + r;
      cA = jb;
      nb = min(r, n - jb - r + 1);
      istart = max(J + 1, J + 1 + (ib - 1) * r - (nq - ic) * r);
    }
    const int base = J + (ib - 1) * r;
    if (!g_wait(a, ic, min(ib + 2, last_prev), s.abort_flag)) return;
    // 1. delayed left rotations of sweeps 1..ic-1 (:806-828 / :892-914)
    if (ic > 1) {
      const int m = min(ldu, n - base);
      const int colB = p0 + r - 1;
      g_delayed_left(S, ib, m, colB <= n ? &B1(base + 1, colB) : nullptr, cA <= n ? &A1(base + 1, cA) : nullptr, s);
    }
    if (nb < 2) {  // :831 / :917 -- nothing to reduce at this step
      g_publish(a, ic, ib);
      if (ib == 1) return;  // the column step skips the whole chase (:831 cycles the ic loop)
      continue;
    }
    for (int e = t; e < nb * nb; e += nt) {  // the B block, row-major in shared memory
      const int i = e / nb, j = e % nb;
      s.Bc[i * ldr + j] = B1(p0 + i, p0 + j);
    }
    __syncthreads();
    // tick: unique per (sweep, step) within the CTA (the sequential mode runs every sweep in one CTA)
    const int tick = (ic << 16) + ib;
    // Warp 0 runs the step's serial part (2-4) and publishes each rotation as it forms it: the
    // left ones after 2 (rflag[0]), right rotation ig after forming it (rflag[ig]).  Warps 1..
    // consume them meanwhile, in the order they are formed: warp 1 multiplies the left ones into
    // U(ib), warp 2 the right ones into V(ib), warps 3.. apply the right ones to the rows (5-6).
    if (t < 32) {
      // 2. rotations reducing the column; lane L holds element L (row p0+L)
      const double x = lane < nb ? A1(p0 + lane, cA) : 0.0;
      double ss = x * x;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const double y = __shfl_down_sync(0xffffffffu, ss, off);
        if (lane + off < 32) ss += y;
      }
      const double Dn = __shfl_down_sync(0xffffffffu, ss, 1);  // squared norm below this element
      const double ri = ss > 0.0 ? rsqrt(ss) : 0.0;
      const double rk = (lane + 1 >= nb || Dn == 0.0) ? x : (x != 0.0 ? copysign(ss * ri, x) : ss * ri);
      const double rn = __shfl_down_sync(0xffffffffu, rk, 1);
      if (lane < nb - 1) {
        double c, sn;
        if (Dn == 0.0) {
          c = 1.0;
          sn = 0.0;
        } else if (x == 0.0) {
          c = 0.0;
          sn = copysign(1.0, rn);
        } else {
          c = fabs(x) * ri;
          sn = rn * copysign(ri, x);
        }
        s.cu[lane + 1] = c;
        s.su[lane + 1] = sn;
      }
      if (lane < nb) A1(p0 + lane, cA) = lane == 0 ? rk : 0.0;
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        *(volatile int*)&s.rflag[0] = tick;
      }
      // 3. left rotations on the B block, one column per lane (:840-843)
      if (lane < nb) {
        double carry = s.Bc[(nb - 1) * ldr + lane];
        for (int ig = nb - 1; ig >= 1; --ig) {
          const double c = s.cu[ig], sn = s.su[ig];
          const double xv = s.Bc[(ig - 1) * ldr + lane];
          s.Bc[ig * ldr + lane] = fma(c, carry, -sn * xv);
          carry = fma(c, xv, sn * carry);
        }
        s.Bc[lane] = carry;
      }
      __syncwarp();
      // 4. right rotations removing B's subdiagonal, bottom to top (:846-854); lane = row
      for (int ig = nb - 1; ig >= 1; --ig) {
        const double f = s.Bc[ig * ldr + ig], g = s.Bc[ig * ldr + ig - 1];
        double c, sn, rr;
        givens(f, g, c, sn, rr);
        __syncwarp();
        if (lane == ig) {
          s.Bc[ig * ldr + ig] = rr;
          s.Bc[ig * ldr + ig - 1] = 0.0;
        } else if (lane < ig) {
          const double xv = s.Bc[lane * ldr + ig], yv = s.Bc[lane * ldr + ig - 1];
          s.Bc[lane * ldr + ig] = fma(c, xv, sn * yv);
          s.Bc[lane * ldr + ig - 1] = fma(c, yv, -sn * xv);
        }
        if (lane == 0) {
          s.cv[ig] = c;
          s.sv[ig] = sn;
          __threadfence_block();
          *(volatile int*)&s.rflag[ig] = tick;
        }
        __syncwarp();
      }
      for (int e = lane; e < nb * nb; e += 32) {
        const int i = e / nb, j = e % nb;
        B1(p0 + i, p0 + j) = s.Bc[i * ldr + j];
      }
    } else if (t < 64) {
      // 6. the left rotations into U(ib) (:970-984)
      if (g_wait_flag(s.rflag, tick, a)) g_accumulate<R, true>(S.U + S.gi(1, 1, ib), ldu, ic, nb, s.cu, s.su, lane);
    } else if (t < 96) {
      // 6. the right rotations into V(ib) (:990-1003), then kept as (c, s) for the staircase updates
      g_accumulate<R, false>(S.V + S.gi(1, 1, ib), ldu, ic, nb, s.cv, s.sv, lane, s.rflag, tick, &a);
      for (int ig = lane + 1; ig <= nb - 1; ig += 32) {
        S.CV[S.ri(ic + ig - 1, ic, ib)] = s.cv[ig];
        S.SV[S.ri(ic + ig - 1, ic, ib)] = s.sv[ig];
      }
    } else {
      // 5. right rotations on the A window and the rows above of A and B, one row per thread
      const int nA = min(n, p0 + r + nb - 1) - p0 + 1, nAbove = p0 - istart;
      const int total = nA + 2 * nAbove, nc = nt - 96;
      int ready = R;
      // one flat index over the three row ranges, so that every thread has a row
      for (int e = t - 96; e < total; e += nc) {
        if (e < nA)
          g_rows_right<R>(A, lda, p0 + e, 1, p0, nb, s.cv, s.sv, 0, 1, s.rflag, tick, a, ready);
        else if (e < nA + nAbove)
          g_rows_right<R>(A, lda, istart + e - nA, 1, p0, nb, s.cv, s.sv, 0, 1, s.rflag, tick, a, ready);
        else
          g_rows_right<R>(B, ldb, istart + e - nA - nAbove, 1, p0, nb, s.cv, s.sv, 0, 1, s.rflag, tick, a, ready);
      }
    }
    __syncthreads();
    g_publish(a, ic, ib);
  }
#undef A1
#undef B1
}

template <int R>
__global__ void __launch_bounds__(kGChaseThreads, 1) k_s2g_chase(GChaseArgs a) {
  extern __shared__ double gsm[];
  __shared__ int s_ic, s_abort;
  GSm s;
  s.ldr = a.r + 1;
  s.Bc = gsm;
  s.cu = s.Bc + (size_t)a.r * s.ldr;
  s.su = s.cu + a.r;
  s.cv = s.su + a.r;
  s.sv = s.cv + a.r;
  s.vec = s.sv + a.r;
  s.rflag = reinterpret_cast<int*>(s.vec + 2 * (a.r + a.nq));
  s.abort_flag = &s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  for (int i = threadIdx.x; i < kGFlags; i += blockDim.x) s.rflag[i] = 0;
  if (!a.pipelined) {
    __syncthreads();
    for (int ic = 1; ic <= a.nq; ++ic) g_run_sweep<R>(a, ic, s);
    return;
  }
  if (threadIdx.x == 0) s_ic = atomicAdd(a.sync.ticket, 1) + 1;
  __syncthreads();
  g_run_sweep<R>(a, s_ic, s);
}

void s2g_launch_chase(cudaStream_t st, double* A, int lda, double* B, int ldb, int n, int J, int r, int nq,
                      const S2GStore& S, const ChaseSync& sync, int sequential, long long spin_limit) {
  GChaseArgs a;
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
  if (a.pipelined) {
    cudaMemsetAsync(sync.prog, 0, sizeof(int) * (nq + 1), st);
    cudaMemsetAsync(sync.ticket, 0, sizeof(int), st);
  }
  count_launch();
  if (r <= 16)
    k_s2g_chase<16><<<a.pipelined ? nq : 1, kGChaseThreads, g_chase_smem_bytes(r, nq), st>>>(a);
  else
    k_s2g_chase<32><<<a.pipelined ? nq : 1, kGChaseThreads, g_chase_smem_bytes(r, nq), st>>>(a);
}

}  // namespace pht
