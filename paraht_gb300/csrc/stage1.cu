// stage1.cu -- stage 1 of the HT reduction on the GPU: (A general, B upper triangular) ->
// (A r-Hessenberg, B upper triangular), accumulating Q <- Q*Q1 and Z <- Z*Z1.
//
// Follows src/ab2rht.f90:8-495 (ab2rht_simple).  Per panel jb (ab2rht.f90:71):
//   1. left generation: QR of the overlapping p*nb x nb blocks of the panel, bottom to top
//      (ab2rht.f90:85-123): reflectors VL, triangular factors TL, R into A (k_s1_lgen,
//      stage1_gen.cu; the general k_s1_left_gen below when the panel exceeds shared memory).
//   2. left ops on B, A and right ops on Q with (VL, TL) (ab2rht.f90:135-250), all blocks in
//      bottom-to-top order, as ordered compact-WY op lists (FP64: wy_apply.cuh; split
//      precision: wy_stream.cuh).
//   3. per block, bottom to top: the right generation computes the RQ of the diagonal L x L
//      block of B, the first nb rows of its orthogonal factor and their LQ (the "RQ->LQ trick",
//      ab2rht.f90:282-312) giving nb right reflectors (VR, TR) (k_s1_rgen; k_s1_right_gen below
//      for L > 128); they are applied to the B rows the next block needs on the critical stream
//      and to the remaining B rows on a side stream (ab2rht.f90:317-367), and the first nb
//      columns of the block are zeroed below the diagonal (ab2rht.f90:329-333).
//   4. right ops on A and Z with (VR, TR), all blocks in order (ab2rht.f90:387-467).
// Generation is FP64; the updates are FP64 or split precision (PARAHT_FLAG_SPLIT).
#include <algorithm>

#include "paraht_internal.cuh"
#include "paraht_impl.h"
#include "stage1_gen.cuh"
#include "split_apply.cuh"
#include "wy_apply.cuh"

namespace pht {

// ------------------------------------------------------------------------------------------
// Triangular factor of a block reflector from the Gram matrix of its vectors:
//   forward  (dlarft 'F'): T upper, T[l][m] = -tau_m * sum_{q=l}^{m-1} T[l][q] G[q][m]
//   backward (dlarft 'B'): T lower, T[m][i] = -tau_i * sum_{l=i+1}^{m} T[m][l] G[l][i]
// G (k x k, ld kg, only the needed triangle) and tau live in shared memory; T is written to
// global memory (ld ldt) with explicit zeros in the unused triangle.  Columns are generated
// one after the other (the recurrence is sequential in m); rows within a column in parallel.
// ------------------------------------------------------------------------------------------
__device__ void form_t_forward(int k, const double* G, int kg, const double* tau, double* Ts, int nbT, double* T,
                               int ldt) {
  // Ts: shared scratch nbT x nbT (ld nbT)
  const int t = threadIdx.x;
  for (int e = t; e < nbT * nbT; e += blockDim.x) Ts[e] = 0.0;
  __syncthreads();
  for (int m = 0; m < k; ++m) {
    if (t < m) {
      double s = 0.0;
      for (int q = t; q < m; ++q) s = fma(Ts[t + q * nbT], G[q + m * kg], s);
      Ts[t + m * nbT] = -tau[m] * s;
    }
    if (t == m) Ts[m + m * nbT] = tau[m];
    __syncthreads();
  }
  for (int e = t; e < nbT * nbT; e += blockDim.x) T[(e % nbT) + (size_t)(e / nbT) * ldt] = Ts[e];
}

__device__ void form_t_backward(int k, const double* G, int kg, const double* tau, double* Ts, int nbT, double* T,
                                int ldt) {
  const int t = threadIdx.x;
  for (int e = t; e < nbT * nbT; e += blockDim.x) Ts[e] = 0.0;
  __syncthreads();
  for (int i = k - 1; i >= 0; --i) {
    if (t == i) Ts[i + i * nbT] = tau[i];
    if (t > i && t < k) {
      double s = 0.0;
      for (int l = i + 1; l <= t; ++l) s = fma(Ts[t + l * nbT], G[l + i * kg], s);
      Ts[t + i * nbT] = -tau[i] * s;
    }
    __syncthreads();
  }
  for (int e = t; e < nbT * nbT; e += blockDim.x) T[(e % nbT) + (size_t)(e / nbT) * ldt] = Ts[e];
}

// ------------------------------------------------------------------------------------------
// Left generation (ab2rht.f90:85-123): for each block bottom to top, Householder QR
// (dgeqr2 semantics) of A(ib:ib2, jb:jb+nb-1); store VL explicitly (unit diagonal, zeros
// above), write R (zeros below) back to A, form TL (dlarft 'F','C').
// Shared memory: G (nb x nb) + Ts (nb x nb) + tau (nb) + reduction, then the P tile (L x nb,
// ld L+1) when it fits; otherwise the tile lives in the global scratch `gscratch` (L2-resident,
// same code path), which lets L = p nb reach 1024 (r = 64, p = 16).
// ------------------------------------------------------------------------------------------
constexpr int kGenThreads = 256;

__global__ void __launch_bounds__(kGenThreads) k_s1_left_gen(double* __restrict__ A, int lda, S1Panel P,
                                                             double* __restrict__ VL, double* __restrict__ TL,
                                                             double* __restrict__ gscratch) {
  extern __shared__ double sm[];
  const int L = P.L, nb = P.nb, ldp = L + 1;
  double* G = sm;                     // nb*nb
  double* Ts = G + nb * nb;           // nb*nb
  double* tau = Ts + nb * nb;         // nb
  double* red = tau + nb;             // 32
  double* Pt = gscratch ? gscratch : red + 32;  // ldp * nb
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarp = blockDim.x >> 5;
  const int jb0 = P.jb0;
  for (int o = 0; o < P.nblocks; ++o) {
    const int ib0 = P.ib(o), nb2 = P.nb2(o), k = min(nb, nb2);
    for (int e = t; e < nb2 * nb; e += blockDim.x) {
      const int i = e % nb2, j = e / nb2;
      Pt[i + j * ldp] = A[(size_t)(ib0 + i) + (size_t)(jb0 + j) * lda];
    }
    __syncthreads();
    for (int j = 0; j < k; ++j) {
      double part = 0.0;
      for (int i = j + 1 + t; i < nb2; i += blockDim.x) part = fma(Pt[i + j * ldp], Pt[i + j * ldp], part);
      const double ss = block_sum(part, red);
      const Reflector h = make_reflector(Pt[j + j * ldp], ss);
      __syncthreads();  // everyone has read alpha
      for (int i = j + 1 + t; i < nb2; i += blockDim.x) Pt[i + j * ldp] *= h.scal;
      __syncthreads();
      if (h.tau != 0.0) {
        for (int c = j + 1 + warp; c < nb; c += nwarp) {
          double s = (lane == 0) ? Pt[j + c * ldp] : 0.0;
          for (int i = j + 1 + lane; i < nb2; i += 32) s = fma(Pt[i + j * ldp], Pt[i + c * ldp], s);
          const double tw = h.tau * warp_sum(s);
          if (lane == 0) Pt[j + c * ldp] -= tw;
          for (int i = j + 1 + lane; i < nb2; i += 32) Pt[i + c * ldp] = fma(-tw, Pt[i + j * ldp], Pt[i + c * ldp]);
        }
      }
      __syncthreads();
      if (t == 0) {
        Pt[j + j * ldp] = h.beta;
        tau[j] = h.tau;
      }
      __syncthreads();
    }
    for (int j = k + t; j < nb; j += blockDim.x) tau[j] = 0.0;
    // VL (explicit), and R / zeros back into A.
    double* V = VL + (size_t)o * L * nb;
    for (int e = t; e < L * nb; e += blockDim.x) {
      const int i = e % L, j = e / L;
      double v = 0.0;
      if (j < k && i < nb2) v = (i > j) ? Pt[i + j * ldp] : (i == j ? 1.0 : 0.0);
      V[i + (size_t)j * L] = v;
    }
    for (int e = t; e < nb2 * nb; e += blockDim.x) {
      const int i = e % nb2, j = e / nb2;
      A[(size_t)(ib0 + i) + (size_t)(jb0 + j) * lda] = (i <= j) ? Pt[i + j * ldp] : 0.0;
    }
    // Gram matrix G[q][m] = v_q . v_m  (q < m < k), v explicit: unit at row q.
    for (int e = t; e < nb * nb; e += blockDim.x) {
      const int q = e % nb, m = e / nb;
      double s = 0.0;
      if (q < m && m < k) {
        s = Pt[m + q * ldp];  // v_q[m] * v_m[m] (= 1)
        for (int i = m + 1; i < nb2; ++i) s = fma(Pt[i + q * ldp], Pt[i + m * ldp], s);
      }
      G[q + m * nb] = s;
    }
    __syncthreads();
    form_t_forward(k, G, nb, tau, Ts, nb, TL + (size_t)o * nb * nb, nb);
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// Right generation for one block (ab2rht.f90:282-312).  S <- B(ib:ib2, ib:ib2) (nb2 x nb2);
// RQ (dgerq2 semantics, rows bottom to top, reflector for row i stored in S(i, 0:i-1) with an
// implicit unit at column i).  If nb2 > nb: M <- first nb rows of the orthogonal factor
// H(1)...H(nb2) (dorgrq), then LQ of M (dgelq2) -> nb forward row-wise reflectors, T forward
// (dlarft 'F','R').  Else: the nb2 RQ reflectors themselves, T backward (dlarft 'B','R').
// VRc (block o) receives the reflectors transposed (column-wise, L x nb), TR the T factor.
// Shared memory: S (nb2 x nb2, ld L+1), M (nb x L), partial sums, G, Ts, tau.
// ------------------------------------------------------------------------------------------
constexpr int kRgenThreads = 512;

__global__ void __launch_bounds__(kRgenThreads) k_s1_right_gen(const double* __restrict__ B, int ldb, S1Panel P, int o,
                                                               double* __restrict__ VRc, double* __restrict__ TR,
                                                               double* __restrict__ gscratch) {
  extern __shared__ double sm[];
  const int L = P.L, nb = P.nb, lds = L + 1;
  const int ib0 = P.ib(o), nb2 = P.nb2(o);
  const int t = threadIdx.x, nt = blockDim.x;
  // S in shared memory when it fits, else in global scratch (same code path).
  double* tauR = sm;                      // L
  double* tauL = tauR + L;                // nb
  double* G = tauL + nb;                  // nb*nb
  double* Ts = G + nb * nb;               // nb*nb
  double* red = Ts + nb * nb;             // 32
  double* part = red + 32;                // kRgenThreads partial sums
  double* S = part + kRgenThreads;        // (L+1)*L when it fits in shared memory
  double* M = S + (size_t)lds * L;        // nb * (L+1)
  if (gscratch) {
    S = gscratch;
    M = gscratch + (size_t)lds * L;
  }
  const int ldm = nb;  // M is nb x nb2, column-major with ld nb: M[r + c*nb]
  for (int e = t; e < nb2 * nb2; e += nt) {
    const int i = e % nb2, j = e / nb2;
    S[i + j * lds] = B[(size_t)(ib0 + i) + (size_t)(ib0 + j) * ldb];
  }
  __syncthreads();
  // ---- RQ, rows bottom to top ----
  const int nq4 = 4;
  for (int i = nb2 - 1; i >= 0; --i) {
    double ps = 0.0;
    for (int c = t; c < i; c += nt) ps = fma(S[i + c * lds], S[i + c * lds], ps);
    const double ss = block_sum(ps, red);
    const Reflector h = make_reflector(S[i + i * lds], ss);
    __syncthreads();
    for (int c = t; c < i; c += nt) S[i + c * lds] *= h.scal;
    __syncthreads();
    if (h.tau != 0.0 && i > 0) {
      // rows rho < i: w = S[rho][i] + sum_{c<i} S[rho][c] v_c
      const int rows_per_pass = nt / nq4;
      for (int rho0 = 0; rho0 < i; rho0 += rows_per_pass) {
        const int lr = t % rows_per_pass, rho = rho0 + lr, qq = t / rows_per_pass;
        const int cpart = (i + nq4 - 1) / nq4;
        const int c0 = qq * cpart, c1 = min(i, c0 + cpart);
        double s = 0.0;
        if (rho < i)
          for (int c = c0; c < c1; ++c) s = fma(S[rho + c * lds], S[i + c * lds], s);
        part[qq * rows_per_pass + lr] = s;
        __syncthreads();
        if (rho < i) {
          const double w = S[rho + i * lds] + ((part[lr] + part[rows_per_pass + lr]) +
                                               (part[2 * rows_per_pass + lr] + part[3 * rows_per_pass + lr]));
          const double tw = h.tau * w;
          for (int c = c0; c < c1; ++c) S[rho + c * lds] = fma(-tw, S[i + c * lds], S[rho + c * lds]);
          if (qq == 0) S[rho + i * lds] -= tw;
        }
        __syncthreads();
      }
    }
    if (t == 0) {
      S[i + i * lds] = h.beta;
      tauR[i] = h.tau;
    }
    __syncthreads();
  }
  double* V = VRc + (size_t)o * L * nb;
  double* Tout = TR + (size_t)o * nb * nb;
  if (nb2 > nb) {
    // ---- M = [I 0] H(1) H(2) ... H(nb2)  (first nb rows of the RQ orthogonal factor) ----
    for (int e = t; e < nb * nb2; e += nt) {
      const int r = e % nb, c = e / nb;
      M[r + c * ldm] = (r == c) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int i = 0; i < nb2; ++i) {
      const double ti = tauR[i];
      if (ti != 0.0) {
        // row r of M: w = sum_{c<=i} M[r][c] v_c ; v_i = 1
        const int ng = nt / nb;  // groups per row
        const int r = t % nb, g = t / nb;
        const int cpart = (i + 1 + ng - 1) / ng;
        const int c0 = g * cpart, c1 = min(i + 1, c0 + cpart);
        double s = 0.0;
        for (int c = c0; c < c1; ++c) s = fma(M[r + c * ldm], (c == i) ? 1.0 : S[i + c * lds], s);
        if (g < ng) part[g * nb + r] = s;
        __syncthreads();
        double w = 0.0;
        for (int gg = 0; gg < ng; ++gg) w += part[gg * nb + r];
        const double tw = ti * w;
        for (int c = c0; c < c1; ++c) M[r + c * ldm] = fma(-tw, (c == i) ? 1.0 : S[i + c * lds], M[r + c * ldm]);
      }
      __syncthreads();
    }
    // ---- LQ of M (dgelq2): row i, columns i..nb2-1 ----
    for (int i = 0; i < nb; ++i) {
      double ps = 0.0;
      for (int c = i + 1 + t; c < nb2; c += nt) ps = fma(M[i + c * ldm], M[i + c * ldm], ps);
      const double ss = block_sum(ps, red);
      const Reflector h = make_reflector(M[i + i * ldm], ss);
      __syncthreads();
      for (int c = i + 1 + t; c < nb2; c += nt) M[i + c * ldm] *= h.scal;
      __syncthreads();
      if (h.tau != 0.0 && i + 1 < nb) {
        const int ng = nt / nb;
        const int r = t % nb, g = t / nb;
        const int len = nb2 - i;
        const int cpart = (len + ng - 1) / ng;
        const int c0 = i + g * cpart, c1 = min(nb2, c0 + cpart);
        double s = 0.0;
        if (r > i)
          for (int c = c0; c < c1; ++c) s = fma(M[r + c * ldm], (c == i) ? 1.0 : M[i + c * ldm], s);
        part[g * nb + r] = s;
        __syncthreads();
        if (r > i) {
          double w = 0.0;
          for (int gg = 0; gg < ng; ++gg) w += part[gg * nb + r];
          const double tw = h.tau * w;
          for (int c = c0; c < c1; ++c) M[r + c * ldm] = fma(-tw, (c == i) ? 1.0 : M[i + c * ldm], M[r + c * ldm]);
        }
      }
      __syncthreads();
      if (t == 0) {
        M[i + i * ldm] = h.beta;
        tauL[i] = h.tau;
      }
      __syncthreads();
    }
    // VRc[c][i] = VR[i][c]: unit at c == i, M[i][c] for c > i, zero before.
    for (int e = t; e < L * nb; e += nt) {
      const int c = e % L, i = e / L;
      double v = 0.0;
      if (c < nb2) v = (c < i) ? 0.0 : (c == i ? 1.0 : M[i + c * ldm]);
      V[c + (size_t)i * L] = v;
    }
    // G[q][m] = VR[q] . VR[m] for q < m
    for (int e = t; e < nb * nb; e += nt) {
      const int q = e % nb, m = e / nb;
      double s = 0.0;
      if (q < m) {
        s = M[q + m * ldm];
        for (int c = m + 1; c < nb2; ++c) s = fma(M[q + c * ldm], M[m + c * ldm], s);
      }
      G[q + m * nb] = s;
    }
    __syncthreads();
    form_t_forward(nb, G, nb, tauL, Ts, nb, Tout, nb);
  } else {
    // Backward row-wise reflectors straight from the RQ (ab2rht.f90:308-309).
    const int k = nb2;
    for (int e = t; e < L * nb; e += nt) {
      const int c = e % L, i = e / L;
      double v = 0.0;
      if (i < k && c < nb2) v = (c < i) ? S[i + c * lds] : (c == i ? 1.0 : 0.0);
      V[c + (size_t)i * L] = v;
    }
    // G[l][i] = v_l . v_i for l > i (support of v_i: columns 0..i)
    for (int e = t; e < nb * nb; e += nt) {
      const int l = e % nb, i = e / nb;
      double s = 0.0;
      if (l > i && l < k) {
        s = S[l + i * lds];  // v_l[i] * v_i[i](=1)
        for (int c = 0; c < i; ++c) s = fma(S[l + c * lds], S[i + c * lds], s);
      }
      G[l + i * nb] = s;
    }
    __syncthreads();
    form_t_backward(k, G, nb, tauR, Ts, nb, Tout, nb);
  }
}

// Zero B(j+1 : ib2, j) for the first nb columns of the block (ab2rht.f90:329-333).
__global__ void k_s1_zero_fill(double* B, int ldb, int ib0, int ib2, int nb) {
  const int j = ib0 + blockIdx.x;
  for (int i = j + 1 + threadIdx.x; i <= ib2; i += blockDim.x) B[(size_t)i + (size_t)j * ldb] = 0.0;
}

// ------------------------------------------------------------------------------------------
// Host driver
// ------------------------------------------------------------------------------------------

static int s1_nblk0(int n, int nb, int p) { return std::max(1, (n - nb + (p - 1) * nb - 1) / ((p - 1) * nb)); }

size_t s1_workspace_bytes(int n, int nb, int p) {
  const int L = p * nb;
  const size_t nblk0 = s1_nblk0(n, nb, p);
  size_t w = 0;
  w += 2 * ((size_t)L * nb * nblk0 * 2 + (size_t)nb * nb * nblk0 * 2);  // two sets of VL, VRc, TL, TR
  w += (size_t)(L + 1) * L + (size_t)nb * (L + 1);                      // global scratch (large-L fallback)
  return w * sizeof(double) + 4096;
}

static size_t left_gen_small(int nb) { return sizeof(double) * ((size_t)2 * nb * nb + nb + 32); }
static size_t left_gen_tile(int L, int nb) { return sizeof(double) * (size_t)(L + 1) * nb; }
static size_t right_gen_small(int L, int nb) {
  return sizeof(double) * ((size_t)L + nb + 2 * (size_t)nb * nb + 32 + kRgenThreads);
}
static size_t right_gen_big(int L, int nb) { return sizeof(double) * ((size_t)(L + 1) * L + (size_t)nb * (L + 1)); }

int s1_gen_grant();
void launch_s1_lgen(cudaStream_t s, double* A, int lda, const S1Panel& P, double* VL, double* TL);
void launch_s1_rgen(cudaStream_t s, const double* B, int ldb, const S1Panel& P, int o, double* VRc, double* TR);

// Stage-1 schedule.  Three streams, as the reference's task graph (ab2rht.f90:85-467) allows:
//   sA (critical): left generation, left update of B, then per block the right generation and
//       the update of the B rows the next block needs (the reference's "lookahead",
//       rows ib-(p-1)nb .. ib2, ab2rht.f90:317-338), then the right update of A;
//   sB: per block, the update of the remaining B rows 1 .. ib-(p-1)nb-1 (ab2rht.f90:343-367),
//       which the lookahead of the next block waits for (the B(3,3) token);
//   sC: left updates of A and Q and the right update of Z (priority-1 tasks).
// Reflector sets alternate between two buffers so that panel k+1 can be generated while sC
// still applies panel k.  With time_components everything runs on sA (the reference inserts
// taskwaits for the same purpose).
int s1_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int nb, int p,
           PhaseTimer* timer) {
  if (n - nb - 1 < 1) return 0;  // ab2rht.f90:71: empty panel loop
  const int L = p * nb;
  const bool serial = timer != nullptr && timer->serial;
  cudaStream_t sA = ctx.stream, sB = serial ? sA : ctx.side, sC = serial ? sA : ctx.side2;
  const size_t nblk0 = s1_nblk0(n, nb, p);
  double* ws = (double*)ctx.workspace(s1_workspace_bytes(n, nb, p));
  if (!ws) return PARAHT_ERR_ALLOC;
  double *VL[2], *VRc[2], *TL[2], *TR[2];
  double* d = ws;
  for (int k = 0; k < 2; ++k) {
    VL[k] = d;
    VRc[k] = VL[k] + (size_t)L * nb * nblk0;
    TL[k] = VRc[k] + (size_t)L * nb * nblk0;
    TR[k] = TL[k] + (size_t)nb * nb * nblk0;
    d = TR[k] + (size_t)nb * nb * nblk0;
  }
  double* gscr = d;

  // fast latency-oriented generation kernels (stage1_gen.cu) when the tiles fit; else the
  // general kernels above
  const bool fast_l = nb <= 64 && s1_lgen_smem(L, nb) <= (size_t)ctx.max_smem;
  const bool fast_r = L <= 128 && s1_rgen_smem_vr(L, nb, false) <= (size_t)ctx.max_smem;
  const bool l_in_smem = left_gen_small(nb) + left_gen_tile(L, nb) <= (size_t)ctx.max_smem;
  const size_t lsm = l_in_smem ? left_gen_small(nb) + left_gen_tile(L, nb) : left_gen_small(nb);
  const size_t rsm_small = right_gen_small(L, nb);
  const bool r_in_smem = rsm_small + right_gen_big(L, nb) <= (size_t)ctx.max_smem;
  const size_t rsm = r_in_smem ? rsm_small + right_gen_big(L, nb) : rsm_small;
  if ((!fast_l && lsm > (size_t)ctx.max_smem) || (!fast_r && rsm_small > (size_t)ctx.max_smem))
    return PARAHT_ERR_NOT_SUPPORTED;
  if (fast_l || fast_r)
    if (const int rc = s1_gen_grant()) return rc;
  if (!fast_l)
    if (const int rc = smem_at_least((const void*)k_s1_left_gen, lsm)) return rc;
  if (!fast_r)
    if (const int rc = smem_at_least((const void*)k_s1_right_gen, rsm)) return rc;

  // split-precision bulk updates (split_apply.cuh) where the op shapes fit; one operand region
  // per launch site: 0 B left, 1 A left, 2 Q, 3 remaining B rows, 4 A and Z right (one list), 5
  // unused
  const bool sp = ctx.split && split_fits(nb, L);
  void* reg[6] = {};
  if (sp)
    for (int i = 0; i < 6; ++i) {
      reg[i] = ctx.split_region(i, (int)nblk0, sizeof(SplitOpData));
      if (!reg[i]) return PARAHT_ERR_ALLOC;
    }
  cudaEvent_t evL = ctx.ev[0], evAL = ctx.ev[1], evLA = ctx.ev[2], evRest = ctx.ev[3], evChain = ctx.ev[4];
  cudaEvent_t evZ[2] = {ctx.ev[5], ctx.ev[6]}, evPrep = ctx.ev[7];
  if (!serial) {  // side streams start after everything already queued on sA
    cudaEventRecord(evL, sA);
    cudaStreamWaitEvent(sB, evL, 0);
    cudaStreamWaitEvent(sC, evL, 0);
    cudaEventRecord(evRest, sB);
    cudaEventRecord(evZ[0], sC);
    cudaEventRecord(evZ[1], sC);
  }
  int k = 0;
  for (int jb0 = 0; jb0 <= n - nb - 2; jb0 += nb, ++k) {  // ab2rht.f90:71 (1-based jb = 1 .. n-nb-1)
    const S1Panel P = make_panel(n, nb, p, jb0);
    const int s = k & 1;
    if (timer) timer->mark(sA, 0);
    if (!serial) cudaStreamWaitEvent(sA, evZ[s], 0);  // set s free again (Z update of panel k-2 done)
    if (fast_l) {
      launch_s1_lgen(sA, A, lda, P, VL[s], TL[s]);
    } else {
      count_launch();
      k_s1_left_gen<<<1, kGenThreads, lsm, sA>>>(A, lda, P, VL[s], TL[s], l_in_smem ? nullptr : gscr);
    }
    if (timer) timer->mark(sA, 2);
    if (!serial) {
      cudaEventRecord(evL, sA);
      cudaStreamWaitEvent(sC, evL, 0);
      cudaStreamWaitEvent(sA, evRest, 0);  // remaining-row B updates of panel k-1 done
    }
    apply_left_any(reg[0], B, ldb, P.ib(P.nblocks - 1), n - 1, GeoS1Left{P, VL[s], TL[s], 0}, P.nblocks, sA);
    apply_left_side(reg[1], A, lda, jb0 + nb, n - 1, GeoS1Left{P, VL[s], TL[s], 1}, P.nblocks, sC);
    if (!serial) cudaEventRecord(evAL, sC);
    apply_right_side(reg[2], Q, ldq, 0, n - 1, GeoS1Q{P, VL[s], TL[s]}, P.nblocks, sC);
    if (timer) timer->mark(sA, 1);
    if (!serial) {
      cudaEventRecord(evLA, sA);  // B left update done: the remaining-row updates may start
      cudaStreamWaitEvent(sB, evLA, 0);
    }
    for (int o = 0; o < P.nblocks; ++o) {
      if (fast_r) {
        launch_s1_rgen(sA, B, ldb, P, o, VRc[s], TR[s]);
      } else {
        count_launch();
        k_s1_right_gen<<<1, kRgenThreads, rsm, sA>>>(B, ldb, P, o, VRc[s], TR[s], r_in_smem ? nullptr : gscr);
      }
      // lookahead rows c1 .. ib2 (c1 = max(1, ib-(p-1)nb), 1-based) after the remaining rows of
      // the previous block (ab2rht.f90:321: depend(in: B(3,3)))
      const int c1 = std::max(0, P.ib(o) - P.stride);
      if (!serial) cudaStreamWaitEvent(sA, evRest, 0);
      GeoS1Right gl{P, VRc[s], TR[s], o};
      gl.row_lo = c1;
      gl.row_hi = P.ib2(o);
      // a small update on the critical chain: FP64, 8 rows per CTA
      launch_apply_right<GeoS1Right, 8>(B, ldb, c1, P.ib2(o), gl, sA);
      if (P.nb2(o) > nb) {
        count_launch();
        k_s1_zero_fill<<<nb, 128, 0, sA>>>(B, ldb, P.ib(o), P.ib2(o), nb);
      }
      if (c1 > 0) {
        if (!serial) {
          cudaEventRecord(evLA, sA);
          cudaStreamWaitEvent(sB, evLA, 0);
        }
        GeoS1Right gr{P, VRc[s], TR[s], o};
        gr.row_lo = 0;
        gr.row_hi = c1 - 1;
        apply_right_any(reg[3], B, ldb, 0, c1 - 1, gr, 1, sB);
        if (!serial) cudaEventRecord(evRest, sB);
      }
    }
    if (timer) timer->mark(sA, 2);
    if (!serial) {
      cudaEventRecord(evChain, sA);
      cudaStreamWaitEvent(sC, evChain, 0);
      cudaStreamWaitEvent(sA, evAL, 0);  // left update of A done before its right update
    }
    // the panel's right reflectors on A and Z (ab2rht.f90:387-467), one prepared list.  The next
    // panel's left generation reads A's rows >= jb0 + 2nb only: those rows stay on the chain, the
    // rows above join the Z update on sC (whose next A left update the next panel's A right
    // update waits for through evAL)
    const GeoS1Right gall{P, VRc[s], TR[s], -1};
    const int split_row = std::min(n, jb0 + 2 * nb);
    prepare_any(reg[4], gall, P.nblocks, sA);
    if (!serial) {
      cudaEventRecord(evPrep, sA);
      cudaStreamWaitEvent(sC, evPrep, 0);
    }
    apply_right_any(reg[4], A, lda, split_row, n - 1, gall, P.nblocks, sA, false);
    apply_right_side(reg[4], A, lda, 0, split_row - 1, gall, P.nblocks, sC, false);
    apply_right_side(reg[4], Z, ldz, 0, n - 1, gall, P.nblocks, sC, false);
    if (!serial) cudaEventRecord(evZ[s], sC);
  }
  if (!serial) {  // join
    cudaEventRecord(evRest, sB);
    cudaStreamWaitEvent(sA, evRest, 0);
    cudaEventRecord(evChain, sC);
    cudaStreamWaitEvent(sA, evChain, 0);
  }
  if (timer) timer->mark(sA, -1);
  return 0;
}

}  // namespace pht
