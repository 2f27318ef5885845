// stage1_gen.cu -- latency-oriented generation kernels of stage 1 (the sequential chain).
//
// On GB300 a dependent FP64 instruction costs about 64 cycles and one SM retires 2 FP64 FMAs
// per cycle, so these kernels keep every small factorisation in shared memory, give each row
// (RQ) or column (QR) a fixed group of 4 or 8 lanes of one warp, and fuse per reflector the
// squared norm and all the dot products into one pass (the norm is the dot product of the
// reflector row/column with itself).  One __syncthreads publishes the reflector scalars, one
// closes the update.  The arithmetic is FP64 throughout.
//
//   k_s1_lgen  left generation of one panel (src/ab2rht.f90:85-123): for each block bottom to
//              top, QR (dgeqr2) of A(ib:ib2, jb:jb+nb-1), VL explicit, R back into A, TL.
//   k_s1_rgen  right generation of one block (src/ab2rht.f90:282-312): RQ of the L x L diagonal
//              block of B (dgerq2), the first nb rows of its orthogonal factor (dorgrq), their
//              LQ (dgelq2) and TR (dlarft 'F','R'); or, when the block has at most nb rows, the
//              backward row-wise reflectors of the RQ itself and TR (dlarft 'B','R').
#include "launch_count.h"
#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "stage1_geom.cuh"

namespace pht {

static inline __host__ __device__ int s1_round16(int x) { return (x + 15) / 16 * 16; }
static inline __host__ __device__ int s1_lgen_pitch(int L) { return s1_round16(L) + 8; }
static inline __host__ __device__ int s1_rgen_pitch(int L) { return s1_round16(L) + 4; }

// Reflector scalars of DLARFG from alpha and the squared norm of x (see make_reflector).
// tau, scal = 1/(alpha-beta), beta.
PHT_DEV Reflector reflector_from_norm2(double alpha, double xnorm2) { return make_reflector(alpha, xnorm2); }

// Sum over groups of G consecutive lanes (G = 4 or 8), result in every lane of the group.
template <int G>
PHT_DEV double group_sum(double v) {
#pragma unroll
  for (int o = 1; o < G; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// T of a block reflector from its Gram matrix (forward: T upper, T[l][m] = -tau_m sum_q T[l][q]
// G[q][m]; backward: T lower, T[m][i] = -tau_i sum_l T[m][l] G[l][i]).  G, tau, Ts in shared
// memory; T written with explicit zeros, ld ldt.  Rows of one column in parallel.
__device__ void t_forward(int k, const double* G, int ldg, const double* tau, double* Ts, int nbT, double* T,
                          int ldt) {
  const int t = threadIdx.x;
  for (int e = t; e < nbT * nbT; e += blockDim.x) Ts[e] = 0.0;
  __syncthreads();
  for (int m = 0; m < k; ++m) {
    if (t < m) {
      double s0 = 0.0, s1 = 0.0;
      int q = t;
      for (; q + 1 < m; q += 2) {
        s0 = fma(Ts[t + q * nbT], G[q + m * ldg], s0);
        s1 = fma(Ts[t + (q + 1) * nbT], G[q + 1 + m * ldg], s1);
      }
      if (q < m) s0 = fma(Ts[t + q * nbT], G[q + m * ldg], s0);
      Ts[t + m * nbT] = -tau[m] * (s0 + s1);
    }
    if (t == m) Ts[m + m * nbT] = tau[m];
    __syncthreads();
  }
  for (int e = t; e < nbT * nbT; e += blockDim.x) T[(e % nbT) + (size_t)(e / nbT) * ldt] = Ts[e];
}

__device__ void t_backward(int k, const double* G, int ldg, const double* tau, double* Ts, int nbT, double* T,
                           int ldt) {
  const int t = threadIdx.x;
  for (int e = t; e < nbT * nbT; e += blockDim.x) Ts[e] = 0.0;
  __syncthreads();
  for (int i = k - 1; i >= 0; --i) {
    if (t == i) Ts[i + i * nbT] = tau[i];
    if (t > i && t < k) {
      double s = 0.0;
      for (int l = i + 1; l <= t; ++l) s = fma(Ts[t + l * nbT], G[l + i * ldg], s);
      Ts[t + i * nbT] = -tau[i] * s;
    }
    __syncthreads();
  }
  for (int e = t; e < nbT * nbT; e += blockDim.x) T[(e % nbT) + (size_t)(e / nbT) * ldt] = Ts[e];
}

// ------------------------------------------------------------------------------------------
// Left generation: one CTA per panel, blocks bottom to top.  Each column c is owned by G = 8
// consecutive lanes of one warp that split its rows; blockDim.x = 8*nb rounded up to a multiple
// of 32 (threads with c >= nb only take part in the shuffles).
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) k_s1_lgen(double* __restrict__ A, int lda, S1Panel P, double* __restrict__ VL,
                                                  double* __restrict__ TL) {
  extern __shared__ double sm[];
  constexpr int G = 8;
  // column pitch = 8 (mod 16) doubles: the two columns a half-warp touches (8 lanes each, rows
  // g = 0..7) fall into different banks
  const int L = P.L, nb = P.nb, ldp = s1_lgen_pitch(L);
  double* Pt = sm;                    // ldp * nb
  double* G2 = Pt + (size_t)ldp * nb;  // nb*nb Gram
  double* Ts = G2 + nb * nb;          // nb*nb
  double* tau = Ts + nb * nb;         // nb
  double* dsm = tau + nb;             // nb   (dot products of the current step)
  double* sc = dsm + nb;              // 4    (tau, scal, beta of the current step)
  const int t = threadIdx.x;
  const int c = t / G, g = t % G;  // column owned, row group
  const int jb0 = P.jb0;
  for (int o = 0; o < P.nblocks; ++o) {
    const int ib0 = P.ib(o), nb2 = P.nb2(o), k = min(nb, nb2);
    for (int e = t; e < nb2 * nb; e += blockDim.x) {
      const int i = e % nb2, j = e / nb2;
      Pt[i + j * ldp] = A[(size_t)(ib0 + i) + (size_t)(jb0 + j) * lda];
    }
    __syncthreads();
    for (int j = 0; j < k; ++j) {
      // d_c = sum_{i>j} P[i][j] * P[i][c]  (c = j: squared norm of the reflector tail)
      double a0 = 0.0, a1 = 0.0;
      if (c >= j && c < nb) {
        int i = j + 1 + g;
        for (; i + G < nb2; i += 2 * G) {
          a0 = fma(Pt[i + j * ldp], Pt[i + c * ldp], a0);
          a1 = fma(Pt[i + G + j * ldp], Pt[i + G + c * ldp], a1);
        }
        if (i < nb2) a0 = fma(Pt[i + j * ldp], Pt[i + c * ldp], a0);
      }
      const double d = group_sum<G>(a0 + a1);
      if (g == 0 && c >= j && c < nb) dsm[c] = d;
      if (c == j && g == 0) {
        const Reflector h = reflector_from_norm2(Pt[j + j * ldp], d);
        sc[0] = h.tau;
        sc[1] = h.scal;
        sc[2] = h.beta;
      }
      __syncthreads();
      const double tj = sc[0], scal = sc[1], beta = sc[2];
      if (c > j && c < nb && tj != 0.0) {
        // w_c = P[j][c] + scal * d_c ;  P[:,c] -= tau * w_c * v,  v = [1; scal * x]
        const double w = Pt[j + c * ldp] + scal * dsm[c];
        const double tw = tj * w, tws = tw * scal;
        for (int i = j + 1 + g; i < nb2; i += G) Pt[i + c * ldp] = fma(-tws, Pt[i + j * ldp], Pt[i + c * ldp]);
        if (g == 0) Pt[j + c * ldp] -= tw;
      }
      __syncthreads();
      if (c == j) {
        for (int i = j + 1 + g; i < nb2; i += G) Pt[i + j * ldp] *= scal;
        if (g == 0) {
          Pt[j + j * ldp] = beta;
          tau[j] = tj;
        }
      }
      // the scaled column j is read again only after the next step's __syncthreads
    }
    __syncthreads();
    for (int j = k + t; j < nb; j += blockDim.x) tau[j] = 0.0;
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
    // Gram G2[q][m] = v_q . v_m (q < m < k): thread per (q, m) pair, split over the G lanes.
    for (int base = 0; base < nb * nb; base += blockDim.x / G) {
      const int e = base + t / G;
      const int q = e % nb, m = e / nb;
      double s = 0.0;
      if (e < nb * nb && q < m && m < k) {
        for (int i = m + 1 + g; i < nb2; i += G) s = fma(Pt[i + q * ldp], Pt[i + m * ldp], s);
      }
      s = group_sum<G>(s);
      if (g == 0 && e < nb * nb) G2[q + m * nb] = (q < m && m < k) ? s + Pt[m + q * ldp] : 0.0;
    }
    __syncthreads();
    t_forward(k, G2, nb, tau, Ts, nb, TL + (size_t)o * nb * nb, nb);
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// Right generation for block o.  blockDim.x == 4 * Lp (Lp = L rounded up to a multiple of 8);
// thread (row rho = t/4, quarter q = t%4) owns columns c = q, q+4, q+8, ... of row rho.
// Shared memory: S (L x L, ld L+1), M (nb x L, ld nb), dvec (L), tauR (L), tauL (nb), G (nb*nb),
// Ts (nb*nb), sc (4).
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) k_s1_rgen(const double* __restrict__ B, int ldb, S1Panel P, int o,
                                                  double* __restrict__ VRc, double* __restrict__ TR, int use_vr) {
  extern __shared__ double sm[];
  constexpr int Q = 4;
  // S column pitch = 4 (mod 16) doubles: a half-warp (4 rows x 4 column classes) hits 16
  // distinct banks.  M (nb x L) is row-major, its rows read along the columns by 2..32 lanes.
  // Vr (optional): the RQ reflectors row-major, read along columns while forming M.
  const int L = P.L, nb = P.nb, lds = s1_rgen_pitch(L), ldm = lds;
  const int ib0 = P.ib(o), nb2 = P.nb2(o);
  double* S = sm;                       // lds * L
  double* M = S + (size_t)lds * L;      // nb * ldm
  double* Vr = M + (size_t)nb * ldm;    // L * L when use_vr
  double* dvec = Vr + (use_vr ? (size_t)L * L : 0);  // L
  double* tauR = dvec + L;              // L
  double* tauL = tauR + L;              // nb
  double* G2 = tauL + nb;               // nb*nb
  double* Ts = G2 + nb * nb;            // nb*nb
  double* sc = Ts + nb * nb;            // 4
  const int t = threadIdx.x, rho = t / Q, q = t % Q;
  for (int e = t; e < nb2 * nb2; e += blockDim.x) {
    const int i = e % nb2, j = e / nb2;
    S[i + j * lds] = B[(size_t)(ib0 + i) + (size_t)(ib0 + j) * ldb];
  }
  __syncthreads();
  // ---- RQ (dgerq2): rows bottom to top; reflector of row i acts on columns 0..i ----
  for (int i = nb2 - 1; i >= 0; --i) {
    // d_rho = sum_{c<i} S[rho][c] S[i][c]   (rho = i: squared norm)
    double a0 = 0.0, a1 = 0.0;
    if (rho <= i) {
      int cc = q;
      for (; cc + Q < i; cc += 2 * Q) {
        a0 = fma(S[rho + cc * lds], S[i + cc * lds], a0);
        a1 = fma(S[rho + (cc + Q) * lds], S[i + (cc + Q) * lds], a1);
      }
      if (cc < i) a0 = fma(S[rho + cc * lds], S[i + cc * lds], a0);
    }
    const double d = group_sum<Q>(a0 + a1);
    if (q == 0 && rho <= i) dvec[rho] = d;
    if (rho == i && q == 0) {
      const Reflector h = reflector_from_norm2(S[i + i * lds], d);
      sc[0] = h.tau;
      sc[1] = h.scal;
      sc[2] = h.beta;
    }
    __syncthreads();
    const double ti = sc[0], scal = sc[1], beta = sc[2];
    if (rho < i && ti != 0.0) {
      const double w = S[rho + i * lds] + scal * dvec[rho];
      const double tw = ti * w, tws = tw * scal;
      for (int cc = q; cc < i; cc += Q) S[rho + cc * lds] = fma(-tws, S[i + cc * lds], S[rho + cc * lds]);
      if (q == 0) S[rho + i * lds] -= tw;
    }
    __syncthreads();
    if (rho == i) {
      for (int cc = q; cc < i; cc += Q) S[i + cc * lds] *= scal;
      if (q == 0) {
        S[i + i * lds] = beta;
        tauR[i] = ti;
      }
    }
  }
  __syncthreads();
  double* V = VRc + (size_t)o * L * nb;
  double* Tout = TR + (size_t)o * nb * nb;
  if (nb2 > nb) {
    // ---- M = [I 0] H(1) H(2) ... H(nb2): first nb rows of the RQ orthogonal factor (dorgrq) ----
    // thread (row r = t / QM, part = t % QM) with QM lanes per row (QM = blockDim/nb, power of 2 <= 32)
    int QM = 1;  // lanes per row: largest power of two <= min(32, blockDim / nb)
    while (2 * QM <= 32 && 2 * QM * nb <= (int)blockDim.x) QM *= 2;
    const int r = t / QM, part = t % QM;
    for (int e = t; e < nb * nb2; e += blockDim.x) M[(e / nb2) * ldm + e % nb2] = ((e / nb2) == (e % nb2)) ? 1.0 : 0.0;
    if (use_vr)  // reflector of row i: S[i][0..i-1], implicit 1 at column i
      for (int e = t; e < nb2 * nb2; e += blockDim.x) {
        const int i = e / nb2, cc = e % nb2;
        Vr[i * L + cc] = cc < i ? S[i + cc * lds] : 0.0;
      }
    __syncthreads();
    // rows of M are independent: each lane group runs through all reflectors without barriers
    for (int i = 0; i < nb2; ++i) {
      const double ti = tauR[i];
      if (ti == 0.0) continue;
      double s = 0.0;
      if (r < nb) {
        if (use_vr)
          for (int cc = part; cc < i; cc += QM) s = fma(M[r * ldm + cc], Vr[i * L + cc], s);
        else
          for (int cc = part; cc < i; cc += QM) s = fma(M[r * ldm + cc], S[i + cc * lds], s);
        if (part == 0) s += M[r * ldm + i];
      }
      // reduce over the QM lanes of this row (QM divides 32)
      for (int off = 1; off < QM; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (r < nb) {
        const double tw = ti * s;
        if (use_vr)
          for (int cc = part; cc < i; cc += QM) M[r * ldm + cc] = fma(-tw, Vr[i * L + cc], M[r * ldm + cc]);
        else
          for (int cc = part; cc < i; cc += QM) M[r * ldm + cc] = fma(-tw, S[i + cc * lds], M[r * ldm + cc]);
        if (part == 0) M[r * ldm + i] -= tw;
      }
    }
    __syncthreads();
    // ---- LQ (dgelq2) of M: reflector i from row i, columns i..nb2-1; same lane layout ----
    for (int i = 0; i < nb; ++i) {
      double s = 0.0;
      if (r >= i && r < nb)
        for (int cc = i + 1 + part; cc < nb2; cc += QM) s = fma(M[r * ldm + cc], M[i * ldm + cc], s);
      for (int off = 1; off < QM; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (r == i && part == 0) {
        dvec[r] = s;
        const Reflector h = reflector_from_norm2(M[i * ldm + i], s);
        sc[0] = h.tau;
        sc[1] = h.scal;
        sc[2] = h.beta;
      } else if (part == 0 && r > i && r < nb) {
        dvec[r] = s;
      }
      __syncthreads();
      const double tl = sc[0], scal = sc[1], beta = sc[2];
      if (r > i && r < nb && tl != 0.0) {
        const double w = M[r * ldm + i] + scal * dvec[r];
        const double tw = tl * w, tws = tw * scal;
        for (int cc = i + 1 + part; cc < nb2; cc += QM) M[r * ldm + cc] = fma(-tws, M[i * ldm + cc], M[r * ldm + cc]);
        if (part == 0) M[r * ldm + i] -= tw;
      }
      __syncthreads();
      if (r == i) {
        for (int cc = i + 1 + part; cc < nb2; cc += QM) M[i * ldm + cc] *= scal;
        if (part == 0) {
          M[i * ldm + i] = beta;
          tauL[i] = tl;
        }
      }
      __syncthreads();
    }
    // VRc[c][i] = VR[i][c]: 1 at c == i, M[i][c] for c > i, 0 before
    for (int e = t; e < L * nb; e += blockDim.x) {
      const int cc = e % L, i = e / L;
      double v = 0.0;
      if (cc < nb2) v = (cc < i) ? 0.0 : (cc == i ? 1.0 : M[i * ldm + cc]);
      V[cc + (size_t)i * L] = v;
    }
    // Gram G2[a][b] = VR[a] . VR[b] (a < b)
    {
      const int e0 = t / QM;
      for (int base = 0; base < nb * nb; base += blockDim.x / QM) {
        const int e = base + e0;
        const int a = e % nb, b = e / nb;
        double s = 0.0;
        if (e < nb * nb && a < b)
          for (int cc = b + 1 + part; cc < nb2; cc += QM) s = fma(M[a * ldm + cc], M[b * ldm + cc], s);
        for (int off = 1; off < QM; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (part == 0 && e < nb * nb) G2[a + b * nb] = (a < b) ? s + M[a * ldm + b] : 0.0;
      }
    }
    __syncthreads();
    t_forward(nb, G2, nb, tauL, Ts, nb, Tout, nb);
  } else {
    // backward row-wise reflectors of the RQ itself (ab2rht.f90:308-309)
    const int k = nb2;
    for (int e = t; e < L * nb; e += blockDim.x) {
      const int cc = e % L, i = e / L;
      double v = 0.0;
      if (i < k && cc < nb2) v = (cc < i) ? S[i + cc * lds] : (cc == i ? 1.0 : 0.0);
      V[cc + (size_t)i * L] = v;
    }
    for (int e = t; e < nb * nb; e += blockDim.x) {
      const int l = e % nb, i = e / nb;
      double s = 0.0;
      if (l > i && l < k) {
        s = S[l + i * lds];
        for (int cc = 0; cc < i; ++cc) s = fma(S[l + cc * lds], S[i + cc * lds], s);
      }
      G2[l + i * nb] = s;
    }
    __syncthreads();
    t_backward(k, G2, nb, tauR, Ts, nb, Tout, nb);
  }
}

size_t s1_lgen_smem(int L, int nb) {
  return sizeof(double) * ((size_t)s1_lgen_pitch(L) * nb + 2 * nb * nb + 2 * nb + 4);
}
static size_t s1_rgen_smem_vr(int L, int nb, bool vr) {
  const size_t p = (size_t)s1_rgen_pitch(L);
  return sizeof(double) * (p * L + (size_t)nb * p + (vr ? (size_t)L * L : 0) + 2 * (size_t)L + nb + 2 * nb * nb + 4);
}
size_t s1_rgen_smem(int L, int nb) { return s1_rgen_smem_vr(L, nb, false); }
int s1_rgen_threads(int L) { return 4 * (((L + 7) / 8) * 8); }  // 4 lanes per row, multiple of 32
int s1_lgen_threads(int nb) { return ((8 * nb + 31) / 32) * 32; }  // 8 lanes per column

void launch_s1_lgen(cudaStream_t s, double* A, int lda, const S1Panel& P, double* VL, double* TL) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_s1_lgen, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    attr = true;
  }
  count_launch();
  k_s1_lgen<<<1, s1_lgen_threads(P.nb), s1_lgen_smem(P.L, P.nb), s>>>(A, lda, P, VL, TL);
}

void launch_s1_rgen(cudaStream_t s, const double* B, int ldb, const S1Panel& P, int o, double* VRc, double* TR) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_s1_rgen, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    attr = true;
  }
  static int max_smem = -1;
  if (max_smem < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  const bool vr = s1_rgen_smem_vr(P.L, P.nb, true) <= (size_t)max_smem;
  count_launch();
  k_s1_rgen<<<1, s1_rgen_threads(P.L), s1_rgen_smem_vr(P.L, P.nb, vr), s>>>(B, ldb, P, o, VRc, TR, vr ? 1 : 0);
}

}  // namespace pht
