// stage1_gen.cuh -- device bodies of the stage-1 generation kernels (one CTA each), shared by
// the single-pencil kernels (stage1_gen.cu) and the persistent batched kernel (batched.cu).
//
// On GB300 a dependent FP64 instruction costs about 64 cycles and one SM retires 2 FP64 FMAs
// per cycle, so these bodies keep every small factorisation in shared memory, give each row
// (RQ) or column (QR) a fixed group of 4 or 8 lanes of one warp, and fuse per reflector the
// squared norm and all the dot products into one pass (the norm is the dot product of the
// reflector row/column with itself).  One __syncthreads publishes the reflector scalars, one
// closes the update.  The arithmetic is FP64 throughout and does not depend on blockDim.x
// beyond the documented minimum (lgen: 8 nb threads; rgen: 64 threads, qm_threads fixes the
// lane split of the dorgrq/LQ phase).
//
//   s1_lgen_body  left generation of one panel (src/ab2rht.f90:85-123): for each block bottom to
//                 top, QR (dgeqr2) of A(ib:ib2, jb:jb+nb-1), VL explicit, R back into A, TL.
//   s1_rgen_body  right generation of one block (src/ab2rht.f90:282-312): RQ of the L x L diagonal
//                 block of B (dgerq2), the first nb rows of its orthogonal factor (dorgrq), their
//                 LQ (dgelq2) and TR (dlarft 'F','R'); or, when the block has at most nb rows, the
//                 backward row-wise reflectors of the RQ itself and TR (dlarft 'B','R').
#pragma once
#include "paraht_internal.cuh"
#include "stage1_geom.cuh"

namespace pht {

inline __host__ __device__ int s1_round16(int x) { return (x + 15) / 16 * 16; }
inline __host__ __device__ int s1_lgen_pitch(int L) { return s1_round16(L) + 8; }
inline __host__ __device__ int s1_rgen_pitch(int L) { return s1_round16(L) + 4; }

// Reflector scalars of DLARFG from alpha and the squared norm of x (see make_reflector_nr):
// tau, scal = 1/(alpha-beta), beta.
PHT_DEV Reflector reflector_from_norm2(double alpha, double xnorm2) { return make_reflector_nr(alpha, xnorm2); }

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
static __device__ void t_forward(int k, const double* G, int ldg, const double* tau, double* Ts, int nbT, double* T,
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

static __device__ void t_backward(int k, const double* G, int ldg, const double* tau, double* Ts, int nbT, double* T,
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
static __device__ void s1_lgen_body(double* __restrict__ A, int lda, const S1Panel& P, double* __restrict__ VL,
                                    double* __restrict__ TL, double* sm) {
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

// M <- M H(0) H(1) ... H(nb2-1) for the nb rows of M (dorgrq), QM lanes per row, the row held in
// registers (column part + QM k in element k; nb2 <= 64).  Reflector i: V[i][c] at
// Vs[i * vsi + c * vsc] for c < i, 1 at c = i, tau tauR[i].  Only the warps that own rows run.
template <int QM>
static __device__ void dorgrq_rows(double* M, int ldm, const double* Vs, int vsi, int vsc, const double* tauR, int nb,
                                   int nb2) {
  constexpr int EL = 64 / QM;
  const int t = threadIdx.x, r = t / QM, part = t % QM;
  if ((t & ~31) >= nb * QM) return;  // warp-uniform: no row of this warp exists
  const bool live = r < nb;
  double m[EL];
#pragma unroll
  for (int k = 0; k < EL; ++k) {
    const int col = part + QM * k;
    m[k] = (live && col < nb2) ? M[r * ldm + col] : 0.0;
  }
  for (int i = 0; i < nb2; ++i) {
    const double ti = tauR[i];
    if (ti == 0.0) continue;
    double vv[EL];
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int k = 0; k < EL; ++k) {
      vv[k] = 0.0;
      if (QM * k <= i) {  // warp-uniform: some lane of this chunk lies at or before column i
        const int col = part + QM * k;
        vv[k] = col < i ? Vs[i * vsi + col * vsc] : (col == i ? 1.0 : 0.0);
        if (k & 1)
          s1 = fma(m[k], vv[k], s1);
        else
          s0 = fma(m[k], vv[k], s0);
      }
    }
    double s = s0 + s1;
#pragma unroll
    for (int off = 1; off < QM; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const double tw = ti * s;
#pragma unroll
    for (int k = 0; k < EL; ++k)
      if (QM * k <= i) m[k] = fma(-tw, vv[k], m[k]);
  }
  if (live)
#pragma unroll
    for (int k = 0; k < EL; ++k) {
      const int col = part + QM * k;
      if (col < nb2) M[r * ldm + col] = m[k];
    }
}

// ------------------------------------------------------------------------------------------
// Right generation for block o.  blockDim.x == 4 * Lp (Lp = L rounded up to a multiple of 8);
// thread (row rho = t/4, quarter q = t%4) owns columns c = q, q+4, q+8, ... of row rho.
// Shared memory: S (L x L, ld L+1), M (nb x L, ld nb), dvec (L), tauR (L), tauL (nb), G (nb*nb),
// Ts (nb*nb), sc (4).
// ------------------------------------------------------------------------------------------
static __device__ void s1_rgen_body(const double* __restrict__ B, int ldb, const S1Panel& P, int o,
                                    double* __restrict__ VRc, double* __restrict__ TR, int use_vr, int qm_threads,
                                    double* sm) {
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
  double* sc = Ts + nb * nb;            // 4, then 2 (L+1) for the published RQ reflectors
  const int t = threadIdx.x;
  for (int e = t; e < nb2 * nb2; e += blockDim.x) {
    const int i = e % nb2, j = e / nb2;
    S[i + j * lds] = B[(size_t)(ib0 + i) + (size_t)(ib0 + j) * ldb];
  }
  __syncthreads();
  // ---- RQ (dgerq2): rows bottom to top; the reflector of row i acts on columns 0..i ----
  // Warp 0 forms the reflectors: in round s it applies reflector s to row s-1 and forms reflector
  // s-1 from it (the critical chain); warps 1.. apply reflector s to the rows below s-1 in the
  // same round (FP64 throughput), so the two overlap.  They hand over through named barriers:
  // ready[s&1] (reflector s published; warp 0 arrives, the others wait) and done[s&1] (rows below
  // s-1 updated by reflector s; the others arrive, warp 0 waits before it touches row s-2).
  // Same-parity generations never overlap: warp 0 publishes reflector r only after waiting for
  // done(r+2), which the others signal after consuming ready(r+2); the others signal done(s) only
  // after waiting for ready(s), which warp 0 publishes after consuming done(s+2).
  {
    const int nthr = blockDim.x, lane = t & 31;
    double* pv = sc + 4;  // two published reflectors: v[0..L-1] (v_s = 1 implied), tau at [L]
    auto bar_sync = [&](int id) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthr) : "memory"); };
    auto bar_arrive = [&](int id) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthr) : "memory"); };
    if (t < 32) {
      // reflector of row r from its current values: scaled tail into S and the publish slot
      auto form = [&](int r) {
        double sg = 0.0;
        for (int c = lane; c < r; c += 32) sg = fma(S[r + c * lds], S[r + c * lds], sg);
        sg = warp_sum(sg);
        const Reflector h = reflector_from_norm2(S[r + r * lds], sg);
        double* v = pv + (r & 1) * (L + 1);
        for (int c = lane; c < r; c += 32) {
          const double x = S[r + c * lds] * h.scal;
          S[r + c * lds] = x;
          v[c] = x;
        }
        if (lane == 0) {
          S[r + r * lds] = h.beta;
          v[L] = h.tau;
          tauR[r] = h.tau;
        }
      };
      if (nb2 >= 1) form(nb2 - 1);
      if (nb2 - 1 >= 1) {
        __threadfence_block();
        bar_arrive(1 + ((nb2 - 1) & 1));
      }
      for (int sr = nb2 - 1; sr >= 1; --sr) {
        if (sr <= nb2 - 2) bar_sync(3 + ((sr + 1) & 1));
        const double* v = pv + (sr & 1) * (L + 1);
        const double tau = v[L];
        const int r = sr - 1;
        double d = 0.0;
        for (int c = lane; c < sr; c += 32) d = fma(S[r + c * lds], v[c], d);
        d = warp_sum(d);
        if (tau != 0.0) {
          const double tw = tau * (S[r + sr * lds] + d);
          for (int c = lane; c < sr; c += 32) S[r + c * lds] = fma(-tw, v[c], S[r + c * lds]);
          if (lane == 0) S[r + sr * lds] -= tw;
        }
        __syncwarp();
        form(r);
        if (r >= 1) {
          __threadfence_block();
          bar_arrive(1 + (r & 1));
        }
      }
      if (nb2 - 1 >= 1) bar_sync(3 + (1 & 1));  // done(1)
    } else {
      const int u = t - 32, g = u / Q, qq = u % Q, G = (nthr - 32) / Q;
      for (int sr = nb2 - 1; sr >= 1; --sr) {
        bar_sync(1 + (sr & 1));
        const double* v = pv + (sr & 1) * (L + 1);
        const double tau = v[L];
        for (int k0 = 0; k0 * G < sr - 1; ++k0) {  // uniform over the warps of this group
          const int rr = g + G * k0;
          double a0 = 0.0, a1 = 0.0;
          if (rr < sr - 1) {
            int cc = qq;
            for (; cc + Q < sr; cc += 2 * Q) {
              a0 = fma(S[rr + cc * lds], v[cc], a0);
              a1 = fma(S[rr + (cc + Q) * lds], v[cc + Q], a1);
            }
            if (cc < sr) a0 = fma(S[rr + cc * lds], v[cc], a0);
          }
          const double dd = group_sum<Q>(a0 + a1);
          if (rr < sr - 1 && tau != 0.0) {
            const double tw = tau * (S[rr + sr * lds] + dd);
            for (int cc = qq; cc < sr; cc += Q) S[rr + cc * lds] = fma(-tw, v[cc], S[rr + cc * lds]);
            if (qq == 0) S[rr + sr * lds] -= tw;
          }
        }
        __threadfence_block();
        bar_arrive(3 + (sr & 1));
      }
    }
  }
  __syncthreads();
  double* V = VRc + (size_t)o * L * nb;
  double* Tout = TR + (size_t)o * nb * nb;
  if (nb2 > nb) {
    // ---- M = [I 0] H(1) H(2) ... H(nb2): first nb rows of the RQ orthogonal factor (dorgrq) ----
    // thread (row r = t / QM, part = t % QM) with QM lanes per row: the largest power of two
    // <= min(32, min(qm_threads, 128) / nb) (qm_threads <= blockDim.x; it fixes the summation
    // order).  At most four warps, one per scheduler: each SM sub-partition issues one FP64
    // instruction per ~64 cycles, so more warps with partly masked lanes only queue behind it.
    int QM = 1;
    while (2 * QM <= 32 && 2 * QM * nb <= min(qm_threads, 128)) QM *= 2;
    const int r = t / QM, part = t % QM;
    for (int e = t; e < nb * nb2; e += blockDim.x) M[(e / nb2) * ldm + e % nb2] = ((e / nb2) == (e % nb2)) ? 1.0 : 0.0;
    if (use_vr)  // reflector of row i: S[i][0..i-1], implicit 1 at column i
      for (int e = t; e < nb2 * nb2; e += blockDim.x) {
        const int i = e / nb2, cc = e % nb2;
        Vr[i * L + cc] = cc < i ? S[i + cc * lds] : 0.0;
      }
    __syncthreads();
    // rows of M are independent: each lane group runs through all reflectors without barriers,
    // its row in registers when it fits (nb2 <= 64)
    const int vsi = use_vr ? L : 1, vsc = use_vr ? 1 : lds;
    const double* Vsrc = use_vr ? Vr : S;
    bool done = false;
    if (nb2 <= 64) {
      switch (QM) {
        case 4:
          dorgrq_rows<4>(M, ldm, Vsrc, vsi, vsc, tauR, nb, nb2);
          done = true;
          break;
        case 8:
          dorgrq_rows<8>(M, ldm, Vsrc, vsi, vsc, tauR, nb, nb2);
          done = true;
          break;
        case 16:
          dorgrq_rows<16>(M, ldm, Vsrc, vsi, vsc, tauR, nb, nb2);
          done = true;
          break;
        case 32:
          dorgrq_rows<32>(M, ldm, Vsrc, vsi, vsc, tauR, nb, nb2);
          done = true;
          break;
        default: break;
      }
    }
    for (int i = 0; i < nb2 && !done; ++i) {
      const double ti = tauR[i];
      if (ti == 0.0) continue;
      double s = 0.0;
      if (r < nb) {
        for (int cc = part; cc < i; cc += QM) s = fma(M[r * ldm + cc], Vsrc[i * vsi + cc * vsc], s);
        if (part == 0) s += M[r * ldm + i];
      }
      // reduce over the QM lanes of this row (QM divides 32)
      for (int off = 1; off < QM; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (r < nb) {
        const double tw = ti * s;
        for (int cc = part; cc < i; cc += QM) M[r * ldm + cc] = fma(-tw, Vsrc[i * vsi + cc * vsc], M[r * ldm + cc]);
        if (part == 0) M[r * ldm + i] -= tw;
      }
    }
    __syncthreads();
    // ---- LQ (dgelq2) of M: reflector i from row i, columns i..nb2-1; same lane layout ----
    // M's rows are orthonormal (the first nb rows of an orthogonal matrix), so the LQ needs no
    // norms or dot products (Householder reconstruction from an orthonormal basis, Ballard et al.
    // 2014): after reflectors 0..i-1, row i is zero before column i and has unit norm, so
    // DLARFG gives |beta| = 1, tau = 1 + |alpha|, scal = sign(alpha) / (1 + |alpha|); every
    // later row r is orthogonal to row i, so its dot product with the reflector tail is
    // -alpha M[r][i] and the update of row r reduces to M[r][c] -= (scal M[r][i]) M[i][c].  The
    // entries M[r][i] this leaves (r > i, DLARFG's L factor, zero up to rounding) are never read.
    // A tail that is exactly zero takes tau = 0 (H = I), as in DLARFG.
    for (int i = 0; i < nb; ++i) {
      bool nz = false;
      if (r == i)
        for (int cc = i + 1 + part; cc < nb2; cc += QM) nz |= M[i * ldm + cc] != 0.0;
      const bool any = __syncthreads_or(nz) != 0;  // also publishes the previous step's rows
      const double alpha = M[i * ldm + i];
      double tl = 0.0, scal = 1.0, beta = alpha;
      if (any) {
        const double aa = fabs(alpha);
        tl = 1.0 + aa;
        scal = copysign(1.0 / tl, alpha);
        beta = -copysign(1.0, alpha);
        if (r > i && r < nb) {
          const double tws = M[r * ldm + i] * scal;
          for (int cc = i + 1 + part; cc < nb2; cc += QM) M[r * ldm + cc] = fma(-tws, M[i * ldm + cc], M[r * ldm + cc]);
        }
      }
      __syncthreads();
      if (r == i) {
        for (int cc = i + 1 + part; cc < nb2; cc += QM) M[i * ldm + cc] *= scal;
        if (part == 0) {
          M[i * ldm + i] = beta;
          tauL[i] = tl;
        }
      }
    }
    __syncthreads();
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

inline size_t s1_lgen_smem(int L, int nb) {
  return sizeof(double) * ((size_t)s1_lgen_pitch(L) * nb + 2 * nb * nb + 2 * nb + 4);
}
inline size_t s1_rgen_smem_vr(int L, int nb, bool vr) {
  const size_t p = (size_t)s1_rgen_pitch(L);
  return sizeof(double) *
         (p * L + (size_t)nb * p + (vr ? (size_t)L * L : 0) + 2 * (size_t)L + nb + 2 * nb * nb + 4 + 2 * ((size_t)L + 1));
}
// 4 lanes per row, a multiple of 32, and at least two warps (warp 0 forms the RQ reflectors, the
// others update the remaining rows)
__host__ __device__ inline int s1_rgen_threads(int L) { return max(64, 4 * (((L + 7) / 8) * 8)); }
inline int s1_lgen_threads(int nb) { return ((8 * nb + 31) / 32) * 32; }  // 8 lanes per column

}  // namespace pht
