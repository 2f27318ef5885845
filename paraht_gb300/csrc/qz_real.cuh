// qz_real.cuh -- generalized eigenvalues of a real Hessenberg-triangular pencil (H, T) by the real
// double-shift QZ iteration (Moler and Stewart 1973; the formulation of LAPACK DHGEQZ with
// JOB='E'), in real arithmetic on the pencil itself.
//
// Every sweep chases a bulge started by the first column of (M - w1)(M - w2), M = H T^-1, where
// w1, w2 are the eigenvalues of the active block's trailing 2 x 2 pencil (a real pair or a complex
// conjugate pair, used through their real sum and product).  Step k applies a 3 x 3 Householder
// reflector to rows k..k+2 (zeroing the bulge below H's subdiagonal), then restores T's triangle
// with a 3 x 3 reflector on columns k..k+2 (zeroing T[k+2][k], T[k+2][k+1]) and a 2 x 2 one on
// columns k, k+1 (zeroing T[k+1][k]); the last step works on two rows and columns.  Blocks of
// order 1 deflate as real eigenvalues, blocks of order 2 as the two eigenvalues of their 2 x 2
// pencil (a complex conjugate pair or two real ones).  By operation count it needs about a quarter
// of the FP64 operations per eigenvalue of the complex single-shift form in qz.cuh (one host core
// runs it 1.7-2x faster), and it returns real eigenvalues with exactly zero imaginary parts and
// complex ones as exact conjugate pairs.
//
// A diagonal entry of T at most eps ||T||_F is set to zero and moved to the bottom of its block
// (left reflectors on rows i, i+1 move it down one place, right ones on columns i-1, i restore
// H's Hessenberg form), where the entry of H beside it is zeroed from the right and the infinite
// eigenvalue deflates with beta = 0 (Moler and Stewart's treatment of a singular T).
//
// Tolerances, scaling and the lane protocol are those of qz.cuh: H and T are scaled by powers of
// two to largest moduli in [1/2, 1), at most 30 n sweeps (status 2), an exceptional shift every 10
// sweeps without deflation; `QzLanes` spreads the row and column passes over the lanes, every
// lane computes every reflector from the same synchronised values.
#pragma once
#include "qz.cuh"

namespace pht {

// Householder reflector of order m (2 or 3): (I - tau u u^T) (x0, x1, x2) = (beta, 0, 0) with
// u = (1, v1, v2) (x2, v2 unused for m = 2); tau = 0 (the identity) when x1 = x2 = 0.  The
// entries are scaled by their largest modulus first, so no square overflows or underflows.
__host__ __device__ inline void qzr_house(int m, double x0, double x1, double x2, double& tau, double& v1, double& v2,
                                          double& beta) {
  if (m < 3) x2 = 0.0;
  v1 = v2 = 0.0;
  if (x1 == 0.0 && x2 == 0.0) {
    tau = 0.0;
    beta = x0;
    return;
  }
  const double sc = fmax(fabs(x0), fmax(fabs(x1), fabs(x2)));
  const double y0 = x0 / sc, y1 = x1 / sc, y2 = x2 / sc;
  const double nrm = sqrt(y0 * y0 + y1 * y1 + y2 * y2);
  const double b = y0 >= 0.0 ? -nrm : nrm;  // beta / sc, of the sign opposite to x0
  tau = (b - y0) / b;
  const double scal = 1.0 / (y0 - b);
  v1 = y1 * scal;
  v2 = y2 * scal;
  beta = b * sc;
}

// Columns (left passes) or rows (right passes) a lane loads before it stores any.  Two keep the
// batched kernel at 168 registers without spills; the addresses are recomputed for the stores
// rather than held.
constexpr int kQzrBatch = 2;

// Reflector from the left on rows i..i+m-1 over columns [a0, c1] of A and [b0, c1] of B (leading
// dimension ld): x <- x - tau u (u^T x) for each column x, u = (1, v1, v2).  The two ranges form
// one index space shared by the lanes.
template <int m>
__host__ __device__ inline void qzr_left(double* A, int a0, double* B, int b0, int c1, int ld, int i, double tau,
                                         double v1, double v2, QzLanes L) {
  const int na = c1 - a0 + 1, tot = na + (c1 - b0 + 1);
  for (int t0 = L.lane; t0 < tot; t0 += kQzrBatch * L.n) {
    double x[kQzrBatch][m];
#pragma unroll
    for (int u = 0; u < kQzrBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        const double* p = (t < na ? A + (size_t)(a0 + t) * ld : B + (size_t)(b0 + t - na) * ld) + i;
#pragma unroll
        for (int r = 0; r < m; ++r) x[u][r] = p[r];
      }
    }
#pragma unroll
    for (int u = 0; u < kQzrBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        double* p = (t < na ? A + (size_t)(a0 + t) * ld : B + (size_t)(b0 + t - na) * ld) + i;
        const double w = tau * (x[u][0] + v1 * x[u][1] + (m == 3 ? v2 * x[u][m - 1] : 0.0));
        p[0] = x[u][0] - w;
        p[1] = x[u][1] - v1 * w;
        if (m == 3) p[m - 1] = x[u][m - 1] - v2 * w;
      }
    }
  }
}

// Reflector from the right on columns j..j+m-1 over rows [r0, a1] of A and [r0, b1] of B, with u
// ordered from the last column: for each row y = (X[.][j+m-1], .., X[.][j]), y <- y - tau (y u) u^T.
// It maps a row (X[r][j], .., X[r][j+m-1]) whose reversed copy built the reflector to
// (0, .., 0, beta).
template <int m>
__host__ __device__ inline void qzr_right(double* A, int a1, double* B, int b1, int r0, int ld, int j, double tau,
                                          double v1, double v2, QzLanes L) {
  const int na = a1 - r0 + 1, tot = na + (b1 - r0 + 1);
  const size_t c0 = (size_t)(m - 1) * ld, c1 = (size_t)(m - 2) * ld;  // the columns paired with 1 and v1
  for (int t0 = L.lane; t0 < tot; t0 += kQzrBatch * L.n) {
    double y[kQzrBatch][m];
#pragma unroll
    for (int u = 0; u < kQzrBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        const double* p = (t < na ? A + r0 + t : B + r0 + t - na) + (size_t)j * ld;
        y[u][0] = p[c0];
        y[u][1] = p[c1];
        if (m == 3) y[u][m - 1] = p[0];
      }
    }
#pragma unroll
    for (int u = 0; u < kQzrBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        double* p = (t < na ? A + r0 + t : B + r0 + t - na) + (size_t)j * ld;
        const double w = tau * (y[u][0] + v1 * y[u][1] + (m == 3 ? v2 * y[u][m - 1] : 0.0));
        p[c0] = y[u][0] - w;
        p[c1] = y[u][1] - v1 * w;
        if (m == 3) p[0] = y[u][m - 1] - v2 * w;
      }
    }
  }
}

// Sum s and product t of the eigenvalues of the 2 x 2 pencil (A, B), B upper triangular and
// nonsingular: the trace and determinant of A B^-1.
__host__ __device__ inline void qzr_pair(double a11, double a12, double a21, double a22, double b11, double b12,
                                         double b22, double& s, double& t) {
  const double m11 = a11 / b11, m21 = a21 / b11;
  const double m12 = (a12 - m11 * b12) / b22, m22 = (a22 - m21 * b12) / b22;
  s = m11 + m22;
  t = m11 * m22 - m12 * m21;
}

// Eigenvalue of the 1 x 1 block at i, beta made nonnegative, unscaled by uh / ut (every lane
// writes the same values).
__host__ __device__ inline void qzr_one(const double* H, const double* T, int ld, int i, double uh, double ut,
                                        double* alphar, double* alphai, double* beta) {
  const double a = H[(size_t)i * ld + i], b = T[(size_t)i * ld + i];
  const double sg = b < 0.0 ? -1.0 : 1.0;
  alphar[i] = uh * (sg * a);
  alphai[i] = 0.0;
  beta[i] = ut * (sg * b);
}

// Eigenvalues of the 2 x 2 block at rows/columns p, p+1: a conjugate pair (positive imaginary
// part first) or two real ones (the larger in modulus from the formula, the other from the
// product), beta = 1 before unscaling.
__host__ __device__ inline void qzr_two(const double* H, const double* T, int ld, int p, double uh, double ut,
                                        double* alphar, double* alphai, double* beta) {
  const size_t c0 = (size_t)p * ld, c1 = (size_t)(p + 1) * ld;
  double s, t;
  qzr_pair(H[c0 + p], H[c1 + p], H[c0 + p + 1], H[c1 + p + 1], T[c0 + p], T[c1 + p], T[c1 + p + 1], s, t);
  const double h = 0.5 * s, disc = h * h - t;
  if (disc < 0.0) {
    const double im = sqrt(-disc);
    alphar[p] = uh * h;
    alphai[p] = uh * im;
    alphar[p + 1] = uh * h;
    alphai[p + 1] = -(uh * im);
  } else {
    const double l1 = h + copysign(sqrt(disc), h);
    const double l2 = l1 != 0.0 ? t / l1 : 0.0;
    alphar[p] = uh * l1;
    alphai[p] = 0.0;
    alphar[p + 1] = uh * l2;
    alphai[p + 1] = 0.0;
  }
  beta[p] = ut;
  beta[p + 1] = ut;
}

// Eigenvalues alphar[j] + i alphai[j] over beta[j] (beta >= 0; beta = 0 for an infinite one) of
// the real pencil held in H, T (column-major, leading dimension ld, H upper Hessenberg, T upper
// triangular; both overwritten).  Returns 0, or 2 when 30 n sweeps did not converge.
__host__ __device__ inline int qz_real_eigs(int n, double* H, double* T, int ld, double* alphar, double* alphai,
                                            double* beta, QzLanes L) {
#define Hh(i, j) H[(size_t)(j) * ld + (i)]
#define Tt(i, j) T[(size_t)(j) * ld + (i)]
  const double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
  double hmax = 0.0, tmax = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= (j + 1 < n ? j + 1 : j); ++i) {
      hmax = fmax(hmax, fabs(Hh(i, j)));
      if (i <= j) tmax = fmax(tmax, fabs(Tt(i, j)));
    }
  double hs = 0.0, ts = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= (j + 1 < n ? j + 1 : j); ++i) {
      if (hmax > 0.0) {
        const double ha = fabs(Hh(i, j)) / hmax;
        hs += ha * ha;
      }
      if (i <= j && tmax > 0.0) {
        const double ta = fabs(Tt(i, j)) / tmax;
        ts += ta * ta;
      }
    }
  int eh = 0, et = 0;
  if (hmax > 0.0) frexp(hmax, &eh);
  if (tmax > 0.0) frexp(tmax, &et);
  eh = eh < -1000 ? -1000 : (eh > 1000 ? 1000 : eh);
  et = et < -1000 ? -1000 : (et > 1000 ? 1000 : et);
  const double sh = ldexp(1.0, -eh), st = ldexp(1.0, -et);
  PHT_QZ_SYNC();  // every lane has read the unscaled entries
  for (long long e = L.lane; e < (long long)n * n; e += L.n) {
    const int j = (int)(e / n), i = (int)(e % n);
    Hh(i, j) = sh * Hh(i, j);
    Tt(i, j) = st * Tt(i, j);
  }
  PHT_QZ_SYNC();
  const double uh = ldexp(1.0, eh), ut = ldexp(1.0, et);  // undo the scaling in alpha and beta
  const double atol = fmax(tiny, eps * (sh * hmax * sqrt(hs))), btol = fmax(tiny, eps * (st * tmax * sqrt(ts)));
  int ilast = n - 1, iter = 0, total = 0;
  const int maxit = 30 * (n > 1 ? n : 1);
  while (ilast >= 0) {
    if (ilast == 0) {
      qzr_one(H, T, ld, 0, uh, ut, alphar, alphai, beta);
      break;
    }
    if (fabs(Hh(ilast, ilast - 1)) <= fmax(atol, eps * (fabs(Hh(ilast, ilast)) + fabs(Hh(ilast - 1, ilast - 1))))) {
      PHT_QZ_SYNC();
      if (L.lane == 0) Hh(ilast, ilast - 1) = 0.0;
      qzr_one(H, T, ld, ilast, uh, ut, alphar, alphai, beta);
      --ilast;
      iter = 0;
      PHT_QZ_SYNC();
      continue;
    }
    int cand = 0;
    for (int i = 1 + L.lane; i < ilast; i += L.n)
      if (fabs(Hh(i, i - 1)) <= fmax(atol, eps * (fabs(Hh(i, i)) + fabs(Hh(i - 1, i - 1))))) cand = i;
    const int ifirst = PHT_QZ_LANE_MAX(cand);
    PHT_QZ_SYNC();
    if (ifirst > 0 && L.lane == 0) Hh(ifirst, ifirst - 1) = 0.0;
    PHT_QZ_SYNC();
    // a negligible diagonal entry of T (an infinite eigenvalue): set it to zero and move it to
    // the bottom of the block, where it deflates with beta = 0
    int jz = -1;
    for (int j = ifirst + L.lane; j <= ilast; j += L.n)
      if (fabs(Tt(j, j)) <= btol) jz = j;
    jz = PHT_QZ_LANE_MAX(jz);
    if (jz >= 0) {
      if (++total > maxit) return 2;
      double tau, w1, w2, bet;
      PHT_QZ_SYNC();
      if (L.lane == 0) Tt(jz, jz) = 0.0;
      PHT_QZ_SYNC();
      if (jz == ilast) {  // zero H[ilast][ilast-1] from the right; T's last row stays zero
        qzr_house(2, Hh(ilast, ilast), Hh(ilast, ilast - 1), 0.0, tau, w1, w2, bet);
        PHT_QZ_SYNC();
        qzr_right<2>(H, ilast, T, ilast - 1, ifirst, ld, ilast - 1, tau, w1, w2, L);
        PHT_QZ_SYNC();
        if (L.lane == 0) Hh(ilast, ilast - 1) = 0.0;
      } else if (jz == ifirst) {  // zero H[ifirst+1][ifirst] from the left: a 1 x 1 block splits off
        qzr_house(2, Hh(jz, jz), Hh(jz + 1, jz), 0.0, tau, w1, w2, bet);
        PHT_QZ_SYNC();
        qzr_left<2>(H, jz, T, jz + 1, ilast, ld, jz, tau, w1, w2, L);
        PHT_QZ_SYNC();
        if (L.lane == 0) Hh(jz + 1, jz) = 0.0;
      } else {  // chase the zero down: rows i, i+1 move it to T[i+1][i+1], columns i-1, i restore H
        for (int i = jz; i < ilast; ++i) {
          qzr_house(2, Tt(i, i + 1), Tt(i + 1, i + 1), 0.0, tau, w1, w2, bet);
          PHT_QZ_SYNC();
          qzr_left<2>(H, i - 1, T, i + 1, ilast, ld, i, tau, w1, w2, L);
          PHT_QZ_SYNC();
          if (L.lane == 0) Tt(i + 1, i + 1) = 0.0;
          PHT_QZ_SYNC();
          qzr_house(2, Hh(i + 1, i), Hh(i + 1, i - 1), 0.0, tau, w1, w2, bet);
          PHT_QZ_SYNC();
          qzr_right<2>(H, i + 1, T, i, ifirst, ld, i - 1, tau, w1, w2, L);
          PHT_QZ_SYNC();
          if (L.lane == 0) Hh(i + 1, i - 1) = 0.0;
          PHT_QZ_SYNC();
        }
      }
      PHT_QZ_SYNC();
      continue;
    }
    if (ilast - ifirst == 1) {  // an isolated 2 x 2 block
      qzr_two(H, T, ld, ifirst, uh, ut, alphar, alphai, beta);
      ilast -= 2;
      iter = 0;
      PHT_QZ_SYNC();
      continue;
    }
    if (++total > maxit) return 2;
    ++iter;
    // the two shifts through their sum s and product t
    double s, t;
    if (iter % 10 == 0) {
      const double w = Hh(ilast, ilast) / Tt(ilast, ilast) +
                       0.75 * fabs(Hh(ilast, ilast - 1)) / fmax(fabs(Tt(ilast - 1, ilast - 1)), tiny);
      s = 2.0 * w;
      t = w * w;
    } else {
      const int p = ilast - 1;
      qzr_pair(Hh(p, p), Hh(p, ilast), Hh(ilast, p), Hh(ilast, ilast), Tt(p, p), Tt(p, ilast), Tt(ilast, ilast), s,
               t);
    }
    // first column of (M - w1)(M - w2) at the top of the block: M e1 = (v1, v2), M^2 e1 = H T^-1 (v1, v2)
    const int a = ifirst;
    const double v1 = Hh(a, a) / Tt(a, a), v2 = Hh(a + 1, a) / Tt(a, a);
    const double u2 = v2 / Tt(a + 1, a + 1), u1 = (v1 - Tt(a, a + 1) * u2) / Tt(a, a);
    double x0 = Hh(a, a) * u1 + Hh(a, a + 1) * u2 - s * v1 + t;
    double x1 = Hh(a + 1, a) * u1 + Hh(a + 1, a + 1) * u2 - s * v2;
    double x2 = Hh(a + 2, a + 1) * u2;
    for (int k = ifirst; k < ilast; ++k) {
      const int m = ilast - k + 1 < 3 ? ilast - k + 1 : 3;
      double tau, w1, w2, bet;
      qzr_house(m, x0, x1, x2, tau, w1, w2, bet);
      PHT_QZ_SYNC();
      if (m == 3)
        qzr_left<3>(H, k > ifirst ? k - 1 : k, T, k, ilast, ld, k, tau, w1, w2, L);
      else
        qzr_left<2>(H, k > ifirst ? k - 1 : k, T, k, ilast, ld, k, tau, w1, w2, L);
      PHT_QZ_SYNC();
      if (k > ifirst && L.lane == 0) {  // the bulge below the subdiagonal, zero by construction
        Hh(k + 1, k - 1) = 0.0;
        if (m == 3) Hh(k + 2, k - 1) = 0.0;
      }
      PHT_QZ_SYNC();
      const int hr1 = k + 3 < ilast ? k + 3 : ilast;
      if (m == 3) {  // zero T[k+2][k], T[k+2][k+1]
        qzr_house(3, Tt(k + 2, k + 2), Tt(k + 2, k + 1), Tt(k + 2, k), tau, w1, w2, bet);
        PHT_QZ_SYNC();
        qzr_right<3>(H, hr1, T, k + 2, ifirst, ld, k, tau, w1, w2, L);
        PHT_QZ_SYNC();
        if (L.lane == 0) {
          Tt(k + 2, k) = 0.0;
          Tt(k + 2, k + 1) = 0.0;
        }
        PHT_QZ_SYNC();
      }
      // zero T[k+1][k]
      qzr_house(2, Tt(k + 1, k + 1), Tt(k + 1, k), 0.0, tau, w1, w2, bet);
      PHT_QZ_SYNC();
      qzr_right<2>(H, hr1, T, k + 1, ifirst, ld, k, tau, w1, w2, L);
      PHT_QZ_SYNC();
      if (L.lane == 0) Tt(k + 1, k) = 0.0;
      PHT_QZ_SYNC();
      if (k + 1 < ilast) {
        x0 = Hh(k + 1, k);
        x1 = Hh(k + 2, k);
        x2 = k + 3 <= ilast ? Hh(k + 3, k) : 0.0;
      }
    }
  }
  return 0;
#undef Hh
#undef Tt
}

}  // namespace pht
