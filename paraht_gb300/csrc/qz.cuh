// qz.cuh -- generalized eigenvalues of a Hessenberg-triangular pencil (H, T) by the QZ iteration
// (Moler and Stewart 1973), the step after the reduction (the reference's driver hands the
// reduced pencil to LAPACK, src/profilereduction.f90:156; DHGEQZ is the QZ that follows DGGHD3).
//
// This is the complex single-shift form: the pencil is copied to complex arithmetic, every sweep
// chases one bulge with complex Givens rotations from the left (rows) and the right (columns), and
// 1 x 1 blocks deflate at the bottom.  The shift is the eigenvalue of the trailing 2 x 2 pencil
// nearest to its last diagonal ratio (Wilkinson), with an exceptional shift every 10 sweeps
// without deflation.  Only eigenvalues are computed, so every rotation touches the active block
// alone.  At most 30 n sweeps.  A diagonal entry of T below eps ||T||_F (an infinite or nearly
// infinite eigenvalue) is reported as unsupported.
//
// The core is written once for the host and the device: `QzLanes` distributes the row/column
// loops over the lanes of one warp on the device (lane, nlanes = 32) and runs them in one thread
// on the host (0, 1); every lane computes the same rotation from the same (synchronised) values.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pht {

struct QzC {
  double re, im;
};
__host__ __device__ inline QzC qz_c(double r, double i = 0.0) { return QzC{r, i}; }
__host__ __device__ inline QzC operator+(QzC a, QzC b) { return QzC{a.re + b.re, a.im + b.im}; }
__host__ __device__ inline QzC operator-(QzC a, QzC b) { return QzC{a.re - b.re, a.im - b.im}; }
__host__ __device__ inline QzC operator*(QzC a, QzC b) { return QzC{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ inline QzC operator*(double s, QzC a) { return QzC{s * a.re, s * a.im}; }
__host__ __device__ inline QzC qz_conj(QzC a) { return QzC{a.re, -a.im}; }
__host__ __device__ inline double qz_abs(QzC a) { return hypot(a.re, a.im); }
__host__ __device__ inline double qz_abs1(QzC a) { return fabs(a.re) + fabs(a.im); }
__host__ __device__ inline QzC qz_div(QzC a, QzC b) {  // a / b, scaled (Smith's method)
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return QzC{(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  const double r = b.re / b.im, d = b.im + b.re * r;
  return QzC{(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
__host__ __device__ inline QzC qz_sqrt(QzC a) {  // principal square root
  const double m = qz_abs(a);
  if (m == 0.0) return qz_c(0.0);
  const double t = sqrt(0.5 * (m + fabs(a.re)));
  if (a.re >= 0.0) return QzC{t, a.im / (2.0 * t)};
  return QzC{fabs(a.im) / (2.0 * t), a.im >= 0.0 ? t : -t};
}

// Complex Givens rotation: c real, s complex with  c f + s g = r,  -conj(s) f + c g = 0.
__host__ __device__ inline void qz_rot(QzC f, QzC g, double& c, QzC& s, QzC& r) {
  const double af = qz_abs(f), ag = qz_abs(g);
  if (ag == 0.0) {
    c = 1.0;
    s = qz_c(0.0);
    r = f;
    return;
  }
  if (af == 0.0) {
    c = 0.0;
    s = (1.0 / ag) * qz_conj(g);
    r = qz_c(ag);
    return;
  }
  const double nrm = hypot(af, ag);
  const QzC ph = (1.0 / af) * f;  // f / |f|
  c = af / nrm;
  s = (1.0 / nrm) * (ph * qz_conj(g));
  r = nrm * ph;
}

struct QzLanes {
  int lane, n;
};

#ifndef PHT_QZ_SYNC
#ifdef __CUDA_ARCH__
#define PHT_QZ_SYNC() __syncwarp()
#else
#define PHT_QZ_SYNC() ((void)0)
#endif
#endif

// rows i, i+1 of X (ld x) over columns [c0, c1]:  x_i <- c x_i + s x_{i+1},  x_{i+1} <- -conj(s) x_i + c x_{i+1}
__host__ __device__ inline void qz_rows(QzC* X, int ldx, int i, int c0, int c1, double c, QzC s, QzLanes L) {
  for (int k = c0 + L.lane; k <= c1; k += L.n) {
    QzC* col = X + (size_t)k * ldx;
    const QzC x = col[i], y = col[i + 1];
    col[i] = c * x + s * y;
    col[i + 1] = c * y - qz_conj(s) * x;
  }
}
// columns j, j+1 of X over rows [r0, r1] with the rotation that zeroes X[k][j] from (f = X[k][j+1],
// g = X[k][j]):  x_{j+1} <- c x_{j+1} + s x_j,  x_j <- -conj(s) x_{j+1} + c x_j
__host__ __device__ inline void qz_cols(QzC* X, int ldx, int j, int r0, int r1, double c, QzC s, QzLanes L) {
  QzC* a = X + (size_t)j * ldx;
  QzC* b = X + (size_t)(j + 1) * ldx;
  for (int k = r0 + L.lane; k <= r1; k += L.n) {
    const QzC x = b[k], y = a[k];
    b[k] = c * x + s * y;
    a[k] = c * y - qz_conj(s) * x;
  }
}

// Eigenvalue of the 2 x 2 pencil (A, B) (B upper triangular, nonsingular) nearest to
// A[1][1] / B[1][1]: the eigenvalues of M = A B^-1.
__host__ __device__ inline QzC qz_shift(QzC a00, QzC a01, QzC a10, QzC a11, QzC b00, QzC b01, QzC b11) {
  // B^-1 = [[1/b00, -b01/(b00 b11)], [0, 1/b11]]
  const QzC i00 = qz_div(qz_c(1.0), b00), i11 = qz_div(qz_c(1.0), b11);
  const QzC i01 = qz_c(0.0) - (i00 * b01 * i11);
  const QzC m00 = a00 * i00, m01 = a00 * i01 + a01 * i11;
  const QzC m10 = a10 * i00, m11 = a10 * i01 + a11 * i11;
  const QzC tr = m00 + m11, det = m00 * m11 - m01 * m10;
  const QzC half = 0.5 * tr;
  const QzC disc = qz_sqrt(half * half - det);
  const QzC l1 = half + disc, l2 = half - disc;
  return qz_abs(l1 - m11) <= qz_abs(l2 - m11) ? l1 : l2;
}

// Eigenvalues alpha[j] / beta[j] of the pencil held in H, T (complex, column-major, leading
// dimension ld, H upper Hessenberg, T upper triangular; both overwritten).  Returns 0, 1 when a
// diagonal entry of T is negligible (unsupported here), 2 when 30 n sweeps did not converge.
__host__ __device__ inline int qz_eigs(int n, QzC* H, QzC* T, int ld, QzC* alpha, QzC* beta, QzLanes L) {
#define Hh(i, j) H[(size_t)(j) * ld + (i)]
#define Tt(i, j) T[(size_t)(j) * ld + (i)]
  const double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
  double hn = 0.0, tn = 0.0;  // Frobenius norms, each lane's share summed serially by every lane
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= (j + 1 < n ? j + 1 : j); ++i) {
      const double ha = qz_abs(Hh(i, j));
      hn += ha * ha;
      if (i <= j) {
        const double ta = qz_abs(Tt(i, j));
        tn += ta * ta;
      }
    }
  const double atol = fmax(tiny, eps * sqrt(hn)), btol = fmax(tiny, eps * sqrt(tn));
  for (int j = 0; j < n; ++j)
    if (qz_abs(Tt(j, j)) <= btol) return 1;
  int ilast = n - 1, iter = 0, total = 0;
  const int maxit = 30 * (n > 1 ? n : 1);
  while (ilast >= 0) {
    if (ilast == 0) {
      alpha[0] = Hh(0, 0);
      beta[0] = Tt(0, 0);
      break;
    }
    // deflation at the bottom
    const double sub = qz_abs(Hh(ilast, ilast - 1));
    if (sub <= fmax(atol, eps * (qz_abs(Hh(ilast, ilast)) + qz_abs(Hh(ilast - 1, ilast - 1))))) {
      PHT_QZ_SYNC();
      if (L.lane == 0) Hh(ilast, ilast - 1) = qz_c(0.0);
      alpha[ilast] = Hh(ilast, ilast);
      beta[ilast] = Tt(ilast, ilast);
      --ilast;
      iter = 0;
      PHT_QZ_SYNC();
      continue;
    }
    // the active block [ifirst, ilast]: up to a negligible subdiagonal
    int ifirst = ilast - 1;
    while (ifirst > 0) {
      const double s2 = qz_abs(Hh(ifirst, ifirst - 1));
      if (s2 <= fmax(atol, eps * (qz_abs(Hh(ifirst, ifirst)) + qz_abs(Hh(ifirst - 1, ifirst - 1))))) break;
      --ifirst;
    }
    PHT_QZ_SYNC();
    if (ifirst > 0 && L.lane == 0) Hh(ifirst, ifirst - 1) = qz_c(0.0);
    PHT_QZ_SYNC();
    for (int j = ifirst; j <= ilast; ++j)
      if (qz_abs(Tt(j, j)) <= btol) return 1;
    if (++total > maxit) return 2;
    ++iter;
    // shift: Wilkinson from the trailing 2 x 2, exceptional every 10 sweeps without deflation
    QzC shift;
    if (iter % 10 == 0) {
      const QzC r = qz_div(Hh(ilast, ilast), Tt(ilast, ilast));
      shift = r + (0.75 * qz_abs(Hh(ilast, ilast - 1)) / fmax(qz_abs(Tt(ilast - 1, ilast - 1)), tiny)) * qz_c(1.0, 0.5);
    } else {
      shift = qz_shift(Hh(ilast - 1, ilast - 1), Hh(ilast - 1, ilast), Hh(ilast, ilast - 1), Hh(ilast, ilast),
                       Tt(ilast - 1, ilast - 1), Tt(ilast - 1, ilast), Tt(ilast, ilast));
    }
    // one sweep: the bulge from (H - shift T) e_ifirst chased to the bottom of the block
    QzC x = Hh(ifirst, ifirst) - shift * Tt(ifirst, ifirst), y = Hh(ifirst + 1, ifirst);
    for (int j = ifirst; j < ilast; ++j) {
      double c;
      QzC s, r;
      qz_rot(x, y, c, s, r);
      PHT_QZ_SYNC();
      const int c0 = j > ifirst ? j - 1 : j;
      qz_rows(H, ld, j, c0, ilast, c, s, L);
      qz_rows(T, ld, j, j, ilast, c, s, L);
      PHT_QZ_SYNC();
      if (j > ifirst && L.lane == 0) Hh(j + 1, j - 1) = qz_c(0.0);  // the bulge, zero by construction
      PHT_QZ_SYNC();
      // T gained T[j+1][j]: remove it with a rotation of columns j, j+1
      double c2;
      QzC s2, r2;
      qz_rot(Tt(j + 1, j + 1), Tt(j + 1, j), c2, s2, r2);
      PHT_QZ_SYNC();
      const int hr1 = j + 2 < ilast ? j + 2 : ilast;
      qz_cols(H, ld, j, ifirst, hr1, c2, s2, L);
      qz_cols(T, ld, j, ifirst, j + 1, c2, s2, L);
      PHT_QZ_SYNC();
      if (L.lane == 0) Tt(j + 1, j) = qz_c(0.0);
      PHT_QZ_SYNC();
      if (j + 1 < ilast) {
        x = Hh(j + 1, j);
        y = Hh(j + 2, j);
      }
    }
  }
  return 0;
#undef Hh
#undef Tt
}

}  // namespace pht

namespace pht {

// One pencil of a batched eigenvalue call: real H, T (device, column-major), the outputs, and the
// offset of its complex scratch (H, T, alpha, beta: qz_work_elems(n) entries) in the call's buffer.
struct QzPencil {
  const double* H;
  const double* T;
  double* alphar;
  double* alphai;
  double* beta;
  long long off;
  int n, ldh, ldt, pad;
};
inline long long qz_work_elems(int n) { return 2ll * n * n + 2ll * n; }
// One warp per pencil on stream s; info[i] receives qz_eigs's status for pencil i.
void launch_qz_eigs(cudaStream_t s, const QzPencil* P, int count, QzC* work, int* info);

}  // namespace pht
