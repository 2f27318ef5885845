// qz.cuh -- generalized eigenvalues of a Hessenberg-triangular pencil (H, T) by the QZ iteration
// (Moler and Stewart 1973), the step after the reduction (the reference's driver hands the
// reduced pencil to LAPACK, src/profilereduction.f90:156; DHGEQZ is the QZ that follows DGGHD3).
//
// This is the complex single-shift form: the pencil is copied to complex arithmetic, every sweep
// chases one bulge with complex Givens rotations from the left (rows) and the right (columns), and
// 1 x 1 blocks deflate at the bottom.  H and T are first scaled by powers of two (exact) to largest
// moduli in [1/2, 1), so pencils near the overflow or underflow thresholds converge like others.
// The shift is the eigenvalue of the trailing 2 x 2 pencil nearest to its last diagonal ratio
// (Wilkinson), with an exceptional shift every 10 sweeps without deflation.  Only eigenvalues are computed, so every rotation touches the active block
// alone.  At most 30 n sweeps.  A diagonal entry of T below eps ||T||_F (an infinite or nearly
// infinite eigenvalue) is reported as unsupported.
//
// The core is written once for the host and the device: `QzLanes` distributes the row/column
// loops over the lanes of one warp or one CTA on the device (lane, nlanes = 32 or the CTA's size)
// and runs them in one thread on the host (0, 1); every lane computes the same rotation from the
// same (synchronised) values, so control flow is uniform over the lanes.
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

__host__ __device__ inline double qz_rsqrt(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

// Complex Givens rotation: c real, s complex with  c f + s g = r,  -conj(s) f + c g = 0.
// Squared moduli and reciprocal square roots where no square can overflow or underflow; hypot
// (scaled) otherwise.
__host__ __device__ inline void qz_rot(QzC f, QzC g, double& c, QzC& s, QzC& r) {
  const bool fz = f.re == 0.0 && f.im == 0.0, gz = g.re == 0.0 && g.im == 0.0;
  if (gz) {
    c = 1.0;
    s = qz_c(0.0);
    r = f;
    return;
  }
  const double f2 = f.re * f.re + f.im * f.im, g2 = g.re * g.re + g.im * g.im;
  const double lo = 1e-290, hi = 1e290;
  if ((fz || (f2 > lo && f2 < hi)) && g2 > lo && g2 < hi) {
    if (fz) {
      const double rg = qz_rsqrt(g2);
      c = 0.0;
      s = rg * qz_conj(g);
      r = qz_c(g2 * rg);
      return;
    }
    const double h2 = f2 + g2, rf = qz_rsqrt(f2), rh = qz_rsqrt(h2);
    const QzC ph = rf * f;  // f / |f|
    c = f2 * rf * rh;       // |f| / sqrt(|f|^2 + |g|^2)
    s = rh * (ph * qz_conj(g));
    r = (h2 * rh) * ph;
    return;
  }
  const double af = qz_abs(f), ag = qz_abs(g);
  if (af == 0.0) {
    c = 0.0;
    s = (1.0 / ag) * qz_conj(g);
    r = qz_c(ag);
    return;
  }
  const double nrm = hypot(af, ag);
  const QzC ph = (1.0 / af) * f;
  c = af / nrm;
  s = (1.0 / nrm) * (ph * qz_conj(g));
  r = nrm * ph;
}

struct QzLanes {
  int lane, n;
};

// The lanes of one pencil: one warp (n = 32) or one whole CTA (n = blockDim.x, a multiple of 32).
__host__ __device__ inline void qz_sync(const QzLanes& L) {
#ifdef __CUDA_ARCH__
  if (L.n > 32)
    __syncthreads();
  else
    __syncwarp();
#endif
}
// Largest v over the lanes, the same on every lane.
__host__ __device__ inline int qz_lane_max(int v, const QzLanes& L) {
#ifdef __CUDA_ARCH__
  int m = __reduce_max_sync(0xffffffffu, v);
  if (L.n > 32) {
    __shared__ int red[32];
    __syncthreads();  // the previous call's readers are done
    if ((L.lane & 31) == 0) red[L.lane >> 5] = m;
    __syncthreads();
    m = red[0];
    for (int w = 1; w < (L.n >> 5); ++w) m = red[w] > m ? red[w] : m;
  }
  return m;
#else
  return v;
#endif
}
#ifndef PHT_QZ_SYNC
#define PHT_QZ_SYNC() qz_sync(L)
#endif
#ifndef PHT_QZ_LANE_MAX
#define PHT_QZ_LANE_MAX(v) qz_lane_max((v), L)
#endif

// Elements a lane loads before it stores any: the row and column passes are chains of round trips
// to L2 otherwise (a pencil's complex copies are far larger than L1).
constexpr int kQzBatch = 4;

// One rotation of rows i, i+1 over columns [a0, c1] of A and [b0, c1] of B (leading dimension ld):
// x_i <- c x_i + s x_{i+1},  x_{i+1} <- -conj(s) x_i + c x_{i+1}.  The two ranges form one index
// space that the lanes share, kQzBatch elements in flight per lane.
__host__ __device__ inline void qz_rows(QzC* A, int a0, QzC* B, int b0, int c1, int ld, int i, double c, QzC s,
                                        QzLanes L) {
  const int na = c1 - a0 + 1, tot = na + (c1 - b0 + 1);
  for (int t0 = L.lane; t0 < tot; t0 += kQzBatch * L.n) {
    QzC* p[kQzBatch];
    QzC x[kQzBatch], y[kQzBatch];
#pragma unroll
    for (int u = 0; u < kQzBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        p[u] = (t < na ? A + (size_t)(a0 + t) * ld : B + (size_t)(b0 + t - na) * ld) + i;
        x[u] = p[u][0];
        y[u] = p[u][1];
      }
    }
#pragma unroll
    for (int u = 0; u < kQzBatch; ++u)
      if (t0 + u * L.n < tot) {
        p[u][0] = c * x[u] + s * y[u];
        p[u][1] = c * y[u] - qz_conj(s) * x[u];
      }
  }
}
// One rotation of columns j, j+1 over rows [r0, a1] of A and [r0, b1] of B, the one that zeroes
// an entry X[k][j] from (f = X[k][j+1], g = X[k][j]):  x_{j+1} <- c x_{j+1} + s x_j,
// x_j <- -conj(s) x_{j+1} + c x_j.
__host__ __device__ inline void qz_cols(QzC* A, int a1, QzC* B, int b1, int r0, int ld, int j, double c, QzC s,
                                        QzLanes L) {
  const int na = a1 - r0 + 1, tot = na + (b1 - r0 + 1);
  for (int t0 = L.lane; t0 < tot; t0 += kQzBatch * L.n) {
    QzC* p[kQzBatch];
    QzC x[kQzBatch], y[kQzBatch];
#pragma unroll
    for (int u = 0; u < kQzBatch; ++u) {
      const int t = t0 + u * L.n;
      if (t < tot) {
        p[u] = (t < na ? A + r0 + t : B + r0 + t - na) + (size_t)j * ld;
        x[u] = p[u][ld];
        y[u] = p[u][0];
      }
    }
#pragma unroll
    for (int u = 0; u < kQzBatch; ++u)
      if (t0 + u * L.n < tot) {
        p[u][ld] = c * x[u] + s * y[u];
        p[u][0] = c * y[u] - qz_conj(s) * x[u];
      }
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
  // Frobenius norms, scaled by the largest modulus so that no square overflows or underflows;
  // every lane sums all entries in the same order and gets the same value
  double hmax = 0.0, tmax = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= (j + 1 < n ? j + 1 : j); ++i) {
      hmax = fmax(hmax, qz_abs(Hh(i, j)));
      if (i <= j) tmax = fmax(tmax, qz_abs(Tt(i, j)));
    }
  double hs = 0.0, ts = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= (j + 1 < n ? j + 1 : j); ++i) {
      if (hmax > 0.0) {
        const double ha = qz_abs(Hh(i, j)) / hmax;
        hs += ha * ha;
      }
      if (i <= j && tmax > 0.0) {
        const double ta = qz_abs(Tt(i, j)) / tmax;
        ts += ta * ta;
      }
    }
  // H and T scaled by powers of two (exact) to largest moduli in [1/2, 1): entries near the
  // underflow threshold keep their precision and the tolerances below stay far above it
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
  for (int j = 0; j < n; ++j)
    if (qz_abs(Tt(j, j)) <= btol) return 1;
  int ilast = n - 1, iter = 0, total = 0;
  const int maxit = 30 * (n > 1 ? n : 1);
  while (ilast >= 0) {
    if (ilast == 0) {
      alpha[0] = uh * Hh(0, 0);
      beta[0] = ut * Tt(0, 0);
      break;
    }
    // deflation at the bottom
    const double sub = qz_abs(Hh(ilast, ilast - 1));
    if (sub <= fmax(atol, eps * (qz_abs(Hh(ilast, ilast)) + qz_abs(Hh(ilast - 1, ilast - 1))))) {
      PHT_QZ_SYNC();
      if (L.lane == 0) Hh(ilast, ilast - 1) = qz_c(0.0);
      alpha[ilast] = uh * Hh(ilast, ilast);
      beta[ilast] = ut * Tt(ilast, ilast);
      --ilast;
      iter = 0;
      PHT_QZ_SYNC();
      continue;
    }
    // the active block [ifirst, ilast]: from the last negligible subdiagonal entry above ilast
    // (every lane tests its share of the positions)
    int cand = 0;
    for (int i = 1 + L.lane; i < ilast; i += L.n)
      if (qz_abs(Hh(i, i - 1)) <= fmax(atol, eps * (qz_abs(Hh(i, i)) + qz_abs(Hh(i - 1, i - 1))))) cand = i;
    const int ifirst = PHT_QZ_LANE_MAX(cand);
    PHT_QZ_SYNC();
    if (ifirst > 0 && L.lane == 0) Hh(ifirst, ifirst - 1) = qz_c(0.0);
    PHT_QZ_SYNC();
    int tiny_t = 0;
    for (int j = ifirst + L.lane; j <= ilast; j += L.n)
      if (qz_abs(Tt(j, j)) <= btol) tiny_t = 1;
    if (PHT_QZ_LANE_MAX(tiny_t)) return 1;
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
      qz_rows(H, j > ifirst ? j - 1 : j, T, j, ilast, ld, j, c, s, L);
      PHT_QZ_SYNC();
      if (j > ifirst && L.lane == 0) Hh(j + 1, j - 1) = qz_c(0.0);  // the bulge, zero by construction
      PHT_QZ_SYNC();
      // T gained T[j+1][j]: remove it with a rotation of columns j, j+1
      double c2;
      QzC s2, r2;
      qz_rot(Tt(j + 1, j + 1), Tt(j + 1, j), c2, s2, r2);
      PHT_QZ_SYNC();
      qz_cols(H, j + 2 < ilast ? j + 2 : ilast, T, j + 1, ifirst, ld, j, c2, s2, L);
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

// One pencil of a batched eigenvalue call (the kernel in qz.cu runs the real double-shift core of
// qz_real.cuh on it): real H, T (device, column-major), the outputs, and the offset of its scratch
// (copies of H and T: qz_work_elems(n) doubles) in the call's buffer.
struct QzPencil {
  const double* H;
  const double* T;
  double* alphar;
  double* alphai;
  double* beta;
  long long off;
  int n, ldh, ldt, pad;
};
inline long long qz_work_elems(int n) { return 2ll * n * n; }
// A CTA of kQzThreads threads runs either one pencil of n >= kQzWholeMin on both its warps (the
// row and column passes on two of the SM's schedulers) or two smaller pencils, one per warp;
// kQzMinBlocks CTAs fit on an SM (at most 168 registers a thread).  pencil[w] < 0: no pencil for
// warp w.  Measured on GB300 with the complex single-shift core against four-warp CTAs and one
// warp per pencil: 967, 797 and 893 pencils/s on 1216 pencils n ~ U{32..256}.
constexpr int kQzThreads = 64;
constexpr int kQzMinBlocks = 6;
constexpr int kQzWholeMin = 128;
struct QzBlock {
  int pencil[4];
  int whole;
};
static_assert(kQzThreads % 32 == 0 && kQzThreads / 32 <= 4, "a CTA holds at most four warps' pencils");
// One CTA per block entry on stream s; info[i] receives qz_eigs's status for pencil i.
void launch_qz_eigs(cudaStream_t s, const QzPencil* P, const QzBlock* blocks, int nblocks, double* work, int* info);

}  // namespace pht
