// paraht_internal.cuh -- shared device helpers and launch geometry for the ParaHT GB300 library.
//
// Conventions
//   * Matrices are column-major FP64 with a leading dimension (as in the reference, whose
//     arrays are Fortran A(lda,*)).  Device code uses 0-based indices; comments that cite the
//     reference use its 1-based indices.
//   * A compact-WY "op" is one block reflector H = I - V T V^T with V stored column-wise and
//     explicitly (unit diagonal and the zeros above it are stored), T k x k.  Left ops apply
//     H^T from the left to a row range of a matrix (dlarfb 'L','T'); right ops apply H from the
//     right to a column range (dlarfb 'R','N').  Row-wise reflectors (LQ/RQ) are stored
//     transposed so that they are column-wise too.
//   * Every bulk update of both stages is a sequence of such ops applied in a fixed order; the
//     order matters where ops overlap and follows the reference's loop order.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#define PHT_DEV __device__ __forceinline__

namespace pht {

constexpr int kWarp = 32;

// Raises a kernel's dynamic shared-memory limit on the current device to at least `bytes`
// (PARAHT_ERR_CUDA when refused).  The limit is one value per kernel and device, shared by every
// context, thread and captured graph, so it only ever grows: a call with smaller tiles never takes
// away the room another call's launch in flight was shaped for.  (api.cu)
int smem_at_least(const void* func, size_t bytes);

// The same for a kernel whose shared memory is fixed, on launch paths: after the first grant on a
// device (bit d of `done`) it costs one cudaGetDevice.  A refusal leaves the bit clear; the launch
// that follows then fails and its error reaches the caller through the stream checks.
inline void smem_once(const void* func, size_t bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return;
  if (smem_at_least(func, bytes) == 0) done.fetch_or(bit, std::memory_order_acq_rel);
}

// ---------------------------------------------------------------------------------------
// CTA-wide sum of one double per thread; every thread receives the total.
// `red` must hold at least blockDim.x/32 doubles of shared memory.
// ---------------------------------------------------------------------------------------
PHT_DEV double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

PHT_DEV double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();  // red may still be read by a previous call
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = (l < nw) ? red[l] : 0.0;
  s = warp_sum(s);
  return s;
}

// Householder generation with the semantics of LAPACK DLARFG: given alpha and the squared norm
// of x, returns tau and the scale factor 1/(alpha-beta) for x; beta replaces alpha.
// Computed redundantly by every thread from identical inputs (bitwise identical results), so no
// broadcast is needed.  tau = 0 (identity) when x == 0, as in DLARFG.
//
// The scalars are formed from one reciprocal square root and one reciprocal, because every
// dependent FP64 instruction costs about 64 cycles on GB300 and this sits on the critical path
// of every chain:  s = alpha^2 + |x|^2,  rho = 1/sqrt(s),  |beta| = s*rho,
//   tau  = (beta - alpha)/beta = 1 + |alpha| rho,
//   scal = 1/(alpha - beta)    = sign(alpha) / (|alpha| + |beta|).
// Unlike DLARFG there is no rescaling loop for |beta| below the safe minimum: entries smaller
// than about 1e-154 (whose squares underflow) are treated as zero.
struct Reflector {
  double tau, scal, beta;
};
PHT_DEV Reflector make_reflector(double alpha, double xnorm2) {
  Reflector h;
  if (xnorm2 == 0.0) {
    h.tau = 0.0;
    h.scal = 1.0;
    h.beta = alpha;
    return h;
  }
  const double s = fma(alpha, alpha, xnorm2);
  const double rho = rsqrt(s);
  const double nrm = s * rho;
  const double aa = fabs(alpha);
  h.beta = -copysign(nrm, alpha);
  h.tau = fma(aa, rho, 1.0);
  h.scal = copysign(1.0 / (aa + nrm), alpha);
  return h;
}

// The same scalars without branches, for the latency-bound factorisation chains: the reciprocal
// square root and the reciprocal come from the hardware approximations (PTX rsqrt.approx.ftz.f64,
// rcp.approx.ftz.f64) refined by two Newton-Raphson steps each (y += y (1 - x y^2) / 2 and
// y += y (1 - x y); each step doubles the correct bits), so the compiler can interleave them
// with independent work (a shuffle reduction) instead of branching into library code.  Within a
// few ulps of make_reflector's values; tau = 0, scal = 1, beta = alpha when xnorm2 == 0.
PHT_DEV double rsqrt_seed(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return y;
}
PHT_DEV double rcp_seed(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return y;
}
PHT_DEV Reflector make_reflector_nr(double alpha, double xnorm2) {
  const double s = fma(alpha, alpha, xnorm2);
  double rho = rsqrt_seed(s);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double e = fma(-s * rho, rho, 1.0);
    rho = fma(0.5 * rho, e, rho);
  }
  const double nrm = s * rho, aa = fabs(alpha);
  const double den = aa + nrm;
  double inv = rcp_seed(den);
#pragma unroll
  for (int it = 0; it < 2; ++it) inv = fma(inv, fma(-den, inv, 1.0), inv);
  const bool zero = xnorm2 == 0.0;
  Reflector h;
  h.tau = zero ? 0.0 : fma(aa, rho, 1.0);
  h.scal = zero ? 1.0 : copysign(inv, alpha);
  h.beta = zero ? alpha : -copysign(nrm, alpha);
  return h;
}

// ---------------------------------------------------------------------------------------
// Compact-WY op descriptors.
// ---------------------------------------------------------------------------------------
struct WYOp {
  int start;  // first row (left op) / first column (right op) of the reflector span
  int len;    // length of the span (rows of V)
  int k;      // number of reflectors (columns of V)
  int lo;     // first column (left op) / first row (right op) that the op touches
  int hi;     // last column (left op) / last row (right op), inclusive
  const double* V;  // len x k, column-major, leading dimension ldv
  int ldv;
  const double* T;  // k x k, column-major, leading dimension ldt
  int ldt;
  // dense = 1: the op is C <- C G (right) / C <- G^T C (left) for an accumulated orthogonal
  // len x len block G (the Givens stage 2); it is stored as V = I (len x len) and T = I - G
  // (k = len), the same product C - C V T V^T, and its algorithmic work is 2 len^2 flops per
  // row instead of 4 len k
  int dense = 0;
};

// Algorithmic flops of an op per strip row (per column for left ops).
PHT_DEV unsigned long long op_row_flops(const WYOp& w) {
  return w.dense ? 2ull * (unsigned long long)w.len * (unsigned long long)w.len
                 : 4ull * (unsigned long long)w.len * (unsigned long long)w.k;
}

}  // namespace pht

// Status word written by device code (bounded waits, argument checks).
struct PhtDeviceStatus {
  int code;
  int where;
};
