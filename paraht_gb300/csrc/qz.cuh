// qz.cuh -- the lane protocol and the batch layout of the GPU QZ iteration (qz_real.cuh holds the
// real double-shift core, qz.cu the batched kernel): the step after the reduction, the
// eigenvalues of the reduced pencil (the reference's driver stops at it,
// src/profilereduction.f90:156; LAPACK DHGEQZ is the QZ that follows DGGHD3).
//
// The core is written once for the host and the device: `QzLanes` distributes its row and column
// passes over the lanes of one warp or one CTA on the device (lane, nlanes = 32 or the CTA's
// size) and runs them in one thread on the host (0, 1); every lane computes the same reflectors
// from the same (synchronised) values, so control flow is uniform over the lanes.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pht {

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
// warp w.  Measured on GB300 (with the complex single-shift core the kernel ran first) against
// four-warp CTAs and one warp per pencil: 967, 797 and 893 pencils/s on 1216 pencils n ~ U{32..256}.
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
