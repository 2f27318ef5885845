// qz.cu -- the batched eigenvalue kernel around the real double-shift QZ core (qz_real.cuh): a
// small pencil per warp, a large pencil per CTA.
#include <cuda_runtime.h>

#include "launch_count.h"
#include "qz_real.cuh"

namespace pht {

__device__ void qz_pencil(const QzPencil& p, double* work, int* info, int idx, QzLanes L) {
  const int n = p.n;
  double* H = work + p.off;
  double* T = H + (size_t)n * n;
  // copies, zero below the Hessenberg / triangular structure
  for (long long e = L.lane; e < (long long)n * n; e += L.n) {
    const int j = (int)(e / n), i = (int)(e % n);
    H[e] = i <= j + 1 ? p.H[(size_t)j * p.ldh + i] : 0.0;
    T[e] = i <= j ? p.T[(size_t)j * p.ldt + i] : 0.0;
  }
  qz_sync(L);
  const int rc = qz_real_eigs(n, H, T, n, p.alphar, p.alphai, p.beta, L);
  if (L.lane == 0) info[idx] = rc;
}

__global__ void __launch_bounds__(kQzThreads, kQzMinBlocks) k_qz_eigs(const QzPencil* __restrict__ P,
                                                                      const QzBlock* __restrict__ blocks,
                                                                      double* __restrict__ work,
                                                                      int* __restrict__ info) {
  const QzBlock b = blocks[blockIdx.x];
  if (b.whole) {  // every thread of the CTA: the branch is uniform over the block
    qz_pencil(P[b.pencil[0]], work, info, b.pencil[0], QzLanes{(int)threadIdx.x, kQzThreads});
    return;
  }
  const int w = (int)(threadIdx.x >> 5);
  const int idx = b.pencil[w];
  if (idx < 0) return;  // the whole warp leaves together; warps of this kind never sync the CTA
  qz_pencil(P[idx], work, info, idx, QzLanes{(int)(threadIdx.x & 31), 32});
}

void launch_qz_eigs(cudaStream_t s, const QzPencil* P, const QzBlock* blocks, int nblocks, double* work, int* info) {
  if (nblocks <= 0) return;
  count_launch();
  k_qz_eigs<<<nblocks, kQzThreads, 0, s>>>(P, blocks, work, info);
}

}  // namespace pht
