// qz.cu -- the batched eigenvalue kernel around the QZ core in qz.cuh: a small pencil per warp, a
// large pencil per CTA.
#include <cuda_runtime.h>

#include "launch_count.h"
#include "qz.cuh"

namespace pht {

__device__ void qz_pencil(const QzPencil& p, QzC* work, int* info, int idx, QzLanes L) {
  const int n = p.n;
  QzC* H = work + p.off;
  QzC* T = H + (size_t)n * n;
  QzC* alpha = T + (size_t)n * n;
  QzC* beta = alpha + n;
  // complex copies, zero below the Hessenberg / triangular structure
  for (long long e = L.lane; e < (long long)n * n; e += L.n) {
    const int j = (int)(e / n), i = (int)(e % n);
    H[e] = qz_c(i <= j + 1 ? p.H[(size_t)j * p.ldh + i] : 0.0);
    T[e] = qz_c(i <= j ? p.T[(size_t)j * p.ldt + i] : 0.0);
  }
  qz_sync(L);
  const int rc = qz_eigs(n, H, T, n, alpha, beta, L);
  qz_sync(L);
  if (rc == 0) {
    // beta real and nonnegative: (alpha, beta) <- (alpha conj(beta) / |beta|, |beta|)
    for (int j = L.lane; j < n; j += L.n) {
      const QzC b = beta[j];
      const double m = qz_abs(b);
      const QzC a = alpha[j] * ((1.0 / m) * qz_conj(b));  // the unit phase first: no overflow
      p.alphar[j] = a.re;
      p.alphai[j] = a.im;
      p.beta[j] = m;
    }
  }
  if (L.lane == 0) info[idx] = rc;
}

__global__ void __launch_bounds__(kQzThreads, kQzMinBlocks) k_qz_eigs(const QzPencil* __restrict__ P,
                                                        const QzBlock* __restrict__ blocks, QzC* __restrict__ work,
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

void launch_qz_eigs(cudaStream_t s, const QzPencil* P, const QzBlock* blocks, int nblocks, QzC* work, int* info) {
  if (nblocks <= 0) return;
  count_launch();
  k_qz_eigs<<<nblocks, kQzThreads, 0, s>>>(P, blocks, work, info);
}

}  // namespace pht
