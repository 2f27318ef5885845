// qz.cu -- the batched eigenvalue kernel around the QZ core in qz.cuh: one warp per pencil.
#include <cuda_runtime.h>

#include "launch_count.h"
#include "qz.cuh"

namespace pht {

constexpr int kQzWarps = 4;  // pencils per block: one warp on each of an SM's four schedulers

__global__ void __launch_bounds__(32 * kQzWarps) k_qz_eigs(const QzPencil* __restrict__ P, int count,
                                                         QzC* __restrict__ work, int* __restrict__ info) {
  const int w = blockIdx.x * kQzWarps + (int)(threadIdx.x >> 5);
  if (w >= count) return;  // the whole warp leaves together
  const int lane = threadIdx.x & 31;
  const QzPencil p = P[w];
  const int n = p.n;
  QzC* H = work + p.off;
  QzC* T = H + (size_t)n * n;
  QzC* alpha = T + (size_t)n * n;
  QzC* beta = alpha + n;
  // complex copies, zero below the Hessenberg / triangular structure
  for (long long e = lane; e < (long long)n * n; e += 32) {
    const int j = (int)(e / n), i = (int)(e % n);
    H[e] = qz_c(i <= j + 1 ? p.H[(size_t)j * p.ldh + i] : 0.0);
    T[e] = qz_c(i <= j ? p.T[(size_t)j * p.ldt + i] : 0.0);
  }
  __syncwarp();
  const int rc = qz_eigs(n, H, T, n, alpha, beta, QzLanes{lane, 32});
  __syncwarp();
  if (rc == 0) {
    // beta real and nonnegative: (alpha, beta) <- (alpha conj(beta) / |beta|, |beta|)
    for (int j = lane; j < n; j += 32) {
      const QzC b = beta[j];
      const double m = qz_abs(b);
      const QzC a = (1.0 / m) * (alpha[j] * qz_conj(b));
      p.alphar[j] = a.re;
      p.alphai[j] = a.im;
      p.beta[j] = m;
    }
  }
  if (lane == 0) info[w] = rc;
}

void launch_qz_eigs(cudaStream_t s, const QzPencil* P, int count, QzC* work, int* info) {
  if (count <= 0) return;
  count_launch();
  k_qz_eigs<<<(count + kQzWarps - 1) / kQzWarps, 32 * kQzWarps, 0, s>>>(P, count, work, info);
}

}  // namespace pht
