// gemm.cu -- FP64 GEMM for the off-diagonal updates of the DGGHD3-compatible entry
// (paraht_gghd3_d): the reduction of the diagonal block rows/columns ilo..ihi produces Q_s and
// Z_s, which then act on the rows above the block, the columns right of it and on Q, Z.
//
// Out (M x N, column-major, ld ldo) = op(X) Y with op(X) = X (M x K, ld ldx) or X^T (X is K x M).
// One 64 x 64 output tile per CTA, 256 threads with 4 x 4 outputs each, K in steps of 16 staged
// in shared memory.  These products are off the critical path (once per call), so a plain
// FP64-pipe tiling is enough.
#include "launch_count.h"
#include "paraht_impl.h"

namespace pht {

template <bool kTX>
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, const double* __restrict__ X, int ldx,
                                                const double* __restrict__ Y, int ldy, double* __restrict__ Out,
                                                int ldo) {
  __shared__ double Xs[16][64 + 1];  // Xs[k][i] = op(X)(i0 + i, k0 + k)
  __shared__ double Ys[16][64 + 1];  // Ys[k][j] = Y(k0 + k, j0 + j)
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  const int t = threadIdx.x, ti = t % 16, tj = t / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = t; e < 16 * 64; e += 256) {
      // lanes run along the contiguous index of X in memory
      const int k = kTX ? e % 16 : e / 64, i = kTX ? e / 16 : e % 64;
      const int gi = i0 + i, gk = k0 + k;
      double xv = 0.0;
      if (gi < M && gk < K) xv = kTX ? X[gk + (size_t)gi * ldx] : X[gi + (size_t)gk * ldx];
      Xs[k][i] = xv;
    }
    for (int e = t; e < 16 * 64; e += 256) {
      const int k = e % 16, j = e / 16;
      const int gk = k0 + k, gj = j0 + j;
      Ys[k][j] = (gk < K && gj < N) ? Y[gk + (size_t)gj * ldy] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      double xr[4], yr[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) xr[a] = Xs[k][ti + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) yr[b] = Ys[k][tj + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(xr[a], yr[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int gi = i0 + ti + 16 * a, gj = j0 + tj + 16 * b;
      if (gi < M && gj < N) Out[gi + (size_t)gj * ldo] = acc[a][b];
    }
}

__global__ void k_set_identity(int n, double* X, int ldx) {
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) X[i + (size_t)j * ldx] = (i == j) ? 1.0 : 0.0;
}

void dgemm(cudaStream_t s, bool tx, int M, int N, int K, const double* X, int ldx, const double* Y, int ldy,
           double* Out, int ldo) {
  if (M <= 0 || N <= 0) return;
  const dim3 grid((M + 63) / 64, (N + 63) / 64);
  count_launch();
  if (tx)
    k_dgemm<true><<<grid, 256, 0, s>>>(M, N, K, X, ldx, Y, ldy, Out, ldo);
  else
    k_dgemm<false><<<grid, 256, 0, s>>>(M, N, K, X, ldx, Y, ldy, Out, ldo);
}

void set_identity(cudaStream_t s, int n, double* X, int ldx) {
  if (n <= 0) return;
  count_launch();
  k_set_identity<<<n, 128, 0, s>>>(n, X, ldx);
}

}  // namespace pht
