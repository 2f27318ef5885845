// stage1_gen.cu -- the stage-1 generation kernels of the single-pencil path (one CTA each; the
// bodies are in stage1_gen.cuh).
#include "launch_count.h"
#include "paraht_impl.h"
#include "stage1_gen.cuh"

namespace pht {

__global__ void __launch_bounds__(512) k_s1_lgen(double* __restrict__ A, int lda, S1Panel P, double* __restrict__ VL,
                                                  double* __restrict__ TL) {
  extern __shared__ double sm[];
  s1_lgen_body(A, lda, P, VL, TL, sm);
}

__global__ void __launch_bounds__(512) k_s1_rgen(const double* __restrict__ B, int ldb, S1Panel P, int o,
                                                  double* __restrict__ VRc, double* __restrict__ TR, int use_vr) {
  extern __shared__ double sm[];
  s1_rgen_body(B, ldb, P, o, VRc, TR, use_vr, (int)blockDim.x, sm);
}

// Grants both generation kernels the full 227 KB of dynamic shared memory on the current device
// (once per process and device in effect: smem_at_least only calls the runtime when the limit grows).
int s1_gen_grant() {
  if (const int rc = smem_at_least((const void*)k_s1_lgen, 227 * 1024)) return rc;
  return smem_at_least((const void*)k_s1_rgen, 227 * 1024);
}

__global__ void k_reflector_selftest(int count, const double* alpha, const double* xnorm2, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const Reflector h = reflector_from_norm2(alpha[i], xnorm2[i]);
  out[3 * i] = h.tau;
  out[3 * i + 1] = h.scal;
  out[3 * i + 2] = h.beta;
}

void launch_reflector_selftest(cudaStream_t s, int count, const double* alpha, const double* xnorm2, double* out) {
  if (count <= 0) return;
  count_launch();
  k_reflector_selftest<<<(count + 255) / 256, 256, 0, s>>>(count, alpha, xnorm2, out);
}

void launch_s1_lgen(cudaStream_t s, double* A, int lda, const S1Panel& P, double* VL, double* TL) {
  count_launch();
  k_s1_lgen<<<1, s1_lgen_threads(P.nb), s1_lgen_smem(P.L, P.nb), s>>>(A, lda, P, VL, TL);
}

void launch_s1_rgen(cudaStream_t s, const double* B, int ldb, const S1Panel& P, int o, double* VRc, double* TR) {
  static int max_smem = -1;
  if (max_smem < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  const bool vr = s1_rgen_smem_vr(P.L, P.nb, true) <= (size_t)max_smem;
  count_launch();
  k_s1_rgen<<<1, s1_rgen_threads(P.L), s1_rgen_smem_vr(P.L, P.nb, vr), s>>>(B, ldb, P, o, VRc, TR, vr ? 1 : 0);
}

}  // namespace pht
