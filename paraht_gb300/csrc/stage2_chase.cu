// stage2_chase.cu -- the pipelined chase kernel of one stage-2 sweep group (one CTA per sweep);
// the sweep itself and its synchronisation are in stage2_chase.cuh.
//
// This file is compiled with -Xptxas -dlcm=cg so that global loads bypass L1 and observe the
// other CTAs' writes after the acquire.
#include "launch_count.h"
#include "stage2_chase.cuh"

namespace pht {

__global__ void __launch_bounds__(kChaseMaxThreads, 1) k_s2_chase(ChaseArgs a) {
  extern __shared__ double sm[];
  __shared__ int s_ic, s_abort;
  const int r = a.r, nq = a.nq;
  Sm s = chase_sm(sm, r, nq, &s_abort);
  if (threadIdx.x == 0) s_abort = 0;
  if (!a.pipelined) {
    __syncthreads();
    for (int ic = 1; ic <= a.nq; ++ic) run_sweep(a, ic, s);
    return;
  }
  if (threadIdx.x == 0) s_ic = atomicAdd(a.sync.ticket, 1) + 1;
  __syncthreads();
  run_sweep(a, s_ic, s);
}

// The chase's bounded wait on a progress word that nothing sets: the failure path of the
// pipelined schedule.  The wait must give up after spin_limit polls, set the status word to
// PARAHT_ERR_TIMEOUT and return, leaving the context usable.  words: [0] status, [1] result
// (1 = the wait succeeded), [2..3] progress words of sweeps 0 and 1 (left at 0).
__global__ void k_s2_wait_selftest(ChaseArgs a, int* result) {
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  __syncthreads();
  const bool ok = wait_prev(a, 2, 1, &s_abort);  // sweep 2 waits for step 1 of sweep 1
  if (threadIdx.x == 0) *result = ok ? 1 : 0;
}

int s2_wait_selftest(cudaStream_t st, int* words, long long spin_limit) {
  ChaseArgs a{};
  a.pipelined = 1;
  a.spin_limit = spin_limit;
  a.sync.status = words;
  a.sync.prog = words + 2;
  a.sync.ticket = nullptr;
  cudaMemsetAsync(words, 0, 4 * sizeof(int), st);
  count_launch();
  k_s2_wait_selftest<<<1, 32, 0, st>>>(a, words + 1);
  int h[2] = {0, 0};
  cudaMemcpyAsync(h, words, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  return h[1] ? 0 : h[0];
}

void s2_launch_chase(cudaStream_t st, double* A, int lda, double* B, int ldb, int n, int J, int r, int nq,
                     const S2Store& S, const ChaseSync& sync, int sequential, long long spin_limit) {
  ChaseArgs a;
  a.A = A;
  a.lda = lda;
  a.B = B;
  a.ldb = ldb;
  a.n = n;
  a.J = J;
  a.r = r;
  a.nq = nq;
  a.S = S;
  a.sync = sync;
  a.spin_limit = spin_limit;
  a.pipelined = sequential ? 0 : 1;
  // 4 lanes per row of the r x r block (the RQ needs nt/4 >= r); eight warps so that the
  // right-reflector updates of the rows above the window have lanes to spread over
  const int nt = kChaseMaxThreads;
  const size_t smem = chase_smem_bytes(r, nq);
  if (a.pipelined) {
    cudaMemsetAsync(sync.prog, 0, sizeof(int) * (nq + 1), st);
    cudaMemsetAsync(sync.ticket, 0, sizeof(int), st);
  }
  count_launch();
  k_s2_chase<<<a.pipelined ? nq : 1, nt, smem, st>>>(a);
}

}  // namespace pht
