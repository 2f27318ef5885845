// s2_common.cuh -- stage-2 reflector storage shared by the chase kernel and the update driver.
#pragma once
#include <cuda_runtime.h>

#include "paraht_internal.cuh"

namespace pht {

// Reflectors of one sweep group: U, V (ldu = r+nq) x nq x nblk, TU, TV nq x nq x nblk,
// tauU, tauV nq x nblk (the reference's U, V, TU, TV, tauU, tauV, src/rht2ht.f90:1389-1394).
// Helpers take the reference's 1-based (i, ic, ib).
struct S2Store {
  double *U, *V, *TU, *TV, *tauU, *tauV;
  int ldu, nq;
  PHT_DEV __host__ size_t ui(int i, int ic, int ib) const {
    return (size_t)(i - 1) + (size_t)(ic - 1) * ldu + (size_t)(ib - 1) * ldu * nq;
  }
  PHT_DEV __host__ size_t ti(int ic, int ib) const { return (size_t)(ic - 1) + (size_t)(ib - 1) * nq; }
  PHT_DEV __host__ size_t tt(int ib) const { return (size_t)(ib - 1) * nq * nq; }
};

// Progress words of one chase launch: prog[ic] = last completed step of sweep ic (1-based),
// ticket = next sweep to start, status = error code (0 ok).
struct ChaseSync {
  int* prog;    // nq + 1 ints
  int* ticket;  // 1 int
  int* status;  // 1 int
};

// Launches the band-only bulge chase of one sweep group (src/rht2ht.f90:1450-1596).
// sequential != 0 runs every sweep in one CTA, one after the other (the reference's order);
// otherwise one CTA per sweep, pipelined (sweep ic runs two steps behind sweep ic-1).
// Self-test of the chase's bounded wait (see stage2_chase.cu): returns the status the wait
// reported (PARAHT_ERR_TIMEOUT expected), words: 4 ints of device memory.
int s2_wait_selftest(cudaStream_t st, int* words, long long spin_limit);

void s2_launch_chase(cudaStream_t st, double* A, int lda, double* B, int ldb, int n, int J, int r, int nq,
                     const S2Store& S, const ChaseSync& sync, int sequential, long long spin_limit);

}  // namespace pht
