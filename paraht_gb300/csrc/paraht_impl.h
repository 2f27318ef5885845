// paraht_impl.h -- host-side internals shared by the stage drivers and the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/paraht.h"
#include "launch_count.h"

namespace pht {

// Records CUDA events at phase boundaries; per-phase device time is accumulated after the
// stream has finished.  mark(s, p) starts phase p (p < 0 ends the current phase).
struct PhaseTimer {
  std::vector<cudaEvent_t> ev;
  std::vector<int> phase;
  size_t used = 0;
  int offset = 0;  // phase index offset (stage 2 phases start at 3)
  bool serial = true;  // the stages run their side-stream work on the timed stream
  void reset(int off) {
    used = 0;
    phase.clear();
    offset = off;
  }
  void mark(cudaStream_t s, int p) {
    if (used == ev.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
    }
    cudaEventRecord(ev[used], s);
    phase.push_back(p < 0 ? -1 : p + offset);
    ++used;
  }
  // Adds the elapsed times into out[0..nout) (call after the stream completed).
  void accumulate(double* out, int nout) {
    for (size_t i = 1; i < used; ++i) {
      const int p = phase[i - 1];
      if (p < 0 || p >= nout) continue;
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ev[i - 1], ev[i]) == cudaSuccess) out[p] += ms * 1e-3;
    }
  }
  ~PhaseTimer() {
    for (auto e : ev) cudaEventDestroy(e);
  }
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int max_smem = 0;
  int num_sms = 0;
  void* ws = nullptr;  // workspace (grown on demand, reused across calls)
  size_t ws_bytes = 0;
  void* ws_fixed = nullptr;  // when set, workspace() hands out this fixed region instead
  size_t ws_fixed_bytes = 0;
  double* stage[4] = {nullptr, nullptr, nullptr, nullptr};  // device copies for host entries
  size_t stage_bytes = 0;
  cudaStream_t side = nullptr;      // second stream for work that overlaps the critical path
  cudaStream_t side2 = nullptr;     // third stream (bulk updates that feed nothing on the critical path)
  cudaStream_t side3 = nullptr, side4 = nullptr;  // stage-2 bulk updates of Q and Z beside those of A, B
  // highest-priority stream for the critical path (generation chains, chase, lookahead): the bulk
  // op-list CTAs live for a whole list and fill the SMs, so a chain kernel waits for a free CTA
  // slot, and the scheduler gives freed slots to the highest-priority stream first.  Calls run on
  // it, joined to the caller's stream by ev_enter / ev_exit.
  cudaStream_t crit = nullptr;
  cudaEvent_t ev_enter = nullptr, ev_exit = nullptr;
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;
  bool lean = false;                 // side3/side4 alias side/side2 (a batched call's worker context)
  cudaEvent_t ev_s2[6] = {};        // stage-2 bulk chains: operands prepared, A joined to B, then the
                                    // Q and Z lists of the groups using store 0 ([2], [3]) and 1 ([4], [5])
  cudaEvent_t ev[8] = {};           // stage-1 dependency events
  int sequential_chase = 0;         // 1: run stage-2 sweeps one after the other in one CTA
  long long spin_limit = 1ll << 24;  // polls before a device-side wait gives up
  int* dstatus = nullptr;  // device status word
  PhaseTimer timer;
  double phase[8] = {0};
  double residue[2] = {0};
  long long launches = 0;  // kernels launched by the last call
  int split = 0;           // split-precision bulk updates (PARAHT_FLAG_SPLIT)
  void* sws = nullptr;     // split-precision per-op operand slots
  size_t sws_bytes = 0;
  size_t sws_region = 0;   // bytes per region (one region per launch site)
  // Returns region r of the split workspace, sized for `ops` ops of `op_bytes` each (6 regions).
  void* split_region(int r, int ops, size_t op_bytes);
  double* dresidue = nullptr;
  void* workspace(size_t bytes);
  int ensure_staging(size_t bytes_each);
  // PARAHT_FLAG_KERNEL_TIMES: event pairs of the timed launches (reused across calls), their
  // sites, and the statistics of the last call
  struct Clock : KernelClock {
    std::vector<cudaEvent_t> ev;
    std::vector<int> site;
    size_t used = 0;
    cudaEvent_t ref = nullptr;  // recorded on the context's stream before the call's first launch
  } kc;
  double kstats[8] = {0};
  // persistent batched kernel (batched.cu): its device buffer (pencil table, queue counter,
  // per-CTA workspace), the host image of the table, and the stream it runs on while the
  // pencils it does not take go through the single-pencil path
  void* bws = nullptr;
  size_t bws_bytes = 0;
  std::vector<char> bhost;
  cudaStream_t bstream = nullptr;
  // worker contexts (paraht_ctx handles) reducing the batch's other pencils concurrently
  std::vector<void*> workers;
  // DGGHD3-compatible entry: Q_s, Z_s of the diagonal block and the GEMM output buffer
  double* gws = nullptr;
  size_t gws_bytes = 0;
};
constexpr int kBatchWorkers = 8;

size_t s1_workspace_bytes(int n, int nb, int p);
size_t s2_workspace_bytes(int n, int r, int nq);
int s1_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int nb,
           int p, PhaseTimer* timer);
int s2_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
           int nq, PhaseTimer* timer);
// Stage 2 with Givens rotations (stage2g.cu); supported for r <= 32, r + nq <= 64.
size_t s2g_workspace_bytes(int n, int r, int nq);
bool s2g_supported(int r, int nq);
int s2g_run(Ctx& ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
            int nq, PhaseTimer* timer);
// Zeroes entries below the structure (lower bandwidth `band` for A, 0 for B) and records the
// largest absolute value zeroed in dres[0] (A) and dres[1] (B).
void zero_fill(cudaStream_t s, int n, double* A, int lda, int band, double* B, int ldb, double* dres);
int check_finite(cudaStream_t s, int n, const double* A, int lda, const double* B, int ldb, int* dflag);
// FP64 GEMM Out = op(X) Y (op = transpose when tx) and identity fill (gemm.cu).
void dgemm(cudaStream_t s, bool tx, int M, int N, int K, const double* X, int ldx, const double* Y, int ldy,
           double* Out, int ldo);
void set_identity(cudaStream_t s, int n, double* X, int ldx);
// smem_at_least (declared in paraht_internal.cuh): dynamic shared-memory limits only ever grow.
int smem_at_least(const void* func, size_t bytes);
// Batched reduction (batched.cu): which pencils the persistent kernel takes, and one launch
// over the pencils idx[] of the batch on stream s.
bool batch_eligible(int n, int r, int p, int nq);
int batch_run(Ctx& x, cudaStream_t s, const std::vector<int>& idx, const int* n, double* const* A, const int* lda,
              double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z, const int* ldz,
              const int* r, const int* p, const int* nq);
// A bucket of a batch plan (batched.cu): the pencils idx[], all taken by the persistent kernel, with
// their table uploaded to a buffer of their own; enqueue = queue reset + one persistent launch.
int batch_bucket_create(Ctx& x, const std::vector<int>& idx, const int* n, double* const* A, const int* lda,
                        double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z,
                        const int* ldz, const int* r, const int* p, const int* nq, void** bucket);
void batch_bucket_enqueue(const void* bucket, cudaStream_t s);
void batch_bucket_destroy(void* bucket);

}  // namespace pht
