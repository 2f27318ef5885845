// api.cu -- the extern "C" boundary of libparaht (declared in include/paraht.h).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <map>
#include <atomic>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "launch_count.h"
#include "paraht_impl.h"
#include "paraht_internal.cuh"
#include "s2_common.cuh"
#include "qz_real.cuh"
#include "split_apply.cuh"

namespace pht {
thread_local long long tl_launches = 0;
thread_local KernelClock* tl_kclock = nullptr;

// Next event pair for a timed launch; events are created on first use and kept by the context.
bool KernelClock::pair(int st, cudaEvent_t* e0, cudaEvent_t* e1) {
  auto* c = static_cast<Ctx::Clock*>(this);
  constexpr size_t kMaxPairs = size_t(1) << 20;
  if (c->used >= kMaxPairs) return false;
  if (2 * c->used + 2 > c->ev.size()) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      cudaGetLastError();
      if (a) cudaEventDestroy(a);
      return false;
    }
    c->ev.push_back(a);
    c->ev.push_back(b);
    c->site.push_back(0);
  }
  *e0 = c->ev[2 * c->used];
  *e1 = c->ev[2 * c->used + 1];
  c->site[c->used] = st;
  ++c->used;
  return true;
}
}

struct paraht_ctx_s {
  pht::Ctx c;
  uint32_t magic;
};
static const uint32_t kMagic = 0x50485431u;  // "PHT1"

namespace pht {

void* Ctx::workspace(size_t bytes) {
  if (ws_fixed) return bytes <= ws_fixed_bytes ? ws_fixed : nullptr;
  if (bytes <= ws_bytes) return ws;
  if (ws) {
    cudaStreamSynchronize(stream);
    cudaFree(ws);
    ws = nullptr;
    ws_bytes = 0;
  }
  const size_t want = bytes + bytes / 4;
  if (cudaMalloc(&ws, want) != cudaSuccess) {
    ws = nullptr;
    cudaGetLastError();
    return nullptr;
  }
  ws_bytes = want;
  return ws;
}

void* Ctx::split_region(int r, int ops, size_t op_bytes) {
  const size_t per = ((size_t)ops * op_bytes + 255) & ~(size_t)255;
  if (per > sws_region) {
    cudaDeviceSynchronize();  // regions may be in use by queued work on any stream
    if (sws) cudaFree(sws);
    sws = nullptr;
    sws_region = 0;
    if (cudaMalloc(&sws, 6 * per) != cudaSuccess) {
      cudaGetLastError();
      sws = nullptr;
      return nullptr;
    }
    sws_region = per;
    sws_bytes = 6 * per;
  }
  return (char*)sws + (size_t)r * sws_region;
}

int Ctx::ensure_staging(size_t bytes_each) {
  if (bytes_each <= stage_bytes) return 0;
  cudaStreamSynchronize(stream);
  for (auto& p : stage) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  stage_bytes = 0;
  for (auto& p : stage) {
    if (cudaMalloc(&p, bytes_each) != cudaSuccess) {
      cudaGetLastError();
      for (auto& q : stage) {
        if (q) cudaFree(q);
        q = nullptr;
      }
      return PARAHT_ERR_ALLOC;
    }
  }
  stage_bytes = bytes_each;
  return 0;
}

// Non-negative doubles order like their bit patterns, so the maximum of |x| can be taken with
// an integer atomicMax.
__global__ void k_zero_fill(int n, double* X, int ldx, int band, unsigned long long* res) {
  const int j = blockIdx.x;
  double m = 0.0;
  for (int i = j + band + 1 + threadIdx.x; i < n; i += blockDim.x) {
    double* p = X + (size_t)i + (size_t)j * ldx;
    m = fmax(m, fabs(*p));
    *p = 0.0;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(res, (unsigned long long)__double_as_longlong(m));
}

void zero_fill(cudaStream_t s, int n, double* A, int lda, int band, double* B, int ldb, double* dres) {
  if (n <= 1) return;
  cudaMemsetAsync(dres, 0, 2 * sizeof(double), s);
  count_launch(2);
  k_zero_fill<<<n, 128, 0, s>>>(n, A, lda, band, (unsigned long long*)dres);
  k_zero_fill<<<n, 128, 0, s>>>(n, B, ldb, 0, (unsigned long long*)(dres + 1));
}

__global__ void k_check_finite(int n, const double* X, int ldx, int* flag) {
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (!isfinite(X[(size_t)i + (size_t)j * ldx])) atomicOr(flag, 1);
}

int smem_at_least(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> granted;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(mu);
  size_t& g = granted[{func, dev}];
  if (bytes <= g) return 0;
  if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  g = bytes;
  return 0;
}

int check_finite(cudaStream_t s, int n, const double* A, int lda, const double* B, int ldb, int* dflag) {
  cudaMemsetAsync(dflag, 0, sizeof(int), s);
  count_launch(2);
  k_check_finite<<<n, 256, 0, s>>>(n, A, lda, dflag);
  k_check_finite<<<n, 256, 0, s>>>(n, B, ldb, dflag);
  int h = 0;
  cudaMemcpyAsync(&h, dflag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return PARAHT_ERR_CUDA;
  return h ? PARAHT_ERR_NONFINITE : 0;
}

}  // namespace pht

using pht::Ctx;

static int ctx_ok(paraht_ctx c) { return c && c->magic == kMagic; }

// lean: a batched call's worker context, whose stage-2 bulk lists share two side streams (B and Q
// on one, A and Z on the other) instead of four, so that the worker contexts of a batch together
// stay within the device's hardware queues (CUDA_DEVICE_MAX_CONNECTIONS, at most 32): streams
// beyond them share queues, and a chain kernel of one pencil then waits behind another
// pencil's bulk launch.  The pencils of the batch provide the concurrency the four streams give
// a lone pencil.
static int ctx_create(paraht_ctx* out, int device, bool lean);

extern "C" int paraht_ctx_create(paraht_ctx* out, int device) { return ctx_create(out, device, false); }

static int ctx_create(paraht_ctx* out, int device, bool lean) {
  if (!out) return -1;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PARAHT_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return -2;
  paraht_ctx c = new (std::nothrow) paraht_ctx_s();
  if (!c) return PARAHT_ERR_ALLOC;
  c->magic = kMagic;
  Ctx& x = c->c;
  x.device = device;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  cudaDeviceGetAttribute(&x.max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  cudaDeviceGetAttribute(&x.num_sms, cudaDevAttrMultiProcessorCount, device);
  int rc = 0;
  if (cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  x.own_stream = true;
  if (!rc && cudaStreamCreateWithFlags(&x.side, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (!rc && cudaEventCreateWithFlags(&x.ev_a, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (!rc && cudaEventCreateWithFlags(&x.ev_b, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (!rc && cudaStreamCreateWithFlags(&x.side2, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  {
    int least = 0, greatest = 0;
    if (!rc && cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    if (!rc && cudaStreamCreateWithPriority(&x.crit, cudaStreamNonBlocking, greatest) != cudaSuccess)
      rc = PARAHT_ERR_CUDA;
    if (!rc && cudaEventCreateWithFlags(&x.ev_enter, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    if (!rc && cudaEventCreateWithFlags(&x.ev_exit, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  }
  if (lean) {
    x.side3 = x.side;
    x.side4 = x.side2;
    x.lean = true;
  } else {
    if (!rc && cudaStreamCreateWithFlags(&x.side3, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    if (!rc && cudaStreamCreateWithFlags(&x.side4, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  }
  for (auto& e : x.ev_s2)
    if (!rc && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  for (auto& e : x.ev)
    if (!rc && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (!rc && cudaMalloc(&x.dstatus, 64) != cudaSuccess) rc = PARAHT_ERR_ALLOC;
  if (!rc && cudaMalloc(&x.dresidue, 2 * sizeof(double)) != cudaSuccess) rc = PARAHT_ERR_ALLOC;
  cudaSetDevice(prev);
  if (rc) {
    cudaGetLastError();
    paraht_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return 0;
}

extern "C" int paraht_ctx_destroy(paraht_ctx c) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  if (x.stream) cudaStreamSynchronize(x.stream);
  if (x.ws) cudaFree(x.ws);
  for (auto p : x.stage)
    if (p) cudaFree(p);
  if (x.dstatus) cudaFree(x.dstatus);
  if (x.dresidue) cudaFree(x.dresidue);
  if (x.own_stream && x.stream) cudaStreamDestroy(x.stream);
  if (x.side) {
    cudaStreamSynchronize(x.side);
    cudaStreamDestroy(x.side);
  }
  for (cudaStream_t* sp : {&x.side2, &x.side3, &x.side4, &x.crit})
    if (*sp && !(x.lean && (sp == &x.side3 || sp == &x.side4))) {  // a lean context's side3/4 alias side/side2
      cudaStreamSynchronize(*sp);
      cudaStreamDestroy(*sp);
    }
  for (auto e : x.ev_s2)
    if (e) cudaEventDestroy(e);
  if (x.ev_enter) cudaEventDestroy(x.ev_enter);
  if (x.ev_exit) cudaEventDestroy(x.ev_exit);
  if (x.bstream) {
    cudaStreamSynchronize(x.bstream);
    cudaStreamDestroy(x.bstream);
  }
  for (void* w : x.workers) paraht_ctx_destroy((paraht_ctx)w);
  x.workers.clear();
  if (x.gws) cudaFree(x.gws);
  if (x.bws) cudaFree(x.bws);
  if (x.ev_a) cudaEventDestroy(x.ev_a);
  if (x.ev_b) cudaEventDestroy(x.ev_b);
  for (auto e : x.kc.ev) cudaEventDestroy(e);
  if (x.kc.ref) cudaEventDestroy(x.kc.ref);
  if (x.kc.dflops) cudaFree(x.kc.dflops);
  for (auto e : x.ev)
    if (e) cudaEventDestroy(e);
  cudaSetDevice(prev);
  c->magic = 0;
  delete c;
  return 0;
}

extern "C" int paraht_ctx_set_stream(paraht_ctx c, void* stream) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  Ctx& x = c->c;
  if (stream) {
    if (x.own_stream && x.stream) {
      cudaStreamSynchronize(x.stream);
      cudaStreamDestroy(x.stream);
    }
    x.stream = (cudaStream_t)stream;
    x.own_stream = false;
  } else if (!x.own_stream) {
    if (cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking) != cudaSuccess) return PARAHT_ERR_CUDA;
    x.own_stream = true;
  }
  return 0;
}

extern "C" int paraht_ctx_phase_times(paraht_ctx c, double* t, int nt) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (!t && nt > 0) return -2;
  for (int i = 0; i < nt && i < 8; ++i) t[i] = c->c.phase[i];
  for (int i = 8; i < nt; ++i) t[i] = 0.0;
  return 0;
}

extern "C" int paraht_ctx_launch_count(paraht_ctx c, long long* count) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (!count) return -2;
  *count = c->c.launches;
  return 0;
}

extern "C" int paraht_ctx_kernel_stats(paraht_ctx c, double* st, int ns) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (!st) return -2;
  for (int i = 0; i < ns && i < 8; ++i) st[i] = c->c.kstats[i];
  return 0;
}

extern "C" int paraht_ctx_fill_residue(paraht_ctx c, double* r, int nr) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  for (int i = 0; i < nr && i < 2; ++i) r[i] = c->c.residue[i];
  return 0;
}

// Argument checks in LAPACK INFO style; `off` shifts the index for entry points with a leading
// ctx argument.  which: 1 = stage 1 (r, p), 2 = stage 2 (r, nq), 3 = both (r, p, nq).
static int check_args(int which, int off, int n, const double* A, int lda, const double* B, int ldb, const double* Q,
                      int ldq, const double* Z, int ldz, int r, int p, int nq) {
  if (n < 0) return -(1 + off);
  const int ldmin = std::max(1, n);
  if (n > 0 && !A) return -(2 + off);
  if (lda < ldmin) return -(3 + off);
  if (n > 0 && !B) return -(4 + off);
  if (ldb < ldmin) return -(5 + off);
  if (n > 0 && !Q) return -(6 + off);
  if (ldq < ldmin) return -(7 + off);
  if (n > 0 && !Z) return -(8 + off);
  if (ldz < ldmin) return -(9 + off);
  if (r < 1 || r > 64) return -(10 + off);
  if (which == 1 && p < 2) return -(11 + off);
  if (which == 2 && (nq < 1 || nq > r)) return -(11 + off);
  if (which == 3) {
    if (p < 2) return -(11 + off);
    if (nq < 1 || nq > r) return -(12 + off);
  }
  return 0;
}

static int finish(Ctx& x) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(x.stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  return 0;
}

// Runs the selected stages on device-resident arrays (stream-ordered; caller synchronises).
static int run_device_on(Ctx& x, int which, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                         double* Z, int ldz, int r, int p, int nq, int flags);
// The same on the context's high-priority stream, which waits for the work already queued on the
// caller's stream and which the caller's stream then waits for.
static int run_device(Ctx& x, int which, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                      int ldz, int r, int p, int nq, int flags) {
  if (!x.crit || n == 0) return run_device_on(x, which, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
  cudaStream_t user = x.stream;
  cudaEventRecord(x.ev_enter, user);
  cudaStreamWaitEvent(x.crit, x.ev_enter, 0);
  x.stream = x.crit;
  const int rc = run_device_on(x, which, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
  x.stream = user;
  cudaEventRecord(x.ev_exit, x.crit);
  cudaStreamWaitEvent(user, x.ev_exit, 0);
  return rc;
}

static int run_device_on(Ctx& x, int which, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                         double* Z, int ldz, int r, int p, int nq, int flags) {
  x.launches = 0;
  if (n == 0) return 0;
  x.split = (flags & PARAHT_FLAG_SPLIT) ? 1 : 0;
  if (x.split) {  // size the per-op operand slots once for both stages
    const int ops = std::max(n / std::max(1, (p - 1) * r) + 2, n / std::max(1, r) + 4);
    if (!x.split_region(0, ops, sizeof(pht::SplitOpData))) return PARAHT_ERR_ALLOC;
  }
  const long long launches0 = pht::tl_launches;
  const bool timed = flags & (PARAHT_FLAG_TIME_COMPONENTS | PARAHT_FLAG_TIME_CHAIN);
  x.timer.serial = (flags & PARAHT_FLAG_TIME_COMPONENTS) != 0;
  const bool ktimes = flags & PARAHT_FLAG_KERNEL_TIMES;
  for (double& v : x.kstats) v = 0.0;
  if (ktimes) {
    if (!x.kc.dflops && cudaMalloc(&x.kc.dflops, 2 * sizeof(unsigned long long)) != cudaSuccess) {
      cudaGetLastError();
      x.kc.dflops = nullptr;
      return PARAHT_ERR_ALLOC;
    }
    cudaMemsetAsync(x.kc.dflops, 0, 2 * sizeof(unsigned long long), x.stream);
    if (!x.kc.ref && cudaEventCreate(&x.kc.ref) != cudaSuccess) {
      cudaGetLastError();
      x.kc.ref = nullptr;
      return PARAHT_ERR_CUDA;
    }
    cudaEventRecord(x.kc.ref, x.stream);
    x.kc.used = 0;
    pht::tl_kclock = &x.kc;
  }
  if (flags & PARAHT_FLAG_CHECK_FINITE) {
    const int rc = pht::check_finite(x.stream, n, A, lda, B, ldb, x.dstatus);
    if (rc) return rc;
  }
  cudaMemsetAsync(x.dstatus, 0, sizeof(int), x.stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (timed) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, x.stream);
  }
  int rc = 0;
  x.sequential_chase = (flags & PARAHT_FLAG_SEQUENTIAL) ? 1 : 0;
  if (which & 1) {
    x.timer.reset(0);
    rc = pht::s1_run(x, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, timed ? &x.timer : nullptr);
    if (!rc && timed) {
      rc = finish(x);
      x.timer.accumulate(x.phase, 8);
    }
  }
  if (!rc && (which & 2)) {
    x.timer.reset(3);
    rc = (flags & PARAHT_FLAG_GIVENS)
             ? pht::s2g_run(x, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, timed ? &x.timer : nullptr)
             : pht::s2_run(x, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, timed ? &x.timer : nullptr);
    if (!rc && timed) {
      rc = finish(x);
      x.timer.accumulate(x.phase, 8);
    }
  }
  int hstatus = 0;
  if (!rc) cudaMemcpyAsync(&hstatus, x.dstatus, sizeof(int), cudaMemcpyDeviceToHost, x.stream);
  if (!rc && !(flags & PARAHT_FLAG_NO_ZERO_FILL)) {
    pht::zero_fill(x.stream, n, A, lda, (which & 2) ? 1 : r, B, ldb, x.dresidue);
    cudaMemcpyAsync(x.residue, x.dresidue, 2 * sizeof(double), cudaMemcpyDeviceToHost, x.stream);
  }
  if (timed) {
    cudaEventRecord(e1, x.stream);
    if (!rc) rc = finish(x);
    float ms = 0;
    if (!rc && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) x.phase[7] = ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (!rc) rc = finish(x);
  if (!rc && hstatus) rc = hstatus;
  pht::tl_kclock = nullptr;
  if (!rc && ktimes) {  // all streams have joined the main stream, which finish() synchronized
    // per launch: duration, and its interval relative to the reference event; the union of the
    // intervals of a site is the time during which at least one of its launches ran (launches on
    // different streams overlap)
    std::vector<std::pair<float, float>> iv[2];
    for (size_t i = 0; i < x.kc.used; ++i) {
      float ms = 0.f, a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&ms, x.kc.ev[2 * i], x.kc.ev[2 * i + 1]) != cudaSuccess ||
          cudaEventElapsedTime(&a, x.kc.ref, x.kc.ev[2 * i]) != cudaSuccess ||
          cudaEventElapsedTime(&b, x.kc.ref, x.kc.ev[2 * i + 1]) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      x.kstats[3 * x.kc.site[i]] += ms * 1e-3;
      x.kstats[3 * x.kc.site[i] + 1] += 1.0;
      iv[x.kc.site[i] & 1].push_back({a, b});
    }
    for (int st = 0; st < 2; ++st) {
      std::sort(iv[st].begin(), iv[st].end());
      double busy = 0.0, lo = 0.0, hi = -1.0;
      for (const auto& p : iv[st]) {
        if (p.first > hi) {
          if (hi > lo) busy += hi - lo;
          lo = p.first;
          hi = p.second;
        } else if (p.second > hi) {
          hi = p.second;
        }
      }
      if (hi > lo) busy += hi - lo;
      x.kstats[6 + st] = busy * 1e-3;
    }
    unsigned long long fl[2] = {0, 0};
    cudaMemcpy(fl, x.kc.dflops, sizeof(fl), cudaMemcpyDeviceToHost);
    x.kstats[2] = (double)fl[0];
    x.kstats[5] = (double)fl[1];
  }
  x.launches = pht::tl_launches - launches0;
  return rc;
}

static int device_entry(paraht_ctx c, int which, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                        double* Z, int ldz, int r, int p, int nq, int flags) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  Ctx& x = c->c;
  int rc = check_args(which, 1, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq);
  if (rc) return rc;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  for (double& v : x.phase) v = 0.0;
  x.residue[0] = x.residue[1] = 0.0;
  rc = run_device(x, which, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
  if (!rc) rc = finish(x);
  cudaSetDevice(prev);
  return rc;
}

extern "C" int paraht_ab2rht_d(paraht_ctx c, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                               double* Z, int ldz, int nb, int p, int flags) {
  return device_entry(c, 1, n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, 1, flags);
}
extern "C" int paraht_rht2ht_d(paraht_ctx c, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                               double* Z, int ldz, int r, int nq, int flags) {
  return device_entry(c, 2, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq, flags);
}
extern "C" int paraht_reduce_d(paraht_ctx c, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                               double* Z, int ldz, int r, int p, int nq, int flags) {
  return device_entry(c, 3, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
}

// ---- stage 2 without allocation: the workspace is a fixed file-scope device array ----
// For callers that cannot allocate during the call (their own memory pool owns the device, or a
// cudaMalloc would synchronise work they keep in flight).  In host code the array's name is only
// a host-side stand-in, so its device address is looked up on every call with the context's
// device current (a cached address would go stale after a cudaDeviceReset or under another
// context).  Calls that overlap on the GPU share the array and race.
static __device__ __align__(256) unsigned char g_noalloc_scratch[PARAHT_NOALLOC_SCRATCH_BYTES];
static std::mutex g_noalloc_mu;
static constexpr int kNoallocFlags = PARAHT_FLAG_CHECK_FINITE | PARAHT_FLAG_NO_ZERO_FILL | PARAHT_FLAG_SEQUENTIAL;

extern "C" int paraht_rht2ht_d_noalloc(paraht_ctx c, int n, double* A, int lda, double* B, int ldb, double* Q,
                                       int ldq, double* Z, int ldz, int r, int nq, int flags) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  Ctx& x = c->c;
  int rc = check_args(2, 1, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq);
  if (rc) return rc;
  // the flags that would allocate (split-precision operand slots, kernel-time counters) or
  // create events (phase and kernel timing) are refused
  if (flags & ~kNoallocFlags) return PARAHT_ERR_NOT_SUPPORTED;
  if (pht::s2_workspace_bytes(n, r, nq) > (size_t)PARAHT_NOALLOC_SCRATCH_BYTES) return PARAHT_ERR_TOO_LARGE;
  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(x.device) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);  // one call at a time from this process
  void* scratch = nullptr;
  if (cudaGetSymbolAddress(&scratch, g_noalloc_scratch) != cudaSuccess || !scratch) {
    cudaGetLastError();
    cudaSetDevice(prev);
    return PARAHT_ERR_CUDA;
  }
  for (double& v : x.phase) v = 0.0;
  x.residue[0] = x.residue[1] = 0.0;
  x.ws_fixed = scratch;
  x.ws_fixed_bytes = PARAHT_NOALLOC_SCRATCH_BYTES;
  rc = run_device(x, 2, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq, flags);
  if (!rc) rc = finish(x);
  x.ws_fixed = nullptr;
  x.ws_fixed_bytes = 0;
  cudaSetDevice(prev);
  return rc;
}

// Host-pointer path: stage the four matrices into the context's device buffers, reduce, copy
// back.  `off` is the argument-index offset (0 for context-free entry points).
static int host_entry(paraht_ctx c, int off, int which, int n, double* A, int lda, double* B, int ldb, double* Q,
                      int ldq, double* Z, int ldz, int r, int p, int nq, int flags) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  Ctx& x = c->c;
  int rc = check_args(which, off, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq);
  if (rc || n == 0) return rc;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  for (double& v : x.phase) v = 0.0;
  x.residue[0] = x.residue[1] = 0.0;
  const int ldd = (n + 3) & ~3;  // 32-byte aligned columns on the device
  rc = x.ensure_staging((size_t)ldd * n * sizeof(double));
  if (!rc) {
    double* h[4] = {A, B, Q, Z};
    const int ld[4] = {lda, ldb, ldq, ldz};
    cudaEvent_t c0, c1, c2, c3;
    cudaEventCreate(&c0);
    cudaEventCreate(&c1);
    cudaEventCreate(&c2);
    cudaEventCreate(&c3);
    cudaEventRecord(c0, x.stream);
    for (int i = 0; i < 4; ++i)
      cudaMemcpy2DAsync(x.stage[i], (size_t)ldd * sizeof(double), h[i], (size_t)ld[i] * sizeof(double),
                        (size_t)n * sizeof(double), n, cudaMemcpyHostToDevice, x.stream);
    cudaEventRecord(c1, x.stream);
    rc = run_device(x, which, n, x.stage[0], ldd, x.stage[1], ldd, x.stage[2], ldd, x.stage[3], ldd, r, p, nq, flags);
    cudaEventRecord(c2, x.stream);
    if (!rc)
      for (int i = 0; i < 4; ++i)
        cudaMemcpy2DAsync(h[i], (size_t)ld[i] * sizeof(double), x.stage[i], (size_t)ldd * sizeof(double),
                          (size_t)n * sizeof(double), n, cudaMemcpyDeviceToHost, x.stream);
    cudaEventRecord(c3, x.stream);
    const int rc2 = finish(x);
    if (!rc) rc = rc2;
    if (!rc) {
      float a = 0, b = 0;
      cudaEventElapsedTime(&a, c0, c1);
      cudaEventElapsedTime(&b, c2, c3);
      x.phase[6] = (a + b) * 1e-3;
    }
    cudaEventDestroy(c0);
    cudaEventDestroy(c1);
    cudaEventDestroy(c2);
    cudaEventDestroy(c3);
  }
  cudaSetDevice(prev);
  return rc;
}

extern "C" int paraht_reduce_host(paraht_ctx c, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                                  double* Z, int ldz, int r, int p, int nq, int flags) {
  return host_entry(c, 1, 3, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
}

// One lazily created context per host thread for the context-free drop-ins.
static thread_local paraht_ctx tl_ctx = nullptr;
static thread_local int tl_dev = -1;
static int default_ctx(paraht_ctx* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_NO_DEVICE;
  }
  if (tl_ctx && tl_dev != dev) {
    paraht_ctx_destroy(tl_ctx);
    tl_ctx = nullptr;
  }
  if (!tl_ctx) {
    const int rc = paraht_ctx_create(&tl_ctx, dev);
    if (rc) return rc;
    tl_dev = dev;
  }
  *out = tl_ctx;
  return 0;
}

extern "C" int paraht_ab2rht(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz,
                             int nb, int p, int time_components) {
  if (const int bad = check_args(1, 0, n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, 1)) return bad;
  if (n == 0) return 0;
  paraht_ctx c;
  const int rc = default_ctx(&c);
  if (rc) return rc;
  return host_entry(c, 0, 1, n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, 1,
                    time_components ? PARAHT_FLAG_TIME_COMPONENTS : 0);
}
extern "C" int paraht_rht2ht(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz,
                             int r, int nq, int time_components) {
  if (const int bad = check_args(2, 0, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq)) return bad;
  if (n == 0) return 0;
  paraht_ctx c;
  const int rc = default_ctx(&c);
  if (rc) return rc;
  return host_entry(c, 0, 2, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq,
                    time_components ? PARAHT_FLAG_TIME_COMPONENTS : 0);
}
extern "C" int paraht_rht2ht_givens(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                                    int ldz, int r, int nq) {
  if (const int bad = check_args(2, 0, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq)) return bad;
  if (n == 0) return 0;
  if (!pht::s2g_supported(r, nq)) return PARAHT_ERR_NOT_SUPPORTED;
  paraht_ctx c;
  const int rc = default_ctx(&c);
  if (rc) return rc;
  return host_entry(c, 0, 2, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, 2, nq, PARAHT_FLAG_GIVENS);
}
extern "C" int paraht_reduce(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz,
                             int r, int p, int nq, int flags) {
  if (const int bad = check_args(3, 0, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq)) return bad;
  if (n == 0) return 0;
  paraht_ctx c;
  const int rc = default_ctx(&c);
  if (rc) return rc;
  return host_entry(c, 0, 3, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
}

// ---- batch plans: a fixed set of pencils reduced by replaying a CUDA graph ----
struct paraht_batch_plan_s {
  uint32_t magic;
  int device;
  std::vector<void*> buckets;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> ev;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int count = 0;
};
static const uint32_t kPlanMagic = 0x50485450u;  // "PHTP"

static void plan_free(paraht_batch_plan pl) {
  if (!pl) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(pl->device);
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  for (void* b : pl->buckets) pht::batch_bucket_destroy(b);
  for (auto st : pl->branch)
    if (st) cudaStreamDestroy(st);
  for (auto e : pl->ev)
    if (e) cudaEventDestroy(e);
  if (pl->cap) cudaStreamDestroy(pl->cap);
  cudaSetDevice(prev);
  pl->magic = 0;
  delete pl;
}

extern "C" int paraht_batch_plan_create(paraht_ctx c, int count, const int* n, double* const* A, const int* lda,
                                        double* const* B, const int* ldb, double* const* Q, const int* ldq,
                                        double* const* Z, const int* ldz, const int* r, const int* p, const int* nq,
                                        int flags, paraht_batch_plan* plan) {
  if (!plan) return -16;
  *plan = nullptr;
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (count < 0) return -2;
  if (count > 0 && (!n || !A || !lda || !B || !ldb || !Q || !ldq || !Z || !ldz || !r || !p || !nq)) return -3;
  if (flags != 0) return PARAHT_ERR_NOT_SUPPORTED;
  for (int i = 0; i < count; ++i) {
    if (check_args(3, 0, n[i], A[i], lda[i], B[i], ldb[i], Q[i], ldq[i], Z[i], ldz[i], r[i], p[i], nq[i])) return -3;
    if (n[i] > PARAHT_BATCH_MAX_N || !pht::batch_eligible(n[i], r[i], p[i], nq[i])) return PARAHT_ERR_NOT_SUPPORTED;
  }
  Ctx& x = c->c;
  auto* pl = new (std::nothrow) paraht_batch_plan_s();
  if (!pl) return PARAHT_ERR_ALLOC;
  pl->magic = kPlanMagic;
  pl->device = x.device;
  pl->count = count;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  // buckets: pencils sharing (r, p, nq), the autotuner's per-size choice; each gets the shared-memory
  // size and workspace of its own parameters
  std::vector<std::pair<std::array<int, 3>, std::vector<int>>> groups;
  for (int i = 0; i < count; ++i) {
    if (n[i] == 0) continue;
    const std::array<int, 3> key{r[i], p[i], nq[i]};
    auto it = std::find_if(groups.begin(), groups.end(), [&](const auto& g) { return g.first == key; });
    if (it == groups.end()) {
      groups.push_back({key, {}});
      it = groups.end() - 1;
    }
    it->second.push_back(i);
  }
  int rc = 0;
  for (const auto& g : groups) {
    void* b = nullptr;
    rc = pht::batch_bucket_create(x, g.second, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, &b);
    if (rc) break;
    pl->buckets.push_back(b);
  }
  // capture: fork one branch per bucket off a private stream, join, end
  if (!rc && cudaStreamCreateWithFlags(&pl->cap, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  const size_t nb = pl->buckets.size();
  for (size_t i = 0; !rc && i < nb; ++i) {
    cudaStream_t st = nullptr;
    cudaEvent_t e = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    pl->branch.push_back(st);
    if (!rc && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    pl->ev.push_back(e);
  }
  cudaEvent_t fork = nullptr;
  if (!rc && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (fork) pl->ev.push_back(fork);
  if (!rc && cudaStreamBeginCapture(pl->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (!rc) {
    cudaEventRecord(fork, pl->cap);
    const long long l0 = pht::tl_launches;
    for (size_t i = 0; i < nb; ++i) {
      cudaStreamWaitEvent(pl->branch[i], fork, 0);
      pht::batch_bucket_enqueue(pl->buckets[i], pl->branch[i]);
      cudaEventRecord(pl->ev[i], pl->branch[i]);
      cudaStreamWaitEvent(pl->cap, pl->ev[i], 0);
    }
    x.launches = pht::tl_launches - l0;
    if (cudaStreamEndCapture(pl->cap, &pl->graph) != cudaSuccess || !pl->graph) rc = PARAHT_ERR_CUDA;
  }
  if (!rc && cudaGraphInstantiate(&pl->exec, pl->graph, 0) != cudaSuccess) rc = PARAHT_ERR_CUDA;
  if (rc) cudaGetLastError();
  cudaSetDevice(prev);
  if (rc) {
    plan_free(pl);
    return rc;
  }
  *plan = pl;
  return 0;
}

extern "C" int paraht_batch_plan_launch(paraht_batch_plan pl, void* stream) {
  if (!pl || pl->magic != kPlanMagic) return PARAHT_ERR_BAD_CTX;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(pl->device);
  const cudaError_t e = cudaGraphLaunch(pl->exec, (cudaStream_t)stream);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_CUDA;
  }
  return 0;
}

extern "C" int paraht_batch_plan_destroy(paraht_batch_plan pl) {
  if (!pl || pl->magic != kPlanMagic) return PARAHT_ERR_BAD_CTX;
  plan_free(pl);
  return 0;
}

extern "C" int paraht_reduce_batched_d(paraht_ctx c, int count, const int* n, double* const* A, const int* lda,
                                       double* const* B, const int* ldb, double* const* Q, const int* ldq,
                                       double* const* Z, const int* ldz, const int* r, const int* p, const int* nq,
                                       int flags) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (count < 0) return -2;
  if (flags & PARAHT_FLAG_GIVENS) return PARAHT_ERR_NOT_SUPPORTED;  // the persistent kernel chases with reflectors
  if (count > 0 && (!n || !A || !lda || !B || !ldb || !Q || !ldq || !Z || !ldz || !r || !p || !nq)) return -3;
  for (int i = 0; i < count; ++i) {
    const int rc = check_args(3, 0, n[i], A[i], lda[i], B[i], ldb[i], Q[i], ldq[i], Z[i], ldz[i], r[i], p[i], nq[i]);
    if (rc) return -3;
  }
  if (count == 0) return 0;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  x.launches = 0;
  const int single_flags =
      flags & ~(PARAHT_FLAG_TIME_COMPONENTS | PARAHT_FLAG_TIME_CHAIN | PARAHT_FLAG_BATCH_LOOP | PARAHT_FLAG_KERNEL_TIMES);
  std::vector<int> small, large;
  for (int i = 0; i < count; ++i) {
    if (n[i] == 0) continue;
    const bool persistent = !(flags & PARAHT_FLAG_BATCH_LOOP) && n[i] <= PARAHT_BATCH_MAX_N &&
                            pht::batch_eligible(n[i], r[i], p[i], nq[i]);
    (persistent ? small : large).push_back(i);
  }
  // the single-pencil path takes the largest pencils first (its workers finish together)
  std::stable_sort(large.begin(), large.end(), [&](int a, int b) { return n[a] > n[b]; });
  int rc = 0;
  long long launches = 0;
  if (!small.empty()) {
    if (!x.bstream && cudaStreamCreateWithFlags(&x.bstream, cudaStreamNonBlocking) != cudaSuccess) rc = PARAHT_ERR_CUDA;
    if (!rc && (flags & PARAHT_FLAG_CHECK_FINITE))
      for (int i : small) {
        rc = pht::check_finite(x.stream, n[i], A[i], lda[i], B[i], ldb[i], x.dstatus);
        if (rc) break;
      }
    if (!rc) {  // after everything queued on the context's stream
      cudaEventRecord(x.ev_a, x.stream);
      cudaStreamWaitEvent(x.bstream, x.ev_a, 0);
      const long long l0 = pht::tl_launches;
      rc = pht::batch_run(x, x.bstream, small, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq);
      launches += pht::tl_launches - l0;
    }
  }
  // the other pencils through the single-pencil path, overlapping the persistent launch: several
  // at once on worker contexts (own streams and workspace, one host thread each), since one
  // pencil's serial chains leave most SMs idle
  // PARAHT_FLAG_BATCH_LOOP: the looped baseline, one paraht_reduce_d after the other on this context
  const int nworkers = (flags & PARAHT_FLAG_BATCH_LOOP) ? 1 : std::min<int>(pht::kBatchWorkers, (int)large.size());
  if (!rc && nworkers <= 1) {
    for (int i : large) {
      rc = run_device(x, 3, n[i], A[i], lda[i], B[i], ldb[i], Q[i], ldq[i], Z[i], ldz[i], r[i], p[i], nq[i],
                      single_flags);
      if (rc) break;
      launches += x.launches;
    }
  } else if (!rc) {
    while ((int)x.workers.size() < nworkers && !rc) {
      paraht_ctx w = nullptr;
      rc = ctx_create(&w, x.device, true);
      if (!rc) x.workers.push_back(w);
    }
    if (!rc) {
      cudaEventRecord(x.ev_b, x.stream);  // the pencils may have been produced on this stream
      for (int k = 0; k < nworkers; ++k) cudaStreamWaitEvent(((paraht_ctx)x.workers[k])->c.stream, x.ev_b, 0);
      std::atomic<int> next(0), err(0);
      std::atomic<long long> wl(0);
      std::vector<std::thread> th;
      for (int k = 0; k < nworkers; ++k)
        th.emplace_back([&, k]() {
          Ctx& wx = ((paraht_ctx)x.workers[k])->c;
          cudaSetDevice(wx.device);
          for (int j = next++; j < (int)large.size() && err.load() == 0; j = next++) {
            const int i = large[j];
            int e = run_device(wx, 3, n[i], A[i], lda[i], B[i], ldb[i], Q[i], ldq[i], Z[i], ldz[i], r[i], p[i], nq[i],
                               single_flags);
            if (!e) e = finish(wx);
            wl += wx.launches;
            if (e) {
              int zero = 0;
              err.compare_exchange_strong(zero, e);
            }
          }
        });
      for (auto& h : th) h.join();
      rc = err.load();
      launches += wl.load();
    }
  }
  if (!small.empty() && x.bstream) {
    const cudaError_t e = cudaStreamSynchronize(x.bstream);
    if (!rc && e != cudaSuccess) rc = PARAHT_ERR_CUDA;
  }
  if (!rc) rc = finish(x);
  x.launches = launches;
  cudaSetDevice(prev);
  return rc;
}

extern "C" int paraht_selftest_wait_timeout(paraht_ctx c, long long spin_limit) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (spin_limit < 1 || spin_limit > (1ll << 20)) return -2;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  const int rc = pht::s2_wait_selftest(x.stream, x.dstatus, spin_limit);
  cudaSetDevice(prev);
  return rc;
}

namespace pht {
void launch_reflector_selftest(cudaStream_t s, int count, const double* alpha, const double* xnorm2, double* out);
}

extern "C" int paraht_selftest_reflector(paraht_ctx c, int count, const double* alpha, const double* xnorm2,
                                         double* out) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (count < 0) return -2;
  if (count > 0 && (!alpha || !xnorm2 || !out)) return -3;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  pht::launch_reflector_selftest(x.stream, count, alpha, xnorm2, out);
  const int rc = finish(x);
  cudaSetDevice(prev);
  return rc;
}

// ---- generalized eigenvalues of Hessenberg-triangular pencils (QZ) ----
static int hgeqz_check(int count, const int* n, const double* const* H, const int* ldh, const double* const* T,
                       const int* ldt, double* const* alphar, double* const* alphai, double* const* beta,
                       const int* info) {
  if (count < 0) return -2;
  if (count == 0) return 0;
  if (!n) return -3;
  if (!H) return -4;
  if (!ldh) return -5;
  if (!T) return -6;
  if (!ldt) return -7;
  if (!alphar) return -8;
  if (!alphai) return -9;
  if (!beta) return -10;
  if (!info) return -11;
  for (int i = 0; i < count; ++i) {
    if (n[i] < 0) return -3;
    const int ldmin = std::max(1, n[i]);
    if (n[i] > 0 && !H[i]) return -4;
    if (ldh[i] < ldmin) return -5;
    if (n[i] > 0 && !T[i]) return -6;
    if (ldt[i] < ldmin) return -7;
    if (n[i] > 0 && !alphar[i]) return -8;
    if (n[i] > 0 && !alphai[i]) return -9;
    if (n[i] > 0 && !beta[i]) return -10;
  }
  return 0;
}

extern "C" int paraht_hgeqz_eigs_d(paraht_ctx c, int count, const int* n, const double* const* H, const int* ldh,
                                   const double* const* T, const int* ldt, double* const* alphar,
                                   double* const* alphai, double* const* beta, int* info) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  if (const int bad = hgeqz_check(count, n, H, ldh, T, ldt, alphar, alphai, beta, info)) return bad;
  if (count == 0) return 0;
  std::vector<pht::QzPencil> tab((size_t)count);
  long long work = 0;
  for (int i = 0; i < count; ++i) {
    tab[i] = pht::QzPencil{H[i], T[i], alphar[i], alphai[i], beta[i], work, n[i], ldh[i], ldt[i], 0};
    work += pht::qz_work_elems(n[i]);
  }
  // CTAs: the largest pencils first, each n >= kQzWholeMin on a CTA of its own, the rest one per
  // warp in decreasing size
  std::vector<int> order((size_t)count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::vector<pht::QzBlock> blocks;
  for (size_t k = 0; k < order.size();) {
    pht::QzBlock b{{-1, -1, -1, -1}, 0};
    if (n[order[k]] >= pht::kQzWholeMin) {
      b.pencil[0] = order[k++];
      b.whole = 1;
    } else {
      for (int w = 0; w < pht::kQzThreads / 32 && k < order.size(); ++w) b.pencil[w] = order[k++];
    }
    blocks.push_back(b);
  }
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t tab_b = up(sizeof(pht::QzPencil) * (size_t)count), info_b = up(sizeof(int) * (size_t)count);
  const size_t blk_b = up(sizeof(pht::QzBlock) * blocks.size());
  const size_t bytes = tab_b + info_b + blk_b + (size_t)work * sizeof(double);
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  char* buf = nullptr;
  if (cudaMalloc(&buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    cudaSetDevice(prev);
    return PARAHT_ERR_ALLOC;
  }
  auto* dtab = reinterpret_cast<pht::QzPencil*>(buf);
  auto* dinfo = reinterpret_cast<int*>(buf + tab_b);
  auto* dblk = reinterpret_cast<pht::QzBlock*>(buf + tab_b + info_b);
  auto* dwork = reinterpret_cast<double*>(buf + tab_b + info_b + blk_b);
  cudaMemcpyAsync(dtab, tab.data(), sizeof(pht::QzPencil) * (size_t)count, cudaMemcpyHostToDevice, x.stream);
  cudaMemcpyAsync(dblk, blocks.data(), sizeof(pht::QzBlock) * blocks.size(), cudaMemcpyHostToDevice, x.stream);
  const long long l0 = pht::tl_launches;
  pht::launch_qz_eigs(x.stream, dtab, dblk, (int)blocks.size(), dwork, dinfo);
  x.launches = pht::tl_launches - l0;
  cudaMemcpyAsync(info, dinfo, sizeof(int) * (size_t)count, cudaMemcpyDeviceToHost, x.stream);
  const int rc = finish(x);
  cudaFree(buf);
  cudaSetDevice(prev);
  return rc;
}

extern "C" int paraht_hgeqz_eigs(int count, const int* n, const double* const* H, const int* ldh,
                                 const double* const* T, const int* ldt, double* const* alphar, double* const* alphai,
                                 double* const* beta, int* info) {
  if (const int bad = hgeqz_check(count, n, H, ldh, T, ldt, alphar, alphai, beta, info)) return bad;
  if (count == 0) return 0;
  paraht_ctx c;
  int rc = default_ctx(&c);
  if (rc) return rc;
  // device copies: per pencil H, T (n x n, leading dimension n) and the three output vectors
  std::vector<long long> off((size_t)count + 1, 0);
  for (int i = 0; i < count; ++i) off[i + 1] = off[i] + 2ll * n[i] * n[i] + 3ll * n[i];
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (size_t)std::max(1ll, off[count])) != cudaSuccess) {
    cudaGetLastError();
    return PARAHT_ERR_ALLOC;
  }
  std::vector<const double*> dH(count), dT(count);
  std::vector<double*> dar(count), dai(count), dbe(count);
  std::vector<int> ld(count);
  for (int i = 0; i < count && !rc; ++i) {
    const size_t m = (size_t)n[i];
    double* p = d + off[i];
    dH[i] = p;
    dT[i] = p + m * m;
    dar[i] = p + 2 * m * m;
    dai[i] = dar[i] + m;
    dbe[i] = dai[i] + m;
    ld[i] = std::max(1, n[i]);
    if (m && (cudaMemcpy2D(p, m * sizeof(double), H[i], (size_t)ldh[i] * sizeof(double), m * sizeof(double), m,
                           cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy2D(p + m * m, m * sizeof(double), T[i], (size_t)ldt[i] * sizeof(double), m * sizeof(double),
                           m, cudaMemcpyHostToDevice) != cudaSuccess))
      rc = PARAHT_ERR_CUDA;
  }
  if (!rc) rc = paraht_hgeqz_eigs_d(c, count, n, dH.data(), ld.data(), dT.data(), ld.data(), dar.data(), dai.data(),
                                    dbe.data(), info);
  for (int i = 0; i < count && !rc; ++i) {
    const size_t b = sizeof(double) * (size_t)n[i];
    if (n[i] && info[i] == 0 &&
        (cudaMemcpy(alphar[i], dar[i], b, cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(alphai[i], dai[i], b, cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(beta[i], dbe[i], b, cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = PARAHT_ERR_CUDA;
  }
  if (rc == PARAHT_ERR_CUDA) cudaGetLastError();
  cudaFree(d);
  return rc;
}

// ---- DGGHD3-compatible entry ----
static int gghd3_check(char compq, char compz, int n, int ilo, int ihi, const double* A, int lda, const double* B,
                       int ldb, const double* Q, int ldq, const double* Z, int ldz, int r, int p, int nq) {
  auto ok = [](char c) { return c == 'N' || c == 'I' || c == 'V' || c == 'n' || c == 'i' || c == 'v'; };
  if (!ok(compq)) return -1;
  if (!ok(compz)) return -2;
  if (n < 0) return -3;
  if (ilo < 1) return -4;
  if (ihi > n || ihi < ilo - 1) return -5;
  const int ldmin = std::max(1, n);
  if (n > 0 && !A) return -6;
  if (lda < ldmin) return -7;
  if (n > 0 && !B) return -8;
  if (ldb < ldmin) return -9;
  const bool wq = compq != 'N' && compq != 'n', wz = compz != 'N' && compz != 'n';
  if (wq && n > 0 && !Q) return -10;
  if ((wq && ldq < ldmin) || ldq < 1) return -11;
  if (wz && n > 0 && !Z) return -12;
  if ((wz && ldz < ldmin) || ldz < 1) return -13;
  if (r < 1 || r > 64) return -14;
  if (p < 2) return -15;
  if (nq < 1 || nq > r) return -16;
  return 0;
}

// On x's stream; A, B, Q, Z device pointers (Q/Z may be null when not referenced).
static int gghd3_device(Ctx& x, char compq, char compz, int n, int ilo, int ihi, double* A, int lda, double* B,
                        int ldb, double* Q, int ldq, double* Z, int ldz, int r, int p, int nq, int flags) {
  const char cq = (char)toupper(compq), cz = (char)toupper(compz);
  const long long l0 = pht::tl_launches;
  if (cq == 'I') pht::set_identity(x.stream, n, Q, ldq);
  if (cz == 'I') pht::set_identity(x.stream, n, Z, ldz);
  const int m = ihi - ilo + 1;
  int rc = 0;
  if (m >= 2) {
    // Q_s, Z_s (m x m) and one GEMM output of at most n x m
    const size_t need = sizeof(double) * (2 * (size_t)m * m + (size_t)std::max(n, 1) * m);
    if (need > x.gws_bytes) {
      if (x.gws) cudaFree(x.gws);
      x.gws = nullptr;
      x.gws_bytes = 0;
      if (cudaMalloc(&x.gws, need) != cudaSuccess) {
        cudaGetLastError();
        return PARAHT_ERR_ALLOC;
      }
      x.gws_bytes = need;
    }
    double* Qs = x.gws;
    double* Zs = Qs + (size_t)m * m;
    double* Tm = Zs + (size_t)m * m;
    pht::set_identity(x.stream, m, Qs, m);
    pht::set_identity(x.stream, m, Zs, m);
    const size_t o = (size_t)(ilo - 1);
    rc = run_device(x, 3, m, A + o + o * lda, lda, B + o + o * ldb, ldb, Qs, m, Zs, m, r, p, nq,
                    flags & ~(PARAHT_FLAG_TIME_COMPONENTS | PARAHT_FLAG_TIME_CHAIN | PARAHT_FLAG_KERNEL_TIMES));
    if (!rc) {
      auto copy_back = [&](double* dst, int ldd, int rows, int cols) {
        cudaMemcpy2DAsync(dst, (size_t)ldd * sizeof(double), Tm, (size_t)rows * sizeof(double),
                          (size_t)rows * sizeof(double), cols, cudaMemcpyDeviceToDevice, x.stream);
      };
      double* M2[2] = {A, B};
      const int ld2[2] = {lda, ldb};
      for (int k = 0; k < 2; ++k) {
        if (ilo > 1) {  // rows above the block: X(1:ilo-1, ilo:ihi) <- X(1:ilo-1, ilo:ihi) Z_s
          double* top = M2[k] + o * ld2[k];
          pht::dgemm(x.stream, false, ilo - 1, m, m, top, ld2[k], Zs, m, Tm, ilo - 1);
          copy_back(top, ld2[k], ilo - 1, m);
        }
        if (ihi < n) {  // columns right of the block: X(ilo:ihi, ihi+1:n) <- Q_s^T X(ilo:ihi, ihi+1:n)
          double* right = M2[k] + o + (size_t)ihi * ld2[k];
          pht::dgemm(x.stream, true, m, n - ihi, m, Qs, m, right, ld2[k], Tm, m);
          copy_back(right, ld2[k], m, n - ihi);
        }
      }
      if (cq != 'N') {  // Q(:, ilo:ihi) <- Q(:, ilo:ihi) Q_s
        double* blk = Q + o * ldq;
        pht::dgemm(x.stream, false, n, m, m, blk, ldq, Qs, m, Tm, n);
        copy_back(blk, ldq, n, m);
      }
      if (cz != 'N') {
        double* blk = Z + o * ldz;
        pht::dgemm(x.stream, false, n, m, m, blk, ldz, Zs, m, Tm, n);
        copy_back(blk, ldz, n, m);
      }
    }
  }
  if (!rc) rc = finish(x);
  x.launches = pht::tl_launches - l0;
  return rc;
}

extern "C" int paraht_gghd3_d(paraht_ctx c, char compq, char compz, int n, int ilo, int ihi, double* A, int lda,
                              double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r, int p, int nq,
                              int flags) {
  if (!ctx_ok(c)) return PARAHT_ERR_BAD_CTX;
  int rc = gghd3_check(compq, compz, n, ilo, ihi, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq);
  if (rc || n == 0) return rc;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  rc = gghd3_device(x, compq, compz, n, ilo, ihi, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags);
  cudaSetDevice(prev);
  return rc;
}

extern "C" int paraht_gghd3(char compq, char compz, int n, int ilo, int ihi, double* A, int lda, double* B, int ldb,
                            double* Q, int ldq, double* Z, int ldz, int r, int p, int nq, int flags) {
  int rc = gghd3_check(compq, compz, n, ilo, ihi, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq);
  if (rc || n == 0) return rc;
  paraht_ctx c;
  rc = default_ctx(&c);
  if (rc) return rc;
  Ctx& x = c->c;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(x.device);
  const int ldd = (n + 3) & ~3;
  rc = x.ensure_staging((size_t)ldd * n * sizeof(double));
  if (!rc) {
    const bool wq = toupper(compq) != 'N', wz = toupper(compz) != 'N';
    double* h[4] = {A, B, Q, Z};
    const int ld[4] = {lda, ldb, ldq, ldz};
    const bool use[4] = {true, true, wq, wz};
    for (int i = 0; i < 4; ++i)
      if (use[i] && !(i >= 2 && toupper(i == 2 ? compq : compz) == 'I'))
        cudaMemcpy2DAsync(x.stage[i], (size_t)ldd * sizeof(double), h[i], (size_t)ld[i] * sizeof(double),
                          (size_t)n * sizeof(double), n, cudaMemcpyHostToDevice, x.stream);
    rc = gghd3_device(x, compq, compz, n, ilo, ihi, x.stage[0], ldd, x.stage[1], ldd, wq ? x.stage[2] : nullptr, ldd,
                      wz ? x.stage[3] : nullptr, ldd, r, p, nq, flags);
    if (!rc)
      for (int i = 0; i < 4; ++i)
        if (use[i])
          cudaMemcpy2DAsync(h[i], (size_t)ld[i] * sizeof(double), x.stage[i], (size_t)ldd * sizeof(double),
                            (size_t)n * sizeof(double), n, cudaMemcpyDeviceToHost, x.stream);
    const int rc2 = finish(x);
    if (!rc) rc = rc2;
  }
  cudaSetDevice(prev);
  return rc;
}

extern "C" const char* paraht_strerror(int s) {
  switch (s) {
    case PARAHT_OK:
      return "success";
    case PARAHT_ERR_CUDA:
      return "CUDA runtime error";
    case PARAHT_ERR_ALLOC:
      return "allocation failed";
    case PARAHT_ERR_TIMEOUT:
      return "device-side wait timed out";
    case PARAHT_ERR_NONFINITE:
      return "non-finite input";
    case PARAHT_ERR_TOO_LARGE:
      return "problem needs more scratch than the fixed array of paraht_rht2ht_d_noalloc";
    case PARAHT_ERR_NOT_SUPPORTED:
      return "not supported";
    case PARAHT_ERR_NO_DEVICE:
      return "no CUDA device";
    case PARAHT_ERR_BAD_CTX:
      return "invalid context";
    default:
      return s < 0 && s >= -20 ? "invalid argument" : "unknown status";
  }
}

extern "C" int paraht_version(void) { return PARAHT_VERSION; }
