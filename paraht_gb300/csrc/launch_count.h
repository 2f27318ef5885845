// launch_count.h -- per-host-thread count of kernels launched by the library (reported per call
// through paraht_ctx_launch_count).
#pragma once

#include <cuda_runtime.h>

namespace pht {
extern thread_local long long tl_launches;
inline void count_launch(long long k = 1) { tl_launches += k; }

// Timing of selected launches (PARAHT_FLAG_KERNEL_TIMES): a launch site asks for an event pair
// of its site (0: stage-1 op lists, 1: stage-2 op lists) and records it around the launch; the
// kernel adds its algorithmic flops to dflops[site].
struct KernelClock {
  unsigned long long* dflops = nullptr;     // device counters, one per site
  bool pair(int site, cudaEvent_t* e0, cudaEvent_t* e1);  // false: out of events
};
extern thread_local KernelClock* tl_kclock;
}  // namespace pht
