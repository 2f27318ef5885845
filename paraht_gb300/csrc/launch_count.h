// launch_count.h -- per-host-thread count of kernels launched by the library (reported per call
// through paraht_ctx_launch_count).
#pragma once

namespace pht {
extern thread_local long long tl_launches;
inline void count_launch(long long k = 1) { tl_launches += k; }
}  // namespace pht
