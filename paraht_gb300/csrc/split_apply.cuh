// split_apply.cuh -- FP64 or split-precision application of a compact-WY op list, chosen per
// launch site.
//
// The FP64 kernels are in wy_apply.cuh, the split-precision (emulated FP64 on the FP16 tensor
// cores) kernel in wy_stream.cuh.  A left op C <- C - V T^T V^T C on column-major C is the right
// op C^T <- C^T - C^T V T V^T on the transpose, so the split kernel sees left ops through the
// strides (rs, cs) = (ldx, 1) and right ops through (1, ldx).
#pragma once
#include "wy_apply.cuh"
#include "wy_stream.cuh"

namespace pht {

// Whether every op of a list fits the split-precision kernel (checked from the parameters).
inline bool split_fits(int k_max, int len_max) { return ws_fits(k_max, len_max); }

// Per-op operand slot of the split-precision kernel.
typedef WsOpDigits SplitOpData;

// Prepares the split-precision operands of a list in `split_slots` (nothing in FP64, where
// split_slots is null), so that launches on other streams can apply it with prepare = false once
// they have waited for this stream.
template <class Geo>
inline void prepare_any(void* split_slots, const Geo& g, int nops, cudaStream_t s) {
  if (split_slots && nops > 0) {
    count_launch();
    k_ws_prep<Geo><<<nops, 128, 0, s>>>(g, (WsOpDigits*)split_slots);
  }
}

// `split_slots` non-null selects split precision; its `nops` slots receive the prepared operands
// (prepare = false: they already hold this list's operands, prepared by an earlier call with the
// same ops on the same stream).
template <class Geo>
inline void apply_left_any(void* split_slots, double* X, int ldx, int col0, int col1, const Geo& g, int nops,
                           cudaStream_t s, bool prepare = true) {
  if (split_slots)
    launch_ws_apply(X, (long long)ldx, 1LL, col0, col1, g, nops, (WsOpDigits*)split_slots, s, prepare);
  else
    launch_apply_left(X, ldx, col0, col1, g, s);
}
template <class Geo>
inline void apply_right_any(void* split_slots, double* X, int ldx, int row0, int row1, const Geo& g, int nops,
                            cudaStream_t s, bool prepare = true) {
  if (split_slots)
    launch_ws_apply(X, 1LL, (long long)ldx, row0, row1, g, nops, (WsOpDigits*)split_slots, s, prepare);
  else
    launch_apply_right(X, ldx, row0, row1, g, s);
}

}  // namespace pht
