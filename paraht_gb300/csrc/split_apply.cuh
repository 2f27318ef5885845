// split_apply.cuh -- FP64 or split-precision application of a compact-WY op list, chosen per
// launch site.
//
// The FP64 kernels are in wy_apply.cuh, the split-precision (emulated FP64 on the FP16 tensor
// cores) kernel in wy_stream.cuh.  A left op C <- C - V T^T V^T C on column-major C is the right
// op C^T <- C^T - C^T V T V^T on the transpose, so the split kernel sees left ops through the
// strides (rs, cs) = (ldx, 1) and right ops through (1, ldx).
#pragma once
#include <algorithm>

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

// Ops [first, first + n) of a list, as a list of their own for the FP64 kernels.
template <class Geo>
struct GeoChunk {
  Geo g;
  int first, n;
  static constexpr int kSite = Geo::kSite;
  __host__ __device__ int count() const { return n; }
  PHT_DEV WYOp op(int o) const { return g.op(first + o); }
};

// A side-stream list, in FP64 applied in launches of at most kSideChunk ops.  Every CTA of a list
// launch applies all of the launch's ops to its strip, so a whole list keeps its CTAs for
// milliseconds; the critical-path kernels (panel factorisations, lookahead updates, the chase)
// are launched on a higher-priority stream but take an SM only when one frees up, and shorter
// side launches free them sooner: one n=8000 FP64 reduction went from 36.2 s to 34.3 s (its
// chase from 14.1 s to 12.9 s).  The split-precision lists stay whole: their CTAs load each
// column window once per launch, and chunking them measured no gain.  The ops still run in list
// order, on one stream.
constexpr int kSideChunk = 32;
// (nops is the number of operand slots to prepare; the list's own length, g.count(), may differ:
// the FP64 path applies a block's staircase reflectors as separate ops)
template <class Geo>
inline void apply_right_side(void* split_slots, double* X, int ldx, int row0, int row1, const Geo& g, int nops,
                             cudaStream_t s, bool prepare = true) {
  if (split_slots) {
    apply_right_any(split_slots, X, ldx, row0, row1, g, nops, s, prepare);
    return;
  }
  const int len = g.count();
  for (int f = 0; f < len; f += kSideChunk)
    launch_apply_right(X, ldx, row0, row1, GeoChunk<Geo>{g, f, std::min(kSideChunk, len - f)}, s);
}
template <class Geo>
inline void apply_left_side(void* split_slots, double* X, int ldx, int col0, int col1, const Geo& g, int nops,
                            cudaStream_t s, bool prepare = true) {
  if (split_slots) {
    apply_left_any(split_slots, X, ldx, col0, col1, g, nops, s, prepare);
    return;
  }
  const int len = g.count();
  for (int f = 0; f < len; f += kSideChunk)
    launch_apply_left(X, ldx, col0, col1, GeoChunk<Geo>{g, f, std::min(kSideChunk, len - f)}, s);
}

}  // namespace pht
