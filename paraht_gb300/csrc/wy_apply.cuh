// wy_apply.cuh -- FP64 application of ordered compact-WY op lists to column strips / row strips.
//
// Each CTA owns a strip of the target matrix (CS columns for left ops, RS rows for right ops)
// and walks the whole op list in order, applying every op that touches the strip.  Ops that
// overlap are therefore applied in list order for every entry, which is the ordering the
// reference's taskloops give each row/column chunk (e.g. src/ab2rht.f90:149-166,
// src/rht2ht.f90:1818-1844).  Strips are independent, so there is no inter-CTA sync.
//
// Geometry classes provide   int count() const;   pht::WYOp op(int i) const;   (device)
#pragma once
#include "launch_count.h"
#include "paraht_internal.cuh"

namespace pht {

constexpr int kApplyThreads = 256;
constexpr int kLeftCS = 32;    // columns per CTA (left ops)
constexpr int kLeftRCH = 128;  // row chunk staged in shared memory
constexpr int kRightCCH = 64;  // column chunk staged in shared memory
constexpr int kMaxK = 64;      // max reflectors per op

// X <- H^T X on the column strip [cbeg, cend] (at most kLeftCS columns) for every op
// (dlarfb 'L','T','F','C'); kApplyThreads threads, shared memory kLeftSmem at smx.  When
// `flops` is given, the op's algorithmic work (4 len k flops per column) is added to it.
template <class Geo>
__device__ void apply_left_strip(double* __restrict__ X, int ldx, int cbeg, int cend, const Geo& g, double* smx,
                                 unsigned long long* flops = nullptr) {
  double(*Xs)[kLeftCS + 1] = reinterpret_cast<double(*)[kLeftCS + 1]>(smx);
  double(*W)[kLeftCS + 1] = reinterpret_cast<double(*)[kLeftCS + 1]>(smx + kLeftRCH * (kLeftCS + 1));
  const int t = threadIdx.x;
  const int nops = g.count();
  for (int o = 0; o < nops; ++o) {
    const WYOp op = g.op(o);
    const int ca = max(cbeg, op.lo), cb = min(cend, op.hi);
    if (ca > cb || op.k <= 0 || op.len <= 0) continue;
    const int w = cb - ca + 1;
    const int k = op.k;
    if (flops && t == 0) atomicAdd(flops, op_row_flops(op) * (unsigned long long)w);
    // ---- pass 1: W = V^T X_sub (k x w) ----
    for (int i = t; i < kMaxK * kLeftCS; i += kApplyThreads) W[i / kLeftCS][i % kLeftCS] = 0.0;
    for (int r0 = 0; r0 < op.len; r0 += kLeftRCH) {
      const int rl = min(kLeftRCH, op.len - r0);
      __syncthreads();
      for (int e = t; e < kLeftRCH * kLeftCS; e += kApplyThreads) {
        const int i = e % kLeftRCH, c = e / kLeftRCH;
        Xs[i][c] = (i < rl && c < w) ? X[(size_t)(op.start + r0 + i) + (size_t)(ca + c) * ldx] : 0.0;
      }
      __syncthreads();
      const int c = t % kLeftCS, mg = t / kLeftCS;  // 8 groups of m
      for (int m = mg; m < k; m += kApplyThreads / kLeftCS) {
        const double* v = op.V + (size_t)m * op.ldv + r0;
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        int i = 0;
        for (; i + 3 < rl; i += 4) {
          a0 = fma(v[i], Xs[i][c], a0);
          a1 = fma(v[i + 1], Xs[i + 1][c], a1);
          a2 = fma(v[i + 2], Xs[i + 2][c], a2);
          a3 = fma(v[i + 3], Xs[i + 3][c], a3);
        }
        for (; i < rl; ++i) a0 = fma(v[i], Xs[i][c], a0);
        W[m][c] += (a0 + a1) + (a2 + a3);
      }
    }
    __syncthreads();
    // ---- W2 = T^T W: W2[m] = sum_l T[l][m] W[l]  (T is stored with explicit zeros) ----
    {
      const int c = t % kLeftCS, mg = t / kLeftCS;
      double acc[kMaxK / (kApplyThreads / kLeftCS)];
      int cnt = 0;
      for (int m = mg; m < k; m += kApplyThreads / kLeftCS) {
        const double* tc = op.T + (size_t)m * op.ldt;
        double s = 0.0;
        for (int l = 0; l < k; ++l) s = fma(tc[l], W[l][c], s);
        acc[cnt++] = s;
      }
      __syncthreads();
      cnt = 0;
      for (int m = mg; m < k; m += kApplyThreads / kLeftCS) W[m][c] = acc[cnt++];
    }
    // ---- pass 2: X_sub -= V W2 ----
    for (int r0 = 0; r0 < op.len; r0 += kLeftRCH) {
      const int rl = min(kLeftRCH, op.len - r0);
      __syncthreads();
      for (int e = t; e < kLeftRCH * kLeftCS; e += kApplyThreads) {
        const int i = e % kLeftRCH, c = e / kLeftRCH;
        if (i < rl && c < w) Xs[i][c] = X[(size_t)(op.start + r0 + i) + (size_t)(ca + c) * ldx];
      }
      __syncthreads();
      const int c = t % kLeftCS;
      for (int i = t / kLeftCS; i < rl; i += kApplyThreads / kLeftCS) {
        double s = 0.0;
        for (int m = 0; m < k; ++m) s = fma(op.V[(size_t)m * op.ldv + r0 + i], W[m][c], s);
        Xs[i][c] -= s;
      }
      __syncthreads();
      for (int e = t; e < kLeftRCH * kLeftCS; e += kApplyThreads) {
        const int i = e % kLeftRCH, c = e / kLeftRCH;
        if (i < rl && c < w) X[(size_t)(op.start + r0 + i) + (size_t)(ca + c) * ldx] = Xs[i][c];
      }
    }
    __syncthreads();
  }
}

template <class Geo>
__global__ void __launch_bounds__(kApplyThreads) k_apply_left(double* __restrict__ X, int ldx, int col0, int col1,
                                                               Geo g, unsigned long long* flops) {
  extern __shared__ double smx[];
  const int cbeg = col0 + blockIdx.x * kLeftCS;
  if (cbeg > col1) return;
  apply_left_strip(X, ldx, cbeg, min(col1, cbeg + kLeftCS - 1), g, smx, flops);
}

// X <- X H on the row strip [rbeg, rend] (at most kRightRS rows) for every op
// (dlarfb 'R','N','F','C'); kApplyThreads threads, shared memory right_smem<kRightRS>() at smx.
// Each row's arithmetic is the same for every strip height: RS = 64 for bulk lists, 8 for small
// critical-path updates (spread over more SMs).
template <class Geo, int kRightRS = 64>
__device__ void apply_right_strip(double* __restrict__ X, int ldx, int rbeg, int rend, const Geo& g, double* smx,
                                  unsigned long long* flops = nullptr) {
  double(*Xs)[kRightRS + 1] = reinterpret_cast<double(*)[kRightRS + 1]>(smx);
  double(*Y)[kRightRS + 1] = reinterpret_cast<double(*)[kRightRS + 1]>(smx + kRightCCH * (kRightRS + 1));
  const int t = threadIdx.x;
  const int nops = g.count();
  constexpr int kGroups = kApplyThreads / kRightRS;
  for (int o = 0; o < nops; ++o) {
    const WYOp op = g.op(o);
    const int ra = max(rbeg, op.lo), rb = min(rend, op.hi);
    if (ra > rb || op.k <= 0 || op.len <= 0) continue;
    const int h = rb - ra + 1;
    const int k = op.k;
    if (flops && t == 0) atomicAdd(flops, op_row_flops(op) * (unsigned long long)h);
    for (int i = t; i < kMaxK * kRightRS; i += kApplyThreads) Y[i / kRightRS][i % kRightRS] = 0.0;
    // ---- pass 1: Y = X_sub V (h x k) ----
    for (int c0 = 0; c0 < op.len; c0 += kRightCCH) {
      const int cl = min(kRightCCH, op.len - c0);
      __syncthreads();
      for (int e = t; e < kRightCCH * kRightRS; e += kApplyThreads) {
        const int rr = e % kRightRS, c = e / kRightRS;
        Xs[c][rr] = (rr < h && c < cl) ? X[(size_t)(ra + rr) + (size_t)(op.start + c0 + c) * ldx] : 0.0;
      }
      __syncthreads();
      const int rr = t % kRightRS, mg = t / kRightRS;
      for (int m = mg; m < k; m += kGroups) {
        const double* v = op.V + (size_t)m * op.ldv + c0;
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        int c = 0;
        for (; c + 3 < cl; c += 4) {
          a0 = fma(Xs[c][rr], v[c], a0);
          a1 = fma(Xs[c + 1][rr], v[c + 1], a1);
          a2 = fma(Xs[c + 2][rr], v[c + 2], a2);
          a3 = fma(Xs[c + 3][rr], v[c + 3], a3);
        }
        for (; c < cl; ++c) a0 = fma(Xs[c][rr], v[c], a0);
        Y[m][rr] += (a0 + a1) + (a2 + a3);
      }
    }
    __syncthreads();
    // ---- Y2 = Y T: Y2[m] = sum_l Y[l] T[l][m]  (upper T for forward, lower for backward) ----
    {
      const int rr = t % kRightRS, mg = t / kRightRS;
      double acc[kMaxK / kGroups];
      int cnt = 0;
      for (int m = mg; m < k; m += kGroups) {
        const double* tc = op.T + (size_t)m * op.ldt;
        double s = 0.0;
        for (int l = 0; l < k; ++l) s = fma(Y[l][rr], tc[l], s);
        acc[cnt++] = s;
      }
      __syncthreads();
      cnt = 0;
      for (int m = mg; m < k; m += kGroups) Y[m][rr] = acc[cnt++];
    }
    // ---- pass 2: X_sub -= Y2 V^T ----
    for (int c0 = 0; c0 < op.len; c0 += kRightCCH) {
      const int cl = min(kRightCCH, op.len - c0);
      __syncthreads();
      for (int e = t; e < kRightCCH * kRightRS; e += kApplyThreads) {
        const int rr = e % kRightRS, c = e / kRightRS;
        if (rr < h && c < cl) Xs[c][rr] = X[(size_t)(ra + rr) + (size_t)(op.start + c0 + c) * ldx];
      }
      __syncthreads();
      const int rr = t % kRightRS;
      for (int c = t / kRightRS; c < cl; c += kGroups) {
        double s = 0.0;
        for (int m = 0; m < k; ++m) s = fma(Y[m][rr], op.V[(size_t)m * op.ldv + c0 + c], s);
        Xs[c][rr] -= s;
      }
      __syncthreads();
      for (int e = t; e < kRightCCH * kRightRS; e += kApplyThreads) {
        const int rr = e % kRightRS, c = e / kRightRS;
        if (rr < h && c < cl) X[(size_t)(ra + rr) + (size_t)(op.start + c0 + c) * ldx] = Xs[c][rr];
      }
    }
    __syncthreads();
  }
}

template <class Geo, int kRightRS = 64>
__global__ void __launch_bounds__(kApplyThreads) k_apply_right(double* __restrict__ X, int ldx, int row0, int row1,
                                                                Geo g, unsigned long long* flops) {
  extern __shared__ double smx[];
  const int rbeg = row0 + blockIdx.x * kRightRS;
  if (rbeg > row1) return;
  apply_right_strip<Geo, kRightRS>(X, ldx, rbeg, min(row1, rbeg + kRightRS - 1), g, smx, flops);
}

constexpr size_t kLeftSmem = sizeof(double) * (size_t)(kLeftRCH + kMaxK) * (kLeftCS + 1);
template <int RS>
constexpr size_t right_smem() { return sizeof(double) * (size_t)(kRightCCH + kMaxK) * (RS + 1); }

// Launch helpers: one CTA per strip; the dynamic shared-memory opt-in is set once per
// instantiation.  Under PARAHT_FLAG_KERNEL_TIMES (tl_kclock set) every bulk launch is bracketed
// by a pair of CUDA events on its stream and counts its algorithmic flops on the device; the
// 8-row critical-path lists are not timed (they sit on the serial chain, where the events would
// add to it).
template <class Geo>
inline void launch_apply_left(double* X, int ldx, int col0, int col1, const Geo& g, cudaStream_t s) {
  if (col1 < col0) return;
  static std::atomic<unsigned long long> done{0};
  smem_once((const void*)k_apply_left<Geo>, kLeftSmem, done);
  const int nblk = (col1 - col0 + 1 + kLeftCS - 1) / kLeftCS;
  count_launch();
  KernelClock* kc = tl_kclock;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool timed = kc && kc->pair(Geo::kSite, &e0, &e1);
  if (timed) cudaEventRecord(e0, s);
  k_apply_left<Geo><<<nblk, kApplyThreads, kLeftSmem, s>>>(X, ldx, col0, col1, g,
                                                           timed ? kc->dflops + Geo::kSite : nullptr);
  if (timed) cudaEventRecord(e1, s);
}
template <class Geo, int RS = 64>
inline void launch_apply_right(double* X, int ldx, int row0, int row1, const Geo& g, cudaStream_t s) {
  if (row1 < row0) return;
  static std::atomic<unsigned long long> done{0};
  smem_once((const void*)k_apply_right<Geo, RS>, right_smem<RS>(), done);
  const int nblk = (row1 - row0 + 1 + RS - 1) / RS;
  count_launch();
  KernelClock* kc = tl_kclock;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool timed = RS == 64 && kc && kc->pair(Geo::kSite, &e0, &e1);
  if (timed) cudaEventRecord(e0, s);
  k_apply_right<Geo, RS><<<nblk, kApplyThreads, right_smem<RS>(), s>>>(X, ldx, row0, row1, g,
                                                                       timed ? kc->dflops + Geo::kSite : nullptr);
  if (timed) cudaEventRecord(e1, s);
}

}  // namespace pht
