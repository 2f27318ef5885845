// batched.cu -- many independent pencils reduced by one persistent launch.
//
// A pencil of moderate size leaves most of the GPU idle in the single-pencil path: its critical
// chains (the stage-1 RQ chain, the stage-2 chase) run on one SM at a time and its bulk
// updates are too small to fill 152 SMs.  Here each CTA reduces whole pencils, one after the
// other, taking the next one from a device-side queue ordered by decreasing size (longest
// first), so that up to (resident CTAs) pencils progress at once and the serial chains of
// different pencils overlap.  A CTA runs exactly the single-pencil FP64 path's device bodies
// in one of its valid orders:
//   stage 1 (src/ab2rht.f90:8-495): per panel the left generation (s1_lgen_body), the left
//     updates of B and A and the right update of Q, per block the right generation
//     (s1_rgen_body) and the update of B rows 1..ib2 followed by the zeroing of the block's
//     first nb columns, then the right updates of A and Z;
//   stage 2 (src/rht2ht.f90:1346-2051): per sweep group the sweeps in order (sequential mode of
//     the chase), TV of every block, the lookahead and delayed updates as the same op lists;
//   exact zeros below the Hessenberg and triangular structure.
// Each matrix entry receives the same operations in the same order as in the single-pencil
// path and every per-row / per-column computation is the same code with the same thread
// layout (256 threads), so the results are bitwise those of paraht_reduce_d without
// PARAHT_FLAG_SPLIT.  The CTA's reflector workspace lives in a per-CTA slice of one device
// buffer.
#include <algorithm>
#include <new>
#include <numeric>
#include <string.h>
#include <vector>

#include "launch_count.h"
#include "paraht_impl.h"
#include "stage1_gen.cuh"
#include "stage2_chase.cuh"
#include "stage2_geom.cuh"
#include "wy_apply.cuh"

namespace pht {

constexpr int kBatchThreads = 256;
static_assert(kBatchThreads == kApplyThreads && kBatchThreads == kChaseMaxThreads,
              "the batched kernel runs the apply and chase bodies with their own thread layout");

struct BatchItem {
  double *A, *B, *Q, *Z;
  int n, lda, ldb, ldq, ldz, r, p, nq;
};

// Doubles of reflector workspace one pencil needs (stage 1 and stage 2 use it one after the other).
static size_t batch_ws_doubles(int n, int r, int p, int nq) {
  const size_t L = (size_t)p * r;
  const size_t nblk0 = std::max(1, (n - r + (p - 1) * r - 1) / std::max(1, (p - 1) * r));
  const size_t s1 = nblk0 * (2 * L * r + 2 * (size_t)r * r);
  const size_t nb0 = std::max(1, (n - 1 + r - 1) / r) + 2;
  const size_t ldu = r + nq;
  const size_t s2 = nb0 * (2 * ldu * nq + 2 * (size_t)nq * nq + 2 * (size_t)nq);
  return std::max(s1, s2);
}

// The whole op list on X, strip by strip (the single-pencil kernels run one strip per CTA).
template <class Geo>
static __device__ void apply_left_cta(double* X, int ldx, int col0, int col1, const Geo& g, double* sm) {
  for (int c = col0; c <= col1; c += kLeftCS) apply_left_strip(X, ldx, c, min(col1, c + kLeftCS - 1), g, sm);
  __syncthreads();
}
template <class Geo>
static __device__ void apply_right_cta(double* X, int ldx, int row0, int row1, const Geo& g, double* sm) {
  for (int r = row0; r <= row1; r += 64) apply_right_strip<Geo, 64>(X, ldx, r, min(row1, r + 63), g, sm);
  __syncthreads();
}

static __device__ void batch_stage1(const BatchItem& P, double* ws, double* sm, int use_vr) {
  const int n = P.n, nb = P.r, p = P.p, L = p * nb;
  if (n - nb - 1 < 1) return;  // ab2rht.f90:71: empty panel loop
  const int nblk0 = max(1, (n - nb + (p - 1) * nb - 1) / ((p - 1) * nb));
  double* VL = ws;
  double* VRc = VL + (size_t)L * nb * nblk0;
  double* TL = VRc + (size_t)L * nb * nblk0;
  double* TR = TL + (size_t)nb * nb * nblk0;
  const int t = threadIdx.x;
  for (int jb0 = 0; jb0 <= n - nb - 2; jb0 += nb) {
    const S1Panel Pn = make_panel(n, nb, p, jb0);
    s1_lgen_body(P.A, P.lda, Pn, VL, TL, sm);
    __syncthreads();
    apply_left_cta(P.B, P.ldb, Pn.ib(Pn.nblocks - 1), n - 1, GeoS1Left{Pn, VL, TL, 0}, sm);
    apply_left_cta(P.A, P.lda, jb0 + nb, n - 1, GeoS1Left{Pn, VL, TL, 1}, sm);
    apply_right_cta(P.Q, P.ldq, 0, n - 1, GeoS1Q{Pn, VL, TL}, sm);
    for (int o = 0; o < Pn.nblocks; ++o) {
      s1_rgen_body(P.B, P.ldb, Pn, o, VRc, TR, use_vr, s1_rgen_threads(L), sm);
      __syncthreads();
      // rows 1 .. ib2: the reference's lookahead rows and the remaining rows (ab2rht.f90:317-367)
      GeoS1Right gb{Pn, VRc, TR, o};
      gb.row_lo = 0;
      gb.row_hi = Pn.ib2(o);
      apply_right_cta(P.B, P.ldb, 0, Pn.ib2(o), gb, sm);
      if (Pn.nb2(o) > nb) {  // ab2rht.f90:329-333
        const int ib0 = Pn.ib(o), ib2 = Pn.ib2(o);
        for (int e = t; e < nb * L; e += blockDim.x) {
          const int j = ib0 + e / L, i = j + 1 + e % L;
          if (i <= ib2) P.B[(size_t)i + (size_t)j * P.ldb] = 0.0;
        }
        __syncthreads();
      }
    }
    apply_right_cta(P.A, P.lda, 0, n - 1, GeoS1Right{Pn, VRc, TR, -1}, sm);
    apply_right_cta(P.Z, P.ldz, 0, n - 1, GeoS1Right{Pn, VRc, TR, -1}, sm);
  }
}

static __device__ void batch_stage2(const BatchItem& P, double* ws, double* sm, int* abort_flag) {
  const int n = P.n, r = P.r, nq = P.nq;
  if (n < 3) return;  // rht2ht.f90:1417: empty loop
  const int nb0 = max(1, (n - 1 + r - 1) / r) + 2;
  const int ldu = r + nq;
  S2Store S;
  S.ldu = ldu;
  S.nq = nq;
  S.U = ws;
  S.V = S.U + (size_t)ldu * nq * nb0;
  S.TU = S.V + (size_t)ldu * nq * nb0;
  S.TV = S.TU + (size_t)nq * nq * nb0;
  S.tauU = S.TV + (size_t)nq * nq * nb0;
  S.tauV = S.tauU + (size_t)nq * nb0;
  const int t = threadIdx.x;
  ChaseArgs a;
  a.A = P.A;
  a.lda = P.lda;
  a.B = P.B;
  a.ldb = P.ldb;
  a.n = n;
  a.r = r;
  a.nq = nq;
  a.S = S;
  a.sync.prog = nullptr;
  a.sync.ticket = nullptr;
  a.sync.status = nullptr;
  a.spin_limit = 0;
  a.pipelined = 0;  // one CTA: the sweeps one after the other, no waits
  for (int J = 1; J <= n - 2; J += nq) {  // rht2ht.f90:1417
    const int nblocks = (n - J + r - 1) / r;
    const int nz = min(nb0, nblocks + 2);
    for (size_t e = t; e < (size_t)ldu * nq * nz; e += blockDim.x) {
      S.U[e] = 0.0;
      S.V[e] = 0.0;
    }
    for (size_t e = t; e < (size_t)nq * nz; e += blockDim.x) {
      S.tauU[e] = 0.0;
      S.tauV[e] = 0.0;
    }
    for (size_t e = t; e < (size_t)nq * nq * nz; e += blockDim.x) S.TU[e] = 0.0;
    __syncthreads();
    a.J = J;
    {
      Sm s = chase_sm(sm, r, nq, abort_flag);
      for (int ic = 1; ic <= nq; ++ic) run_sweep(a, ic, s);
    }
    __syncthreads();
    for (int ib = 1; ib <= nblocks; ++ib) {
      s2_form_t_body(n, J, r, nq, ib, S, sm);
      __syncthreads();
    }
    GeoS2 g{S, n, J, r, nq, nblocks, kLaRight};
    g.blk = 0;
    apply_right_cta(P.B, P.ldb, J, n - 1, g, sm);
    apply_right_cta(P.A, P.lda, J, n - 1, g, sm);
    g.kind = kLaLeftB;
    apply_left_cta(P.B, P.ldb, J, n - 1, g, sm);
    g.kind = kLaLeftA;
    apply_left_cta(P.A, P.lda, J, n - 1, g, sm);
    g.kind = kUpRight;
    apply_right_cta(P.B, P.ldb, 0, n - 1, g, sm);
    apply_right_cta(P.A, P.lda, 0, n - 1, g, sm);
    g.kind = kUpLeft;
    apply_left_cta(P.B, P.ldb, J, n - 1, g, sm);
    apply_left_cta(P.A, P.lda, J, n - 1, g, sm);
    g.kind = kUpQ;
    apply_right_cta(P.Q, P.ldq, 0, n - 1, g, sm);
    g.kind = kUpZ;
    apply_right_cta(P.Z, P.ldz, 0, n - 1, g, sm);
  }
}

// Exact zeros below the first subdiagonal of A and below the diagonal of B.
static __device__ void batch_zero_fill(const BatchItem& P) {
  const int n = P.n;
  for (int j = threadIdx.x >> 5; j < n; j += blockDim.x >> 5)
    for (int i = j + 2 + (threadIdx.x & 31); i < n; i += 32) P.A[(size_t)i + (size_t)j * P.lda] = 0.0;
  for (int j = threadIdx.x >> 5; j < n; j += blockDim.x >> 5)
    for (int i = j + 1 + (threadIdx.x & 31); i < n; i += 32) P.B[(size_t)i + (size_t)j * P.ldb] = 0.0;
  __syncthreads();
}

__global__ void __launch_bounds__(kBatchThreads, 2) k_batch_reduce(const BatchItem* __restrict__ items,
                                                                   const int* __restrict__ order, int count,
                                                                   int* next, double* ws, size_t ws_stride,
                                                                   int use_vr) {
  extern __shared__ __align__(16) double smb[];
  __shared__ int s_item, s_abort;
  double* myws = ws + (size_t)blockIdx.x * ws_stride;
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(next, 1);
      s_abort = 0;
    }
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= count) return;
    const BatchItem P = items[order[it]];
    batch_stage1(P, myws, smb, use_vr);
    batch_stage2(P, myws, smb, &s_abort);
    batch_zero_fill(P);
  }
}

// Whether the persistent kernel takes a pencil of these parameters: one CTA of 256 threads runs
// every generation body with the single-pencil thread layout when L = p r <= 64.
bool batch_eligible(int n, int r, int p, int nq) {
  (void)n;
  (void)nq;
  return (size_t)p * r <= 64;
}

// Launch shape of one persistent launch over `count` pencils: shared memory (the largest body; the
// RQ reflector copy of the right generation only if two CTAs still fit per SM), grid, and the
// per-CTA workspace in doubles.
static int batch_shape(Ctx& x, const BatchItem* items, int count, size_t& smem, int& grid, int& use_vr,
                       size_t& wsd) {
  wsd = 0;
  int Lmax = 0, rmax = 0, nqmax = 0;
  for (int k = 0; k < count; ++k) {
    wsd = std::max(wsd, batch_ws_doubles(items[k].n, items[k].r, items[k].p, items[k].nq));
    Lmax = std::max(Lmax, items[k].p * items[k].r);
    rmax = std::max(rmax, items[k].r);
    nqmax = std::max(nqmax, items[k].nq);
  }
  const size_t base = std::max({kLeftSmem, right_smem<64>(), s1_lgen_smem(Lmax, rmax), chase_smem_bytes(rmax, nqmax),
                                sizeof(double) * 2 * (size_t)nqmax * nqmax});
  const size_t with_vr = std::max(base, s1_rgen_smem_vr(Lmax, rmax, true));
  const size_t without_vr = std::max(base, s1_rgen_smem_vr(Lmax, rmax, false));
  use_vr = with_vr <= (size_t)x.max_smem / 2 - 1024 ? 1 : 0;
  smem = use_vr ? with_vr : without_vr;
  if (smem > (size_t)x.max_smem - 1024) return PARAHT_ERR_NOT_SUPPORTED;  // static __shared__ words too
  if (const int rc = smem_at_least((const void*)k_batch_reduce, smem)) return rc;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_reduce, kBatchThreads, smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  grid = std::min(count, per_sm * std::max(1, x.num_sms));
  return 0;
}

// Byte layout of a launch's device buffer: items | order | queue counter | per-CTA workspace
// (256-byte aligned slices).
struct BatchLayout {
  size_t items_b, order_b, stride, total;
};
static BatchLayout batch_layout(int count, size_t wsd, int grid) {
  BatchLayout l;
  l.items_b = ((sizeof(BatchItem) * count + 255) / 256) * 256;
  l.order_b = ((sizeof(int) * count + 255) / 256) * 256;
  l.stride = ((wsd * sizeof(double) + 255) / 256) * 256;
  l.total = l.items_b + l.order_b + 256 + l.stride * grid;
  return l;
}

// Host image of the pencil table and the queue order (longest first: decreasing n).
static void batch_table(const BatchItem* items, int count, const BatchLayout& l, std::vector<char>& host) {
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return items[a].n > items[b].n; });
  host.assign(l.items_b + l.order_b, 0);
  memcpy(host.data(), items, sizeof(BatchItem) * count);
  memcpy(host.data() + l.items_b, order.data(), sizeof(int) * count);
}

static void batch_enqueue_raw(char* d, const BatchLayout& l, int count, int grid, size_t smem, int use_vr,
                              cudaStream_t s) {
  int* dnext = (int*)(d + l.items_b + l.order_b);
  cudaMemsetAsync(dnext, 0, sizeof(int), s);
  count_launch();
  k_batch_reduce<<<grid, kBatchThreads, smem, s>>>((const BatchItem*)d, (const int*)(d + l.items_b), count, dnext,
                                                   (double*)(d + l.items_b + l.order_b + 256), l.stride / sizeof(double),
                                                   use_vr);
}

// Reduces the eligible pencils `idx` of the batch with one persistent launch on stream s.
// Returns 0 or a PARAHT_ERR_* code; the launch is asynchronous.
int batch_run(Ctx& x, cudaStream_t s, const std::vector<int>& idx, const int* n, double* const* A, const int* lda,
              double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z, const int* ldz,
              const int* r, const int* p, const int* nq) {
  const int count = (int)idx.size();
  if (count == 0) return 0;
  std::vector<BatchItem> items(count);
  for (int k = 0; k < count; ++k) {
    const int i = idx[k];
    items[k] = BatchItem{A[i], B[i], Q[i], Z[i], n[i], lda[i], ldb[i], ldq[i], ldz[i], r[i], p[i], nq[i]};
  }
  size_t smem = 0, wsd = 0;
  int grid = 0, use_vr = 0;
  if (const int rc = batch_shape(x, items.data(), count, smem, grid, use_vr, wsd)) return rc;
  const BatchLayout l = batch_layout(count, wsd, grid);
  if (l.total > x.bws_bytes) {
    if (x.bws) cudaFree(x.bws);
    x.bws = nullptr;
    x.bws_bytes = 0;
    if (cudaMalloc(&x.bws, l.total) != cudaSuccess) {
      cudaGetLastError();
      return PARAHT_ERR_ALLOC;
    }
    x.bws_bytes = l.total;
  }
  batch_table(items.data(), count, l, x.bhost);
  cudaMemcpyAsync(x.bws, x.bhost.data(), l.items_b + l.order_b, cudaMemcpyHostToDevice, s);
  batch_enqueue_raw((char*)x.bws, l, count, grid, smem, use_vr, s);
  return cudaGetLastError() == cudaSuccess ? 0 : PARAHT_ERR_CUDA;
}

// ---- plans: one bucket of pencils sharing (r, p, nq), with its own buffer and launch shape ----
struct BatchBucket {
  char* buf = nullptr;
  BatchLayout l{};
  int count = 0, grid = 0, use_vr = 0;
  size_t smem = 0;
};

int batch_bucket_create(Ctx& x, const std::vector<int>& idx, const int* n, double* const* A, const int* lda,
                        double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z,
                        const int* ldz, const int* r, const int* p, const int* nq, void** out) {
  *out = nullptr;
  auto* b = new (std::nothrow) BatchBucket();
  if (!b) return PARAHT_ERR_ALLOC;
  b->count = (int)idx.size();
  std::vector<BatchItem> items(b->count);
  for (int k = 0; k < b->count; ++k) {
    const int i = idx[k];
    items[k] = BatchItem{A[i], B[i], Q[i], Z[i], n[i], lda[i], ldb[i], ldq[i], ldz[i], r[i], p[i], nq[i]};
  }
  size_t wsd = 0;
  int rc = batch_shape(x, items.data(), b->count, b->smem, b->grid, b->use_vr, wsd);
  if (!rc) {
    b->l = batch_layout(b->count, wsd, b->grid);
    if (cudaMalloc((void**)&b->buf, b->l.total) != cudaSuccess) {
      cudaGetLastError();
      b->buf = nullptr;
      rc = PARAHT_ERR_ALLOC;
    }
  }
  if (!rc) {
    std::vector<char> host;
    batch_table(items.data(), b->count, b->l, host);
    if (cudaMemcpy(b->buf, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      rc = PARAHT_ERR_CUDA;
    }
  }
  if (rc) {
    batch_bucket_destroy(b);
    return rc;
  }
  *out = b;
  return 0;
}

void batch_bucket_enqueue(const void* bucket, cudaStream_t s) {
  const auto* b = static_cast<const BatchBucket*>(bucket);
  batch_enqueue_raw(b->buf, b->l, b->count, b->grid, b->smem, b->use_vr, s);
}

void batch_bucket_destroy(void* bucket) {
  auto* b = static_cast<BatchBucket*>(bucket);
  if (!b) return;
  if (b->buf) cudaFree(b->buf);
  delete b;
}

}  // namespace pht
