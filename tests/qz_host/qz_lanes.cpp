// Host build of the GPU QZ core (paraht_gb300/csrc/qz_real.cuh, real double shift) for the CPU
// tests: `nlanes` host
// threads stand in for the lanes of one pencil, a std::barrier for each lane synchronisation and
// a barrier-published maximum for the lane reduction, so a missing synchronisation in the
// lane-split loops shows up here as a wrong result, a lane-dependent status (99) or a deadlock
// (the test runs under a timeout) instead of on a GPU.  nlanes = 1 is the plain host path.
#include <barrier>
#include <thread>
#include <vector>

static thread_local std::barrier<>* tl_bar = nullptr;
static thread_local int tl_lane = 0, tl_nlanes = 1;
static int g_lane_vals[256];

static int lanes_max(int v) {
  tl_bar->arrive_and_wait();  // every lane has read the previous maximum
  g_lane_vals[tl_lane] = v;
  tl_bar->arrive_and_wait();
  int m = g_lane_vals[0];
  for (int l = 1; l < tl_nlanes; ++l) m = g_lane_vals[l] > m ? g_lane_vals[l] : m;
  return m;
}

#define PHT_QZ_SYNC() tl_bar->arrive_and_wait()
#define PHT_QZ_LANE_MAX(v) lanes_max(v)
#include "qz_real.cuh"

// Eigenvalues of (H, T) (column-major, leading dimensions ldh, ldt; entries below the structure
// ignored) as (alphar + i alphai) / beta with beta >= 0, as the device kernel reports them.
// Returns qz_real_eigs's status, or 99 if the lanes disagreed on it.
extern "C" int qzr_lanes(int nlanes, int n, const double* H, int ldh, const double* T, int ldt, double* alphar,
                         double* alphai, double* beta) {
  if (nlanes < 1 || nlanes > 256 || n < 0) return -1;
  std::vector<double> h((size_t)n * n), t((size_t)n * n), ar(n), ai(n), be(n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      h[(size_t)j * n + i] = i <= j + 1 ? H[(size_t)j * ldh + i] : 0.0;
      t[(size_t)j * n + i] = i <= j ? T[(size_t)j * ldt + i] : 0.0;
    }
  std::barrier<> bar(nlanes);
  std::vector<int> rc(nlanes);
  std::vector<std::thread> lanes;
  for (int l = 0; l < nlanes; ++l)
    lanes.emplace_back([&, l] {
      tl_bar = &bar;
      tl_lane = l;
      tl_nlanes = nlanes;
      rc[l] = pht::qz_real_eigs(n, h.data(), t.data(), n, ar.data(), ai.data(), be.data(), pht::QzLanes{l, nlanes});
    });
  for (auto& th : lanes) th.join();
  for (int l = 1; l < nlanes; ++l)
    if (rc[l] != rc[0]) return 99;
  if (rc[0] == 0)
    for (int j = 0; j < n; ++j) {
      alphar[j] = ar[j];
      alphai[j] = ai[j];
      beta[j] = be[j];
    }
  return rc[0];
}
