// Launch accounting: a global count of this library's kernel launches and an
// optional per-class CUDA-event timer.  Events are recorded on the stream the
// kernel is launched on, so a caller can time one kernel class inside a long
// step without a profiler.  Off by default; costs one branch per launch.
#include <atomic>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace candmc {

static std::atomic<long long> g_launches{0};

struct ProfRec {
  cudaEvent_t e0, e1;
  double work;
};

static std::mutex g_prof_mu;
static unsigned g_prof_mask = 0;
static std::vector<ProfRec> g_prof[kProfClasses];

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

long long launch_total() { return g_launches.load(); }

bool prof_on(int cls) { return (g_prof_mask >> cls) & 1u; }

ProfScope::ProfScope(int cls, double work, cudaStream_t s) : cls_(cls), work_(work), s_(s) {
  count_launch();
  if (!prof_on(cls)) {
    cls_ = -1;
    return;
  }
  cudaEventCreate(&e0_);
  cudaEventCreate(&e1_);
  cudaEventRecord(e0_, s_);
}

ProfScope::~ProfScope() {
  if (cls_ < 0) return;
  cudaEventRecord(e1_, s_);
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_prof[cls_].push_back({e0_, e1_, work_});
}

}  // namespace candmc

using namespace candmc;

extern "C" {

long long candmc_launch_count(void) { return g_launches.load(); }

int candmc_profile_begin(unsigned mask) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  for (auto& v : g_prof) {
    for (auto& r : v) {
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
    v.clear();
  }
  g_prof_mask = mask;
  return CANDMC_OK;
}

int candmc_profile_end(int ncls, double* ms, double* work, long long* launches) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_prof_mask = 0;
  int rc = CANDMC_OK;
  for (int c = 0; c < kProfClasses; ++c) {
    double t = 0.0, w = 0.0;
    for (auto& r : g_prof[c]) {
      float e = 0.f;
      cudaError_t err = cudaEventSynchronize(r.e1);
      if (err == cudaSuccess) err = cudaEventElapsedTime(&e, r.e0, r.e1);
      if (err != cudaSuccess) rc = cuda_status(err, "profile events");
      t += e;
      w += r.work;
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
    if (c < ncls) {
      if (ms) ms[c] = t;
      if (work) work[c] = w;
      if (launches) launches[c] = (long long)g_prof[c].size();
    }
    g_prof[c].clear();
  }
  return rc;
}

}  // extern "C"
