// prof.cu -- launch counter and per-kernel-class CUDA-event timing.
#include <vector>

#include "common.cuh"

namespace zg {

std::atomic<unsigned long long> g_launches{0};
bool g_profiling = false;

namespace {
struct Pending {
  cudaEvent_t b, e;
  int tag;
  double flops, bytes;
};
std::mutex g_pmu;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
struct Acc {
  unsigned long long launches = 0;
  double ms = 0, flops = 0, bytes = 0;
} g_acc[kNumTags];

cudaEvent_t take() {
  if (g_pool.empty()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t e = g_pool.back();
  g_pool.pop_back();
  return e;
}

void drain_locked() {
  for (auto &p : g_pending) {
    float ms = 0;
    if (cudaEventSynchronize(p.e) == cudaSuccess && cudaEventElapsedTime(&ms, p.b, p.e) == cudaSuccess) {
      Acc &a = g_acc[p.tag];
      a.launches += 1;
      a.ms += ms;
      a.flops += p.flops;
      a.bytes += p.bytes;
    }
    g_pool.push_back(p.b);
    g_pool.push_back(p.e);
  }
  g_pending.clear();
}
}  // namespace

void prof_record(cudaStream_t s, int tag, double, double, cudaEvent_t *begin) {
  std::lock_guard<std::mutex> lk(g_pmu);
  (void)tag;
  *begin = take();
  cudaEventRecord(*begin, s);
}

void prof_end(cudaStream_t s, cudaEvent_t begin, int tag, double flops, double bytes) {
  std::lock_guard<std::mutex> lk(g_pmu);
  if (!begin) return;
  cudaEvent_t e = take();
  cudaEventRecord(e, s);
  g_pending.push_back({begin, e, tag, flops, bytes});
  if (g_pending.size() > 20000) drain_locked();
}

}  // namespace zg

using namespace zg;

extern "C" {

// Turns per-kernel-class event timing on (1) or off (0); turning it on clears
// the accumulated figures.
void zml_gpu_profile(int enable) {
  std::lock_guard<std::mutex> lk(g_pmu);
  if (enable) {
    drain_locked();
    for (auto &a : g_acc) a = Acc{};
  }
  g_profiling = enable != 0;
}

// Launches, device milliseconds, algorithmic flops and bytes of one kernel
// class (see ProfTag) since profiling was enabled.  Returns 0, or -1 for a
// bad tag.
int zml_gpu_profile_read(int tag, unsigned long long *launches, double *ms, double *flops,
                         double *bytes) {
  if (tag < 0 || tag >= kNumTags) return -1;
  std::lock_guard<std::mutex> lk(g_pmu);
  drain_locked();
  const Acc &a = g_acc[tag];
  if (launches) *launches = a.launches;
  if (ms) *ms = a.ms;
  if (flops) *flops = a.flops;
  if (bytes) *bytes = a.bytes;
  return 0;
}

// Number of kernels this library has launched in this process.
unsigned long long zml_gpu_launch_count(void) { return g_launches.load(); }

}  // extern "C"
