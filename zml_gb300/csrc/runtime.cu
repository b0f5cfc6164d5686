// runtime.cu -- error reporting, device query, per-stream workspaces.
#include "common.cuh"

#include <cstdarg>
#include <map>
#include <utility>
#include <vector>

namespace zg {

static thread_local char g_last_error[512] = "";

void set_last_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

const char *last_error() { return g_last_error; }

static std::mutex g_mu;
static std::map<int, DeviceInfo> g_dev;

int device_info(DeviceInfo *out) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_dev.find(dev);
  if (it == g_dev.end()) {
    DeviceInfo d;
    d.device = dev;
    cudaDeviceProp p;
    ZG_CUDA(cudaGetDeviceProperties(&p, dev));
    d.num_sms = p.multiProcessorCount;
    d.cc_major = p.major;
    d.cc_minor = p.minor;
    d.smem_optin = p.sharedMemPerBlockOptin;
    it = g_dev.emplace(dev, d).first;
  }
  *out = it->second;
  return 0;
}

static std::vector<int (*)(long long)> &spin_setters() {
  static std::vector<int (*)(long long)> v;  // built during static initialisation
  return v;
}

int register_spin_setter(int (*set)(long long)) {
  spin_setters().push_back(set);
  return 0;
}

int set_spin_limit(long long tries) {
  if (tries <= 0) tries = kSpinLimit;
  for (auto set : spin_setters()) {
    if (set(tries) != 0) {
      set_last_error("set_spin_limit: cudaMemcpyToSymbol failed");
      return kErrCuda;
    }
  }
  return 0;
}

static std::map<std::pair<int, const void *>, int> g_smem_optin;

int smem_optin_raw(const void *func, int bytes) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  int &have = g_smem_optin[{dev, func}];
  if (bytes > have) {
    ZG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    have = bytes;
  }
  return 0;
}

struct StreamState {
  Workspace ws[kNumSlots];
  Control *ctl = nullptr;
};

static std::map<std::pair<int, cudaStream_t>, StreamState> g_streams;

static StreamState *state_for(cudaStream_t s, int *err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *err = kErrCuda;
    return nullptr;
  }
  *err = 0;
  return &g_streams[{dev, s}];
}

int workspace(cudaStream_t stream, int slot, size_t bytes, void **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  int err;
  StreamState *st = state_for(stream, &err);
  if (!st) return err;
  if (slot < 0 || slot >= kNumSlots) {
    set_last_error("workspace: bad slot %d", slot);
    return kErrInvalid;
  }
  Workspace &w = st->ws[slot];
  if (w.bytes < bytes) {
    if (w.ptr) {
      ZG_CUDA(cudaStreamSynchronize(stream));
      cudaFree(w.ptr);
      w.ptr = nullptr;
      w.bytes = 0;
    }
    size_t want = bytes + (bytes >> 3) + 256;
    if (cudaMalloc(&w.ptr, want) != cudaSuccess) {
      cudaGetLastError();
      set_last_error("workspace: cudaMalloc(%zu) failed", want);
      return kErrAlloc;
    }
    w.bytes = want;
  }
  *out = w.ptr;
  return 0;
}

static std::mutex g_la_mu;
static std::map<std::pair<int, cudaStream_t>, Lookahead> g_la;

int lookahead(cudaStream_t s, Lookahead **out) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_la_mu);
  Lookahead &l = g_la[{dev, s}];
  if (!l.panel) {
    int least = 0, greatest = 0;
    ZG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    ZG_CUDA(cudaStreamCreateWithPriority(&l.panel, cudaStreamNonBlocking, greatest));
    ZG_CUDA(cudaStreamCreateWithPriority(&l.bulk, cudaStreamNonBlocking, least));
    const unsigned fl = cudaEventDisableTiming;
    ZG_CUDA(cudaEventCreateWithFlags(&l.first, fl));
    ZG_CUDA(cudaEventCreateWithFlags(&l.end_panel, fl));
    ZG_CUDA(cudaEventCreateWithFlags(&l.end_bulk, fl));
    for (int q = 0; q < Lookahead::kRing; ++q) {
      ZG_CUDA(cudaEventCreateWithFlags(&l.upd[q], fl));
      ZG_CUDA(cudaEventCreateWithFlags(&l.bulk_done[q], fl));
    }
  }
  *out = &l;
  return 0;
}

int control(cudaStream_t stream, Control **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  int err;
  StreamState *st = state_for(stream, &err);
  if (!st) return err;
  if (!st->ctl) {
    if (cudaMalloc(&st->ctl, sizeof(Control)) != cudaSuccess) {
      cudaGetLastError();
      set_last_error("control: cudaMalloc failed");
      return kErrAlloc;
    }
  }
  ZG_CUDA(cudaMemsetAsync(st->ctl, 0, sizeof(Control), stream));
  *out = st->ctl;
  return 0;
}

int check_status(cudaStream_t stream, Control *ctl, int *info_out) {
  Control h;
  ZG_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(Control), cudaMemcpyDeviceToHost, stream));
  ZG_CUDA(cudaStreamSynchronize(stream));
  if (h.status) {
    set_last_error("device-side wait timed out (status 0x%x)", h.status);
    return kErrTimeout;
  }
  if (info_out) *info_out = h.info;
  return 0;
}

}  // namespace zg
