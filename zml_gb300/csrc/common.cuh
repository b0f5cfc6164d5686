// common.cuh -- shared runtime pieces of the zml_gb300 CUDA library (sm_103a).
//
// Conventions used by every kernel file:
//   * matrices are column-major with a leading dimension (the LAPACK layout
//     zml's Zig kernels use after their row-major -> column-major swaps,
//     linalg/blas/gemm.zig:48-65); row-major callers are transposed at the
//     C-ABI boundary;
//   * enum values are the CBLAS codes (reference include/cblas.h:11-38);
//   * no kernel traps or asserts: every wait is bounded and reports through a
//     device status word that the host reads after the launch.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>

namespace zg {

enum : int {
  kRowMajor = 101, kColMajor = 102,
  kNoTrans = 111, kTrans = 112, kConjTrans = 113, kConjNoTrans = 114,
  kUpper = 121, kLower = 122,
  kNonUnit = 131, kUnit = 132,
  kLeft = 141, kRight = 142,
};

// Library error codes (negative, below every LAPACK -(argument index)).
enum : int {
  kErrCuda = -1001,      // a CUDA runtime call failed (see zml_gpu_last_error)
  kErrAlloc = -1002,     // device allocation failed
  kErrNoDevice = -1003,  // no usable sm_103 device
  kErrTimeout = -1004,   // a bounded device-side wait gave up
  kErrInvalid = -1005,   // invalid argument to an extension entry point
};

// Status bits written by kernels into the per-call device status word.
enum : unsigned { kStatusBarrierTimeout = 1u, kStatusQueueTimeout = 2u, kStatusMbarTimeout = 4u };

void set_last_error(const char *fmt, ...);
const char *last_error();

#define ZG_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ::zg::set_last_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                  \
                           cudaGetErrorString(e_));                                    \
      return ::zg::kErrCuda;                                                           \
    }                                                                                  \
  } while (0)

#define ZG_TRY(expr)          \
  do {                        \
    int r_ = (expr);          \
    if (r_ < 0) return r_;    \
  } while (0)

// ---------------------------------------------------------------------------
// Per-(device, stream) workspace.  Calls are stream ordered; two calls on the
// same stream reuse the same buffers safely.  The buffer only grows.
struct Workspace {
  void *ptr = nullptr;
  size_t bytes = 0;
};

struct DeviceInfo {
  int device = -1;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
};

int device_info(DeviceInfo *out);  // for the current device

// Allows `func` up to `bytes` of dynamic shared memory on the current device.
// The attribute belongs to one device, so it is set once per (device, kernel)
// and again only for a larger size.
int smem_optin_raw(const void *func, int bytes);
template <typename F> int smem_optin(F *func, int bytes) {
  return smem_optin_raw(reinterpret_cast<const void *>(func), bytes);
}

// Workspace slots: every user owns its slot, so a nested routine never
// reallocates a buffer its caller still holds.
enum Slot : int {
  kSlotA = 0, kSlotAT = 1,    // C ABI: staged / transposed first matrix
  kSlotB = 2, kSlotBT = 3,    // C ABI: second matrix (B)
  kSlotPiv = 4,               // C ABI: pivots
  kSlotC = 5,                 // C ABI: third matrix (gemm/syrk C)
  kSlotX = 6, kSlotXT = 7,    // C ABI: solution X
  kSlotPanel = 8,             // LU panel candidate exchange; one-launch trsv publication
  kSlotIRVec = 9,             // refinement vectors
  kSlotLowLU = 10,            // low-precision factor copy, pivots, permutation
  kSlotL16 = 11, kSlotU16 = 12,  // 16-bit L21 / U12 operands of the tensor-core update
  kSlotBatch = 13,            // batched solver descriptors
  kSlotSwap = 14,             // composed row-interchange pairs
  kSlotQR = 15,               // QR: V, T, W, split-K partials, panel exchange
  kSlotSym = 16,              // full symmetric FP64 copy for the mixed Cholesky solve
  kSlotSel = 17,              // selector feature statistics
  kSlotSelNet = 18,           // selector network parameters, input, logits, work
  kSlotF64LU = 19,            // FP64 LU copy and pivots of the selector's last resort
  kSlotInvL = 20,             // mixed LU: inverse of the unit-lower diagonal block, block row
  kSlotZExp = 21,             // complex GEMM: the expanded real 2m x 2k operand
  kSlotZOpB = 22,             // complex GEMM: op(B) materialized
  kSlotZTmp = 23,             // complex herk / syrk: the full product
  kSlotZTr = 24,              // complex trsm: the transposed right-hand side (right side)
  kSlotSytrf = 25,            // Bunch-Kaufman: the step's block size read back by the host
  kSlotOzA = 26, kSlotOzB = 27,  // FP64-by-slices GEMM: the BF16 slices of A and B, exponents
  kSlotOzC = 28,              // FP64-by-slices GEMM: the FP32 accumulators
  kSlotChunk = 29,            // mixed LU of a host A: the replayed blocks' 16-bit operands
  kSlotOzT = 30,              // FP64 slice Cholesky: the next block's L21 rows, transposed
  kNumSlots = 31
};

// Returns a device buffer of at least `bytes` bound to `stream` in `slot`.
int workspace(cudaStream_t stream, int slot, size_t bytes, void **out);

// Streams and events of a blocked factorization's lookahead, one set per
// (device, caller stream), created on first use and kept: a high-priority
// panel stream for the critical chain of panels and next-block updates, a
// low-priority bulk stream for the rest of each trailing update, and the
// events that order them (kRing in flight).  The LU and Cholesky drivers that
// use it never run inside one another on the same caller stream.
struct Lookahead {
  static constexpr int kRing = 4;
  cudaStream_t panel = nullptr, bulk = nullptr;
  cudaEvent_t first = nullptr, upd[kRing] = {}, bulk_done[kRing] = {}, end_panel = nullptr,
              end_bulk = nullptr;
};
int lookahead(cudaStream_t s, Lookahead **out);

// Small per-stream control block: grid-barrier counters and a status word.
struct Control {
  unsigned int barrier[2];   // arrive counter, generation
  unsigned int status;       // kStatus* bits
  int info;                  // LAPACK info produced on the device
  unsigned int queue;        // work-queue head for persistent kernels
  unsigned int pad[3];
};
int control(cudaStream_t stream, Control **out);  // zeroed on the stream before return

// Copies the device status word back and converts timeouts to kErrTimeout.
int check_status(cudaStream_t stream, Control *ctl, int *info_out);

// Bounded spin limit for device-side waits (~1 s at GB300 clocks).
constexpr long long kSpinLimit = 1ll << 22;
// The limit the waits use, per device: kSpinLimit unless
// zml_gpu_set_spin_limit changed it.  Without relocatable device code every
// translation unit holds its own copy, so each registers a setter and one
// host call updates them all.
static __device__ long long g_spin_limit = kSpinLimit;
__device__ __forceinline__ long long spin_limit() { return g_spin_limit; }
int register_spin_setter(int (*set)(long long));
int set_spin_limit(long long tries);  // every translation unit, current device
namespace {
inline int set_spin_limit_here(long long tries) {
  return cudaMemcpyToSymbol(g_spin_limit, &tries, sizeof tries) == cudaSuccess ? 0 : -1001;
}
const int g_spin_setter_registered = register_spin_setter(&set_spin_limit_here);
}  // namespace

// ---------------------------------------------------------------------------
// Device helpers
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a cooperative launch.  ctl->barrier[0] counts
// arrivals monotonically over the launch (zeroed before it): phase g is
// complete once it reaches (g + 1) * nblocks, so a waiter sees the last
// arrival directly.  The wait is bounded; on timeout the status bit is set
// and the CTA carries on (the host then reports kErrTimeout).
// Arrival is a release reduction and the wait an acquire load: with the CTA
// barriers around them, every write of the CTA before the barrier is visible
// to every CTA after it.
__device__ __forceinline__ void grid_barrier(Control *ctl, unsigned nblocks, unsigned &gen) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = (gen + 1) * nblocks;
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&ctl->barrier[0]), "r"(1u)
                 : "memory");
    long long spins = 0;
    const long long lim = spin_limit();
    while (ld_acquire(&ctl->barrier[0]) < target) {
      if (++spins > lim) {
        atomicOr(&ctl->status, kStatusBarrierTimeout);
        break;
      }
    }
  }
  ++gen;
  __syncthreads();
}

template <typename T> struct Real;
template <> struct Real<double> {
  static __device__ __forceinline__ double sfmin() { return 2.2250738585072014e-308; }
};
template <> struct Real<float> {
  static __device__ __forceinline__ float sfmin() { return 1.17549435e-38f; }
};

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// Launch accounting.  Every kernel launch goes through ZG_LAUNCH, which counts
// it and, while profiling is enabled (zml_gpu_profile), brackets it with CUDA
// events on its stream and files it under a kernel class with the launch's
// algorithmic flops and bytes.
enum ProfTag : int {
  kTagGemmTC = 0, kTagGemmSimt, kTagPanel, kTagTrsmDiag, kTagLaswp, kTagTrsv, kTagGemv,
  kTagConvert, kTagPotf2, kTagVector, kTagBatched, kTagQR, kTagMLP, kTagOther, kNumTags
};
extern std::atomic<unsigned long long> g_launches;  // calls from several threads / streams
extern bool g_profiling;
void prof_record(cudaStream_t s, int tag, double flops, double bytes, cudaEvent_t *begin);
void prof_end(cudaStream_t s, cudaEvent_t begin, int tag, double flops, double bytes);

#define ZG_LAUNCH(tag, flops, bytes, stream, ...)                                     \
  do {                                                                                \
    cudaEvent_t zg_ev0_ = nullptr;                                                    \
    if (::zg::g_profiling) ::zg::prof_record((stream), (tag), 0, 0, &zg_ev0_);        \
    __VA_ARGS__;                                                                      \
    ++::zg::g_launches;                                                               \
    if (::zg::g_profiling) ::zg::prof_end((stream), zg_ev0_, (tag), (flops), (bytes)); \
    ZG_CUDA(cudaGetLastError());                                                      \
  } while (0)

}  // namespace zg
