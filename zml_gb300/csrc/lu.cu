// lu.cu -- LU with partial pivoting: getrf / getrs / laswp on the GPU.
//
// Replaces zml's lapack/getrf.zig:14-152 (blocked right-looking loop),
// getrf2.zig:14-210 (panel), laswp.zig:12-96 and getrs.zig:13-142.
//
// The panel (m x nb, nb <= 64 for FP64, <= 128 for FP32) is factored by ONE
// cooperative launch: every CTA keeps a contiguous slab of the panel's rows
// in shared memory for the whole panel; per column it finds its local
// pivot candidate, publishes (|value|, row, row contents) to a global
// exchange slot, meets the other CTAs at one bounded grid barrier, and then
// every CTA reduces the candidates identically, swaps, scales and applies
// the rank-1 update to its own rows.  The pivot rule is zml's iamax
// (blas/iamax.zig:29-38): the first maximum of |a(i,k)| over i >= k wins,
// NaN never displaces the running maximum, so ties resolve to the lowest row.
// The column is scaled by the reciprocal of the pivot when |pivot| >= sfmin,
// else divided (getrf2.zig:65-87).
#include <algorithm>
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace zg {

// Comparison key of candidate row i for pivot column k (see header comment).
template <typename T> __device__ __forceinline__ T pivot_key(T v, bool first) {
  if (v != v) return first ? T(INFINITY) : T(-INFINITY);
  return fabs(v);
}

template <typename T>
__device__ __forceinline__ void better(T &bk, int &bi, T k2, int i2) {
  if (k2 > bk || (k2 == bk && i2 < bi)) { bk = k2; bi = i2; }
}

template <typename T>
__device__ void block_argmax(T &key, int &idx, T *sk, int *si) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T k2 = __shfl_xor_sync(0xffffffffu, key, off);
    int i2 = __shfl_xor_sync(0xffffffffu, idx, off);
    better(key, idx, k2, i2);
  }
  if (lane == 0) { sk[warp] = key; si[warp] = idx; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    key = lane < nw ? sk[lane] : T(-INFINITY);
    idx = lane < nw ? si[lane] : 0x7fffffff;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      T k2 = __shfl_xor_sync(0xffffffffu, key, off);
      int i2 = __shfl_xor_sync(0xffffffffu, idx, off);
      better(key, idx, k2, i2);
    }
    if (lane == 0) { sk[0] = key; si[0] = idx; }
  }
  __syncthreads();
  key = sk[0];
  idx = si[0];
  __syncthreads();
}

// Exchange layout (T words): for parity p in {0,1}:
//   cand[p][b] : [key, row, v_0 .. v_{nb-1}]  (stride nb + 2), b < gridDim.x
//   rowk[p]    : [v_0 .. v_{nb-1}]
// FP32 keys: the candidate (|v| or -inf for a NaN off the diagonal, row) is
// one 64-bit word -- the key's order-preserving bits + 1 (0 for -inf) above
// 0xffffffff - row -- whose maximum is the pivot (largest key, then lowest
// row).  Every CTA folds its word into winners[k] with atomicMax before the
// barrier and reads the single word after it.
__device__ __forceinline__ unsigned long long pack_candidate(float key, int idx) {
  const unsigned ord = key == -INFINITY ? 0u : __float_as_uint(key) + 1u;
  return ((unsigned long long)ord << 32) | (unsigned)(0xffffffffu - (unsigned)idx);
}

template <typename T>
__global__ void __launch_bounds__(256) panel_lu_kernel(int m, int nb, T *__restrict__ A, long lda,
                                                       int *__restrict__ ipiv, int ipiv_base,
                                                       Control *ctl, int info_base, int R,
                                                       T *__restrict__ xchg,
                                                       unsigned long long *__restrict__ winners) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *S = reinterpret_cast<T *>(smem_raw);  // S[c * R + r], column-major slab
  __shared__ T sk[32];
  __shared__ int si[32];
  __shared__ T urow[128];                  // pivot row of the current column
  const int b = blockIdx.x, nblk = gridDim.x, tid = threadIdx.x;
  const int r0 = b * R, rows = max(0, min(R, m - r0));
  const int stride = nb + 2;
  T *cand[2] = {xchg, xchg + (long)nblk * stride};
  T *rowk[2] = {xchg + 2L * nblk * stride, xchg + 2L * nblk * stride + nb};
  unsigned gen = 0;

  for (int e = tid; e < rows * nb; e += blockDim.x) {
    int r = e % rows, c = e / rows;
    S[c * R + r] = A[(r0 + r) + (long)c * lda];
  }
  __syncthreads();

  const int kmax = min(m, nb);
  for (int k = 0; k < kmax; ++k) {
    const int p = k & 1;
    // 1. local candidate among rows i >= k
    T key = T(-INFINITY);
    int idx = 0x7fffffff;
    for (int r = tid; r < rows; r += blockDim.x) {
      const int gi = r0 + r;
      if (gi < k) continue;
      better(key, idx, pivot_key(S[k * R + r], gi == k), gi);
    }
    block_argmax(key, idx, sk, si);
    T *my = cand[p] + (long)b * stride;
    if (sizeof(T) == sizeof(float)) {
      if (tid == 0) atomicMax(winners + k, pack_candidate((float)key, idx));
    } else if (tid == 0) {
      my[0] = key;
      my[1] = idx == 0x7fffffff ? T(-1) : T(idx);
    }
    if (idx != 0x7fffffff)
      for (int c = tid; c < nb; c += blockDim.x) my[2 + c] = S[c * R + (idx - r0)];
    if (k >= r0 && k < r0 + rows)
      for (int c = tid; c < nb; c += blockDim.x) rowk[p][c] = S[c * R + (k - r0)];
    // 2. meet every CTA
    grid_barrier(ctl, nblk, gen);
    // 3. global pivot: identical in every CTA
    int win = 0;
    if (sizeof(T) == sizeof(float)) {
      const unsigned long long w = __ldcg(winners + k);
      idx = (int)(0xffffffffu - (unsigned)(w & 0xffffffffu));
    } else {
      key = T(-INFINITY);
      idx = 0x7fffffff;
      for (int q = tid; q < nblk; q += blockDim.x) {
        const T *cq = cand[p] + (long)q * stride;
        const T kq = __ldcg(cq), rq = __ldcg(cq + 1);
        better(key, idx, kq, rq < T(0) ? 0x7fffffff : (int)rq);
      }
      block_argmax(key, idx, sk, si);
    }
    // A pivot row outside [k, m) only arises after a barrier timeout (stale
    // exchange words): row k stands in, so that every index below -- the
    // candidate slot, the swap, ipiv and the interchanges run on it later --
    // stays inside the matrix.  The host then reports the timeout.
    if (idx < k || idx >= m) idx = k;
    // locate the slot that holds row idx
    win = idx / R;
    const T *prow = cand[p] + (long)win * stride + 2;
    for (int c = tid; c < nb; c += blockDim.x) urow[c] = __ldcg(prow + c);
    __syncthreads();
    const T piv = urow[k];
    if (b == 0 && tid == 0) {
      ipiv[k] = idx + 1 + ipiv_base;
      if (piv == T(0)) atomicCAS(&ctl->info, 0, k + 1 + info_base);
    }
    if (piv != T(0) && idx != k) {  // 4. swap rows k and idx
      if (k >= r0 && k < r0 + rows)
        for (int c = tid; c < nb; c += blockDim.x) S[c * R + (k - r0)] = urow[c];
      if (idx >= r0 && idx < r0 + rows)
        for (int c = tid; c < nb; c += blockDim.x) S[c * R + (idx - r0)] = __ldcg(rowk[p] + c);
      __syncthreads();
    }
    // 5. scale the column below the pivot, 6. rank-1 update of the slab:
    // thread = (row lane, column phase); no index division in the loops.
    const int rb = max(0, k + 1 - r0);  // first local row strictly below k
    const int lr = tid & 127, cph = tid >> 7;  // 128 row lanes x 2 column phases
    if (piv != T(0)) {
      const bool recip = fabs(piv) >= Real<T>::sfmin();
      const T rp = T(1) / piv;
      for (int r = rb + tid; r < rows; r += blockDim.x)
        S[k * R + r] = recip ? S[k * R + r] * rp : S[k * R + r] / piv;
      __syncthreads();
    }
    for (int r = rb + lr; r < rows; r += 128) {
      const T l = S[k * R + r];
      T *row = S + r;
      for (int c = k + 1 + cph; c < nb; c += 2) row[c * R] -= l * urow[c];
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * nb; e += blockDim.x) {
    int r = e % rows, c = e / rows;
    A[(r0 + r) + (long)c * lda] = S[c * R + r];
  }
}

// Rows per CTA of the cooperative panel (0: spread over every SM, at least
// 8 rows each).
static std::atomic<int> g_panel_rows{kPanelRowsDefault};
int set_panel_rows(int rows) { return g_panel_rows.exchange(rows < 0 ? kPanelRowsDefault : rows); }

template <typename T>
int panel_lu(int m, int nb, T *A, long lda, int *ipiv, int ipiv_base, Control *ctl, int info_base,
             cudaStream_t s) {
  if (m <= 0 || nb <= 0) return 0;
  if (nb > 128) {
    set_last_error("panel_lu: nb %d > 128", nb);
    return kErrInvalid;
  }
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  // rows per CTA: the tuning target (fewer CTAs make the per-column grid
  // barrier cheaper, taller slabs the per-column update longer), at least
  // m / SMs (one CTA per SM), at most what fits in shared memory
  const size_t limit = di.smem_optin - 4096;
  const int rmax = (int)(limit / ((size_t)nb * sizeof(T)));
  const int target = g_panel_rows.load();
  int R = target > 0 ? std::min(rmax, target) : 8;
  R = std::max(R, ceil_div(m, di.num_sms));
  if (R > rmax) {
    set_last_error("panel_lu: panel %d x %d too tall for %d SMs", m, nb, di.num_sms);
    return kErrInvalid;
  }
  int nblk = ceil_div(m, R);
  R = ceil_div(m, nblk);
  nblk = ceil_div(m, R);
  const size_t smem = (size_t)R * nb * sizeof(T);
  void *xchg;
  const size_t nx = sizeof(T) * (2L * nblk * (nb + 2) + 2L * nb);
  ZG_TRY(workspace(s, kSlotPanel, nx + 8 * (size_t)nb + 256, &xchg));
  // per-column winner words (FP32 panels), zeroed per launch
  unsigned long long *winners =
      (unsigned long long *)(((uintptr_t)xchg + nx + 255) & ~(uintptr_t)255);
  if (sizeof(T) == sizeof(float)) ZG_CUDA(cudaMemsetAsync(winners, 0, 8 * (size_t)nb, s));
  ZG_TRY(smem_optin(panel_lu_kernel<T>, (int)limit));
  // barrier counters are per launch
  ZG_CUDA(cudaMemsetAsync(&ctl->barrier[0], 0, 2 * sizeof(unsigned), s));
  T *xp = (T *)xchg;
  void *args[] = {&m, &nb, &A, &lda, &ipiv, &ipiv_base, &ctl, &info_base, &R, &xp, &winners};
  ZG_LAUNCH(kTagPanel, 1.0 * m * nb * nb, 2.0 * sizeof(T) * m * nb, s,
            ZG_CUDA(cudaLaunchCooperativeKernel((void *)panel_lu_kernel<T>, dim3(nblk), dim3(256),
                                                args, smem, s)));
  return 0;
}

// Row interchanges (laswp.zig:12-96).  The sequence of swaps k1..k2 (1-based,
// forward for incx > 0, backward otherwise) is first composed into a list of
// (destination row, source row) pairs -- at most 2 (k2-k1+1) rows move -- and
// then every column gathers its moved rows and scatters them in parallel, so
// no column walks a chain of dependent swaps.
constexpr int kSwapMax = 256;  // pivots per composed chunk

// The composition, one thread per row that can move: the rows k1-1 .. k2-1
// and every row outside them that a pivot names (at its first occurrence).
// Each traces back through the swaps to the row whose content it ends with;
// the traces are independent, so the block's cost is one pass over the
// pivots instead of a chain of dependent swaps in shared memory.  A row that
// keeps its content emits no pair; the pairs' order does not matter (the
// apply kernel loads every source before it stores).
__global__ void __launch_bounds__(256) laswp_prep_kernel(int k1, int k2,
                                                         const int *__restrict__ ipiv, int incx,
                                                         int *pairs, int *npairs) {
  __shared__ int piv[kSwapMax];  // the chunk's pivots (0-based target rows)
  __shared__ int np;
  const int t = threadIdx.x;
  const int base = k1 - 1, len = k2 - k1 + 1;
  if (t == 0) np = 0;
  for (int i = t; i < len; i += blockDim.x) piv[i] = ipiv[base + i] - 1;
  __syncthreads();
  for (int e = t; e < 2 * len; e += blockDim.x) {
    int x;  // a destination row
    if (e < len) {
      x = base + e;
    } else {
      const int i = e - len, p = piv[i];
      if (p >= base && p < base + len) continue;
      bool first = true;
      for (int j = 0; j < i && first; ++j) first = piv[j] != p;
      if (!first) continue;
      x = p;
    }
    // content of x after the swaps = content of y before them: x taken back
    // through the swaps in reverse order of application
    int y = x;
    if (incx > 0) {
      for (int q = len - 1; q >= 0; --q) {
        const int k = base + q, p = piv[q];
        y = y == k ? p : (y == p ? k : y);
      }
    } else {
      for (int q = 0; q < len; ++q) {
        const int k = base + q, p = piv[q];
        y = y == k ? p : (y == p ? k : y);
      }
    }
    if (y != x) {
      const int c = atomicAdd(&np, 1);
      pairs[2 * c] = x;
      pairs[2 * c + 1] = y;
    }
  }
  __syncthreads();
  if (t == 0) *npairs = np;
}

// One warp per column, lanes over the pairs: every moved value of the column
// is loaded into registers (all loads of the column in flight at once, and
// all inside one column's span of memory), then the warp stores them.  Loads
// and stores go through L2 only: the mixed LU runs this kernel beside kernels
// of another stream that rewrite the same columns, and a line this SM cached
// earlier would be stale.
template <typename T>
__global__ void __launch_bounds__(256) laswp_apply_kernel(int n, T *A, long lda,
                                                               const int *__restrict__ pairs,
                                                               const int *__restrict__ npairs) {
  __shared__ int pr[4 * kSwapMax];
  const int np = *npairs;
  for (int e = threadIdx.x; e < 2 * np; e += blockDim.x) pr[e] = pairs[e];
  __syncthreads();
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  constexpr int kPer = 2 * kSwapMax / 32;  // pairs a lane holds at most
  for (int c = blockIdx.x * wpb + (threadIdx.x >> 5); c < n; c += gridDim.x * wpb) {
    T *col = A + (long)c * lda;
    T v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int t = lane + 32 * u;
      if (t < np) v[u] = __ldcg(col + pr[2 * t + 1]);
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int t = lane + 32 * u;
      if (t < np) __stcg(col + pr[2 * t], v[u]);
    }
    __syncwarp();
  }
}

// A composed row interchange: device pairs (dst, src) and their count.
struct SwapPlan {
  int *pairs = nullptr, *np = nullptr;
  int rows = 0;  // pivots composed (bounds the pair count by 2 rows)
};

static int laswp_compose(int k1, int k2, const int *ipiv, int incx, SwapPlan *plan, int slot,
                         cudaStream_t s) {
  void *w;
  ZG_TRY(workspace(s, slot, sizeof(int) * (4 * kSwapMax + 8), &w));
  plan->pairs = (int *)w;
  plan->np = plan->pairs + 4 * kSwapMax;
  plan->rows = k2 - k1 + 1;
  ZG_LAUNCH(kTagLaswp, 0, 0, s,
            laswp_prep_kernel<<<1, 256, 0, s>>>(k1, k2, ipiv, incx, plan->pairs, plan->np));
  return 0;
}

template <typename T>
static int laswp_apply(int n, T *A, long lda, const SwapPlan &plan, cudaStream_t s) {
  if (n <= 0 || plan.rows <= 0) return 0;
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const int grid = std::min(ceil_div(n, 8), di.num_sms * 8);
  ZG_LAUNCH(kTagLaswp, 0, 4.0 * sizeof(T) * n * plan.rows, s,
            laswp_apply_kernel<T><<<grid, 256, 0, s>>>(n, A, lda, plan.pairs, plan.np));
  return 0;
}

int laswp_reserve(cudaStream_t s) {
  void *w;
  return workspace(s, kSlotSwap, sizeof(int) * (4 * kSwapMax + 8), &w);
}

template <typename T>
int laswp_dev(int n, T *A, long lda, int k1, int k2, const int *ipiv, int incx, cudaStream_t s) {
  if (n <= 0 || k2 < k1) return 0;
  for (int q = 0;; ++q) {  // long pivot ranges in chunks, in application order
    int lo, hi;
    if (incx > 0) {
      lo = k1 + q * kSwapMax;
      if (lo > k2) break;
      hi = std::min(k2, lo + kSwapMax - 1);
    } else {
      hi = k2 - q * kSwapMax;
      if (hi < k1) break;
      lo = std::max(k1, hi - kSwapMax + 1);
    }
    SwapPlan plan;
    ZG_TRY(laswp_compose(lo, hi, ipiv, incx, &plan, kSlotSwap, s));
    ZG_TRY(laswp_apply<T>(n, A, lda, plan, s));
  }
  return 0;
}

// The interchanges of one panel (rows k1..k2, forward) applied to the column
// ranges [0, c_left) and [c_right, n) with one composition.
template <typename T>
int laswp_panel(int c_left, int c_right, int n, T *A, long lda, int k1, int k2, const int *ipiv,
                cudaStream_t s) {
  if (k2 < k1) return 0;
  if (k2 - k1 + 1 > kSwapMax) {
    ZG_TRY(laswp_dev<T>(c_left, A, lda, k1, k2, ipiv, 1, s));
    return laswp_dev<T>(n - c_right, A + (long)c_right * lda, lda, k1, k2, ipiv, 1, s);
  }
  SwapPlan plan;
  ZG_TRY(laswp_compose(k1, k2, ipiv, 1, &plan, kSlotSwap, s));
  ZG_TRY(laswp_apply<T>(c_left, A, lda, plan, s));
  return laswp_apply<T>(n - c_right, A + (long)c_right * lda, lda, plan, s);
}

template <typename T> static int lu_block() { return sizeof(T) == 8 ? 64 : 128; }

// FP32 panels go to the cluster-resident panel where it applies.
template <typename T>
static int panel_any(int m, int nb, T *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool tournament) {
  bool done = false;
  if constexpr (sizeof(T) == sizeof(float))
    ZG_TRY(panel_lu_cluster(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s, &done, nullptr, 0,
                            nullptr, 0, tournament));
  else
    ZG_TRY(panel_lu_cluster(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s, &done));
  if (done) return 0;
  return panel_lu<T>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s);
}

// The blocks of getrf_simt.  Lookahead: a block's trailing update is split
// into the next block's columns (triangular solve and GEMM on the panel
// stream) and the rest (on the bulk stream), so the bulk of the update runs
// beside the next block's panel.  Block b's panel waits for block b-2's bulk
// update, the last to touch its columns; block b's full-width interchanges
// for block b-1's, which still reads block b-1's L21.  Each element's
// arithmetic is that of one update over all the columns (the GEMM's tiles and
// K order do not depend on N; every column of the triangular solve is
// independent).
template <typename T>
static int getrf_simt_blocks(int m, int n, T *A, long lda, int *ipiv, Control *ctl,
                             Lookahead &la, bool tournament) {
  constexpr int R = Lookahead::kRing;
  const cudaStream_t s = la.panel, sb = la.bulk;
  const int nb = lu_block<T>();
  const int mn = min(m, n);
  for (int j = 0, b = 0; j < mn; j += nb, ++b) {
    const int jb = min(nb, mn - j);
    T *Ajj = A + j + (long)j * lda;
    if (b >= 2) ZG_CUDA(cudaStreamWaitEvent(s, la.bulk_done[(b - 2) % R], 0));
    ZG_TRY(panel_any<T>(m - j, jb, Ajj, lda, ipiv + j, j, ctl, j, s, tournament));
    if (b >= 1) ZG_CUDA(cudaStreamWaitEvent(s, la.bulk_done[(b - 1) % R], 0));
    ZG_TRY(laswp_panel<T>(j, std::min(n, j + jb), n, A, lda, j + 1, j + jb, ipiv, s));
    const int rest = n - j - jb;
    if (rest > 0) {
      T *Aright = A + (long)(j + jb) * lda;
      // the next block's columns now, on the panel stream ...
      const int near = min(nb, rest);
      ZG_TRY(trsm_dev<T>(kLeft, kLower, kNoTrans, kUnit, jb, near, T(1), Ajj, lda, Aright + j,
                         lda, s));
      if (j + jb < m)
        ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, m - j - jb, near, jb, T(-1), Ajj + jb, lda,
                            Aright + j, lda, T(1), Aright + j + jb, lda, 0, s));
      // ... the rest on the bulk stream, beside the next block's panel
      if (rest > near) {
        ZG_CUDA(cudaEventRecord(la.upd[b % R], s));
        ZG_CUDA(cudaStreamWaitEvent(sb, la.upd[b % R], 0));
        T *Af = Aright + (long)near * lda;
        ZG_TRY(trsm_dev<T>(kLeft, kLower, kNoTrans, kUnit, jb, rest - near, T(1), Ajj, lda,
                           Af + j, lda, sb));
        if (j + jb < m)
          ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, m - j - jb, rest - near, jb, T(-1), Ajj + jb,
                              lda, Af + j, lda, T(1), Af + j + jb, lda, 0, sb));
      }
    }
    ZG_CUDA(cudaEventRecord(la.bulk_done[b % R], sb));
  }
  return 0;
}

template <typename T>
int getrf_simt(int m, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s,
               bool tournament) {
  *info = 0;
  if (m <= 0 || n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  // both internal streams start after the caller's earlier work, and the
  // caller's stream resumes after both (also after a failure part way)
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = getrf_simt_blocks<T>(m, n, A, lda, ipiv, ctl, *la, tournament);
  ZG_CUDA(cudaEventRecord(la->end_panel, la->panel));
  ZG_CUDA(cudaEventRecord(la->end_bulk, la->bulk));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_panel, 0));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_bulk, 0));
  if (rc != 0) return rc;
  return check_status(s, ctl, info);
}

// FP64 LUs from n = 2048 up take their trailing updates on the tensor cores
// (getrf_oz, exact slices of the FP64 operands); smaller ones, FP32 and a
// caller that chose zml_gpu_fp64_updates(0) stay on getrf_simt.
template <typename T>
int getrf_dev(int m, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s,
              bool tournament) {
  if constexpr (sizeof(T) == sizeof(double)) {
    if (fp64_updates_on_tensor_cores(m, n)) {
      if (m <= 0 || n <= 0) {
        *info = 0;
        return 0;
      }
      return getrf_oz(m, n, reinterpret_cast<double *>(A), lda, ipiv, info, s);
    }
  }
  return getrf_simt<T>(m, n, A, lda, ipiv, info, s, tournament);
}

// ---------------------------------------------------------------------------
// One right-hand side against a triangle of an FP64 factor in one launch
// (getrs, potrs): T x = rhs with T = op(A) lower (a forward solve) or upper (a
// backward solve), op(A) = A or A^T, unit or non-unit diagonal.  128-row
// blocks, one CTA each, claimed in dependency order by ticket: a CTA streams
// its block row's off-diagonal tiles (128 x 64 halves, the next half
// prefetched; for A^T the lanes run along A's columns so that the loads stay
// coalesced), each multiplied by the x an earlier block published, then solves
// its diagonal block by substitution (the backward-stable arithmetic of trsm,
// not an inverse) and publishes its x.  GB300 runs about two FP64 FMAs per
// clock per SM, so the substitution keeps only each 32-row sub-triangle on its
// serial chain (one warp, a row a lane, x_k by shuffle, multiplies by
// reciprocals of the diagonal formed up front) and all 16 warps subtract the
// solved sub-block from the rows still to solve.  Publication: a buffer
// pre-filled with an all-ones word, polled word by word (bounded; a timeout
// sets the stream's status bit).
constexpr int kFB = 128, kFT = 512, kFH = 16;  // block rows, threads, values a thread per half tile
constexpr int kFLD = kFB + 1;                  // the diagonal block's leading dimension in SMEM
constexpr unsigned long long kFEmpty = ~0ull;

__device__ __forceinline__ unsigned long long ld_relaxed_b64(const double *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// One 32-row sub-triangle by substitution, a row a lane: x_k broadcast by
// shuffle, then subtracted from the rows still to solve; a unit diagonal
// keeps the multiply off the chain.
template <bool UPPER, bool UNIT>
__device__ __forceinline__ double chain32(double y, const double *dcol, const double *rd,
                                          int lane) {
#pragma unroll
  for (int s = 0; s < 32; ++s) {
    const int k = UPPER ? 31 - s : s;
    if (!UNIT && lane == k) y *= rd[k];
    const double xk = __shfl_sync(0xffffffffu, y, k);
    if (UPPER ? lane < k : lane > k) y = fma(-dcol[k * kFLD], xk, y);
  }
  return y;
}

template <bool TRANS>
__global__ void __launch_bounds__(kFT) trsv_f64_kernel(int n, const double *__restrict__ A,
                                                       long lda, const double *rhs_in, double *x,
                                                       double *xpub, unsigned *ticket,
                                                       bool upper, bool unit, unsigned *status) {
  extern __shared__ double sD[];  // the diagonal block of op(A), sD[i + j kFLD]
  __shared__ unsigned sb;
  __shared__ double part[4][kFB];
  __shared__ double xs[kFB];
  __shared__ double rd[kFB];  // reciprocals of the diagonal
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sb = atomicAdd(ticket, 1u);
  __syncthreads();
  const int nblk = (n + kFB - 1) / kFB, t = sb;
  const int blk = upper ? nblk - 1 - t : t;
  const int r0 = blk * kFB, rows = min(kFB, n - r0);
  const int lr = tid % kFB, ph = tid / kFB;
  for (int e = tid; e < kFB * kFB; e += kFT) {
    // A's contiguous index runs over the threads: op(A) row i for A, column for A^T
    const int a = e % kFB, b = e / kFB;
    const int i = TRANS ? b : a, j = TRANS ? a : b;
    sD[i + j * kFLD] = (a < rows && b < rows) ? __ldcg(A + (r0 + a) + (long)(r0 + b) * lda)
                                              : (i == j ? 1.0 : 0.0);
  }
  if (tid < kFB)
    rd[tid] = (!unit && tid < rows) ? 1.0 / __ldcg(A + (r0 + tid) + (long)(r0 + tid) * lda) : 1.0;
  const double rhs = tid < rows ? rhs_in[r0 + tid] : 0.0;
  auto col0 = [&](int q) { return (upper ? nblk - 1 - q : q) * kFB; };
  // A: thread (lr, ph) holds row lr, columns ph + 4 j of the half tile.
  // A^T: warp w holds rows 8 w .. 8 w + 7, lane columns lane and lane + 32.
  auto load_half = [&](int hq, double (&v)[kFH]) {
    const int c0 = col0(hq >> 1) + 64 * (hq & 1);
    if constexpr (!TRANS) {
      const bool ok = lr < rows;
#pragma unroll
      for (int j = 0; j < kFH; ++j) {
        const int c = c0 + ph + 4 * j;
        v[j] = (ok && c < n) ? __ldcs(A + r0 + lr + (long)c * lda) : 0.0;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int rr = 8 * warp + k;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          const int c = c0 + lane + 32 * m;
          v[2 * k + m] = (rr < rows && c < n) ? __ldcs(A + c + (long)(r0 + rr) * lda) : 0.0;
        }
      }
    }
  };
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = 0.0;
  double cur[kFH], nxt[kFH];
  const int nh = 2 * t;
  if (nh > 0) load_half(0, cur);
  for (int hq = 0; hq < nh; ++hq) {
    if (hq + 1 < nh) load_half(hq + 1, nxt);
    if ((hq & 1) == 0) {
      if (tid < kFB) {
        const int c = col0(hq >> 1) + tid;
        double xv = 0.0;
        if (c < n) {
          unsigned long long w = ld_relaxed_b64(xpub + c);
          long long spins = 0;
          const long long lim = spin_limit();
          while (w == kFEmpty) {
            if (++spins > lim) {
              atomicOr(status, kStatusQueueTimeout);
              break;
            }
            if (spins > 64) __nanosleep(32);
            w = ld_relaxed_b64(xpub + c);
          }
          xv = __longlong_as_double((long long)w);
        }
        xs[tid] = xv;
      }
      __syncthreads();
    }
    if constexpr (!TRANS) {
      // each half tile summed on its own, then added to the running sums: the
      // depth of a sum grows with the tiles, not with the columns
      const int xo = 64 * (hq & 1) + ph;
      double p0 = cur[0] * xs[xo], p1 = cur[1] * xs[xo + 4];
#pragma unroll
      for (int j = 2; j < kFH; j += 2) {
        p0 = fma(cur[j], xs[xo + 4 * j], p0);
        p1 = fma(cur[j + 1], xs[xo + 4 * (j + 1)], p1);
      }
      acc[0] += p0;
      acc[1] += p1;
    } else {
      const double x0 = xs[64 * (hq & 1) + lane], x1 = xs[64 * (hq & 1) + lane + 32];
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] += fma(cur[2 * k + 1], x1, cur[2 * k] * x0);
    }
    if (hq & 1) __syncthreads();  // xs free for the next tile
#pragma unroll
    for (int j = 0; j < kFH; ++j) cur[j] = nxt[j];
  }
  if constexpr (!TRANS) {
    part[ph][lr] = acc[0] + acc[1];
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      double v = acc[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) {
        part[0][8 * warp + k] = v;
        part[1][8 * warp + k] = 0.0;
        part[2][8 * warp + k] = 0.0;
        part[3][8 * warp + k] = 0.0;
      }
    }
  }
  __syncthreads();
  if (tid < kFB)
    xs[tid] = tid < rows ? rhs - ((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]))
                         : 0.0;
  __syncthreads();
  // the diagonal block (padded with the identity past `rows`)
  for (int s4 = 0; s4 < 4; ++s4) {
    const int o = 32 * (upper ? 3 - s4 : s4);
    if (warp == 0) {
      const double *dcol = sD + o + lane + o * kFLD;
      double y = xs[o + lane];
      if (!upper)
        y = unit ? chain32<false, true>(y, dcol, rd + o, lane)
                 : chain32<false, false>(y, dcol, rd + o, lane);
      else
        y = unit ? chain32<true, true>(y, dcol, rd + o, lane)
                 : chain32<true, false>(y, dcol, rd + o, lane);
      xs[o + lane] = y;
    }
    __syncthreads();
    const int lo = upper ? 0 : o + 32, hi = upper ? o : kFB;  // rows still to solve
    if (lo < hi) {
      if (lr >= lo && lr < hi) {
        double a = 0.0;
#pragma unroll
        for (int c = 0; c < 8; ++c)
          a = fma(sD[lr + (o + 8 * ph + c) * kFLD], xs[o + 8 * ph + c], a);
        part[ph][lr] = a;
      }
      __syncthreads();
      if (tid >= lo && tid < hi)
        xs[tid] -= (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
      __syncthreads();
    }
  }
  if (tid < rows) {
    const double v = xs[tid];
    x[r0 + tid] = v;
    xpub[r0 + tid] = v != v ? __longlong_as_double(0x7ff8000000000000ll) : v;
  }
}

// Y = P B for nrhs columns, P the interchanges ipiv[0..n) applied in
// increasing order (dlaswp incx = 1, forward) or decreasing order (incx = -1):
// row i of Y is row sigma(i) of B, found by undoing the interchanges from the
// last applied to the first (an interchange of rows j and p moves whatever sits
// at j to p and back), one thread a row.  An index outside [1, n] yields NaN
// rows instead of an out-of-bounds read.
__global__ void __launch_bounds__(128) perm_gather_kernel(int n, int nrhs,
                                                          const int *__restrict__ ipiv,
                                                          bool forward,
                                                          const double *__restrict__ B, long ldb,
                                                          double *Y, long ldy) {
  __shared__ int sp[1024];
  const int i = blockIdx.x * 128 + threadIdx.x;
  int pos = i;
  for (int q = 0; q * 1024 < n; ++q) {
    const int lo = forward ? max(0, n - 1024 * (q + 1)) : 1024 * q;
    const int len = forward ? n - 1024 * q - lo : min(1024, n - lo);
    __syncthreads();
    for (int e = threadIdx.x; e < len; e += 128) sp[e] = ipiv[lo + e] - 1;
    __syncthreads();
    if (forward) {
#pragma unroll 8
      for (int e = len - 1; e >= 0; --e) {
        const int p = sp[e], j = lo + e;
        pos = pos == j ? p : (pos == p ? j : pos);
      }
    } else {
#pragma unroll 8
      for (int e = 0; e < len; ++e) {
        const int p = sp[e], j = lo + e;
        pos = pos == j ? p : (pos == p ? j : pos);
      }
    }
  }
  if (i < n) {
    const bool ok = (unsigned)pos < (unsigned)n;
    for (int c = 0; c < nrhs; ++c)
      Y[i + (long)c * ldy] = ok ? __ldcg(B + pos + (long)c * ldb)
                                : __longlong_as_double(0x7ff8000000000000ll);
  }
}

int perm_gather_f64(int n, int nrhs, const int *ipiv, bool forward, const double *B, long ldb,
                    double *Y, long ldy, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  ZG_LAUNCH(kTagLaswp, 0, 16.0 * n * nrhs, s,
            perm_gather_kernel<<<ceil_div(n, 128), 128, 0, s>>>(n, nrhs, ipiv, forward, B, ldb,
                                                                Y, ldy));
  return 0;
}

template <bool TRANS>
static int trsv_f64_launch(int n, const double *A, long lda, const double *rhs, double *x,
                           bool upper, bool unit, double *xpub, unsigned *ticket,
                           unsigned *status, cudaStream_t s) {
  const size_t smem = sizeof(double) * kFB * kFLD;
  ZG_TRY(smem_optin(trsv_f64_kernel<TRANS>, (int)smem));
  ZG_LAUNCH(kTagTrsmDiag, 1.0 * n * n, 4.0 * n * n + 16.0 * n, s,
            trsv_f64_kernel<TRANS><<<ceil_div(n, kFB), kFT, smem, s>>>(
                n, A, lda, rhs, x, xpub, ticket, upper, unit, status));
  return 0;
}

int trsv_f64(int n, const double *A, long lda, bool trans, bool upper, bool unit,
             const double *rhs, double *x, double *xw, Control *ctl, cudaStream_t s) {
  if (n <= 0) return 0;
  unsigned *ticket = reinterpret_cast<unsigned *>(xw);
  double *xpub = xw + 1;
  ZG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
  ZG_CUDA(cudaMemsetAsync(xpub, 0xff, sizeof(double) * n, s));
  if (trans) return trsv_f64_launch<true>(n, A, lda, rhs, x, upper, unit, xpub, ticket,
                                          &ctl->status, s);
  return trsv_f64_launch<false>(n, A, lda, rhs, x, upper, unit, xpub, ticket, &ctl->status, s);
}

template <typename T>
int getrs_dev(int trans, int n, int nrhs, const T *A, long lda, const int *ipiv, T *B, long ldb,
              cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  const bool nt = trans == kNoTrans || trans == kConjNoTrans;
  if constexpr (sizeof(T) == sizeof(double)) {
    // a few right-hand sides: one launch per column and triangle
    if (nrhs <= kTrsvMaxRhs && n >= kTrsvMinN) {
      void *w;
      ZG_TRY(workspace(s, kSlotPanel, sizeof(double) * ((size_t)n * (nrhs + 1) + 1), &w));
      double *xw = (double *)w, *Y = xw + n + 1;
      double *Bd = reinterpret_cast<double *>(B);
      const double *Ad = reinterpret_cast<const double *>(A);
      Control *ctl;  // one status word for every solve of the call
      ZG_TRY(control(s, &ctl));
      if (nt) {  // x = U^-1 L^-1 P b
        ZG_TRY(perm_gather_f64(n, nrhs, ipiv, true, Bd, ldb, Y, n, s));
        for (int c = 0; c < nrhs; ++c) {
          double *x = Bd + (long)c * ldb;
          ZG_TRY(trsv_f64(n, Ad, lda, false, false, true, Y + (long)c * n, x, xw, ctl, s));
          ZG_TRY(trsv_f64(n, Ad, lda, false, true, false, x, x, xw, ctl, s));
        }
      } else {  // x = P^T L^-T U^-T b
        for (int c = 0; c < nrhs; ++c) {
          double *y = Y + (long)c * n;
          ZG_TRY(trsv_f64(n, Ad, lda, true, false, false, Bd + (long)c * ldb, y, xw, ctl, s));
          ZG_TRY(trsv_f64(n, Ad, lda, true, true, true, y, y, xw, ctl, s));
        }
        ZG_TRY(perm_gather_f64(n, nrhs, ipiv, false, Y, n, Bd, ldb, s));
      }
      return check_status(s, ctl, nullptr);  // a poll that ran out: kErrTimeout
    }
  }
  if (nt) {
    ZG_TRY(laswp_dev<T>(nrhs, B, ldb, 1, n, ipiv, 1, s));
    ZG_TRY(trsm_dev<T>(kLeft, kLower, kNoTrans, kUnit, n, nrhs, T(1), A, lda, B, ldb, s));
    ZG_TRY(trsm_dev<T>(kLeft, kUpper, kNoTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
  } else {
    ZG_TRY(trsm_dev<T>(kLeft, kUpper, kTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
    ZG_TRY(trsm_dev<T>(kLeft, kLower, kTrans, kUnit, n, nrhs, T(1), A, lda, B, ldb, s));
    ZG_TRY(laswp_dev<T>(nrhs, B, ldb, 1, n, ipiv, -1, s));
  }
  return 0;
}

#define INST(T)                                                                                 \
  template int laswp_panel<T>(int, int, int, T *, long, int, int, const int *, cudaStream_t);    \
  template int panel_lu<T>(int, int, T *, long, int *, int, Control *, int, cudaStream_t);      \
  template int laswp_dev<T>(int, T *, long, int, int, const int *, int, cudaStream_t);          \
  template int getrf_dev<T>(int, int, T *, long, int *, int *, cudaStream_t, bool);          \
  template int getrf_simt<T>(int, int, T *, long, int *, int *, cudaStream_t, bool);                   \
  template int getrs_dev<T>(int, int, int, const T *, long, const int *, T *, long, cudaStream_t);
INST(double)
INST(float)
#undef INST
// complex elements: the interchanges move 16- / 8-byte pairs
template int laswp_dev<double2>(int, double2 *, long, int, int, const int *, int, cudaStream_t);
template int laswp_dev<float2>(int, float2 *, long, int, int, const int *, int, cudaStream_t);

}  // namespace zg

// ===========================================================================
// LU without any allocation: zml_gpu_dgetrf_noalloc.
//
// Some callers cannot allocate device memory at solve time: hosts whose device
// memory belongs to another allocator (a framework's caching allocator, a fixed
// arena set up at start-up, which a cudaMalloc from the library would fragment
// or overrun), and real-time loops that may not allocate after initialisation.  This entry point gives them the FP64
// getrf with every scratch buffer it needs -- the panel's control words, the
// candidate-pivot exchange and the composed row-interchange pairs -- carved
// from one static device array that every GPU loading the library holds
// until the process exits.  The caller passes only the matrix, the pivot
// vector and the info pointer.
namespace zg {
namespace {

constexpr int kNaMaxCtas = 256;   // panel CTAs the exchange has room for (SMs per device)
constexpr int kNaNb = 64;         // panel width of the FP64 factorization
constexpr size_t kNaCtlBytes = 256;
constexpr size_t kNaSwapBytes = sizeof(int) * (4 * kSwapMax + 8);
constexpr size_t kNaSwapOff = kNaCtlBytes;
constexpr size_t kNaXchgOff = (kNaSwapOff + kNaSwapBytes + 255) / 256 * 256;
constexpr size_t kNaXchgWords = 2 * (size_t)kNaMaxCtas * (kNaNb + 2) + 2 * kNaNb;
constexpr size_t kNaBytes = kNaXchgOff + sizeof(double) * kNaXchgWords;  // ~273 KB

// The scratch.  Shared by every call on a device: calls that overlap on the
// GPU (two streams, two host threads) race on it.  Its control words are
// cleared at the start of every call; the rest needs no initial value.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NaDevice {
  unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
  int sms = 0;
  int smem_optin = 0;
};
constexpr int kNaMaxDevices = 64;
NaDevice g_na_dev[kNaMaxDevices];
std::mutex g_na_mu;

// Once per device, with that device current: resolve the array's device
// address (the host-side symbol is only a stand-in and must never be passed
// to a kernel) and the launch limits.  Runs on the first call on a device.
int noalloc_setup(NaDevice **out) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) {
    set_last_error("dgetrf_noalloc: device ordinal %d beyond %d", dev, kNaMaxDevices);
    return kErrInvalid;
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  NaDevice &d = g_na_dev[dev];
  if (!d.scratch) {
    void *p = nullptr;
    ZG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    ZG_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    ZG_CUDA(cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    ZG_CUDA(cudaFuncSetAttribute(panel_lu_kernel<double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 d.smem_optin - 4096));
    d.scratch = (unsigned char *)p;
  }
  *out = &d;
  return 0;
}

// Rows one panel launch can hold: every CTA keeps R rows x kNaNb columns in
// shared memory, at most one CTA per SM.
int noalloc_max_rows(const NaDevice &d) {
  const int rmax = (d.smem_optin - 4096) / (kNaNb * (int)sizeof(double));
  return std::min(d.sms, kNaMaxCtas) * rmax;
}

int na_panel(const NaDevice &d, int m, int nb, double *A, long lda, int *ipiv, int base,
             Control *ctl, double *xchg, cudaStream_t s) {
  int nblk = std::min(std::min(d.sms, kNaMaxCtas), ceil_div(m, 8));
  int R = ceil_div(m, nblk);
  nblk = ceil_div(m, R);
  const size_t smem = (size_t)R * nb * sizeof(double);
  ZG_CUDA(cudaMemsetAsync(&ctl->barrier[0], 0, 2 * sizeof(unsigned), s));
  unsigned long long *winners = nullptr;  // used by FP32 panels only
  void *args[] = {&m, &nb, &A, &lda, &ipiv, &base, &ctl, &base, &R, &xchg, &winners};
  ZG_LAUNCH(kTagPanel, 1.0 * m * nb * nb, 2.0 * sizeof(double) * m * nb, s,
            ZG_CUDA(cudaLaunchCooperativeKernel((void *)panel_lu_kernel<double>, dim3(nblk),
                                                dim3(256), args, smem, s)));
  return 0;
}

int na_laswp(const NaDevice &d, int n, double *A, long lda, int k1, int k2, const int *ipiv,
             int *pairs, cudaStream_t s) {
  if (n <= 0 || k2 < k1) return 0;
  int *np = pairs + 4 * kSwapMax;
  ZG_LAUNCH(kTagLaswp, 0, 0, s, laswp_prep_kernel<<<1, 256, 0, s>>>(k1, k2, ipiv, 1, pairs, np));
  const int grid = std::min(ceil_div(n, 8), d.sms * 8);
  ZG_LAUNCH(kTagLaswp, 0, 4.0 * sizeof(double) * n * (k2 - k1 + 1), s,
            laswp_apply_kernel<double><<<grid, 256, 0, s>>>(n, A, lda, pairs, np));
  return 0;
}

}  // namespace
}  // namespace zg

using namespace zg;

// FP64 getrf (partial pivoting, 1-based ipiv, LAPACK info) on device memory
// with no allocation; same factorization, bit for bit, as zml_gpu_dgetrf with
// its updates on the FP64 pipe (below min(m, n) = 2048, or after
// zml_gpu_fp64_updates(0)); above that zml_gpu_dgetrf's default tensor-core
// updates agree with it to rounding.
// Returns 0, -(bad argument index), or a library error (ZML_GPU_ERR_INVALID
// with a message when m exceeds what one panel can hold on this device).
extern "C" int zml_gpu_dgetrf_noalloc(int m, int n, double *dA, int ldda, int *dipiv, int *info,
                                      void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, m)) return -4;
  if (info) *info = 0;
  if (m == 0 || n == 0) return 0;
  NaDevice *d;
  ZG_TRY(noalloc_setup(&d));
  if (m > noalloc_max_rows(*d)) {
    set_last_error("dgetrf_noalloc: m = %d exceeds the %d rows one panel holds on this device", m,
                   noalloc_max_rows(*d));
    return kErrInvalid;
  }
  if (d->sms > kNaMaxCtas) {
    set_last_error("dgetrf_noalloc: %d SMs exceed the scratch's %d panel slots", d->sms,
                   kNaMaxCtas);
    return kErrInvalid;
  }
  cudaStream_t s = (cudaStream_t)stream;
  Control *ctl = reinterpret_cast<Control *>(d->scratch);
  int *pairs = reinterpret_cast<int *>(d->scratch + kNaSwapOff);
  double *xchg = reinterpret_cast<double *>(d->scratch + kNaXchgOff);
  ZG_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Control), s));  // counters, status, info start at zero
  const long lda = ldda;
  const int mn = std::min(m, n);
  for (int j = 0; j < mn; j += kNaNb) {
    const int jb = std::min(kNaNb, mn - j);
    double *Ajj = dA + j + (long)j * lda;
    ZG_TRY(na_panel(*d, m - j, jb, Ajj, lda, dipiv + j, j, ctl, xchg, s));
    ZG_TRY(na_laswp(*d, j, dA, lda, j + 1, j + jb, dipiv, pairs, s));
    if (j + jb < n) {
      double *Aright = dA + (long)(j + jb) * lda;
      ZG_TRY(na_laswp(*d, n - j - jb, Aright, lda, j + 1, j + jb, dipiv, pairs, s));
      ZG_TRY(trsm_dev<double>(kLeft, kLower, kNoTrans, kUnit, jb, n - j - jb, 1.0, Ajj, lda,
                              Aright + j, lda, s));
      if (j + jb < m)
        ZG_TRY(gemm_simt<double>(kNoTrans, kNoTrans, m - j - jb, n - j - jb, jb, -1.0, Ajj + jb,
                                 lda, Aright + j, lda, 1.0, Aright + j + jb, lda, 0, s));
    }
  }
  int inf = 0;
  ZG_TRY(check_status(s, ctl, &inf));
  if (info) *info = inf;
  return 0;
}
