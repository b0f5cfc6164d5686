// LU panel (FP32, partial pivoting) factored by one thread-block cluster.
//
// The mixed-precision LU factors each 128-column half-panel of an FP32
// matrix with partial pivoting (the unblocked step of getrf.zig:56-79, the
// getf2 loop of getf2.zig).  Its cost is the chain of pivot searches: every
// column needs the largest entry of the whole remaining column before the
// next column can start.  A grid-wide barrier through L2 costs about 1.3 us
// and the pivot row is one more dependent L2 read; a cluster barrier costs
// about 0.4 us and candidate rows can be pushed into every CTA's shared
// memory before it, so a column takes one barrier and no dependent global
// read.
//
// Layout.  Up to 16 CTAs of 512 threads form one cluster; CTA q owns the
// panel rows [q R, (q+1) R), R = 512 RPT, and thread t owns rows
// q R + t + 512 i, i < RPT.  The panel is factored in sub-panels of W
// columns (W RPT = 64 FP32 registers a thread).  Within a sub-panel the
// columns not yet factored live in registers, rotated so that the current
// column is always register 0 (every register index stays static and the
// column loop needs no unrolling); finished columns move to shared memory.
//   per column k: local argmax (one packed 64-bit word: |v| order bits above
//   the inverted row, so the maximum is the largest |v|, lowest row on a
//   tie) folded with a shared-memory atomicMax; the CTA's winning row, its
//   word and the old row k are pushed into every CTA's exchange slots; one
//   cluster barrier; every warp reduces the words with shuffles, and every
//   CTA swaps, scales and updates its rows.
// Between sub-panels: the sub-panel is written back; its interchanges are
// composed into (destination, source) pairs and applied to the panel's other
// columns (column-partitioned over the CTAs); U12 = L11^-1 A12 is solved by
// every CTA into shared memory (CTA 0 writes it back) and each CTA updates
// its own rows of the columns to the right, A22 -= L21 U12, with L21 loaded
// into registers.
#include "common.cuh"
#include "kernels.h"

namespace zg {
namespace {

constexpr int kPcThreads = 512;
constexpr int kPcMaxCta = 16;
constexpr int kPcMaxNb = 128;
constexpr int kPcSlot = 64;          // row values; entries W..63 stay zero
constexpr int kPcMaxRight = kPcMaxNb - 16;
constexpr int kPcUStride = 36;       // U12 tile row stride (16-byte aligned rows)

__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cl_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
__device__ __forceinline__ unsigned remote_addr(const void *local, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster(unsigned addr, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(unsigned addr, unsigned long long v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// Candidate word of row `row` with value v for pivot column k: a NaN counts
// as +inf on the diagonal and as -inf below it; -inf orders below every
// finite key.  Zero means "no candidate".
__device__ __forceinline__ unsigned long long pc_word(float v, int row, int k) {
  float key = fabsf(v);
  if (v != v) key = row == k ? INFINITY : -INFINITY;
  const unsigned ord = key == -INFINITY ? 0u : __float_as_uint(key) + 1u;
  return ((unsigned long long)ord << 32) | (unsigned)(0xffffffffu - (unsigned)row);
}
__device__ __forceinline__ int pc_row(unsigned long long w) {
  return (int)(0xffffffffu - (unsigned)(w & 0xffffffffu));
}

struct __align__(16) PcShared {
  float slot[2][kPcMaxCta][kPcSlot];  // candidate rows pushed by every CTA (parity k & 1)
  float rowk[2][32];                  // row k before the interchange, pushed by CTA 0
  float cand[32];                     // this CTA's winning row, staged for the push
  float krow[32];                     // row k, staged by its owner
  unsigned long long cmax[2];         // this CTA's best candidate word (atomicMax)
  unsigned long long skey[2][kPcMaxCta];  // every CTA's best word, pushed by that CTA
  int piv[32];                        // pivot rows of the sub-panel (panel-relative)
  int mdst[64], msrc[64];             // the sub-panel's interchanges, composed
  float L11[32][33];                  // unit-lower diagonal block of the sub-panel
  alignas(16) float U[kPcMaxRight][kPcUStride];  // U12 by right column: U[c][k]
};

// Row whose old content ends in row x after the swaps (c0 + t, piv[t]), t < ws.
__device__ __forceinline__ int pc_trace(int x, int c0, int ws, const int *piv) {
  for (int t = ws - 1; t >= 0; --t) {
    const int k = c0 + t, p = piv[t];
    if (x == k) x = p;
    else if (x == p) x = k;
  }
  return x;
}

template <int RPT, int W>
__global__ void __launch_bounds__(kPcThreads, 1)
    panel_cluster_kernel(int m, int nb, float *__restrict__ A, long lda, int *__restrict__ ipiv,
                         int ipiv_base, Control *ctl, int info_base) {
  static_assert(W <= 32 && W % 4 == 0 && RPT * W <= 64, "sub-panel shape");
  __shared__ PcShared sh;
  extern __shared__ __align__(16) float Lsm[];  // finished columns: Lsm[c R + local row]
  const int rank = (int)cl_rank(), nct = (int)cl_size();
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int R = kPcThreads * RPT;
  const int r0 = rank * R;
  float v[RPT][W];
  for (int e = tid; e < 2 * kPcMaxCta * kPcSlot; e += kPcThreads) (&sh.slot[0][0][0])[e] = 0.f;
  if (tid < 2) sh.cmax[tid] = 0;
  // every CTA of the cluster runs, and its slots are zero, before any remote write
  cl_sync();

  for (int c0 = 0; c0 < nb; c0 += W) {
    const int ws = min(W, nb - c0);
    // A. the thread's rows of the sub-panel
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int row = r0 + tid + i * kPcThreads;
#pragma unroll
      for (int c = 0; c < W; ++c)
        v[i][c] = (row < m && c < ws) ? __ldcg(A + row + (long)(c0 + c) * lda) : 0.f;
    }

    // B. factor the sub-panel, one cluster barrier per column.  v[i][c]
    // holds column kk + c of the thread's rows; Lsm holds columns < kk.
#pragma unroll 1
    for (int kk = 0; kk < ws; ++kk) {
      const int k = c0 + kk, par = k & 1;
      unsigned long long best = 0;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int row = r0 + tid + i * kPcThreads;
        if (row >= k && row < m) best = max(best, pc_word(v[i][0], row, k));
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) best = max(best, __shfl_xor_sync(~0u, best, off));
      if (lane == 0 && best != 0) atomicMax(&sh.cmax[par], best);
      __syncthreads();
      // every thread has read the previous column's word: clear it for the next
      if (tid == 0) sh.cmax[par ^ 1] = 0;
      const unsigned long long cbest = sh.cmax[par];
      const int wrow = cbest != 0 ? pc_row(cbest) : -1;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int row = r0 + tid + i * kPcThreads, lr = tid + i * kPcThreads;
        if (row == wrow || row == k) {
          float *dst = row == wrow ? sh.cand : sh.krow;
          for (int c = 0; c < kk; ++c) dst[c] = Lsm[c * R + lr];
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (kk + c < W) dst[kk + c] = v[i][c];
          if (row == wrow && row == k)
            for (int c = 0; c < W; ++c) sh.krow[c] = sh.cand[c];
        }
      }
      __syncthreads();
      if (warp == 0) {
        const float val = lane < W ? sh.cand[lane] : 0.f;
        for (int d = 0; d < nct; ++d) {
          st_cluster(remote_addr(&sh.slot[par][rank][lane], d), val);
          if (lane == 0) st_cluster(remote_addr(&sh.skey[par][rank], d), cbest);
        }
      } else if (warp == 1 && rank == 0) {  // row k < nb <= R lies in CTA 0
        const float val = lane < W ? sh.krow[lane] : 0.f;
        for (int d = 0; d < nct; ++d) st_cluster(remote_addr(&sh.rowk[par][lane], d), val);
      }
      cl_sync();
      // the cluster's pivot, identical in every CTA
      unsigned long long g = lane < nct ? sh.skey[par][lane] : 0ull;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) g = max(g, __shfl_xor_sync(~0u, g, off));
      const int p = pc_row(g);
      const float *prow = sh.slot[par][p / R];
      const float piv = prow[kk];
      const bool swap = piv != 0.f && p != k;
      if (tid == 0) {
        sh.piv[kk] = swap ? p : k;
        if (rank == 0) {
          ipiv[k] = p + 1 + ipiv_base;
          if (piv == 0.f) atomicCAS(&ctl->info, 0, k + 1 + info_base);
        }
      }
      const bool recip = fabsf(piv) >= Real<float>::sfmin();
      const float rp = 1.f / piv;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int row = r0 + tid + i * kPcThreads, lr = tid + i * kPcThreads;
        if (swap && (row == k || row == p)) {
          const float *src = row == k ? prow : sh.rowk[par];
          for (int c = 0; c < kk; ++c) Lsm[c * R + lr] = src[c];
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (kk + c < W) v[i][c] = src[kk + c];
        }
        float x = v[i][0];
        const bool below = row > k && row < m;
        if (below && piv != 0.f) x = recip ? x * rp : x / piv;
        Lsm[kk * R + lr] = x;
        // rotate: column kk + 1 + c moves to register c
        if (below) {
#pragma unroll
          for (int c = 0; c + 1 < W; ++c) v[i][c] = fmaf(-x, prow[kk + 1 + c], v[i][c + 1]);
        } else {
#pragma unroll
          for (int c = 0; c + 1 < W; ++c) v[i][c] = v[i][c + 1];
        }
        v[i][W - 1] = 0.f;
      }
    }
    __syncthreads();

    // C. the factored sub-panel back to the panel; L21 into registers
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int row = r0 + tid + i * kPcThreads, lr = tid + i * kPcThreads;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        v[i][c] = c < ws ? Lsm[c * R + lr] : 0.f;
        if (row < m && c < ws) A[row + (long)(c0 + c) * lda] = v[i][c];
      }
    }
    __threadfence();
    cl_sync();

    // E. the sub-panel's interchanges in the panel's other columns
    if (tid < 2 * W) {
      int dst = -1, src = -1;
      if (tid < ws) {
        dst = c0 + tid;
      } else if (tid >= W && tid - W < ws) {
        const int t = tid - W, x = sh.piv[t];
        bool first = x >= c0 + ws;
        for (int u = 0; u < t && first; ++u) first = sh.piv[u] != x;
        if (first) dst = x;
      }
      if (dst >= 0) {
        src = pc_trace(dst, c0, ws, sh.piv);
        if (src == dst) dst = -1;
      }
      sh.mdst[tid] = dst;
      sh.msrc[tid] = src;
    }
    __syncthreads();
    {
      constexpr int kEnt = 2 * W, kCpr = kPcThreads / kEnt;  // entries per column, columns per round
      const int no = nb - ws;                                // the other columns
      const int mine = no > rank ? (no - rank + nct - 1) / nct : 0;
      const int e = tid % kEnt;
      const int dst = sh.mdst[e], src = sh.msrc[e];
      for (int base = 0; base < mine; base += kCpr) {
        const int jl = base + tid / kEnt;
        const bool act = jl < mine && dst >= 0;
        float val = 0.f;
        long col = 0;
        if (act) {
          const int j = rank + jl * nct;
          col = j < c0 ? j : j + ws;
          val = __ldcg(A + src + col * lda);
        }
        __syncthreads();
        if (act) A[dst + col * lda] = val;
      }
    }
    __threadfence();
    cl_sync();

    // G. U12 = L11^-1 A12 over the right columns, in every CTA
    const int nr = nb - c0 - ws;
    if (nr > 0) {
      for (int e = tid; e < ws * ws; e += kPcThreads) {
        const int r = e % ws, c = e / ws;
        sh.L11[r][c] = __ldcg(A + (c0 + r) + (long)(c0 + c) * lda);
      }
      for (int e = tid; e < ws * nr; e += kPcThreads) {
        const int r = e % ws, c = e / ws;
        sh.U[c][r] = __ldcg(A + (c0 + r) + (long)(c0 + ws + c) * lda);
      }
      __syncthreads();
      if (tid < nr) {
        float u[W];
#pragma unroll
        for (int r = 0; r < W; ++r) u[r] = r < ws ? sh.U[tid][r] : 0.f;
#pragma unroll
        for (int r = 1; r < W; ++r)
#pragma unroll
          for (int q = 0; q < r; ++q) u[r] = fmaf(-sh.L11[r][q], u[q], u[r]);
#pragma unroll
        for (int r = 0; r < W; ++r) sh.U[tid][r] = r < ws ? u[r] : 0.f;
      }
      __syncthreads();
      if (rank == 0)
        for (int e = tid; e < ws * nr; e += kPcThreads) {
          const int r = e % ws, c = e / ws;
          A[(c0 + r) + (long)(c0 + ws + c) * lda] = sh.U[c][r];
        }
      // H. A22 -= L21 U12 on this CTA's rows below the sub-panel
      const int rs = c0 + ws;
      for (int cb = 0; cb < nr; cb += 4) {
        float a[4][RPT];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * kPcThreads;
            a[q][i] = (cb + q < nr && row >= rs && row < m)
                          ? __ldcg(A + row + (long)(rs + cb + q) * lda)
                          : 0.f;
          }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (cb + q < nr) {
            const float *u = sh.U[cb + q];
#pragma unroll
            for (int k4 = 0; k4 < W / 4; ++k4) {
              const float4 uu = *reinterpret_cast<const float4 *>(u + 4 * k4);
#pragma unroll
              for (int i = 0; i < RPT; ++i) {
                a[q][i] = fmaf(-v[i][4 * k4 + 0], uu.x, a[q][i]);
                a[q][i] = fmaf(-v[i][4 * k4 + 1], uu.y, a[q][i]);
                a[q][i] = fmaf(-v[i][4 * k4 + 2], uu.z, a[q][i]);
                a[q][i] = fmaf(-v[i][4 * k4 + 3], uu.w, a[q][i]);
              }
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * kPcThreads;
            if (cb + q < nr && row >= rs && row < m) A[row + (long)(rs + cb + q) * lda] = a[q][i];
          }
      }
    }
    __syncthreads();
  }
}

struct PcState {
  bool checked = false, ok = false;
};

template <int RPT, int W>
int launch_pc(int m, int nb, float *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
              int info_base, cudaStream_t s, bool *launched) {
  constexpr int R = kPcThreads * RPT;
  const int nct = ceil_div(m, R);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = nct;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(nct);
  cfg.blockDim = dim3(kPcThreads);
  const size_t lsm = sizeof(float) * R * W;
  cfg.dynamicSmemBytes = lsm;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  static PcState st[kPcMaxCta + 1];
  if (!st[nct].checked) {
    st[nct].checked = true;
    ZG_CUDA(cudaFuncSetAttribute(panel_cluster_kernel<RPT, W>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    ZG_CUDA(cudaFuncSetAttribute(panel_cluster_kernel<RPT, W>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm));
    int nclusters = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveClusters(&nclusters, (void *)panel_cluster_kernel<RPT, W>, &cfg);
    if (e != cudaSuccess) (void)cudaGetLastError();
    st[nct].ok = e == cudaSuccess && nclusters >= 1;
  }
  if (!st[nct].ok) return 0;
  ZG_LAUNCH(kTagPanel, 1.0 * m * nb * nb, 2.0 * sizeof(float) * m * nb, s,
            ZG_CUDA(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<RPT, W>, m, nb, A, lda, ipiv,
                                       ipiv_base, ctl, info_base)));
  *launched = true;
  return 0;
}

}  // namespace

int panel_lu_cluster(int m, int nb, float *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool *launched) {
  *launched = false;
  if (m <= 0 || nb <= 0) {
    *launched = true;
    return 0;
  }
  if (nb > kPcMaxNb || m < nb) return 0;
  if (m <= kPcMaxCta * kPcThreads * 2)
    return launch_pc<2, 32>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s, launched);
  if (m <= kPcMaxCta * kPcThreads * 4)
    return launch_pc<4, 16>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s, launched);
  return 0;
}

}  // namespace zg
