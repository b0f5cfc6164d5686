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
// Layout.  Up to 16 CTAs of T <= 512 threads form one cluster; CTA q owns
// the panel rows [q R, (q+1) R), R = T RPT, and thread t owns rows
// q R + t + T i, i < RPT.  T is the smallest multiple of 32 (at least 128
// and enough for nb rows) that spreads the rows over 16 CTAs, so shorter
// panels get less work a thread.  The panel is factored in sub-panels of W
// columns (W RPT = 64 FP32 registers a thread).  Within a sub-panel the
// columns not yet factored live in registers, rotated so that the current
// column is always register 0 (every register index stays static and the
// column loop needs no unrolling); finished columns move to shared memory.
//   per column k: local argmax (one packed 64-bit word: |v| order bits above
//   the inverted row, so the maximum is the largest |v|, lowest row on a
//   tie) folded with a shared-memory atomicMax; the CTA's winning row, its
//   word and the old row k are pushed into every CTA's exchange slots with
//   st.async, each store completing its bytes on the destination's mbarrier
//   (no cluster barrier, no fence); every CTA waits for its own mbarrier,
//   reduces the words with redux.sync, swaps, scales and updates its rows.
// Between sub-panels: the sub-panel is written back; its interchanges are
// composed into (destination, source) pairs and applied to the panel's other
// columns and to up to two extra column ranges beside the panel (the rest of
// the caller's column block), column-partitioned over the CTAs; U12 =
// L11^-1 A12 is solved by every CTA into shared memory (CTA 0 writes it
// back) and each CTA updates
// its own rows of the columns to the right, A22 -= L21 U12, with L21 loaded
// into registers.
#include <map>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace zg {
namespace {

constexpr int kPcThreads = 512;
constexpr int kPcMaxCta = 16;
constexpr int kPcMaxNb = 128;
constexpr int kPcSlot = 64;          // row values; entries W..63 stay zero
constexpr int kPcMaxRight = kPcMaxNb - 8;  // right of the first sub-panel (W >= 8)
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
// Remote stores that complete their bytes on the destination CTA's mbarrier.
__device__ __forceinline__ void st_async(unsigned addr, float v, unsigned mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(
                   addr),
               "f"(v), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void st_async(unsigned addr, unsigned long long v, unsigned mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(
                   addr),
               "l"(v), "r"(mbar)
               : "memory");
}

__device__ __forceinline__ void st_async(unsigned addr, double v, unsigned mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(
                   addr),
               "l"(__double_as_longlong(v)), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void st_async(unsigned addr, int v, unsigned mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(
                   addr),
               "r"(v), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ float fmae(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmae(double a, double b, double c) { return fma(a, b, c); }
// four consecutive elements of a 16-byte aligned shared-memory row
__device__ __forceinline__ void load4(const float *p, float &a, float &b, float &c, float &d) {
  const float4 q = *reinterpret_cast<const float4 *>(p);
  a = q.x;
  b = q.y;
  c = q.z;
  d = q.w;
}
__device__ __forceinline__ void load4(const double *p, double &a, double &b, double &c,
                                      double &d) {
  const double2 q0 = reinterpret_cast<const double2 *>(p)[0];
  const double2 q1 = reinterpret_cast<const double2 *>(p)[1];
  a = q0.x;
  b = q0.y;
  c = q1.x;
  d = q1.y;
}

// binary64 candidate key of row `row` with value v for pivot column k: the
// bits of |v| + 1 (positive doubles order as integers), a NaN counting as
// +inf on the diagonal and as "no candidate" (0) below it.  Ties of the key
// go to the lower row, so (key, row) orders exactly as the restatement's
// first-maximum search.
__device__ __forceinline__ unsigned long long pd_key(double v, int row, int k) {
  double key = fabs(v);
  if (v != v) key = row == k ? INFINITY : -INFINITY;
  return key == -INFINITY ? 0ull : (unsigned long long)__double_as_longlong(key) + 1ull;
}
// The warp's largest (key, row): the largest key, then the lowest row among
// the lanes that hold it; every lane receives it.
__device__ __forceinline__ void warp_lexmax(unsigned long long &key, int &row) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mh = __reduce_max_sync(~0u, hi);
  const unsigned ml = __reduce_max_sync(~0u, hi == mh ? lo : 0u);
  const unsigned long long mk = ((unsigned long long)mh << 32) | ml;
  const int r = (int)__reduce_min_sync(~0u, key == mk ? (unsigned)row : 0xffffffffu);
  key = mk;
  row = r;
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
// The tournament's word: as pc_word, but a NaN below the diagonal orders just
// above zero instead of at zero, so that every row still in play remains a
// candidate and each elimination step always finds a pivot row.
__device__ __forceinline__ unsigned long long tw_word(float v, int row, int k) {
  float key = fabsf(v);
  if (v != v) key = row == k ? INFINITY : -INFINITY;
  const unsigned ord = key == -INFINITY ? 1u : __float_as_uint(key) + 2u;
  return ((unsigned long long)ord << 32) | (unsigned)(0xffffffffu - (unsigned)row);
}
// Warp maximum of 64-bit words: the high halves first, then the low halves
// among the lanes that hold the highest one.
__device__ __forceinline__ unsigned long long warp_max64(unsigned long long w) {
  const unsigned hi = (unsigned)(w >> 32), lo = (unsigned)w;
  const unsigned mh = __reduce_max_sync(~0u, hi);
  const unsigned ml = __reduce_max_sync(~0u, hi == mh ? lo : 0u);
  return ((unsigned long long)mh << 32) | ml;
}
__device__ __forceinline__ int pc_row(unsigned long long w) {
  return (int)(0xffffffffu - (unsigned)(w & 0xffffffffu));
}

// Exchange buffers are used round robin over three columns.  Column k + 3's
// pushes into buffer k % 3 cannot start before this CTA has pushed column
// k + 2, by which time every thread here is done with column k's rows.
constexpr int kPcBuf = 3;

template <typename E> struct __align__(16) PcShared {
  // Exchanged rows at column kk, 64 words: [c] = column kk + 1 + c (zero
  // past the register window), [32] = column kk, [33 + c] = finished column
  // c < kk.
  E slot[kPcBuf][kPcMaxCta][kPcSlot];      // candidate rows pushed by every CTA
  E rowk[kPcBuf][kPcSlot];                 // row k before the interchange, pushed by CTA 0
  E cand[33];                              // this CTA's winning row (register part), staged
  E krow[33];                              // row k (register part), staged by its owner
  unsigned long long cmax[2];              // this CTA's best candidate word (atomicMax)
  unsigned long long skey[kPcBuf][kPcMaxCta];  // every CTA's best word, pushed by that CTA
  // binary64: each warp's best (key, row) and every CTA's best row beside its key
  unsigned long long wkey[2][kPcThreads / 32];
  int wrow[2][kPcThreads / 32];
  int srow[kPcBuf][kPcMaxCta];
  uint64_t mbar[kPcBuf];                   // completes when a column's pushes have all landed
  int piv[32];                             // pivot rows of the sub-panel (panel-relative)
  int mdst[64], msrc[64];                  // the sub-panel's interchanges, composed
  E L11[32][33];                           // unit-lower diagonal block of the sub-panel
  // tournament pivoting (TOURN): the CTA's local candidates, the cluster's
  // pivot rows in order, U11 of the sub-panel and 1 / its diagonal, the
  // argmax words of the final elimination and the exchange's mbarrier
  int lcand[32];
  int fpiv[32];
  E U11[32][33];
  E rdiag[32];
  unsigned long long fmax[2];
  uint64_t tmbar;
  alignas(16) E U[kPcMaxRight][kPcUStride];  // U12 by right column: U[c][k]
};

// Bytes of the exchange state at the start of the dynamic shared memory
// (16-byte aligned, so the finished columns after it are too).
template <typename E> __host__ __device__ constexpr int pc_state_bytes() {
  return (int)((sizeof(PcShared<E>) + 15) / 16 * 16);
}

// Row whose old content ends in row x after the swaps (c0 + t, piv[t]), t < ws.
__device__ __forceinline__ int pc_trace(int x, int c0, int ws, const int *piv) {
  for (int t = ws - 1; t >= 0; --t) {
    const int k = c0 + t, p = piv[t];
    if (x == k) x = p;
    else if (x == p) x = k;
  }
  return x;
}

template <typename E, int RPT, int W, bool TOURN>
__global__ void __launch_bounds__(kPcThreads, 1)
    panel_cluster_kernel(int m, int nb, E *__restrict__ A, long lda, int *__restrict__ ipiv,
                         int ipiv_base, Control *ctl, int info_base, E *XL, int xl, E *XR,
                         int xr) {
  static_assert(W >= 8 && W <= 32 && W % 4 == 0 && RPT * W <= 64, "sub-panel shape");
  // the exchange state, then the finished columns: Lsm[c LD + local row]
  extern __shared__ __align__(16) unsigned char pc_smem[];
  PcShared<E> &sh = *reinterpret_cast<PcShared<E> *>(pc_smem);
  E *Lsm = reinterpret_cast<E *>(pc_smem + pc_state_bytes<E>());
  const int rank = (int)cl_rank(), nct = (int)cl_size();
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int T = blockDim.x, nwarps = T >> 5, R = T * RPT;
  const int LD = R + 1;  // Lsm column stride, odd: a row's finished columns hit distinct banks
  const int r0 = rank * R;
  E v[RPT][W];
  constexpr bool kF64 = sizeof(E) == 8;
  for (int e = tid; e < kPcBuf * kPcMaxCta * kPcSlot; e += T) (&sh.slot[0][0][0])[e] = E(0);
  // bytes landing in this CTA per column: every CTA's candidate row (two
  // values a lane) and word (binary64: key and row), and row k from CTA 0
  const unsigned xbytes = nct * (2 * 32 * sizeof(E) + 8 + (kF64 ? 4 : 0)) + 2 * 32 * sizeof(E);
  // tournament: every CTA's W candidate rows (W values and the row) and, from
  // CTA 0, the sub-panel's W top rows land in this CTA's Lsm once per sub-panel
  const unsigned tbytes = (unsigned)(nct * W * (W + 1) + W * W) * 4u;
  if (tid < 2) sh.cmax[tid] = sh.fmax[tid] = 0;
  if (tid == 0) {
    if constexpr (TOURN) {
      tc::mbar_init(&sh.tmbar, 1);
      tc::fence_barrier_init();
      tc::mbar_expect_tx(&sh.tmbar, tbytes);
    } else {
      for (int q = 0; q < kPcBuf; ++q) tc::mbar_init(&sh.mbar[q], 1);
      tc::fence_barrier_init();
      for (int q = 0; q < kPcBuf; ++q) tc::mbar_expect_tx(&sh.mbar[q], xbytes);
    }
  }
  // every CTA of the cluster runs, and its slots and mbarriers are ready,
  // before any remote write
  cl_sync();

  for (int c0 = 0; c0 < nb; c0 += W) {
    const int ws = min(W, nb - c0);
    // A. the thread's rows of the sub-panel
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int row = r0 + tid + i * T;
#pragma unroll
      for (int c = 0; c < W; ++c)
        v[i][c] = (row < m && c < ws) ? __ldcg(A + row + (long)(c0 + c) * lda) : E(0);
    }

    if constexpr (TOURN) {
      // B'. Tournament pivoting (communication-avoiding LU, flat tree over the
      // cluster): the sub-panel's pivots come from one exchange instead of one
      // per column.
      //  1. every CTA runs partial-pivot elimination on its own rows only (a
      //     CTA-wide argmax a column, no cluster traffic) to pick W candidate
      //     rows;
      //  2. it pushes their original values (re-read from A, which still holds
      //     the sub-panel as it entered) into every CTA, and CTA 0 also pushes
      //     the sub-panel's top W rows;
      //  3. every CTA eliminates the <= 16 W candidates in the same order and
      //     so chooses the same W pivot rows, with U11 and the pivot rows'
      //     multipliers L11;
      //  4. each row's multipliers are its original values times U11^-1
      //     (forward substitution), which is what elimination with those
      //     pivots computes; the results go to Lsm for phase C.
      float *rcv = Lsm;                          // [nct W][W + 1]: values, then the row
      float *top = Lsm + (long)nct * W * (W + 1);  // [W][W]: rows c0 .. c0 + W - 1
      // 1. local selection
      if (tid < 2) sh.cmax[tid] = sh.fmax[tid] = 0;
      __syncthreads();
      unsigned used = 0;  // bit i: the thread's row i is a candidate already
#pragma unroll 1
      for (int kk = 0; kk < ws; ++kk) {
        const int k = c0 + kk, par = kk & 1;
        unsigned long long best = 0;
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T;
          if (!((used >> i) & 1u) && row >= c0 && row < m)
            best = max(best, tw_word(v[i][0], row, k));
        }
        best = warp_max64(best);
        if (lane == 0 && best != 0) atomicMax(&sh.cmax[par], best);
        __syncthreads();
        if (tid == 0) sh.cmax[par ^ 1] = 0;
        const unsigned long long cb = sh.cmax[par];
        const int lrow = cb != 0 ? pc_row(cb) : -1;
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T;
          if (row == lrow) {
#pragma unroll
            for (int c = 0; c + 1 < W; ++c) sh.cand[c] = v[i][c + 1];
            sh.cand[32] = v[i][0];
            used |= 1u << i;
          }
        }
        if (tid == 0) sh.lcand[kk] = lrow;
        __syncthreads();
        const float piv = lrow >= 0 ? sh.cand[32] : 0.f;
        const bool recip = fabsf(piv) >= Real<float>::sfmin();
        const float rp = 1.f / piv;
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T;
          if (!((used >> i) & 1u) && row >= c0 && row < m && lrow >= 0) {
            float x = v[i][0];
            if (piv != 0.f) x = recip ? x * rp : x / piv;
#pragma unroll
            for (int c = 0; c + 1 < W; ++c) v[i][c] = fmaf(-x, sh.cand[c], v[i][c + 1]);
          } else {
#pragma unroll
            for (int c = 0; c + 1 < W; ++c) v[i][c] = v[i][c + 1];
          }
          v[i][W - 1] = 0.f;
        }
      }
      for (int kk = ws + tid; kk < W; kk += T) sh.lcand[kk] = -1;
      __syncthreads();
      // 2. the exchange: slot q of CTA `rank` lands in rcv row rank W + q
      for (int q = warp; q < W; q += nwarps) {
        const int row = sh.lcand[q];
        const float val = (row >= 0 && lane < ws) ? __ldcg(A + row + (long)(c0 + lane) * lda) : 0.f;
        for (int d = 0; d < nct; ++d) {
          const unsigned mb = remote_addr(&sh.tmbar, d);
          const unsigned dst = remote_addr(rcv + (long)(rank * W + q) * (W + 1), d);
          if (lane < W) st_async(dst + 4u * lane, val, mb);
          if (lane == 0) st_async(dst + 4u * W, __int_as_float(row), mb);
        }
      }
      if (rank == 0)
        for (int t = warp; t < W; t += nwarps) {
          const float val =
              (t < ws && lane < ws) ? __ldcg(A + (c0 + t) + (long)(c0 + lane) * lda) : 0.f;
          for (int d = 0; d < nct; ++d) {
            const unsigned mb = remote_addr(&sh.tmbar, d);
            if (lane < W) st_async(remote_addr(top + t * W + lane, d), val, mb);
          }
        }
      tc::mbar_wait(&sh.tmbar, (c0 / W) & 1, &ctl->status);
      if (tid == 0) tc::mbar_expect_tx(&sh.tmbar, tbytes);  // armed for the next sub-panel
      // 3. the final elimination over the candidates, one a thread, the same
      // in every CTA; a candidate's multipliers are kept in its rcv row
      const int ncand = nct * W;
      int cid = -1;
      float cr[W];
#pragma unroll
      for (int c = 0; c < W; ++c) cr[c] = 0.f;
      if (tid < ncand) {
        cid = __float_as_int(rcv[tid * (W + 1) + W]);
        if (cid < c0 || cid >= m) cid = -1;  // an empty slot (or words left by a timeout)
#pragma unroll
        for (int c = 0; c < W; ++c) cr[c] = rcv[tid * (W + 1) + c];
      }
      bool cdone = cid < 0;
#pragma unroll 1
      for (int j = 0; j < ws; ++j) {
        const int k = c0 + j, par = j & 1;
        unsigned long long best = cdone ? 0ull : tw_word(cr[0], cid, k);
        best = warp_max64(best);
        if (lane == 0 && best != 0) atomicMax(&sh.fmax[par], best);
        __syncthreads();
        if (tid == 0) sh.fmax[par ^ 1] = 0;
        const unsigned long long g = sh.fmax[par];
        const int prow = g != 0 ? pc_row(g) : -1;
        if (!cdone && cid == prow) {  // this candidate is pivot j: U11 row j, L11 row j
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (j + c < W) sh.U11[j][j + c] = cr[c];
          for (int c = 0; c < j; ++c) sh.L11[j][c] = rcv[tid * (W + 1) + c];
          cdone = true;
        }
        if (tid == 0) {
          sh.fpiv[j] = prow;
          if (prow < 0) {  // no candidate left (only after a timeout): a zero step
#pragma unroll 1
            for (int c = j; c < W; ++c) sh.U11[j][c] = 0.f;
            for (int c = 0; c < j; ++c) sh.L11[j][c] = 0.f;
          }
        }
        __syncthreads();
        const float piv = sh.U11[j][j];
        const bool recip = fabsf(piv) >= Real<float>::sfmin();
        const float rp = 1.f / piv;
        if (!cdone) {
          float x = cr[0];
          if (piv != 0.f) x = recip ? x * rp : x / piv;
          rcv[tid * (W + 1) + j] = x;
#pragma unroll
          for (int c = 0; c + 1 < W; ++c)
            cr[c] = j + 1 + c < W ? fmaf(-x, sh.U11[j][min(j + 1 + c, W - 1)], cr[c + 1]) : 0.f;
        } else {
#pragma unroll
          for (int c = 0; c + 1 < W; ++c) cr[c] = cr[c + 1];
        }
        cr[W - 1] = 0.f;
      }
      // the interchanges in LAPACK's form: step t swaps row c0 + t with the
      // row where pivot row fpiv[t] sits after steps 0 .. t-1
      if (tid == 0) {
        for (int t = 0; t < ws; ++t) {
          int pos = sh.fpiv[t];
          if (pos < c0 || pos >= m) pos = c0 + t;
          for (int u = 0; u < t; ++u) {
            if (pos == c0 + u) pos = sh.piv[u];
            else if (pos == sh.piv[u]) pos = c0 + u;
          }
          sh.piv[t] = pos;
          if (rank == 0) {
            ipiv[c0 + t] = pos + 1 + ipiv_base;
            if (sh.U11[t][t] == 0.f) atomicCAS(&ctl->info, 0, c0 + t + 1 + info_base);
          }
        }
      }
      if (tid < W) {
        const float u = tid < ws ? sh.U11[tid][tid] : 1.f;
        sh.rdiag[tid] = 1.f / u;
      }
      __syncthreads();
      // 4. every row of this CTA: its factored sub-panel row into registers
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int lr = tid + i * T, x = r0 + lr;
        if (x >= m) {
#pragma unroll
          for (int c = 0; c < W; ++c) v[i][c] = 0.f;
        } else if (x < c0) {  // an earlier pivot row: unchanged
#pragma unroll
          for (int c = 0; c < W; ++c) v[i][c] = c < ws ? __ldcg(A + x + (long)(c0 + c) * lda) : 0.f;
        } else if (x < c0 + ws) {  // pivot position: L11 row, then U11 row
          const int t = x - c0;
#pragma unroll
          for (int c = 0; c < W; ++c) v[i][c] = c < ws ? (c < t ? sh.L11[t][c] : sh.U11[t][c]) : 0.f;
        } else {
          int src = pc_trace(x, c0, ws, sh.piv);  // x itself, or a displaced top row
          if (src < c0 || src >= c0 + ws) src = x;
#pragma unroll
          for (int c = 0; c < W; ++c) {
            float a = 0.f;
            if (c < ws) a = src == x ? __ldcg(A + x + (long)(c0 + c) * lda) : top[(src - c0) * W + c];
#pragma unroll
            for (int q = 0; q < c; ++q) a = fmaf(-v[i][q], sh.U11[q][c], a);
            if (c < ws) {
              const float u = sh.U11[c][c];
              if (u != 0.f) a = fabsf(u) >= Real<float>::sfmin() ? a * sh.rdiag[c] : a / u;
            }
            v[i][c] = c < ws ? a : 0.f;
          }
        }
      }
      __syncthreads();  // every read of rcv / top is done: Lsm takes the results
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int lr = tid + i * T;
#pragma unroll
        for (int c = 0; c < W; ++c)
          if (c < ws) Lsm[c * LD + lr] = v[i][c];
      }
      __syncthreads();
    } else {
      // B. factor the sub-panel, one exchange per column.  v[i][c] holds
      // column kk + c of the thread's rows; Lsm holds columns < kk.
  #pragma unroll 1
      for (int kk = 0; kk < ws; ++kk) {
        const int k = c0 + kk, par = k & 1, b = k % kPcBuf;
        unsigned long long cbest;  // the CTA's candidate word (binary64: its key)
        int wrow;                  // its row, -1 when the CTA has none
        if constexpr (!kF64) {
          unsigned long long best = 0;
  #pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * T;
            if (row >= k && row < m) best = max(best, pc_word(v[i][0], row, k));
          }
          best = warp_max64(best);
          if (lane == 0 && best != 0) atomicMax(&sh.cmax[par], best);
          __syncthreads();
          // every thread has read the previous column's word: clear it for the next
          if (tid == 0) sh.cmax[par ^ 1] = 0;
          cbest = sh.cmax[par];
          wrow = cbest != 0 ? pc_row(cbest) : -1;
        } else {
          // binary64 keys need the whole 64 bits: (key, row) pairs reduced
          // per warp, then over the CTA's warps (by every warp alike)
          unsigned long long key = 0;
          int krow_ = 0x7fffffff;
  #pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * T;
            if (row >= k && row < m) {
              const unsigned long long w = pd_key(v[i][0], row, k);
              if (w > key) {  // rows of a thread ascend: the first maximum stays
                key = w;
                krow_ = row;
              }
            }
          }
          warp_lexmax(key, krow_);
          if (lane == 0) {
            sh.wkey[par][warp] = key;
            sh.wrow[par][warp] = krow_;
          }
          __syncthreads();
          key = lane < nwarps ? sh.wkey[par][lane] : 0ull;
          krow_ = lane < nwarps ? sh.wrow[par][lane] : 0x7fffffff;
          warp_lexmax(key, krow_);
          cbest = key;
          wrow = key != 0 ? krow_ : -1;
        }
        // owners stage the register part of the CTA's winning row and of row k:
        // [c] = column kk + 1 + c, [32] = column kk
  #pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T;
          if (row == wrow || row == k) {
            E *dst = row == wrow ? sh.cand : sh.krow;
  #pragma unroll
            for (int c = 0; c + 1 < W; ++c) dst[c] = v[i][c + 1];
  #pragma unroll
            for (int c = W - 1; c < 32; ++c) dst[c] = E(0);
            dst[32] = v[i][0];
            if (row == wrow && row == k)
  #pragma unroll
              for (int c = 0; c < 33; ++c) sh.krow[c] = sh.cand[c];
          }
        }
        __syncthreads();
        // warp w pushes to CTAs w, w + nwarps, ...: the candidate, its word,
        // and (CTA 0) row k
        if (warp < nct) {
          E lo = E(0), hi = E(0);
          if (wrow >= 0) {
            lo = sh.cand[lane];
            hi = lane == 0 ? sh.cand[32] : (lane - 1 < kk ? Lsm[(lane - 1) * LD + (wrow - r0)] : E(0));
          }
          E klo = E(0), khi = E(0);
          if (rank == 0) {  // row k < nb <= R lies in CTA 0
            klo = sh.krow[lane];
            khi = lane == 0 ? sh.krow[32] : (lane - 1 < kk ? Lsm[(lane - 1) * LD + k] : E(0));
          }
          for (int d = warp; d < nct; d += nwarps) {
            const unsigned mb = remote_addr(&sh.mbar[b], d);
            st_async(remote_addr(&sh.slot[b][rank][lane], d), lo, mb);
            st_async(remote_addr(&sh.slot[b][rank][32 + lane], d), hi, mb);
            if (lane == 0) st_async(remote_addr(&sh.skey[b][rank], d), cbest, mb);
            if (kF64 && lane == 1) st_async(remote_addr(&sh.srow[b][rank], d), wrow, mb);
            if (rank == 0) {
              st_async(remote_addr(&sh.rowk[b][lane], d), klo, mb);
              st_async(remote_addr(&sh.rowk[b][32 + lane], d), khi, mb);
            }
          }
        }
        // this column's pushes from every CTA have landed; then the buffer is
        // armed for column k + kPcBuf
        tc::mbar_wait(&sh.mbar[b], (k / kPcBuf) & 1, &ctl->status);
        if (tid == 0) tc::mbar_expect_tx(&sh.mbar[b], xbytes);
        // the cluster's pivot, identical in every CTA
        int p;
        if constexpr (!kF64) {
          p = pc_row(warp_max64(lane < nct ? sh.skey[b][lane] : 0ull));
        } else {
          unsigned long long gk = lane < nct ? sh.skey[b][lane] : 0ull;
          int gr = lane < nct && gk != 0 ? sh.srow[b][lane] : 0x7fffffff;
          warp_lexmax(gk, gr);
          p = gr;
        }
        // a row outside [k, m) only after an exchange timed out (stale words):
        // row k stands in, so that the slot index and the swaps stay in range
        if (p < k || p >= m) p = k;
        const E *prow = sh.slot[b][p / R];
        const E piv = prow[32];
        const bool swap = piv != E(0) && p != k;
        if (tid == 0) {
          sh.piv[kk] = swap ? p : k;
          if (rank == 0) {
            ipiv[k] = p + 1 + ipiv_base;
            if (piv == E(0)) atomicCAS(&ctl->info, 0, k + 1 + info_base);
          }
        }
        if (swap) {  // the finished part of rows k and p, one warp each
          if (warp == nwarps - 2 && rank == 0 && lane < kk) Lsm[lane * LD + k] = prow[33 + lane];
          if (warp == nwarps - 1 && p / R == rank && lane < kk)
            Lsm[lane * LD + (p - r0)] = sh.rowk[b][33 + lane];
        }
        const bool recip = fabs(piv) >= Real<E>::sfmin();
        const E rp = E(1) / piv;
        const int live = ws - 1 - kk;  // columns right of kk still to update
  #pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T, lr = tid + i * T;
          if (swap && (row == k || row == p)) {
            const E *src = row == k ? prow : sh.rowk[b];
            v[i][0] = src[32];
  #pragma unroll
            for (int c = 1; c < W; ++c) v[i][c] = src[c - 1];
          }
          E x = v[i][0];
          const bool below = row > k && row < m;
          if (below && piv != E(0)) {
            if (recip) x *= rp;
            else x = x / piv;
          }
          Lsm[kk * LD + lr] = x;
          // rotate: column kk + 1 + c moves to register c; only the first
          // `live` positions carry data, the rest are zero.  Rows not below
          // the pivot move without arithmetic (an inf in the pivot row must
          // not reach them through 0 * inf).
          if (below) {
            if (live > W / 2) {
  #pragma unroll
              for (int j = 0; j < W / 4; ++j) {
                E q0, q1, q2, q3;
                load4(prow + 4 * j, q0, q1, q2, q3);
                v[i][4 * j + 0] = fmae(-x, q0, v[i][4 * j + 1]);
                v[i][4 * j + 1] = fmae(-x, q1, v[i][4 * j + 2]);
                v[i][4 * j + 2] = fmae(-x, q2, v[i][4 * j + 3]);
                if (4 * j + 4 < W) v[i][4 * j + 3] = fmae(-x, q3, v[i][4 * j + 4]);
              }
            } else {
  #pragma unroll
              for (int j = 0; j < W / 8; ++j) {
                E q0, q1, q2, q3;
                load4(prow + 4 * j, q0, q1, q2, q3);
                v[i][4 * j + 0] = fmae(-x, q0, v[i][4 * j + 1]);
                v[i][4 * j + 1] = fmae(-x, q1, v[i][4 * j + 2]);
                v[i][4 * j + 2] = fmae(-x, q2, v[i][4 * j + 3]);
                v[i][4 * j + 3] = fmae(-x, q3, v[i][4 * j + 4]);
              }
            }
          } else {
  #pragma unroll
            for (int c = 0; c + 1 < W; ++c) v[i][c] = v[i][c + 1];
          }
          if (live <= W / 2) {
  #pragma unroll
            for (int c = W / 2; c + 1 < W; ++c) v[i][c] = E(0);
          }
          v[i][W - 1] = E(0);
        }
      }
      __syncthreads();
    }

    // C. the factored sub-panel back to the panel; L21 into registers
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int row = r0 + tid + i * T, lr = tid + i * T;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        v[i][c] = c < ws ? Lsm[c * LD + lr] : E(0);
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
      constexpr int kEnt = 2 * W;  // entries per column
      const int kCpr = T / kEnt;   // columns per round
      const int no = nb - ws;                                // the other panel columns
      const int ntot = no + xl + xr;                         // and the extra ranges
      const int mine = ntot > rank ? (ntot - rank + nct - 1) / nct : 0;
      const int e = tid % kEnt;
      const int dst = sh.mdst[e], src = sh.msrc[e];
      auto column = [&](int jl) {
        const int j = rank + jl * nct;
        if (j < no) return A + (long)(j < c0 ? j : j + ws) * lda;
        if (j < no + xl) return XL + (long)(j - no) * lda;
        return XR + (long)(j - no - xl) * lda;
      };
      // up to kRounds rounds of columns gathered into registers behind one
      // barrier, then scattered (threads past kCpr whole columns sit out)
      constexpr int kRounds = 16;
      const bool part = tid < kCpr * kEnt && dst >= 0;
      for (int base = 0; base < mine; base += kRounds * kCpr) {
        E val[kRounds];
#pragma unroll
        for (int u = 0; u < kRounds; ++u) {
          const int jl = base + u * kCpr + tid / kEnt;
          val[u] = (part && jl < mine) ? __ldcg(column(jl) + src) : E(0);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kRounds; ++u) {
          const int jl = base + u * kCpr + tid / kEnt;
          if (part && jl < mine) column(jl)[dst] = val[u];
        }
      }
    }
    __threadfence();
    cl_sync();

    // G. U12 = L11^-1 A12 over the right columns, in every CTA
    const int nr = nb - c0 - ws;
    if (nr > 0) {
      // lanes over rows (contiguous), warps over columns, several loads in flight
      {
        E t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int c = warp + nwarps * u;
          t[u] = (lane < ws && c < ws) ? __ldcg(A + (c0 + lane) + (long)(c0 + c) * lda) : E(0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int c = warp + nwarps * u;
          if (lane < ws && c < ws) sh.L11[lane][c] = t[u];
        }
        for (int cb = 0; cb < nr; cb += 8 * nwarps) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int c = cb + warp + nwarps * u;
            t[u] = (lane < ws && c < nr) ? __ldcg(A + (c0 + lane) + (long)(c0 + ws + c) * lda)
                                         : E(0);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int c = cb + warp + nwarps * u;
            if (lane < ws && c < nr) sh.U[c][lane] = t[u];
          }
        }
      }
      __syncthreads();
      // every CTA holds its copy of A12 before CTA 0 overwrites those rows
      // with U12 below: without this barrier a CTA slowed by other work on
      // its SM could load rows already solved and solve them a second time
      cl_sync();
      if (tid < nr) {
        E u[W];
#pragma unroll
        for (int r = 0; r < W; ++r) u[r] = r < ws ? sh.U[tid][r] : E(0);
#pragma unroll
        for (int q = 0; q + 1 < W; ++q)
#pragma unroll
          for (int r = q + 1; r < W; ++r) u[r] = fmae(-sh.L11[r][q], u[q], u[r]);
#pragma unroll
        for (int r = 0; r < W; ++r) sh.U[tid][r] = r < ws ? u[r] : E(0);
      }
      __syncthreads();
      if (rank == 0)
        for (int e = tid; e < ws * nr; e += T) {
          const int r = e % ws, c = e / ws;
          A[(c0 + r) + (long)(c0 + ws + c) * lda] = sh.U[c][r];
        }
      // H. A22 -= L21 U12 on this CTA's rows below the sub-panel
      const int rs = c0 + ws;
      // four columns a step; the next step's loads are issued before this
      // step's arithmetic so their latency overlaps it
      E a[4][RPT], an[4][RPT];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const int row = r0 + tid + i * T;
          a[q][i] = (q < nr && row >= rs && row < m) ? __ldcg(A + row + (long)(rs + q) * lda) : E(0);
        }
      for (int cb = 0; cb < nr; cb += 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * T, col = cb + 4 + q;
            an[q][i] = (col < nr && row >= rs && row < m)
                           ? __ldcg(A + row + (long)(rs + col) * lda)
                           : E(0);
          }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const E *u = sh.U[min(cb + q, nr - 1)];
#pragma unroll
          for (int k4 = 0; k4 < W / 4; ++k4) {
            E u0, u1, u2, u3;
            load4(u + 4 * k4, u0, u1, u2, u3);
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
              a[q][i] = fmae(-v[i][4 * k4 + 0], u0, a[q][i]);
              a[q][i] = fmae(-v[i][4 * k4 + 1], u1, a[q][i]);
              a[q][i] = fmae(-v[i][4 * k4 + 2], u2, a[q][i]);
              a[q][i] = fmae(-v[i][4 * k4 + 3], u3, a[q][i]);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int row = r0 + tid + i * T;
            if (cb + q < nr && row >= rs && row < m) A[row + (long)(rs + cb + q) * lda] = a[q][i];
            a[q][i] = an[q][i];
          }
      }
    }
    __syncthreads();
  }
}

// Occupancy check of a kernel variant on its largest shape, once per device.
struct PcState {
  bool checked = false, ok = false;
};
std::mutex g_pc_mu;
std::map<std::pair<int, const void *>, PcState> g_pc_state;

template <typename E, int RPT, int W, bool TOURN>
int launch_pc(int m, int nb, E *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
              int info_base, cudaStream_t s, bool *launched, E *XL, int xl, E *XR, int xr) {
  // rows spread over up to 16 CTAs; a CTA holds at least nb rows (row k of
  // every column lies in CTA 0) and at most 512 RPT.  The tournament runs 512
  // threads, so that its final elimination has a thread for each of the
  // nct W candidates.
  int T = ceil_div(ceil_div(m, kPcMaxCta * RPT), 32) * 32;
  T = std::max(T, ceil_div(ceil_div(nb, RPT), 32) * 32);
  T = std::max(T, 128);
  if (TOURN) T = kPcThreads;
  if (T > kPcThreads) return 0;
  const int R = T * RPT, nct = ceil_div(m, R);
  if (nct > kPcMaxCta) return 0;
  // dynamic shared memory: the exchange state, then the finished columns
  // (for the tournament also the candidate exchange)
  auto smem_bytes = [](int rows, int ncta) {
    const long fin = (long)(rows + 1) * W;
    const long xch = TOURN ? (long)ncta * W * (W + 1) + (long)W * W : 0;
    return (size_t)pc_state_bytes<E>() + sizeof(E) * (size_t)std::max(fin, xch);
  };
  const size_t lsm = smem_bytes(R, nct);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = nct;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(nct);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = lsm;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // one check per variant and device on its largest shape: 16 CTAs of 512 threads
  auto *kern = panel_cluster_kernel<E, RPT, W, TOURN>;
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  const size_t lmax = smem_bytes(kPcThreads * RPT, kPcMaxCta);
  {
    std::lock_guard<std::mutex> lk(g_pc_mu);
    PcState &st = g_pc_state[{dev, (const void *)kern}];
    if (!st.checked) {
      st.checked = true;
      DeviceInfo di;
      ZG_TRY(device_info(&di));
      if (lmax > di.smem_optin) return 0;  // st.ok stays false
      ZG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      ZG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lmax));
      cudaLaunchConfig_t big = cfg;
      cudaLaunchAttribute bat[1] = {at[0]};
      bat[0].val.clusterDim.x = kPcMaxCta;
      big.gridDim = dim3(kPcMaxCta);
      big.blockDim = dim3(kPcThreads);
      big.dynamicSmemBytes = lmax;
      big.attrs = bat;
      int nclusters = 0;
      const cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, (void *)kern, &big);
      if (e != cudaSuccess) (void)cudaGetLastError();
      st.ok = e == cudaSuccess && nclusters >= 1;
    }
    if (!st.ok) return 0;
  }
  ZG_LAUNCH(kTagPanel, 1.0 * m * nb * nb, 2.0 * sizeof(E) * m * nb, s,
            ZG_CUDA(cudaLaunchKernelEx(&cfg, kern, m, nb, A, lda, ipiv, ipiv_base, ctl, info_base,
                                       XL, xl, XR, xr)));
  *launched = true;
  return 0;
}

template <int RPT, int W>
int launch_pc_any(bool tourn, int m, int nb, float *A, long lda, int *ipiv, int ipiv_base,
                  Control *ctl, int info_base, cudaStream_t s, bool *launched, float *XL, int xl,
                  float *XR, int xr) {
  if (tourn)
    return launch_pc<float, RPT, W, true>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                          launched, XL, xl, XR, xr);
  return launch_pc<float, RPT, W, false>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                         launched, XL, xl, XR, xr);
}

}  // namespace

int panel_lu_cluster(int m, int nb, float *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool *launched, float *XL, int xl, float *XR,
                     int xr, bool tournament) {
  *launched = false;
  if (m <= 0 || nb <= 0) {
    *launched = true;
    return 0;
  }
  if (nb > kPcMaxNb || m < nb || xl < 0 || xr < 0) return 0;
  if (m <= kPcMaxCta * kPcThreads)
    return launch_pc_any<1, 32>(tournament, m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                launched, XL, xl, XR, xr);
  if (m <= kPcMaxCta * kPcThreads * 2)
    return launch_pc_any<2, 32>(tournament, m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                launched, XL, xl, XR, xr);
  if (m <= kPcMaxCta * kPcThreads * 4)
    return launch_pc_any<4, 16>(tournament, m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                launched, XL, xl, XR, xr);
  return 0;
}

// The FP64 panel on one cluster: exact (key, row) pivot selection, 32-column
// sub-panels, one row a thread (the finished columns, 131 KB, fit beside the
// exchange state, about 80 KB).  Taller panels (more than 8192 rows) return
// unlaunched: with two or four rows a thread the finished columns allow only
// 16- or 8-column sub-panels, whose transitions made the panel slower than
// the cooperative one (n = 16384 FP64 LU: 207 against 130 ms of panels).
int panel_lu_cluster(int m, int nb, double *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool *launched, double *XL, int xl,
                     double *XR, int xr) {
  *launched = false;
  if (m <= 0 || nb <= 0) {
    *launched = true;
    return 0;
  }
  if (nb > kPcMaxNb || m < nb || xl < 0 || xr < 0) return 0;
  if (m <= kPcMaxCta * kPcThreads)
    return launch_pc<double, 1, 32, false>(m, nb, A, lda, ipiv, ipiv_base, ctl, info_base, s,
                                           launched, XL, xl, XR, xr);
  return 0;
}

}  // namespace zg
