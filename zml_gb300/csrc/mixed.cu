// mixed.cu -- mixed-precision LU / Cholesky with FP64 iterative refinement.
//
// Factorization ("the low-precision getrf"): the matrix is held in FP32; the
// blocked right-looking loop of lapack/getrf.zig:52-144 runs with NB = 256:
// each 256-wide panel is factored in FP32 (cooperative panel kernel on two
// 128-wide halves), the block row of U is solved in FP32, and the trailing
// update A22 -= L21 U12 runs on the tcgen05 tensor cores with L21 and U12
// rounded to BF16 (or FP16) and FP32 accumulation.
//
// Solve: plain iterative refinement (x += U^-1 L^-1 P r) or GMRES-IR
// (restarted GMRES on the left-preconditioned system (LU)^-1 A d = (LU)^-1 r).
// The residual r = b - A x, the update and the GMRES orthogonalisation are
// FP64; the preconditioner applies the FP32 factors with FP64 accumulation.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "kernels_mixed.h"
#include "kernels_selector.h"
#include "kernels_tc.h"

namespace zg {

// ---------------------------------------------------------------------------
// Conversions
template <typename H> __device__ __forceinline__ H to16(float v);
template <> __device__ __forceinline__ __nv_bfloat16 to16(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half to16(float v) { return __float2half_rn(v); }

// rows x k block of a column-major fp32 matrix -> row-major (K-major) 16-bit
// with row stride ldo (transpose through shared memory).  split: the row is
// written three times, [hi | hi | lo] with hi = bf16(v), lo = bf16(v - hi),
// each segment ldk wide (the A side of the three-product split GEMM).
template <typename H>
__global__ void to_kmajor_t_kernel(int rows, int k, const float *A, long lda, H *out, long ldo,
                                   int ldk, bool split, bool bside) {
  __shared__ float t[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int c = threadIdx.y; c < 32; c += 8) {
    int r = r0 + threadIdx.x, kk = k0 + c;
    t[c][threadIdx.x] = (r < rows && kk < k) ? __ldcg(A + r + (long)kk * lda) : 0.f;
  }
  __syncthreads();
  for (int c = threadIdx.y; c < 32; c += 8) {
    int r = r0 + c, kk = k0 + threadIdx.x;
    if (r >= rows || kk >= ldk) continue;
    const float v = kk < k ? t[threadIdx.x][c] : 0.f;
    const H hi = to16<H>(v);
    H *o = out + (long)r * ldo + kk;
    o[0] = hi;
    if (split) {  // A side [hi | hi | lo], B side [hi | lo | hi]
      const H lo = to16<H>(v - (float)hi);
      o[ldk] = bside ? lo : hi;
      o[2 * ldk] = bside ? hi : lo;
    }
  }
}

// k x cols block of a column-major fp32 matrix (k contiguous) -> 16-bit with
// column stride ldo (already K-major).  split: [hi | lo | hi] (the B side).
template <typename H>
__global__ void to_kmajor_n_kernel(int k, int cols, const float *A, long lda, H *out, long ldo,
                                   int ldk, bool split) {
  long total = (long)ldk * cols;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    int kk = e % ldk, c = e / ldk;
    const float v = kk < k ? __ldcg(A + kk + (long)c * lda) : 0.f;
    const H hi = to16<H>(v);
    H *o = out + (long)c * ldo + kk;
    o[0] = hi;
    if (split) {
      o[ldk] = to16<H>(v - (float)hi);
      o[2 * ldk] = hi;
    }
  }
}

static int grid1d(long total) { return (int)std::min<long>((total + 255) / 256, 152L * 16); }

// ldk: segment width (>= k, multiple of 8); the operand row stride is ldk,
// or 3 ldk for the split (bf16x3) form.
static int to_kmajor_t(int prec, int rows, int k, const float *A, long lda, void *out, int ldk,
                       cudaStream_t s, bool bside = false) {
  if (rows <= 0) return 0;
  const bool split = prec == kPrecBF16x3;
  const long ldo = split ? 3L * ldk : ldk;
  dim3 grid(ceil_div(rows, 32), ceil_div(ldk, 32)), blk(32, 8);
  if (prec == kPrecFP16)
    ZG_LAUNCH(kTagConvert, 0, 4.0 * rows * k + 2.0 * rows * ldo, s,
              to_kmajor_t_kernel<__half><<<grid, blk, 0, s>>>(rows, k, A, lda, (__half *)out, ldo,
                                                              ldk, false, false));
  else
    ZG_LAUNCH(kTagConvert, 0, 4.0 * rows * k + 2.0 * rows * ldo, s,
              to_kmajor_t_kernel<__nv_bfloat16><<<grid, blk, 0, s>>>(
                  rows, k, A, lda, (__nv_bfloat16 *)out, ldo, ldk, split, bside));
  return 0;
}

static int to_kmajor_n(int prec, int k, int cols, const float *A, long lda, void *out, int ldk,
                       cudaStream_t s) {
  if (cols <= 0) return 0;
  const bool split = prec == kPrecBF16x3;
  const long ldo = split ? 3L * ldk : ldk;
  const int g = grid1d((long)ldk * cols);
  if (prec == kPrecFP16)
    ZG_LAUNCH(kTagConvert, 0, 4.0 * cols * k + 2.0 * cols * ldo, s,
              to_kmajor_n_kernel<__half><<<g, 256, 0, s>>>(k, cols, A, lda, (__half *)out, ldo,
                                                           ldk, false));
  else
    ZG_LAUNCH(kTagConvert, 0, 4.0 * cols * k + 2.0 * cols * ldo, s,
              to_kmajor_n_kernel<__nv_bfloat16><<<g, 256, 0, s>>>(
                  k, cols, A, lda, (__nv_bfloat16 *)out, ldo, ldk, split));
  return 0;
}

// ---------------------------------------------------------------------------
// Block-row solves of the low-precision LU through explicit inverses of the
// unit-lower diagonal blocks: U12 = L11^-1 A12 as one FP32 GEMM instead of a
// chain of latency-bound substitutions.  (The FP64 LU keeps the TRSM of
// getrf.zig:104-114; here the factors only precondition the refinement.)

// X (nb x nb, ld ldx) <- L^-1 for the unit-lower nb x nb block L (ld ldl),
// nb <= 128.
constexpr int kInvN = 128, kInvLd = kInvN + 1;
// One column of the identity per warp (16 CTAs of 8 warps for nb = 128): lane l holds rows l, l + 32, l + 64, l + 96 of the column;
// step k broadcasts the solved x_k from its lane and every lane updates its
// rows below k.  L sits in shared memory with an odd stride, so the lanes'
// reads of one column hit distinct banks.
constexpr int kInvColsPerCta = 8;
__global__ void __launch_bounds__(32 * kInvColsPerCta)
    inv_unit_lower_cols_kernel(int nb, const float *__restrict__ L, long ldl, float *X, long ldx) {
  extern __shared__ float sLc[];  // sLc[i * kInvLd + k] = L(i, k)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int j0 = blockIdx.x * kInvColsPerCta;
  // columns j0 .. nb-1 below the diagonal are all this CTA's columns touch;
  // thread = (row t & 127, column phase t >> 7), column-contiguous loads with
  // eight in flight a thread
  {
    const int i = tid & 127, cp = tid >> 7;
    for (int k0 = j0 + cp; k0 < nb; k0 += 16) {
      float t[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + 2 * u;
        t[u] = (k < nb && i > k && i < nb) ? __ldcg(L + i + (long)k * ldl) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + 2 * u;
        if (k < nb && i < nb) sLc[i * kInvLd + k] = t[u];
      }
    }
  }
  __syncthreads();
  const int j = j0 + warp;
  if (j >= nb) return;
  float x[kInvN / 32];
#pragma unroll
  for (int q = 0; q < kInvN / 32; ++q) x[q] = (lane + 32 * q == j) ? 1.f : 0.f;
  for (int k = j; k < nb - 1; ++k) {
    const int kq = k >> 5;  // static register choice: no local-memory indexing
    const float xs = kq == 0 ? x[0] : kq == 1 ? x[1] : kq == 2 ? x[2] : x[3];
    const float xk = __shfl_sync(~0u, xs, k & 31);
#pragma unroll
    for (int q = 0; q < kInvN / 32; ++q) {
      const int i = lane + 32 * q;
      if (i > k && i < nb) x[q] = fmaf(-sLc[i * kInvLd + k], xk, x[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < kInvN / 32; ++q) {
    const int i = lane + 32 * q;
    if (i < nb) X[i + (long)j * ldx] = i < j ? 0.f : x[q];
  }
}

static int inv_unit_lower(int nb, const float *L, long ldl, float *X, long ldx, cudaStream_t s) {
  if (nb <= 0) return 0;
  const int smem = kInvN * kInvLd * sizeof(float);
  ZG_TRY(smem_optin(inv_unit_lower_cols_kernel, smem));
  ZG_LAUNCH(kTagTrsmDiag, nb * (double)nb * nb / 3.0, 0, s,
            inv_unit_lower_cols_kernel<<<ceil_div(nb, kInvColsPerCta), 32 * kInvColsPerCta, smem,
                                         s>>>(nb, L, ldl, X, ldx));
  return 0;
}

// C = alpha A B + beta C for small NN products (one thread per element of C,
// the K loop in registers): the 128 x 128 x 128 block products of the mixed
// LU, too small to fill the GPU with 64 x 64 tiles.
__global__ void gemm_small_kernel(int m, int n, int k, float alpha, const float *__restrict__ A,
                                  long lda, const float *__restrict__ B, long ldb, float beta,
                                  float *__restrict__ C, long ldc) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= m || j >= n) return;
  float a0 = 0.f, a1 = 0.f;
  int q = 0;
  for (; q + 1 < k; q += 2) {
    a0 = fmaf(__ldcg(A + i + (long)q * lda), __ldcg(B + q + (long)j * ldb), a0);
    a1 = fmaf(__ldcg(A + i + (long)(q + 1) * lda), __ldcg(B + q + 1 + (long)j * ldb), a1);
  }
  if (q < k) a0 = fmaf(__ldcg(A + i + (long)q * lda), __ldcg(B + q + (long)j * ldb), a0);
  const float v = alpha * (a0 + a1);
  C[i + (long)j * ldc] = beta == 0.f ? v : v + beta * __ldcg(C + i + (long)j * ldc);
}

// C (m x n) = alpha A B + beta C for m, k <= 128: one CTA per 32 columns of
// C loads all of A (column-major, padded) and its k x 32 slice of B into
// shared memory, then every thread forms a 4 x 4 register tile (rows lane +
// 32 u, columns warp + 8 v).  The slice of B is read completely before any
// of C is written, so C may be B itself (beta = 0).
constexpr int kG128 = 128;
__global__ void __launch_bounds__(256) gemm128_kernel(int m, int n, int k, float alpha,
                                                      const float *A, long lda, const float *B,
                                                      long ldb, float beta, float *C, long ldc) {
  extern __shared__ float g128[];
  float *sA = g128;                      // sA[q * (kG128 + 1) + r] = A(r, q)
  float *sB = g128 + kG128 * (kG128 + 1);  // sB[q * 33 + c] = B(q, j0 + c)
  const int j0 = blockIdx.x * 32, nc = min(32, n - j0);
  // thread = (row t & 127, column phase t >> 7): column-contiguous loads, eight
  // independent loads in flight a thread
  const int lr = threadIdx.x & 127, cp = threadIdx.x >> 7;
  for (int q0 = cp; q0 < k; q0 += 16) {
    float t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + 2 * u;
      t[u] = (lr < m && q < k) ? __ldcg(A + lr + (long)q * lda) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + 2 * u;
      if (q < k) sA[q * (kG128 + 1) + lr] = t[u];
    }
  }
  {
    float t[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int c = cp + 2 * u;
      t[u] = (lr < k && c < nc) ? __ldcg(B + lr + (long)(j0 + c) * ldb) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) sB[lr * 33 + cp + 2 * u] = t[u];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float acc[4][4] = {};
  for (int q = 0; q < k; ++q) {
    float a[4], bv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = sA[q * (kG128 + 1) + lane + 32 * u];
#pragma unroll
    for (int v = 0; v < 4; ++v) bv[v] = sB[q * 33 + warp + 8 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], bv[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = lane + 32 * u, c = warp + 8 * v;
      if (r < m && c < nc) {
        float *cp = C + r + (long)(j0 + c) * ldc;
        *cp = beta != 0.f ? fmaf(alpha, acc[u][v], beta * __ldcg(cp)) : alpha * acc[u][v];
      }
    }
}

static int gemm_small(int m, int n, int k, float alpha, const float *A, long lda, const float *B,
                      long ldb, float beta, float *C, long ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  if (m <= kG128 && k <= kG128) {
    const int smem = sizeof(float) * (kG128 * (kG128 + 1) + kG128 * 33);
    ZG_TRY(smem_optin(gemm128_kernel, smem));
    ZG_LAUNCH(kTagGemmSimt, 2.0 * m * n * k, 4.0 * ((double)m * k + (double)k * n + 2.0 * m * n),
              s, gemm128_kernel<<<ceil_div(n, 32), 256, smem, s>>>(m, n, k, alpha, A, lda, B, ldb,
                                                                  beta, C, ldc));
    return 0;
  }
  ZG_LAUNCH(kTagGemmSimt, 2.0 * m * n * k, 4.0 * ((double)m * k + (double)k * n + 2.0 * m * n), s,
            gemm_small_kernel<<<dim3(ceil_div(m, 32), ceil_div(n, 8)), 256, 0, s>>>(
                m, n, k, alpha, A, lda, B, ldb, beta, C, ldc));
  return 0;
}

// B (k x cols, ld ldb) <- Linv B with Linv (k x k, ld ldi): in place for
// k <= 128, otherwise through a scratch copy T (k x cols, ld k).
static int apply_inverse(int k, int cols, const float *Linv, long ldi, float *B, long ldb, float *T,
                         cudaStream_t s) {
  if (k <= 0 || cols <= 0) return 0;
  if (k <= kG128) return gemm_small(k, cols, k, 1.f, Linv, ldi, B, ldb, 0.f, B, ldb, s);  // in place
  if (cols <= 256)
    ZG_TRY(gemm_small(k, cols, k, 1.f, Linv, ldi, B, ldb, 0.f, T, k, s));
  else
    ZG_TRY(gemm_simt<float>(kNoTrans, kNoTrans, k, cols, k, 1.f, Linv, ldi, B, ldb, 0.f, T, k, 0,
                            s));
  ZG_CUDA(cudaMemcpy2DAsync(B, sizeof(float) * ldb, T, sizeof(float) * k, sizeof(float) * k, cols,
                            cudaMemcpyDeviceToDevice, s));
  return 0;
}

// ---------------------------------------------------------------------------
// Low-precision LU of an n x n FP32 matrix (partial pivoting, ipiv 1-based).
//
// Lookahead: a 256-column block's trailing update is split into the next
// block's columns (on the panel stream, at high priority) and the rest (on
// a low-priority bulk stream), so the bulk of the update runs beside the
// next block's panel, which holds 16 SMs for most of its time.  Events keep
// the order: block b's panel waits for the bulk update of block b-2 (the
// last one to touch its columns), block b's full-width interchanges for
// that of block b-1.  The 16-bit operand buffers alternate by block parity.

namespace {
// A factored while it arrives from pinned host memory: its columns come in
// chunks on a copy stream, each chunk is converted to FP32 on its own stream
// and there receives, in order, the updates of the blocks factored before
// it joins the main loop (replayed from their saved 16-bit operands); from
// its join block on, the main loop updates it like any other column.
struct ChunkStreams {
  static constexpr int kMax = 8;
  cudaStream_t copy = nullptr, ck[kMax] = {};
  cudaEvent_t copied[kMax] = {}, caught[kMax] = {}, copy_end = nullptr;
  std::vector<cudaEvent_t> ops;  // block b's saved operands and pivots are final
};
std::mutex g_cs_mu;
std::map<std::pair<int, cudaStream_t>, ChunkStreams> g_cs;

int chunk_streams(cudaStream_t s, int nblocks, ChunkStreams **out) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cs_mu);
  ChunkStreams &c = g_cs[{dev, s}];
  const unsigned fl = cudaEventDisableTiming;
  if (!c.copy) {
    int least = 0, greatest = 0;
    ZG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    ZG_CUDA(cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking));
    ZG_CUDA(cudaEventCreateWithFlags(&c.copy_end, fl));
    for (int q = 0; q < ChunkStreams::kMax; ++q) {
      ZG_CUDA(cudaStreamCreateWithPriority(&c.ck[q], cudaStreamNonBlocking, least));
      ZG_CUDA(cudaEventCreateWithFlags(&c.copied[q], fl));
      ZG_CUDA(cudaEventCreateWithFlags(&c.caught[q], fl));
    }
  }
  while ((int)c.ops.size() < nblocks) {
    cudaEvent_t e;
    ZG_CUDA(cudaEventCreateWithFlags(&e, fl));
    c.ops.push_back(e);
  }
  *out = &c;
  return 0;
}

// The geometry of one streamed factorization (BF16x3 updates, NB = 256).
struct ChunkPlan {
  int nck = 0;                         // chunk count
  int c0[ChunkStreams::kMax + 1] = {}; // chunk c: columns c0[c] .. c0[c+1]-1 (512-multiples)
  int wmax = 0;                        // widest chunk
  int join[ChunkStreams::kMax] = {};   // block before whose interchanges chunk c joins
  int bmax = 0;                        // blocks 0 .. bmax-1 keep their operands for replays
  uint16_t *savedL = nullptr;          // their L21 operands, one after the other
  uint16_t *savedLi = nullptr;         // their L11^-1 operands, NB x ldo each
  std::vector<size_t> offL;            // element offset of block b's L21 operand in savedL
  ChunkStreams *cs = nullptr;
};

// Block b's update of chunk c on the chunk's stream, as the main loop makes
// it on joined columns: the block's interchanges, U12 = L11^-1 A12 on the
// tensor cores, then A22 -= L21 U12.  The arithmetic per element is the
// main loop's (same operands, same K order), so the factors do not depend
// on when a chunk arrived.
static int replay_block(const ChunkPlan &cp, int c, int b, int n, float *A, long lda,
                        const int *ipiv, unsigned *status) {
  constexpr int NB = 256, ldk = NB;
  constexpr long ldo = 3L * ldk;
  const int j = b * NB, c0 = cp.c0[c], wc = cp.c0[c + 1] - c0;
  const cudaStream_t st = cp.cs->ck[c];
  ZG_CUDA(cudaStreamWaitEvent(st, cp.cs->ops[b], 0));
  float *Ac = A + (long)c0 * lda;
  ZG_TRY(laswp_dev<float>(wc, Ac, lda, j + 1, j + NB, ipiv, 1, st));
  void *wu;
  ZG_TRY(workspace(st, kSlotU16, sizeof(uint16_t) * (size_t)wc * ldo, &wu));
  ZG_TRY(to_kmajor_n(kPrecBF16x3, NB, wc, Ac + j, lda, wu, ldk, st));
  ZG_TRY(gemm_tc(NB, wc, (int)ldo, 1.f, cp.savedLi + (size_t)b * NB * ldo, ldo, wu, ldo, 0.f,
                 Ac + j, lda, 1, status, st));
  ZG_TRY(to_kmajor_n(kPrecBF16x3, NB, wc, Ac + j, lda, wu, ldk, st));
  ZG_TRY(gemm_tc(n - j - NB, wc, (int)ldo, -1.f, cp.savedL + cp.offL[b], ldo, wu, ldo, 1.f,
                 Ac + j + NB, lda, 1, status, st));
  return 0;
}
}  // namespace

static int getrf_lowp_blocks(int n, float *A, long lda, int *ipiv, int prec, Control *ctl,
                             cudaStream_t s, Lookahead &la, ChunkPlan *cp = nullptr);

// Pivoting of the low-precision LU's panels.  The factors only precondition
// the refinement, so they need not carry partial pivoting's exact pivots:
// tournament pivoting needs one cluster exchange per 32-column sub-panel
// instead of one per column, but its two CTA-wide elimination rounds per
// column measured slower on GB300 (n = 16384: 72.9 against 41.0 ms of panels
// a solve), so partial pivoting is the default.
static std::atomic<int> g_tournament{0};

int set_mixed_tournament(int on) { return g_tournament.exchange(on != 0 ? 1 : 0); }

int getrf_lowp(int n, float *A, long lda, int *ipiv, int prec, Control *ctl, cudaStream_t s) {
  if (n <= 0) return 0;
  if (prec == kPrecFP32) {
    int info = 0;
    return getrf_dev<float>(n, n, A, lda, ipiv, &info, s, g_tournament.load() != 0) < 0
               ? kErrCuda
               : 0;
  }
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  // both internal streams start after the caller's earlier work and the
  // caller's stream resumes after both
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = getrf_lowp_blocks(n, A, lda, ipiv, prec, ctl, s, *la);
  ZG_CUDA(cudaEventRecord(la->end_panel, la->panel));
  ZG_CUDA(cudaEventRecord(la->end_bulk, la->bulk));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_panel, 0));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_bulk, 0));
  return rc;
}

static int getrf_lowp_blocks(int n, float *A, long lda, int *ipiv, int prec, Control *ctl,
                             cudaStream_t s, Lookahead &la, ChunkPlan *cp) {
  constexpr int NB = 256, NBP = 128;
  const int segs = prec == kPrecBF16x3 ? 3 : 1;
  const size_t nop = (size_t)n * NB * segs;  // 16-bit elements of one operand buffer
  void *wl0, *wu0, *wi;
  ZG_TRY(workspace(s, kSlotL16, sizeof(uint16_t) * 2 * nop, &wl0));
  ZG_TRY(workspace(s, kSlotU16, sizeof(uint16_t) * 2 * nop, &wu0));
  // L11^-1 (NB x NB), a temporary NBP x NBP block, and the block row's scratch
  const size_t ntb = prec == kPrecBF16x3 ? (size_t)NBP * NBP : (size_t)NB * n;
  ZG_TRY(workspace(s, kSlotInvL,
                   sizeof(float) * ((size_t)NB * NB + NBP * NBP + ntb) +
                       sizeof(uint16_t) * (size_t)NB * NB * segs + 256,
                   &wi));
  // L11^-1, a product scratch, the block row's scratch, L11^-1 as a 16-bit operand
  float *Linv = (float *)wi, *Ttmp = Linv + NB * NB, *Tb = Ttmp + NBP * NBP;
  void *wli = Tb + ntb;
  const cudaStream_t sp = la.panel, sb = la.bulk;
  constexpr int R = Lookahead::kRing;
  // columns the main loop updates: all n, or the chunks joined so far
  int lim = n, joined = 0;
  if (cp) {
    lim = 0;
    ZG_CUDA(cudaStreamWaitEvent(sp, cp->cs->caught[0], 0));  // block 0's panel reads chunk 0
  }
  for (int j = 0, b = 0; j < n; j += NB, ++b) {
    const int jb = std::min(NB, n - j);
    const bool keep = cp && b < cp->bmax;  // a later chunk replays this block
    uint16_t *wl = keep ? cp->savedL + cp->offL[b] : (uint16_t *)wl0 + (b & 1) * nop;
    uint16_t *wu = (uint16_t *)wu0 + (b & 1) * nop;
    // this block's columns were last updated by block b-2's bulk update
    if (b >= 2) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 2) % R], 0));
    ZG_CUDA(cudaMemsetAsync(Linv, 0, sizeof(float) * NB * NB, sp));
    // panel: two FP32 half-panels (one cluster each) with an update between
    for (int p = 0; p < jb; p += NBP) {
      const int r = j + p, pb = std::min(NBP, jb - p);
      const int right = j + jb - r - pb;
      // the half-panel, its interchanges applied inside the block's other columns
      bool done = false;
      ZG_TRY(panel_lu_cluster(n - r, pb, A + r + (long)r * lda, lda, ipiv + r, r, ctl, r, sp,
                              &done, A + r + (long)j * lda, r - j, A + r + (long)(r + pb) * lda,
                              right, g_tournament.load() != 0));
      if (!done) {
        ZG_TRY(panel_lu<float>(n - r, pb, A + r + (long)r * lda, lda, ipiv + r, r, ctl, r, sp));
        ZG_TRY(laswp_panel<float>(r - j, r + pb - j, jb, A + (long)j * lda, lda, r + 1, r + pb,
                                  ipiv, sp));
      }
      // the half-panel's unit-lower diagonal block, inverted into L11^-1
      float *Dinv = Linv + p + (long)p * NB;
      ZG_TRY(inv_unit_lower(pb, A + r + (long)r * lda, lda, Dinv, NB, sp));
      if (right > 0) {
        float *Ar = A + (long)(r + pb) * lda;
        ZG_TRY(apply_inverse(pb, right, Dinv, NB, Ar + r, lda, Tb, sp));
        const int rows = n - r - pb;
        if (prec == kPrecBF16x3 && rows > 0) {
          // the second half-panel's update in the block's update precision
          const int ldk = ((pb + 7) / 8) * 8;
          const long ldo = (long)ldk * segs;
          ZG_TRY(to_kmajor_t(prec, rows, pb, A + (r + pb) + (long)r * lda, lda, wl, ldk, sp));
          ZG_TRY(to_kmajor_n(prec, pb, right, Ar + r, lda, wu, ldk, sp));
          ZG_TRY(gemm_tc(rows, right, (int)ldo, -1.f, wl, ldo, wu, ldo, 1.f, Ar + r + pb, lda, 1,
                         &ctl->status, sp));
        } else {
          ZG_TRY(gemm_simt<float>(kNoTrans, kNoTrans, rows, right, pb, -1.f,
                                  A + (r + pb) + (long)r * lda, lda, Ar + r, lda, 1.f,
                                  Ar + r + pb, lda, 0, sp));
        }
      }
    }
    if (jb > NBP) {
      // L11^-1 = [La^-1 0; -Lb^-1 Lc La^-1  Lb^-1]
      const int pb2 = jb - NBP;
      ZG_TRY(gemm_small(pb2, NBP, NBP, 1.f, A + (j + NBP) + (long)j * lda, lda, Linv, NB, 0.f,
                        Ttmp, NBP, sp));
      ZG_TRY(gemm_small(pb2, NBP, pb2, -1.f, Linv + NBP + (long)NBP * NB, NB, Ttmp, NBP, 0.f,
                        Linv + NBP, NB, sp));
    }
    // the interchanges reach every other column: wait for block b-1's bulk update
    if (b >= 1) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 1) % R], 0));
    // chunks due now join, caught up through block b-1
    while (cp && joined < cp->nck && cp->join[joined] <= b) {
      ZG_CUDA(cudaStreamWaitEvent(sp, cp->cs->caught[joined], 0));
      lim = cp->c0[joined + 1];
      ++joined;
    }
    ZG_TRY(laswp_panel<float>(j, j + jb, lim, A, lda, j + 1, j + jb, ipiv, sp));
    const int rest = n - j - jb;   // rows below the block
    if (rest <= 0) break;
    const int rc = lim - j - jb;   // columns right of the block that the main loop updates
    float *A12 = A + j + (long)(j + jb) * lda;
    // U12 = L11^-1 A12.  BF16x3 (about 16 bits, the precision of its trailing
    // updates): on the tensor cores, A12 read through its 16-bit copy and U12
    // written over A12 in FP32.  Plain BF16 / FP16 would cut U's rows to 8 /
    // 11 bits, so there the product is an FP32 GEMM.
    const int ldk = ((jb + 7) / 8) * 8;
    const long ldo = (long)ldk * segs;
    void *wlib = keep ? (void *)(cp->savedLi + (size_t)b * NB * ldo) : wli;
    if (prec == kPrecBF16x3) {
      ZG_TRY(to_kmajor_t(prec, jb, jb, Linv, NB, wlib, ldk, sp));
      ZG_TRY(to_kmajor_n(prec, jb, rc, A12, lda, wu, ldk, sp));
      ZG_TRY(gemm_tc(jb, rc, (int)ldo, 1.f, wlib, ldo, wu, ldo, 0.f, A12, lda, 1, &ctl->status,
                     sp));
    } else {
      ZG_TRY(apply_inverse(jb, rc, Linv, NB, A12, lda, Tb, sp));
    }
    // 16-bit operands: L21 (rest x jb) and U12^T (rc x jb), K-major
    ZG_TRY(to_kmajor_t(prec, rest, jb, A + (j + jb) + (long)j * lda, lda, wl, ldk, sp));
    if (keep) {  // the chunks not yet joined replay this block on their own streams
      ZG_CUDA(cudaEventRecord(cp->cs->ops[b], sp));
      for (int c = joined; c < cp->nck; ++c) {
        ZG_TRY(replay_block(*cp, c, b, n, A, lda, ipiv, &ctl->status));
        if (cp->join[c] == b + 1) ZG_CUDA(cudaEventRecord(cp->cs->caught[c], cp->cs->ck[c]));
      }
    }
    ZG_TRY(to_kmajor_n(prec, jb, rc, A12, lda, wu, ldk, sp));
    const int abt = prec == kPrecFP16 ? 0 : 1;  // 16-bit operand type: FP16 0, BF16 1
    // the next block's columns now, on the panel stream ...
    const int near = std::min(NB, rc);
    ZG_TRY(gemm_tc(rest, near, (int)ldo, -1.f, wl, ldo, wu, ldo, 1.f, A12 + jb, lda, abt,
                   &ctl->status, sp));
    // ... the rest on the bulk stream, beside the next block's panel
    if (rc > near) {
      ZG_CUDA(cudaEventRecord(la.upd[b % R], sp));
      ZG_CUDA(cudaStreamWaitEvent(sb, la.upd[b % R], 0));
      ZG_TRY(gemm_tc(rest, rc - near, (int)ldo, -1.f, wl, ldo, wu + (long)near * ldo, ldo, 1.f,
                     A12 + jb + (long)near * lda, lda, abt, &ctl->status, sb));
    }
    ZG_CUDA(cudaEventRecord(la.bulk_done[b % R], sb));
  }
  return 0;
}
// Low-precision Cholesky (lower) of an n x n SPD FP32 matrix: FP32 64-wide
// diagonal blocks, FP32 block-column TRSM, trailing SYRK on the tensor cores
// (lower 128 x 128 tiles only), NB = 256.  The first non-positive pivot lands
// in ctl->info.  Lookahead as in getrf_lowp: the next block's columns (its
// diagonal tiles and the rows below them) on the panel stream, the rest of
// the SYRK on the bulk stream.  Block b's diagonal block waits for block b-2's
// bulk update, the last to touch its columns; block b's near update for block
// b-1's, which updates the same columns; the 16-bit operand buffers alternate
// by block parity.  The tiles computed and every tile's arithmetic are those
// of one SYRK over the whole trailing matrix.
static int potrf_lowp_blocks(int n, float *A, long lda, int prec, Control *ctl, cudaStream_t s,
                             Lookahead &la) {
  constexpr int NB = 256;
  constexpr int R = Lookahead::kRing;
  const cudaStream_t sp = la.panel, sb = la.bulk;
  const int segs = prec == kPrecBF16x3 ? 3 : 1;
  const size_t nop = (size_t)n * NB * segs;
  void *wl0, *wu0;
  ZG_TRY(workspace(s, kSlotL16, sizeof(uint16_t) * 2 * nop, &wl0));
  ZG_TRY(workspace(s, kSlotU16, sizeof(uint16_t) * 2 * nop, &wu0));
  const int abt = prec == kPrecFP16 ? 0 : 1;
  for (int j = 0, b = 0; j < n; j += NB, ++b) {
    const int jb = std::min(NB, n - j);
    float *Ajj = A + j + (long)j * lda;
    uint16_t *wl = (uint16_t *)wl0 + (b & 1) * nop, *wu = (uint16_t *)wu0 + (b & 1) * nop;
    if (b >= 2) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 2) % R], 0));
    ZG_TRY(potrf_launch<float>(kLower, jb, Ajj, lda, ctl, j, sp));
    const int rest = n - j - jb;
    if (rest > 0) {
      float *A21 = Ajj + jb;
      ZG_TRY(trsm_dev<float>(kRight, kLower, kTrans, kNonUnit, rest, jb, 1.f, Ajj, lda, A21, lda,
                             sp));
      const int ldk = ((jb + 7) / 8) * 8;
      ZG_TRY(to_kmajor_t(prec, rest, jb, A21, lda, wl, ldk, sp, false));
      ZG_TRY(to_kmajor_t(prec, rest, jb, A21, lda, wu, ldk, sp, true));
      const long ldo = (long)ldk * segs;
      // the next block's columns now, once block b-1's bulk update is done ...
      if (b >= 1) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 1) % R], 0));
      const int near = std::min(NB, rest);
      float *C = A21 + (long)jb * lda;  // the trailing matrix
      ZG_TRY(gemm_tc(near, near, (int)ldo, -1.f, wl, ldo, wu, ldo, 1.f, C, lda, abt,
                     &ctl->status, sp, /*tri=*/1));
      if (rest > near) {
        ZG_TRY(gemm_tc(rest - near, near, (int)ldo, -1.f, wl + (long)near * ldo, ldo, wu, ldo,
                       1.f, C + near, lda, abt, &ctl->status, sp));
        // ... the rest on the bulk stream, beside the next block's diagonal
        // block and triangular solve
        ZG_CUDA(cudaEventRecord(la.upd[b % R], sp));
        ZG_CUDA(cudaStreamWaitEvent(sb, la.upd[b % R], 0));
        ZG_TRY(gemm_tc(rest - near, rest - near, (int)ldo, -1.f, wl + (long)near * ldo, ldo,
                       wu + (long)near * ldo, ldo, 1.f, C + near + (long)near * lda, lda, abt,
                       &ctl->status, sb, /*tri=*/1));
      }
    }
    ZG_CUDA(cudaEventRecord(la.bulk_done[b % R], sb));
  }
  return 0;
}

int potrf_lowp(int n, float *A, long lda, int prec, Control *ctl, cudaStream_t s) {
  if (n <= 0) return 0;
  if (prec == kPrecFP32) return potrf_launch<float>(kLower, n, A, lda, ctl, 0, s);
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = potrf_lowp_blocks(n, A, lda, prec, ctl, s, *la);
  ZG_CUDA(cudaEventRecord(la->end_panel, la->panel));
  ZG_CUDA(cudaEventRecord(la->end_bulk, la->bulk));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_panel, 0));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_bulk, 0));
  return rc;
}

// The strict lower triangle mirrored into the upper one (A(j,i) = A(i,j)),
// through shared-memory tiles.
template <typename T>
__global__ void mirror_lower_kernel(int n, T *A, long lda) {
  __shared__ T t[32][33];
  const int bi = blockIdx.x, bj = blockIdx.y;  // source tile (rows bi, cols bj), bi >= bj
  if (bi < bj) return;
  const int i0 = bi * 32, j0 = bj * 32;
  for (int c = threadIdx.y; c < 32; c += 8) {
    const int i = i0 + threadIdx.x, j = j0 + c;
    t[c][threadIdx.x] = (i < n && j < n) ? A[i + (long)j * lda] : T(0);
  }
  __syncthreads();
  for (int c = threadIdx.y; c < 32; c += 8) {
    const int i = j0 + threadIdx.x, j = i0 + c;  // destination (i, j) = source (j, i)
    if (i < n && j < n && j > i) A[i + (long)j * lda] = t[threadIdx.x][c];
  }
}

template <typename T> int mirror_lower(int n, T *A, long lda, cudaStream_t s) {
  dim3 grid(ceil_div(n, 32), ceil_div(n, 32)), blk(32, 8);
  ZG_LAUNCH(kTagConvert, 0, 1.0 * sizeof(T) * n * n, s,
            mirror_lower_kernel<T><<<grid, blk, 0, s>>>(n, A, lda));
  return 0;
}

// Full symmetric FP64 copy (ld n) of the `uplo` triangle of A.
__global__ void sym_full_kernel(int n, const double *A, long lda, bool lower, double *S) {
  const long total = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % n, j = e / n;
    const bool in = lower ? i >= j : i <= j;
    S[e] = in ? A[i + (long)j * lda] : A[j + (long)i * lda];
  }
}

// ---------------------------------------------------------------------------
// FP64 residual r = b - A x (column-major A), deterministic two-pass GEMV.
constexpr int kGemvRows = 256, kGemvCols = 512;

__global__ void gemv_partial_kernel(int n, int ncols, const double *__restrict__ A, long lda,
                                    const double *__restrict__ x, double *__restrict__ part) {
  const int i = blockIdx.x * kGemvRows + threadIdx.x;
  const int c0 = blockIdx.y * kGemvCols, c1 = min(ncols, c0 + kGemvCols);
  __shared__ double xs[kGemvCols];
  for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) xs[c - c0] = x[c];
  __syncthreads();
  if (i >= n) return;
  double acc0 = 0, acc1 = 0;
  const double *a = A + i + (long)c0 * lda;
  int c = c0;
  // unrolled so that several columns' loads are in flight per thread (the
  // two accumulators keep their summation order)
#pragma unroll 8
  for (; c + 1 < c1; c += 2, a += 2 * lda) {
    acc0 = fma(a[0], xs[c - c0], acc0);
    acc1 = fma(a[lda], xs[c + 1 - c0], acc1);
  }
  if (c < c1) acc0 = fma(a[0], xs[c - c0], acc0);
  part[(long)blockIdx.y * n + i] = acc0 + acc1;
}

__global__ void gemv_finish_kernel(int n, int nparts, const double *part, const double *b,
                                   double *r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0;
  for (int p = 0; p < nparts; ++p) acc += part[(long)p * n + i];
  r[i] = b ? b[i] - acc : acc;
}

// y = A x  (b == nullptr)  or  y = b - A x
int gemv_d(int n, const double *A, long lda, const double *x, const double *b, double *y,
           double *part, cudaStream_t s) {
  const int nparts = ceil_div(n, kGemvCols);
  dim3 grid(ceil_div(n, kGemvRows), nparts);
  ZG_LAUNCH(kTagGemv, 2.0 * n * n, 8.0 * n * n + 8.0 * n * (nparts + 1), s, gemv_partial_kernel<<<grid, kGemvRows, 0, s>>>(n, n, A, lda, x, part));
  ZG_LAUNCH(kTagGemv, 0, 0, s, gemv_finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, nparts, part, b, y));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Triangular solves with the FP32 factors, FP64 vectors ("sync-free").
//
// The factor is cut into 128-row blocks.  One CTA per block row claims its
// block in dependency order through a ticket, streams its off-diagonal tiles
// L(blk, cb) (the load of the next tile is issued before waiting for the
// current one's x, so the HBM stream overlaps the dependency chain),
// accumulates L(blk, cb) x(cb) in FP64 as earlier blocks publish, and then
// applies the FP64 inverse of its diagonal block (precomputed once per
// factorization) and publishes x(blk).  lower = unit lower L (forward),
// upper = non-unit upper U (backward).
//
// Publication needs no flag and no fence: x(blk) is written to a separate
// buffer that starts filled with an all-ones word (a NaN no arithmetic
// produces; a computed NaN is published in canonical form), and a consumer
// polls the 8-byte words themselves, so the value arrives with the first
// load that sees it.
constexpr int kTB = 128;          // block rows
constexpr int kTT = 512;          // threads: 128 rows x 4 column phases
constexpr int kTC = kTB / 4;      // columns per phase and tile

__device__ __forceinline__ void trsv_load_tile(float (&v)[kTC], const float *A, long lda, int row,
                                               bool row_ok, int c0, int ph, int n) {
#pragma unroll
  for (int j = 0; j < kTC; ++j) {
    const int c = c0 + ph + 4 * j;
    v[j] = (row_ok && c < n) ? __ldcs(A + row + (long)c * lda) : 0.f;
  }
}

// F = float: every product FP32 (GB300's FP64 rate is a small fraction of
// FP32; right for well-conditioned factors), tile sums accumulated as a
// compensated FP32 pair.  F = double: products, sums and the diagonal
// inverse in FP64, for ill-conditioned factors where an FP32 triangular
// solve would not apply (LU)^-1.  x stays FP64.
constexpr unsigned long long kTrsvEmpty = ~0ull;  // an unpublished x word

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const double *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

template <typename F>
__global__ void __launch_bounds__(kTT) trsv_lowp_kernel(int n, const float *__restrict__ A, long lda,
                                                        const F *__restrict__ Dinv, double *x,
                                                        double *xpub, unsigned *ticket,
                                                        bool upper, unsigned *status) {
  extern __shared__ __align__(16) unsigned char tsv_raw[];
  F *DiS = reinterpret_cast<F *>(tsv_raw);  // this block's diagonal inverse, column-major
  __shared__ unsigned sb;
  __shared__ double part[4][kTB];
  __shared__ float partf[2][4][kTB];
  __shared__ F xs2[2][kTB];
  __shared__ F ys[kTB];
  const int tid = threadIdx.x;
  if (tid == 0) sb = atomicAdd(ticket, 1u);
  __syncthreads();
  const int nblk = (n + kTB - 1) / kTB;
  const int t = sb;
  const int blk = upper ? nblk - 1 - t : t;
  const int r0 = blk * kTB, rows = min(kTB, n - r0);
  const int lr = tid % kTB, ph = tid / kTB;
  const int row = r0 + lr;
  const bool row_ok = lr < rows;
  // fetched up front: the diagonal inverse and this block's right-hand side
  {
    const float4 *src = reinterpret_cast<const float4 *>(Dinv + (long)blk * kTB * kTB);
    float4 *dst = reinterpret_cast<float4 *>(DiS);
    const int words = kTB * kTB * (int)sizeof(F) / 16;
    for (int e = tid; e < words; e += kTT) dst[e] = __ldcs(src + e);
  }
  const double rhs = (ph == 0 && row_ok) ? x[row] : 0.0;
  // FP32 forms: the running sum of tile products is an unevaluated pair
  // (ah + al, TwoSum), as accurate as an FP64 accumulator for this length
  // without touching the FP64 pipe; FP64 forms accumulate in FP64
  double acc = 0;
  float ah = 0.f, al = 0.f;
  // tiles in the order they become ready; A tiles prefetched two ahead and
  // the next tile's x fetched while the current one is multiplied
  auto tile_col = [&](int q) { return (upper ? nblk - 1 - q : q) * kTB; };
  auto fetch_x = [&](int q, F *dst) {
    if (tid < kTB) {
      const int c = tile_col(q) + tid;
      F xv = F(0);
      if (c < n) {
        unsigned long long w = ld_relaxed_u64(xpub + c);
        long long spins = 0;
        const long long lim = spin_limit();
        while (w == kTrsvEmpty) {
          if (++spins > lim) {
            atomicOr(status, kStatusQueueTimeout);
            break;
          }
          if (spins > 64) __nanosleep(32);
          w = ld_relaxed_u64(xpub + c);
        }
        xv = (F)__longlong_as_double((long long)w);
      }
      dst[tid] = xv;
    }
  };
  float cur[kTC], nxt[kTC], nn[kTC];
  if (t > 0) {
    trsv_load_tile(cur, A, lda, row, row_ok, tile_col(0), ph, n);
    if (t > 1) trsv_load_tile(nxt, A, lda, row, row_ok, tile_col(1), ph, n);
    fetch_x(0, xs2[0]);
  }
  __syncthreads();
  for (int q = 0; q < t; ++q) {
    if (q + 2 < t) trsv_load_tile(nn, A, lda, row, row_ok, tile_col(q + 2), ph, n);
    if (q + 1 < t) fetch_x(q + 1, xs2[(q + 1) & 1]);
    const F *xq = xs2[q & 1];
    F p0 = 0, p1 = 0;
#pragma unroll
    for (int j = 0; j < kTC; j += 2) {
      p0 = fma((F)cur[j], xq[ph + 4 * j], p0);
      p1 = fma((F)cur[j + 1], xq[ph + 4 * (j + 1)], p1);
    }
    if constexpr (sizeof(F) == sizeof(float)) {
      const float pt = p0 + p1, sum = ah + pt, bv = sum - ah;
      al += (ah - (sum - bv)) + (pt - bv);
      ah = sum;
    } else {
      acc += (double)p0 + (double)p1;
    }
    // x of tile q + 1 visible; xs2[q & 1] free for tile q + 2
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kTC; ++j) {
      cur[j] = nxt[j];
      nxt[j] = nn[j];
    }
  }
  if constexpr (sizeof(F) == sizeof(float)) {
    partf[0][ph][lr] = ah;
    partf[1][ph][lr] = al;
  } else {
    part[ph][lr] = acc;
  }
  __syncthreads();
  if (tid < kTB) {
    double sum;
    if constexpr (sizeof(F) == sizeof(float)) {
      float sh_ = partf[0][0][tid], sl = partf[1][0][tid];
#pragma unroll
      for (int q = 1; q < 4; ++q) {
        const float h = partf[0][q][tid], t2 = sh_ + h, bv = t2 - sh_;
        sl += (sh_ - (t2 - bv)) + (h - bv) + partf[1][q][tid];
        sh_ = t2;
      }
      sum = (double)sh_ + (double)sl;
    } else {
      sum = part[0][tid] + part[1][tid] + part[2][tid] + part[3][tid];
    }
    ys[tid] = row_ok ? (F)(rhs - sum) : F(0);
  }
  __syncthreads();
  // x(blk) = inv(D) * rhs
  F y0 = 0, y1 = 0;
#pragma unroll 8
  for (int j = ph; j < kTB; j += 8) {
    y0 = fma(DiS[lr + j * kTB], ys[j], y0);
    y1 = fma(DiS[lr + (j + 4) * kTB], ys[j + 4], y1);
  }
  if constexpr (sizeof(F) == sizeof(float))
    partf[0][ph][lr] = y0 + y1;
  else
    part[ph][lr] = (double)y0 + (double)y1;
  __syncthreads();
  if (tid < kTB && row_ok) {
    double xv;
    if constexpr (sizeof(F) == sizeof(float))
      xv = (double)((partf[0][0][tid] + partf[0][1][tid]) + (partf[0][2][tid] + partf[0][3][tid]));
    else
      xv = part[0][tid] + part[1][tid] + part[2][tid] + part[3][tid];
    x[row] = xv;
    xpub[row] = xv != xv ? __longlong_as_double(0x7ff8000000000000ll) : xv;
  }
}

// FP64 inverses of the kTB x kTB diagonal blocks of the FP32 LU factors:
// inv(L_bb) (unit lower) into Linv, inv(U_bb) into Uinv, each column-major
// kTB x kTB per block (zero outside the triangle).  In-place triangular
// inversion in shared memory, one CTA per block.
__global__ void __launch_bounds__(512) invert_diag_kernel(int n, const float *__restrict__ A,
                                                          long lda, double *Linv, double *Uinv,
                                                          float *Linv32, float *Uinv32,
                                                          bool lower_unit) {
  extern __shared__ double T[];  // T[i + j * kTB]
  const int blk = blockIdx.x, upper = blockIdx.y;
  const int r0 = blk * kTB, rows = min(kTB, n - r0);
  const int tid = threadIdx.x;
  for (int e = tid; e < kTB * kTB; e += blockDim.x) {
    const int i = e % kTB, j = e / kTB;
    double v = 0;
    if (i < rows && j < rows) {
      if (upper) v = i <= j ? (double)A[(r0 + i) + (long)(r0 + j) * lda] : 0.0;
      else if (lower_unit) v = i > j ? (double)A[(r0 + i) + (long)(r0 + j) * lda] : (i == j ? 1.0 : 0.0);
      else v = i >= j ? (double)A[(r0 + i) + (long)(r0 + j) * lda] : 0.0;
    } else if (i == j) {
      v = 1.0;  // padding rows of the last block: identity
    }
    T[e] = v;
  }
  __syncthreads();
  if (upper) {
    // columns left to right: T(j,j) = 1/U(j,j); T(0:j, j) = -T(j,j) T(0:j,0:j) U(0:j, j)
    for (int j = 0; j < kTB; ++j) {
      const double djj = 1.0 / T[j + j * kTB];
      double v = 0;
      if (tid < j) {
        for (int k = tid; k < j; ++k) v = fma(T[tid + k * kTB], T[k + j * kTB], v);
      }
      __syncthreads();
      if (tid < j) T[tid + j * kTB] = -djj * v;
      if (tid == j) T[j + j * kTB] = djj;
      __syncthreads();
    }
  } else {
    // columns right to left: T(j+1:, j) = -T(j+1:, j+1:) L(j+1:, j) / L(j, j),
    // T(j, j) = 1 / L(j, j) (1 for the unit lower factor of LU)
    for (int j = kTB - 1; j >= 0; --j) {
      const double djj = lower_unit ? 1.0 : 1.0 / T[j + j * kTB];
      double v = 0;
      const int i = j + 1 + tid;
      if (i < kTB) {
        for (int k = j + 1; k <= i; ++k) v = fma(T[i + k * kTB], T[k + j * kTB], v);
      }
      __syncthreads();
      if (i < kTB) T[i + j * kTB] = -v * djj;
      if (tid == 0) T[j + j * kTB] = djj;
      __syncthreads();
    }
  }
  double *out = (upper ? Uinv : Linv) + (long)blk * kTB * kTB;
  float *out32 = (upper ? Uinv32 : Linv32) + (long)blk * kTB * kTB;
  for (int e = tid; e < kTB * kTB; e += blockDim.x) {
    out[e] = T[e];
    out32[e] = (float)T[e];
  }
}

int invert_diag_blocks(int n, const float *A, long lda, double *Linv, double *Uinv, float *Linv32,
                       float *Uinv32, bool lower_unit, cudaStream_t s) {
  const int nblk = ceil_div(n, kTB);
  const size_t smem = sizeof(double) * kTB * kTB;
  ZG_TRY(smem_optin(invert_diag_kernel, (int)smem));
  ZG_LAUNCH(kTagTrsv, 2.0 * nblk * kTB * kTB * kTB / 3, 8.0 * nblk * kTB * kTB * 3, s,
            invert_diag_kernel<<<dim3(nblk, 2), 512, smem, s>>>(n, A, lda, Linv, Uinv, Linv32,
                                                                Uinv32, lower_unit));
  return 0;
}

// x <- op^-1 x with op = unit-lower L (upper=false) or non-unit upper U of
// the FP32 LU factors in A, Dinv their diagonal-block inverses (FP32 or
// FP64: the arithmetic of the solve).  work: 8-byte aligned, trsv_work_bytes(n).
size_t trsv_work_bytes(int n) { return sizeof(double) * ((size_t)n + 1); }

template <typename F>
int trsv_lowp(int n, const float *A, long lda, const F *Dinv, double *x, bool upper,
              unsigned *work, unsigned *status, cudaStream_t s) {
  if (n <= 0) return 0;
  const int nblk = ceil_div(n, kTB);
  double *xpub = reinterpret_cast<double *>(work) + 1;
  ZG_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned), s));
  ZG_CUDA(cudaMemsetAsync(xpub, 0xff, sizeof(double) * n, s));
  const size_t smem = sizeof(F) * kTB * kTB;
  ZG_TRY(smem_optin(trsv_lowp_kernel<F>, (int)smem));
  ZG_LAUNCH(kTagTrsv, 1.0 * n * n, 2.0 * n * n + 16.0 * n + sizeof(F) * nblk * kTB * kTB, s,
            trsv_lowp_kernel<F><<<nblk, kTT, smem, s>>>(n, A, lda, Dinv, x, xpub, work, upper,
                                                        status));
  return 0;
}

// d[i] = r[perm[i]]: the row interchanges of getrf as one gather (perm is the
// composition of the ipiv swaps, built once per factorization).
__global__ void gather_kernel(int n, const double *r, const int *perm, double *d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = r[perm[i]];
}

int perm_from_ipiv(int n, const int *ipiv_dev, int *perm_dev, cudaStream_t s) {
  std::vector<int> ip(n), pm(n);
  ZG_CUDA(cudaMemcpyAsync(ip.data(), ipiv_dev, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  ZG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) pm[i] = i;
  for (int i = 0; i < n; ++i) {
    const int p = ip[i] - 1;
    if (p >= 0 && p < n && p != i) std::swap(pm[i], pm[p]);
  }
  ZG_CUDA(cudaMemcpyAsync(perm_dev, pm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  ZG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// d = (LU)^-1 P r applied in FP64 with the FP32 factors.
struct LowLU {
  const float *LU;
  long lda;
  const int *perm;
  const double *Linv, *Uinv;      // FP64 diagonal-block inverses
  const float *Linv32, *Uinv32;   // their FP32 roundings
  bool f64 = false;               // apply in FP64 arithmetic
};

int lu_apply(int n, const LowLU &f, const double *r, double *d, unsigned *work, unsigned *status,
             cudaStream_t s) {
  const float *LU = f.LU;
  const long lda = f.lda;
  const int *perm = f.perm;
  ZG_LAUNCH(kTagVector, 0, 0, s, gather_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, r, perm, d));
  ZG_CUDA(cudaGetLastError());
  if (f.f64) {
    ZG_TRY(trsv_lowp<double>(n, LU, lda, f.Linv, d, false, work, status, s));
    ZG_TRY(trsv_lowp<double>(n, LU, lda, f.Uinv, d, true, work, status, s));
  } else {
    ZG_TRY(trsv_lowp<float>(n, LU, lda, f.Linv32, d, false, work, status, s));
    ZG_TRY(trsv_lowp<float>(n, LU, lda, f.Uinv32, d, true, work, status, s));
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Small FP64 vector kernels (single block reductions are enough at n <= 64k).
__global__ void absmax_kernel(int n, const double *x, double *out) {
  __shared__ double sm[256];
  double m = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[i]));
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

// One pass over the FP64 matrix: B = fp32(A), and the row sums of |A| for
// ||A||_inf, as FP32 partial sums over 512-column chunks (positive terms, at
// most 512 a chunk: relative error below 1e-4, ample for a norm that only
// scales the backward error) that a second kernel adds in FP64.  n rows;
// ncols columns (all n, or one column chunk starting on a 512-column group).
__global__ void __launch_bounds__(kGemvRows) d2s_rowabs_kernel(int n, int ncols, const double *A,
                                                                long lda, float *B, long ldb,
                                                                float *part) {
  const int i = blockIdx.x * kGemvRows + threadIdx.x;
  const int c0 = blockIdx.y * kGemvCols, c1 = min(ncols, c0 + kGemvCols);
  if (i >= n) return;
  float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
  int j = c0;
  for (; j + 3 < c1; j += 4) {
    const double a0 = A[i + (long)j * lda], a1 = A[i + (long)(j + 1) * lda];
    const double a2 = A[i + (long)(j + 2) * lda], a3 = A[i + (long)(j + 3) * lda];
    const float f0 = (float)a0, f1 = (float)a1, f2 = (float)a2, f3 = (float)a3;
    B[i + (long)j * ldb] = f0;
    B[i + (long)(j + 1) * ldb] = f1;
    B[i + (long)(j + 2) * ldb] = f2;
    B[i + (long)(j + 3) * ldb] = f3;
    acc0 += fabsf(f0);
    acc1 += fabsf(f1);
    acc2 += fabsf(f2);
    acc3 += fabsf(f3);
  }
  for (; j < c1; ++j) {
    const float f = (float)A[i + (long)j * lda];
    B[i + (long)j * ldb] = f;
    acc0 += fabsf(f);
  }
  part[(long)blockIdx.y * n + i] = (acc0 + acc1) + (acc2 + acc3);
}

// Row sums of |A| over 512-column chunks in FP64 (the FP64 solve's norm);
// gemv_finish_kernel adds the chunks.
__global__ void __launch_bounds__(kGemvRows) rowabs_partial_kernel(int n, const double *A, long lda,
                                                                    double *part) {
  const int i = blockIdx.x * kGemvRows + threadIdx.x;
  const int c0 = blockIdx.y * kGemvCols, c1 = min(n, c0 + kGemvCols);
  if (i >= n) return;
  double acc0 = 0, acc1 = 0;
  int j = c0;
  for (; j + 1 < c1; j += 2) {
    acc0 += fabs(A[i + (long)j * lda]);
    acc1 += fabs(A[i + (long)(j + 1) * lda]);
  }
  if (j < c1) acc0 += fabs(A[i + (long)j * lda]);
  part[(long)blockIdx.y * n + i] = acc0 + acc1;
}

__global__ void rowabs_finish_kernel(int n, int nparts, const float *part, double *rs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0;
  for (int p = 0; p < nparts; ++p) acc += (double)part[(long)p * n + i];
  rs[i] = acc;
}

__global__ void axpy_kernel(int n, double a, const double *x, double *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

// h[j] = V(:, j) . w for j < k   (V column-major, ldv)
__global__ void gs_dots_kernel(int n, int k, const double *V, long ldv, const double *w,
                               double *h) {
  __shared__ double sm[256];
  const int j = blockIdx.x;
  double acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc = fma(V[i + (long)j * ldv], w[i], acc);
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) h[j] = sm[0];
}

// w -= V(:, 0:k) h ; out <- optional copy
__global__ void gs_update_kernel(int n, int k, const double *V, long ldv, const double *h,
                                 double *w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = w[i];
  for (int j = 0; j < k; ++j) acc -= V[i + (long)j * ldv] * h[j];
  w[i] = acc;
}

__global__ void nrm2_kernel(int n, const double *x, double *out) {
  __shared__ double sm[256];
  double acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc = fma(x[i], x[i], acc);
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sqrt(sm[0]);
}

__global__ void scale_copy_kernel(int n, double a, const double *x, double *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}

// x += V(:, 0:k) y
__global__ void combine_kernel(int n, int k, const double *V, long ldv, const double *y,
                               double *x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0;
  for (int j = 0; j < k; ++j) acc = fma(V[i + (long)j * ldv], y[j], acc);
  x[i] += acc;
}

// ---------------------------------------------------------------------------
struct IRWork {
  double *r, *d, *part, *scal, *V, *w, *h;
  unsigned *tw;
};

static int host_scalar(const double *d, double *h, cudaStream_t s) {
  ZG_CUDA(cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, s));
  ZG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// Normwise backward error of x for A x = b: ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
static int berr_of(int n, const double *A, long lda, const double *b, const double *x, double anrm,
                   double bnrm, IRWork &w, double *berr, cudaStream_t s) {
  ZG_TRY(gemv_d(n, A, lda, x, b, w.r, w.part, s));
  ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, w.r, w.scal));
  ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, x, w.scal + 1));
  ZG_CUDA(cudaGetLastError());
  double h[2];
  ZG_CUDA(cudaMemcpyAsync(h, w.scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  ZG_CUDA(cudaStreamSynchronize(s));
  const double den = anrm * h[1] + bnrm;
  *berr = den > 0 ? h[0] / den : h[0];
  return 0;
}

// GMRES on (LU)^-1 A d = (LU)^-1 r with restart m; returns after `inner`
// iterations or when the preconditioned residual fell by `rtol`.
constexpr int kGmresStallSteps = 16;

static int gmres_correction(int n, const double *A, long lda, const LowLU &f, IRWork &w, int m,
                            double rtol, int *iters, Control *ctl, cudaStream_t s) {
  const int b1 = ceil_div(n, 256);
  double *V = w.V;  // n x (m+1)
  // z = M^-1 r ; beta = ||z|| ; v0 = z / beta
  ZG_TRY(lu_apply(n, f, w.r, w.w, w.tw, &ctl->status, s));
  ZG_LAUNCH(kTagVector, 0, 0, s, nrm2_kernel<<<1, 256, 0, s>>>(n, w.w, w.scal));
  double beta;
  ZG_TRY(host_scalar(w.scal, &beta, s));
  ZG_CUDA(cudaMemsetAsync(w.d, 0, sizeof(double) * n, s));
  if (!(beta > 0) || !std::isfinite(beta)) return 0;
  ZG_LAUNCH(kTagVector, 0, 0, s, scale_copy_kernel<<<b1, 256, 0, s>>>(n, 1.0 / beta, w.w, V));
  std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
  g[0] = beta;
  int k = 0;
  std::vector<double> hcol(m + 1);
  for (; k < m; ++k) {
    // w = M^-1 A v_k
    ZG_TRY(gemv_d(n, A, lda, V + (long)k * n, nullptr, w.d, w.part, s));
    ZG_TRY(lu_apply(n, f, w.d, w.w, w.tw, &ctl->status, s));
    // classical Gram-Schmidt, twice
    ZG_CUDA(cudaMemsetAsync(w.h, 0, sizeof(double) * 2 * (m + 1), s));
    for (int pass = 0; pass < 2; ++pass) {
      ZG_LAUNCH(kTagVector, 0, 0, s, gs_dots_kernel<<<k + 1, 256, 0, s>>>(n, k + 1, V, n, w.w, w.h + pass * (m + 1)));
      ZG_LAUNCH(kTagVector, 0, 0, s, gs_update_kernel<<<b1, 256, 0, s>>>(n, k + 1, V, n, w.h + pass * (m + 1), w.w));
    }
    ZG_LAUNCH(kTagVector, 0, 0, s, nrm2_kernel<<<1, 256, 0, s>>>(n, w.w, w.scal));
    ZG_CUDA(cudaGetLastError());
    std::vector<double> hh(2 * (m + 1));
    ZG_CUDA(cudaMemcpyAsync(hh.data(), w.h, sizeof(double) * 2 * (m + 1), cudaMemcpyDeviceToHost, s));
    double hk1;
    ZG_CUDA(cudaMemcpyAsync(&hk1, w.scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    ZG_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i <= k; ++i) hcol[i] = hh[i] + hh[(m + 1) + i];
    hcol[k + 1] = hk1;
    if (hk1 > 0 && k + 1 <= m)
      ZG_LAUNCH(kTagVector, 0, 0, s, scale_copy_kernel<<<b1, 256, 0, s>>>(n, 1.0 / hk1, w.w, V + (long)(k + 1) * n));
    // Givens rotations on the new Hessenberg column
    for (int i = 0; i < k; ++i) {
      const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
      hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
      hcol[i] = t;
    }
    const double rho = std::hypot(hcol[k], hcol[k + 1]);
    cs[k] = rho > 0 ? hcol[k] / rho : 1.0;
    sn[k] = rho > 0 ? hcol[k + 1] / rho : 0.0;
    hcol[k] = rho;
    hcol[k + 1] = 0;
    g[k + 1] = -sn[k] * g[k];
    g[k] = cs[k] * g[k];
    for (int i = 0; i <= k; ++i) H[i + k * (m + 1)] = hcol[i];
    ++*iters;
    if (std::fabs(g[k + 1]) <= rtol * beta || !(hk1 > 0)) {
      ++k;
      break;
    }
    // a cycle whose first 16 steps fell short of the geometric rate that
    // reaches rtol within the restart (|g| / beta <= rtol^(16 / m)) is stuck
    // on a spread of small eigenvalues (factors too far from A for its
    // conditioning) that would take O(n) more steps: it ends here, its partial
    // correction is applied, and refinement decides early -- another cycle if
    // the backward error halved, else a different arithmetic or the FP64
    // factorization
    if (k + 1 == kGmresStallSteps && m > kGmresStallSteps &&
        std::fabs(g[k + 1]) > std::pow(rtol, (double)kGmresStallSteps / m) * beta) {
      ++k;
      break;
    }
  }
  // back substitution H y = g, d = V y
  std::vector<double> y(k, 0.0);
  for (int i = k - 1; i >= 0; --i) {
    double t = g[i];
    for (int j = i + 1; j < k; ++j) t -= H[i + j * (m + 1)] * y[j];
    y[i] = H[i + i * (m + 1)] != 0 ? t / H[i + i * (m + 1)] : 0.0;
  }
  ZG_CUDA(cudaMemcpyAsync(w.h, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
  ZG_CUDA(cudaMemsetAsync(w.d, 0, sizeof(double) * n, s));
  ZG_LAUNCH(kTagVector, 0, 0, s, combine_kernel<<<b1, 256, 0, s>>>(n, k, V, n, w.h, w.d));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// State of one low-precision factorization, shared by the refinement calls
// that use it (the workspace slots stay valid until the next factorization on
// the stream).
struct MpirCtx {
  int n = 0, m = 1;
  const double *A = nullptr;  // FP64 matrix of the residuals (full, column-major)
  long lda = 0;
  double anrm = 0;            // ||A||_inf
  Control *ctl = nullptr;
  LowLU f{};
  IRWork w{};
};

// The queued part of getrf_lowp_host: the chunk copies, the conversions and
// the factorization with its replays (the caller joins every stream after it).
static int chunked_factor(int n, const double *Ah, long ldh, double *Ad, float *LU, int *ipiv,
                          float *rpart, Control *ctl, cudaStream_t s, Lookahead &la,
                          ChunkPlan &cp) {
  ChunkStreams *cs = cp.cs;
  for (int c = 0; c < cp.nck; ++c) {
    const long c0 = cp.c0[c];
    const int wc = cp.c0[c + 1] - cp.c0[c];
    ZG_CUDA(cudaMemcpy2DAsync(Ad + c0 * n, sizeof(double) * n, Ah + c0 * ldh,
                              sizeof(double) * ldh, sizeof(double) * n, wc,
                              cudaMemcpyHostToDevice, cs->copy));
    ZG_CUDA(cudaEventRecord(cs->copied[c], cs->copy));
  }
  for (int c = 0; c < cp.nck; ++c) {
    const long c0 = cp.c0[c];
    const int wc = cp.c0[c + 1] - cp.c0[c];
    const cudaStream_t st = cs->ck[c];
    ZG_CUDA(cudaStreamWaitEvent(st, cs->copied[c], 0));
    ZG_LAUNCH(kTagConvert, 0, 12.0 * n * wc, st,
              d2s_rowabs_kernel<<<dim3(ceil_div(n, kGemvRows), ceil_div(wc, kGemvCols)),
                                  kGemvRows, 0, st>>>(n, wc, Ad + c0 * n, n, LU + c0 * n, n,
                                                      rpart + (c0 / kGemvCols) * n));
    if (cp.join[c] == 0) ZG_CUDA(cudaEventRecord(cs->caught[c], st));
  }
  return getrf_lowp_blocks(n, LU, n, ipiv, kPrecBF16x3, ctl, s, la, &cp);
}

// BF16x3 LU of an n x n A that arrives from pinned host memory (column-major,
// ld ldh): its FP64 copy lands in Ad (ld n) and its FP32 copy in LU (ld n),
// with the row sums of |A| as 512-column partials in rpart, chunk by chunk,
// while the factorization runs on the chunks already there.  The factors
// equal those of getrf_lowp on the whole FP32 copy.
static int getrf_lowp_host(int n, const double *Ah, long ldh, double *Ad, float *LU, int *ipiv,
                           float *rpart, Control *ctl, cudaStream_t s) {
  constexpr int NB = 256;
  constexpr long ldo = 3L * NB;
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  ChunkStreams *cs;
  ZG_TRY(chunk_streams(s, ceil_div(n, NB), &cs));
  ChunkPlan cp;
  cp.cs = cs;
  // a 512-column first chunk (the first panel waits only for it), the rest
  // in equal chunks of whole 512-column groups
  const int rest = ceil_div(ceil_div(n - kGemvCols, ChunkStreams::kMax - 1), kGemvCols) *
                   kGemvCols;
  cp.c0[0] = 0;
  cp.c0[1] = kGemvCols;
  cp.nck = 1;
  while (cp.c0[cp.nck] < n) {
    cp.c0[cp.nck + 1] = std::min(n, cp.c0[cp.nck] + rest);
    ++cp.nck;
  }
  // a chunk joins at the first block of the chunk before it, so its replays
  // run beside the factorization of that chunk
  for (int c = 0; c < cp.nck; ++c) {
    cp.join[c] = c == 0 ? 0 : cp.c0[c - 1] / NB;
    cp.wmax = std::max(cp.wmax, cp.c0[c + 1] - cp.c0[c]);
  }
  cp.bmax = cp.join[cp.nck - 1];
  cp.offL.resize(cp.bmax + 1);
  size_t tot = 0;
  for (int b = 0; b < cp.bmax; ++b) {
    cp.offL[b] = tot;
    tot += (size_t)(n - (b + 1) * NB) * ldo;
  }
  void *w;
  ZG_TRY(workspace(s, kSlotChunk, sizeof(uint16_t) * (tot + (size_t)cp.bmax * NB * ldo), &w));
  cp.savedL = (uint16_t *)w;
  cp.savedLi = cp.savedL + tot;
  // the chunk streams' buffers, sized before anything is queued: no
  // allocation (nor its synchronisation) between the queued copies
  for (int c = 0; c < cp.nck; ++c) {
    void *t;
    ZG_TRY(workspace(cs->ck[c], kSlotU16, sizeof(uint16_t) * (size_t)cp.wmax * ldo, &t));
    ZG_TRY(laswp_reserve(cs->ck[c]));
  }
  // everything after the caller's earlier work, which may still read Ad, LU
  // or rpart
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(cs->copy, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = chunked_factor(n, Ah, ldh, Ad, LU, ipiv, rpart, ctl, s, *la, cp);
  // the caller's stream resumes after every internal stream, also after a
  // failure part way (no copy from the caller's buffer may outlive the call)
  int jrc = 0;
  auto join = [&](cudaEvent_t e, cudaStream_t from) {
    if (cudaEventRecord(e, from) != cudaSuccess || cudaStreamWaitEvent(s, e, 0) != cudaSuccess)
      jrc = kErrCuda;
  };
  join(cs->copy_end, cs->copy);
  join(la->end_panel, la->panel);
  join(la->end_bulk, la->bulk);
  for (int c = 0; c < cp.nck; ++c) join(cs->caught[c], cs->ck[c]);
  if (jrc != 0) set_last_error("getrf_lowp_host: joining the internal streams failed");
  return rc != 0 ? rc : jrc;
}

bool mixed_streams_host(int n, const MpirOpts &o) {
  return n >= kChunkMinN && o.prec == kPrecBF16x3;
}

// Factor phase.  spd: A symmetric positive definite, only its `lower` (else
// upper) triangle is read; factored by the low-precision Cholesky.
// Otherwise general, LU.  res->info receives the factorization's info.
// Ah (general A, BF16x3, n >= kChunkMinN only): A is copied from this pinned
// host matrix (ld ldh) into A (ld n) during the factorization.
static int mpir_factor(bool spd, bool lower, int n, const double *A, long lda, const MpirOpts &o,
                       MpirCtx *c, MpirResult *res, cudaStream_t s, const double *Ah = nullptr,
                       long ldh = 0) {
  *res = MpirResult{};
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  if (spd) {  // the refinement works on the full symmetric FP64 matrix
    void *ws;
    ZG_TRY(workspace(s, kSlotSym, sizeof(double) * (size_t)n * n, &ws));
    ZG_LAUNCH(kTagConvert, 0, 16.0 * n * n, s,
              sym_full_kernel<<<grid1d((long)n * n), 256, 0, s>>>(n, A, lda, lower, (double *)ws));
    A = (const double *)ws;
    lda = n;
  }
  const int m = std::max(1, std::min(o.gmres_restart, 200));
  // workspace: FP32 factor copy, ipiv, perm and FP64 vectors
  void *wf, *wv;
  const size_t nf = (size_t)n * n;
  const size_t ninv = (size_t)ceil_div(n, kTB) * kTB * kTB;
  ZG_TRY(workspace(s, kSlotLowLU,
                   sizeof(float) * nf + 3 * sizeof(double) * ninv + 2 * sizeof(int) * (size_t)n + 512,
                   &wf));
  float *LU = (float *)wf;
  double *Linv = (double *)(((uintptr_t)(LU + nf) + 255) & ~(uintptr_t)255);
  double *Uinv = Linv + ninv;
  float *Linv32 = (float *)(Uinv + ninv);
  float *Uinv32 = Linv32 + ninv;
  int *ipiv = (int *)(Uinv32 + ninv);
  int *perm = ipiv + n;
  LowLU f{LU, (long)n, perm, Linv, Uinv, Linv32, Uinv32, o.apply == kApplyF64};
  const int nparts = ceil_div(n, kGemvCols);
  const size_t nv = (size_t)n * (4 + nparts + (m + 1)) + 4 * (m + 2) + 64;
  ZG_TRY(workspace(s, kSlotIRVec, sizeof(double) * nv + trsv_work_bytes(n), &wv));
  IRWork w;
  double *p = (double *)wv;
  w.r = p; p += n;
  w.d = p; p += n;
  w.w = p; p += n;
  w.part = p; p += (size_t)n * nparts;
  w.V = p; p += (size_t)n * (m + 1);
  w.h = p; p += 2 * (m + 2);
  w.scal = p; p += 8;
  w.tw = (unsigned *)p;

  // the FP32 working copy of A and ||A||_inf, in one pass over A
  float *rpart = reinterpret_cast<float *>(w.part);  // n x nparts floats fit in w.part
  double anrm = 0;
  if (!Ah) {
    ZG_LAUNCH(kTagConvert, 0, 12.0 * n * n, s,
              d2s_rowabs_kernel<<<dim3(ceil_div(n, kGemvRows), nparts), kGemvRows, 0, s>>>(
                  n, n, A, lda, LU, n, rpart));
    ZG_LAUNCH(kTagVector, 0, 0, s,
              rowabs_finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, nparts, rpart, w.r));
    ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, w.r, w.scal));
    ZG_CUDA(cudaGetLastError());
    ZG_TRY(host_scalar(w.scal, &anrm, s));
  }

  // factor in low precision (with A's arrival, for a host A)
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  if (Ah)
    ZG_TRY(getrf_lowp_host(n, Ah, ldh, const_cast<double *>(A), LU, ipiv, rpart, ctl, s));
  else if (spd)
    ZG_TRY(potrf_lowp(n, LU, n, o.prec, ctl, s));
  else
    ZG_TRY(getrf_lowp(n, LU, n, ipiv, o.prec, ctl, s));
  cudaEventRecord(e1, s);
  if (Ah) {
    ZG_LAUNCH(kTagVector, 0, 0, s,
              rowabs_finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, nparts, rpart, w.r));
    ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, w.r, w.scal));
    ZG_CUDA(cudaGetLastError());
  }
  int info = 0;
  ZG_TRY(check_status(s, ctl, &info));
  if (Ah) ZG_TRY(host_scalar(w.scal, &anrm, s));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  res->factor_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  res->info = info;
  if (info != 0) return 0;
  if (spd) {
    // U = L^T into the free upper triangle; no interchanges
    ZG_TRY(mirror_lower<float>(n, LU, n, s));
    std::vector<int> id(n);
    for (int i = 0; i < n; ++i) id[i] = i;
    ZG_CUDA(cudaMemcpyAsync(perm, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    ZG_CUDA(cudaStreamSynchronize(s));
  } else {
    ZG_TRY(perm_from_ipiv(n, ipiv, perm, s));
  }
  ZG_TRY(invert_diag_blocks(n, LU, n, Linv, Uinv, Linv32, Uinv32, !spd, s));
  c->n = n;
  c->m = m;
  c->A = A;
  c->lda = lda;
  c->anrm = anrm;
  c->ctl = ctl;
  c->f = f;
  c->w = w;
  return 0;
}

// Refinement phase on the factors of c.  warm: X already holds an iterate
// (a previous refinement call's result) and refinement continues from it;
// otherwise it starts from x0 = (LU)^-1 P b.  Fills res's iteration fields.
static int mpir_refine(MpirCtx &c, const MpirOpts &o, int nrhs, const double *B, long ldb,
                       double *X, long ldx, bool warm, MpirResult *res, cudaStream_t s) {
  const int n = c.n, m = c.m;
  const double *A = c.A;
  const long lda = c.lda;
  const double anrm = c.anrm;
  Control *ctl = c.ctl;
  LowLU &f = c.f;
  IRWork &w = c.w;
  res->converged = 1;
  for (int q = 0; q < nrhs; ++q) {
    const double *b = B + (long)q * ldb;
    double *x = X + (long)q * ldx;
    ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, b, w.scal));
    double bnrm;
    ZG_TRY(host_scalar(w.scal, &bnrm, s));
    // x0 = (LU)^-1 P b
    if (!warm) ZG_TRY(lu_apply(n, f, b, x, w.tw, &ctl->status, s));
    double berr = 0, prev = INFINITY;
    ZG_TRY(berr_of(n, A, lda, b, x, anrm, bnrm, w, &berr, s));  // leaves r = b - A x
    if (q == 0) res->berr_history[0] = berr;
    int it = 0;
    const double tol = o.tol > 0 ? o.tol : 0.0;
    while (it < o.max_iter) {
      if (berr <= tol) break;
      if (it > 0 && berr > 0.5 * prev) {
        // no progress: with FP32 application, retry in FP64 arithmetic
        // (ill-conditioned factors); otherwise the floor is reached, or the
        // factors cannot take the error down to tol -- stop either way
        if (f.f64 || o.apply != kApplyAuto || berr < 1e3 * 1.1102230246251565e-16) break;
        f.f64 = true;
        res->switched_f64 = 1;
      }
      prev = std::min(prev, berr);
      if (o.mode == kModeGMRES) {
        ZG_TRY(gmres_correction(n, A, lda, f, w, m, o.gmres_rtol, &res->inner_iters, ctl, s));
      } else {
        ZG_TRY(lu_apply(n, f, w.r, w.d, w.tw, &ctl->status, s));
      }
      ZG_LAUNCH(kTagVector, 0, 0, s, axpy_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, 1.0, w.d, x));
      ++it;
      ZG_TRY(berr_of(n, A, lda, b, x, anrm, bnrm, w, &berr, s));
      if (q == 0 && it < 32) res->berr_history[it] = berr;
      if (std::isfinite(berr) && berr > prev && berr <= 1e3 * prev) {
        // the step made the iterate worse (a correction through factors too
        // ill-conditioned for its arithmetic): take it back, so that what
        // follows starts from the best iterate, not from the damaged one
        ZG_LAUNCH(kTagVector, 0, 0, s,
                  axpy_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, -1.0, w.d, x));
        ZG_TRY(berr_of(n, A, lda, b, x, anrm, bnrm, w, &berr, s));
      }
      if (!std::isfinite(berr) || berr > 1e3 * prev) {  // diverged
        if (f.f64 || o.apply != kApplyAuto) break;
        f.f64 = true;  // restart the refinement from the first solve in FP64
        res->switched_f64 = 1;
        ZG_TRY(lu_apply(n, f, b, x, w.tw, &ctl->status, s));
        ZG_TRY(berr_of(n, A, lda, b, x, anrm, bnrm, w, &berr, s));
        prev = INFINITY;
      }
    }
    res->iters = std::max(res->iters, it);
    res->berr = std::max(res->berr, berr);
    const bool ok = std::isfinite(berr) && (tol > 0 ? berr <= tol : berr <= 64 * 1.1102230246251565e-16);
    if (!ok) res->converged = 0;
  }
  ZG_TRY(check_status(s, ctl, nullptr));
  return 0;
}

// ---------------------------------------------------------------------------
// The plain FP64 factorizations, on a copy of A, as the last resort of the
// mixed solvers (their refinement stopped short) and of the precision ladder.

// Largest normwise backward error over the nrhs columns of X for A X = B (A
// full, column-major); infinite if any column's is not finite.
static int berr_cols(int n, int nrhs, const double *A, long lda, const double *B, long ldb,
                     const double *X, long ldx, IRWork &w, double *berr, cudaStream_t s) {
  const int nparts = ceil_div(n, kGemvCols);
  ZG_LAUNCH(kTagGemv, 0, 8.0 * n * n, s,
            rowabs_partial_kernel<<<dim3(ceil_div(n, kGemvRows), nparts), kGemvRows, 0, s>>>(
                n, A, lda, w.part));
  ZG_LAUNCH(kTagGemv, 0, 0, s,
            gemv_finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, nparts, w.part, nullptr, w.r));
  ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, w.r, w.scal));
  double anrm;
  ZG_TRY(host_scalar(w.scal, &anrm, s));
  *berr = 0;
  for (int q = 0; q < nrhs; ++q) {
    const double *b = B + (long)q * ldb;
    ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, b, w.scal));
    double bnrm, e;
    ZG_TRY(host_scalar(w.scal, &bnrm, s));
    ZG_TRY(berr_of(n, A, lda, b, X + (long)q * ldx, anrm, bnrm, w, &e, s));
    *berr = std::isfinite(e) ? std::max(*berr, e) : INFINITY;
  }
  return 0;
}

// Workspace of the FP64 fallback: the factor copy (ld n), the pivots and the
// vectors of berr_cols.
static int fp64_work(int n, double **F, int **piv, IRWork *w, cudaStream_t s) {
  const int nparts = ceil_div(n, kGemvCols);
  const size_t nd = (size_t)n * n + (size_t)n * (1 + nparts) + 8;
  void *wp;
  ZG_TRY(workspace(s, kSlotF64LU, sizeof(double) * nd + sizeof(int) * (size_t)n + 256, &wp));
  *F = (double *)wp;
  *w = IRWork{};
  w->r = *F + (size_t)n * n;
  w->part = w->r + n;
  w->scal = w->part + (size_t)n * nparts;
  *piv = (int *)(w->scal + 8);
  return 0;
}

// Plain FP64 partial-pivot LU and solve (the reference's gesv, getrf.zig:14 +
// getrs.zig:13) on a copy of A, with the largest backward error over the
// columns; X is left unset when info > 0.
static int fp64_solve(int n, int nrhs, const double *A, long lda, const double *B, long ldb,
                      double *X, long ldx, double *berr, int *info, cudaStream_t s) {
  double *LU;
  int *piv;
  IRWork w;
  ZG_TRY(fp64_work(n, &LU, &piv, &w, s));
  ZG_CUDA(cudaMemcpy2DAsync(LU, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n,
                            n, cudaMemcpyDeviceToDevice, s));
  *berr = INFINITY;
  ZG_TRY(getrf_dev<double>(n, n, LU, n, piv, info, s));
  if (*info != 0) return 0;
  ZG_CUDA(cudaMemcpy2DAsync(X, sizeof(double) * ldx, B, sizeof(double) * ldb, sizeof(double) * n,
                            nrhs, cudaMemcpyDeviceToDevice, s));
  ZG_TRY(getrs_dev<double>(kNoTrans, n, nrhs, LU, n, piv, X, ldx, s));
  return berr_cols(n, nrhs, A, lda, B, ldb, X, ldx, w, berr, s);
}

// The SPD counterpart (posv.zig:15: potrf.zig:17 + potrs.zig:15) on a copy of
// the `lower` (else upper) triangle of A; the backward error is measured on
// the full symmetric matrix, which is rebuilt into the Sym slot.
static int fp64_posv(bool lower, int n, int nrhs, const double *A, long lda, const double *B,
                     long ldb, double *X, long ldx, double *berr, int *info, cudaStream_t s) {
  double *F;
  int *piv;
  IRWork w;
  ZG_TRY(fp64_work(n, &F, &piv, &w, s));
  ZG_CUDA(cudaMemcpy2DAsync(F, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n,
                            n, cudaMemcpyDeviceToDevice, s));
  *berr = INFINITY;
  const int uplo = lower ? kLower : kUpper;
  ZG_TRY(potrf_dev<double>(uplo, n, F, n, info, s));
  if (*info != 0) return 0;
  ZG_CUDA(cudaMemcpy2DAsync(X, sizeof(double) * ldx, B, sizeof(double) * ldb, sizeof(double) * n,
                            nrhs, cudaMemcpyDeviceToDevice, s));
  ZG_TRY(potrs_dev<double>(uplo, n, nrhs, F, n, X, ldx, s));
  void *ws;
  ZG_TRY(workspace(s, kSlotSym, sizeof(double) * (size_t)n * n, &ws));
  ZG_LAUNCH(kTagConvert, 0, 16.0 * n * n, s,
            sym_full_kernel<<<grid1d((long)n * n), 256, 0, s>>>(n, A, lda, lower, (double *)ws));
  return berr_cols(n, nrhs, (const double *)ws, n, B, ldb, X, ldx, w, berr, s);
}

static int solve_mpir_dev(bool spd, bool lower, int n, int nrhs, const double *A, long lda,
                          const double *B, long ldb, double *X, long ldx, const MpirOpts &o,
                          MpirResult *res, cudaStream_t s, const double *Ah = nullptr,
                          long ldh = 0) {
  *res = MpirResult{};
  if (n <= 0 || nrhs <= 0) return 0;
  MpirCtx c;
  ZG_TRY(mpir_factor(spd, lower, n, A, lda, o, &c, res, s, Ah, ldh));
  if (res->info == 0) ZG_TRY(mpir_refine(c, o, nrhs, B, ldb, X, ldx, false, res, s));
  if (!o.fallback || (res->info == 0 && res->converged)) return 0;
  // the safety net: the low-precision factors could not take the backward
  // error down to the target, so the FP64 factorization solves the system
  double berr = INFINITY;
  int info = 0;
  if (spd)
    ZG_TRY(fp64_posv(lower, n, nrhs, A, lda, B, ldb, X, ldx, &berr, &info, s));
  else
    ZG_TRY(fp64_solve(n, nrhs, A, lda, B, ldb, X, ldx, &berr, &info, s));
  res->fp64_fallback = 1;
  res->info = info;
  res->berr = berr;
  // the FP64 factorization's backward error is FP64 accuracy by definition
  // (at n = 16384 it can lie above 64 u, or a little above a tol taken from
  // another FP64 solve)
  res->converged = info == 0 && std::isfinite(berr);
  return 0;
}

int gesv_mpir_dev(int n, int nrhs, const double *A, long lda, const double *B, long ldb,
                  double *X, long ldx, const MpirOpts &o, MpirResult *res, cudaStream_t s) {
  return solve_mpir_dev(false, false, n, nrhs, A, lda, B, ldb, X, ldx, o, res, s);
}

int gesv_mpir_host(int n, int nrhs, const double *Ah, long ldh, double *Ad, const double *B,
                   long ldb, double *X, long ldx, const MpirOpts &o, MpirResult *res,
                   cudaStream_t s) {
  if (!mixed_streams_host(n, o)) {
    set_last_error("gesv_mpir_host: needs n >= %d and BF16x3 updates", kChunkMinN);
    return kErrInvalid;
  }
  return solve_mpir_dev(false, false, n, nrhs, Ad, n, B, ldb, X, ldx, o, res, s, Ah, ldh);
}

int posv_mpir_dev(bool lower, int n, int nrhs, const double *A, long lda, const double *B,
                  long ldb, double *X, long ldx, const MpirOpts &o, MpirResult *res,
                  cudaStream_t s) {
  return solve_mpir_dev(true, lower, n, nrhs, A, lda, B, ldb, X, ldx, o, res, s);
}

// ---------------------------------------------------------------------------
// Precision selection.

// u_i = (-1)^i (1 + i / n): the start of the inverse iteration, with no
// structure a test matrix family shares
__global__ void cond_start_kernel(int n, double *u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) u[i] = (i & 1 ? -1.0 : 1.0) * (1.0 + (double)i / n);
}
// y = x / *den when *den is positive and finite, else y = x
__global__ void scale_inv_kernel(int n, const double *den, const double *x, double *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double d = *den;
  if (i < n) y[i] = (d > 0 && d <= 1.79e308) ? x[i] / d : x[i];
}

// A few-step condition estimate from the low-precision factors of c:
// `steps` steps of inverse iteration z = (LU)^-1 P u, u = z / ||z||_inf,
// whose last ||z||_inf (with ||u||_inf = 1) is a lower estimate of
// ||A^-1||_inf; kappa = ||A||_inf times it.  Scratch: the first two Krylov
// columns of c's work, which no refinement call keeps between calls.
static int cond_estimate(MpirCtx &c, int steps, double *kappa, cudaStream_t s) {
  const int n = c.n, b1 = ceil_div(n, 256);
  double *u = c.w.V, *z = c.w.V + n;
  ZG_LAUNCH(kTagVector, 0, 0, s, cond_start_kernel<<<b1, 256, 0, s>>>(n, u));
  ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, u, c.w.scal + 2));
  ZG_LAUNCH(kTagVector, 0, 0, s, scale_inv_kernel<<<b1, 256, 0, s>>>(n, c.w.scal + 2, u, u));
  for (int it = 0; it < steps; ++it) {
    ZG_TRY(lu_apply(n, c.f, u, z, c.w.tw, &c.ctl->status, s));
    ZG_LAUNCH(kTagVector, 0, 0, s, absmax_kernel<<<1, 256, 0, s>>>(n, z, c.w.scal + 2));
    ZG_LAUNCH(kTagVector, 0, 0, s, scale_inv_kernel<<<b1, 256, 0, s>>>(n, c.w.scal + 2, z, u));
  }
  ZG_CUDA(cudaGetLastError());
  double zn;
  ZG_TRY(host_scalar(c.w.scal + 2, &zn, s));
  *kappa = c.anrm * zn;
  return 0;
}

void probe_features(const MpirResult &pr, double kappa, float *f) {
  // log10 of a backward error, clamped to [1e-18, 1e2] (non-finite: 1e2)
  auto lg = [](double v) {
    if (!std::isfinite(v)) v = 1e2;
    return (float)std::log10(std::min(1e2, std::max(v, 1e-18)));
  };
  if (pr.info != 0) {
    f[12] = f[13] = f[14] = 0.f;
    f[15] = 1.f;
    return;
  }
  const double h0 = pr.berr_history[0];
  const double h1 = pr.iters >= 1 ? pr.berr_history[1] : h0;
  f[12] = lg(h0);
  f[13] = lg(h1) - lg(h0);
  // log10 of the condition estimate, in [0, 20] (non-finite: 20)
  const double k = std::isfinite(kappa) ? std::min(std::max(kappa, 1.0), 1e20) : 1e20;
  f[14] = (float)std::log10(k);
  f[15] = pr.switched_f64 ? 0.5f : 0.f;
}

int gesv_auto_dev(int n, int nrhs, const double *A, long lda, const double *B, long ldb, double *X,
                  long ldx, const float *model, float confidence, int max_iter, AutoResult *r,
                  cudaStream_t s) {
  *r = AutoResult{};
  const auto t0 = std::chrono::steady_clock::now();
  auto finish = [&]() -> int {
    ZG_CUDA(cudaStreamSynchronize(s));
    r->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
  };
  if (n <= 0 || nrhs <= 0) {
    r->used = kClassBF16;
    r->converged = 1;
    return finish();
  }
  if (max_iter <= 0) max_iter = 10;
  const int probe_steps = std::min(2, max_iter);
  const int np = selector_num_params();
  void *wn;
  const size_t nnet = (size_t)np + kSelFeatures + 8 + mlp_work_floats(1) + 64;
  ZG_TRY(workspace(s, kSlotSelNet, sizeof(float) * nnet, &wn));
  float *dP = (float *)wn, *dx = dP + np, *dz = dx + kSelFeatures, *dwork = dz + 8;

  // structural features, then the probe: BF16 factors and their first
  // refinement steps
  float feat[kSelFeatures];
  ZG_TRY(selector_features(n, A, lda, dx, s));
  ZG_CUDA(cudaMemcpyAsync(feat, dx, sizeof feat, cudaMemcpyDeviceToHost, s));
  MpirOpts o;
  o.prec = kPrecBF16;
  o.mode = kModeGMRES;
  o.max_iter = probe_steps;
  o.gmres_rtol = 1e-6;  // the probe features are the backward errors after 1e-6 GMRES steps
  MpirCtx c;
  MpirResult pr;
  ZG_TRY(mpir_factor(false, false, n, A, lda, o, &c, &pr, s));
  r->attempts = 1;
  double kappa = 0;
  if (pr.info == 0) {
    ZG_TRY(mpir_refine(c, o, nrhs, B, ldb, X, ldx, false, &pr, s));
    ZG_TRY(cond_estimate(c, kCondSteps, &kappa, s));
  }
  ZG_CUDA(cudaStreamSynchronize(s));
  probe_features(pr, kappa, feat);
  std::copy(feat, feat + kSelFeatures, r->features);
  if (pr.info == 0 && pr.converged) {
    r->used = kClassBF16;
    r->converged = 1;
    r->iters = pr.iters;
    r->berr = pr.berr;
    return finish();
  }

  int start = kClassBF16;
  if (model) {
    const float *mu = model + np, *sd = mu + kSelFeatures;
    float xin[kSelFeatures], z[kNumClasses];
    for (int k = 0; k < kSelFeatures; ++k) xin[k] = (feat[k] - mu[k]) / sd[k];
    ZG_CUDA(cudaMemcpyAsync(dP, model, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    ZG_CUDA(cudaMemcpyAsync(dx, xin, sizeof xin, cudaMemcpyHostToDevice, s));
    ZG_TRY(mlp_forward(1, dx, dP, dz, dwork, s));
    ZG_CUDA(cudaGetLastError());
    ZG_CUDA(cudaMemcpyAsync(z, dz, sizeof z, cudaMemcpyDeviceToHost, s));
    ZG_CUDA(cudaStreamSynchronize(s));
    double zmax = z[0], den = 0, cum = 0;
    for (int k = 1; k < kNumClasses; ++k) zmax = std::max(zmax, (double)z[k]);
    for (int k = 0; k < kNumClasses; ++k) den += std::exp(z[k] - zmax);
    start = kClassFP64;
    for (int k = 0; k < kNumClasses; ++k) {
      r->proba[k] = (float)(std::exp(z[k] - zmax) / den);
      cum += r->proba[k];
      if (cum >= confidence && start == kClassFP64) start = k;
    }
    r->predicted = start;
  }

  for (int cls = start; cls < kNumClasses; ++cls) {
    if (cls == kClassBF16) {
      // continue the probe's refinement from its iterate (it stopped early
      // only when it stagnated, and then BF16 has failed)
      if (pr.info != 0 || pr.iters < probe_steps || max_iter <= pr.iters) continue;
      MpirOpts oc = o;
      oc.max_iter = max_iter - pr.iters;
      MpirResult cr;
      ZG_TRY(mpir_refine(c, oc, nrhs, B, ldb, X, ldx, true, &cr, s));
      if (cr.converged) {
        r->used = kClassBF16;
        r->converged = 1;
        r->iters = pr.iters + cr.iters;
        r->berr = cr.berr;
        return finish();
      }
      continue;
    }
    if (cls == kClassFP64) {
      int info = 0;
      double berr = INFINITY;
      ZG_TRY(fp64_solve(n, nrhs, A, lda, B, ldb, X, ldx, &berr, &info, s));
      ++r->attempts;
      r->used = kClassFP64;
      r->info = info;
      r->berr = berr;
      r->converged = info == 0 && berr <= 64 * 1.1102230246251565e-16;
      return finish();
    }
    MpirOpts oc;
    oc.prec = kClassPrec[cls];
    oc.mode = kModeGMRES;
    oc.max_iter = max_iter;
    MpirResult cr;
    ZG_TRY(solve_mpir_dev(false, false, n, nrhs, A, lda, B, ldb, X, ldx, oc, &cr, s));
    ++r->attempts;
    if (cr.info == 0 && cr.converged) {
      r->used = cls;
      r->converged = 1;
      r->iters = cr.iters;
      r->berr = cr.berr;
      return finish();
    }
  }
  return finish();
}

}  // namespace zg
