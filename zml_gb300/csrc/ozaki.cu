// ozaki.cu -- FP64 trailing updates on the BF16 tensor cores by error-free
// splitting.
//
// The FP64 LU and Cholesky spend nearly all their flops in updates C -= A B
// with k = 256, the block width.  GB300 runs FP64 at about 1.1 TFLOP/s and
// BF16 on tcgen05 at about 1.9 PFLOP/s, so the update is computed the way
// Ozaki's scheme does it (Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59,
// 2012), in the integer-slice form of Ootomo, Ozaki and Yokota (IJHPCA, 2024):
//   * every row of A and every column of B is scaled by a power of two, 2^e,
//     so that its largest entry lies below 2^7, and cut into S = 8 slices of
//     integers, |x_0| <= 128 and |x_i| <= 64 after it, each exact in BF16:
//     row = 2^(e - 7) (x_0 + 2^-7 x_1 + ... + 2^-49 x_7) to within 2^-56 of its
//     largest entry;
//   * the slice products are grouped by d = i + j.  For each d the sum of
//     A_i B_(d-i)^T is one BF16 GEMM over the slices laid side by side along K
//     (A as [A_0 | A_1 | ... | A_7], B as [B_7 | ... | B_1 | B_0], so that the
//     first (d+1) k columns of A's layout meet the last (d+1) k of B's).  The
//     tensor cores accumulate in FP32; with k <= 256 every partial sum for
//     d <= 3 is an integer below 2^24, so those four products are exact.  The
//     groups d = 4 .. 7 share one accumulator (scaled by 2^-7 per step of d),
//     whose rounding stays below 2^-52 of the leading term;
//   * an FP64 kernel forms C -= 2^(e_r + e_c - 14) (C_0 + 2^-7 C_1 + 2^-14 C_2
//     + 2^-21 C_3 + 2^-28 C_4).
// Products with i + j >= 8 are dropped.  On N(0,1) data the result lies within
// about 6 u of |A| |B| of the exact product, against about 5 u for an FP64
// GEMM's own rounding.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "common.cuh"
#include "kernels.h"
#include "kernels_tc.h"

namespace zg {

namespace {

constexpr int kOzS = 8;        // slices
constexpr int kOzMaxK = 256;   // k that keeps the d <= 3 sums exact in FP32
constexpr int kOzAcc = 5;      // FP32 accumulators: d = 0, 1, 2, 3 and 4..7
constexpr int kOzRows = 32;    // rows of A a block splits
constexpr int kOzMinN = 2048;  // smaller LUs keep their updates on the FP64 pipe

// Exponent e with max|row| < 2^e (0 for a zero row).
__device__ __forceinline__ int oz_exponent(double mx) {
  if (!(mx > 0) || !isfinite(mx)) return 0;
  int e;
  (void)frexp(mx, &e);
  return e;
}

// The slices of one value scaled to |v| < 2^7: q_i = rint(v), v = (v - q_i) 2^7.
__device__ __forceinline__ void oz_slices(double v, float (&q)[kOzS]) {
#pragma unroll
  for (int i = 0; i < kOzS; ++i) {
    const double t = rint(v);
    q[i] = (float)t;
    v = (v - t) * 128.0;
  }
}

// Rows of A (m x k, column-major, k <= 256): per row its exponent and the S
// slices, written K-major with row stride S kp -- forward [X_0 .. X_7] into
// fwd and / or reversed [X_7 .. X_0] into rev (null: not wanted).  Columns k
// .. kp-1 of every slice are zero.  One block per 32 rows, transposed through
// shared memory.
__global__ void __launch_bounds__(256) oz_split_rows_kernel(int m, int k, const double *__restrict__ A,
                                                            long lda, int kp, __nv_bfloat16 *fwd,
                                                            __nv_bfloat16 *rev, int *ex) {
  extern __shared__ double ozt[];  // ozt[r * (kOzMaxK + 1) + c]
  __shared__ int er[kOzRows];
  constexpr int LD = kOzMaxK + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * kOzRows;
  for (int e = tid; e < kOzRows * k; e += blockDim.x) {
    const int r = e & (kOzRows - 1), c = e >> 5;
    ozt[r * LD + c] = r0 + r < m ? A[(r0 + r) + (long)c * lda] : 0.0;
  }
  __syncthreads();
  for (int r = warp; r < kOzRows; r += blockDim.x >> 5) {
    double mx = 0;
    for (int c = lane; c < k; c += 32) mx = fmax(mx, fabs(ozt[r * LD + c]));
    // a NaN anywhere makes the row's maximum NaN
    for (int c = lane; c < k; c += 32)
      if (ozt[r * LD + c] != ozt[r * LD + c]) mx = ozt[r * LD + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(~0u, mx, o);
      mx = (y != y || mx != mx) ? (y != y ? y : mx) : fmax(mx, y);
    }
    if (lane == 0) er[r] = oz_exponent(mx);
  }
  __syncthreads();
  const long ldo = (long)kOzS * kp;
  const int half = kp >> 1;
  for (int e = tid; e < kOzRows * half; e += blockDim.x) {
    const int r = e / half, c = 2 * (e - r * half);
    if (r0 + r >= m) continue;
    const int sh = 7 - er[r];
    const double x0 = c < k ? ozt[r * LD + c] : 0.0, x1 = c + 1 < k ? ozt[r * LD + c + 1] : 0.0;
    float q0[kOzS], q1[kOzS];
    oz_slices(ldexp(x0, sh), q0);
    oz_slices(ldexp(x1, sh), q1);
    __nv_bfloat16 *fr = fwd ? fwd + (long)(r0 + r) * ldo + c : nullptr;
    __nv_bfloat16 *rr = rev ? rev + (long)(r0 + r) * ldo + c : nullptr;
#pragma unroll
    for (int i = 0; i < kOzS; ++i) {
      const __nv_bfloat162 p = __floats2bfloat162_rn(q0[i], q1[i]);  // integers: exact
      if (fr) *reinterpret_cast<__nv_bfloat162 *>(fr + (long)i * kp) = p;
      if (rr) *reinterpret_cast<__nv_bfloat162 *>(rr + (long)(kOzS - 1 - i) * kp) = p;
    }
  }
  if (tid < kOzRows && r0 + tid < m) ex[r0 + tid] = er[tid];
}

// Columns of B (k x n, column-major): per column its exponent and the slices,
// reversed layout [X_7 .. X_0] with row stride S kp (one warp per column).
__global__ void __launch_bounds__(256) oz_split_cols_kernel(int k, int n, const double *__restrict__ B,
                                                            long ldb, int kp, __nv_bfloat16 *rev,
                                                            int *ex) {
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (col >= n) return;
  constexpr int kPer = kOzMaxK / 32;
  double x[kPer];
  double mx = 0;
  bool nan = false;
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int c = lane + 32 * t;
    x[t] = c < k ? B[c + (long)col * ldb] : 0.0;
    mx = fmax(mx, fabs(x[t]));
    nan |= x[t] != x[t];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(~0u, mx, o));
  nan = __any_sync(~0u, nan);
  const int e = oz_exponent(nan ? NAN : mx);
  const long ldo = (long)kOzS * kp;
  __nv_bfloat16 *out = rev + (long)col * ldo;
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int c = lane + 32 * t;
    if (c >= kp) continue;
    float q[kOzS];
    oz_slices(ldexp(nan && x[t] == x[t] ? NAN : x[t], 7 - e), q);
#pragma unroll
    for (int i = 0; i < kOzS; ++i) out[(long)(kOzS - 1 - i) * kp + c] = __float2bfloat16_rn(q[i]);
  }
  if (lane == 0) ex[col] = e;
}

// C (m x n) -= 2^(er + ec - 14) (C_0 + 2^-7 C_1 + 2^-14 C_2 + 2^-21 C_3 + 2^-28 C_4)
// with the accumulators W (m x n each, ld ldw, one after the other); lower:
// only r >= c.
__global__ void oz_combine_kernel(int m, int n, double *__restrict__ C, long ldc,
                                  const float *__restrict__ W, long ldw, long wstride,
                                  const int *__restrict__ er, const int *__restrict__ ec,
                                  bool lower) {
  const long total = (long)m * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int r = (int)(e % m), c = (int)(e / m);
    if (lower && r < c) continue;
    const long w = r + (long)c * ldw;
    double acc = (double)W[w + 4 * wstride];
    acc = acc * 0.0078125 + (double)W[w + 3 * wstride];
    acc = acc * 0.0078125 + (double)W[w + 2 * wstride];
    acc = acc * 0.0078125 + (double)W[w + wstride];
    acc = acc * 0.0078125 + (double)W[w];
    double *cp = C + r + (long)c * ldc;
    *cp -= ldexp(acc, er[r] + ec[c] - 14);
  }
}

__global__ void ipiv_add_kernel(int n, int *ipiv, int add) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ipiv[i] += add;
}

std::atomic<int> g_oz_mode{1};  // 1: tensor-core updates above the threshold

}  // namespace

int set_fp64_updates(int mode) { return g_oz_mode.exchange(mode != 0 ? 1 : 0); }
bool fp64_updates_on_tensor_cores(int m, int n) {
  return g_oz_mode.load() != 0 && std::min(m, n) >= kOzMinN;
}

// C (m x n) -= A B with A m x k (lda) and B k x n (ldb), FP64, column-major,
// k <= 256.  syrk: C -= A A^T on C's lower triangle (m == n; B unused).
int dgemm_oz_sub(int m, int n, int k, const double *A, long lda, const double *B, long ldb,
                 double *C, long ldc, bool syrk, unsigned *status, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  if (k > kOzMaxK) {
    set_last_error("dgemm_oz_sub: k = %d > %d", k, kOzMaxK);
    return kErrInvalid;
  }
  if (syrk && m != n) return kErrInvalid;
  const int kp = (k + 63) / 64 * 64;
  const long ldo = (long)kOzS * kp;
  // chunks of C's columns bound the FP32 accumulators
  const int nc = std::min(n, 4096);
  const long ldw = m;
  const size_t aop = sizeof(__nv_bfloat16) * (size_t)m * ldo;
  const size_t bop = sizeof(__nv_bfloat16) * (size_t)n * ldo;
  const size_t acc = sizeof(float) * (size_t)ldw * nc * kOzAcc;
  void *wa, *wb, *wc;
  ZG_TRY(workspace(s, kSlotOzA, aop + sizeof(int) * (size_t)m + 512, &wa));
  ZG_TRY(workspace(s, kSlotOzB, bop + sizeof(int) * (size_t)n + 512, &wb));
  ZG_TRY(workspace(s, kSlotOzC, acc, &wc));
  __nv_bfloat16 *Af = (__nv_bfloat16 *)wa;
  int *ea = (int *)((char *)wa + ((aop + 255) & ~(size_t)255));
  __nv_bfloat16 *Br = (__nv_bfloat16 *)wb;
  int *eb = (int *)((char *)wb + ((bop + 255) & ~(size_t)255));
  float *W = (float *)wc;
  const int smem = sizeof(double) * kOzRows * (kOzMaxK + 1);
  ZG_TRY(smem_optin(oz_split_rows_kernel, smem));
  ZG_LAUNCH(kTagConvert, 0, 8.0 * m * k + 2.0 * m * ldo * (syrk ? 2 : 1), s,
            oz_split_rows_kernel<<<ceil_div(m, kOzRows), 256, smem, s>>>(
                m, k, A, lda, kp, Af, syrk ? Br : nullptr, ea));
  if (!syrk)
    ZG_LAUNCH(kTagConvert, 0, 8.0 * n * k + 2.0 * n * ldo, s,
              oz_split_cols_kernel<<<ceil_div(n, 8), 256, 0, s>>>(k, n, B, ldb, kp, Br, eb));
  const int *ecol = syrk ? ea : eb;
  for (int c0 = 0; c0 < n; c0 += nc) {
    const int w = std::min(nc, n - c0);
    // syrk: rows above the chunk's first column hold no lower-triangle entries
    const int r0 = syrk ? c0 : 0, rows = m - r0;
    for (int d = 0; d < kOzS; ++d) {
      const int slot = std::min(d, kOzAcc - 1);
      const float alpha = d < kOzAcc - 1 ? 1.f : ldexpf(1.f, -7 * (d - (kOzAcc - 1)));
      const float beta = d <= kOzAcc - 1 ? 0.f : 1.f;
      ZG_TRY(gemm_tc(rows, w, (d + 1) * kp, alpha, Af + (long)r0 * ldo, ldo,
                     Br + (long)(kOzS - 1 - d) * kp + (long)c0 * ldo, ldo, beta,
                     W + (size_t)slot * ldw * nc, ldw, 1, status, s, syrk ? 1 : 0));
    }
    const long total = (long)rows * w;
    const int grid = (int)std::min<long>((total + 255) / 256, 152L * 8);
    ZG_LAUNCH(kTagConvert, 0, (8.0 * 2 + 4.0 * kOzAcc) * total, s,
              oz_combine_kernel<<<grid, 256, 0, s>>>(rows, w, C + r0 + (long)c0 * ldc, ldc, W, ldw,
                                                     (long)ldw * nc, ea + r0, ecol + c0, syrk));
  }
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// FP64 LU with partial pivoting, blocked with NB = 256: each 256-column panel
// is factored by the FP64-pipe getrf (64-column cooperative panels, its own
// small updates), the interchanges reach the other columns, U12 = L11^-1 A12
// is a triangular solve, and the trailing update A22 -= L21 U12 -- nearly all
// of the flops -- runs on the tensor cores through dgemm_oz_sub.  The loop is
// getrf.zig:52-136's with a wider block.
int getrf_oz(int m, int n, double *A, long lda, int *ipiv, int *info, cudaStream_t s) {
  constexpr int NB = 256;
  *info = 0;
  const int mn = std::min(m, n);
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  for (int j = 0; j < mn; j += NB) {
    const int jb = std::min(NB, mn - j);
    double *Ajj = A + j + (long)j * lda;
    int iinfo = 0;
    ZG_TRY(getrf_simt<double>(m - j, jb, Ajj, lda, ipiv + j, &iinfo, s));
    if (*info == 0 && iinfo > 0) *info = iinfo + j;
    ZG_LAUNCH(kTagVector, 0, 0, s, ipiv_add_kernel<<<ceil_div(jb, 256), 256, 0, s>>>(jb, ipiv + j, j));
    ZG_TRY(laswp_panel<double>(j, std::min(n, j + jb), n, A, lda, j + 1, j + jb, ipiv, s));
    if (j + jb < n) {
      double *A12 = A + j + (long)(j + jb) * lda;
      ZG_TRY(trsm_dev<double>(kLeft, kLower, kNoTrans, kUnit, jb, n - j - jb, 1.0, Ajj, lda, A12,
                              lda, s));
      if (j + jb < m) {
        ZG_TRY(dgemm_oz_sub(m - j - jb, n - j - jb, jb, Ajj + jb, lda, A12, lda, A12 + jb, lda,
                            false, &ctl->status, s));
        // the next panel's getrf re-arms the stream's status word: read it now
        ZG_TRY(check_status(s, ctl, nullptr));
      }
    }
  }
  return check_status(s, ctl, nullptr);
}

// FP64 Cholesky A = L L^T (lower), right-looking with NB = 256: the diagonal
// block by the FP64-pipe potrf (64-wide steps), the block column by a
// triangular solve, and the trailing SYRK A22 -= L21 L21^T on the tensor cores
// through dgemm_oz_sub's lower form.  The first non-positive pivot lands in
// info (1-based), as potrf2.zig:37-47 reports it.
int potrf_oz(int n, double *A, long lda, int *info, cudaStream_t s) {
  constexpr int NB = 256;
  *info = 0;
  if (n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  for (int j = 0; j < n; j += NB) {
    const int jb = std::min(NB, n - j);
    double *Ajj = A + j + (long)j * lda;
    ZG_TRY(potrf_launch<double>(kLower, jb, Ajj, lda, ctl, j, s));
    const int rest = n - j - jb;
    if (rest <= 0) break;
    double *A21 = Ajj + jb;
    ZG_TRY(trsm_dev<double>(kRight, kLower, kTrans, kNonUnit, rest, jb, 1.0, Ajj, lda, A21, lda, s));
    ZG_TRY(dgemm_oz_sub(rest, rest, jb, A21, lda, nullptr, 0, A21 + (long)jb * lda, lda, true,
                        &ctl->status, s));
  }
  return check_status(s, ctl, info);
}

}  // namespace zg
