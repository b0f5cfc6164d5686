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
#include <map>
#include <mutex>

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

// Bits of |x| (sign cleared): for finite x they order as |x| does, and a
// NaN or inf has every exponent bit set.
__device__ __forceinline__ unsigned long long oz_abits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
constexpr unsigned long long kOzInfBits = 0x7ff0000000000000ull;

// Exponent e with max|row| < 2^e (0 for a zero or non-finite row), from the
// bits of the row's largest |x|: frexp's exponent, taken from the exponent
// field (normal) or the leading-zero count of the fraction (subnormal).
__device__ __forceinline__ int oz_exponent_bits(unsigned long long b) {
  if (b == 0 || b >= kOzInfBits) return 0;
  const int ex = (int)(b >> 52);
  if (ex != 0) return ex - 1022;
  return -1010 - __clzll((long long)b);  // b < 2^52: 2^(-1074) b in [2^(e-1), 2^e)
}

// 2^p as a double for the normal range, else 0 (the caller uses ldexp then).
__device__ __forceinline__ double oz_pow2(int p) {
  return (p >= -1022 && p <= 1023) ? __longlong_as_double((long long)(p + 1023) << 52) : 0.0;
}

// The S slices of x, a value of a row (column) whose entries lie below 2^e in
// magnitude: N = x 2^(56 - e) rounded to an integer (|N| < 2^56; exact unless
// x lies more than 2^3 below 2^(e - 53)), then N's balanced base-2^7 digits
// from the top, q_i = round(r / 2^(49 - 7 i)), r -= q_i 2^(49 - 7 i): |q_0| <= 128,
// |q_i| <= 64, and N = sum q_i 2^(49 - 7 i) exactly.  N is formed from x's
// fraction and exponent by shifts with round-half-even -- the value the
// scaling x 2^(56 - e) (exact) rounded by __double2ll_rn gives -- so the whole
// split runs on the integer pipes.  A non-finite row (nan set) gives NaN
// slices.
__device__ __forceinline__ void oz_slices(double x, int e, bool nan, float (&q)[kOzS]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int ex = (int)((bits >> 52) & 0x7ff);
  if (nan || ex == 0x7ff) {
#pragma unroll
    for (int i = 0; i < kOzS; ++i) q[i] = __int_as_float(0x7fc00000);
    return;
  }
  unsigned long long mant = bits & 0xfffffffffffffull;
  if (ex != 0) mant |= 1ull << 52;
  else ex = 1;  // subnormal: 2^(1 - 1075) times the fraction
  const int t = ex - 1019 - e;  // |x| 2^(56 - e) = mant 2^t, t <= 3
  unsigned long long a;
  if (t >= 0) {
    a = mant << t;
  } else if (t < -63) {
    a = 0;
  } else {
    const int k = -t;
    a = mant >> k;
    const unsigned long long rem = mant & ((1ull << k) - 1), half = 1ull << (k - 1);
    if (rem > half || (rem == half && (a & 1))) ++a;
  }
  long long r = (bits >> 63) ? -(long long)a : (long long)a;
#pragma unroll
  for (int i = 0; i < kOzS - 1; ++i) {
    const int sh = 49 - 7 * i;
    const long long t2 = (r + (1ll << (sh - 1))) >> sh;
    r -= t2 << sh;
    q[i] = (float)(int)t2;
  }
  q[kOzS - 1] = (float)(int)r;
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
  __shared__ bool bad[kOzRows];
  constexpr int LD = kOzMaxK + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * kOzRows;
  for (int e = tid; e < kOzRows * k; e += blockDim.x) {
    const int r = e & (kOzRows - 1), c = e >> 5;
    ozt[r * LD + c] = r0 + r < m ? A[(r0 + r) + (long)c * lda] : 0.0;
  }
  __syncthreads();
  for (int r = warp; r < kOzRows; r += blockDim.x >> 5) {
    unsigned long long mx = 0;  // the bits of the largest |x| (integers order them)
    for (int c = lane; c < k; c += 32) mx = max(mx, oz_abits(ozt[r * LD + c]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(~0u, mx, o));
    if (lane == 0) {
      er[r] = oz_exponent_bits(mx);
      bad[r] = mx >= kOzInfBits;
    }
  }
  __syncthreads();
  const long ldo = (long)kOzS * kp;
  const int half = kp >> 1;
  for (int e = tid; e < kOzRows * half; e += blockDim.x) {
    const int r = e / half, c = 2 * (e - r * half);
    if (r0 + r >= m) continue;
    const double x0 = c < k ? ozt[r * LD + c] : 0.0, x1 = c + 1 < k ? ozt[r * LD + c + 1] : 0.0;
    float q0[kOzS], q1[kOzS];
    oz_slices(x0, er[r], bad[r], q0);
    oz_slices(x1, er[r], bad[r], q1);
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
  unsigned long long mx = 0;
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int c = lane + 32 * t;
    x[t] = c < k ? B[c + (long)col * ldb] : 0.0;
    mx = max(mx, oz_abits(x[t]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(~0u, mx, o));
  const bool nonfinite = mx >= kOzInfBits;
  const int e = oz_exponent_bits(mx);
  const long ldo = (long)kOzS * kp;
  __nv_bfloat16 *out = rev + (long)col * ldo;
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int c = lane + 32 * t;
    if (c >= kp) continue;
    float q[kOzS];
    oz_slices(x[t], e, nonfinite, q);
#pragma unroll
    for (int i = 0; i < kOzS; ++i) out[(long)(kOzS - 1 - i) * kp + c] = __float2bfloat16_rn(q[i]);
  }
  if (lane == 0) ex[col] = e;
}

// C (m x n) -= 2^(er + ec - 14) (C_0 + 2^-7 C_1 + 2^-14 C_2 + 2^-21 C_3 + 2^-28 C_4)
// with the accumulators W (m x n each, ld ldw, wstride apart); lower: only
// r >= c.  C_0 .. C_3 are integers below 2^24 in magnitude, so they fold into
// one 64-bit integer exactly, I = 2^21 C_0 + 2^14 C_1 + 2^7 C_2 + C_3; the
// FP64 pipe then sees one conversion, one FMA for C_4 and one FMA into C.
// A thread takes kOzCR rows (256 apart) of kOzCC columns, so that a block
// moves enough bytes to be worth its launch and a thread has its loads of
// several elements in flight.
constexpr int kOzCR = 4, kOzCC = 4;
// Exact conversions on the integer pipes, which keep GB300's narrow FP64
// pipe (under one instruction a clock per SM) for the two FMAs that round:
// an integer |I| < 2^53 normalised by its leading-zero count into a double's
// exponent and fraction; a normal float's sign, exponent and mantissa moved
// into a double's fields (zero, subnormal, inf and NaN take the hardware
// conversion).
__device__ __forceinline__ double oz_ll2d(long long I) {
  if (I == 0) return 0.0;
  const unsigned long long a = I < 0 ? 0ull - (unsigned long long)I : (unsigned long long)I;
  const int lz = __clzll((long long)a);  // >= 11
  const unsigned long long frac = (a << (lz + 1)) >> 12;  // the bits below the leading one
  return __longlong_as_double((long long)((I < 0 ? 1ull << 63 : 0ull) |
                                          ((unsigned long long)(1086 - lz) << 52) | frac));
}
__device__ __forceinline__ double oz_f2d(float f) {
  const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                          ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double oz_fold(float w0, float w1, float w2, float w3, float w4) {
  if (isfinite(w0) && isfinite(w1) && isfinite(w2) && isfinite(w3)) {
    const long long I = ((long long)__float2int_rn(w0) << 21) + ((long long)__float2int_rn(w1) << 14) +
                        ((long long)__float2int_rn(w2) << 7) + (long long)__float2int_rn(w3);
    return fma(oz_f2d(w4), 0.0078125, oz_ll2d(I));  // |I| < 2^46
  }
  return (double)(w0 + w1 + w2 + w3 + w4);  // a NaN / inf operand reaches C as NaN
}
__global__ void __launch_bounds__(256) oz_combine_kernel(int m, int n, double *__restrict__ C,
                                                         long ldc, const float *__restrict__ W,
                                                         long ldw, long wstride,
                                                         const int *__restrict__ er,
                                                         const int *__restrict__ ec, bool lower) {
  const int r0 = blockIdx.x * (256 * kOzCR) + threadIdx.x, c0 = blockIdx.y * kOzCC;
#pragma unroll
  for (int cc = 0; cc < kOzCC; ++cc) {
    const int c = c0 + cc;
    if (c >= n) break;
    const int ecc = ec[c] - 35;
    float w[kOzCR][kOzAcc];
#pragma unroll
    for (int q = 0; q < kOzCR; ++q) {
      const int r = r0 + 256 * q;
      const float *wp = W + r + (long)c * ldw;
      const bool in = r < m && !(lower && r < c);
#pragma unroll
      for (int a = 0; a < kOzAcc; ++a) w[q][a] = in ? __ldcs(wp + a * wstride) : 0.f;
    }
#pragma unroll
    for (int q = 0; q < kOzCR; ++q) {
      const int r = r0 + 256 * q;
      if (r >= m || (lower && r < c)) continue;
      const double x = oz_fold(w[q][0], w[q][1], w[q][2], w[q][3], w[q][4]);
      const int p = er[r] + ecc;
      double *cp = C + r + (long)c * ldc;
      // the scale 2^p as a normal double when p is in range (an integer test)
      *cp = (p >= -1022 && p <= 1023) ? fma(-x, oz_pow2(p), *cp) : *cp - ldexp(x, p);
    }
  }
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
    const double total = (double)rows * w;
    const dim3 grid(ceil_div(rows, 256 * kOzCR), ceil_div(w, kOzCC));
    ZG_LAUNCH(kTagConvert, 0, (8.0 * 2 + 4.0 * kOzAcc) * total, s,
              oz_combine_kernel<<<grid, 256, 0, s>>>(rows, w, C + r0 + (long)c0 * ldc, ldc, W, ldw,
                                                     (long)ldw * nc, ea + r0, ecol + c0, syrk));
  }
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// FP64 LU with partial pivoting, blocked with NB = 256 -- the loop of
// getrf.zig:52-136 with a wider block.  Each 256-column block is factored as
// two 128-column halves by the cooperative FP64 panel (the pivot search of
// getrf2.zig:45-89 over the whole column), with the right half's update from
// the left one between them; the interchanges then reach the other columns,
// U12 = L11^-1 A12 is a triangular solve, and the trailing update
// A22 -= L21 U12 -- nearly all of the flops -- runs on the tensor cores
// through dgemm_oz_sub, as does the half-panel update (k = 128).  Every wait
// reports into one status word, read once at the end.
static int getrf_oz_blocks(int m, int n, double *A, long lda, int *ipiv, Control *ctl,
                           Lookahead &la);

int getrf_oz(int m, int n, double *A, long lda, int *ipiv, int *info, cudaStream_t s) {
  *info = 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  // both internal streams start after the caller's earlier work, and the
  // caller's stream resumes after both (also after a failure part way)
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = getrf_oz_blocks(m, n, A, lda, ipiv, ctl, *la);
  ZG_CUDA(cudaEventRecord(la->end_panel, la->panel));
  ZG_CUDA(cudaEventRecord(la->end_bulk, la->bulk));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_panel, 0));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_bulk, 0));
  if (rc != 0) return rc;
  return check_status(s, ctl, info);
}

// The blocks of getrf_oz.  Lookahead: a block's trailing update is split into
// the next block's columns (triangular solve and slice GEMM on the panel
// stream) and the rest (on the bulk stream), so the bulk of the update runs
// beside the next block's panels.  Block b's panels wait for the bulk update
// of block b-2, the last to touch their columns; block b's full-width
// interchanges for that of block b-1, which still reads block b-1's L21.
// Splitting the columns changes no element's arithmetic: the slices scale
// by rows of L21 and by columns of U12, and each column of the triangular
// solve is independent.
static int getrf_oz_blocks(int m, int n, double *A, long lda, int *ipiv, Control *ctl,
                           Lookahead &la) {
  constexpr int NB = 256;
  constexpr int R = Lookahead::kRing;
  const cudaStream_t s = la.panel, sb = la.bulk;
  const int mn = std::min(m, n);
  // sub-panel width: 64 columns.  On GB300 a panel's FP64 arithmetic runs on
  // the few SMs of its cluster at the FP64 pipe's rate, so narrower panels,
  // with the slice update between them on the tensor cores, cost less
  const int NBP = 64;
  for (int j = 0, b = 0; j < mn; j += NB, ++b) {
    const int jb = std::min(NB, mn - j);
    double *Ab = A + (long)j * lda;  // the block's columns
    if (b >= 2) ZG_CUDA(cudaStreamWaitEvent(s, la.bulk_done[(b - 2) % R], 0));
    for (int p = 0; p < jb; p += NBP) {
      const int r = j + p, pb = std::min(NBP, jb - p), right = jb - p - pb;
      double *Arr = A + r + (long)r * lda;
      // the half-panel on one thread-block cluster, its interchanges applied
      // to the block's other columns inside it; else the cooperative panel
      bool done = false;
      ZG_TRY(panel_lu_cluster(m - r, pb, Arr, lda, ipiv + r, r, ctl, r, s, &done, Ab + r, p,
                              Arr + (long)pb * lda, right));
      if (!done) {
        ZG_TRY(panel_lu<double>(m - r, pb, Arr, lda, ipiv + r, r, ctl, r, s));
        ZG_TRY(laswp_panel<double>(p, p + pb, jb, Ab, lda, r + 1, r + pb, ipiv, s));
      }
      if (right > 0) {
        double *Ar = Arr + (long)pb * lda;  // rows r.., the block's columns right of the half
        ZG_TRY(trsm_dev<double>(kLeft, kLower, kNoTrans, kUnit, pb, right, 1.0, Arr, lda, Ar, lda,
                                s));
        if (r + pb < m)
          ZG_TRY(dgemm_oz_sub(m - r - pb, right, pb, Arr + pb, lda, Ar, lda, Ar + pb, lda, false,
                              &ctl->status, s));
      }
    }
    // the block's interchanges in every column outside it
    if (b >= 1) ZG_CUDA(cudaStreamWaitEvent(s, la.bulk_done[(b - 1) % R], 0));
    ZG_TRY(laswp_panel<double>(j, std::min(n, j + jb), n, A, lda, j + 1, j + jb, ipiv, s));
    const int rest = n - j - jb;
    if (rest > 0) {
      double *Ajj = A + j + (long)j * lda;
      double *A12 = A + j + (long)(j + jb) * lda;
      // the next block's columns now, on the panel stream ...
      const int near = std::min(NB, rest);
      ZG_TRY(trsm_dev<double>(kLeft, kLower, kNoTrans, kUnit, jb, near, 1.0, Ajj, lda, A12, lda,
                              s));
      if (j + jb < m)
        ZG_TRY(dgemm_oz_sub(m - j - jb, near, jb, Ajj + jb, lda, A12, lda, A12 + jb, lda, false,
                            &ctl->status, s));
      // ... the rest on the bulk stream, beside the next block's panels
      if (rest > near) {
        ZG_CUDA(cudaEventRecord(la.upd[b % R], s));
        ZG_CUDA(cudaStreamWaitEvent(sb, la.upd[b % R], 0));
        double *A12f = A12 + (long)near * lda;
        ZG_TRY(trsm_dev<double>(kLeft, kLower, kNoTrans, kUnit, jb, rest - near, 1.0, Ajj, lda,
                                A12f, lda, sb));
        if (j + jb < m)
          ZG_TRY(dgemm_oz_sub(m - j - jb, rest - near, jb, Ajj + jb, lda, A12f, lda, A12f + jb,
                              lda, false, &ctl->status, sb));
      }
    }
    ZG_CUDA(cudaEventRecord(la.bulk_done[b % R], sb));
  }
  return 0;
}

// FP64 Cholesky A = L L^T (lower), right-looking with NB = 256: the diagonal
// block by the FP64-pipe potrf (64-wide steps), the block column by a
// triangular solve, and the trailing SYRK A22 -= L21 L21^T on the tensor cores
// through dgemm_oz_sub's lower form.  The first non-positive pivot lands in
// info (1-based), as potrf2.zig:37-47 reports it.  Lookahead as in getrf_oz:
// the next block's columns (its diagonal block by the lower SYRK, the rows
// below it by a GEMM against its rows of L21 transposed) on the panel stream,
// the rest of the SYRK on the bulk stream.  Block b's diagonal block and
// triangular solve wait for block b-2's bulk update, the last to touch their
// columns; block b's near update waits for block b-1's, which updates the same
// columns.  The strictly upper triangle is never written.
static int potrf_oz_blocks(int n, double *A, long lda, Control *ctl, Lookahead &la) {
  constexpr int NB = 256;
  constexpr int R = Lookahead::kRing;
  const cudaStream_t sp = la.panel, sb = la.bulk;
  void *wt;
  ZG_TRY(workspace(sp, kSlotOzT, sizeof(double) * NB * NB, &wt));
  double *T = (double *)wt;
  for (int j = 0, b = 0; j < n; j += NB, ++b) {
    const int jb = std::min(NB, n - j);
    double *Ajj = A + j + (long)j * lda;
    if (b >= 2) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 2) % R], 0));
    ZG_TRY(potrf_launch<double>(kLower, jb, Ajj, lda, ctl, j, sp));
    const int rest = n - j - jb;
    if (rest > 0) {
      double *A21 = Ajj + jb;
      ZG_TRY(trsm_dev<double>(kRight, kLower, kTrans, kNonUnit, rest, jb, 1.0, Ajj, lda, A21, lda,
                              sp));
      // the next block's columns now, on the panel stream, once block b-1's
      // bulk update (which also updates them) is done ...
      if (b >= 1) ZG_CUDA(cudaStreamWaitEvent(sp, la.bulk_done[(b - 1) % R], 0));
      const int near = std::min(NB, rest);
      ZG_TRY(dgemm_oz_sub(near, near, jb, A21, lda, nullptr, 0, A21 + (long)jb * lda, lda, true,
                          &ctl->status, sp));
      if (rest > near) {
        ZG_TRY(transpose_dev<double>(near, jb, A21, lda, T, jb, sp));
        ZG_TRY(dgemm_oz_sub(rest - near, near, jb, A21 + near, lda, T, jb,
                            A21 + near + (long)jb * lda, lda, false, &ctl->status, sp));
        // ... the rest on the bulk stream, beside the next block's diagonal
        // block and triangular solve
        ZG_CUDA(cudaEventRecord(la.upd[b % R], sp));
        ZG_CUDA(cudaStreamWaitEvent(sb, la.upd[b % R], 0));
        ZG_TRY(dgemm_oz_sub(rest - near, rest - near, jb, A21 + near, lda, nullptr, 0,
                            A21 + near + (long)(jb + near) * lda, lda, true, &ctl->status, sb));
      }
    }
    ZG_CUDA(cudaEventRecord(la.bulk_done[b % R], sb));
  }
  return 0;
}

int potrf_oz(int n, double *A, long lda, int *info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  Lookahead *la;
  ZG_TRY(lookahead(s, &la));
  ZG_CUDA(cudaEventRecord(la->first, s));
  ZG_CUDA(cudaStreamWaitEvent(la->panel, la->first, 0));
  ZG_CUDA(cudaStreamWaitEvent(la->bulk, la->first, 0));
  const int rc = potrf_oz_blocks(n, A, lda, ctl, *la);
  ZG_CUDA(cudaEventRecord(la->end_panel, la->panel));
  ZG_CUDA(cudaEventRecord(la->end_bulk, la->bulk));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_panel, 0));
  ZG_CUDA(cudaStreamWaitEvent(s, la->end_bulk, 0));
  if (rc != 0) return rc;
  return check_status(s, ctl, info);
}

}  // namespace zg
