// zlapack.cu -- complex triangular solve, LU (getrf, getrs) and Cholesky
// (potrf, potrs) on the GPU, binary64 and binary32 components.
//
// The factorizations keep the reference's own structure: the blocked
// right-looking getrf (nb = 64) whose panels are factored by the recursive
// getrf2, and the blocked left-looking potrf (nb = 64) with the recursive
// potrf2 on its diagonal blocks (lapack/getrf.zig, getrf2.zig, potrf.zig,
// potrf2.zig).  Everything of level 3 inside them -- the trailing updates,
// the triangular solves' off-diagonal blocks, the Hermitian rank-k updates --
// runs as real GEMMs on the expanded operand (zblas.cu); the kernels here are
// the column pivot of getrf2 (first maximum of |re| + |im|, zml's iamax),
// the 1x1 Cholesky step, and the substitution on 64 x 64 diagonal blocks.
// Complex arithmetic follows zml's cfloat: the fused product
// (cfloat.zig:149-174) and Smith's division (cfloat.zig:206-290).
#include <climits>

#include "common.cuh"
#include "kernels.h"

namespace zg {

template <typename C2, typename R>
__device__ __forceinline__ C2 cmake(R re, R im) {
  C2 z;
  z.x = re;
  z.y = im;
  return z;
}
template <typename C2>
__device__ __forceinline__ C2 cmulz(C2 x, C2 y) {
  return cmake<C2>(fma(x.x, y.x, (-x.y) * y.y), fma(x.x, y.y, x.y * y.x));
}
template <typename C2>
__device__ __forceinline__ C2 csubz(C2 x, C2 y) {
  return cmake<C2>(x.x - y.x, x.y - y.y);
}
template <typename C2>
__device__ __forceinline__ C2 cdivz(C2 x, C2 y) {
  if (fabs(y.y) < fabs(y.x)) {
    const auto t1 = y.y / y.x;
    const auto t2 = decltype(t1)(1) / fma(t1, y.y, y.x);
    return cmake<C2>(fma(x.y, t1, x.x) * t2, fma(-x.x, t1, x.y) * t2);
  }
  const auto t1 = y.x / y.y;
  const auto t2 = decltype(t1)(1) / fma(t1, y.x, y.y);
  return cmake<C2>(fma(x.x, t1, x.y) * t2, fma(x.y, t1, -x.x) * t2);
}

// LAPACK's info: the smallest failing column (1-based) wins.
__device__ __forceinline__ void record_info(int *info, int v) {
  int old = *(volatile int *)info;
  while (old == 0 || v < old) {
    const int prev = atomicCAS(info, old, v);
    if (prev == old) break;
    old = prev;
  }
}

constexpr int kZB = 64;  // diagonal block of the substitution, and nb of getrf / potrf

// op(A)_kk X = B_k for the nb x nb diagonal block of op(A) and all nrhs
// columns of B_k: thread (i, c) holds row i of column 4 blockIdx.x + c;
// per step k the solved x_k is published in shared memory and subtracted
// from the rows still to solve (b_i -= x_k a_ik, trsm.zig:147, 232).
template <typename R, typename C2>
__global__ void __launch_bounds__(256) ctrsm_diag_kernel(int nb, int nrhs, const C2 *A, long lda,
                                                         bool nota, bool cj, bool lower, bool unit,
                                                         C2 *B, long ldb) {
  extern __shared__ __align__(16) unsigned char zsm[];
  C2 *sA = reinterpret_cast<C2 *>(zsm);  // kZB x (kZB + 1): 66.5 KB for binary64
  __shared__ C2 xs[4][kZB];
  const int i = threadIdx.x, c = threadIdx.y, tid = i + kZB * c;
  for (int e = tid; e < nb * nb; e += 256) {
    const int r = e % nb, q = e / nb;
    C2 v = nota ? A[r + (long)q * lda] : A[q + (long)r * lda];
    if (cj) v.y = -v.y;
    sA[r + q * (kZB + 1)] = v;
  }
  const int j = blockIdx.x * 4 + c;
  C2 x = cmake<C2>(R(0), R(0));
  if (i < nb && j < nrhs) x = B[i + (long)j * ldb];
  __syncthreads();
  for (int s = 0; s < nb; ++s) {
    const int k = lower ? s : nb - 1 - s;
    if (i == k) {
      if (!unit) x = cdivz(x, sA[k + k * (kZB + 1)]);
      xs[c][k] = x;
    }
    __syncthreads();
    if (lower ? (i > k && i < nb) : i < k) x = csubz(x, cmulz(xs[c][k], sA[i + k * (kZB + 1)]));
  }
  if (i < nb && j < nrhs) B[i + (long)j * ldb] = x;
}

// getrf2's one-column case (getrf2.zig:41-89): the pivot is the first
// maximum of |re| + |im| (a NaN at the top blocks the search, a NaN below is
// never chosen, as iamax's strict '>' behaves); rows 0 and ii swap in this
// column; the column below is scaled by 1 / a0 when |a0|_1 >= sfmin, else
// divided by a0; a zero pivot records info.
template <typename R, typename C2>
__global__ void __launch_bounds__(1024) zgetf2_col_kernel(int m, C2 *A, int *ipiv, int *info,
                                                          int col, R sfmin) {
  __shared__ R bv[32];
  __shared__ int bi[32];
  __shared__ C2 piv;
  __shared__ int ii_s;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  R best = R(-1);
  int besti = INT_MAX;
  for (int r = t; r < m; r += blockDim.x) {
    const C2 v = A[r];
    const R a = fabs(v.x) + fabs(v.y);
    if (a > best) {  // NaN never
      best = a;
      besti = r;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const R ov = __shfl_down_sync(0xffffffffu, best, off);
    const int oi = __shfl_down_sync(0xffffffffu, besti, off);
    if (ov > best || (ov == best && oi < besti)) {
      best = ov;
      besti = oi;
    }
  }
  if (lane == 0) {
    bv[w] = best;
    bi[w] = besti;
  }
  __syncthreads();
  if (t == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
      if (bv[q] > best || (bv[q] == best && bi[q] < besti)) {
        best = bv[q];
        besti = bi[q];
      }
    const C2 a0 = A[0];
    const R abs0 = fabs(a0.x) + fabs(a0.y);
    int ii = (abs0 != abs0 || besti == INT_MAX) ? 0 : besti;
    ipiv[0] = ii + 1;
    const C2 p = A[ii];
    if (p.x != R(0) || p.y != R(0)) {
      if (ii != 0) {
        A[ii] = a0;
        A[0] = p;
      }
    } else {
      record_info(info, col + 1);
      ii = -1;
    }
    piv = p;
    ii_s = ii;
  }
  __syncthreads();
  if (ii_s < 0) return;
  const C2 p = piv;
  const bool recip = fabs(p.x) + fabs(p.y) >= sfmin;
  // 1 / p as (1 + 0i) / p (test/cfloat/div.zig:42-44), then x * (1 / p)
  const C2 rp = cdivz(cmake<C2>(R(1), R(0)), p);
  for (int r = 1 + t; r < m; r += blockDim.x) A[r] = recip ? cmulz(A[r], rp) : cdivz(A[r], p);
}

// getrf2's one-row case (getrf2.zig:35-40)
template <typename C2>
__global__ void zgetf2_row_kernel(const C2 *A, int *ipiv, int *info, int col) {
  ipiv[0] = 1;
  if (A[0].x == 0 && A[0].y == 0) record_info(info, col + 1);
}

__global__ void ipiv_add_kernel(int *ipiv, int cnt, int add) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    ipiv[i] += add;
}

// potrf2's 1 x 1 case (potrf2.zig:37-54): re(a) must be positive and not a
// NaN; a <- (sqrt(re a), 0)
template <typename R, typename C2>
__global__ void zpotf_base_kernel(C2 *A, int *info, int col) {
  const R ajj = A[0].x;
  if (ajj <= R(0) || ajj != ajj) {
    record_info(info, col + 1);
    return;
  }
  A[0] = cmake<C2>(sqrt(ajj), R(0));
}

template <typename R>
int ztrsm_dev(int side, int uplo, int transa, int diag, int m, int n, const R *alpha, const R *A,
              long lda, R *B, long ldb, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (m <= 0 || n <= 0) return 0;
  const R one[2] = {R(1), R(0)}, mone[2] = {R(-1), R(0)}, zero[2] = {R(0), R(0)};
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  const bool aone = alpha[0] == R(1) && alpha[1] == R(0);
  if (azero)  // B = 0 (trsm.zig:99-113)
    return zgemm_dev<R>(kNoTrans, kNoTrans, m, n, 0, zero, A, lda, A, lda, zero, B, ldb, s);
  if (side == kRight) {
    // X op(A) = alpha B  <=>  op(A)^T X^T = alpha B^T
    void *w;
    ZG_TRY(workspace(s, kSlotZTr, sizeof(C2) * (size_t)m * n, &w));
    C2 *Bt = (C2 *)w;
    ZG_TRY(transpose_dev<C2>(m, n, (const C2 *)B, ldb, Bt, n, s));
    const int ta2 = transa == kNoTrans ? kTrans
                  : transa == kTrans ? kNoTrans
                  : transa == kConjTrans ? kConjNoTrans : kConjTrans;
    ZG_TRY(ztrsm_dev<R>(kLeft, uplo, ta2, diag, n, m, alpha, A, lda, (R *)Bt, n, s));
    return transpose_dev<C2>(n, m, Bt, n, (C2 *)B, ldb, s);
  }
  if (!aone)
    ZG_TRY(zgemm_dev<R>(kNoTrans, kNoTrans, m, n, 0, zero, A, lda, A, lda, alpha, B, ldb, s));
  const bool nota = transa == kNoTrans || transa == kConjNoTrans;
  const bool cj = transa == kConjNoTrans || transa == kConjTrans;
  const bool lower = (uplo == kLower) == nota;  // op(A) lower triangular
  const C2 *Ac = (const C2 *)A;
  C2 *Bc = (C2 *)B;
  const size_t smem = sizeof(C2) * kZB * (kZB + 1);
  ZG_TRY(smem_optin(ctrsm_diag_kernel<R, C2>, (int)smem));
  const int nblk = ceil_div(m, kZB);
  for (int q = 0; q < nblk; ++q) {
    const int b = lower ? q : nblk - 1 - q;
    const int k0 = b * kZB, kb = std::min(kZB, m - k0);
    dim3 grid(ceil_div(n, 4)), block(kZB, 4);
    ZG_LAUNCH(kTagTrsmDiag, 4.0 * kb * kb * n, 16.0 * sizeof(R) * kb * n, s,
              (ctrsm_diag_kernel<R, C2><<<grid, block, smem, s>>>(kb, n, Ac + k0 + (long)k0 * lda,
                                                               lda, nota, cj, lower,
                                                               diag == kUnit, Bc + k0, ldb)));
    // the rows still to solve lose op(A)[rows, block] X_block
    const int r0 = lower ? k0 + kb : 0, rn = lower ? m - k0 - kb : k0;
    if (rn > 0) {
      const C2 *Asub = nota ? Ac + r0 + (long)k0 * lda : Ac + k0 + (long)r0 * lda;
      ZG_TRY(zgemm_dev<R>(transa, kNoTrans, rn, n, kb, mone, (const R *)Asub, lda,
                          (const R *)(Bc + k0), ldb, one, (R *)(Bc + r0), ldb, s));
    }
  }
  return 0;
}

// getrf2 (getrf2.zig:14-210) on the GPU: the same recursion, ipiv relative
// to the block passed in, col the block's first column in the whole matrix
// (for info).
template <typename R>
static int zgetrf2_rec(int m, int n, typename Cx<R>::T *A, long lda, int *ipiv, int col, int *info,
                       cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (m == 0 || n == 0) return 0;
  if (m == 1) {
    ZG_LAUNCH(kTagPanel, 0, 0, s, (zgetf2_row_kernel<C2><<<1, 1, 0, s>>>(A, ipiv, info, col)));
    return 0;
  }
  if (n == 1) {
    const R sfmin = sizeof(R) == 8 ? R(2.2250738585072014e-308) : R(1.17549435e-38f);
    ZG_LAUNCH(kTagPanel, 8.0 * m, 2.0 * sizeof(C2) * m, s,
              (zgetf2_col_kernel<R, C2><<<1, 1024, 0, s>>>(m, A, ipiv, info, col, sfmin)));
    return 0;
  }
  const R one[2] = {R(1), R(0)}, mone[2] = {R(-1), R(0)};
  const int mn = std::min(m, n), n1 = mn / 2, n2 = n - n1;
  ZG_TRY(zgetrf2_rec<R>(m, n1, A, lda, ipiv, col, info, s));
  ZG_TRY(laswp_dev<C2>(n2, A + (long)n1 * lda, lda, 1, n1, ipiv, 1, s));
  ZG_TRY(ztrsm_dev<R>(kLeft, kLower, kNoTrans, kUnit, n1, n2, one, (const R *)A, lda,
                      (R *)(A + (long)n1 * lda), lda, s));
  ZG_TRY(zgemm_dev<R>(kNoTrans, kNoTrans, m - n1, n2, n1, mone, (const R *)(A + n1), lda,
                      (const R *)(A + (long)n1 * lda), lda, one, (R *)(A + n1 + (long)n1 * lda),
                      lda, s));
  ZG_TRY(zgetrf2_rec<R>(m - n1, n2, A + n1 + (long)n1 * lda, lda, ipiv + n1, col + n1, info, s));
  ZG_LAUNCH(kTagPanel, 0, 0, s, (ipiv_add_kernel<<<1, 256, 0, s>>>(ipiv + n1, mn - n1, n1)));
  ZG_TRY(laswp_dev<C2>(n1, A, lda, n1 + 1, mn, ipiv, 1, s));
  return 0;
}

// getrf (getrf.zig:14-152): blocked right-looking, nb = 64, getrf2 panels.
template <typename R>
int zgetrf_dev(int m, int n, R *Ar, long lda, int *ipiv, int *info, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  *info = 0;
  if (m <= 0 || n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  C2 *A = (C2 *)Ar;
  const R one[2] = {R(1), R(0)}, mone[2] = {R(-1), R(0)};
  const int mn = std::min(m, n);
  if (kZB >= mn) {
    ZG_TRY(zgetrf2_rec<R>(m, n, A, lda, ipiv, 0, &ctl->info, s));
    return check_status(s, ctl, info);
  }
  for (int j = 0; j < mn; j += kZB) {
    const int jb = std::min(mn - j, kZB);
    C2 *Ajj = A + j + (long)j * lda;
    ZG_TRY(zgetrf2_rec<R>(m - j, jb, Ajj, lda, ipiv + j, j, &ctl->info, s));
    ZG_LAUNCH(kTagPanel, 0, 0, s,
              (ipiv_add_kernel<<<1, 256, 0, s>>>(ipiv + j, std::min(m, j + jb) - j, j)));
    ZG_TRY(laswp_dev<C2>(j, A, lda, j + 1, j + jb, ipiv, 1, s));
    if (j + jb < n) {
      ZG_TRY(laswp_dev<C2>(n - j - jb, A + (long)(j + jb) * lda, lda, j + 1, j + jb, ipiv, 1, s));
      ZG_TRY(ztrsm_dev<R>(kLeft, kLower, kNoTrans, kUnit, jb, n - j - jb, one, (const R *)Ajj, lda,
                          (R *)(A + j + (long)(j + jb) * lda), lda, s));
      if (j + jb < m)
        ZG_TRY(zgemm_dev<R>(kNoTrans, kNoTrans, m - j - jb, n - j - jb, jb, mone,
                            (const R *)(A + j + jb + (long)j * lda), lda,
                            (const R *)(A + j + (long)(j + jb) * lda), lda, one,
                            (R *)(A + j + jb + (long)(j + jb) * lda), lda, s));
    }
  }
  return check_status(s, ctl, info);
}

// getrs (getrs.zig:13-142)
template <typename R>
int zgetrs_dev(int trans, int n, int nrhs, const R *A, long lda, const int *ipiv, R *B, long ldb,
               cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (n <= 0 || nrhs <= 0) return 0;
  const R one[2] = {R(1), R(0)};
  const bool nt = trans == kNoTrans || trans == kConjNoTrans;
  if (nt) {
    ZG_TRY(laswp_dev<C2>(nrhs, (C2 *)B, ldb, 1, n, ipiv, 1, s));
    ZG_TRY(ztrsm_dev<R>(kLeft, kLower, trans, kUnit, n, nrhs, one, A, lda, B, ldb, s));
    ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, trans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
  } else {
    ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, trans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
    ZG_TRY(ztrsm_dev<R>(kLeft, kLower, trans, kUnit, n, nrhs, one, A, lda, B, ldb, s));
    ZG_TRY(laswp_dev<C2>(nrhs, (C2 *)B, ldb, 1, n, ipiv, -1, s));
  }
  return 0;
}

// potrf2 (potrf2.zig:17-217) on the GPU: after a failure the later steps
// still run (their results are unspecified) and info keeps the first.
template <typename R>
static int zpotrf2_rec(int uplo, int n, typename Cx<R>::T *A, long lda, int col, int *info,
                       cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (n == 0) return 0;
  if (n == 1) {
    ZG_LAUNCH(kTagPotf2, 0, 0, s, (zpotf_base_kernel<R, C2><<<1, 1, 0, s>>>(A, info, col)));
    return 0;
  }
  const R one[2] = {R(1), R(0)}, mone[2] = {R(-1), R(0)};
  const int n1 = n / 2, n2 = n - n1;
  ZG_TRY(zpotrf2_rec<R>(uplo, n1, A, lda, col, info, s));
  C2 *A22 = A + n1 + (long)n1 * lda;
  if (uplo == kUpper) {
    C2 *A12 = A + (long)n1 * lda;
    ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, kConjTrans, kNonUnit, n1, n2, one, (const R *)A, lda,
                        (R *)A12, lda, s));
    ZG_TRY(zsyherk_dev<R>(true, kUpper, kConjTrans, n2, n1, mone, (const R *)A12, lda, one,
                          (R *)A22, lda, s));
  } else {
    C2 *A21 = A + n1;
    ZG_TRY(ztrsm_dev<R>(kRight, kLower, kConjTrans, kNonUnit, n2, n1, one, (const R *)A, lda,
                        (R *)A21, lda, s));
    ZG_TRY(zsyherk_dev<R>(true, kLower, kNoTrans, n2, n1, mone, (const R *)A21, lda, one,
                          (R *)A22, lda, s));
  }
  return zpotrf2_rec<R>(uplo, n2, A22, lda, col + n1, info, s);
}

// potrf (potrf.zig:17-240): blocked left-looking, nb = 64.
template <typename R> int zpotrf_dev(int uplo, int n, R *Ar, long lda, int *info, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  *info = 0;
  if (n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  C2 *A = (C2 *)Ar;
  const R one[2] = {R(1), R(0)}, mone[2] = {R(-1), R(0)};
  if (kZB >= n) {
    ZG_TRY(zpotrf2_rec<R>(uplo, n, A, lda, 0, &ctl->info, s));
    return check_status(s, ctl, info);
  }
  for (int j = 0; j < n; j += kZB) {
    const int jb = std::min(kZB, n - j);
    C2 *Ajj = A + j + (long)j * lda;
    if (uplo == kUpper) {
      ZG_TRY(zsyherk_dev<R>(true, kUpper, kConjTrans, jb, j, mone, (const R *)(A + (long)j * lda),
                            lda, one, (R *)Ajj, lda, s));
      ZG_TRY(zpotrf2_rec<R>(kUpper, jb, Ajj, lda, j, &ctl->info, s));
      if (j + jb < n) {
        ZG_TRY(zgemm_dev<R>(kConjTrans, kNoTrans, jb, n - j - jb, j, mone,
                            (const R *)(A + (long)j * lda), lda,
                            (const R *)(A + (long)(j + jb) * lda), lda, one,
                            (R *)(A + j + (long)(j + jb) * lda), lda, s));
        ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, kConjTrans, kNonUnit, jb, n - j - jb, one,
                            (const R *)Ajj, lda, (R *)(A + j + (long)(j + jb) * lda), lda, s));
      }
    } else {
      ZG_TRY(zsyherk_dev<R>(true, kLower, kNoTrans, jb, j, mone, (const R *)(A + j), lda, one,
                            (R *)Ajj, lda, s));
      ZG_TRY(zpotrf2_rec<R>(kLower, jb, Ajj, lda, j, &ctl->info, s));
      if (j + jb < n) {
        ZG_TRY(zgemm_dev<R>(kNoTrans, kConjTrans, n - j - jb, jb, j, mone,
                            (const R *)(A + j + jb), lda, (const R *)(A + j), lda, one,
                            (R *)(A + j + jb + (long)j * lda), lda, s));
        ZG_TRY(ztrsm_dev<R>(kRight, kLower, kConjTrans, kNonUnit, n - j - jb, jb, one,
                            (const R *)Ajj, lda, (R *)(A + j + jb + (long)j * lda), lda, s));
      }
    }
  }
  return check_status(s, ctl, info);
}

// potrs (potrs.zig:15-117)
template <typename R>
int zpotrs_dev(int uplo, int n, int nrhs, const R *A, long lda, R *B, long ldb, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  const R one[2] = {R(1), R(0)};
  if (uplo == kUpper) {
    ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, kConjTrans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
    ZG_TRY(ztrsm_dev<R>(kLeft, kUpper, kNoTrans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
  } else {
    ZG_TRY(ztrsm_dev<R>(kLeft, kLower, kNoTrans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
    ZG_TRY(ztrsm_dev<R>(kLeft, kLower, kConjTrans, kNonUnit, n, nrhs, one, A, lda, B, ldb, s));
  }
  return 0;
}

#define ZINST(R)                                                                                \
  template int ztrsm_dev<R>(int, int, int, int, int, int, const R *, const R *, long, R *, long, \
                            cudaStream_t);                                                      \
  template int zgetrf_dev<R>(int, int, R *, long, int *, int *, cudaStream_t);                  \
  template int zgetrs_dev<R>(int, int, int, const R *, long, const int *, R *, long,            \
                             cudaStream_t);                                                     \
  template int zpotrf_dev<R>(int, int, R *, long, int *, cudaStream_t);                         \
  template int zpotrs_dev<R>(int, int, int, const R *, long, R *, long, cudaStream_t);
ZINST(double)
ZINST(float)
#undef ZINST

}  // namespace zg
