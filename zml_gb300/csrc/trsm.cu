// trsm.cu -- triangular solves with many right-hand sides.
//
// Replaces zml's blas/trsm.zig:66-735 (all eight side/uplo/trans branches,
// unit and non-unit diagonals) as used by getrf.zig:107, getrs.zig:55/72,
// potrf.zig:215 and potrs.zig:78/95.  Blocked: a 64 x 64 diagonal block of
// op(A) is solved in shared memory by one kernel (forward or backward
// substitution, one column of B per lane group), and the rest of B is
// updated by GEMM.  Right-side solves run the same substitution on B^T.
// Like the reference, the left-side non-unit step divides by a(k,k) and the
// right-side step multiplies by its reciprocal (trsm.zig:137 vs 459-484).
#include "common.cuh"
#include "kernels.h"

namespace zg {

constexpr int kTrsmNB = 64;  // diagonal block
constexpr int kTrsmNC = 32;  // right-hand sides per CTA

// Solves op(Ad) X = Bblk for one nbk x nbk diagonal block.
//   lower: forward substitution, else backward.
//   right: the block is B^T (rows of B are the right-hand sides), the
//          effective matrix is op(A)^T and the pivot is applied as a
//          reciprocal product.
template <typename T>
__global__ void __launch_bounds__(256) trsm_diag_kernel(int nbk, int nrhs, const T *__restrict__ A,
                                                        long lda, bool transA, bool right,
                                                        bool lower_eff, bool unit, T *B, long ldb) {
  __shared__ T As[kTrsmNB][kTrsmNB + 1];  // As[i][k] = effective matrix (i, k)
  __shared__ T Bs[kTrsmNB][kTrsmNC + 1];  // Bs[k][c]
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * kTrsmNC;
  const int nc = min(kTrsmNC, nrhs - c0);
  // effective(i,k) = op(A)(i,k) for left, op(A)(k,i) for right; with
  // op(A)(i,k) = transA ? A(k,i) : A(i,k).
  const bool flip = transA != right;  // effective(i,k) = flip ? A(k,i) : A(i,k)
  for (int e = tid; e < nbk * nbk; e += 256) {
    int i = e % nbk, k = e / nbk;  // A(i,k) read contiguous along i
    T v = A[i + (long)k * lda];
    if (flip) As[k][i] = v; else As[i][k] = v;
  }
  for (int e = tid; e < nbk * nc; e += 256) {
    int k, c;
    if (!right) { k = e % nbk; c = e / nbk; Bs[k][c] = B[k + (long)(c0 + c) * ldb]; }
    else        { c = e % nc; k = e / nc; Bs[k][c] = B[(c0 + c) + (long)k * ldb]; }
  }
  __syncthreads();
  for (int s = 0; s < nbk; ++s) {
    const int k = lower_eff ? s : nbk - 1 - s;
    if (!unit) {
      const T d = As[k][k];
      const T r = right ? T(1) / d : T(0);
      for (int c = tid; c < nc; c += 256) Bs[k][c] = right ? Bs[k][c] * r : Bs[k][c] / d;
      __syncthreads();
    }
    const int lo = lower_eff ? k + 1 : 0, hi = lower_eff ? nbk : k;
    const int cnt = (hi - lo) * nc;
    for (int e = tid; e < cnt; e += 256) {
      const int i = lo + e % (hi - lo), c = e / (hi - lo);
      Bs[i][c] -= As[i][k] * Bs[k][c];
    }
    __syncthreads();
  }
  for (int e = tid; e < nbk * nc; e += 256) {
    int k, c;
    if (!right) { k = e % nbk; c = e / nbk; B[k + (long)(c0 + c) * ldb] = Bs[k][c]; }
    else        { c = e % nc; k = e / nc; B[(c0 + c) + (long)k * ldb] = Bs[k][c]; }
  }
}

template <typename T>
__global__ void scale_kernel(int m, int n, T alpha, T *B, long ldb) {
  long total = (long)m * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    T *p = B + i + (long)j * ldb;
    *p = alpha == T(0) ? T(0) : *p * alpha;
  }
}

template <typename T> int scale_dev(int m, int n, T alpha, T *B, long ldb, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  long total = (long)m * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  ZG_LAUNCH(kTagVector, 0, 0, s, scale_kernel<T><<<blocks, 256, 0, s>>>(m, n, alpha, B, ldb));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
__global__ void transpose_kernel(int rows, int cols, const T *src, long lds, T *dst, long ldd) {
  __shared__ T tile[32][33];
  int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    int r = r0 + threadIdx.x, c = c0 + k;
    if (r < rows && c < cols) tile[k][threadIdx.x] = src[r + (long)c * lds];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    int c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) dst[c + (long)r * ldd] = tile[threadIdx.x][k];
  }
}

// dst (cols x rows) = src (rows x cols)^T, both column-major.
template <typename T>
int transpose_dev(int rows, int cols, const T *src, long lds, T *dst, long ldd, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return 0;
  dim3 grid(ceil_div(rows, 32), ceil_div(cols, 32)), block(32, 8);
  ZG_LAUNCH(kTagConvert, 0, 0, s, transpose_kernel<T><<<grid, block, 0, s>>>(rows, cols, src, lds, dst, ldd));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// Left diagonal-block solve for at most 8 right-hand sides: one warp per
// column of B, lane l holding rows l and l + 32 in registers; x_k goes to
// every lane by shuffle, so a step needs no block barrier.  The arithmetic
// per element is that of trsm_diag_kernel (divide by a(k,k), then
// b_i -= a(i,k) x_k in step order).
template <typename T>
__global__ void __launch_bounds__(256) trsm_diag_few_kernel(int nbk, int nrhs,
                                                            const T *__restrict__ A, long lda,
                                                            bool transA, bool lower_eff, bool unit,
                                                            T *B, long ldb) {
  __shared__ T As[kTrsmNB][kTrsmNB + 1];  // As[i][k] = op(A)(i, k)
  for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) {
    const int i = e % nbk, k = e / nbk;
    const T v = A[i + (long)k * lda];
    if (transA) As[k][i] = v; else As[i][k] = v;
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w >= nrhs) return;
  T *b = B + (long)w * ldb;
  const int i0 = lane, i1 = lane + 32;
  T x0 = i0 < nbk ? b[i0] : T(0), x1 = i1 < nbk ? b[i1] : T(0);
  for (int s = 0; s < nbk; ++s) {
    const int k = lower_eff ? s : nbk - 1 - s;
    const T v0 = __shfl_sync(0xffffffffu, x0, k & 31), v1 = __shfl_sync(0xffffffffu, x1, k & 31);
    T xk = k < 32 ? v0 : v1;
    if (!unit) {
      xk = xk / As[k][k];
      if (i0 == k) x0 = xk;
      if (i1 == k) x1 = xk;
    }
    if (i0 < nbk && (lower_eff ? i0 > k : i0 < k)) x0 -= As[i0][k] * xk;
    if (i1 < nbk && (lower_eff ? i1 > k : i1 < k)) x1 -= As[i1][k] * xk;
  }
  if (i0 < nbk) b[i0] = x0;
  if (i1 < nbk) b[i1] = x1;
}

constexpr int kFewRhsMax = 8;  // trsm_diag_few_kernel: one warp per right-hand side


template <typename T>
static int diag_solve(int nbk, int nrhs, const T *A, long lda, bool transA, bool right,
                      bool lower_eff, bool unit, T *B, long ldb, cudaStream_t s) {
  if (nbk <= 0 || nrhs <= 0) return 0;
  if (!right && nrhs <= kFewRhsMax) {
    ZG_LAUNCH(kTagTrsmDiag, 1.0 * nbk * nbk * nrhs, sizeof(T) * (1.0 * nbk * nbk + 2.0 * nbk * nrhs),
              s, trsm_diag_few_kernel<T><<<1, 256, 0, s>>>(nbk, nrhs, A, lda, transA, lower_eff,
                                                           unit, B, ldb));
    return 0;
  }
  int grid = ceil_div(nrhs, kTrsmNC);
  ZG_LAUNCH(kTagTrsmDiag, 1.0 * nbk * nbk * nrhs, sizeof(T) * (1.0 * nbk * nbk + 2.0 * nbk * nrhs), s, trsm_diag_kernel<T><<<grid, 256, 0, s>>>(nbk, nrhs, A, lda, transA, right, lower_eff, unit, B,
                                           ldb));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// Block update of a left solve with few right-hand sides (n <= kSkinny):
// C (m x n) -= op(A) (m x k) X (k x n), k <= 64.  A CTA covers 32 rows; its
// 8 warps each take 8 of the k columns (eight loads in flight per thread, a
// warp's loads contiguous along the rows), and the 8 partial sums of each
// row are added in shared memory in a fixed order.  A GEMM tile would spend
// a whole 64 x 64 output tile of FP64 work per column here.
constexpr int kSkinny = 16;
template <typename T>
__global__ void __launch_bounds__(256) skinny_update_kernel(int m, int n, int k, bool tr,
                                                            const T *__restrict__ A, long lda,
                                                            const T *__restrict__ X, long ldx,
                                                            T *__restrict__ C, long ldc) {
  __shared__ T xs[kTrsmNB * kSkinny];          // xs[q * n + j] = X(q, j)
  __shared__ T red[8][32][kSkinny + 1];        // partial sums by k-slice
  for (int e = threadIdx.x; e < k * n; e += blockDim.x) {
    const int q = e % k, j = e / k;
    xs[q * n + j] = X[q + (long)j * ldx];
  }
  __syncthreads();
  const int lr = threadIdx.x & 31, ks = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lr;
  T acc[kSkinny];
#pragma unroll
  for (int j = 0; j < kSkinny; ++j) acc[j] = T(0);
  if (i < m) {
    const int q0 = ks * 8;
    T a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u;
      a[u] = q < k ? (tr ? A[q + (long)i * lda] : A[i + (long)q * lda]) : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u;
      if (q < k)
#pragma unroll
        for (int j = 0; j < kSkinny; ++j)
          if (j < n) acc[j] = fma(a[u], xs[q * n + j], acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < kSkinny; ++j)
    if (j < n) red[ks][lr][j] = acc[j];
  __syncthreads();
  if (ks == 0 && i < m)
    for (int j = 0; j < n; ++j) {
      T sum = red[0][lr][j];
#pragma unroll
      for (int q = 1; q < 8; ++q) sum += red[q][lr][j];
      C[i + (long)j * ldc] -= sum;
    }
}

template <typename T>
static int skinny_update(int m, int n, int k, bool tr, const T *A, long lda, const T *X, long ldx,
                         T *C, long ldc, cudaStream_t s) {
  if (m <= 0) return 0;
  ZG_LAUNCH(kTagGemmSimt, 2.0 * m * n * k, sizeof(T) * ((double)m * k + 2.0 * m * n), s,
            skinny_update_kernel<T><<<ceil_div(m, 32), 256, 0, s>>>(m, n, k, tr, A, lda, X, ldx,
                                                                     C, ldc));
  return 0;
}

template <typename T>
int trsm_dev(int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *A, long lda,
             T *B, long ldb, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  if (alpha == T(0)) return scale_dev<T>(m, n, T(0), B, ldb, s);
  if (alpha != T(1)) ZG_TRY(scale_dev<T>(m, n, alpha, B, ldb, s));
  const bool tr = transa == kTrans || transa == kConjTrans;
  const bool unit = diag == kUnit;
  const int NB = kTrsmNB;
  if (side == kLeft) {
    const bool lower_eff = (uplo == kLower) != tr;  // op(A) lower triangular
    const int nblk = ceil_div(m, NB);
    for (int t = 0; t < nblk; ++t) {
      const int b = lower_eff ? t : nblk - 1 - t;
      const int kb = b * NB, nbk = min(NB, m - kb);
      ZG_TRY(diag_solve<T>(nbk, n, A + kb + (long)kb * lda, lda, tr, false, lower_eff, unit,
                           B + kb, ldb, s));
      if (lower_eff && kb + nbk < m) {  // B[kb+nbk:] -= op(A)[kb+nbk:, kb:kb+nbk] X
        const int rows = m - kb - nbk;
        const T *Ab = tr ? A + kb + (long)(kb + nbk) * lda : A + (kb + nbk) + (long)kb * lda;
        if (n <= kSkinny)
          ZG_TRY(skinny_update<T>(rows, n, nbk, tr, Ab, lda, B + kb, ldb, B + kb + nbk, ldb, s));
        else
          ZG_TRY(gemm_simt<T>(tr ? kTrans : kNoTrans, kNoTrans, rows, n, nbk, T(-1), Ab, lda,
                              B + kb, ldb, T(1), B + kb + nbk, ldb, 0, s));
      } else if (!lower_eff && kb > 0) {  // B[0:kb] -= op(A)[0:kb, kb:kb+nbk] X
        const T *Ab = tr ? A + kb : A + (long)kb * lda;
        if (n <= kSkinny)
          ZG_TRY(skinny_update<T>(kb, n, nbk, tr, Ab, lda, B + kb, ldb, B, ldb, s));
        else
          ZG_TRY(gemm_simt<T>(tr ? kTrans : kNoTrans, kNoTrans, kb, n, nbk, T(-1), Ab, lda, B + kb,
                              ldb, T(1), B, ldb, 0, s));
      }
    }
  } else {
    const bool upper_eff = (uplo == kUpper) != tr;  // op(A) upper: forward over columns
    const int nblk = ceil_div(n, NB);
    for (int t = 0; t < nblk; ++t) {
      const int b = upper_eff ? t : nblk - 1 - t;
      const int kb = b * NB, nbk = min(NB, n - kb);
      // X_b op(A)_bb = B_b  <=>  op(A)_bb^T X_b^T = B_b^T: lower when op(A) upper
      ZG_TRY(diag_solve<T>(nbk, m, A + kb + (long)kb * lda, lda, tr, true, upper_eff, unit,
                           B + (long)kb * ldb, ldb, s));
      if (upper_eff && kb + nbk < n) {  // B[:, kb+nbk:] -= X_b op(A)[kb.., kb+nbk..]
        const int cols = n - kb - nbk;
        const T *Ab = tr ? A + (kb + nbk) + (long)kb * lda : A + kb + (long)(kb + nbk) * lda;
        ZG_TRY(gemm_simt<T>(kNoTrans, tr ? kTrans : kNoTrans, m, cols, nbk, T(-1),
                            B + (long)kb * ldb, ldb, Ab, lda, T(1), B + (long)(kb + nbk) * ldb,
                            ldb, 0, s));
      } else if (!upper_eff && kb > 0) {  // B[:, 0:kb] -= X_b op(A)[kb.., 0:kb]
        const T *Ab = tr ? A + (long)kb * lda : A + kb;
        ZG_TRY(gemm_simt<T>(kNoTrans, tr ? kTrans : kNoTrans, m, kb, nbk, T(-1),
                            B + (long)kb * ldb, ldb, Ab, lda, T(1), B, ldb, 0, s));
      }
    }
  }
  return 0;
}

#define INST(T)                                                                                \
  template int trsm_dev<T>(int, int, int, int, int, int, T, const T *, long, T *, long,        \
                           cudaStream_t);                                                      \
  template int scale_dev<T>(int, int, T, T *, long, cudaStream_t);                             \
  template int transpose_dev<T>(int, int, const T *, long, T *, long, cudaStream_t);
INST(double)
INST(float)
#undef INST
template int transpose_dev<double2>(int, int, const double2 *, long, double2 *, long, cudaStream_t);
template int transpose_dev<float2>(int, int, const float2 *, long, float2 *, long, cudaStream_t);

}  // namespace zg
