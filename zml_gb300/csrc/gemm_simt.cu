// gemm_simt.cu -- FP64 / FP32 GEMM and SYRK on the CUDA cores.
//
// Replaces the loop nests of zml's blas/gemm.zig:68-1027 and
// blas/syrk.zig:60-366 for the column-major kernels every LAPACK routine on
// the path calls (getrf.zig:125 trailing update, potrf.zig:150/197, larfb).
// tcgen05 has no f64 kind, so FP64 runs here on DFMA: a 64x64 CTA tile,
// 256 threads, 4x4 register micro-tiles, operands staged through shared
// memory in the canonical [k][m] / [k][n] layout for any transpose.
//
// tri selects the SYRK form: 0 = full C, 1 = lower triangle (i >= j),
// 2 = upper triangle (i <= j); tiles outside the triangle are skipped.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace zg {

// gridDim.z > 1 splits K: CTA z covers l in [z*kchunk, (z+1)*kchunk) and
// writes its partial product to C + z*cz (beta ignored, partials reduced by
// splitk_reduce_kernel).
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_simt_kernel(int transa, int transb, int m, int n, int k,
                                                        T alpha, const T *__restrict__ A, long lda,
                                                        const T *__restrict__ B, long ldb, T beta,
                                                        T *__restrict__ C, long ldc, int tri,
                                                        int kchunk, long cz) {
  const int i0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
  const int kbeg = blockIdx.z * kchunk, kend = min(k, kbeg + kchunk);
  C += blockIdx.z * cz;
  if (tri == 1 && i0 + BM - 1 < j0) return;  // tile strictly above the diagonal
  if (tri == 2 && j0 + BN - 1 < i0) return;  // tile strictly below the diagonal

  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;  // 16 x 16 threads, each 4 x 4
  T acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0;

  const bool ta = transa == kTrans || transa == kConjTrans;
  const bool tb = transb == kTrans || transb == kConjTrans;

  for (int l0 = kbeg; l0 < kend; l0 += BK) {
    // A tile: op(A)(i, l) for i in [i0, i0+BM), l in [l0, l0+BK)
    for (int e = tid; e < BM * BK; e += 256) {
      int ii, ll;
      if (!ta) { ii = e % BM; ll = e / BM; }   // contiguous along i
      else     { ll = e % BK; ii = e / BK; }   // contiguous along l
      const int gi = i0 + ii, gl = l0 + ll;
      T v = 0;
      if (gi < m && gl < kend) v = ta ? A[gl + (long)gi * lda] : A[gi + (long)gl * lda];
      As[ll][ii] = v;
    }
    // B tile: op(B)(l, j)
    for (int e = tid; e < BN * BK; e += 256) {
      int jj, ll;
      if (!tb) { ll = e % BK; jj = e / BK; }   // contiguous along l
      else     { jj = e % BN; ll = e / BN; }   // contiguous along j
      const int gj = j0 + jj, gl = l0 + ll;
      T v = 0;
      if (gj < n && gl < kend) v = tb ? B[gj + (long)gl * ldb] : B[gl + (long)gj * ldb];
      Bs[ll][jj] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < BK; ++ll) {
      T a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[ll][tx + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[ll][ty + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = j0 + ty + 16 * c;
    if (j >= n) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = i0 + tx + 16 * r;
      if (i >= m) continue;
      if (tri == 1 && i < j) continue;
      if (tri == 2 && i > j) continue;
      T *p = C + i + (long)j * ldc;
      if (gridDim.z > 1) *p = acc[r][c];
      else *p = beta == T(0) ? alpha * acc[r][c] : alpha * acc[r][c] + beta * *p;
    }
  }
}

template <typename T>
int gemm_simt(int transa, int transb, int m, int n, int k, T alpha, const T *A, long lda,
              const T *B, long ldb, T beta, T *C, long ldc, int tri, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  if ((alpha == T(0) || k == 0) && beta == T(1)) return 0;
  if (alpha == T(0)) k = 0;
  constexpr int BM = 64, BN = 64, BK = 16;
  dim3 grid(ceil_div(m, BM), ceil_div(n, BN));
  if (grid.y > 65535) {
    set_last_error("gemm: n too large for the grid");
    return kErrInvalid;
  }
  ZG_LAUNCH(kTagGemmSimt, 2.0 * m * n * k, sizeof(T) * ((double)m * k + (double)k * n + 2.0 * m * n), s, gemm_simt_kernel<T, BM, BN, BK><<<grid, 256, 0, s>>>(transa, transb, m, n, k, alpha, A, lda, B,
                                                       ldb, beta, C, ldc, tri, k, 0));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

// C = alpha * sum_z P_z + beta * C over `splits` partials P_z (m x n, ld m).
template <typename T>
__global__ void splitk_reduce_kernel(int m, int n, int splits, const T *__restrict__ P, T alpha,
                                     T beta, T *__restrict__ C, long ldc) {
  const long total = (long)m * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % m, j = e / m;
    T acc = 0;
    for (int z = 0; z < splits; ++z) acc += P[(long)z * total + e];
    T *p = C + i + (long)j * ldc;
    *p = beta == T(0) ? alpha * acc : alpha * acc + beta * *p;
  }
}

// GEMM with K split over `splits` CTA layers (for short-and-wide outputs with
// a long K, e.g. W = V^T C of the block reflector); work: splits*m*n scratch.
template <typename T>
int gemm_simt_splitk(int transa, int transb, int m, int n, int k, T alpha, const T *A, long lda,
                     const T *B, long ldb, T beta, T *C, long ldc, int splits, T *work,
                     cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  if (splits <= 1 || k <= 0) return gemm_simt<T>(transa, transb, m, n, k, alpha, A, lda, B, ldb,
                                                 beta, C, ldc, 0, s);
  constexpr int BM = 64, BN = 64, BK = 16;
  const int kchunk = ((ceil_div(k, splits) + BK - 1) / BK) * BK;
  splits = ceil_div(k, kchunk);
  dim3 grid(ceil_div(m, BM), ceil_div(n, BN), splits);
  ZG_LAUNCH(kTagGemmSimt, 2.0 * m * n * k, sizeof(T) * ((double)m * k + (double)k * n + 2.0 * m * n * splits), s,
            gemm_simt_kernel<T, BM, BN, BK><<<grid, 256, 0, s>>>(transa, transb, m, n, k, T(1), A,
                                                                 lda, B, ldb, T(0), work, m, 0,
                                                                 kchunk, (long)m * n));
  const long total = (long)m * n;
  ZG_LAUNCH(kTagGemmSimt, 0, sizeof(T) * total * (splits + 2), s,
            splitk_reduce_kernel<T><<<(int)std::min<long>((total + 255) / 256, 152L * 8), 256, 0,
                                      s>>>(m, n, splits, work, alpha, beta, C, ldc));
  return 0;
}
template int gemm_simt_splitk<double>(int, int, int, int, int, double, const double *, long,
                                      const double *, long, double, double *, long, int, double *,
                                      cudaStream_t);
template int gemm_simt_splitk<float>(int, int, int, int, int, float, const float *, long,
                                     const float *, long, float, float *, long, int, float *,
                                     cudaStream_t);

template int gemm_simt<double>(int, int, int, int, int, double, const double *, long,
                               const double *, long, double, double *, long, int, cudaStream_t);
template int gemm_simt<float>(int, int, int, int, int, float, const float *, long, const float *,
                              long, float, float *, long, int, cudaStream_t);

// SYRK: C <- alpha op(A) op(A)^T + beta C on one triangle (blas/syrk.zig).
template <typename T>
int syrk_dev(int uplo, int trans, int n, int k, T alpha, const T *A, long lda, T beta, T *C,
             long ldc, cudaStream_t s) {
  const bool nt = trans == kNoTrans;
  return gemm_simt<T>(nt ? kNoTrans : kTrans, nt ? kTrans : kNoTrans, n, n, k, alpha, A, lda, A,
                      lda, beta, C, ldc, uplo == kLower ? 1 : 2, s);
}
template int syrk_dev<double>(int, int, int, int, double, const double *, long, double, double *,
                              long, cudaStream_t);
template int syrk_dev<float>(int, int, int, int, float, const float *, long, float, float *, long,
                             cudaStream_t);

}  // namespace zg
