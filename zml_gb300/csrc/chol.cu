// chol.cu -- Cholesky factorization and solve: potrf / potrs on the GPU.
//
// Replaces zml's lapack/potrf.zig:17-240, potrf2.zig:17-217 and
// potrs.zig:15-117.  The reference is left-looking (Crout: syrk into the
// diagonal block, gemm into the block column, trsm); on the GPU the same
// factorization runs right-looking so each step's trailing SYRK is one large
// launch: factor the nb x nb diagonal block in shared memory, TRSM the block
// column, SYRK-update the trailing triangle.  A non-positive or NaN pivot
// records info = (1-based column) exactly as potrf2.zig:37-47; the first one
// wins.  Entries updated after that column are unspecified, as in LAPACK.
#include "common.cuh"
#include "kernels.h"

namespace zg {

constexpr int kCholNB = 64;

// Unblocked Cholesky of one nb x nb diagonal block held in shared memory.
// lower: A = L L^T (column k: sqrt, reciprocal scale, rank-1 update of the
// trailing triangle); upper works on the transpose.
template <typename T>
__global__ void __launch_bounds__(256) potf2_kernel(int nb, T *A, long lda, bool lower,
                                                    Control *ctl, int info_base) {
  __shared__ T S[kCholNB][kCholNB + 1];  // S[i][j] = L(i, j), i >= j
  __shared__ int failed;
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    int i = e % nb, j = e / nb;
    T v = A[i + (long)j * lda];
    if (lower) { if (i >= j) S[i][j] = v; }
    else { if (i <= j) S[j][i] = v; }  // U(i,j) = L(j,i)
  }
  if (tid == 0) failed = 0;
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    const T ajj = S[k][k];
    if (!(ajj > T(0))) {  // <= 0 or NaN
      if (tid == 0) {
        failed = 1;
        atomicCAS(&ctl->info, 0, info_base + k + 1);
      }
      __syncthreads();
      break;
    }
    const T d = sqrt(ajj);
    const T r = T(1) / d;
    __syncthreads();
    if (tid == 0) S[k][k] = d;
    for (int i = k + 1 + tid; i < nb; i += blockDim.x) S[i][k] *= r;
    __syncthreads();
    const int n2 = nb - k - 1;
    for (int e = tid; e < n2 * n2; e += blockDim.x) {
      const int i = k + 1 + e % n2, j = k + 1 + e / n2;
      if (i >= j) S[i][j] -= S[i][k] * S[j][k];
    }
    __syncthreads();
  }
  (void)failed;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    int i = e % nb, j = e / nb;
    if (lower) { if (i >= j) A[i + (long)j * lda] = S[i][j]; }
    else { if (i <= j) A[i + (long)j * lda] = S[j][i]; }
  }
}

// The blocked loop alone (no control block, no host sync): the first
// non-positive pivot lands in ctl->info (1-based + info_base).
template <typename T>
int potrf_launch(int uplo, int n, T *A, long lda, Control *ctl, int info_base, cudaStream_t s) {
  const bool lower = uplo == kLower;
  const int nb = kCholNB;
  for (int j = 0; j < n; j += nb) {
    const int jb = min(nb, n - j);
    T *Ajj = A + j + (long)j * lda;
    ZG_LAUNCH(kTagPotf2, jb * jb * jb / 3.0, 2.0 * sizeof(T) * jb * jb, s,
              potf2_kernel<T><<<1, 256, 0, s>>>(jb, Ajj, lda, lower, ctl, info_base + j));
    const int rest = n - j - jb;
    if (rest <= 0) break;
    if (lower) {
      T *A21 = Ajj + jb;
      ZG_TRY(trsm_dev<T>(kRight, kLower, kTrans, kNonUnit, rest, jb, T(1), Ajj, lda, A21, lda, s));
      ZG_TRY(syrk_dev<T>(kLower, kNoTrans, rest, jb, T(-1), A21, lda, T(1), A21 + (long)jb * lda,
                         lda, s));
    } else {
      T *A12 = Ajj + (long)jb * lda;
      ZG_TRY(trsm_dev<T>(kLeft, kUpper, kTrans, kNonUnit, jb, rest, T(1), Ajj, lda, A12, lda, s));
      ZG_TRY(syrk_dev<T>(kUpper, kTrans, rest, jb, T(-1), A12, lda, T(1), A12 + jb, lda, s));
    }
  }
  return 0;
}

template <typename T> int potrf_dev(int uplo, int n, T *A, long lda, int *info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return 0;
  // from n = 2048 up the FP64 lower Cholesky takes its trailing SYRKs on the
  // tensor cores (exact slices, ozaki.cu); the upper form and smaller sizes
  // stay on the FP64 pipe
  if constexpr (sizeof(T) == sizeof(double))
    if (uplo == kLower && fp64_updates_on_tensor_cores(n, n))
      return potrf_oz(n, reinterpret_cast<double *>(A), lda, info, s);
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  ZG_TRY(potrf_launch<T>(uplo, n, A, lda, ctl, 0, s));
  return check_status(s, ctl, info);
}

template <typename T>
int potrs_dev(int uplo, int n, int nrhs, const T *A, long lda, T *B, long ldb, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  if constexpr (sizeof(T) == sizeof(double)) {
    // a few right-hand sides: one launch per column and triangle
    if (nrhs <= kTrsvMaxRhs && n >= kTrsvMinN) {
      void *w;
      ZG_TRY(workspace(s, kSlotPanel, sizeof(double) * ((size_t)n + 1), &w));
      double *xw = (double *)w;
      const double *Ad = reinterpret_cast<const double *>(A);
      const bool up = uplo == kUpper;  // A = U^T U, else A = L L^T
      Control *ctl;  // one status word for every solve of the call
      ZG_TRY(control(s, &ctl));
      for (int c = 0; c < nrhs; ++c) {
        double *x = reinterpret_cast<double *>(B) + (long)c * ldb;
        ZG_TRY(trsv_f64(n, Ad, lda, up, false, false, x, x, xw, ctl, s));
        ZG_TRY(trsv_f64(n, Ad, lda, !up, true, false, x, x, xw, ctl, s));
      }
      return check_status(s, ctl, nullptr);  // a poll that ran out: kErrTimeout
    }
  }
  if (uplo == kUpper) {
    ZG_TRY(trsm_dev<T>(kLeft, kUpper, kTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
    ZG_TRY(trsm_dev<T>(kLeft, kUpper, kNoTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
  } else {
    ZG_TRY(trsm_dev<T>(kLeft, kLower, kNoTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
    ZG_TRY(trsm_dev<T>(kLeft, kLower, kTrans, kNonUnit, n, nrhs, T(1), A, lda, B, ldb, s));
  }
  return 0;
}

#define INST(T)                                                                       \
  template int potrf_launch<T>(int, int, T *, long, Control *, int, cudaStream_t);   \
  template int potrf_dev<T>(int, int, T *, long, int *, cudaStream_t);                \
  template int potrs_dev<T>(int, int, int, const T *, long, T *, long, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace zg
