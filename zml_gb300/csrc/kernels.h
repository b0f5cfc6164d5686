// kernels.h -- internal (C++) launchers shared between the kernel files and
// the C ABI.  All pointers are device pointers; matrices are column-major.
#pragma once
#include "common.cuh"

namespace zg {

// gemm_simt.cu -- C <- alpha op(A) op(B) + beta C on CUDA cores; tri: 0 full,
// 1 lower, 2 upper triangle of C (SYRK).
template <typename T>
int gemm_simt(int transa, int transb, int m, int n, int k, T alpha, const T *A, long lda,
              const T *B, long ldb, T beta, T *C, long ldc, int tri, cudaStream_t s);
template <typename T>
int syrk_dev(int uplo, int trans, int n, int k, T alpha, const T *A, long lda, T beta, T *C,
             long ldc, cudaStream_t s);
// K split over `splits` CTA layers, partials in work (splits*m*n), then reduced.
template <typename T>
int gemm_simt_splitk(int transa, int transb, int m, int n, int k, T alpha, const T *A, long lda,
                     const T *B, long ldb, T beta, T *C, long ldc, int splits, T *work,
                     cudaStream_t s);

// The storage type of a complex number with components R.
template <typename R> struct Cx;
template <> struct Cx<double> { using T = double2; };
template <> struct Cx<float> { using T = float2; };

// zblas.cu -- complex level 3 on the real SIMT GEMM.  Complex matrices are
// interleaved (re, im) pairs of R, leading dimensions in complex elements,
// scalars as {re, im}.  zgemm: C <- alpha op(A) op(B) + beta C, any of the
// four transposes.  zsyherk: the triangle of C <- alpha op(A) op(A)^H + beta C
// (herm; alpha, beta real) or alpha op(A) op(A)^T + beta C, trans kNoTrans
// (A n x k) or kConjTrans / kTrans (A k x n).
template <typename R>
int zgemm_dev(int ta, int tb, int m, int n, int k, const R *alpha, const R *A, long lda,
              const R *B, long ldb, const R *beta, R *C, long ldc, cudaStream_t s);
template <typename R>
int zsyherk_dev(bool herm, int uplo, int trans, int n, int k, const R *alpha, const R *A, long lda,
                const R *beta, R *C, long ldc, cudaStream_t s);

// zlapack.cu -- complex triangular solve, LU and Cholesky (same storage
// conventions; ipiv device, 1-based; info as LAPACK's, read back on the
// stream).  ztrsm_dev: B <- alpha op(A)^-1 B (left) or alpha B op(A)^-1.
template <typename R>
int ztrsm_dev(int side, int uplo, int transa, int diag, int m, int n, const R *alpha, const R *A,
              long lda, R *B, long ldb, cudaStream_t s);
template <typename R> int zgetrf_dev(int m, int n, R *A, long lda, int *ipiv, int *info,
                                     cudaStream_t s);
template <typename R>
int zgetrs_dev(int trans, int n, int nrhs, const R *A, long lda, const int *ipiv, R *B, long ldb,
               cudaStream_t s);
template <typename R> int zpotrf_dev(int uplo, int n, R *A, long lda, int *info, cudaStream_t s);
// zqr.cu: complex Householder QR (interleaved (re, im) pairs, lda in complex
// elements), tau[min(m, n)] complex.
template <typename R> int zgeqrf_dev(int m, int n, R *A, long lda, R *tau, cudaStream_t s);
template <typename R>
int zpotrs_dev(int uplo, int n, int nrhs, const R *A, long lda, R *B, long ldb, cudaStream_t s);

// sytrf.cu -- Bunch-Kaufman A = U D U^T / L D L^T (LAPACK ipiv and info).
template <typename T>
int sytrf_dev(int uplo, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s);
// Hermitian Bunch-Kaufman (hetf2), complex T (double2 / float2)
template <typename T>
int hetrf_dev(int uplo, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s);

// qr.cu -- Householder QR (geqrf) with the T factor of each panel.
template <typename T> int geqrf_dev(int m, int n, T *A, long lda, T *tau, cudaStream_t s);
// The first n columns of Q from geqrf's reflectors (k of them) stored in A.
template <typename T>
int orgqr_dev(int m, int n, int k, T *A, long lda, const T *tau, cudaStream_t s);

// trsm.cu -- B <- alpha op(A)^-1 B (left) or alpha B op(A)^-1 (right).
template <typename T>
int trsm_dev(int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *A, long lda,
             T *B, long ldb, cudaStream_t s);
template <typename T> int scale_dev(int m, int n, T alpha, T *B, long ldb, cudaStream_t s);
template <typename T>
int transpose_dev(int rows, int cols, const T *src, long lds, T *dst, long ldd, cudaStream_t s);

// lu.cu
template <typename T>
int laswp_dev(int n, T *A, long lda, int k1, int k2, const int *ipiv, int incx, cudaStream_t s);
// Sizes the interchange workspace of stream s now (laswp_dev then allocates
// nothing on s).
int laswp_reserve(cudaStream_t s);
// One panel's interchanges (rows k1..k2, forward, 1-based) on the column
// ranges [0, c_left) and [c_right, n), composed once.
template <typename T>
int laswp_panel(int c_left, int c_right, int n, T *A, long lda, int k1, int k2, const int *ipiv,
                cudaStream_t s);
// Partial-pivot LU of the m x nb panel at A (leading dim lda); writes
// ipiv[0..nb) (1-based, relative to the panel's first row, plus ipiv_base)
// and records the first zero pivot (1-based column + info_base) in ctl->info.
template <typename T>
int panel_lu(int m, int nb, T *A, long lda, int *ipiv, int ipiv_base, Control *ctl, int info_base,
             cudaStream_t s);
// The same panel (FP32, m >= nb, nb <= 128, m <= 32768) factored by one
// thread-block cluster; *launched is false when the shape or the device
// leaves it to panel_lu.  The interchanges are also applied to the xl
// columns at XL and the xr columns at XR (leading dim lda, rows aligned with
// the panel's), as laswp would.
// tournament: pivots by tournament (communication-avoiding LU) instead of
// partial pivoting -- one cluster exchange per 32-column sub-panel instead of
// one per column; P A = L U still holds, with different pivots.
int panel_lu_cluster(int m, int nb, float *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool *launched, float *XL = nullptr,
                     int xl = 0, float *XR = nullptr, int xr = 0, bool tournament = false);
// The same for an FP64 panel (partial pivoting only).
int panel_lu_cluster(int m, int nb, double *A, long lda, int *ipiv, int ipiv_base, Control *ctl,
                     int info_base, cudaStream_t s, bool *launched, double *XL = nullptr,
                     int xl = 0, double *XR = nullptr, int xr = 0);
// tournament: FP32 panels by tournament pivoting (see panel_lu_cluster).
// FP64 from n = 2048 up: getrf_oz (tensor-core updates), else getrf_simt.
template <typename T>
int getrf_dev(int m, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s,
              bool tournament = false);
// The blocked LU with every update on the FP32 / FP64 pipe (nb 128 / 64).
template <typename T>
int getrf_simt(int m, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s,
               bool tournament = false);
// ozaki.cu: FP64 C (m x n) -= A (m x k) B (k x n), k <= 256, on the BF16
// tensor cores through exact integer slices of A and B (syrk: C -= A A^T on
// C's lower triangle, B unused); getrf with NB 256 and those updates; the
// switch between FP64-pipe and tensor-core updates.
int dgemm_oz_sub(int m, int n, int k, const double *A, long lda, const double *B, long ldb,
                 double *C, long ldc, bool syrk, unsigned *status, cudaStream_t s);
int getrf_oz(int m, int n, double *A, long lda, int *ipiv, int *info, cudaStream_t s);
int potrf_oz(int n, double *A, long lda, int *info, cudaStream_t s);  // lower
int set_fp64_updates(int mode);                    // returns the previous mode
// Rows per CTA targeted by the cooperative FP64 / FP32 panel (0: spread over
// every SM); returns the previous target; negative restores the default.
constexpr int kPanelRowsDefault = 0;
int set_panel_rows(int rows);
bool fp64_updates_on_tensor_cores(int m, int n);
template <typename T>
int getrs_dev(int trans, int n, int nrhs, const T *A, long lda, const int *ipiv, T *B, long ldb,
              cudaStream_t s);

// chol.cu
template <typename T>
int potrf_launch(int uplo, int n, T *A, long lda, Control *ctl, int info_base, cudaStream_t s);
template <typename T> int potrf_dev(int uplo, int n, T *A, long lda, int *info, cudaStream_t s);
// Triangular solve of one FP64 column in one launch: x = op(A)^-1 rhs, op(A)
// = A or A^T (trans), lower or upper, unit or non-unit diagonal; rhs may be
// x.  xw: n + 1 doubles of device scratch.  A poll that runs out sets a bit
// in ctl->status, which the caller reads with check_status.
int trsv_f64(int n, const double *A, long lda, bool trans, bool upper, bool unit,
             const double *rhs, double *x, double *xw, Control *ctl, cudaStream_t s);
// Y = P B, P the interchanges ipiv (1-based, n of them) applied in increasing
// (forward) or decreasing order; Y must not overlap B.
int perm_gather_f64(int n, int nrhs, const int *ipiv, bool forward, const double *B, long ldb,
                    double *Y, long ldy, cudaStream_t s);
// getrs / potrs take the one-launch solves for up to this many right-hand
// sides from this order on (FP64).
constexpr int kTrsvMaxRhs = 4, kTrsvMinN = 512;

template <typename T>
int potrs_dev(int uplo, int n, int nrhs, const T *A, long lda, T *B, long ldb, cudaStream_t s);

}  // namespace zg
