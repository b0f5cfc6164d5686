/*
 * clapack.h -- dense factor-and-solve of libzml_gb300 (GB300, sm_103a).
 *
 * The reference's include/clapack.h is an empty shell (clapack.h:1-12); the
 * LAPACK C signatures zml itself uses are the LAPACKE ones it calls when
 * built with -Dlink_lapacke (src/linalg/lapack.zig:1169, 1575, 2103, 3012,
 * 3466, 3948, 5121).  This header declares exactly those, so zml's
 * LAPACK dispatch (lapack.zig) can be pointed at this library, plus
 * GPU extensions below.
 *
 * Conventions (LAPACKE): layout is LAPACK_ROW_MAJOR (101) or
 * LAPACK_COL_MAJOR (102); the return value is 0, -(index of the first bad
 * argument), or the positive LAPACK info (first zero pivot for getrf, first
 * non-positive leading minor for potrf).  ipiv is 1-based.  Library failures
 * return codes <= -1000; zml_gpu_last_error() describes them.
 *
 * Pointers may be host memory (staged to the GPU and back) or device /
 * managed memory (used in place).  Calls are synchronous.  Device operands
 * are read after all work queued earlier on the legacy default stream; a
 * caller that fills them on another stream synchronizes that stream first.
 */
#ifndef ZML_GB300_CLAPACK_H
#define ZML_GB300_CLAPACK_H

#ifdef __cplusplus
extern "C" {
#endif

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

#define ZML_GPU_ERR_CUDA (-1001)
#define ZML_GPU_ERR_ALLOC (-1002)
#define ZML_GPU_ERR_NODEVICE (-1003)
#define ZML_GPU_ERR_TIMEOUT (-1004)
#define ZML_GPU_ERR_INVALID (-1005)

/* ---- LAPACKE-shaped drop-ins ------------------------------------------- */
/* replaces zml.linalg.lapack.getrf (lapack.zig:1130; kernel lapack/getrf.zig:14) */
int LAPACKE_dgetrf(int matrix_layout, int m, int n, double *a, int lda, int *ipiv);
int LAPACKE_sgetrf(int matrix_layout, int m, int n, float *a, int lda, int *ipiv);
/* replaces zml.linalg.lapack.getrs (lapack.zig:1517; kernel lapack/getrs.zig:13) */
int LAPACKE_dgetrs(int matrix_layout, char trans, int n, int nrhs, const double *a, int lda,
                   const int *ipiv, double *b, int ldb);
int LAPACKE_sgetrs(int matrix_layout, char trans, int n, int nrhs, const float *a, int lda,
                   const int *ipiv, float *b, int ldb);
/* replaces zml.linalg.lapack.gesv (lapack.zig:2051; kernel lapack/gesv.zig:13) */
int LAPACKE_dgesv(int matrix_layout, int n, int nrhs, double *a, int lda, int *ipiv, double *b,
                  int ldb);
int LAPACKE_sgesv(int matrix_layout, int n, int nrhs, float *a, int lda, int *ipiv, float *b,
                  int ldb);
/* replaces zml.linalg.lapack.potrf (lapack.zig:2975; kernel lapack/potrf.zig:17) */
int LAPACKE_dpotrf(int matrix_layout, char uplo, int n, double *a, int lda);
int LAPACKE_spotrf(int matrix_layout, char uplo, int n, float *a, int lda);
/* replaces zml.linalg.lapack.potrs (lapack.zig:3412; kernel lapack/potrs.zig:15) */
int LAPACKE_dpotrs(int matrix_layout, char uplo, int n, int nrhs, const double *a, int lda,
                   double *b, int ldb);
int LAPACKE_spotrs(int matrix_layout, char uplo, int n, int nrhs, const float *a, int lda,
                   float *b, int ldb);
/* replaces zml.linalg.lapack.posv (lapack.zig:3896; kernel lapack/posv.zig:15) */
int LAPACKE_dposv(int matrix_layout, char uplo, int n, int nrhs, double *a, int lda, double *b,
                  int ldb);
int LAPACKE_sposv(int matrix_layout, char uplo, int n, int nrhs, float *a, int lda, float *b,
                  int ldb);

/* replaces zml.linalg.lapack.sytrf (lapack.zig:4400-4409; kernel
 * lapack/sytrf.zig:17, used by linalg/bunchkaufman.zig:180-726):
 * Bunch-Kaufman A = U D U^T or L D L^T of the uplo triangle, D with 1x1 and
 * 2x2 blocks; ipiv as LAPACK's dsytrf (k+1 for a 1x1 block with interchange
 * row k, -(p+1) on both columns of a 2x2 block); info > 0: D(info,info) is
 * zero (the first such column in the order the factorization runs). */
int LAPACKE_dsytrf(int matrix_layout, char uplo, int n, double *a, int lda, int *ipiv);
int LAPACKE_ssytrf(int matrix_layout, char uplo, int n, float *a, int lda, int *ipiv);

/* ---- complex (zml's cfloat branches of the same routines) ---------------
 * Matrices are interleaved (re, im) pairs (LAPACKE's lapack_complex_double /
 * lapack_complex_float layout), passed as void pointers; trans 'N', 'T' or
 * 'C'; potrf factors the Hermitian matrix (A = U^H U or L L^H, the diagonal
 * real).  Called by lapack.zig:1181/1190 (getrf), 1592/1606 (getrs),
 * 2117/2128 (gesv), 3023/3031 (potrf), 3482/3495 (potrs), 3962/3973 (posv). */
int LAPACKE_zgetrf(int matrix_layout, int m, int n, void *a, int lda, int *ipiv);
int LAPACKE_cgetrf(int matrix_layout, int m, int n, void *a, int lda, int *ipiv);
int LAPACKE_zgetrs(int matrix_layout, char trans, int n, int nrhs, const void *a, int lda,
                   const int *ipiv, void *b, int ldb);
int LAPACKE_cgetrs(int matrix_layout, char trans, int n, int nrhs, const void *a, int lda,
                   const int *ipiv, void *b, int ldb);
int LAPACKE_zgesv(int matrix_layout, int n, int nrhs, void *a, int lda, int *ipiv, void *b,
                  int ldb);
int LAPACKE_cgesv(int matrix_layout, int n, int nrhs, void *a, int lda, int *ipiv, void *b,
                  int ldb);
int LAPACKE_zpotrf(int matrix_layout, char uplo, int n, void *a, int lda);
int LAPACKE_cpotrf(int matrix_layout, char uplo, int n, void *a, int lda);
int LAPACKE_zpotrs(int matrix_layout, char uplo, int n, int nrhs, const void *a, int lda,
                   void *b, int ldb);
int LAPACKE_cpotrs(int matrix_layout, char uplo, int n, int nrhs, const void *a, int lda,
                   void *b, int ldb);
int LAPACKE_zposv(int matrix_layout, char uplo, int n, int nrhs, void *a, int lda, void *b,
                  int ldb);
int LAPACKE_cposv(int matrix_layout, char uplo, int n, int nrhs, void *a, int lda, void *b,
                  int ldb);
/* complex QR (lapack.zig:5138 LAPACKE_cgeqrf, :5152 LAPACKE_zgeqrf; kernel
 * lapack/geqrf.zig:18 over cfloat): R on and above the diagonal, the
 * Householder vectors below it, tau[min(m,n)] complex; H(i) = I - tau_i v v^H
 * and A = H(0) ... H(k-1) R. */
int LAPACKE_zgeqrf(int matrix_layout, int m, int n, void *a, int lda, void *tau);
int LAPACKE_cgeqrf(int matrix_layout, int m, int n, void *a, int lda, void *tau);
/* complex symmetric Bunch-Kaufman (lapack.zig:4430 LAPACKE_zsytrf and its
 * cfloat twin; kernel lapack/sytrf.zig:17 over cfloat): A = U D U^T or
 * L D L^T without conjugation, pivot magnitudes |re| + |im|; ipiv and info as
 * LAPACKE_dsytrf. */
int LAPACKE_zsytrf(int matrix_layout, char uplo, int n, void *a, int lda, int *ipiv);
int LAPACKE_csytrf(int matrix_layout, char uplo, int n, void *a, int lda, int *ipiv);
/* Hermitian Bunch-Kaufman (lapack.zig:4556 LAPACKE_zhetrf and its cfloat
 * twin; kernel lapack/hetrf.zig:17 with hetf2.zig): A = U D U^H or L D L^H,
 * D Hermitian with real 1x1 blocks, the diagonal pivot magnitude |re a_kk|;
 * ipiv and info as LAPACKE_dsytrf. */
int LAPACKE_zhetrf(int matrix_layout, char uplo, int n, void *a, int lda, int *ipiv);
int LAPACKE_chetrf(int matrix_layout, char uplo, int n, void *a, int lda, int *ipiv);

/* replaces zml.linalg.lapack.geqrf (lapack.zig:5060; kernel lapack/geqrf.zig:18):
 * R in the upper triangle, the Householder vectors below it, tau[min(m,n)] */
int LAPACKE_dgeqrf(int matrix_layout, int m, int n, double *a, int lda, double *tau);
int LAPACKE_sgeqrf(int matrix_layout, int m, int n, float *a, int lda, float *tau);
/* replaces zml.linalg.lapack.orgqr (lapack.zig:5279 calls LAPACKE_dorgqr;
 * kernel lapack/orgqr.zig:18 with org2r.zig:18):
 * a (m x n, n <= m) <- the first n columns of Q = H(1) ... H(k) from the k
 * reflectors geqrf left below the diagonal of a, k <= n.  Used by the
 * reference's QR.q (qr.zig:44-156). */
int LAPACKE_dorgqr(int matrix_layout, int m, int n, int k, double *a, int lda, const double *tau);
int LAPACKE_sorgqr(int matrix_layout, int m, int n, int k, float *a, int lda, const float *tau);
/* replaces zml.linalg.lapack.laswp (kernel lapack/laswp.zig:12): row
 * interchanges k1..k2 (1-based) of n columns, |incx| = 1 */
int LAPACKE_dlaswp(int matrix_layout, int n, double *a, int lda, int k1, int k2, const int *ipiv,
                   int incx);
int LAPACKE_slaswp(int matrix_layout, int n, float *a, int lda, int k1, int k2, const int *ipiv,
                   int incx);

/* ---- GPU extensions: device pointers, column-major, stream ordered ------
 * `stream` is a cudaStream_t (NULL = legacy default stream).  The call
 * returns after the stream has drained (info is a host value). */
/* device-pointer form of LAPACKE_zgeqrf (interleaved complex, column-major) */
int zml_gpu_zgeqrf(int m, int n, void *dA, int ldda, void *dtau, void *stream);
/* device-pointer form of getrf (lapack/getrf.zig:14) */
int zml_gpu_dgetrf(int m, int n, double *dA, int ldda, int *dipiv, int *info, void *stream);
/* FP64 getrf on device memory that allocates nothing; no counterpart in the
 * reference.  For callers that cannot allocate device memory at solve time:
 * hosts whose device memory belongs to another allocator (a caching pool or a
 * fixed arena that a cudaMalloc from the library would fragment or overrun),
 * and loops that must not allocate after start-up.  Same factorization, bit
 * for bit, as zml_gpu_dgetrf with its updates on the FP64 pipe (always below
 * min(m, n) = 2048, or after zml_gpu_fp64_updates(0)); from 2048 up
 * zml_gpu_dgetrf's default tensor-core updates agree with it to rounding.  Its
 * scratch is one static device array of about 273 KB that every GPU loading
 * the library holds until exit; the first
 * call on a device resolves that array's address, once, under a lock.  Every
 * call shares the array: calls that overlap on the GPU race.
 * Limit: m at most what one 64-column panel holds in shared memory (about 446
 * rows per SM), on devices of at most 256 SMs; larger sizes return
 * ZML_GPU_ERR_INVALID with a message in zml_gpu_last_error(). */
int zml_gpu_dgetrf_noalloc(int m, int n, double *dA, int ldda, int *dipiv, int *info,
                           void *stream);
/* device-pointer form of getrs (lapack/getrs.zig:13) */
int zml_gpu_dgetrs(char trans, int n, int nrhs, const double *dA, int ldda, const int *dipiv,
                   double *dB, int lddb, void *stream);
/* device-pointer form of potrf (lapack/potrf.zig:17) */
int zml_gpu_dpotrf(char uplo, int n, double *dA, int ldda, int *info, void *stream);
/* device-pointer form of potrs (lapack/potrs.zig:15) */
int zml_gpu_dpotrs(char uplo, int n, int nrhs, const double *dA, int ldda, double *dB, int lddb,
                   void *stream);
/* device-pointer form of geqrf (lapack/geqrf.zig:18) */
int zml_gpu_dgeqrf(int m, int n, double *dA, int ldda, double *dtau, void *stream);
/* device-pointer form of orgqr (lapack/orgqr.zig:18) */
int zml_gpu_dorgqr(int m, int n, int k, double *dA, int ldda, const double *dtau, void *stream);
/* device-pointer form of gemm (blas/gemm.zig:14), CBLAS transpose codes */
int zml_gpu_dgemm(int transa, int transb, int m, int n, int k, double alpha, const double *dA,
                  int ldda, const double *dB, int lddb, double beta, double *dC, int lddc,
                  void *stream);

/* Tensor-core GEMM, the low-precision trailing update of the mixed-precision
 * factorizations (the 16-bit form of blas/gemm.zig:14 as called by
 * getrf.zig:125): C (fp32, column-major) <- alpha * A * B^T + beta * C with
 * A (m x k) and B (n x k) 16-bit, K-major, row strides lda/ldb a multiple of
 * 8 elements.  prec: 0 = fp16, 1 = bf16.  FP32 accumulation. */
int zml_gpu_gemm_lowp(int prec, int m, int n, int k, float alpha, const void *dA, int lda,
                      const void *dB, int ldb, float beta, float *dC, int ldc, void *stream);

/* ---- mixed precision: low-precision factorization + FP64 refinement ----- */
/* Outcome of a mixed-precision solve (no counterpart in the reference, whose
 * path is FP64 only). */
typedef struct zml_mpir_result {
  int info;              /* info (> 0: zero pivot / non-positive minor) of the
                            factorization whose solution is returned: the
                            low-precision one, or the FP64 one after a fallback */
  int iters;             /* outer refinement steps (max over right-hand sides) */
  int inner_iters;       /* total GMRES iterations */
  int converged;         /* 1 if every right-hand side reached FP64 backward error */
  int switched_f64;      /* 1 if the solves moved from FP32 to FP64 arithmetic */
  int fp64_fallback;     /* 1 if the low-precision factorization failed or
                            refinement stopped short of tol, and the system was
                            solved again by the plain FP64 getrf+getrs
                            (potrf+potrs for zml_*posv_mpir) */
  double berr;           /* largest final ||b - A x||inf / (||A||inf ||x||inf + ||b||inf) */
  double factor_ms;      /* device time of the factorization */
  double berr_history[32]; /* backward error per outer step, first right-hand side */
} zml_mpir_result;

#define ZML_PREC_FP16 0
#define ZML_PREC_BF16 1
#define ZML_PREC_FP32 2
#define ZML_PREC_BF16X3 3 /* hi+lo split, three BF16 products: ~16-bit updates */
#define ZML_REFINE_IR 0
#define ZML_REFINE_GMRES 1

/* Solves A X = B (the problem of lapack/gesv.zig:13) to FP64 backward error:
 * LU with trailing updates in `prec` (tensor cores for fp16/bf16/bf16x3,
 * FP32 panels), then plain IR or GMRES-IR with FP64 residuals.  A and B are not
 * modified.  tol = 0 refines until the backward error stops improving.  When
 * the low-precision LU fails or refinement stops short (of tol, or of 64 u
 * with tol = 0), the system is solved again by the FP64 LU (fp64_fallback).
 * Host or device pointers.  A column-major A in page-locked host memory
 * (cudaHostAlloc / cudaHostRegister) with n >= 4096 and ZML_PREC_BF16X3 is
 * copied in column chunks while the LU factors the chunks already copied;
 * the result is bit for bit the device-pointer call's, and res->factor_ms
 * then includes the copy. */
int zml_dgesv_mpir(int matrix_layout, int n, int nrhs, const double *a, int lda, const double *b,
                   int ldb, double *x, int ldx, int prec, int mode, double tol, int max_iter,
                   zml_mpir_result *res);
/* LAPACK dsgesv semantics (FP32 factorization, FP64 refinement, FP64 LU
 * fallback with *iter < 0); the mixed-precision form of gesv.zig:13. */
int LAPACKE_dsgesv(int matrix_layout, int n, int nrhs, double *a, int lda, int *ipiv, double *b,
                   int ldb, double *x, int ldx, int *iter);
/* The SPD problem of lapack/posv.zig:15 to FP64 backward error: Cholesky
 * with trailing SYRK updates in `prec` (tensor cores for fp16/bf16/bf16x3),
 * then IR / GMRES-IR with FP64 residuals.  Only the `uplo` triangle of A is
 * read; A and B are not modified.  Falls back to the FP64 Cholesky as
 * zml_dgesv_mpir falls back to the FP64 LU.  Host or device pointers. */
int zml_dposv_mpir(int matrix_layout, char uplo, int n, int nrhs, const double *a, int lda,
                   const double *b, int ldb, double *x, int ldx, int prec, int mode, double tol,
                   int max_iter, zml_mpir_result *res);
/* LAPACK dsposv semantics (FP32 Cholesky, FP64 refinement, FP64 potrf
 * fallback with *iter < 0); the mixed-precision form of posv.zig:15. */
int LAPACKE_dsposv(int matrix_layout, char uplo, int n, int nrhs, double *a, int lda, double *b,
                   int ldb, double *x, int ldx, int *iter);
/* Device-pointer, stream-ordered form of zml_dposv_mpir (column-major). */
int zml_gpu_dposv_mpir(char uplo, int n, int nrhs, const double *dA, int ldda, const double *dB,
                       int lddb, double *dX, int lddx, int prec, int mode, double tol,
                       int max_iter, zml_mpir_result *res, void *stream);
/* Device-pointer, stream-ordered form of zml_dgesv_mpir (column-major). */
int zml_gpu_dgesv_mpir(int n, int nrhs, const double *dA, int ldda, const double *dB, int lddb,
                       double *dX, int lddx, int prec, int mode, double tol, int max_iter,
                       zml_mpir_result *res, void *stream);

/* ---- batched small solves (no counterpart in the reference) -------------
 * count systems A_i X_i = B_i, n_i in 1..256, packed back to back in device
 * memory: A_i (n_i x n_i, ld n_i) at offset sum_{j<i} n_j^2, B_i and X_i
 * (n_i x nrhs, ld n_i) at sum_{j<i} n_j nrhs, ipiv_i at sum_{j<i} n_j.
 * spd[i] != 0: lower Cholesky (potrf + potrs of potrf.zig:17 / potrs.zig:15),
 * else partial-pivot LU (getrf + getrs of getrf.zig:14 / getrs.zig:13).
 * prec 0: FP64 (A overwritten by its factors); prec 1: FP32 factors + FP64
 * iterative refinement (A untouched; iters[i] = refinement steps).
 * info[i] as LAPACK.  The plan does the host work once; execute is one
 * memset and one persistent launch (capturable); run_graph captures it in a
 * CUDA graph on first use and replays it. */
int zml_gpu_batched_plan_create(void **plan, int count, const int *n, const int *spd, int nrhs,
                                int prec, int max_ir);
int zml_gpu_batched_execute(void *plan, double *dA, const double *dB, double *dX, int *dipiv,
                            int *dinfo, int *diters, void *stream);
int zml_gpu_batched_run_graph(void *plan, double *dA, const double *dB, double *dX, int *dipiv,
                              int *dinfo, int *diters, void *stream);
void zml_gpu_batched_plan_destroy(void *plan);
/* Per-size-class warp schedule (warps per matrix: 1, 2, 4, 8 or 16; class i holds n <= edges[i]):
 * read (set = 0) or replace (set = 1).  Returns the number of classes. */
int zml_gpu_batched_schedule(int prec, int *warps, int *edges, int cap, int set);
/* Times every warp count for every class and keeps the fastest; chosen[i]
 * and ms[i] (may be NULL) receive the result per class. */
int zml_gpu_batched_autotune(int prec, int nrhs, int *chosen, double *ms, void *stream);

/* ---- learned precision selector (no counterpart in the reference) ---------
 * Structural features of an n x n FP64 matrix (device), 16 floats: [0] log2 n,
 * [1] log10 scale, [2] row-scale spread, [3] column-scale spread, [4]-[5]
 * diagonal dominance (worst, mean), [6] asymmetry, [7] entry spread, [8]
 * diagonal spread, [9]-[11] norm ratios; [12]-[15] are left for the caller's
 * refinement probe. */
int zml_gpu_selector_features(int n, const double *dA, int ldda, float *dfeat, void *stream);
/* MLP 16 -> 64 -> 64 -> 5 (ReLU), BF16 operands with FP32 accumulation,
 * parameters packed W1[64x16] b1 W2[64x64] b2 W3[5x64] b3 (FP32 master). */
int zml_gpu_mlp_num_params(void);
long zml_gpu_mlp_work_floats(int batch);
int zml_gpu_mlp_forward(int batch, const float *dX, const float *dP, float *dLogits, float *dWork,
                        void *stream);
/* Softmax cross-entropy gradients of the mean loss over the batch (dG), the
 * per-sample losses (dLoss). */
int zml_gpu_mlp_gradients(int batch, const float *dX, const int *dy, const float *dP, float *dG,
                          float *dLoss, float *dWork, void *stream);
int zml_gpu_mlp_adam(float *dP, const float *dG, float *dM, float *dV, float lr, float beta1,
                     float beta2, float eps, int step, float weight_decay, void *stream);
/* Floats of a selector model: the MLP parameters, then the means and the
 * scales of the 16 input features (input k = (f_k - mean_k) / scale_k). */
int zml_gpu_selector_model_floats(void);

/* Precision classes of the ladder, cheapest first. */
#define ZML_CLASS_BF16 0
#define ZML_CLASS_FP16 1
#define ZML_CLASS_BF16X3 2
#define ZML_CLASS_FP32 3
#define ZML_CLASS_FP64 4 /* plain FP64 LU (getrf.zig:14 + getrs.zig:13) */

typedef struct zml_auto_result {
  int info;          /* info of the returned attempt */
  int predicted;     /* class chosen by the network, -1 if none was consulted */
  int used;          /* class of the returned solution */
  int attempts;      /* factorizations performed, the BF16 probe included */
  int converged;     /* 1 if every column reached backward error <= 64 u */
  int iters;         /* refinement steps of the returned attempt */
  double berr;       /* its largest normwise backward error */
  double ms;         /* wall time of the call */
  float features[16]; /* the selector's input features: [0]-[11] as
                         zml_gpu_selector_features; [12] log10 of the first
                         BF16 backward error, [13] log10 of the first step's
                         ratio, [14] log10 of a condition estimate,
                         ||A||inf times ||z||inf after 3 steps of inverse
                         iteration with the BF16 factors (0 if they failed),
                         [15] 1 if the BF16 LU failed (0.5 if the solves moved
                         to FP64 arithmetic) */
  float proba[5];    /* predicted class probabilities */
  int reserved;
} zml_auto_result;

/* A X = B (the problem of lapack/gesv.zig:13) to FP64 backward error by the
 * precision ladder BF16 -> FP16 -> BF16x3 -> FP32 (GMRES-IR, at most
 * max_iter steps each; 0 = 10) -> FP64 LU.  The BF16 attempt comes first and
 * its first two refinement steps are the probe that completes the features;
 * given a model (host memory, zml_gpu_selector_model_floats floats), the
 * ladder then resumes at the smallest class whose cumulative predicted
 * probability reaches `confidence` (0 < confidence <= 1) instead of the next
 * rung.  The FP64 LU is the fallback of every path.  A and B are not
 * modified.  Host or device pointers. */
int zml_dgesv_auto(int matrix_layout, int n, int nrhs, const double *a, int lda, const double *b,
                   int ldb, double *x, int ldx, const float *model, float confidence,
                   int max_iter, zml_auto_result *res);
/* Device-pointer, stream-ordered form of zml_dgesv_auto (column-major). */
int zml_gpu_dgesv_auto(int n, int nrhs, const double *dA, int ldda, const double *dB, int lddb,
                       double *dX, int lddx, const float *model, float confidence, int max_iter,
                       zml_auto_result *res, void *stream);

/* ---- instrumentation ------------------------------------------------------
 * Kernel classes: 0 tensor-core GEMM, 1 CUDA-core GEMM/SYRK, 2 LU panel,
 * 3 TRSM diagonal block, 4 row interchanges, 5 low-precision TRSV, 6 FP64
 * GEMV / residual, 7 conversions, 8 Cholesky diagonal block, 9 vector ops,
 * 10 batched solver, 11 QR, 12 selector MLP, 13 other. */
/* Enables (1) or disables (0) CUDA-event timing of every launch, by class;
 * enabling clears the accumulated figures. */
void zml_gpu_profile(int enable);
/* Launches, device ms, algorithmic flops and bytes of one class so far. */
int zml_gpu_profile_read(int kernel_class, unsigned long long *launches, double *ms,
                         double *flops, double *bytes);
/* Kernels launched by this library in this process. */
unsigned long long zml_gpu_launch_count(void);

/* Text of the last library error on this thread. */
const char *zml_gpu_last_error(void);
/* Iteration limit of every bounded device-side wait of the library (grid
 * barriers, mbarrier waits, polls of published values) on the current
 * device; tries <= 0 restores the default of 1 << 22 (about a second).  A
 * wait that runs out sets a status bit and its kernel finishes with every
 * index kept in range; the call then returns ZML_GPU_ERR_TIMEOUT.  For tests
 * of that path; no counterpart in the reference. */
int zml_gpu_set_spin_limit(long long tries);
/* Pivoting of the mixed-precision LU's panels (zml_*gesv_mpir, the ladder):
 * 1 tournament pivoting (a communication-avoiding LU whose 32-column
 * sub-panels need one exchange between the panel's thread blocks instead of
 * one per column), 0 partial pivoting (the default, faster on GB300).
 * Returns the previous setting.  No counterpart in the reference (its getrf2
 * pivots partially). */
int zml_gpu_mixed_panel(int tournament);
/* Where the FP64 factorizations (getrf, potrf and what calls them) run their
 * trailing updates from n = 2048 up: 1 (the default) on the BF16 tensor
 * cores, each FP64 operand cut into eight exact 7-bit integer slices whose
 * products are accumulated exactly where it matters (about the accuracy of an
 * FP64 GEMM); 0 on the FP64 pipe.  Returns the previous mode.  No counterpart
 * in the reference (an FP64 loop nest). */
int zml_gpu_fp64_updates(int mode);
/* Rows per thread block that the cooperative LU panel (the FP64 panel, and
 * the FP32 one where the cluster panel does not apply) aims for: fewer,
 * taller blocks make its per-column grid barrier cheaper and its per-column
 * update longer.  0 spreads the panel over every SM; a negative value
 * restores the default.  The factorization is the same for every value.
 * Returns the previous setting.  No counterpart in the reference. */
int zml_gpu_panel_rows(int rows);
/* The FP64 update those factorizations use, on device memory (column-major):
 * C (m x n) -= A (m x k) B (k x n) with k <= 256, by exact 7-bit slices of A's
 * rows and B's columns multiplied on the BF16 tensor cores; lower != 0:
 * C -= A A^T on C's lower triangle only (m == n, dB unused).  About the
 * accuracy of an FP64 GEMM (the slices keep 56 bits of each row's / column's
 * largest entry).  No counterpart in the reference. */
int zml_gpu_dgemm_slices(int m, int n, int k, const double *dA, int ldda, const double *dB,
                         int lddb, double *dC, int lddc, int lower, void *stream);
/* FP32 LU with tournament pivoting on device memory (column-major), the
 * factorization the mixed solver preconditions with: P A = L U as sgetrf's,
 * ipiv in LAPACK's form, but each 32-column sub-panel's pivots are chosen
 * among candidates the panel's thread blocks nominate from their own rows, so
 * they can differ from partial pivoting's.  info > 0: a zero pivot.  No
 * counterpart in the reference. */
int zml_gpu_sgetrf_calu(int m, int n, float *dA, int ldda, int *dipiv, int *info, void *stream);
/* ABI version of this library. */
int zml_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif
