/*
 * cblas.h -- level-3 BLAS of libzml_gb300 (GB300, sm_103a).
 *
 * Same prototypes and enumeration codes as the reference's include/cblas.h
 * (enums :11-38; gemm :216-217, syrk :235-236, trsm :250-251), so a C caller
 * of zml's libblas links against this library unchanged.  Only the real
 * single- and double-precision routines on the factor-and-solve path are
 * provided.
 *
 * Pointers may be host memory (staged to the GPU and back) or device /
 * managed memory (used in place).  Calls are synchronous.  Device operands
 * are read after all work queued earlier on the legacy default stream; a
 * caller that fills them on another stream synchronizes that stream first.
 * Invalid arguments return silently, as zml's src/cblas.zig does.
 */
#ifndef ZML_GB300_CBLAS_H
#define ZML_GB300_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE {
  CblasNoTrans = 111,
  CblasTrans = 112,
  CblasConjTrans = 113,
  CblasConjNoTrans = 114
} CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
typedef CBLAS_ORDER CBLAS_LAYOUT;

/* reference include/cblas.h:216 -> src/cblas.zig:523 -> blas/gemm.zig */
void cblas_sgemm(const CBLAS_ORDER order, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const int m, const int n, const int k,
                 const float alpha, const float *a, const int lda, const float *b, const int ldb,
                 const float beta, float *c, const int ldc);
/* reference include/cblas.h:217 -> src/cblas.zig:526 -> blas/gemm.zig */
void cblas_dgemm(const CBLAS_ORDER order, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const int m, const int n, const int k,
                 const double alpha, const double *a, const int lda, const double *b,
                 const int ldb, const double beta, double *c, const int ldc);
/* reference include/cblas.h:235 -> src/cblas.zig:584 -> blas/syrk.zig */
void cblas_ssyrk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const float alpha, const float *a, const int lda,
                 const float beta, float *c, const int ldc);
/* reference include/cblas.h:236 -> src/cblas.zig:587 -> blas/syrk.zig */
void cblas_dsyrk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const double alpha, const double *a, const int lda,
                 const double beta, double *c, const int ldc);
/* reference include/cblas.h:250 -> src/cblas.zig:633 -> blas/trsm.zig */
void cblas_strsm(const CBLAS_ORDER order, const CBLAS_SIDE side, const CBLAS_UPLO uplo,
                 const CBLAS_TRANSPOSE transa, const CBLAS_DIAG diag, const int m, const int n,
                 const float alpha, const float *a, const int lda, float *b, const int ldb);
/* reference include/cblas.h:251 -> src/cblas.zig:636 -> blas/trsm.zig */
void cblas_dtrsm(const CBLAS_ORDER order, const CBLAS_SIDE side, const CBLAS_UPLO uplo,
                 const CBLAS_TRANSPOSE transa, const CBLAS_DIAG diag, const int m, const int n,
                 const double alpha, const double *a, const int lda, double *b, const int ldb);

/* Complex level 3 (reference include/cblas.h:218-219, 224-225, 237-238):
 * matrices are interleaved (re, im) pairs, leading dimensions in complex
 * elements; alpha / beta point to one {re, im} pair (herk: real scalars).
 * Computed as real GEMMs on the GPU (a complex product is four real ones). */
void cblas_cgemm(const CBLAS_ORDER order, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const int m, const int n, const int k,
                 const void *alpha, const void *a, const int lda, const void *b, const int ldb,
                 const void *beta, void *c, const int ldc);
void cblas_zgemm(const CBLAS_ORDER order, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const int m, const int n, const int k,
                 const void *alpha, const void *a, const int lda, const void *b, const int ldb,
                 const void *beta, void *c, const int ldc);
void cblas_cherk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const float alpha, const void *a, const int lda,
                 const float beta, void *c, const int ldc);
void cblas_zherk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const double alpha, const void *a, const int lda,
                 const double beta, void *c, const int ldc);
void cblas_csyrk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const void *alpha, const void *a, const int lda,
                 const void *beta, void *c, const int ldc);
void cblas_zsyrk(const CBLAS_ORDER order, const CBLAS_UPLO uplo, const CBLAS_TRANSPOSE trans,
                 const int n, const int k, const void *alpha, const void *a, const int lda,
                 const void *beta, void *c, const int ldc);
/* reference include/cblas.h:252-253: B <- alpha op(A)^-1 B or alpha B op(A)^-1 */
void cblas_ctrsm(const CBLAS_ORDER order, const CBLAS_SIDE side, const CBLAS_UPLO uplo,
                 const CBLAS_TRANSPOSE transa, const CBLAS_DIAG diag, const int m, const int n,
                 const void *alpha, const void *a, const int lda, void *b, const int ldb);
void cblas_ztrsm(const CBLAS_ORDER order, const CBLAS_SIDE side, const CBLAS_UPLO uplo,
                 const CBLAS_TRANSPOSE transa, const CBLAS_DIAG diag, const int m, const int n,
                 const void *alpha, const void *a, const int lda, void *b, const int ldb);

#ifdef __cplusplus
}
#endif
#endif
