/*
 * zml_oracle.h -- CPU restatement of zml's dense factor-and-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle and the timed
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the GPU product path never calls it.
 *
 * Every routine restates a Zig routine of srmadrid/zml loop for loop, in the
 * same operation order, with IEEE binary64/binary32 arithmetic and no FMA
 * contraction (built with -ffp-contract=off), so that its results are the
 * reference's bit for bit.  Each definition in oracle_impl.h cites the Zig
 * file and lines it follows.
 *
 * Enumerations use the CBLAS codes of include/cblas.h (reference
 * include/cblas.h:11-38): layout 101/102, transpose 111-114, uplo 121/122,
 * diag 131/132, side 141/142.
 *
 * Error convention: a Zig routine that returns error.InvalidArgument returns
 * ZO_EINVAL (-1) here; LAPACK routines otherwise return their `info` (>= 0).
 * iamax returns the 0-based index (zml's u32 result).
 */
#ifndef ZML_ORACLE_H
#define ZML_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ZO_EINVAL (-1)

/* trsm as written in the reference reads b[k + j*lda] where b[k + j*ldb]
 * is meant (blas/trsm.zig:139,179,224,247).  1 (default) restates that
 * exactly; 0 uses ldb.  The two agree whenever lda == ldb. */
void zo_set_trsm_as_written(int on);

#define ZO_DECL(T, P)                                                                          \
  int P##gemm(int order, int transa, int transb, int m, int n, int k, T alpha, const T *a,    \
              int lda, const T *b, int ldb, T beta, T *c, int ldc);                           \
  int P##trsm(int order, int side, int uplo, int transa, int diag, int m, int n, T alpha,     \
              const T *a, int lda, T *b, int ldb);                                            \
  int P##syrk(int order, int uplo, int trans, int n, int k, T alpha, const T *a, int lda,     \
              T beta, T *c, int ldc);                                                         \
  int P##trmm(int order, int side, int uplo, int transa, int diag, int m, int n, T alpha,     \
              const T *a, int lda, T *b, int ldb);                                            \
  int P##gemv(int order, int transa, int m, int n, T alpha, const T *a, int lda, const T *x,  \
              int incx, T beta, T *y, int incy);                                              \
  int P##ger(int order, int m, int n, T alpha, const T *x, int incx, const T *y, int incy,    \
             T *a, int lda);                                                                  \
  int P##iamax(int n, const T *x, int incx);                                                  \
  int P##scal(int n, T alpha, T *x, int incx);                                                \
  int P##swap(int n, T *x, int incx, T *y, int incy);                                         \
  int P##copy(int n, const T *x, int incx, T *y, int incy);                                   \
  int P##axpy(int n, T alpha, const T *x, int incx, T *y, int incy);                          \
  T P##nrm2(int n, const T *x, int incx);                                                     \
  T P##lamch(char cmach);                                                                     \
  int P##laswp(int order, int n, T *a, int lda, int k1, int k2, const int *ipiv, int incx);   \
  int P##getrf2(int order, int m, int n, T *a, int lda, int *ipiv);                           \
  int P##getrf(int order, int m, int n, T *a, int lda, int *ipiv);                            \
  int P##getrs(int order, int trans, int n, int nrhs, const T *a, int lda, const int *ipiv,   \
               T *b, int ldb);                                                                \
  int P##gesv(int order, int n, int nrhs, T *a, int lda, int *ipiv, T *b, int ldb);           \
  int P##potrf2(int order, int uplo, int n, T *a, int lda);                                   \
  int P##potrf(int order, int uplo, int n, T *a, int lda);                                    \
  int P##potrs(int order, int uplo, int n, int nrhs, const T *a, int lda, T *b, int ldb);     \
  int P##posv(int order, int uplo, int n, int nrhs, T *a, int lda, T *b, int ldb);            \
  T P##lapy3(T x, T y, T z);                                                                  \
  int P##larfg(int n, T *alpha, T *x, int incx, T *tau);                                      \
  int P##larf1f(int order, int side, int m, int n, const T *v, int incv, T tau, T *c,         \
                int ldc, T *work);                                                            \
  int P##geqr2(int order, int m, int n, T *a, int lda, T *tau, T *work);                      \
  int P##larft(int order, int direct, int storev, int n, int k, const T *v, int ldv,          \
               const T *tau, T *t, int ldt);                                                  \
  int P##larfb(int order, int side, int trans, int direct, int storev, int m, int n, int k,   \
               const T *v, int ldv, const T *t, int ldt, T *c, int ldc, T *work, int ldwork); \
  int P##geqrf(int order, int m, int n, T *a, int lda, T *tau, T *work, int lwork); \
  int P##org2r(int order, int m, int n, int k, T *a, int lda, const T *tau, T *work);        \
  int P##orgqr(int order, int m, int n, int k, T *a, int lda, const T *tau, T *work,          \
               int lwork);                                                                    \
  int P##syr(int order, int uplo, int n, T alpha, const T *x, int incx, T *a, int lda);       \
  int P##gemmtr(int order, int uplo, int transa, int transb, int n, int k, T alpha,           \
                const T *a, int lda, const T *b, int ldb, T beta, T *c, int ldc);             \
  int P##sytf2(int order, int uplo, int n, T *a, int lda, int *ipiv);                         \
  int P##lasyf(int order, int uplo, int n, int nb, int *kb, T *a, int lda, int *ipiv, T *w,   \
               int ldw);                                                                      \
  int P##sytrf(int order, int uplo, int n, T *a, int lda, int *ipiv, T *work, int lwork);

ZO_DECL(double, zo_d_)
ZO_DECL(float, zo_s_)
#undef ZO_DECL

/* Threaded forms (column-major, binary64) of zo_d_getrf and zo_d_potrf for the
 * large parity cases: bit-identical results (oracle_mt.h).  margin
 * (optional, min(m, n) entries) receives each column's pivot gap. */
int zo_d_getrf_mt(int m, int n, double *a, int lda, int *ipiv, double *margin, int threads);
int zo_d_potrf_mt(int uplo, int n, double *a, int lda, int threads);

/* ---- complex (cfloat) ----------------------------------------------------
 * Interleaved (re, im) pairs: numpy complex128 / complex64.  The arithmetic
 * restates zml's cfloat operations (cfloat.zig), whose products and Smith
 * divisions use explicit fused multiply-adds; herk takes real alpha, beta. */
typedef struct { double re, im; } zo_cf64;
typedef struct { float re, im; } zo_cf32;

/* A real x divided by a complex y.  zml's own test pins x / y
 * (test/cfloat/div.zig:42-44); cfloat.zig:489-492 as written computes y / x.
 * 0 (default) restates the tested quotient, 1 the code as written.  getrf2
 * reaches it as div(1, a[0]) (lapack/getrf2.zig:66-75). */
void zo_set_cdiv_as_written(int on);

#define ZO_ZDECL(Z, R, P)                                                                      \
  int P##gemm(int order, int transa, int transb, int m, int n, int k, Z alpha, const Z *a,    \
              int lda, const Z *b, int ldb, Z beta, Z *c, int ldc);                           \
  int P##trsm(int order, int side, int uplo, int transa, int diag, int m, int n, Z alpha,     \
              const Z *a, int lda, Z *b, int ldb);                                            \
  int P##syrk(int order, int uplo, int trans, int n, int k, Z alpha, const Z *a, int lda,     \
              Z beta, Z *c, int ldc);                                                         \
  int P##herk(int order, int uplo, int trans, int n, int k, R alpha, const Z *a, int lda,     \
              R beta, Z *c, int ldc);                                                         \
  int P##trmm(int order, int side, int uplo, int transa, int diag, int m, int n, Z alpha,     \
              const Z *a, int lda, Z *b, int ldb);                                            \
  int P##gemv(int order, int transa, int m, int n, Z alpha, const Z *a, int lda, const Z *x,  \
              int incx, Z beta, Z *y, int incy);                                              \
  int P##geru(int order, int m, int n, Z alpha, const Z *x, int incx, const Z *y, int incy,   \
              Z *a, int lda);                                                                 \
  int P##gerc(int order, int m, int n, Z alpha, const Z *x, int incx, const Z *y, int incy,   \
              Z *a, int lda);                                                                 \
  int P##iamax(int n, const Z *x, int incx);                                                  \
  int P##scal(int n, Z alpha, Z *x, int incx);                                                \
  int P##laswp(int order, int n, Z *a, int lda, int k1, int k2, const int *ipiv, int incx);   \
  int P##getrf2(int order, int m, int n, Z *a, int lda, int *ipiv);                           \
  int P##getrf(int order, int m, int n, Z *a, int lda, int *ipiv);                            \
  int P##getrs(int order, int trans, int n, int nrhs, const Z *a, int lda, const int *ipiv,   \
               Z *b, int ldb);                                                                \
  int P##gesv(int order, int n, int nrhs, Z *a, int lda, int *ipiv, Z *b, int ldb);           \
  int P##potrf2(int order, int uplo, int n, Z *a, int lda);                                   \
  int P##potrf(int order, int uplo, int n, Z *a, int lda);                                    \
  int P##potrs(int order, int uplo, int n, int nrhs, const Z *a, int lda, Z *b, int ldb);     \
  int P##posv(int order, int uplo, int n, int nrhs, Z *a, int lda, Z *b, int ldb);            \
  R P##nrm2(int n, const Z *x, int incx);                                                     \
  int P##larfg(int n, Z *alpha, Z *x, int incx, Z *tau);                                      \
  int P##larf1f(int order, int side, int m, int n, const Z *v, int incv, Z tau, Z *c,         \
                int ldc, Z *work);                                                            \
  int P##geqr2(int order, int m, int n, Z *a, int lda, Z *tau, Z *work);                      \
  int P##larft(int order, int direct, int storev, int n, int k, const Z *v, int ldv,          \
               const Z *tau, Z *t, int ldt);                                                  \
  int P##larfb(int order, int side, int trans, int direct, int storev, int m, int n, int k,   \
               const Z *v, int ldv, const Z *t, int ldt, Z *c, int ldc, Z *work, int ldwork); \
  int P##geqrf(int order, int m, int n, Z *a, int lda, Z *tau, Z *work, int lwork);          \
  int P##her(int order, int uplo, int n, R alpha, const Z *x, int incx, Z *a, int lda);       \
  int P##hetf2(int order, int uplo, int n, Z *a, int lda, int *ipiv);                         \
  int P##lahef(int order, int uplo, int n, int nb, int *kb, Z *a, int lda, int *ipiv, Z *w,   \
               int ldw);                                                                      \
  int P##hetrf(int order, int uplo, int n, Z *a, int lda, int *ipiv, Z *work, int lwork);      \
  int P##syr(int order, int uplo, int n, Z alpha, const Z *x, int incx, Z *a, int lda);        \
  int P##sytf2(int order, int uplo, int n, Z *a, int lda, int *ipiv);                         \
  int P##lasyf(int order, int uplo, int n, int nb, int *kb, Z *a, int lda, int *ipiv, Z *w,   \
               int ldw);                                                                      \
  int P##sytrf(int order, int uplo, int n, Z *a, int lda, int *ipiv, Z *work, int lwork);

ZO_ZDECL(zo_cf64, double, zo_z_)
ZO_ZDECL(zo_cf32, float, zo_c_)
#undef ZO_ZDECL

/* ilaenv restatement (lapack/ilaenv.zig): ispec 1 = NB, 2 = NBMIN, 3 = NX.
 * name is the 6-letter routine name, e.g. "DGETRF". */
int zo_ilaenv(int ispec, const char *name, int n1, int n2, int n3, int n4);

/* Deterministic seeded inputs shared by the oracle and the GPU tests:
 * SplitMix64 stream -> U(lo,hi) or N(0,1) by Box-Muller (glibc log/cos/sin),
 * identical bits on every host. */
void zo_fill_uniform(double *x, long long count, unsigned long long seed, double lo, double hi);
void zo_fill_normal(double *x, long long count, unsigned long long seed);

#ifdef __cplusplus
}
#endif
#endif
