/*
 * zml_linalg.h -- the decomposition API of zml.linalg (owning factor objects)
 * over libzml_gb300's GPU factorizations, FP64.
 *
 * Mirrors src/linalg/lu.zig (PLU, plu), src/linalg/cholesky.zig (LLT, UTU,
 * llt, utu, cholesky), src/linalg/bunchkaufman.zig (LDLT, UDUT, ldlt, udut,
 * bunchkaufman) and src/linalg/qr.zig (QR, qr, QR.q, QR.r): the
 * constructor copies the input matrix into storage the factor object owns
 * (host memory, in the input's layout), factors it with the library's GPU
 * LAPACK (getrf / potrf / geqrf, orgqr for Q), and the accessors return
 * views into that storage.  Errors are the reference's: a zero pivot or a
 * non-positive leading minor is ZML_ERR_SINGULAR_MATRIX (error.SingularMatrix,
 * lu.zig:212-213, cholesky.zig:124-125) and the object is not created; bad
 * arguments are ZML_ERR_INVALID_ARGUMENT; library failures are <= -1000.
 */
#ifndef ZML_GB300_LINALG_H
#define ZML_GB300_LINALG_H

#ifdef __cplusplus
extern "C" {
#endif

#define ZML_ERR_INVALID_ARGUMENT (-2000) /* error.InvalidArgument */
#define ZML_ERR_SINGULAR_MATRIX (-2001)  /* error.SingularMatrix */
#define ZML_ERR_OUT_OF_MEMORY (-2002)    /* error.OutOfMemory */

/* A dense matrix or a view of one: element (i, j) is data[i + j*ld]
 * (layout 102, column-major) or data[i*ld + j] (layout 101, row-major).
 * uplo / diag describe triangular views (0 = general; 121 upper, 122 lower;
 * 131 non-unit, 132 unit), as matrix.Triangular(T, uplo, diag, order). */
typedef struct zml_dmatrix {
  double *data;
  int rows, cols, ld;
  int layout;
  int uplo, diag;
  int owns_data; /* 1: release with zml_dmatrix_deinit */
} zml_dmatrix;

void zml_dmatrix_deinit(zml_dmatrix *m);

/* ---- LU with partial pivoting: PLU(f64, order) (lu.zig:62-126) ---------- */
typedef struct zml_plu_s zml_plu_t;
/* plu (lu.zig:178-216): copies the m x n matrix a, getrf. */
int zml_plu(int layout, int m, int n, const double *a, int lda, zml_plu_t **out);
void zml_plu_deinit(zml_plu_t *f);
/* PLU.p (lu.zig:82-99): the row permutation, m entries, as the reference
 * builds it from ipiv (identity, then the interchanges applied last to
 * first): A = P L U with row i of A equal to row perm[i] of L U. */
int zml_plu_p(const zml_plu_t *f, unsigned *perm);
/* PLU.l (lu.zig:101-109): unit lower m x min(m,n); PLU.u (lu.zig:111-119):
 * upper min(m,n) x n; views into the factor storage. */
zml_dmatrix zml_plu_l(const zml_plu_t *f);
zml_dmatrix zml_plu_u(const zml_plu_t *f);
/* The 1-based pivot indices, min(m,n) of them. */
const int *zml_plu_ipiv(const zml_plu_t *f);

/* ---- Cholesky: LLT / UTU (cholesky.zig:17-94) --------------------------- */
typedef struct zml_chol_s zml_chol_t;
/* llt (cholesky.zig:95-131): A = L L^T from the `uplo` triangle of the
 * symmetric n x n matrix a (the other triangle is not read). */
int zml_llt(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out);
/* utu (cholesky.zig:133-169): A = U^T U. */
int zml_utu(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out);
/* cholesky (cholesky.zig:171-188): llt for a lower-stored matrix, utu for an
 * upper-stored one. */
int zml_cholesky(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out);
void zml_chol_deinit(zml_chol_t *f);
/* LLT.l (cholesky.zig:37-45) / UTU.u (:76-84): the factor, a non-unit
 * triangular view (uplo 122 for LLT, 121 for UTU). */
zml_dmatrix zml_chol_factor(const zml_chol_t *f);

/* ---- Householder QR: QR(f64, order) (qr.zig:21-185) ------------------- */
#define ZML_QR_FULL 0        /* Mode.full */
#define ZML_QR_ECONOMICAL 1  /* Mode.economical */
typedef struct zml_qr_s zml_qr_t;
/* qr (qr.zig:192-263): copies a, geqrf. */
int zml_qr(int layout, int m, int n, const double *a, int lda, zml_qr_t **out);
void zml_qr_deinit(zml_qr_t *f);
/* QR.q (qr.zig:44-159): a new owned matrix, m x m (full) or m x min(m,n)
 * (economical), formed by orgqr from the stored reflectors. */
int zml_qr_q(const zml_qr_t *f, int mode, zml_dmatrix *q);
/* QR.r (qr.zig:161-177): the upper-triangular view, m x n (full) or
 * min(m,n) x n (economical), into the factor storage. */
zml_dmatrix zml_qr_r(const zml_qr_t *f, int mode);
/* The min(m,n) reflector scalars. */
const double *zml_qr_tau(const zml_qr_t *f);

/* ---- matmul facade (linalg/matmul.zig:19, its dense cases) -------------- */
#define ZML_ERR_DIMENSION_MISMATCH (-2003) /* error.DimensionMismatch */
/* c = a b as a new owned general matrix in a's layout (matmul/dgedge.zig:11-41:
 * gemm with b transposed when its layout differs from a's), on the GPU GEMM.
 * a or b may be triangular views (uplo / diag): they are multiplied as the
 * dense matrices they stand for (zeros outside the triangle, ones on a unit
 * diagonal), as matmul.zig's element loops for those cases do.  a->cols must
 * equal b->rows. */
int zml_dmatmul(const zml_dmatrix *a, const zml_dmatrix *b, zml_dmatrix *c);
/* y = a x (matmul/dgedv.zig:11, gemv): x has a->cols entries, y a->rows,
 * strides incx / incy (non-zero; negative as in BLAS). */
int zml_dmatvec(const zml_dmatrix *a, const double *x, int incx, double *y, int incy);
/* y = x^T b (matmul/dvdge.zig:11, gemv transposed): x has b->rows entries,
 * y b->cols. */
int zml_dvecmat(const double *x, int incx, const zml_dmatrix *b, double *y, int incy);

/* ---- Bunch-Kaufman: LDLT / UDUT (bunchkaufman.zig:20-179) -------------- */
#define ZML_ERR_FACTORIZATION_FAILED (-2004) /* linalg.Error.FactorizationFailed */
/* One object type for both forms; the ldlt_* accessors require a lower
 * (LDLT) object and the udut_* ones an upper (UDUT) object. */
typedef struct zml_bk_s zml_ldlt_t;
typedef struct zml_bk_s zml_udut_t;
/* ldlt (bunchkaufman.zig:180-443): copies the `uplo` triangle of the n x n
 * symmetric a into the lower triangle of a packed matrix (copyInverseUplo when
 * upper-stored) and factors it with dsytrf, A = P L D L^T P^T.  Any info != 0
 * is ZML_ERR_FACTORIZATION_FAILED and no object is created. */
int zml_ldlt(int layout, char uplo, int n, const double *a, int lda, zml_ldlt_t **out);
/* udut (bunchkaufman.zig:445-707): the same into the upper triangle,
 * A = P U D U^T P^T. */
int zml_udut(int layout, char uplo, int n, const double *a, int lda, zml_udut_t **out);
/* bunchkaufman (bunchkaufman.zig:709-726): ldlt for a lower-stored matrix
 * (*lo set, *up NULL), udut for an upper-stored one (*up set, *lo NULL). */
int zml_bunchkaufman(int layout, char uplo, int n, const double *a, int lda, zml_ldlt_t **lo,
                     zml_udut_t **up);
/* LDLT.init / UDUT.init (bunchkaufman.zig:27-34, 107-114): an object over an
 * existing dsytrf factor (lower / upper, leading dimension ld) and its ipiv,
 * both copied (the reference takes ownership of its arguments instead). */
int zml_ldlt_init(int layout, int n, const double *f, int ld, const int *ipiv, zml_ldlt_t **out);
int zml_udut_init(int layout, int n, const double *f, int ld, const int *ipiv, zml_udut_t **out);
void zml_ldlt_deinit(zml_ldlt_t *f);
void zml_udut_deinit(zml_udut_t *f);
/* LDLT.p / UDUT.p (:43-55, :123-135): perm (n entries) from the identity by
 * ipiv's interchanges in factorization order (lpermute / upermute), so that
 * (P^T A P)(i, j) = A(perm[i], perm[j]); the reference returns the
 * Permutation over perm transposed. */
int zml_ldlt_p(const zml_ldlt_t *f, unsigned *perm);
int zml_udut_p(const zml_udut_t *f, unsigned *perm);
/* LDLT.l / UDUT.u (:57-72, :137-152): a new owned n x n unit-triangular
 * matrix in the object's layout (lconvert / uconvert: the multipliers, rows
 * permuted into P's order; zero outside the triangle, one on the diagonal).
 * data is NULL when the allocation fails. */
zml_dmatrix zml_ldlt_l(const zml_ldlt_t *f);
zml_dmatrix zml_udut_u(const zml_udut_t *f);
/* LDLT.d / UDUT.d (:74-89, :154-169): the block-diagonal D as a tridiagonal
 * (sub and sup n-1 entries, diag n), zero between blocks.  Returns 0,
 * ZML_ERR_INVALID_ARGUMENT, or ZML_ERR_OUT_OF_MEMORY (nothing written) when
 * its scratch cannot be allocated. */
int zml_ldlt_d(const zml_ldlt_t *f, double *sub, double *diag, double *sup);
int zml_udut_d(const zml_udut_t *f, double *sub, double *diag, double *sup);
const int *zml_ldlt_ipiv(const zml_ldlt_t *f);
const int *zml_udut_ipiv(const zml_udut_t *f);

#ifdef __cplusplus
}
#endif
#endif
