// api.cu -- zml.linalg's decomposition objects (include/zml_linalg.h) over
// the library's GPU LAPACK.  Host code only.
//
// Mirrors src/linalg/lu.zig:62-216 (PLU, plu), cholesky.zig:17-188 (LLT, UTU,
// llt, utu, cholesky) and qr.zig:21-263 (QR, qr, QR.q, QR.r).  As in the
// reference the constructor copies the input (host memory, same layout,
// packed leading dimension), factors the copy in place (here through
// LAPACKE_dgetrf / dpotrf / dgeqrf, which stage to the GPU), and fails with
// SingularMatrix without creating the object when the factorization reports
// info > 0.  Two deliberate differences: QR keeps tau alive for QR.q (qr.zig
// frees it when qr returns), and QR.q copies only the columns the factor
// storage has (qr.zig:57-68 copies m columns from an m x n array in full
// mode; orgqr overwrites the extra ones with identity columns either way).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "clapack.h"
#include "zml_linalg.h"

struct zml_plu_s {
  int layout, m, n, ld;
  double *lu;
  int *ipiv;
};

struct zml_chol_s {
  int layout, n;
  bool lower;
  double *f;
};

struct zml_qr_s {
  int layout, m, n, ld;
  double *qr;
  double *tau;
};

namespace {

bool layout_ok(int layout) { return layout == LAPACK_ROW_MAJOR || layout == LAPACK_COL_MAJOR; }

long at(int layout, int i, int j, long ld) {
  return layout == LAPACK_COL_MAJOR ? i + j * ld : i * ld + j;
}

// Packed copy (ld = rows for column-major, cols for row-major), as
// matrix.General.copy.
double *copy_matrix(int layout, int m, int n, const double *a, int lda, int *ld_out) {
  const int ld = std::max(1, layout == LAPACK_COL_MAJOR ? m : n);
  double *d = (double *)std::malloc(sizeof(double) * std::max<size_t>(1, (size_t)m * n));
  if (!d) return nullptr;
  const int outer = layout == LAPACK_COL_MAJOR ? n : m, inner = layout == LAPACK_COL_MAJOR ? m : n;
  for (int o = 0; o < outer; ++o)
    std::memcpy(d + (size_t)o * ld, a + (size_t)o * lda, sizeof(double) * inner);
  *ld_out = ld;
  return d;
}

zml_dmatrix view(double *data, int rows, int cols, int ld, int layout, int uplo, int diag) {
  zml_dmatrix v;
  v.data = data;
  v.rows = rows;
  v.cols = cols;
  v.ld = ld;
  v.layout = layout;
  v.uplo = uplo;
  v.diag = diag;
  v.owns_data = 0;
  return v;
}

// LAPACKE result -> the API's error: numerical info > 0 is SingularMatrix,
// library failures pass through.
int status_of(int info) {
  if (info > 0) return ZML_ERR_SINGULAR_MATRIX;
  if (info < 0 && info > -1000) return ZML_ERR_INVALID_ARGUMENT;
  return info;
}

int chol_new(int layout, char uplo, int n, const double *a, int lda, bool lower, zml_chol_t **out) {
  if (!out) return ZML_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  uplo = (char)(uplo == 'l' ? 'L' : uplo == 'u' ? 'U' : uplo);
  if (!layout_ok(layout) || (uplo != 'L' && uplo != 'U') || n < 0 || lda < std::max(1, n) ||
      (!a && n > 0))
    return ZML_ERR_INVALID_ARGUMENT;
  double *f = (double *)std::calloc(std::max<size_t>(1, (size_t)n * n), sizeof(double));
  if (!f) return ZML_ERR_OUT_OF_MEMORY;
  // the stored triangle, mirrored into the one being factored when they
  // differ (copyInverseUplo), the other triangle zero
  const bool src_lower = uplo == 'L';
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      if (lower ? i < j : i > j) continue;
      const bool in_src = src_lower ? i >= j : i <= j;
      f[at(layout, i, j, n)] = in_src ? a[at(layout, i, j, lda)] : a[at(layout, j, i, lda)];
    }
  const int info = n > 0 ? LAPACKE_dpotrf(layout, lower ? 'L' : 'U', n, f, n) : 0;
  if (info != 0) {
    std::free(f);
    return status_of(info);
  }
  zml_chol_t *c = (zml_chol_t *)std::malloc(sizeof(zml_chol_t));
  if (!c) {
    std::free(f);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  c->layout = layout;
  c->n = n;
  c->lower = lower;
  c->f = f;
  *out = c;
  return 0;
}

}  // namespace

extern "C" {

void zml_dmatrix_deinit(zml_dmatrix *m) {
  if (!m) return;
  if (m->owns_data) std::free(m->data);
  std::memset(m, 0, sizeof *m);
}

// ---- PLU ----
int zml_plu(int layout, int m, int n, const double *a, int lda, zml_plu_t **out) {
  if (!out) return ZML_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!layout_ok(layout) || m < 0 || n < 0 ||
      lda < std::max(1, layout == LAPACK_COL_MAJOR ? m : n) || (!a && m > 0 && n > 0))
    return ZML_ERR_INVALID_ARGUMENT;
  int ld = 1;
  double *lu = copy_matrix(layout, m, n, a, lda, &ld);
  int *ipiv = (int *)std::calloc(std::max(1, std::min(m, n)), sizeof(int));
  zml_plu_t *f = (zml_plu_t *)std::malloc(sizeof(zml_plu_t));
  if (!lu || !ipiv || !f) {
    std::free(lu);
    std::free(ipiv);
    std::free(f);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  const int info = (m > 0 && n > 0) ? LAPACKE_dgetrf(layout, m, n, lu, ld, ipiv) : 0;
  if (info != 0) {
    std::free(lu);
    std::free(ipiv);
    std::free(f);
    return status_of(info);
  }
  f->layout = layout;
  f->m = m;
  f->n = n;
  f->ld = ld;
  f->lu = lu;
  f->ipiv = ipiv;
  *out = f;
  return 0;
}

void zml_plu_deinit(zml_plu_t *f) {
  if (!f) return;
  std::free(f->lu);
  std::free(f->ipiv);
  std::free(f);
}

int zml_plu_p(const zml_plu_t *f, unsigned *perm) {
  if (!f || (!perm && f->m > 0)) return ZML_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < f->m; ++i) perm[i] = (unsigned)i;
  for (int i = std::min(f->m, f->n) - 1; i >= 0; --i) std::swap(perm[i], perm[f->ipiv[i] - 1]);
  return 0;
}

zml_dmatrix zml_plu_l(const zml_plu_t *f) {
  return view(f->lu, f->m, std::min(f->m, f->n), f->ld, f->layout, 122, 132);
}

zml_dmatrix zml_plu_u(const zml_plu_t *f) {
  return view(f->lu, std::min(f->m, f->n), f->n, f->ld, f->layout, 121, 131);
}

const int *zml_plu_ipiv(const zml_plu_t *f) { return f ? f->ipiv : nullptr; }

// ---- LLT / UTU ----
int zml_llt(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out) {
  return chol_new(layout, uplo, n, a, lda, true, out);
}

int zml_utu(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out) {
  return chol_new(layout, uplo, n, a, lda, false, out);
}

int zml_cholesky(int layout, char uplo, int n, const double *a, int lda, zml_chol_t **out) {
  const bool lower = uplo == 'L' || uplo == 'l';
  return chol_new(layout, uplo, n, a, lda, lower, out);
}

void zml_chol_deinit(zml_chol_t *f) {
  if (!f) return;
  std::free(f->f);
  std::free(f);
}

zml_dmatrix zml_chol_factor(const zml_chol_t *f) {
  return view(f->f, f->n, f->n, std::max(1, f->n), f->layout, f->lower ? 122 : 121, 131);
}

// ---- QR ----
int zml_qr(int layout, int m, int n, const double *a, int lda, zml_qr_t **out) {
  if (!out) return ZML_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!layout_ok(layout) || m < 0 || n < 0 ||
      lda < std::max(1, layout == LAPACK_COL_MAJOR ? m : n) || (!a && m > 0 && n > 0))
    return ZML_ERR_INVALID_ARGUMENT;
  int ld = 1;
  double *qr = copy_matrix(layout, m, n, a, lda, &ld);
  double *tau = (double *)std::calloc(std::max(1, std::min(m, n)), sizeof(double));
  zml_qr_t *f = (zml_qr_t *)std::malloc(sizeof(zml_qr_t));
  if (!qr || !tau || !f) {
    std::free(qr);
    std::free(tau);
    std::free(f);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  const int info = (m > 0 && n > 0) ? LAPACKE_dgeqrf(layout, m, n, qr, ld, tau) : 0;
  if (info != 0) {
    std::free(qr);
    std::free(tau);
    std::free(f);
    return status_of(info);
  }
  f->layout = layout;
  f->m = m;
  f->n = n;
  f->ld = ld;
  f->qr = qr;
  f->tau = tau;
  *out = f;
  return 0;
}

void zml_qr_deinit(zml_qr_t *f) {
  if (!f) return;
  std::free(f->qr);
  std::free(f->tau);
  std::free(f);
}

int zml_qr_q(const zml_qr_t *f, int mode, zml_dmatrix *q) {
  if (!f || !q || (mode != ZML_QR_FULL && mode != ZML_QR_ECONOMICAL))
    return ZML_ERR_INVALID_ARGUMENT;
  const int m = f->m, k = std::min(f->m, f->n);
  const int cols = mode == ZML_QR_FULL ? m : k;
  const int ldq = std::max(1, f->layout == LAPACK_COL_MAJOR ? m : cols);
  double *d = (double *)std::calloc(std::max<size_t>(1, (size_t)m * cols), sizeof(double));
  if (!d) return ZML_ERR_OUT_OF_MEMORY;
  const int ncopy = std::min(cols, f->n);
  for (int j = 0; j < ncopy; ++j)
    for (int i = 0; i < m; ++i) d[at(f->layout, i, j, ldq)] = f->qr[at(f->layout, i, j, f->ld)];
  int info = 0;
  if (k == 0)  // no reflectors: Q is the identity
    for (int j = 0; j < std::min(m, cols); ++j) d[at(f->layout, j, j, ldq)] = 1.0;
  else
    info = LAPACKE_dorgqr(f->layout, m, cols, k, d, ldq, f->tau);
  if (info != 0) {
    std::free(d);
    return status_of(info);
  }
  *q = view(d, m, cols, ldq, f->layout, 0, 0);
  q->owns_data = 1;
  return 0;
}

zml_dmatrix zml_qr_r(const zml_qr_t *f, int mode) {
  return view(f->qr, mode == ZML_QR_FULL ? f->m : std::min(f->m, f->n), f->n, f->ld, f->layout, 121,
              131);
}

const double *zml_qr_tau(const zml_qr_t *f) { return f ? f->tau : nullptr; }

}  // extern "C"
