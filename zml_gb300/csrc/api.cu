// api.cu -- zml.linalg's decomposition objects (include/zml_linalg.h) over
// the library's GPU LAPACK.  Host code only.
//
// Mirrors src/linalg/lu.zig:62-216 (PLU, plu), cholesky.zig:17-188 (LLT, UTU,
// llt, utu, cholesky), bunchkaufman.zig:20-726 (LDLT, UDUT, ldlt, udut,
// bunchkaufman) and qr.zig:21-263 (QR, qr, QR.q, QR.r).  As in the
// reference the constructor copies the input (host memory, same layout,
// packed leading dimension), factors the copy in place (here through
// LAPACKE_dgetrf / dpotrf / dgeqrf, which stage to the GPU), and fails with
// SingularMatrix without creating the object when the factorization reports
// info > 0.  Two deliberate differences: QR keeps tau alive for QR.q (qr.zig
// frees it when qr returns), and QR.q copies only the columns the factor
// storage has (qr.zig:57-68 copies m columns from an m x n array in full
// mode; orgqr overwrites the extra ones with identity columns either way).
//
// The matmul facade (linalg/matmul.zig:19) routes its dense cases to the
// library's GEMM: matrix x matrix as matmul/dgedge.zig:11-41 (result in a's
// layout, b transposed when its layout differs), matrix x vector and vector
// x matrix as dgedv.zig:11 / dvdge.zig:11 (gemv, here one-column GEMMs).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "cblas.h"
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

// LDLT (upper false) or UDUT (upper true): the packed n x n dsytrf factor in
// `layout` and its ipiv (LAPACK's convention, 1-based).
struct zml_bk_s {
  int layout, n;
  bool upper;
  double *f;
  int *ipiv;
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

zml_bk_s *bk_new(int layout, int n, bool upper, double *f, const int *ipiv) {
  zml_bk_s *o = (zml_bk_s *)std::malloc(sizeof(zml_bk_s));
  int *p = (int *)std::malloc(sizeof(int) * std::max(1, n));
  if (!o || !p) {
    std::free(o);
    std::free(p);
    return nullptr;
  }
  if (n > 0) std::memcpy(p, ipiv, sizeof(int) * n);
  o->layout = layout;
  o->n = n;
  o->upper = upper;
  o->f = f;
  o->ipiv = p;
  return o;
}

// ldlt / udut (bunchkaufman.zig:180-707, the LAPACKE branch): the stored
// triangle (mirrored when it is not the one factored) into a zeroed packed
// copy, then dsytrf on the factored triangle.
int bk_factor(int layout, char uplo, int n, const double *a, int lda, bool upper, zml_bk_s **out) {
  if (!out) return ZML_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  uplo = (char)(uplo == 'l' ? 'L' : uplo == 'u' ? 'U' : uplo);
  if (!layout_ok(layout) || (uplo != 'L' && uplo != 'U') || n < 0 || lda < std::max(1, n) ||
      (!a && n > 0))
    return ZML_ERR_INVALID_ARGUMENT;
  double *f = (double *)std::calloc(std::max<size_t>(1, (size_t)n * n), sizeof(double));
  int *ipiv = (int *)std::calloc(std::max(1, n), sizeof(int));
  if (!f || !ipiv) {
    std::free(f);
    std::free(ipiv);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  const bool src_lower = uplo == 'L';
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      if (upper ? i > j : i < j) continue;
      const bool in_src = src_lower ? i >= j : i <= j;
      f[at(layout, i, j, n)] = in_src ? a[at(layout, i, j, lda)] : a[at(layout, j, i, lda)];
    }
  const int info = n > 0 ? LAPACKE_dsytrf(layout, upper ? 'U' : 'L', n, f, n, ipiv) : 0;
  if (info != 0) {
    std::free(f);
    std::free(ipiv);
    // bunchkaufman.zig:231-232: any non-zero info fails the factorization
    return info > 0 ? ZML_ERR_FACTORIZATION_FAILED : status_of(info);
  }
  zml_bk_s *o = bk_new(layout, n, upper, f, ipiv);
  std::free(ipiv);
  if (!o) {
    std::free(f);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  *out = o;
  return 0;
}

int bk_init(int layout, int n, const double *f, int ld, const int *ipiv, bool upper,
            zml_bk_s **out) {
  if (!out) return ZML_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!layout_ok(layout) || n < 0 || ld < std::max(1, n) || ((!f || !ipiv) && n > 0))
    return ZML_ERR_INVALID_ARGUMENT;
  // every interchange row inside the matrix; a 2x2 block's partner inside too
  for (int i = 0; i < n; ++i) {
    const int r = ipiv[i] > 0 ? ipiv[i] : -ipiv[i];
    if (ipiv[i] == 0 || r > n) return ZML_ERR_INVALID_ARGUMENT;
    if (ipiv[i] < 0 && (upper ? i == 0 : i == n - 1)) return ZML_ERR_INVALID_ARGUMENT;
  }
  int ldc = 1;
  double *c = copy_matrix(layout, n, n, f, ld, &ldc);
  if (!c) return ZML_ERR_OUT_OF_MEMORY;
  zml_bk_s *o = bk_new(layout, n, upper, c, ipiv);
  if (!o) {
    std::free(c);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  *out = o;
  return 0;
}

// lpermute / upermute (bunchkaufman.zig:426-443, 690-707): ipiv's
// interchanges applied to the identity in factorization order (forward for
// L, backward for U); a 2x2 block's interchange acts on its second (L) or
// first (U) row.
void bk_permute(const zml_bk_s *o, unsigned *p) {
  const int n = o->n;
  const int *ipiv = o->ipiv;
  for (int i = 0; i < n; ++i) p[i] = (unsigned)i;
  if (!o->upper) {
    for (int i = 0; i < n; ++i) {
      if (ipiv[i] > 0) {
        std::swap(p[i], p[ipiv[i] - 1]);
      } else {
        std::swap(p[i + 1], p[-ipiv[i] - 1]);
        ++i;
      }
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      if (ipiv[i] > 0) {
        std::swap(p[i], p[ipiv[i] - 1]);
      } else {
        std::swap(p[i - 1], p[-ipiv[i] - 1]);
        --i;
      }
    }
  }
}

// lconvert / uconvert (bunchkaufman.zig:312-424, 576-688): walks the blocks
// in factorization order, tracking the permutation p as bk_permute does;
// each block's multiplier columns are copied into t (when given) and the
// rows of the columns already placed (L: left of the block, U: right of it)
// are swapped along p's cycle until p[i] == i; D's blocks go to
// (sub, diag, sup) (when given), zero between blocks.  Returns
// ZML_ERR_OUT_OF_MEMORY, with nothing written, when the permutation's scratch
// cannot be allocated.
int bk_convert(const zml_bk_s *o, double *t, double *sub, double *diag, double *sup) {
  const int n = o->n, lay = o->layout;
  const int *ipiv = o->ipiv;
  const double *a = o->f;
  unsigned *p = (unsigned *)std::malloc(sizeof(unsigned) * std::max(1, n));
  if (!p) return ZML_ERR_OUT_OF_MEMORY;
  for (int i = 0; i < n; ++i) p[i] = (unsigned)i;
  auto A = [&](int i, int j) { return a[at(lay, i, j, n)]; };
  auto T = [&](int i, int j) -> double & { return t[at(lay, i, j, n)]; };
  auto settle = [&](int i, int c0, int c1) {
    while (p[i] != (unsigned)i) {
      const unsigned jr = p[i];
      if (t)
        for (int j = c0; j < c1; ++j) std::swap(T(i, j), T((int)jr, j));
      std::swap(p[i], p[jr]);
    }
  };
  if (!o->upper) {
    for (int i = 0; i < n; ++i) {
      if (ipiv[i] > 0) {
        std::swap(p[i], p[ipiv[i] - 1]);
        if (diag) {
          diag[i] = A(i, i);
          if (i < n - 1) sub[i] = sup[i] = 0.0;
        }
        if (t)
          for (int j = i + 1; j < n; ++j) T(j, i) = A(j, i);
        settle(i, 0, i);
      } else {
        std::swap(p[i + 1], p[-ipiv[i] - 1]);
        if (diag) {
          diag[i] = A(i, i);
          sub[i] = sup[i] = A(i + 1, i);
          diag[i + 1] = A(i + 1, i + 1);
        }
        if (t) {
          T(i + 1, i) = 0.0;
          for (int j = i + 2; j < n; ++j) {
            T(j, i) = A(j, i);
            T(j, i + 1) = A(j, i + 1);
          }
        }
        ++i;
        settle(i, 0, i - 1);
        if (diag && i < n - 1) sub[i] = sup[i] = 0.0;
      }
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      if (ipiv[i] > 0) {
        std::swap(p[i], p[ipiv[i] - 1]);
        if (diag) {
          diag[i] = A(i, i);
          if (i < n - 1) sub[i] = sup[i] = 0.0;
        }
        if (t)
          for (int j = 0; j < i; ++j) T(j, i) = A(j, i);
        settle(i, i + 1, n);
      } else {
        std::swap(p[i - 1], p[-ipiv[i] - 1]);
        if (diag) {
          diag[i - 1] = A(i - 1, i - 1);
          sub[i - 1] = sup[i - 1] = A(i - 1, i);
          diag[i] = A(i, i);
          if (i < n - 1) sub[i] = sup[i] = 0.0;
        }
        if (t) {
          for (int j = 0; j < i - 1; ++j) {
            T(j, i - 1) = A(j, i - 1);
            T(j, i) = A(j, i);
          }
          T(i - 1, i) = 0.0;
        }
        --i;
        settle(i, i + 2, n);
      }
    }
  }
  std::free(p);
  return 0;
}

// The unit triangle of the factor, owned by the caller; NULL data when an
// allocation fails.
zml_dmatrix bk_triangle(const zml_bk_s *o) {
  const int n = o->n;
  double *t = (double *)std::calloc(std::max<size_t>(1, (size_t)n * n), sizeof(double));
  if (t) {
    for (int i = 0; i < n; ++i) t[at(o->layout, i, i, n)] = 1.0;
    if (bk_convert(o, t, nullptr, nullptr, nullptr) != 0) {
      std::free(t);
      t = nullptr;
    }
  }
  zml_dmatrix v = view(t, n, n, std::max(1, n), o->layout, o->upper ? 121 : 122, 132);
  v.owns_data = t ? 1 : 0;
  return v;
}

int bk_d(const zml_bk_s *o, double *sub, double *diag, double *sup) {
  if ((o->n > 0 && !diag) || (o->n > 1 && (!sub || !sup))) return ZML_ERR_INVALID_ARGUMENT;
  return bk_convert(o, nullptr, sub, diag, sup);
}

void bk_free(zml_bk_s *o) {
  if (!o) return;
  std::free(o->f);
  std::free(o->ipiv);
  std::free(o);
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

namespace {

bool matrix_ok(const zml_dmatrix *x) {
  if (!x || !layout_ok(x->layout) || x->rows < 0 || x->cols < 0) return false;
  if (x->uplo != 0 && x->uplo != 121 && x->uplo != 122) return false;
  if (x->uplo != 0 && x->diag != 131 && x->diag != 132) return false;
  const int inner = x->layout == LAPACK_COL_MAJOR ? x->rows : x->cols;
  if (x->ld < std::max(1, inner)) return false;
  return x->data || (long)x->rows * x->cols == 0;
}

// Element (i, j) of the dense matrix a view stands for.
double element(const zml_dmatrix &x, int i, int j) {
  if (x.uplo != 0) {
    if (x.uplo == 121 ? i > j : i < j) return 0.0;
    if (i == j && x.diag == 132) return 1.0;
  }
  return x.data[at(x.layout, i, j, x.ld)];
}

// A general operand for GEMM: the view itself, or (triangular views) a packed
// dense copy in the view's layout, returned in *tmp for the caller to free.
const double *operand(const zml_dmatrix &x, int *ld, double **tmp) {
  *tmp = nullptr;
  if (x.uplo == 0) {
    *ld = x.ld;
    return x.data;
  }
  const int pld = std::max(1, x.layout == LAPACK_COL_MAJOR ? x.rows : x.cols);
  double *d = (double *)std::malloc(sizeof(double) * std::max<size_t>(1, (size_t)x.rows * x.cols));
  if (!d) return nullptr;
  for (int i = 0; i < x.rows; ++i)
    for (int j = 0; j < x.cols; ++j) d[at(x.layout, i, j, pld)] = element(x, i, j);
  *tmp = d;
  *ld = pld;
  return d;
}

long vindex(int i, int len, int inc) { return inc > 0 ? (long)i * inc : (long)(len - 1 - i) * -inc; }

// y (len_y) = op(a) x (len_x), op = a or a^T, through a one-column GEMM.
int gemv_facade(const zml_dmatrix *a, bool trans, const double *x, int incx, double *y,
                int incy) {
  if (!matrix_ok(a) || incx == 0 || incy == 0) return ZML_ERR_INVALID_ARGUMENT;
  const int len_x = trans ? a->rows : a->cols, len_y = trans ? a->cols : a->rows;
  if ((!x && len_x > 0) || (!y && len_y > 0)) return ZML_ERR_INVALID_ARGUMENT;
  if (len_y == 0) return 0;
  double *xc = (double *)std::malloc(sizeof(double) * std::max(1, len_x));
  double *yc = (double *)std::malloc(sizeof(double) * len_y);
  double *tmp = nullptr;
  int lda = 0;
  const double *A = xc && yc ? operand(*a, &lda, &tmp) : nullptr;
  if (!A) {
    std::free(xc);
    std::free(yc);
    return ZML_ERR_OUT_OF_MEMORY;
  }
  for (int i = 0; i < len_x; ++i) xc[i] = x[vindex(i, len_x, incx)];
  if (len_x == 0) {
    std::fill(yc, yc + len_y, 0.0);
  } else {
    // one column: ld 1 in row-major order, the vector length in column-major
    const bool col = a->layout == LAPACK_COL_MAJOR;
    cblas_dgemm((CBLAS_ORDER)a->layout, trans ? CblasTrans : CblasNoTrans, CblasNoTrans, len_y, 1,
                len_x, 1.0, A, lda, xc, col ? len_x : 1, 0.0, yc, col ? len_y : 1);
  }
  for (int i = 0; i < len_y; ++i) y[vindex(i, len_y, incy)] = yc[i];
  std::free(tmp);
  std::free(xc);
  std::free(yc);
  return 0;
}

}  // namespace

extern "C" {

int zml_dmatmul(const zml_dmatrix *a, const zml_dmatrix *b, zml_dmatrix *c) {
  if (!c) return ZML_ERR_INVALID_ARGUMENT;
  std::memset(c, 0, sizeof *c);
  if (!matrix_ok(a) || !matrix_ok(b)) return ZML_ERR_INVALID_ARGUMENT;
  if (a->cols != b->rows) return ZML_ERR_DIMENSION_MISMATCH;
  const int m = a->rows, k = a->cols, n = b->cols;
  const int layout = a->layout;
  const int ldc = std::max(1, layout == LAPACK_COL_MAJOR ? m : n);
  double *d = (double *)std::calloc(std::max<size_t>(1, (size_t)m * n), sizeof(double));
  if (!d) return ZML_ERR_OUT_OF_MEMORY;
  if (m > 0 && n > 0 && k > 0) {
    double *ta = nullptr, *tb = nullptr;
    int lda = 0, ldb = 0;
    const double *A = operand(*a, &lda, &ta), *B = operand(*b, &ldb, &tb);
    if (!A || !B) {
      std::free(ta);
      std::free(tb);
      std::free(d);
      return ZML_ERR_OUT_OF_MEMORY;
    }
    cblas_dgemm((CBLAS_ORDER)layout, CblasNoTrans,
                b->layout == layout ? CblasNoTrans : CblasTrans, m, n, k, 1.0, A, lda, B, ldb, 0.0,
                d, ldc);
    std::free(ta);
    std::free(tb);
  }
  *c = view(d, m, n, ldc, layout, 0, 0);
  c->owns_data = 1;
  return 0;
}

int zml_dmatvec(const zml_dmatrix *a, const double *x, int incx, double *y, int incy) {
  return gemv_facade(a, false, x, incx, y, incy);
}

int zml_dvecmat(const double *x, int incx, const zml_dmatrix *b, double *y, int incy) {
  return gemv_facade(b, true, x, incx, y, incy);
}

// ---- Bunch-Kaufman ----
int zml_ldlt(int layout, char uplo, int n, const double *a, int lda, zml_ldlt_t **out) {
  return bk_factor(layout, uplo, n, a, lda, false, out);
}

int zml_udut(int layout, char uplo, int n, const double *a, int lda, zml_udut_t **out) {
  return bk_factor(layout, uplo, n, a, lda, true, out);
}

int zml_bunchkaufman(int layout, char uplo, int n, const double *a, int lda, zml_ldlt_t **lo,
                     zml_udut_t **up) {
  if (!lo || !up) return ZML_ERR_INVALID_ARGUMENT;
  *lo = *up = nullptr;
  if (uplo == 'L' || uplo == 'l') return bk_factor(layout, uplo, n, a, lda, false, lo);
  if (uplo == 'U' || uplo == 'u') return bk_factor(layout, uplo, n, a, lda, true, up);
  return ZML_ERR_INVALID_ARGUMENT;
}

int zml_ldlt_init(int layout, int n, const double *f, int ld, const int *ipiv, zml_ldlt_t **out) {
  return bk_init(layout, n, f, ld, ipiv, false, out);
}

int zml_udut_init(int layout, int n, const double *f, int ld, const int *ipiv, zml_udut_t **out) {
  return bk_init(layout, n, f, ld, ipiv, true, out);
}

void zml_ldlt_deinit(zml_ldlt_t *f) { bk_free(f); }
void zml_udut_deinit(zml_udut_t *f) { bk_free(f); }

int zml_ldlt_p(const zml_ldlt_t *f, unsigned *perm) {
  if (!f || f->upper || (!perm && f->n > 0)) return ZML_ERR_INVALID_ARGUMENT;
  bk_permute(f, perm);
  return 0;
}

int zml_udut_p(const zml_udut_t *f, unsigned *perm) {
  if (!f || !f->upper || (!perm && f->n > 0)) return ZML_ERR_INVALID_ARGUMENT;
  bk_permute(f, perm);
  return 0;
}

zml_dmatrix zml_ldlt_l(const zml_ldlt_t *f) {
  if (!f || f->upper) return view(nullptr, 0, 0, 1, LAPACK_COL_MAJOR, 0, 0);
  return bk_triangle(f);
}

zml_dmatrix zml_udut_u(const zml_udut_t *f) {
  if (!f || !f->upper) return view(nullptr, 0, 0, 1, LAPACK_COL_MAJOR, 0, 0);
  return bk_triangle(f);
}

int zml_ldlt_d(const zml_ldlt_t *f, double *sub, double *diag, double *sup) {
  if (!f || f->upper) return ZML_ERR_INVALID_ARGUMENT;
  return bk_d(f, sub, diag, sup);
}

int zml_udut_d(const zml_udut_t *f, double *sub, double *diag, double *sup) {
  if (!f || !f->upper) return ZML_ERR_INVALID_ARGUMENT;
  return bk_d(f, sub, diag, sup);
}

const int *zml_ldlt_ipiv(const zml_ldlt_t *f) { return f ? f->ipiv : nullptr; }
const int *zml_udut_ipiv(const zml_udut_t *f) { return f ? f->ipiv : nullptr; }

}  // extern "C"
