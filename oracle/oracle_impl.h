/*
 * oracle_impl.h -- type-generic body of the zml oracle (TEST INFRASTRUCTURE).
 *
 * Included once per element type by zml_oracle.c with
 *   T  = the element type (double / float)
 *   P(x) = the exported name prefix (zo_d_x / zo_s_x)
 * Every function restates the cited Zig routine of srmadrid/zml in the same
 * loop order and the same association of each product and sum.  Column-major
 * kernels (k_*) are reached through the same row-major -> column-major
 * argument swaps as the Zig front ends.
 */

/* ---- small helpers ------------------------------------------------------ */
/* linalg/utils.zig:4-6 */
static inline long P(idx)(int order, int i, int j, int ld) {
  return order == ZO_COL ? (long)i + (long)j * ld : (long)i * ld + j;
}
/* linalg/utils.zig:13-19 */
static inline int P(col_ld)(int order, int ld) { return order == ZO_COL ? 1 : ld; }

/* ---- BLAS level 1 -------------------------------------------------------- */

/* blas/iamax.zig:11-68 (real branch 29-38): strict '>' so the first maximum
 * (lowest index) wins; NaN never replaces the running maximum. */
int P(iamax)(int n, const T *x, int incx) {
  if (n <= 0 || incx <= 0) return ZO_EINVAL;
  if (n == 1) return 0;
  int imax = 0;
  T max = ZO_ABS(x[0]);
  long ix = incx;
  for (int i = 1; i < n; ++i) {
    T absx = ZO_ABS(x[ix]);
    if (absx > max) {
      max = absx;
      imax = i;
    }
    ix += incx;
  }
  return imax;
}

/* blas/scal.zig:14-41: early return when alpha == 1. */
int P(scal)(int n, T alpha, T *x, int incx) {
  if (n < 0 || incx <= 0) return ZO_EINVAL;
  if (n == 0) return 0;
  if (alpha == (T)1) return 0;
  long ix = 0;
  for (int i = 0; i < n; ++i) {
    x[ix] = x[ix] * alpha;
    ix += incx;
  }
  return 0;
}

/* blas/swap.zig:14-55 */
int P(swap)(int n, T *x, int incx, T *y, int incy) {
  if (n < 0) return ZO_EINVAL;
  if (n == 0) return 0;
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  long iy = incy < 0 ? (long)(-n + 1) * incy : 0;
  for (int i = 0; i < n; ++i) {
    T temp = x[ix];
    x[ix] = y[iy];
    y[iy] = temp;
    ix += incx;
    iy += incy;
  }
  return 0;
}

/* blas/copy.zig */
int P(copy)(int n, const T *x, int incx, T *y, int incy) {
  if (n < 0) return ZO_EINVAL;
  if (n == 0) return 0;
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  long iy = incy < 0 ? (long)(-n + 1) * incy : 0;
  for (int i = 0; i < n; ++i) {
    y[iy] = x[ix];
    ix += incx;
    iy += incy;
  }
  return 0;
}

/* blas/axpy.zig: y += alpha * x, quick return when alpha == 0. */
int P(axpy)(int n, T alpha, const T *x, int incx, T *y, int incy) {
  if (n < 0) return ZO_EINVAL;
  if (n == 0) return 0;
  if (alpha == (T)0) return 0;
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  long iy = incy < 0 ? (long)(-n + 1) * incy : 0;
  for (int i = 0; i < n; ++i) {
    y[iy] = y[iy] + alpha * x[ix];
    ix += incx;
    iy += incy;
  }
  return 0;
}

/* ---- BLAS level 3: gemm ---------------------------------------------------- */

/* blas/gemm.zig:68-1027 (k_gemm).  For real T, conj_no_trans behaves as
 * no_trans and conj_trans as trans (conj is the identity). */
static int P(k_gemm)(int transa, int transb, int m, int n, int k, T alpha, const T *a, int lda,
                     const T *b, int ldb, T beta, T *c, int ldc) {
  const int nota = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int notb = transb == ZO_NOTRANS || transb == ZO_CONJNOTRANS;
  const int nrowa = nota ? m : k;
  const int nrowb = notb ? k : n;
  if (m < 0 || n < 0 || k < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, nrowb) ||
      ldc < ZO_MAX(1, m))
    return ZO_EINVAL;                                           /* 101-102 */
  if (m == 0 || n == 0 || ((alpha == (T)0 || k == 0) && beta == (T)1)) return 0; /* 105-108 */

#define C_(i, j) c[(long)(i) + (long)(j) * ldc]
#define A_(i, j) a[(long)(i) + (long)(j) * lda]
#define B_(i, j) b[(long)(i) + (long)(j) * ldb]
  if (alpha == (T)0) { /* 111-140 */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) C_(i, j) = beta == (T)0 ? (T)0 : C_(i, j) * beta;
    return 0;
  }
  if (notb && nota) { /* 146-191: NN axpy form */
    for (int j = 0; j < n; ++j) {
      if (beta == (T)0) {
        for (int i = 0; i < m; ++i) C_(i, j) = 0;
      } else if (beta != (T)1) {
        for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) * beta;
      }
      for (int l = 0; l < k; ++l) {
        const T temp = alpha * B_(l, j);
        for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) + temp * A_(i, l);
      }
    }
  } else if (notb && !nota) { /* 339-398: TN dot form */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) {
        T temp = 0;
        for (int l = 0; l < k; ++l) temp = temp + A_(l, i) * B_(l, j);
        if (beta == (T)0) {
          C_(i, j) = alpha * temp;
        } else if (beta == (T)1) {
          C_(i, j) = C_(i, j) + alpha * temp;
        } else {
          C_(i, j) = C_(i, j) * beta;
          C_(i, j) = C_(i, j) + alpha * temp;
        }
      }
  } else if (!notb && nota) { /* 585-634 (NT), 682-729 (NC) */
    for (int j = 0; j < n; ++j) {
      if (beta == (T)0) {
        for (int i = 0; i < m; ++i) C_(i, j) = 0;
      } else if (beta != (T)1) {
        for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) * beta;
      }
      for (int l = 0; l < k; ++l) {
        const T temp = alpha * B_(j, l);
        for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) + temp * A_(i, l);
      }
    }
  } else { /* 782-898: TT dot form */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) {
        T temp = 0;
        for (int l = 0; l < k; ++l) temp = temp + A_(l, i) * B_(j, l);
        if (beta == (T)0) {
          C_(i, j) = alpha * temp;
        } else if (beta == (T)1) {
          C_(i, j) = C_(i, j) + alpha * temp;
        } else {
          C_(i, j) = C_(i, j) * beta;
          C_(i, j) = C_(i, j) + alpha * temp;
        }
      }
  }
  return 0;
}

/* blas/gemm.zig:14-66: row-major maps to column-major by swapping the
 * operands (A<->B, m<->n). */
int P(gemm)(int order, int transa, int transb, int m, int n, int k, T alpha, const T *a, int lda,
            const T *b, int ldb, T beta, T *c, int ldc) {
  if (order == ZO_COL)
    return P(k_gemm)(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  return P(k_gemm)(transb, transa, n, m, k, alpha, b, ldb, a, lda, beta, c, ldc);
}

/* ---- BLAS level 3: trsm ---------------------------------------------------- */

/* blas/trsm.zig:66-735 (k_trsm).  The left/no-trans divisions read
 * b[k + j*lda] as written (139, 179, 224, 247) unless as-written mode is off. */
static int P(k_trsm)(int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *a,
                     int lda, T *b, int ldb) {
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int nrowa = side == ZO_LEFT ? m : n;
  const int nonunit = diag == ZO_NONUNIT;
  const long ldq = zo_trsm_as_written ? lda : ldb; /* leading dim of the quirky read */
  if (m < 0 || n < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, m)) return ZO_EINVAL; /* 91 */
  if (m == 0 || n == 0) return 0;
#define BB(i, j) b[(long)(i) + (long)(j) * ldb]
  if (alpha == (T)0) { /* 99-113 */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) BB(i, j) = 0;
    return 0;
  }
  if (side == ZO_LEFT) {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 117-201: back substitution */
        for (int j = 0; j < n; ++j) {
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * alpha;
          for (int k = m - 1; k >= 0; --k) {
            if (BB(k, j) != (T)0) {
              if (nonunit) BB(k, j) = b[(long)k + (long)j * ldq] / A_(k, k);
              for (int i = 0; i < k; ++i) BB(i, j) = BB(i, j) - BB(k, j) * A_(i, k);
            }
          }
        }
      } else { /* 202-270: forward substitution */
        for (int j = 0; j < n; ++j) {
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * alpha;
          for (int k = 0; k < m; ++k) {
            if (BB(k, j) != (T)0) {
              if (nonunit) BB(k, j) = b[(long)k + (long)j * ldq] / A_(k, k);
              for (int i = k + 1; i < m; ++i) BB(i, j) = BB(i, j) - BB(k, j) * A_(i, k);
            }
          }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 272-337: dot form, op(A) = A^T lower */
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < m; ++i) {
            T temp = BB(i, j) * alpha;
            for (int k = 0; k < i; ++k) temp = temp - A_(k, i) * BB(k, j);
            if (nonunit) temp = temp / A_(i, i);
            BB(i, j) = temp;
          }
      } else { /* 338-404 */
        for (int j = 0; j < n; ++j)
          for (int i = m - 1; i >= 0; --i) {
            T temp = BB(i, j) * alpha;
            for (int k = i + 1; k < m; ++k) temp = temp - A_(k, i) * BB(k, j);
            if (nonunit) temp = temp / A_(i, i);
            BB(i, j) = temp;
          }
      }
    }
  } else {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 408-487 */
        for (int j = 0; j < n; ++j) {
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * alpha;
          for (int k = 0; k < j; ++k)
            if (A_(k, j) != (T)0)
              for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) - A_(k, j) * BB(i, k);
          if (nonunit) {
            T temp = (T)1 / A_(j, j);
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * temp;
          }
        }
      } else { /* 488-568 */
        for (int j = n - 1; j >= 0; --j) {
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * alpha;
          for (int k = j + 1; k < n; ++k)
            if (A_(k, j) != (T)0)
              for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) - A_(k, j) * BB(i, k);
          if (nonunit) {
            T temp = (T)1 / A_(j, j);
            for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) * temp;
          }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 570-647 */
        for (int k = n - 1; k >= 0; --k) {
          if (nonunit) {
            T temp = (T)1 / A_(k, k);
            for (int i = 0; i < m; ++i) BB(i, k) = BB(i, k) * temp;
          }
          for (int j = 0; j < k; ++j)
            if (A_(j, k) != (T)0) {
              T temp = A_(j, k);
              for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) - temp * BB(i, k);
            }
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, k) = BB(i, k) * alpha;
        }
      } else { /* 648-727 */
        for (int k = 0; k < n; ++k) {
          if (nonunit) {
            T temp = (T)1 / A_(k, k);
            for (int i = 0; i < m; ++i) BB(i, k) = BB(i, k) * temp;
          }
          for (int j = k + 1; j < n; ++j)
            if (A_(j, k) != (T)0) {
              T temp = A_(j, k);
              for (int i = 0; i < m; ++i) BB(i, j) = BB(i, j) - temp * BB(i, k);
            }
          if (alpha != (T)1)
            for (int i = 0; i < m; ++i) BB(i, k) = BB(i, k) * alpha;
        }
      }
    }
  }
#undef BB
  return 0;
}

/* blas/trsm.zig:18-64: row-major -> side.invert(), uplo.invert(), m<->n. */
int P(trsm)(int order, int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *a,
            int lda, T *b, int ldb) {
  if (order == ZO_COL) return P(k_trsm)(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return P(k_trsm)(side == ZO_LEFT ? ZO_RIGHT : ZO_LEFT, uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER,
                   transa, diag, n, m, alpha, a, lda, b, ldb);
}

/* ---- BLAS level 3: syrk ---------------------------------------------------- */

/* blas/syrk.zig:60-366 (k_syrk).  Rejects the conjugate transposes (82-84). */
static int P(k_syrk)(int uplo, int trans, int n, int k, T alpha, const T *a, int lda, T beta, T *c,
                     int ldc) {
  const int nrowa = trans == ZO_NOTRANS ? n : k;
  if (trans == ZO_CONJNOTRANS || trans == ZO_CONJTRANS || n < 0 || k < 0 ||
      lda < ZO_MAX(1, nrowa) || ldc < ZO_MAX(1, n))
    return ZO_EINVAL;
  if (n == 0 || ((alpha == (T)0 || k == 0) && beta == (T)1)) return 0; /* 87-90 */
  if (alpha == (T)0) {                                                 /* 93-151 */
    for (int j = 0; j < n; ++j) {
      int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      for (int i = i0; i < i1; ++i) C_(i, j) = beta == (T)0 ? (T)0 : C_(i, j) * beta;
    }
    return 0;
  }
  if (trans == ZO_NOTRANS) { /* 153-252 */
    for (int j = 0; j < n; ++j) {
      int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      if (beta == (T)0) {
        for (int i = i0; i < i1; ++i) C_(i, j) = 0;
      } else if (beta != (T)1) {
        for (int i = i0; i < i1; ++i) C_(i, j) = C_(i, j) * beta;
      }
      for (int l = 0; l < k; ++l) {
        if (A_(j, l) != (T)0) {
          const T temp = alpha * A_(j, l);
          for (int i = i0; i < i1; ++i) C_(i, j) = C_(i, j) + temp * A_(i, l);
        }
      }
    }
  } else { /* 253-359 */
    for (int j = 0; j < n; ++j) {
      int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      for (int i = i0; i < i1; ++i) {
        T temp = 0;
        for (int l = 0; l < k; ++l) temp = temp + A_(l, i) * A_(l, j);
        if (beta == (T)0) {
          C_(i, j) = alpha * temp;
        } else {
          C_(i, j) = C_(i, j) * beta;
          C_(i, j) = C_(i, j) + alpha * temp;
        }
      }
    }
  }
  return 0;
}

/* blas/syrk.zig:15-58: row-major -> uplo.invert(), trans.invert(). */
int P(syrk)(int order, int uplo, int trans, int n, int k, T alpha, const T *a, int lda, T beta,
            T *c, int ldc) {
  if (order == ZO_COL) return P(k_syrk)(uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
  return P(k_syrk)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, zo_trans_invert(trans), n, k, alpha, a,
                   lda, beta, c, ldc);
}

/* ---- LAPACK: machine constants and LU ---------------------------------------- */

/* lapack/lamch.zig:15-78 with rnd == 1: eps = floatEps/2, sfmin = floatMin
 * (1/floatMax is smaller than floatMin for binary32/64). */
T P(lamch)(char cmach) {
  const T eps = ZO_EPS * (T)0.5;
  switch (cmach) {
    case 'e': return eps;
    case 's': {
      T sfmin = ZO_TMIN;
      const T small = (T)1 / ZO_TMAX;
      if (small >= sfmin) sfmin = small * ((T)1 + eps);
      return sfmin;
    }
    case 'b': return 2;
    case 'p': return eps * 2;
    case 'o': return ZO_TMAX;
    case 'u': return ZO_TMIN;
    default: return eps;
  }
}

/* lapack/laswp.zig:12-96: interchanges in blocks of 32 columns, then the
 * remainder; negative incx walks the pivots backwards. ipiv is 1-based. */
int P(laswp)(int order, int n, T *a, int lda, int k1, int k2, const int *ipiv, int incx) {
  if (n < 0 || (order == ZO_ROW && lda < ZO_MAX(1, n)) || incx == 0) return ZO_EINVAL;
  if (n == 0) return 0;
  int ix0, I1, I2, inc;
  if (incx > 0) {
    ix0 = k1 - 1; I1 = k1 - 1; I2 = k2 - 1; inc = 1;
  } else {
    ix0 = k1 - 1 + (k1 - k2) * incx; I1 = k2 - 1; I2 = k1 - 1; inc = -1;
  }
  const int n32 = (n >> 5) << 5;
  if (n32 != 0) {
    for (int j = 0; j < n32; j += 32) {
      int ix = ix0;
      for (int i = I1; i != I2 + inc; i += inc) {
        const int ip = ipiv[ix] - 1;
        if (ip != i)
          for (int k = j; k < j + 32; ++k) {
            T temp = a[P(idx)(order, i, k, lda)];
            a[P(idx)(order, i, k, lda)] = a[P(idx)(order, ip, k, lda)];
            a[P(idx)(order, ip, k, lda)] = temp;
          }
        ix += incx;
      }
    }
  }
  if (n32 != n) {
    int ix = ix0;
    for (int i = I1; i != I2 + inc; i += inc) {
      const int ip = ipiv[ix] - 1;
      if (ip != i)
        for (int k = n32; k < n; ++k) {
          T temp = a[P(idx)(order, i, k, lda)];
          a[P(idx)(order, i, k, lda)] = a[P(idx)(order, ip, k, lda)];
          a[P(idx)(order, ip, k, lda)] = temp;
        }
      ix += incx;
    }
  }
  return 0;
}

/* Test hook, off unless set: the one-column step of getrf2 records each
 * column's relative gap between its largest and second-largest candidate,
 * (top1 - top2) / top1, at margin_out[ipiv - margin_ipiv].  The parity tests
 * stop comparing pivots at the first column whose gap is a near-tie. */
static double *P(margin_out) = 0;
static const int *P(margin_ipiv) = 0;

/* lapack/getrf2.zig:14-210: recursive LU with partial pivoting. */
int P(getrf2)(int order, int m, int n, T *a, int lda, int *ipiv) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  int info = 0;
  if (m == 0 || n == 0) return info;
  if (m == 1) { /* 35-40 */
    ipiv[0] = 1;
    if (a[0] == (T)0) info = 1;
  } else if (n == 1) { /* 41-89 */
    const T sfmin = P(lamch)('s');
    const int ii = P(iamax)(m, a, P(col_ld)(order, lda));
    ipiv[0] = ii + 1;
    if (P(margin_out)) {
      const double top = ZO_ABS(a[P(idx)(order, ii, 0, lda)]);
      double second = 0;
      for (int i = 0; i < m; ++i)
        if (i != ii && ZO_ABS(a[P(idx)(order, i, 0, lda)]) > second)
          second = ZO_ABS(a[P(idx)(order, i, 0, lda)]);
      P(margin_out)[ipiv - P(margin_ipiv)] = top > 0 ? (top - second) / top : 0.0;
    }
    if (a[P(idx)(order, ii, 0, lda)] != (T)0) {
      if (ii != 0) {
        T temp = a[0];
        a[0] = a[P(idx)(order, ii, 0, lda)];
        a[P(idx)(order, ii, 0, lda)] = temp;
      }
      if (ZO_ABS(a[0]) >= sfmin) {
        P(scal)(m - 1, (T)1 / a[0], a + P(idx)(order, 1, 0, lda), P(col_ld)(order, lda));
      } else {
        for (int i = 0; i < m - 1; ++i)
          a[P(idx)(order, i + 1, 0, lda)] = a[P(idx)(order, i + 1, 0, lda)] / a[0];
      }
    } else {
      info = 1;
    }
  } else { /* 90-196 */
    const int n1 = ZO_MIN(m, n) / 2;
    const int n2 = n - n1;
    int iinfo = P(getrf2)(order, m, n1, a, lda, ipiv);
    if (info == 0 && iinfo > 0) info = iinfo;
    P(laswp)(order, n2, a + P(idx)(order, 0, n1, lda), lda, 1, n1, ipiv, 1);
    P(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, n1, n2, (T)1, a, lda,
            a + P(idx)(order, 0, n1, lda), lda);
    P(gemm)(order, ZO_NOTRANS, ZO_NOTRANS, m - n1, n2, n1, (T)-1, a + P(idx)(order, n1, 0, lda),
            lda, a + P(idx)(order, 0, n1, lda), lda, (T)1, a + P(idx)(order, n1, n1, lda), lda);
    iinfo = P(getrf2)(order, m - n1, n2, a + P(idx)(order, n1, n1, lda), lda, ipiv + n1);
    if (info == 0 && iinfo > 0) info = iinfo + n1;
    for (int i = n1; i < ZO_MIN(m, n); ++i) ipiv[i] = ipiv[i] + n1;
    P(laswp)(order, n1, a, lda, n1 + 1, ZO_MIN(m, n), ipiv, 1);
  }
  return info;
}

/* lapack/getrf.zig:14-152: right-looking blocked LU, nb = ilaenv = 64. */
int P(getrf)(int order, int m, int n, T *a, int lda, int *ipiv) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  int info = 0;
  if (m == 0 || n == 0) return info;
  const int nb = zo_ilaenv(1, "DGETRF", m, n, -1, -1);
  const int mn = ZO_MIN(m, n);
  if (nb <= 1 || nb >= mn) return P(getrf2)(order, m, n, a, lda, ipiv);
  for (int j = 0; j < mn; j += nb) {
    const int jb = ZO_MIN(mn - j, nb);
    const int iinfo = P(getrf2)(order, m - j, jb, a + P(idx)(order, j, j, lda), lda, ipiv + j);
    if (info == 0 && iinfo > 0) info = iinfo + j;
    for (int i = j; i < ZO_MIN(m, j + jb); ++i) ipiv[i] = ipiv[i] + j;
    P(laswp)(order, j, a, lda, j + 1, j + jb, ipiv, 1);
    if (j + jb < n) {
      P(laswp)(order, n - j - jb, a + P(idx)(order, 0, j + jb, lda), lda, j + 1, j + jb, ipiv, 1);
      P(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, jb, n - j - jb, (T)1,
              a + P(idx)(order, j, j, lda), lda, a + P(idx)(order, j, j + jb, lda), lda);
      if (j + jb < m)
        P(gemm)(order, ZO_NOTRANS, ZO_NOTRANS, m - j - jb, n - j - jb, jb, (T)-1,
                a + P(idx)(order, j + jb, j, lda), lda, a + P(idx)(order, j, j + jb, lda), lda,
                (T)1, a + P(idx)(order, j + jb, j + jb, lda), lda);
    }
  }
  return info;
}

/* lapack/getrs.zig:13-142 */
int P(getrs)(int order, int trans, int n, int nrhs, const T *a, int lda, const int *ipiv, T *b,
             int ldb) {
  const int nota = trans == ZO_NOTRANS || trans == ZO_CONJNOTRANS;
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  if (nota) {
    P(laswp)(order, nrhs, b, ldb, 1, n, ipiv, 1);
    P(trsm)(order, ZO_LEFT, ZO_LOWER, trans, ZO_UNIT, n, nrhs, (T)1, a, lda, b, ldb);
    P(trsm)(order, ZO_LEFT, ZO_UPPER, trans, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
  } else {
    P(trsm)(order, ZO_LEFT, ZO_UPPER, trans, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
    P(trsm)(order, ZO_LEFT, ZO_LOWER, trans, ZO_UNIT, n, nrhs, (T)1, a, lda, b, ldb);
    P(laswp)(order, nrhs, b, ldb, 1, n, ipiv, -1);
  }
  return 0;
}

/* lapack/gesv.zig:13-70 */
int P(gesv)(int order, int n, int nrhs, T *a, int lda, int *ipiv, T *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  int info = P(getrf)(order, n, n, a, lda, ipiv);
  if (info == 0) P(getrs)(order, ZO_NOTRANS, n, nrhs, a, lda, ipiv, b, ldb);
  return info;
}

/* ---- LAPACK: Cholesky ------------------------------------------------------ */

/* lapack/potrf2.zig:17-217: recursive Cholesky. */
int P(potrf2)(int order, int uplo, int n, T *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0) return 0;
  if (n == 1) { /* 37-54 */
    const T ajj = a[0];
    if (ajj <= (T)0 || ajj != ajj) return 1;
    a[0] = ZO_SQRT(ajj);
    return 0;
  }
  const int n1 = n / 2, n2 = n - n1;
  int iinfo = P(potrf2)(order, uplo, n1, a, lda);
  if (iinfo != 0) return iinfo;
  if (uplo == ZO_UPPER) { /* 72-118 */
    P(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, n1, n2, (T)1, a, lda,
            a + P(idx)(order, 0, n1, lda), lda);
    P(syrk)(order, uplo, ZO_TRANS, n2, n1, (T)-1, a + P(idx)(order, 0, n1, lda), lda, (T)1,
            a + P(idx)(order, n1, n1, lda), lda);
  } else { /* 133-190 */
    P(trsm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n2, n1, (T)1, a, lda,
            a + P(idx)(order, n1, 0, lda), lda);
    P(syrk)(order, uplo, ZO_NOTRANS, n2, n1, (T)-1, a + P(idx)(order, n1, 0, lda), lda, (T)1,
            a + P(idx)(order, n1, n1, lda), lda);
  }
  iinfo = P(potrf2)(order, uplo, n2, a + P(idx)(order, n1, n1, lda), lda);
  if (iinfo != 0) return iinfo + n1;
  return 0;
}

/* lapack/potrf.zig:17-240: blocked left-looking Cholesky, nb = 64. */
int P(potrf)(int order, int uplo, int n, T *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0) return 0;
  const int nb = zo_ilaenv(1, "DPOTRF", n, -1, -1, -1);
  if (nb <= 1 || nb >= n) return P(potrf2)(order, uplo, n, a, lda);
  int info = 0;
  if (uplo == ZO_UPPER) { /* 52-141 */
    for (int j = 0; j < n; j += nb) {
      const int jb = ZO_MIN(nb, n - j);
      P(syrk)(order, ZO_UPPER, ZO_TRANS, jb, j, (T)-1, a + P(idx)(order, 0, j, lda), lda, (T)1,
              a + P(idx)(order, j, j, lda), lda);
      info = P(potrf2)(order, ZO_UPPER, jb, a + P(idx)(order, j, j, lda), lda);
      if (info != 0) return info + j;
      if (j + jb < n) {
        P(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, jb, n - j - jb, j, (T)-1,
                a + P(idx)(order, 0, j, lda), lda, a + P(idx)(order, 0, j + jb, lda), lda, (T)1,
                a + P(idx)(order, j, j + jb, lda), lda);
        P(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, jb, n - j - jb, (T)1,
                a + P(idx)(order, j, j, lda), lda, a + P(idx)(order, j, j + jb, lda), lda);
      }
    }
  } else { /* 144-231 */
    for (int j = 0; j < n; j += nb) {
      const int jb = ZO_MIN(nb, n - j);
      P(syrk)(order, ZO_LOWER, ZO_NOTRANS, jb, j, (T)-1, a + P(idx)(order, j, 0, lda), lda, (T)1,
              a + P(idx)(order, j, j, lda), lda);
      info = P(potrf2)(order, ZO_LOWER, jb, a + P(idx)(order, j, j, lda), lda);
      if (info != 0) return info + j;
      if (j + jb < n) {
        P(gemm)(order, ZO_NOTRANS, ZO_CONJTRANS, n - j - jb, jb, j, (T)-1,
                a + P(idx)(order, j + jb, 0, lda), lda, a + P(idx)(order, j, 0, lda), lda, (T)1,
                a + P(idx)(order, j + jb, j, lda), lda);
        P(trsm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n - j - jb, jb, (T)1,
                a + P(idx)(order, j, j, lda), lda, a + P(idx)(order, j + jb, j, lda), lda);
      }
    }
  }
  return info;
}

/* lapack/potrs.zig:15-117 */
int P(potrs)(int order, int uplo, int n, int nrhs, const T *a, int lda, T *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  if (uplo == ZO_UPPER) {
    P(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
    P(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
  } else {
    P(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
    P(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n, nrhs, (T)1, a, lda, b, ldb);
  }
  return 0;
}

/* lapack/posv.zig:15-70 */
int P(posv)(int order, int uplo, int n, int nrhs, T *a, int lda, T *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  int info = P(potrf)(order, uplo, n, a, lda);
  if (info == 0) P(potrs)(order, uplo, n, nrhs, a, lda, b, ldb);
  return info;
}

#undef A_
#undef B_
#undef C_
