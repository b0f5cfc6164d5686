/*
 * oracle_qr_impl.h -- type-generic Householder QR part of the zml oracle
 * (TEST INFRASTRUCTURE).  Included after oracle_impl.h with the same T / P.
 * Direction codes: 'F' forward / 'B' backward; storage 'C' columnwise /
 * 'R' rowwise (lapack.zig:52-75).
 */

#define A_(i, j) a[(long)(i) + (long)(j) * lda]
#define B_(i, j) b[(long)(i) + (long)(j) * ldb]

/* blas/trmm.zig:65-724 (k_trmm) */
static int P(k_trmm)(int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *a,
                     int lda, T *b, int ldb) {
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int nonunit = diag == ZO_NONUNIT;
  const int nrowa = side == ZO_LEFT ? m : n;
  if (m < 0 || n < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, m)) return ZO_EINVAL;
  if (m == 0 || n == 0) return 0;
  if (alpha == (T)0) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) B_(i, j) = 0;
    return 0;
  }
  if (side == ZO_LEFT) {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 118-190 */
        for (int j = 0; j < n; ++j)
          for (int k = 0; k < m; ++k)
            if (B_(k, j) != (T)0) {
              const T temp1 = alpha * B_(k, j);
              for (int i = 0; i < k; ++i) B_(i, j) = B_(i, j) + temp1 * A_(i, k);
              B_(k, j) = nonunit ? temp1 * A_(k, k) : temp1;
            }
      } else { /* 191-259 */
        for (int j = 0; j < n; ++j)
          for (int k = m - 1; k >= 0; --k)
            if (B_(k, j) != (T)0) {
              const T temp1 = alpha * B_(k, j);
              B_(k, j) = temp1;
              if (nonunit) B_(k, j) = B_(k, j) * A_(k, k);
              for (int i = k + 1; i < m; ++i) B_(i, j) = B_(i, j) + temp1 * A_(i, k);
            }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 261-323 */
        for (int j = 0; j < n; ++j)
          for (int i = m - 1; i >= 0; --i) {
            T temp = B_(i, j);
            if (nonunit) temp = temp * A_(i, i);
            for (int k = 0; k < i; ++k) temp = temp + A_(k, i) * B_(k, j);
            B_(i, j) = alpha * temp;
          }
      } else { /* 324-386 */
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < m; ++i) {
            T temp = B_(i, j);
            if (nonunit) temp = temp * A_(i, i);
            for (int k = i + 1; k < m; ++k) temp = temp + A_(k, i) * B_(k, j);
            B_(i, j) = alpha * temp;
          }
      }
    }
  } else {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 391-479 */
        for (int j = n - 1; j >= 0; --j) {
          T temp = alpha;
          if (nonunit) temp = temp * A_(j, j);
          for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) * temp;
          for (int k = 0; k < j; ++k)
            if (A_(k, j) != (T)0) {
              temp = alpha * A_(k, j);
              for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) + temp * B_(i, k);
            }
        }
      } else { /* 480-568 */
        for (int j = 0; j < n; ++j) {
          T temp = alpha;
          if (nonunit) temp = temp * A_(j, j);
          for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) * temp;
          for (int k = j + 1; k < n; ++k)
            if (A_(k, j) != (T)0) {
              temp = alpha * A_(k, j);
              for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) + temp * B_(i, k);
            }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 571-642 */
        for (int k = 0; k < n; ++k) {
          for (int j = 0; j < k; ++j)
            if (A_(j, k) != (T)0) {
              T temp = alpha;
              temp = temp * A_(j, k);
              for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) + temp * B_(i, k);
            }
          T temp = alpha;
          if (nonunit) temp = temp * A_(k, k);
          if (temp != (T)1)
            for (int i = 0; i < m; ++i) B_(i, k) = B_(i, k) * temp;
        }
      } else { /* 643-716 */
        for (int k = n - 1; k >= 0; --k) {
          for (int j = k + 1; j < n; ++j)
            if (A_(j, k) != (T)0) {
              T temp = alpha;
              temp = temp * A_(j, k);
              for (int i = 0; i < m; ++i) B_(i, j) = B_(i, j) + temp * B_(i, k);
            }
          T temp = alpha;
          if (nonunit) temp = temp * A_(k, k);
          if (temp != (T)1)
            for (int i = 0; i < m; ++i) B_(i, k) = B_(i, k) * temp;
        }
      }
    }
  }
  return 0;
}

/* blas/trmm.zig:14-63: row-major -> side.invert(), uplo.invert(), m<->n. */
int P(trmm)(int order, int side, int uplo, int transa, int diag, int m, int n, T alpha, const T *a,
            int lda, T *b, int ldb) {
  if (order == ZO_COL) return P(k_trmm)(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return P(k_trmm)(side == ZO_LEFT ? ZO_RIGHT : ZO_LEFT, uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER,
                   transa, diag, n, m, alpha, a, lda, b, ldb);
}

/* blas/gemv.zig:62-365 (k_gemv) */
static int P(k_gemv)(int transa, int m, int n, T alpha, const T *a, int lda, const T *x, int incx,
                     T beta, T *y, int incy) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, m) || incx == 0 || incy == 0) return ZO_EINVAL;
  if (m == 0 || n == 0 || (alpha == (T)0 && beta == (T)1)) return 0;
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int lenx = notr ? n : m, leny = notr ? m : n;
  const long kx = incx < 0 ? (long)(-lenx + 1) * incx : 0;
  const long ky = incy < 0 ? (long)(-leny + 1) * incy : 0;
  if (beta != (T)1) { /* 111-157 */
    long iy = ky;
    for (int i = 0; i < leny; ++i) {
      y[iy] = beta == (T)0 ? (T)0 : y[iy] * beta;
      iy += incy;
    }
  }
  if (alpha == (T)0) return 0;
  if (notr) { /* 160-252 */
    long jx = kx;
    for (int j = 0; j < n; ++j) {
      const T temp = alpha * x[jx];
      long iy = ky;
      for (int i = 0; i < m; ++i) {
        y[iy] = y[iy] + temp * A_(i, j);
        iy += incy;
      }
      jx += incx;
    }
  } else { /* 253-358 */
    long jy = ky;
    for (int j = 0; j < n; ++j) {
      T temp = 0;
      long ix = kx;
      for (int i = 0; i < m; ++i) {
        temp = temp + A_(i, j) * x[ix];
        ix += incx;
      }
      y[jy] = y[jy] + alpha * temp;
      jy += incy;
    }
  }
  return 0;
}

/* blas/gemv.zig:14-60: row-major -> transa.invert(), m<->n. */
int P(gemv)(int order, int transa, int m, int n, T alpha, const T *a, int lda, const T *x, int incx,
            T beta, T *y, int incy) {
  if (order == ZO_COL) return P(k_gemv)(transa, m, n, alpha, a, lda, x, incx, beta, y, incy);
  return P(k_gemv)(zo_trans_invert(transa), n, m, alpha, a, lda, x, incx, beta, y, incy);
}

/* blas/ger.zig:14-128 */
static int P(k_ger)(int m, int n, T alpha, const T *x, int incx, const T *y, int incy, T *a,
                    int lda) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, m) || incx == 0 || incy == 0) return ZO_EINVAL;
  if (m == 0 || n == 0 || alpha == (T)0) return 0;
  long jy = incy < 0 ? (long)(-n + 1) * incy : 0;
  const long kx = incx < 0 ? (long)(-m + 1) * incx : 0;
  for (int j = 0; j < n; ++j) {
    if (y[jy] != (T)0) {
      const T temp = alpha * y[jy];
      long ix = kx;
      for (int i = 0; i < m; ++i) {
        A_(i, j) = A_(i, j) + x[ix] * temp;
        ix += incx;
      }
    }
    jy += incy;
  }
  return 0;
}
int P(ger)(int order, int m, int n, T alpha, const T *x, int incx, const T *y, int incy, T *a,
           int lda) {
  if (order == ZO_COL) return P(k_ger)(m, n, alpha, x, incx, y, incy, a, lda);
  return P(k_ger)(n, m, alpha, y, incy, x, incx, a, lda);
}

/* blas/nrm2.zig:14-134, real branch: Blue's scaled sum of squares with the
 * thresholds as written there (bit size in place of mantissa digits, and
 * amed squared again when folded into abig). */
T P(nrm2)(int n, const T *x, int incx) {
  if (n < 0) return (T)-1;
  if (n == 0) return 0;
  const T huge = ZO_TMAX;
  const T tsml = (T)ldexp(1.0, (int)ceil((ZO_EMIN - 1) * 0.5));
  const T tbig = (T)ldexp(1.0, (int)floor((ZO_EMAX - ZO_BITS + 1) * 0.5));
  const T ssml = (T)ldexp(1.0, -(int)floor((ZO_EMIN - ZO_BITS) * 0.5));
  const T sbig = (T)ldexp(1.0, -(int)ceil((ZO_EMAX + ZO_BITS - 1) * 0.5));
  T scl = 1, sumsq = 0, abig = 0, amed = 0, asml = 0;
  int notbig = 1;
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  for (int i = 0; i < n; ++i) {
    const T ax = ZO_ABS(x[ix]);
    if (ax > tbig) {
      abig += (ax * sbig) * (ax * sbig);
      notbig = 0;
    } else if (ax < tsml) {
      if (notbig) asml += (ax * ssml) * (ax * ssml);
    } else {
      amed += ax * ax;
    }
    ix += incx;
  }
  if (abig > 0) {
    if (amed > 0 || amed > huge || amed != amed) abig += (amed * sbig) * (amed * sbig);
    scl = (T)1 / sbig;
    sumsq = abig;
  } else if (asml > 0) {
    if (amed > 0 || amed > huge || amed != amed) {
      const T sqrt_amed = ZO_SQRT(amed);
      const T sqrt_asml = ZO_SQRT(asml) / ssml;
      const T ymin = sqrt_asml > sqrt_amed ? sqrt_amed : sqrt_asml;
      const T ymax = sqrt_asml > sqrt_amed ? sqrt_asml : sqrt_amed;
      scl = 1;
      sumsq = (ymax * ymax) * ((T)1 + (ymin / ymax) * (ymin / ymax));
    } else {
      scl = (T)1 / ssml;
      sumsq = asml;
    }
  } else {
    scl = 1;
    sumsq = amed;
  }
  return scl * ZO_SQRT(sumsq);
}

/* lapack/lapy3.zig: sqrt(x^2+y^2+z^2) scaled by the largest magnitude. */
T P(lapy3)(T x, T y, T z) {
  const T hugeval = ZO_TMAX;
  const T xabs = ZO_ABS(x), yabs = ZO_ABS(y), zabs = ZO_ABS(z);
  const T yz = yabs > zabs ? yabs : zabs; /* ops.max */
  const T w = xabs > yz ? xabs : yz;
  if (w == 0 || w > hugeval) return (xabs + yabs) + zabs;
  return w * ZO_SQRT(((xabs / w) * (xabs / w) + (yabs / w) * (yabs / w)) +
                     (zabs / w) * (zabs / w));
}

/* lapack/larfg.zig:17-170 (real): H*(alpha;x) = (beta;0), tau, v(0)=1. */
int P(larfg)(int n, T *alpha, T *x, int incx, T *tau) {
  if (n <= 0) {
    *tau = 0;
    return 0;
  }
  T xnorm = P(nrm2)(n - 1, x, incx);
  if (xnorm == (T)0) {
    *tau = 0;
    return 0;
  }
  T beta = -ZO_COPYSIGN(P(lapy3)(*alpha, (T)0, xnorm), *alpha);
  const T safmin = P(lamch)('s') / P(lamch)('e');
  const T rsafmn = (T)1 / safmin;
  int knt = 0;
  if (ZO_ABS(beta) < safmin) {
    while (ZO_ABS(beta) < safmin && knt < 20) {
      P(scal)(n - 1, rsafmn, x, incx);
      beta = beta * rsafmn;
      *alpha = *alpha * rsafmn;
      ++knt;
    }
    xnorm = P(nrm2)(n - 1, x, incx);
    beta = -ZO_COPYSIGN(P(lapy3)(*alpha, (T)0, xnorm), *alpha);
  }
  *tau = (beta - *alpha) / beta;
  *alpha = (T)1 / (*alpha - beta);
  P(scal)(n - 1, *alpha, x, incx);
  for (int j = 0; j < knt; ++j) beta = beta * safmin;
  *alpha = beta;
  return 0;
}

/* lapack/ilalc.zig: last non-zero column (1-based count). */
static int P(ilalc)(int order, int m, int n, const T *a, int lda) {
  if (m == 0 || n == 0) return 0;
  if (a[P(idx)(order, 0, n - 1, lda)] != (T)0 || a[P(idx)(order, m - 1, n - 1, lda)] != (T)0)
    return n;
  for (int j = n - 1; j >= 0; --j)
    for (int i = 0; i < m; ++i)
      if (a[P(idx)(order, i, j, lda)] != (T)0) return j + 1;
  return 0;
}

/* lapack/ilalr.zig: last non-zero row (1-based count). */
static int P(ilalr)(int order, int m, int n, const T *a, int lda) {
  if (m == 0 || n == 0) return 0;
  if (a[P(idx)(order, m - 1, 0, lda)] != (T)0 || a[P(idx)(order, m - 1, n - 1, lda)] != (T)0)
    return m;
  int result = 0;
  for (int j = 0; j < n; ++j) {
    int i = m - 1;
    while (a[P(idx)(order, ZO_MAX(0, i), j, lda)] == (T)0 && i >= 0) --i;
    result = ZO_MAX(result, i + 1);
  }
  return result;
}

/* lapack/larf1f.zig:17-259: apply H = I - tau*v*v^T with v(0) = 1 implied. */
int P(larf1f)(int order, int side, int m, int n, const T *v, int incv, T tau, T *c, int ldc,
              T *work) {
  int lastv = 1, lastc = 0;
  if (tau != (T)0) {
    lastv = side == ZO_LEFT ? m : n;
    long i = incv > 0 ? (long)(lastv - 1) * incv : 0;
    while (lastv > 1 && v[i] == (T)0) {
      lastv -= 1;
      i -= incv;
    }
    lastc = side == ZO_LEFT ? P(ilalc)(order, lastv, n, c, ldc) : P(ilalr)(order, m, lastv, c, ldc);
  }
  if (lastc == 0) return 0;
  const int rld = order == ZO_COL ? ldc : 1; /* utils.row_ld */
  const int cld = P(col_ld)(order, ldc);
  if (side == ZO_LEFT) {
    if (lastv == 1) {
      P(scal)(lastc, (T)1 - tau, c, rld);
    } else {
      P(gemv)(order, ZO_TRANS, lastv - 1, lastc, (T)1, c + P(idx)(order, 1, 0, ldc), ldc, v + incv,
              incv, (T)0, work, 1);
      P(axpy)(lastc, (T)1, c, rld, work, 1);
      P(axpy)(lastc, -tau, work, 1, c, rld);
      P(ger)(order, lastv - 1, lastc, -tau, v + incv, incv, work, 1, c + P(idx)(order, 1, 0, ldc),
             ldc);
    }
  } else {
    if (lastv == 1) {
      P(scal)(lastc, (T)1 - tau, c, cld);
    } else {
      P(gemv)(order, ZO_NOTRANS, lastc, lastv - 1, (T)1, c + P(idx)(order, 0, 1, ldc), ldc,
              v + incv, incv, (T)0, work, 1);
      P(axpy)(lastc, (T)1, c, cld, work, 1);
      P(axpy)(lastc, -tau, work, 1, c, cld);
      P(ger)(order, lastc, lastv - 1, -tau, work, 1, v + incv, incv, c + P(idx)(order, 0, 1, ldc),
             ldc);
    }
  }
  return 0;
}

/* lapack/geqr2.zig:17-59 */
int P(geqr2)(int order, int m, int n, T *a, int lda, T *tau, T *work) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  const int cld = P(col_ld)(order, lda);
  for (int i = 0; i < ZO_MIN(m, n); ++i) {
    P(larfg)(m - i, &a[P(idx)(order, i, i, lda)],
             a + P(idx)(order, ZO_MIN(i + 1, m - 1), i, lda), cld, &tau[i]);
    if (i < n - 1)
      P(larf1f)(order, ZO_LEFT, m - i, n - i - 1, a + P(idx)(order, i, i, lda), cld, tau[i],
                a + P(idx)(order, i, i + 1, lda), lda, work);
  }
  return 0;
}

/* lapack/larft.zig:18-231, the QR branch (forward, columnwise): recursive
 * T factor after Elmroth and Gustavson. */
int P(larft)(int order, int direct, int storev, int n, int k, const T *v, int ldv, const T *tau,
             T *t, int ldt) {
  if (n == 0 || k == 0) return 0;
  if (n == 1 || k == 1) {
    t[P(idx)(order, 0, 0, ldt)] = tau[0];
    return 0;
  }
  if (!(direct == 'F' && storev == 'C')) return ZO_EINVAL; /* not on this path */
  const int l = k / 2;
  P(larft)(order, direct, storev, n, l, v, ldv, tau, t, ldt);
  P(larft)(order, direct, storev, n - l, k - l, v + P(idx)(order, l, l, ldv), ldv, tau + l,
           t + P(idx)(order, l, l, ldt), ldt);
  for (int j = 0; j < l; ++j)
    for (int i = 0; i < k - l; ++i) t[P(idx)(order, j, l + i, ldt)] = v[P(idx)(order, l + i, j, ldv)];
  P(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, l, k - l, (T)1,
          v + P(idx)(order, l, l, ldv), ldv, t + P(idx)(order, 0, l, ldt), ldt);
  P(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, l, k - l, n - k, (T)1, v + P(idx)(order, k, 0, ldv), ldv,
          v + P(idx)(order, k, l, ldv), ldv, (T)1, t + P(idx)(order, 0, l, ldt), ldt);
  P(trmm)(order, ZO_LEFT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, l, k - l, (T)-1, t, ldt,
          t + P(idx)(order, 0, l, ldt), ldt);
  P(trmm)(order, ZO_RIGHT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, l, k - l, (T)1,
          t + P(idx)(order, l, l, ldt), ldt, t + P(idx)(order, 0, l, ldt), ldt);
  return 0;
}

/* linalg.zig:122-129 (Transpose.reverse) */
static int P(trans_reverse)(int t) {
  switch (t) {
    case ZO_NOTRANS: return ZO_CONJTRANS;
    case ZO_TRANS: return ZO_CONJNOTRANS;
    case ZO_CONJNOTRANS: return ZO_TRANS;
    default: return ZO_NOTRANS;
  }
}

/* lapack/larfb.zig:20-178, side left / forward / columnwise:
 * C <- H^T C (trans) or H C via W = C^T V. */
int P(larfb)(int order, int side, int trans, int direct, int storev, int m, int n, int k,
             const T *v, int ldv, const T *t, int ldt, T *c, int ldc, T *work, int ldwork) {
  if (m <= 0 || n <= 0) return 0;
  if (!(storev == 'C' && direct == 'F' && side == ZO_LEFT)) return ZO_EINVAL; /* not on path */
  const int rldc = order == ZO_COL ? ldc : 1;
  const int cldw = P(col_ld)(order, ldwork);
  for (int j = 0; j < k; ++j) /* W := C1^T (lacgv is the identity for real T) */
    P(copy)(n, c + P(idx)(order, j, 0, ldc), rldc, work + P(idx)(order, 0, j, ldwork), cldw);
  P(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, n, k, (T)1, v, ldv, work, ldwork);
  if (m > k)
    P(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, n, k, m - k, (T)1, c + P(idx)(order, k, 0, ldc), ldc,
            v + P(idx)(order, k, 0, ldv), ldv, (T)1, work, ldwork);
  P(trmm)(order, ZO_RIGHT, ZO_UPPER, P(trans_reverse)(trans), ZO_NONUNIT, n, k, (T)1, t, ldt, work,
          ldwork);
  if (m > k)
    P(gemm)(order, ZO_NOTRANS, ZO_CONJTRANS, m - k, n, k, (T)-1, v + P(idx)(order, k, 0, ldv), ldv,
            work, ldwork, (T)1, c + P(idx)(order, k, 0, ldc), ldc);
  P(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_UNIT, n, k, (T)1, v, ldv, work, ldwork);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < n; ++i)
      c[P(idx)(order, j, i, ldc)] = c[P(idx)(order, j, i, ldc)] - work[P(idx)(order, i, j, ldwork)];
  return 0;
}

/* lapack/geqrf.zig:18-157: blocked Householder QR, nb = 32, nx = 128.
 * lwork == -1 is a workspace query that stores n*nb in work[0]. */
int P(geqrf)(int order, int m, int n, T *a, int lda, T *tau, T *work, int lwork) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n) ||
      (lwork != -1 && (lwork < 1 || (m > 0 && lwork < ZO_MAX(1, n)))))
    return ZO_EINVAL;
  const int k = ZO_MIN(m, n);
  int nb = zo_ilaenv(1, "DGEQRF", m, n, -1, -1);
  if (lwork == -1) {
    work[0] = (T)(k == 0 ? 1 : n * nb);
    return 0;
  }
  if (k == 0) {
    work[0] = 1;
    return 0;
  }
  int nbmin = 2, nx = 0, iws = n, ldwork = 0;
  if (nb > 1 && nb < k) {
    nx = ZO_MAX(0, zo_ilaenv(3, "DGEQRF", m, n, -1, -1));
    if (nx < k) {
      ldwork = order == ZO_COL ? n : nb;
      iws = ldwork * nb;
      if (lwork < iws) {
        nb = lwork / ldwork;
        nbmin = ZO_MAX(2, zo_ilaenv(2, "DGEQRF", m, n, -1, -1));
      }
    }
  }
  int i = 0;
  if (nb >= nbmin && nb < k && nx < k) {
    for (; i < k - nx; i += nb) {
      const int ib = ZO_MIN(k - i, nb);
      P(geqr2)(order, m - i, ib, a + P(idx)(order, i, i, lda), lda, tau + i, work);
      if (i + ib < n) {
        P(larft)(order, 'F', 'C', m - i, ib, a + P(idx)(order, i, i, lda), lda, tau + i, work,
                 ldwork);
        P(larfb)(order, ZO_LEFT, ZO_CONJTRANS, 'F', 'C', m - i, n - i - ib, ib,
                 a + P(idx)(order, i, i, lda), lda, work, ldwork,
                 a + P(idx)(order, i, i + ib, lda), lda, work + P(idx)(order, ib, 0, ldwork),
                 ldwork);
      }
    }
  }
  if (i < k) P(geqr2)(order, m - i, n - i, a + P(idx)(order, i, i, lda), lda, tau + i, work);
  work[0] = (T)iws;
  return 0;
}

/* lapack/org2r.zig:18-102: the first n columns of Q = H(0) H(1) ... H(k-1)
 * from the reflectors stored below the diagonal of a (geqrf's output),
 * unblocked, the reflectors applied last to first. */
int P(org2r)(int order, int m, int n, int k, T *a, int lda, const T *tau, T *work) {
  if (m < 0 || n < 0 || n > m || k < 0 || k > n || lda < ZO_MAX(1, order == ZO_COL ? m : n))
    return ZO_EINVAL;
  if (n == 0) return 0;
  for (int j = k; j < n; ++j) { /* columns k..n-1 start as unit vectors */
    for (int l = 0; l < m; ++l) a[P(idx)(order, l, j, lda)] = (T)0;
    a[P(idx)(order, j, j, lda)] = (T)1;
  }
  for (int i = k - 1; i >= 0; --i) {
    if (i < n - 1)
      P(larf1f)(order, ZO_LEFT, m - i, n - i - 1, a + P(idx)(order, i, i, lda),
                P(col_ld)(order, lda), tau[i], a + P(idx)(order, i, i + 1, lda), lda, work);
    if (i < m - 1)
      P(scal)(m - i - 1, -tau[i], a + P(idx)(order, i + 1, i, lda), P(col_ld)(order, lda));
    a[P(idx)(order, i, i, lda)] = (T)1 - tau[i];
    for (int l = 0; l < i; ++l) a[P(idx)(order, l, i, lda)] = (T)0;
  }
  return 0;
}

/* lapack/orgqr.zig:18-194: blocked form, nb = 32, nx = 128; the last
 * (k - kk) reflectors by org2r, then each nb-block by larft + larfb on the
 * columns to its right and org2r on its own columns.  lwork == -1 stores
 * n*nb in work[0]. */
int P(orgqr)(int order, int m, int n, int k, T *a, int lda, const T *tau, T *work, int lwork) {
  if (m < 0 || n < 0 || n > m || k < 0 || k > n || lda < ZO_MAX(1, order == ZO_COL ? m : n) ||
      (lwork < ZO_MAX(1, n) && lwork != -1))
    return ZO_EINVAL;
  int nb = zo_ilaenv(1, "DORGQR", m, n, k, -1);
  if (lwork == -1) {
    work[0] = (T)(ZO_MAX(1, n) * nb);
    return 0;
  }
  if (n == 0) {
    work[0] = 1;
    return 0;
  }
  int nbmin = 2, nx = 0, iws = n, ldwork = 0;
  if (nb > 1 && nb < k) {
    nx = ZO_MAX(0, zo_ilaenv(3, "DORGQR", m, n, k, -1));
    if (nx < k) {
      ldwork = order == ZO_COL ? n : nb;
      iws = ldwork * nb;
      if (lwork < iws) {
        nb = lwork / ldwork;
        nbmin = ZO_MAX(2, zo_ilaenv(2, "DORGQR", m, n, k, -1));
      }
    }
  }
  int ki = 0, kk = 0;
  if (nb >= nbmin && nb < k && nx < k) {
    ki = ((k - nx - 1) / nb) * nb;
    kk = ZO_MIN(k, ki + nb);
    for (int j = kk; j < n; ++j)
      for (int i = 0; i < kk; ++i) a[P(idx)(order, i, j, lda)] = (T)0;
  }
  if (kk < n)
    P(org2r)(order, m - kk, n - kk, k - kk, a + P(idx)(order, kk, kk, lda), lda, tau + kk, work);
  if (kk > 0) {
    for (int i = ki; i >= 0; i -= nb) {
      const int ib = ZO_MIN(k - i, nb);
      if (i + ib < n) {
        P(larft)(order, 'F', 'C', m - i, ib, a + P(idx)(order, i, i, lda), lda, tau + i, work,
                 ldwork);
        P(larfb)(order, ZO_LEFT, ZO_NOTRANS, 'F', 'C', m - i, n - i - ib, ib,
                 a + P(idx)(order, i, i, lda), lda, work, ldwork,
                 a + P(idx)(order, i, i + ib, lda), lda, work + P(idx)(order, ib, 0, ldwork),
                 ldwork);
      }
      P(org2r)(order, m - i, ib, ib, a + P(idx)(order, i, i, lda), lda, tau + i, work);
      for (int j = i; j < i + ib; ++j)
        for (int l = 0; l < i; ++l) a[P(idx)(order, l, j, lda)] = (T)0;
    }
  }
  work[0] = (T)iws;
  return 0;
}

#undef A_
#undef B_
