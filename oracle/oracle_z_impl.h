/*
 * oracle_z_impl.h -- the complex (cfloat) body of the zml oracle (TEST
 * INFRASTRUCTURE).
 *
 * Included once per component type by zml_oracle.c with
 *   R     = the component type (double / float), ZT = struct {R re, im}
 *   ZP(x) = the exported name prefix (zo_z_x / zo_c_x)
 *   ZFMA  = the fused multiply-add of R (fma / fmaf)
 * The arithmetic restates zml's cfloat operations (cfloat.zig) with their
 * explicit fused multiply-adds; every BLAS / LAPACK routine restates the
 * cited generic Zig routine of srmadrid/zml in its loop order and with each
 * product's operands in the order written there (zml's complex product
 * rounds its imaginary part asymmetrically).  Complex arrays are
 * interleaved (re, im) pairs, the layout of numpy's complex128 / complex64.
 */

/* ---- cfloat arithmetic ---------------------------------------------------- */
static inline ZT ZP(c)(R re, R im) {
  ZT z;
  z.re = re;
  z.im = im;
  return z;
}
/* cfloat.zig:75-88 / 112-125 */
static inline ZT ZP(cadd)(ZT x, ZT y) { return ZP(c)(x.re + y.re, x.im + y.im); }
static inline ZT ZP(csub)(ZT x, ZT y) { return ZP(c)(x.re - y.re, x.im - y.im); }
/* cfloat.zig:149-174: re = fma(x.re, y.re, -x.im * y.im),
 * im = fma(x.re, y.im, x.im * y.re). */
static inline ZT ZP(cmul)(ZT x, ZT y) {
  return ZP(c)(ZFMA(x.re, y.re, (-x.im) * y.im), ZFMA(x.re, y.im, x.im * y.re));
}
/* cfloat.zig:206-290: Smith's division with fused updates, the ratio taken
 * against the larger component of y (strictly larger real part). */
static inline ZT ZP(cdiv)(ZT x, ZT y) {
  if (ZO_ABS(y.im) < ZO_ABS(y.re)) {
    const R t1 = y.im / y.re;
    const R t2 = (R)1 / ZFMA(t1, y.im, y.re);
    return ZP(c)(ZFMA(x.im, t1, x.re) * t2, ZFMA(-x.re, t1, x.im) * t2);
  }
  const R t1 = y.re / y.im;
  const R t2 = (R)1 / ZFMA(t1, y.re, y.im);
  return ZP(c)(ZFMA(x.re, t1, x.im) * t2, ZFMA(x.im, t1, -x.re) * t2);
}
/* cfloat.zig:322-334 */
static inline ZT ZP(cconj)(ZT x) { return ZP(c)(x.re, -x.im); }
/* conj when the flag says so (the conj_* transposes) */
static inline ZT ZP(cj)(ZT x, int conj) { return conj ? ZP(cconj)(x) : x; }
/* cfloat/abs1.zig:11-17: |re| + |im| */
static inline R ZP(cabs1)(ZT x) { return ZO_ABS(x.re) + ZO_ABS(x.im); }
/* cfloat.zig eq: both components equal (a real operand has im = 0) */
static inline int ZP(ceq)(ZT x, ZT y) { return x.re == y.re && x.im == y.im; }
static inline int ZP(cis0)(ZT x) { return x.re == (R)0 && x.im == (R)0; }
static inline int ZP(cis1)(ZT x) { return x.re == (R)1 && x.im == (R)0; }
static const ZT ZP(zero) = {(R)0, (R)0};
static const ZT ZP(one) = {(R)1, (R)0};
static const ZT ZP(mone) = {(R)-1, (R)0};

/* A real x divided by a complex y: x / y, the quotient zml's own test pins
 * (test/cfloat/div.zig:42-44: div(7, 1 + 2i) = 1.4 - 2.8i), formed as
 * (x + 0i) / y with the division above.  cfloat.zig:489-492 as written
 * returns y / x for this operand order; zo_set_cdiv_as_written(1) restates
 * that instead.  getrf2.zig:66-75 reaches it as div(1, a[0]). */
static inline ZT ZP(crdiv)(R x, ZT y) {
  if (zo_cdiv_as_written) return ZP(c)(y.re / x, y.im / x); /* cfloat.zig:292-305 divReal */
  return ZP(cdiv)(ZP(c)(x, (R)0), y);
}

#define ZA_(i, j) a[(long)(i) + (long)(j) * lda]
#define ZB_(i, j) b[(long)(i) + (long)(j) * ldb]
#define ZC_(i, j) c[(long)(i) + (long)(j) * ldc]

/* ---- BLAS level 1 ------------------------------------------------------------ */

/* blas/iamax.zig:39-53 (complex branch): the first maximum of |re| + |im|
 * (strict '>'), NaN never replaces the running maximum. */
int ZP(iamax)(int n, const ZT *x, int incx) {
  if (n <= 0 || incx <= 0) return ZO_EINVAL;
  if (n == 1) return 0;
  int imax = 0;
  R max = ZP(cabs1)(x[0]);
  long ix = incx;
  for (int i = 1; i < n; ++i) {
    const R absx = ZP(cabs1)(x[ix]);
    if (absx > max) {
      max = absx;
      imax = i;
    }
    ix += incx;
  }
  return imax;
}

/* blas/scal.zig:9-41: x *= alpha, early return when alpha == 1. */
int ZP(scal)(int n, ZT alpha, ZT *x, int incx) {
  if (n < 0 || incx <= 0) return ZO_EINVAL;
  if (n == 0) return 0;
  if (ZP(cis1)(alpha)) return 0;
  long ix = 0;
  for (int i = 0; i < n; ++i) {
    x[ix] = ZP(cmul)(x[ix], alpha);
    ix += incx;
  }
  return 0;
}

/* ---- BLAS level 3: gemm ---------------------------------------------------- */

/* blas/gemm.zig:68-1027 (k_gemm): the four loop forms of the real routine
 * (NN and NT axpy forms, TN and TT dot forms), with a or b conjugated for
 * the conj_no_trans / conj_trans operands (noconja / noconjb, 93-96). */
static int ZP(k_gemm)(int transa, int transb, int m, int n, int k, ZT alpha, const ZT *a, int lda,
                      const ZT *b, int ldb, ZT beta, ZT *c, int ldc) {
  const int nota = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int notb = transb == ZO_NOTRANS || transb == ZO_CONJNOTRANS;
  const int cja = !(transa == ZO_NOTRANS || transa == ZO_TRANS);
  const int cjb = !(transb == ZO_NOTRANS || transb == ZO_TRANS);
  const int nrowa = nota ? m : k;
  const int nrowb = notb ? k : n;
  if (m < 0 || n < 0 || k < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, nrowb) ||
      ldc < ZO_MAX(1, m))
    return ZO_EINVAL;                                                         /* 101-102 */
  if (m == 0 || n == 0 || ((ZP(cis0)(alpha) || k == 0) && ZP(cis1)(beta))) return 0; /* 105-108 */
  if (ZP(cis0)(alpha)) { /* 111-140 */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) ZC_(i, j) = ZP(cis0)(beta) ? ZP(zero) : ZP(cmul)(ZC_(i, j), beta);
    return 0;
  }
  if (nota) { /* 142-336 (b not transposed), 584-778 (b transposed): axpy forms */
    /* operand order as written: alpha * b and temp * a in the plain NN branch
     * (171, 179), b * alpha and a * temp in every other one (218-226, 267-275,
     * 314-322, 613-621, 660-668, 709-717, 756-764) */
    const int plain = notb && !cja && !cjb;
    for (int j = 0; j < n; ++j) {
      if (ZP(cis0)(beta)) {
        for (int i = 0; i < m; ++i) ZC_(i, j) = ZP(zero);
      } else if (!ZP(cis1)(beta)) {
        for (int i = 0; i < m; ++i) ZC_(i, j) = ZP(cmul)(ZC_(i, j), beta);
      }
      for (int l = 0; l < k; ++l) {
        const ZT bl = ZP(cj)(notb ? ZB_(l, j) : ZB_(j, l), cjb);
        const ZT temp = plain ? ZP(cmul)(alpha, bl) : ZP(cmul)(bl, alpha);
        for (int i = 0; i < m; ++i) {
          const ZT al = ZP(cj)(ZA_(i, l), cja);
          ZC_(i, j) = ZP(cadd)(ZC_(i, j), plain ? ZP(cmul)(temp, al) : ZP(cmul)(al, temp));
        }
      }
    }
  } else { /* 337-583 (b not transposed), 779-1020 (b transposed): dot forms */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) {
        ZT temp = ZP(zero);
        for (int l = 0; l < k; ++l) {
          const ZT bl = notb ? ZB_(l, j) : ZB_(j, l);
          temp = ZP(cadd)(temp, ZP(cmul)(ZP(cj)(ZA_(l, i), cja), ZP(cj)(bl, cjb)));
        }
        if (ZP(cis0)(beta)) {
          ZC_(i, j) = ZP(cmul)(alpha, temp);
        } else if (ZP(cis1)(beta)) {
          ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(alpha, temp));
        } else {
          ZC_(i, j) = ZP(cmul)(ZC_(i, j), beta);
          ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(alpha, temp));
        }
      }
  }
  return 0;
}

/* blas/gemm.zig:14-66: row-major maps to column-major by swapping the
 * operands (A<->B, m<->n). */
int ZP(gemm)(int order, int transa, int transb, int m, int n, int k, ZT alpha, const ZT *a,
             int lda, const ZT *b, int ldb, ZT beta, ZT *c, int ldc) {
  if (order == ZO_COL)
    return ZP(k_gemm)(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  return ZP(k_gemm)(transb, transa, n, m, k, alpha, b, ldb, a, lda, beta, c, ldc);
}

/* ---- BLAS level 3: trsm ---------------------------------------------------- */

/* blas/trsm.zig:66-735 (k_trsm), the real routine's loops with a
 * conjugated for conj_no_trans / conj_trans.  The left/no-trans divisions
 * read b[k + j*lda] as written (137, 177, 222, 245) unless as-written mode
 * is off.  Operand order as written, including alpha * b at 208 and 343
 * (b * alpha elsewhere). */
static int ZP(k_trsm)(int side, int uplo, int transa, int diag, int m, int n, ZT alpha,
                      const ZT *a, int lda, ZT *b, int ldb) {
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int cj = !(transa == ZO_NOTRANS || transa == ZO_TRANS);
  const int nrowa = side == ZO_LEFT ? m : n;
  const int nonunit = diag == ZO_NONUNIT;
  const long ldq = zo_trsm_as_written ? lda : ldb;
  if (m < 0 || n < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, m)) return ZO_EINVAL; /* 91 */
  if (m == 0 || n == 0) return 0;
  if (ZP(cis0)(alpha)) { /* 99-113 */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(zero);
    return 0;
  }
  if (side == ZO_LEFT) {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 117-201: back substitution */
        for (int j = 0; j < n; ++j) {
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), alpha);
          for (int k = m - 1; k >= 0; --k) {
            if (!ZP(cis0)(ZB_(k, j))) {
              if (nonunit)
                ZB_(k, j) = ZP(cdiv)(b[(long)k + (long)j * ldq], ZP(cj)(ZA_(k, k), cj));
              for (int i = 0; i < k; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(ZB_(k, j), ZP(cj)(ZA_(i, k), cj)));
            }
          }
        }
      } else { /* 202-270: forward substitution */
        for (int j = 0; j < n; ++j) {
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(alpha, ZB_(i, j));
          for (int k = 0; k < m; ++k) {
            if (!ZP(cis0)(ZB_(k, j))) {
              if (nonunit)
                ZB_(k, j) = ZP(cdiv)(b[(long)k + (long)j * ldq], ZP(cj)(ZA_(k, k), cj));
              for (int i = k + 1; i < m; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(ZB_(k, j), ZP(cj)(ZA_(i, k), cj)));
            }
          }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 272-337: dot form, op(A) lower */
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < m; ++i) {
            ZT temp = ZP(cmul)(ZB_(i, j), alpha);
            for (int k = 0; k < i; ++k)
              temp = ZP(csub)(temp, ZP(cmul)(ZP(cj)(ZA_(k, i), cj), ZB_(k, j)));
            if (nonunit) temp = ZP(cdiv)(temp, ZP(cj)(ZA_(i, i), cj));
            ZB_(i, j) = temp;
          }
      } else { /* 338-404 */
        for (int j = 0; j < n; ++j)
          for (int i = m - 1; i >= 0; --i) {
            ZT temp = ZP(cmul)(alpha, ZB_(i, j));
            for (int k = i + 1; k < m; ++k)
              temp = ZP(csub)(temp, ZP(cmul)(ZP(cj)(ZA_(k, i), cj), ZB_(k, j)));
            if (nonunit) temp = ZP(cdiv)(temp, ZP(cj)(ZA_(i, i), cj));
            ZB_(i, j) = temp;
          }
      }
    }
  } else {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 408-487 */
        for (int j = 0; j < n; ++j) {
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), alpha);
          for (int k = 0; k < j; ++k)
            if (!ZP(cis0)(ZA_(k, j)))
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(ZP(cj)(ZA_(k, j), cj), ZB_(i, k)));
          if (nonunit) {
            const ZT temp = ZP(cdiv)(ZP(one), ZP(cj)(ZA_(j, j), cj));
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), temp);
          }
        }
      } else { /* 488-568 */
        for (int j = n - 1; j >= 0; --j) {
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), alpha);
          for (int k = j + 1; k < n; ++k)
            if (!ZP(cis0)(ZA_(k, j)))
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(ZP(cj)(ZA_(k, j), cj), ZB_(i, k)));
          if (nonunit) {
            const ZT temp = ZP(cdiv)(ZP(one), ZP(cj)(ZA_(j, j), cj));
            for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), temp);
          }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 570-647 */
        for (int k = n - 1; k >= 0; --k) {
          if (nonunit) {
            const ZT temp = ZP(cdiv)(ZP(one), ZP(cj)(ZA_(k, k), cj));
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), temp);
          }
          for (int j = 0; j < k; ++j)
            if (!ZP(cis0)(ZA_(j, k))) {
              const ZT temp = ZP(cj)(ZA_(j, k), cj);
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), alpha);
        }
      } else { /* 648-727 */
        for (int k = 0; k < n; ++k) {
          if (nonunit) {
            const ZT temp = ZP(cdiv)(ZP(one), ZP(cj)(ZA_(k, k), cj));
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), temp);
          }
          for (int j = k + 1; j < n; ++j)
            if (!ZP(cis0)(ZA_(j, k))) {
              const ZT temp = ZP(cj)(ZA_(j, k), cj);
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(csub)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
          if (!ZP(cis1)(alpha))
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), alpha);
        }
      }
    }
  }
  return 0;
}

/* blas/trsm.zig:18-64: row-major -> side.invert(), uplo.invert(), m<->n. */
int ZP(trsm)(int order, int side, int uplo, int transa, int diag, int m, int n, ZT alpha,
             const ZT *a, int lda, ZT *b, int ldb) {
  if (order == ZO_COL) return ZP(k_trsm)(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return ZP(k_trsm)(side == ZO_LEFT ? ZO_RIGHT : ZO_LEFT, uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER,
                    transa, diag, n, m, alpha, a, lda, b, ldb);
}

/* ---- BLAS level 3: syrk (complex symmetric) and herk ------------------------ */

/* blas/syrk.zig:60-366 (k_syrk): C = alpha A A^T + beta C without any
 * conjugation; rejects the conjugate transposes (82-84). */
static int ZP(k_syrk)(int uplo, int trans, int n, int k, ZT alpha, const ZT *a, int lda, ZT beta,
                      ZT *c, int ldc) {
  const int nrowa = trans == ZO_NOTRANS ? n : k;
  if (trans == ZO_CONJNOTRANS || trans == ZO_CONJTRANS || n < 0 || k < 0 ||
      lda < ZO_MAX(1, nrowa) || ldc < ZO_MAX(1, n))
    return ZO_EINVAL;
  if (n == 0 || ((ZP(cis0)(alpha) || k == 0) && ZP(cis1)(beta))) return 0; /* 87-90 */
  if (ZP(cis0)(alpha)) {                                                 /* 93-151 */
    for (int j = 0; j < n; ++j) {
      const int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      for (int i = i0; i < i1; ++i)
        ZC_(i, j) = ZP(cis0)(beta) ? ZP(zero) : ZP(cmul)(ZC_(i, j), beta);
    }
    return 0;
  }
  if (trans == ZO_NOTRANS) { /* 153-252 */
    for (int j = 0; j < n; ++j) {
      const int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      if (ZP(cis0)(beta)) {
        for (int i = i0; i < i1; ++i) ZC_(i, j) = ZP(zero);
      } else if (!ZP(cis1)(beta)) {
        for (int i = i0; i < i1; ++i) ZC_(i, j) = ZP(cmul)(ZC_(i, j), beta);
      }
      for (int l = 0; l < k; ++l) {
        if (!ZP(cis0)(ZA_(j, l))) {
          const ZT temp = ZP(cmul)(alpha, ZA_(j, l));
          for (int i = i0; i < i1; ++i)
            ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(temp, ZA_(i, l)));
        }
      }
    }
  } else { /* 253-359 */
    for (int j = 0; j < n; ++j) {
      const int i0 = uplo == ZO_UPPER ? 0 : j, i1 = uplo == ZO_UPPER ? j + 1 : n;
      for (int i = i0; i < i1; ++i) {
        ZT temp = ZP(zero);
        for (int l = 0; l < k; ++l) temp = ZP(cadd)(temp, ZP(cmul)(ZA_(l, i), ZA_(l, j)));
        if (ZP(cis0)(beta)) {
          ZC_(i, j) = ZP(cmul)(alpha, temp);
        } else {
          ZC_(i, j) = ZP(cmul)(ZC_(i, j), beta);
          ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(alpha, temp));
        }
      }
    }
  }
  return 0;
}

/* blas/syrk.zig:15-58: row-major -> uplo.invert(), trans.invert(). */
int ZP(syrk)(int order, int uplo, int trans, int n, int k, ZT alpha, const ZT *a, int lda,
             ZT beta, ZT *c, int ldc) {
  if (order == ZO_COL) return ZP(k_syrk)(uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
  return ZP(k_syrk)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, zo_trans_invert(trans), n, k, alpha,
                    a, lda, beta, c, ldc);
}

/* A complex value scaled by a real one, component by component
 * (cfloat.zig:176-189 mulReal, reached by mul with one real operand). */
static inline ZT ZP(cscale)(ZT x, R s) { return ZP(c)(x.re * s, x.im * s); }

/* blas/herk.zig:60-504 (k_herk): C = alpha A A^H + beta C (no_trans) or
 * alpha A^H A + beta C (conj_trans) with real alpha and beta; the diagonal
 * keeps only its real part.  Rejects trans and conj_no_trans (83-85). */
static int ZP(k_herk)(int uplo, int trans, int n, int k, R alpha, const ZT *a, int lda, R beta,
                      ZT *c, int ldc) {
  const int nrowa = trans == ZO_NOTRANS ? n : k;
  if (trans == ZO_CONJNOTRANS || trans == ZO_TRANS || n < 0 || k < 0 ||
      lda < ZO_MAX(1, nrowa) || ldc < ZO_MAX(1, n))
    return ZO_EINVAL;
  if (n == 0 || ((alpha == (R)0 || k == 0) && beta == (R)1)) return 0; /* 88-91 */
  const int up = uplo == ZO_UPPER;
  if (alpha == (R)0) { /* 94-166 */
    for (int j = 0; j < n; ++j) {
      const int i0 = up ? 0 : j + 1, i1 = up ? j : n;
      if (beta == (R)0) {
        for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i) ZC_(i, j) = ZP(zero);
      } else {
        if (!up) ZC_(j, j) = ZP(c)(beta * ZC_(j, j).re, (R)0);
        for (int i = i0; i < i1; ++i) ZC_(i, j) = ZP(cscale)(ZC_(i, j), beta);
        if (up) ZC_(j, j) = ZP(c)(beta * ZC_(j, j).re, (R)0);
      }
    }
    return 0;
  }
  if (trans == ZO_NOTRANS) { /* 168-315 */
    for (int j = 0; j < n; ++j) {
      const int i0 = up ? 0 : j + 1, i1 = up ? j : n; /* the off-diagonal rows of column j */
      if (beta == (R)0) {
        for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i) ZC_(i, j) = ZP(zero);
      } else if (beta != (R)1) {
        if (!up) ZC_(j, j) = ZP(c)(beta * ZC_(j, j).re, (R)0);
        for (int i = i0; i < i1; ++i) ZC_(i, j) = ZP(cscale)(ZC_(i, j), beta);
        if (up) ZC_(j, j) = ZP(c)(beta * ZC_(j, j).re, (R)0);
      } else {
        ZC_(j, j) = ZP(c)(ZC_(j, j).re, (R)0);
      }
      for (int l = 0; l < k; ++l) {
        if (!ZP(cis0)(ZA_(j, l))) {
          const ZT temp = ZP(cscale)(ZP(cconj)(ZA_(j, l)), alpha);
          if (up) {
            for (int i = i0; i < i1; ++i)
              ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(temp, ZA_(i, l)));
            ZC_(j, j) = ZP(c)(ZC_(j, j).re + ZP(cmul)(temp, ZA_(j, l)).re, (R)0);
          } else {
            ZC_(j, j) = ZP(c)(ZC_(j, j).re + ZP(cmul)(temp, ZA_(j, l)).re, (R)0);
            for (int i = i0; i < i1; ++i)
              ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cmul)(temp, ZA_(i, l)));
          }
        }
      }
    }
  } else { /* 316-500 */
    for (int j = 0; j < n; ++j) {
      const int i0 = up ? 0 : j + 1, i1 = up ? j : n;
      for (int pass = 0; pass < 2; ++pass) {
        /* upper: the off-diagonal entries, then the diagonal; lower: the reverse */
        const int diag = up ? pass == 1 : pass == 0;
        if (diag) {
          R rtemp = 0;
          for (int l = 0; l < k; ++l)
            rtemp = rtemp + ZP(cmul)(ZP(cconj)(ZA_(l, j)), ZA_(l, j)).re;
          if (beta == (R)0) {
            ZC_(j, j) = ZP(c)(alpha * rtemp, (R)0);
          } else {
            ZC_(j, j) = ZP(c)(beta * ZC_(j, j).re, (R)0);
            ZC_(j, j) = ZP(c)(ZC_(j, j).re + alpha * rtemp, ZC_(j, j).im);
          }
        } else {
          for (int i = i0; i < i1; ++i) {
            ZT temp = ZP(zero);
            for (int l = 0; l < k; ++l)
              temp = ZP(cadd)(temp, ZP(cmul)(ZP(cconj)(ZA_(l, i)), ZA_(l, j)));
            if (beta == (R)0) {
              ZC_(i, j) = ZP(cscale)(temp, alpha);
            } else {
              ZC_(i, j) = ZP(cscale)(ZC_(i, j), beta);
              ZC_(i, j) = ZP(cadd)(ZC_(i, j), ZP(cscale)(temp, alpha));
            }
          }
        }
      }
    }
  }
  return 0;
}

/* blas/herk.zig:14-58: row-major -> uplo.invert(), trans.reverse()
 * (no_trans <-> conj_trans, linalg.zig:121-128). */
int ZP(herk)(int order, int uplo, int trans, int n, int k, R alpha, const ZT *a, int lda, R beta,
             ZT *c, int ldc) {
  if (order == ZO_COL) return ZP(k_herk)(uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
  const int rt = trans == ZO_NOTRANS ? ZO_CONJTRANS
               : trans == ZO_TRANS ? ZO_CONJNOTRANS
               : trans == ZO_CONJNOTRANS ? ZO_TRANS : ZO_NOTRANS;
  return ZP(k_herk)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, rt, n, k, alpha, a, lda, beta, c, ldc);
}

/* ---- BLAS level 3: trmm ---------------------------------------------------- */

/* blas/trmm.zig:65-724 (k_trmm), the real routine's loops with a
 * conjugated for conj_no_trans / conj_trans; operand order as written. */
static int ZP(k_trmm)(int side, int uplo, int transa, int diag, int m, int n, ZT alpha,
                      const ZT *a, int lda, ZT *b, int ldb) {
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int cj = !(transa == ZO_NOTRANS || transa == ZO_TRANS);
  const int nonunit = diag == ZO_NONUNIT;
  const int nrowa = side == ZO_LEFT ? m : n;
  if (m < 0 || n < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, m)) return ZO_EINVAL;
  if (m == 0 || n == 0) return 0;
  if (ZP(cis0)(alpha)) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(zero);
    return 0;
  }
  if (side == ZO_LEFT) {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 118-190 */
        for (int j = 0; j < n; ++j)
          for (int k = 0; k < m; ++k)
            if (!ZP(cis0)(ZB_(k, j))) {
              const ZT temp1 = ZP(cmul)(alpha, ZB_(k, j));
              for (int i = 0; i < k; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp1, ZP(cj)(ZA_(i, k), cj)));
              ZB_(k, j) = nonunit ? ZP(cmul)(temp1, ZP(cj)(ZA_(k, k), cj)) : temp1;
            }
      } else { /* 191-259 */
        for (int j = 0; j < n; ++j)
          for (int k = m - 1; k >= 0; --k)
            if (!ZP(cis0)(ZB_(k, j))) {
              const ZT temp1 = ZP(cmul)(alpha, ZB_(k, j));
              ZB_(k, j) = temp1;
              if (nonunit) ZB_(k, j) = ZP(cmul)(ZB_(k, j), ZP(cj)(ZA_(k, k), cj));
              for (int i = k + 1; i < m; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp1, ZP(cj)(ZA_(i, k), cj)));
            }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 261-323 */
        for (int j = 0; j < n; ++j)
          for (int i = m - 1; i >= 0; --i) {
            ZT temp = ZB_(i, j);
            if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(i, i), cj));
            for (int k = 0; k < i; ++k)
              temp = ZP(cadd)(temp, ZP(cmul)(ZP(cj)(ZA_(k, i), cj), ZB_(k, j)));
            ZB_(i, j) = ZP(cmul)(alpha, temp);
          }
      } else { /* 324-386 */
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < m; ++i) {
            ZT temp = ZB_(i, j);
            if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(i, i), cj));
            for (int k = i + 1; k < m; ++k)
              temp = ZP(cadd)(temp, ZP(cmul)(ZP(cj)(ZA_(k, i), cj), ZB_(k, j)));
            ZB_(i, j) = ZP(cmul)(alpha, temp);
          }
      }
    }
  } else {
    if (notr) {
      if (uplo == ZO_UPPER) { /* 391-479 */
        for (int j = n - 1; j >= 0; --j) {
          ZT temp = alpha;
          if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(j, j), cj));
          for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), temp);
          for (int k = 0; k < j; ++k)
            if (!ZP(cis0)(ZA_(k, j))) {
              temp = ZP(cmul)(alpha, ZP(cj)(ZA_(k, j), cj));
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
        }
      } else { /* 480-568 */
        for (int j = 0; j < n; ++j) {
          ZT temp = alpha;
          if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(j, j), cj));
          for (int i = 0; i < m; ++i) ZB_(i, j) = ZP(cmul)(ZB_(i, j), temp);
          for (int k = j + 1; k < n; ++k)
            if (!ZP(cis0)(ZA_(k, j))) {
              temp = ZP(cmul)(alpha, ZP(cj)(ZA_(k, j), cj));
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
        }
      }
    } else {
      if (uplo == ZO_UPPER) { /* 571-642 */
        for (int k = 0; k < n; ++k) {
          for (int j = 0; j < k; ++j)
            if (!ZP(cis0)(ZA_(j, k))) {
              ZT temp = alpha;
              temp = ZP(cmul)(temp, ZP(cj)(ZA_(j, k), cj));
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
          ZT temp = alpha;
          if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(k, k), cj));
          if (!ZP(cis1)(temp))
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), temp);
        }
      } else { /* 643-716 */
        for (int k = n - 1; k >= 0; --k) {
          for (int j = k + 1; j < n; ++j)
            if (!ZP(cis0)(ZA_(j, k))) {
              ZT temp = alpha;
              temp = ZP(cmul)(temp, ZP(cj)(ZA_(j, k), cj));
              for (int i = 0; i < m; ++i)
                ZB_(i, j) = ZP(cadd)(ZB_(i, j), ZP(cmul)(temp, ZB_(i, k)));
            }
          ZT temp = alpha;
          if (nonunit) temp = ZP(cmul)(temp, ZP(cj)(ZA_(k, k), cj));
          if (!ZP(cis1)(temp))
            for (int i = 0; i < m; ++i) ZB_(i, k) = ZP(cmul)(ZB_(i, k), temp);
        }
      }
    }
  }
  return 0;
}

/* blas/trmm.zig:14-63: row-major -> side.invert(), uplo.invert(), m<->n. */
int ZP(trmm)(int order, int side, int uplo, int transa, int diag, int m, int n, ZT alpha,
             const ZT *a, int lda, ZT *b, int ldb) {
  if (order == ZO_COL) return ZP(k_trmm)(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return ZP(k_trmm)(side == ZO_LEFT ? ZO_RIGHT : ZO_LEFT, uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER,
                    transa, diag, n, m, alpha, a, lda, b, ldb);
}

/* ---- BLAS level 2: gemv, geru, gerc --------------------------------------- */

/* blas/gemv.zig:62-365 (k_gemv); conj_no_trans forms y = alpha conj(A) x +
 * beta y, conj_trans y = alpha A^H x + beta y (noconj, 93). */
static int ZP(k_gemv)(int transa, int m, int n, ZT alpha, const ZT *a, int lda, const ZT *x,
                      int incx, ZT beta, ZT *y, int incy) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, m) || incx == 0 || incy == 0) return ZO_EINVAL;
  if (m == 0 || n == 0 || (ZP(cis0)(alpha) && ZP(cis1)(beta))) return 0;
  const int notr = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int cj = !(transa == ZO_NOTRANS || transa == ZO_TRANS);
  const int lenx = notr ? n : m, leny = notr ? m : n;
  const long kx = incx < 0 ? (long)(-lenx + 1) * incx : 0;
  const long ky = incy < 0 ? (long)(-leny + 1) * incy : 0;
  if (!ZP(cis1)(beta)) { /* 111-157 */
    long iy = ky;
    for (int i = 0; i < leny; ++i) {
      y[iy] = ZP(cis0)(beta) ? ZP(zero) : ZP(cmul)(y[iy], beta);
      iy += incy;
    }
  }
  if (ZP(cis0)(alpha)) return 0;
  if (notr) { /* 161-252 */
    long jx = kx;
    for (int j = 0; j < n; ++j) {
      const ZT temp = ZP(cmul)(alpha, x[jx]);
      long iy = ky;
      for (int i = 0; i < m; ++i) {
        y[iy] = ZP(cadd)(y[iy], ZP(cmul)(temp, ZP(cj)(ZA_(i, j), cj)));
        iy += incy;
      }
      jx += incx;
    }
  } else { /* 253-358 */
    long jy = ky;
    for (int j = 0; j < n; ++j) {
      ZT temp = ZP(zero);
      long ix = kx;
      for (int i = 0; i < m; ++i) {
        temp = ZP(cadd)(temp, ZP(cmul)(ZP(cj)(ZA_(i, j), cj), x[ix]));
        ix += incx;
      }
      y[jy] = ZP(cadd)(y[jy], ZP(cmul)(alpha, temp));
      jy += incy;
    }
  }
  return 0;
}

/* blas/gemv.zig:14-60: row-major -> transa.invert(), m<->n. */
int ZP(gemv)(int order, int transa, int m, int n, ZT alpha, const ZT *a, int lda, const ZT *x,
             int incx, ZT beta, ZT *y, int incy) {
  if (order == ZO_COL) return ZP(k_gemv)(transa, m, n, alpha, a, lda, x, incx, beta, y, incy);
  return ZP(k_gemv)(zo_trans_invert(transa), n, m, alpha, a, lda, x, incx, beta, y, incy);
}

/* blas/geru.zig:33-120 and gerc.zig:33-186: A += alpha x y^T (geru) or
 * alpha x y^H (gerc); column j skipped when y[j] == 0.  cy conjugates y
 * (gerc column-major), cx conjugates x (gerc row-major: the operands swap,
 * gerc.zig:26-30, and the conjugation moves onto the new x). */
static int ZP(k_ger)(int m, int n, ZT alpha, const ZT *x, int incx, const ZT *y, int incy, ZT *a,
                     int lda, int cx, int cy) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, m) || incx == 0 || incy == 0) return ZO_EINVAL;
  if (m == 0 || n == 0 || ZP(cis0)(alpha)) return 0;
  long jy = incy < 0 ? (long)(-n + 1) * incy : 0;
  const long kx = incx < 0 ? (long)(-m + 1) * incx : 0;
  for (int j = 0; j < n; ++j) {
    if (!ZP(cis0)(y[jy])) {
      const ZT temp = ZP(cmul)(alpha, ZP(cj)(y[jy], cy));
      long ix = kx;
      for (int i = 0; i < m; ++i) {
        ZA_(i, j) = ZP(cadd)(ZA_(i, j), ZP(cmul)(ZP(cj)(x[ix], cx), temp));
        ix += incx;
      }
    }
    jy += incy;
  }
  return 0;
}
int ZP(geru)(int order, int m, int n, ZT alpha, const ZT *x, int incx, const ZT *y, int incy,
             ZT *a, int lda) {
  if (order == ZO_COL) return ZP(k_ger)(m, n, alpha, x, incx, y, incy, a, lda, 0, 0);
  return ZP(k_ger)(n, m, alpha, y, incy, x, incx, a, lda, 0, 0);
}
int ZP(gerc)(int order, int m, int n, ZT alpha, const ZT *x, int incx, const ZT *y, int incy,
             ZT *a, int lda) {
  if (order == ZO_COL) return ZP(k_ger)(m, n, alpha, x, incx, y, incy, a, lda, 0, 1);
  return ZP(k_ger)(n, m, alpha, y, incy, x, incx, a, lda, 1, 0);
}

/* ---- LAPACK: LU ------------------------------------------------------------ */

/* lapack/laswp.zig:12-96 (element-type generic): interchanges in blocks of
 * 32 columns, then the remainder; negative incx walks the pivots backwards. */
int ZP(laswp)(int order, int n, ZT *a, int lda, int k1, int k2, const int *ipiv, int incx) {
  if (n < 0 || (order == ZO_ROW && lda < ZO_MAX(1, n)) || incx == 0) return ZO_EINVAL;
  if (n == 0) return 0;
  int ix0, I1, I2, inc;
  if (incx > 0) {
    ix0 = k1 - 1; I1 = k1 - 1; I2 = k2 - 1; inc = 1;
  } else {
    ix0 = k1 - 1 + (k1 - k2) * incx; I1 = k2 - 1; I2 = k1 - 1; inc = -1;
  }
  const int n32 = (n >> 5) << 5;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j1 = j0 < n32 ? j0 + 32 : n;
    int ix = ix0;
    for (int i = I1; i != I2 + inc; i += inc) {
      const int ip = ipiv[ix] - 1;
      if (ip != i)
        for (int k = j0; k < j1; ++k) {
          const ZT temp = a[zo_index(order, i, k, lda)];
          a[zo_index(order, i, k, lda)] = a[zo_index(order, ip, k, lda)];
          a[zo_index(order, ip, k, lda)] = temp;
        }
      ix += incx;
    }
    if (j1 == n) break;
  }
  return 0;
}

/* lapack/getrf2.zig:14-210: recursive LU with partial pivoting; the pivot
 * is the first maximum of |re| + |im| (iamax), the column is scaled by
 * 1 / a[0] when |a[0]|_1 >= sfmin (div(1, a[0]), see crdiv), else divided
 * entry by entry. */
int ZP(getrf2)(int order, int m, int n, ZT *a, int lda, int *ipiv) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  int info = 0;
  if (m == 0 || n == 0) return info;
  const int cl = order == ZO_COL ? 1 : lda;
  if (m == 1) { /* 35-40 */
    ipiv[0] = 1;
    if (ZP(cis0)(a[0])) info = 1;
  } else if (n == 1) { /* 41-89 */
    const R sfmin = ZP(lamch_s)();
    const int ii = ZP(iamax)(m, a, cl);
    ipiv[0] = ii + 1;
    if (!ZP(cis0)(a[zo_index(order, ii, 0, lda)])) {
      if (ii != 0) {
        const ZT temp = a[0];
        a[0] = a[zo_index(order, ii, 0, lda)];
        a[zo_index(order, ii, 0, lda)] = temp;
      }
      if (ZP(cabs1)(a[0]) >= sfmin) {
        ZP(scal)(m - 1, ZP(crdiv)((R)1, a[0]), a + zo_index(order, 1, 0, lda), cl);
      } else {
        for (int i = 0; i < m - 1; ++i)
          a[zo_index(order, i + 1, 0, lda)] = ZP(cdiv)(a[zo_index(order, i + 1, 0, lda)], a[0]);
      }
    } else {
      info = 1;
    }
  } else { /* 90-196 */
    const int n1 = ZO_MIN(m, n) / 2;
    const int n2 = n - n1;
    int iinfo = ZP(getrf2)(order, m, n1, a, lda, ipiv);
    if (info == 0 && iinfo > 0) info = iinfo;
    ZP(laswp)(order, n2, a + zo_index(order, 0, n1, lda), lda, 1, n1, ipiv, 1);
    ZP(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, n1, n2, ZP(one), a, lda,
             a + zo_index(order, 0, n1, lda), lda);
    ZP(gemm)(order, ZO_NOTRANS, ZO_NOTRANS, m - n1, n2, n1, ZP(mone),
             a + zo_index(order, n1, 0, lda), lda, a + zo_index(order, 0, n1, lda), lda, ZP(one),
             a + zo_index(order, n1, n1, lda), lda);
    iinfo = ZP(getrf2)(order, m - n1, n2, a + zo_index(order, n1, n1, lda), lda, ipiv + n1);
    if (info == 0 && iinfo > 0) info = iinfo + n1;
    for (int i = n1; i < ZO_MIN(m, n); ++i) ipiv[i] = ipiv[i] + n1;
    ZP(laswp)(order, n1, a, lda, n1 + 1, ZO_MIN(m, n), ipiv, 1);
  }
  return info;
}

/* lapack/getrf.zig:14-152: right-looking blocked LU, nb = ilaenv = 64. */
int ZP(getrf)(int order, int m, int n, ZT *a, int lda, int *ipiv) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  int info = 0;
  if (m == 0 || n == 0) return info;
  const int nb = zo_ilaenv(1, "DGETRF", m, n, -1, -1);
  const int mn = ZO_MIN(m, n);
  if (nb <= 1 || nb >= mn) return ZP(getrf2)(order, m, n, a, lda, ipiv);
  for (int j = 0; j < mn; j += nb) {
    const int jb = ZO_MIN(mn - j, nb);
    const int iinfo = ZP(getrf2)(order, m - j, jb, a + zo_index(order, j, j, lda), lda, ipiv + j);
    if (info == 0 && iinfo > 0) info = iinfo + j;
    for (int i = j; i < ZO_MIN(m, j + jb); ++i) ipiv[i] = ipiv[i] + j;
    ZP(laswp)(order, j, a, lda, j + 1, j + jb, ipiv, 1);
    if (j + jb < n) {
      ZP(laswp)(order, n - j - jb, a + zo_index(order, 0, j + jb, lda), lda, j + 1, j + jb, ipiv,
                1);
      ZP(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, jb, n - j - jb, ZP(one),
               a + zo_index(order, j, j, lda), lda, a + zo_index(order, j, j + jb, lda), lda);
      if (j + jb < m)
        ZP(gemm)(order, ZO_NOTRANS, ZO_NOTRANS, m - j - jb, n - j - jb, jb, ZP(mone),
                 a + zo_index(order, j + jb, j, lda), lda, a + zo_index(order, j, j + jb, lda),
                 lda, ZP(one), a + zo_index(order, j + jb, j + jb, lda), lda);
    }
  }
  return info;
}

/* lapack/getrs.zig:13-142: trans N / conj_no_trans: laswp, L, U; trans T /
 * conj_trans: U^T (U^H), L^T (L^H), laswp backwards. */
int ZP(getrs)(int order, int trans, int n, int nrhs, const ZT *a, int lda, const int *ipiv, ZT *b,
              int ldb) {
  const int nota = trans == ZO_NOTRANS || trans == ZO_CONJNOTRANS;
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  if (nota) {
    ZP(laswp)(order, nrhs, b, ldb, 1, n, ipiv, 1);
    ZP(trsm)(order, ZO_LEFT, ZO_LOWER, trans, ZO_UNIT, n, nrhs, ZP(one), a, lda, b, ldb);
    ZP(trsm)(order, ZO_LEFT, ZO_UPPER, trans, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
  } else {
    ZP(trsm)(order, ZO_LEFT, ZO_UPPER, trans, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
    ZP(trsm)(order, ZO_LEFT, ZO_LOWER, trans, ZO_UNIT, n, nrhs, ZP(one), a, lda, b, ldb);
    ZP(laswp)(order, nrhs, b, ldb, 1, n, ipiv, -1);
  }
  return 0;
}

/* lapack/gesv.zig:13-70 */
int ZP(gesv)(int order, int n, int nrhs, ZT *a, int lda, int *ipiv, ZT *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  const int info = ZP(getrf)(order, n, n, a, lda, ipiv);
  if (info == 0) ZP(getrs)(order, ZO_NOTRANS, n, nrhs, a, lda, ipiv, b, ldb);
  return info;
}

/* ---- LAPACK: Cholesky (Hermitian) ----------------------------------------- */

/* lapack/potrf2.zig:17-217: recursive Cholesky, A = U^H U or L L^H; a
 * diagonal entry is re(a) (its imaginary part is not read), and a
 * non-positive or NaN one stops the factorization. */
int ZP(potrf2)(int order, int uplo, int n, ZT *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0) return 0;
  if (n == 1) { /* 37-54 */
    const R ajj = a[0].re;
    if (ajj <= (R)0 || ajj != ajj) return 1;
    a[0] = ZP(c)(ZO_SQRT(ajj), (R)0);
    return 0;
  }
  const int n1 = n / 2, n2 = n - n1;
  int iinfo = ZP(potrf2)(order, uplo, n1, a, lda);
  if (iinfo != 0) return iinfo;
  if (uplo == ZO_UPPER) { /* 72-130 */
    ZP(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, n1, n2, ZP(one), a, lda,
             a + zo_index(order, 0, n1, lda), lda);
    ZP(herk)(order, uplo, ZO_CONJTRANS, n2, n1, (R)-1, a + zo_index(order, 0, n1, lda), lda,
             (R)1, a + zo_index(order, n1, n1, lda), lda);
  } else { /* 133-197 */
    ZP(trsm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n2, n1, ZP(one), a, lda,
             a + zo_index(order, n1, 0, lda), lda);
    ZP(herk)(order, uplo, ZO_NOTRANS, n2, n1, (R)-1, a + zo_index(order, n1, 0, lda), lda, (R)1,
             a + zo_index(order, n1, n1, lda), lda);
  }
  iinfo = ZP(potrf2)(order, uplo, n2, a + zo_index(order, n1, n1, lda), lda);
  if (iinfo != 0) return iinfo + n1;
  return 0;
}

/* lapack/potrf.zig:17-240: blocked left-looking Cholesky, nb = 64, herk for
 * the diagonal block updates (59-90, 149-180). */
int ZP(potrf)(int order, int uplo, int n, ZT *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0) return 0;
  const int nb = zo_ilaenv(1, "DPOTRF", n, -1, -1, -1);
  if (nb <= 1 || nb >= n) return ZP(potrf2)(order, uplo, n, a, lda);
  int info = 0;
  if (uplo == ZO_UPPER) { /* 52-141 */
    for (int j = 0; j < n; j += nb) {
      const int jb = ZO_MIN(nb, n - j);
      ZP(herk)(order, ZO_UPPER, ZO_CONJTRANS, jb, j, (R)-1, a + zo_index(order, 0, j, lda), lda,
               (R)1, a + zo_index(order, j, j, lda), lda);
      info = ZP(potrf2)(order, ZO_UPPER, jb, a + zo_index(order, j, j, lda), lda);
      if (info != 0) return info + j;
      if (j + jb < n) {
        ZP(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, jb, n - j - jb, j, ZP(mone),
                 a + zo_index(order, 0, j, lda), lda, a + zo_index(order, 0, j + jb, lda), lda,
                 ZP(one), a + zo_index(order, j, j + jb, lda), lda);
        ZP(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, jb, n - j - jb, ZP(one),
                 a + zo_index(order, j, j, lda), lda, a + zo_index(order, j, j + jb, lda), lda);
      }
    }
  } else { /* 144-231 */
    for (int j = 0; j < n; j += nb) {
      const int jb = ZO_MIN(nb, n - j);
      ZP(herk)(order, ZO_LOWER, ZO_NOTRANS, jb, j, (R)-1, a + zo_index(order, j, 0, lda), lda,
               (R)1, a + zo_index(order, j, j, lda), lda);
      info = ZP(potrf2)(order, ZO_LOWER, jb, a + zo_index(order, j, j, lda), lda);
      if (info != 0) return info + j;
      if (j + jb < n) {
        ZP(gemm)(order, ZO_NOTRANS, ZO_CONJTRANS, n - j - jb, jb, j, ZP(mone),
                 a + zo_index(order, j + jb, 0, lda), lda, a + zo_index(order, j, 0, lda), lda,
                 ZP(one), a + zo_index(order, j + jb, j, lda), lda);
        ZP(trsm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n - j - jb, jb, ZP(one),
                 a + zo_index(order, j, j, lda), lda, a + zo_index(order, j + jb, j, lda), lda);
      }
    }
  }
  return info;
}

/* lapack/potrs.zig:15-117: U^H U x = b or L L^H x = b. */
int ZP(potrs)(int order, int uplo, int n, int nrhs, const ZT *a, int lda, ZT *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  if (uplo == ZO_UPPER) {
    ZP(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_CONJTRANS, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
    ZP(trsm)(order, ZO_LEFT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
  } else {
    ZP(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_NOTRANS, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
    ZP(trsm)(order, ZO_LEFT, ZO_LOWER, ZO_CONJTRANS, ZO_NONUNIT, n, nrhs, ZP(one), a, lda, b, ldb);
  }
  return 0;
}

/* lapack/posv.zig:15-70 */
int ZP(posv)(int order, int uplo, int n, int nrhs, ZT *a, int lda, ZT *b, int ldb) {
  if (n < 0 || nrhs < 0 || lda < ZO_MAX(1, n) || ldb < ZO_MAX(1, order == ZO_COL ? n : nrhs))
    return ZO_EINVAL;
  if (n == 0 || nrhs == 0) return 0;
  const int info = ZP(potrf)(order, uplo, n, a, lda);
  if (info == 0) ZP(potrs)(order, uplo, n, nrhs, a, lda, b, ldb);
  return info;
}

#undef ZA_
#undef ZB_
#undef ZC_

/* ---- complex Householder QR (geqrf and the branches it takes) ------------- */

/* blas/copy.zig and lapack/lacgv.zig (element-type generic) */
static int ZP(copy)(int n, const ZT *x, int incx, ZT *y, int incy) {
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0, iy = incy < 0 ? (long)(-n + 1) * incy : 0;
  for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] = x[ix];
  return 0;
}
static void ZP(lacgv)(int n, ZT *x, int incx) {
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  for (int i = 0; i < n; ++i, ix += incx) x[ix].im = -x[ix].im;
}

/* blas/nrm2.zig:60-134 (cfloat branch): Blue's scaled sum of squares as in
 * the real branch, every element contributing its re and then its im part. */
R ZP(nrm2)(int n, const ZT *x, int incx) {
  if (n < 0) return (R)-1;
  if (n == 0) return 0;
  const R huge = ZR_TMAX;
  const R tsml = (R)ldexp(1.0, (int)ceil((ZR_EMIN - 1) * 0.5));
  const R tbig = (R)ldexp(1.0, (int)floor((ZR_EMAX - ZR_BITS + 1) * 0.5));
  const R ssml = (R)ldexp(1.0, -(int)floor((ZR_EMIN - ZR_BITS) * 0.5));
  const R sbig = (R)ldexp(1.0, -(int)ceil((ZR_EMAX + ZR_BITS - 1) * 0.5));
  R scl = 1, sumsq = 0, abig = 0, amed = 0, asml = 0;
  int notbig = 1;
  long ix = incx < 0 ? (long)(-n + 1) * incx : 0;
  for (int i = 0; i < n; ++i) {
    for (int part = 0; part < 2; ++part) {
      const R ax = ZO_ABS(part == 0 ? x[ix].re : x[ix].im);
      if (ax > tbig) {
        abig += (ax * sbig) * (ax * sbig);
        notbig = 0;
      } else if (ax < tsml) {
        if (notbig) asml += (ax * ssml) * (ax * ssml);
      } else {
        amed += ax * ax;
      }
    }
    ix += incx;
  }
  if (abig > 0) {
    if (amed > 0 || amed > huge || amed != amed) abig += (amed * sbig) * (amed * sbig);
    scl = (R)1 / sbig;
    sumsq = abig;
  } else if (asml > 0) {
    if (amed > 0 || amed > huge || amed != amed) {
      const R sqrt_amed = ZO_SQRT(amed);
      const R sqrt_asml = ZO_SQRT(asml) / ssml;
      const R ymin = sqrt_asml > sqrt_amed ? sqrt_amed : sqrt_asml;
      const R ymax = sqrt_asml > sqrt_amed ? sqrt_asml : sqrt_amed;
      scl = 1;
      sumsq = (ymax * ymax) * ((R)1 + (ymin / ymax) * (ymin / ymax));
    } else {
      scl = (R)1 / ssml;
      sumsq = asml;
    }
  } else {
    scl = 1;
    sumsq = amed;
  }
  return scl * ZO_SQRT(sumsq);
}

/* lapack/larfg.zig:17-170 (complex): H^H (alpha; x) = (beta; 0) with beta
 * real; tau = (beta - alpha) / beta; x scaled by 1 / (alpha - beta), the
 * real-by-complex quotient of crdiv (larfg.zig:130-137 reaches it as
 * div(1, alpha - beta)); H = I when x = 0 and alpha is real. */
int ZP(larfg)(int n, ZT *alpha, ZT *x, int incx, ZT *tau) {
  if (n <= 0) {
    *tau = ZP(zero);
    return 0;
  }
  R xnorm = ZP(nrm2)(n - 1, x, incx);
  if (xnorm == (R)0 && alpha->im == (R)0) {
    *tau = ZP(zero);
    return 0;
  }
  R beta = -ZCOPYSIGN(ZLAPY3(alpha->re, alpha->im, xnorm), alpha->re);
  const R safmin = ZLAMCH('s') / ZLAMCH('e');
  const R rsafmn = (R)1 / safmin;
  int knt = 0;
  if (ZO_ABS(beta) < safmin) {
    while (ZO_ABS(beta) < safmin && knt < 20) {
      ZP(scal)(n - 1, ZP(c)(rsafmn, (R)0), x, incx);
      beta = beta * rsafmn;
      *alpha = ZP(cscale)(*alpha, rsafmn);
      ++knt;
    }
    xnorm = ZP(nrm2)(n - 1, x, incx);
    beta = -ZCOPYSIGN(ZLAPY3(alpha->re, alpha->im, xnorm), alpha->re);
  }
  *tau = ZP(c)((-alpha->re + beta) / beta, (-alpha->im) / beta);
  *alpha = ZP(crdiv)((R)1, ZP(c)(alpha->re - beta, alpha->im));
  ZP(scal)(n - 1, *alpha, x, incx);
  for (int j = 0; j < knt; ++j) beta = beta * safmin;
  *alpha = ZP(c)(beta, (R)0);
  return 0;
}

/* lapack/ilalc.zig: the last non-zero column (1-based count), 0 if none */
static int ZP(ilalc)(int order, int m, int n, const ZT *a, int lda) {
  if (n == 0) return 0;
  if (!ZP(cis0)(a[zo_index(order, 0, n - 1, lda)]) ||
      !ZP(cis0)(a[zo_index(order, m - 1, n - 1, lda)]))
    return n;
  for (int j = n - 1; j >= 0; --j)
    for (int i = 0; i < m; ++i)
      if (!ZP(cis0)(a[zo_index(order, i, j, lda)])) return j + 1;
  return 0;
}

/* lapack/larf1f.zig:17-259, side left (the only side geqr2 takes):
 * C <- (I - tau v v^H) C with v(0) = 1 implied: w = C(1:,:)^H v(1:) +
 * conj(C(0,:)), C(0,:) -= tau conj(w), C(1:,:) -= tau v(1:) w^H (gerc). */
int ZP(larf1f)(int order, int side, int m, int n, const ZT *v, int incv, ZT tau, ZT *c, int ldc,
               ZT *work) {
  if (side != ZO_LEFT) return ZO_EINVAL; /* not on this path */
  int lastv = 1, lastc = 0;
  if (!ZP(cis0)(tau)) {
    lastv = m;
    long i = incv > 0 ? (long)(lastv - 1) * incv : 0;
    while (lastv > 1 && ZP(cis0)(v[i])) {
      lastv -= 1;
      i -= incv;
    }
    lastc = ZP(ilalc)(order, lastv, n, c, ldc);
  }
  if (lastc == 0) return 0;
  const int rld = order == ZO_COL ? ldc : 1;
  if (lastv == 1) {
    ZP(scal)(lastc, ZP(c)(-tau.re + (R)1, -tau.im), c, rld);
    return 0;
  }
  ZP(gemv)(order, ZO_CONJTRANS, lastv - 1, lastc, ZP(one), c + zo_index(order, 1, 0, ldc), ldc,
           v + incv, incv, ZP(zero), work, 1);
  for (int i = 0; i < lastc; ++i)
    work[i] = ZP(cadd)(work[i], ZP(cconj)(c[zo_index(order, 0, i, ldc)]));
  for (int i = 0; i < lastc; ++i)
    c[zo_index(order, 0, i, ldc)] =
        ZP(csub)(c[zo_index(order, 0, i, ldc)], ZP(cmul)(tau, ZP(cconj)(work[i])));
  ZP(gerc)(order, lastv - 1, lastc, ZP(c)(-tau.re, -tau.im), v + incv, incv, work, 1,
           c + zo_index(order, 1, 0, ldc), ldc);
  return 0;
}

/* lapack/geqr2.zig:17-59: H(i) from larfg, applied as H(i)^H (conj(tau)). */
int ZP(geqr2)(int order, int m, int n, ZT *a, int lda, ZT *tau, ZT *work) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n)) return ZO_EINVAL;
  const int cld = order == ZO_COL ? 1 : lda;
  for (int i = 0; i < ZO_MIN(m, n); ++i) {
    ZP(larfg)(m - i, &a[zo_index(order, i, i, lda)], a + zo_index(order, ZO_MIN(i + 1, m - 1), i, lda),
              cld, &tau[i]);
    if (i < n - 1)
      ZP(larf1f)(order, ZO_LEFT, m - i, n - i - 1, a + zo_index(order, i, i, lda), cld,
                 ZP(cconj)(tau[i]), a + zo_index(order, i, i + 1, lda), lda, work);
  }
  return 0;
}

/* lapack/larft.zig:18-231, the QR branch (forward, columnwise): the
 * recursive T factor, V's entries copied conjugated (larft.zig:104-112). */
int ZP(larft)(int order, int direct, int storev, int n, int k, const ZT *v, int ldv,
              const ZT *tau, ZT *t, int ldt) {
  if (n == 0 || k == 0) return 0;
  if (n == 1 || k == 1) {
    t[zo_index(order, 0, 0, ldt)] = tau[0];
    return 0;
  }
  if (!(direct == 'F' && storev == 'C')) return ZO_EINVAL; /* not on this path */
  const int l = k / 2;
  ZP(larft)(order, direct, storev, n, l, v, ldv, tau, t, ldt);
  ZP(larft)(order, direct, storev, n - l, k - l, v + zo_index(order, l, l, ldv), ldv, tau + l,
            t + zo_index(order, l, l, ldt), ldt);
  for (int j = 0; j < l; ++j)
    for (int i = 0; i < k - l; ++i)
      t[zo_index(order, j, l + i, ldt)] = ZP(cconj)(v[zo_index(order, l + i, j, ldv)]);
  ZP(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, l, k - l, ZP(one),
           v + zo_index(order, l, l, ldv), ldv, t + zo_index(order, 0, l, ldt), ldt);
  ZP(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, l, k - l, n - k, ZP(one),
           v + zo_index(order, k, 0, ldv), ldv, v + zo_index(order, k, l, ldv), ldv, ZP(one),
           t + zo_index(order, 0, l, ldt), ldt);
  ZP(trmm)(order, ZO_LEFT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, l, k - l, ZP(mone), t, ldt,
           t + zo_index(order, 0, l, ldt), ldt);
  ZP(trmm)(order, ZO_RIGHT, ZO_UPPER, ZO_NOTRANS, ZO_NONUNIT, l, k - l, ZP(one),
           t + zo_index(order, l, l, ldt), ldt, t + zo_index(order, 0, l, ldt), ldt);
  return 0;
}

/* lapack/larfb.zig:20-178, side left / forward / columnwise: W := C1^H
 * (copy, lacgv), the T factor applied with trans.reverse(), C1 -= W^H. */
int ZP(larfb)(int order, int side, int trans, int direct, int storev, int m, int n, int k,
              const ZT *v, int ldv, const ZT *t, int ldt, ZT *c, int ldc, ZT *work, int ldwork) {
  if (m <= 0 || n <= 0) return 0;
  if (!(storev == 'C' && direct == 'F' && side == ZO_LEFT)) return ZO_EINVAL; /* not on path */
  const int rldc = order == ZO_COL ? ldc : 1;
  const int cldw = order == ZO_COL ? 1 : ldwork;
  const int rtrans = trans == ZO_NOTRANS ? ZO_CONJTRANS
                   : trans == ZO_TRANS ? ZO_CONJNOTRANS
                   : trans == ZO_CONJNOTRANS ? ZO_TRANS : ZO_NOTRANS; /* linalg.zig:121-128 */
  for (int j = 0; j < k; ++j) {
    ZP(copy)(n, c + zo_index(order, j, 0, ldc), rldc, work + zo_index(order, 0, j, ldwork), cldw);
    ZP(lacgv)(n, work + zo_index(order, 0, j, ldwork), cldw);
  }
  ZP(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_NOTRANS, ZO_UNIT, n, k, ZP(one), v, ldv, work, ldwork);
  if (m > k)
    ZP(gemm)(order, ZO_CONJTRANS, ZO_NOTRANS, n, k, m - k, ZP(one), c + zo_index(order, k, 0, ldc),
             ldc, v + zo_index(order, k, 0, ldv), ldv, ZP(one), work, ldwork);
  ZP(trmm)(order, ZO_RIGHT, ZO_UPPER, rtrans, ZO_NONUNIT, n, k, ZP(one), t, ldt, work, ldwork);
  if (m > k)
    ZP(gemm)(order, ZO_NOTRANS, ZO_CONJTRANS, m - k, n, k, ZP(mone), v + zo_index(order, k, 0, ldv),
             ldv, work, ldwork, ZP(one), c + zo_index(order, k, 0, ldc), ldc);
  ZP(trmm)(order, ZO_RIGHT, ZO_LOWER, ZO_CONJTRANS, ZO_UNIT, n, k, ZP(one), v, ldv, work, ldwork);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < n; ++i)
      c[zo_index(order, j, i, ldc)] =
          ZP(csub)(c[zo_index(order, j, i, ldc)], ZP(cconj)(work[zo_index(order, i, j, ldwork)]));
  return 0;
}

/* lapack/geqrf.zig:18-157 (cfloat): blocked Householder QR, nb = 32,
 * nx = 128, the block reflector applied as H^H (conj_trans, :116). */
int ZP(geqrf)(int order, int m, int n, ZT *a, int lda, ZT *tau, ZT *work, int lwork) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, order == ZO_COL ? m : n) ||
      (lwork != -1 && (lwork < 1 || (m > 0 && lwork < ZO_MAX(1, n)))))
    return ZO_EINVAL;
  const int k = ZO_MIN(m, n);
  int nb = zo_ilaenv(1, "DGEQRF", m, n, -1, -1);
  if (lwork == -1) {
    work[0] = ZP(c)((R)(k == 0 ? 1 : n * nb), (R)0);
    return 0;
  }
  if (k == 0) {
    work[0] = ZP(one);
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
      ZP(geqr2)(order, m - i, ib, a + zo_index(order, i, i, lda), lda, tau + i, work);
      if (i + ib < n) {
        ZP(larft)(order, 'F', 'C', m - i, ib, a + zo_index(order, i, i, lda), lda, tau + i, work,
                  ldwork);
        ZP(larfb)(order, ZO_LEFT, ZO_CONJTRANS, 'F', 'C', m - i, n - i - ib, ib,
                  a + zo_index(order, i, i, lda), lda, work, ldwork,
                  a + zo_index(order, i, i + ib, lda), lda, work + zo_index(order, ib, 0, ldwork),
                  ldwork);
      }
    }
  }
  if (i < k) ZP(geqr2)(order, m - i, n - i, a + zo_index(order, i, i, lda), lda, tau + i, work);
  work[0] = ZP(c)((R)iws, (R)0);
  return 0;
}

/* ---- Hermitian Bunch-Kaufman (unblocked) ------------------------------------ */

/* blas/her.zig:19-380 (k_her): A := alpha x x^H + A on the uplo triangle,
 * alpha real, the diagonal kept real; column j skipped when x[j] == 0 (its
 * diagonal still made real); row-major inverts uplo and conjugates x[i]
 * where column-major conjugates x[j] (her.zig:12-16). */
#define HZ_(i, j) a[(long)(i) + (long)(j) * lda]
static int ZP(k_her)(int uplo, int n, R alpha, const ZT *x, int incx, ZT *a, int lda, int noconj) {
  if (n < 0 || lda < ZO_MAX(1, n) || incx == 0) return ZO_EINVAL;
  if (n == 0 || alpha == (R)0) return 0;
  const long kx = incx < 0 ? (long)(-n + 1) * incx : 0;
  long jx = kx;
  for (int j = 0; j < n; ++j) {
    if (!ZP(cis0)(x[jx])) {
      const ZT temp = ZP(cscale)(noconj ? ZP(cconj)(x[jx]) : x[jx], alpha);
      const ZT xj = noconj ? x[jx] : ZP(cconj)(x[jx]);
      if (uplo == ZO_UPPER) {
        long ix = kx;
        for (int i = 0; i < j; ++i, ix += incx)
          HZ_(i, j) = ZP(cadd)(HZ_(i, j), ZP(cmul)(ZP(cj)(x[ix], !noconj), temp));
        HZ_(j, j) = ZP(c)(HZ_(j, j).re + ZP(cmul)(xj, temp).re, (R)0);
      } else {
        HZ_(j, j) = ZP(c)(HZ_(j, j).re + ZP(cmul)(xj, temp).re, (R)0);
        long ix = jx;
        for (int i = j + 1; i < n; ++i) {
          ix += incx;
          HZ_(i, j) = ZP(cadd)(HZ_(i, j), ZP(cmul)(ZP(cj)(x[ix], !noconj), temp));
        }
      }
    } else {
      HZ_(j, j) = ZP(c)(HZ_(j, j).re, (R)0);
    }
    jx += incx;
  }
  return 0;
}
#undef HZ_
int ZP(her)(int order, int uplo, int n, R alpha, const ZT *x, int incx, ZT *a, int lda) {
  if (order == ZO_COL) return ZP(k_her)(uplo, n, alpha, x, incx, a, lda, 1);
  return ZP(k_her)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, n, alpha, x, incx, a, lda, 0);
}

/* lapack/hetf2.zig:13-666: unblocked Bunch-Kaufman of a Hermitian matrix
 * (LAPACK zhetf2): pivot magnitudes |re a_kk| and |re| + |im| elsewhere, the
 * interchange conjugates the entries it moves across the diagonal, 1x1 steps
 * update with her and a real scaling, 2x2 steps with d = |a_k-1,k| and the
 * conjugated multipliers.  One deliberate difference: for a 2x2 block
 * without interchange the upper branch clears the imaginary part of
 * a(k+1, k+1) as written (hetf2.zig:180-187; past the matrix when
 * k = n - 1); LAPACK's zhetf2 clears a(k-1, k-1), the block's other
 * diagonal entry, and so does this restatement. */
int ZP(hetf2)(int order, int uplo, int n, ZT *a, int lda, int *ipiv) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  int info = 0;
  const R alpha = ((R)1 + ZO_SQRT((R)17)) / (R)8;
  const int cl = order == ZO_COL ? 1 : lda, rl = order == ZO_COL ? lda : 1;
#define HA(i, j) a[zo_index(order, (i), (j), lda)]
  const int up = uplo == ZO_UPPER;
  int k = up ? n - 1 : 0;
  while (up ? k >= 0 : k < n) {
    int kstep = 1, imax = 0, kp;
    const R absakk = ZO_ABS(HA(k, k).re);
    R colmax = 0;
    if (up ? k > 0 : k < n - 1) {
      imax = up ? ZP(iamax)(k, a + zo_index(order, 0, k, lda), cl)
                : k + 1 + ZP(iamax)(n - k - 1, a + zo_index(order, k + 1, k, lda), cl);
      colmax = ZP(cabs1)(HA(imax, k));
    }
    if (ZO_MAX(absakk, colmax) == (R)0 || absakk != absakk) {
      if (info == 0) info = k + 1;
      kp = k;
    } else {
      if (absakk >= alpha * colmax) {
        kp = k;
      } else {
        int jmax;
        R rowmax;
        if (up) {
          jmax = imax + 1 + ZP(iamax)(k - imax, a + zo_index(order, imax, imax + 1, lda), rl);
          rowmax = ZP(cabs1)(HA(imax, jmax));
          if (imax > 0) {
            jmax = ZP(iamax)(imax, a + zo_index(order, 0, imax, lda), cl);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(HA(jmax, imax)));
          }
        } else {
          jmax = k + ZP(iamax)(imax - k, a + zo_index(order, imax, k, lda), rl);
          rowmax = ZP(cabs1)(HA(imax, jmax));
          if (imax < n - 1) {
            jmax = imax + 1 + ZP(iamax)(n - imax - 1, a + zo_index(order, imax + 1, imax, lda), cl);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(HA(jmax, imax)));
          }
        }
        if (absakk >= alpha * (colmax * (colmax / rowmax))) {
          kp = k;
        } else if (ZP(cabs1)(HA(imax, imax)) >= alpha * rowmax) {
          kp = imax;
        } else {
          kp = imax;
          kstep = 2;
        }
      }
      const int kk = up ? k - kstep + 1 : k + kstep - 1;
      if (kp != kk) {
        if (up) {
          for (int i = 0; i < kp; ++i) {
            const ZT t = HA(i, kk);
            HA(i, kk) = HA(i, kp);
            HA(i, kp) = t;
          }
          for (int j = kp + 1; j < kk; ++j) {
            const ZT t = ZP(cconj)(HA(j, kk));
            HA(j, kk) = ZP(cconj)(HA(kp, j));
            HA(kp, j) = t;
          }
        } else {
          for (int i = kp + 1; i < n; ++i) {
            const ZT t = HA(i, kk);
            HA(i, kk) = HA(i, kp);
            HA(i, kp) = t;
          }
          for (int j = kk + 1; j < kp; ++j) {
            const ZT t = ZP(cconj)(HA(j, kk));
            HA(j, kk) = ZP(cconj)(HA(kp, j));
            HA(kp, j) = t;
          }
        }
        HA(kp, kk) = ZP(cconj)(HA(kp, kk));
        const R r1 = HA(kk, kk).re;
        HA(kk, kk) = ZP(c)(HA(kp, kp).re, (R)0);
        HA(kp, kp) = ZP(c)(r1, (R)0);
        if (kstep == 2) {
          HA(k, k).im = 0;
          const int o = up ? k - 1 : k + 1;
          const ZT t = HA(o, k);
          HA(o, k) = HA(kp, k);
          HA(kp, k) = t;
        }
      } else {
        HA(k, k).im = 0;
        if (kstep == 2) HA(up ? k - 1 : k + 1, up ? k - 1 : k + 1).im = 0;
      }
      if (kstep == 1) {
        if (up || k < n - 1) {
          const R r1 = (R)1 / HA(k, k).re;
          const int len = up ? k : n - k - 1;
          ZT *x = up ? a + zo_index(order, 0, k, lda) : a + zo_index(order, k + 1, k, lda);
          ZP(her)(order, uplo, len, -r1, x, cl, up ? a : a + zo_index(order, k + 1, k + 1, lda),
                  lda);
          long ix = 0;
          for (int i = 0; i < len; ++i, ix += cl) x[ix] = ZP(cscale)(x[ix], r1);
        }
      } else if (up ? k > 1 : k < n - 2) {
        const int o = up ? k - 1 : k + 1; /* the block's other column */
        R d = hypot(HA(o, k).re, HA(o, k).im);
        const R dother = HA(o, o).re / d; /* d22 (upper) / d11 (lower) */
        const R dk = HA(k, k).re / d;     /* d11 (upper) / d22 (lower) */
        const R t = (R)1 / (dk * dother - (R)1);
        const ZT dd = ZP(c)(HA(o, k).re / d, HA(o, k).im / d); /* d12 / d21 */
        d = t / d;
        for (int q = 0; q < (up ? k - 1 : n - k - 2); ++q) {
          const int j = up ? k - 2 - q : k + 2 + q;
          ZT wk, wo;
          if (up) { /* wkm1 = d (d11 a_j,k-1 - conj(d12) a_jk), wk = d (d22 a_jk - d12 a_j,k-1) */
            wo = ZP(cscale)(ZP(csub)(ZP(cscale)(HA(j, o), dk), ZP(cmul)(ZP(cconj)(dd), HA(j, k))), d);
            wk = ZP(cscale)(ZP(csub)(ZP(cscale)(HA(j, k), dother), ZP(cmul)(dd, HA(j, o))), d);
          } else { /* wk = d (d11 a_jk - d21 a_j,k+1), wkp1 = d (d22 a_j,k+1 - conj(d21) a_jk) */
            wk = ZP(cscale)(ZP(csub)(ZP(cscale)(HA(j, k), dother), ZP(cmul)(dd, HA(j, o))), d);
            wo = ZP(cscale)(ZP(csub)(ZP(cscale)(HA(j, o), dk), ZP(cmul)(ZP(cconj)(dd), HA(j, k))), d);
          }
          const int i0 = up ? 0 : j, i1 = up ? j + 1 : n;
          for (int i = (up ? j : i0); up ? i >= i0 : i < i1; i += up ? -1 : 1)
            HA(i, j) = ZP(csub)(HA(i, j), ZP(cadd)(ZP(cmul)(HA(i, k), ZP(cconj)(wk)),
                                                   ZP(cmul)(HA(i, o), ZP(cconj)(wo))));
          HA(j, k) = wk;
          HA(j, o) = wo;
          HA(j, j) = ZP(c)(HA(j, j).re, (R)0);
        }
      }
    }
    if (kstep == 1) {
      ipiv[k] = kp + 1;
    } else {
      ipiv[k] = -(kp + 1);
      ipiv[up ? k - 1 : k + 1] = -(kp + 1);
    }
    k = up ? k - kstep : k + kstep;
  }
#undef HA
  return info;
}

/* ---- blocked Hermitian Bunch-Kaufman (hetrf over lahef) -------------------- */

/* blas/gemmtr.zig:69-1032 (complex): the uplo triangle of
 * C := alpha op(A) op(B) + beta C, the loops of complex gemm with the row
 * range cut to the triangle (operand order as gemm's). */
static int ZP(k_gemmtr)(int uplo, int transa, int transb, int n, int k, ZT alpha, const ZT *a,
                        int lda, const ZT *b, int ldb, ZT beta, ZT *c, int ldc) {
  const int nota = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int notb = transb == ZO_NOTRANS || transb == ZO_CONJNOTRANS;
  const int cja = !(transa == ZO_NOTRANS || transa == ZO_TRANS);
  const int cjb = !(transb == ZO_NOTRANS || transb == ZO_TRANS);
  if (n < 0 || k < 0) return ZO_EINVAL;
  if (n == 0) return 0;
  const int up = uplo == ZO_UPPER;
#define GA(i, j) a[(long)(i) + (long)(j) * lda]
#define GB(i, j) b[(long)(i) + (long)(j) * ldb]
#define GC(i, j) c[(long)(i) + (long)(j) * ldc]
  if (ZP(cis0)(alpha)) {
    for (int j = 0; j < n; ++j)
      for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i)
        GC(i, j) = ZP(cis0)(beta) ? ZP(zero) : ZP(cmul)(GC(i, j), beta);
    return 0;
  }
  if (nota) {
    const int plain = notb && !cja && !cjb;
    for (int j = 0; j < n; ++j) {
      const int i0 = up ? 0 : j, i1 = up ? j + 1 : n;
      if (ZP(cis0)(beta)) {
        for (int i = i0; i < i1; ++i) GC(i, j) = ZP(zero);
      } else if (!ZP(cis1)(beta)) {
        for (int i = i0; i < i1; ++i) GC(i, j) = ZP(cmul)(GC(i, j), beta);
      }
      for (int l = 0; l < k; ++l) {
        const ZT bl = ZP(cj)(notb ? GB(l, j) : GB(j, l), cjb);
        const ZT temp = plain ? ZP(cmul)(alpha, bl) : ZP(cmul)(bl, alpha);
        for (int i = i0; i < i1; ++i) {
          const ZT al = ZP(cj)(GA(i, l), cja);
          GC(i, j) = ZP(cadd)(GC(i, j), plain ? ZP(cmul)(temp, al) : ZP(cmul)(al, temp));
        }
      }
    }
  } else {
    for (int j = 0; j < n; ++j)
      for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i) {
        ZT temp = ZP(zero);
        for (int l = 0; l < k; ++l)
          temp = ZP(cadd)(temp, ZP(cmul)(ZP(cj)(GA(l, i), cja), ZP(cj)(notb ? GB(l, j) : GB(j, l), cjb)));
        if (ZP(cis0)(beta)) {
          GC(i, j) = ZP(cmul)(alpha, temp);
        } else if (ZP(cis1)(beta)) {
          GC(i, j) = ZP(cadd)(GC(i, j), ZP(cmul)(alpha, temp));
        } else {
          GC(i, j) = ZP(cmul)(GC(i, j), beta);
          GC(i, j) = ZP(cadd)(GC(i, j), ZP(cmul)(alpha, temp));
        }
      }
  }
#undef GA
#undef GB
#undef GC
  return 0;
}
static int ZP(gemmtr)(int order, int uplo, int transa, int transb, int n, int k, ZT alpha,
                      const ZT *a, int lda, const ZT *b, int ldb, ZT beta, ZT *c, int ldc) {
  if (order == ZO_COL)
    return ZP(k_gemmtr)(uplo, transa, transb, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  return ZP(k_gemmtr)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, transb, transa, n, k, alpha, b, ldb,
                      a, lda, beta, c, ldc);
}

static inline void ZP(swapv)(int n, ZT *x, int incx, ZT *y, int incy) {
  for (long i = 0, ix = 0, iy = 0; i < n; ++i, ix += incx, iy += incy) {
    const ZT t = x[ix];
    x[ix] = y[iy];
    y[iy] = t;
  }
}

/* lapack/lahef.zig:17-1034 (LAPACK zlahef with gemmtr): up to nb columns of
 * the Hermitian Bunch-Kaufman factorization with W = U12 D (upper) or
 * L21 D (lower) built alongside (conjugated rows by lacgv, real
 * diagonals), the rest of the triangle updated by gemmtr, the interchanges
 * of U12 / L21 undone; *kb = the columns factored.  The 2x2 step's
 * d21 = t / d21 is the real-by-complex quotient of crdiv. */
int ZP(lahef)(int order, int uplo, int n, int nb, int *kb, ZT *a, int lda, int *ipiv, ZT *w,
              int ldw) {
  int info = 0;
  const R alpha = ((R)1 + ZO_SQRT((R)17)) / (R)8;
  const int cl = order == ZO_COL ? 1 : lda, rl = order == ZO_COL ? lda : 1;
  const int clw = order == ZO_COL ? 1 : ldw, rlw = order == ZO_COL ? ldw : 1;
#define LA(i, j) a[zo_index(order, (i), (j), lda)]
#define LW(i, j) w[zo_index(order, (i), (j), ldw)]
#define PA(i, j) (a + zo_index(order, (i), (j), lda))
#define PW(i, j) (w + zo_index(order, (i), (j), ldw))
  if (uplo == ZO_UPPER) {
    int k = n - 1, kw;
    while (1) {
      kw = nb + k - n;
      if ((k <= n - nb && nb < n) || k < 0) break;
      ZP(copy)(k, PA(0, k), cl, PW(0, kw), clw);
      LW(k, kw) = ZP(c)(LA(k, k).re, (R)0);
      if (k < n - 1) {
        ZP(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), ZP(mone), PA(0, k + 1), lda, PW(k, kw + 1),
                 rlw, ZP(one), PW(0, kw), clw);
        LW(k, kw) = ZP(c)(LW(k, kw).re, (R)0);
      }
      int kstep = 1, imax = 0, kp;
      const R absakk = ZO_ABS(LW(k, kw).re);
      R colmax = 0;
      if (k > 0) {
        imax = ZP(iamax)(k, PW(0, kw), clw);
        colmax = ZP(cabs1)(LW(imax, kw));
      }
      if (ZO_MAX(absakk, colmax) == (R)0) {
        if (info == 0) info = k + 1;
        kp = k;
        LA(k, k) = ZP(c)(LA(k, k).re, (R)0);
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          ZP(copy)(imax, PA(0, imax), cl, PW(0, kw - 1), clw);
          LW(imax, kw - 1) = ZP(c)(LA(imax, imax).re, (R)0);
          ZP(copy)(k - imax, PA(imax, imax + 1), rl, PW(imax + 1, kw - 1), clw);
          ZP(lacgv)(k - imax, PW(imax + 1, kw - 1), clw);
          if (k < n - 1) {
            ZP(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), ZP(mone), PA(0, k + 1), lda,
                     PW(imax, kw + 1), rlw, ZP(one), PW(0, kw - 1), clw);
            LW(imax, kw - 1) = ZP(c)(LW(imax, kw - 1).re, (R)0);
          }
          int jmax = imax + 1 + ZP(iamax)(k - imax, PW(imax + 1, kw - 1), clw);
          R rowmax = ZP(cabs1)(LW(jmax, kw - 1));
          if (imax > 0) {
            jmax = ZP(iamax)(imax, PW(0, kw - 1), clw);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(LW(jmax, kw - 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(LW(imax, kw - 1).re) >= alpha * rowmax) {
            kp = imax;
            ZP(copy)(k + 1, PW(0, kw - 1), clw, PW(0, kw), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k - kstep + 1, kkw = nb + kk - n;
        if (kp != kk) {
          LA(kp, kp) = ZP(c)(LA(kk, kk).re, (R)0);
          ZP(copy)(kk - kp - 1, PA(kp + 1, kk), cl, PA(kp, kp + 1), rl);
          ZP(lacgv)(kk - kp - 1, PA(kp, kp + 1), rl);
          if (kp > 0) ZP(copy)(kp, PA(0, kk), cl, PA(0, kp), cl);
          if (k < n - 1) ZP(swapv)(n - (k + 1), PA(kk, k + 1), rl, PA(kp, k + 1), rl);
          ZP(swapv)(n - kk, PW(kk, kkw), rlw, PW(kp, kkw), rlw);
        }
        if (kstep == 1) {
          ZP(copy)(k + 1, PW(0, kw), clw, PA(0, k), cl);
          if (k > 0) {
            const R r1 = (R)1 / LA(k, k).re;
            for (int i = 0; i < k; ++i) LA(i, k) = ZP(cscale)(LA(i, k), r1);
            ZP(lacgv)(k, PW(0, kw), clw);
          }
        } else {
          if (k > 1) {
            ZT d21 = LW(k - 1, kw);
            const ZT d11 = ZP(cdiv)(LW(k, kw), ZP(cconj)(d21));
            const ZT d22 = ZP(cdiv)(LW(k - 1, kw - 1), d21);
            const R t = (R)1 / (ZP(cmul)(d11, d22).re - (R)1);
            d21 = ZP(crdiv)(t, d21);
            for (int j = 0; j < k - 1; ++j) {
              LA(j, k - 1) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d11, LW(j, kw - 1)), LW(j, kw)));
              LA(j, k) = ZP(cmul)(ZP(cconj)(d21), ZP(csub)(ZP(cmul)(d22, LW(j, kw)), LW(j, kw - 1)));
            }
          }
          LA(k - 1, k - 1) = LW(k - 1, kw - 1);
          LA(k - 1, k) = LW(k - 1, kw);
          LA(k, k) = LW(k, kw);
          ZP(lacgv)(k, PW(0, kw), clw);
          ZP(lacgv)(k - 1, PW(0, kw - 1), clw);
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k - 1] = -(kp + 1);
      }
      k -= kstep;
    }
    ZP(gemmtr)(order, ZO_UPPER, ZO_NOTRANS, ZO_TRANS, k + 1, n - (k + 1), ZP(mone), PA(0, k + 1),
               lda, PW(0, kw + 1), ldw, ZP(one), a, lda);
    int j = k + 1;
    while (j < n) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j += 1;
      }
      j += 1;
      if (jp - 1 != jj && j < n) ZP(swapv)(n - j, PA(jp - 1, j), rl, PA(jj, j), rl);
    }
    *kb = n - k - 1;
  } else {
    int k = 0;
    while (1) {
      if ((k >= nb - 1 && nb < n) || k > n - 1) break;
      LW(k, k) = ZP(c)(LA(k, k).re, (R)0);
      if (k < n - 1) ZP(copy)(n - k - 1, PA(k + 1, k), cl, PW(k + 1, k), clw);
      ZP(gemv)(order, ZO_NOTRANS, n - k, k, ZP(mone), PA(k, 0), lda, PW(k, 0), rlw, ZP(one),
               PW(k, k), clw);
      LW(k, k) = ZP(c)(LW(k, k).re, (R)0);
      int kstep = 1, imax = 0, kp;
      const R absakk = ZO_ABS(LW(k, k).re);
      R colmax = 0;
      if (k < n - 1) {
        imax = k + 1 + ZP(iamax)(n - k - 1, PW(k + 1, k), clw);
        colmax = ZP(cabs1)(LW(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (R)0) {
        if (info == 0) info = k + 1;
        kp = k;
        LA(k, k) = ZP(c)(LA(k, k).re, (R)0);
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          ZP(copy)(imax - k, PA(imax, k), rl, PW(k, k + 1), clw);
          ZP(lacgv)(imax - k, PW(k, k + 1), clw);
          LW(imax, k + 1) = ZP(c)(LA(imax, imax).re, (R)0);
          if (imax < n - 1) ZP(copy)(n - imax - 1, PA(imax + 1, imax), cl, PW(imax + 1, k + 1), clw);
          ZP(gemv)(order, ZO_NOTRANS, n - k, k, ZP(mone), PA(k, 0), lda, PW(imax, 0), rlw, ZP(one),
                   PW(k, k + 1), clw);
          LW(imax, k + 1) = ZP(c)(LW(imax, k + 1).re, (R)0);
          int jmax = k + ZP(iamax)(imax - k, PW(k, k + 1), clw);
          R rowmax = ZP(cabs1)(LW(jmax, k + 1));
          if (imax < n - 1) {
            jmax = imax + 1 + ZP(iamax)(n - imax - 1, PW(imax + 1, k + 1), clw);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(LW(jmax, k + 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(LW(imax, k + 1).re) >= alpha * rowmax) {
            kp = imax;
            ZP(copy)(n - k, PW(k, k + 1), clw, PW(k, k), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k + kstep - 1;
        if (kp != kk) {
          LA(kp, kp) = ZP(c)(LA(kk, kk).re, (R)0);
          ZP(copy)(kp - kk - 1, PA(kk + 1, kk), cl, PA(kp, kk + 1), rl);
          ZP(lacgv)(kp - kk - 1, PA(kp, kk + 1), rl);
          if (kp < n - 1) ZP(copy)(n - kp - 1, PA(kp + 1, kk), cl, PA(kp + 1, kp), cl);
          if (k > 0) ZP(swapv)(k, PA(kk, 0), rl, PA(kp, 0), rl);
          ZP(swapv)(kk + 1, PW(kk, 0), rlw, PW(kp, 0), rlw);
        }
        if (kstep == 1) {
          ZP(copy)(n - k, PW(k, k), clw, PA(k, k), cl);
          if (k < n - 1) {
            const R r1 = (R)1 / LA(k, k).re;
            for (int i = k + 1; i < n; ++i) LA(i, k) = ZP(cscale)(LA(i, k), r1);
            ZP(lacgv)(n - k - 1, PW(k + 1, k), clw);
          }
        } else {
          if (k < n - 2) {
            ZT d21 = LW(k + 1, k);
            const ZT d11 = ZP(cdiv)(LW(k + 1, k + 1), d21);
            const ZT d22 = ZP(cdiv)(LW(k, k), ZP(cconj)(d21));
            const R t = (R)1 / (ZP(cmul)(d11, d22).re - (R)1);
            d21 = ZP(crdiv)(t, d21);
            for (int j = k + 2; j < n; ++j) {
              LA(j, k) = ZP(cmul)(ZP(cconj)(d21), ZP(csub)(ZP(cmul)(d11, LW(j, k)), LW(j, k + 1)));
              LA(j, k + 1) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d22, LW(j, k + 1)), LW(j, k)));
            }
          }
          LA(k, k) = LW(k, k);
          LA(k + 1, k) = LW(k + 1, k);
          LA(k + 1, k + 1) = LW(k + 1, k + 1);
          ZP(lacgv)(n - k - 1, PW(k + 1, k), clw);
          ZP(lacgv)(n - k - 2, PW(k + 2, k + 1), clw);
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k + 1] = -(kp + 1);
      }
      k += kstep;
    }
    ZP(gemmtr)(order, ZO_LOWER, ZO_NOTRANS, ZO_TRANS, n - k, k, ZP(mone), PA(k, 0), lda, PW(k, 0),
               ldw, ZP(one), PA(k, k), lda);
    int j = k - 1;
    while (j > 0) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j -= 1;
      }
      j -= 1;
      if (jp - 1 != jj && j >= 0) ZP(swapv)(j + 1, PA(jp - 1, 0), rl, PA(jj, 0), rl);
    }
    *kb = k;
  }
#undef LA
#undef LW
#undef PA
#undef PW
  return info;
}

/* lapack/hetrf.zig:17-187: blocks of nb = ilaenv("CHETRF") = 64 by lahef
 * while more than nb columns remain, the rest by hetf2 (LAPACK zhetrf). */
int ZP(hetrf)(int order, int uplo, int n, ZT *a, int lda, int *ipiv, ZT *work, int lwork) {
  if (n < 0 || lda < ZO_MAX(1, n) || (lwork < 1 && lwork != -1)) return ZO_EINVAL;
  int info = 0;
  int nb = zo_ilaenv(1, "CHETRF", n, -1, -1, -1);
  work[0] = ZP(c)((R)ZO_MAX(1, n * nb), (R)0);
  if (lwork == -1) return info;
  int nbmin = 2;
  const int ldwork = order == ZO_COL ? n : nb;
  if (nb > 1 && nb < n && lwork < ldwork * nb) {
    nb = ZO_MAX(lwork / ldwork, 1);
    nbmin = ZO_MAX(2, zo_ilaenv(2, "DSYTRF", n, -1, -1, -1));
  }
  if (nb < nbmin) nb = n;
  if (uplo == ZO_UPPER) {
    int k = n - 1;
    while (k >= 0) {
      int kb, iinfo;
      if (k + 1 > nb) {
        iinfo = ZP(lahef)(order, ZO_UPPER, k + 1, nb, &kb, a, lda, ipiv, work, ldwork);
      } else {
        iinfo = ZP(hetf2)(order, ZO_UPPER, k + 1, a, lda, ipiv);
        kb = k + 1;
      }
      if (info == 0 && iinfo > 0) info = iinfo;
      k -= kb;
    }
  } else {
    int k = 0;
    while (k < n) {
      int kb, iinfo;
      if (k <= n - nb - 1) {
        iinfo = ZP(lahef)(order, ZO_LOWER, n - k, nb, &kb, a + zo_index(order, k, k, lda), lda,
                          ipiv + k, work, ldwork);
      } else {
        iinfo = ZP(hetf2)(order, ZO_LOWER, n - k, a + zo_index(order, k, k, lda), lda, ipiv + k);
        kb = n - k;
      }
      if (info == 0 && iinfo > 0) info = iinfo + k;
      for (int j = k; j < k + kb; ++j) ipiv[j] = ipiv[j] > 0 ? ipiv[j] + k : ipiv[j] - k;
      k += kb;
    }
  }
  return info;
}

/* ---- complex symmetric Bunch-Kaufman (sytrf over lasyf / sytf2) ------------ */
/* The same routines as the real ones, instantiated for cfloat: A = U D U^T or
 * L D L^T without conjugation, pivots chosen by |re| + |im|.  zml's scalar
 * "1 / z" (the 1x1 step's r1, the 2x2 step's t) is a real by complex
 * quotient and goes through crdiv; sub(z, 1) is component-wise. */

static inline ZT ZP(sub1)(ZT z) { return ZP(c)(z.re - (R)1, z.im); }

/* blas/syr.zig:32-225 (complex): A := alpha x x^T + A on the uplo triangle,
 * column j skipped when x[j] == 0; row-major inverts uplo. */
static int ZP(k_syr)(int uplo, int n, ZT alpha, const ZT *x, int incx, ZT *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n) || incx == 0) return ZO_EINVAL;
  if (n == 0 || ZP(cis0)(alpha)) return 0;
  const long kx = incx < 0 ? (long)(-n + 1) * incx : 0;
  long jx = kx;
#define YA(i, j) a[(long)(i) + (long)(j) * lda]
  for (int j = 0; j < n; ++j) {
    if (!ZP(cis0)(x[jx])) {
      const ZT temp = ZP(cmul)(x[jx], alpha);
      if (uplo == ZO_UPPER) {
        long ix = kx;
        for (int i = 0; i < j; ++i) {
          YA(i, j) = ZP(cadd)(YA(i, j), ZP(cmul)(x[ix], temp));
          ix += incx;
        }
        YA(j, j) = ZP(cadd)(YA(j, j), ZP(cmul)(x[jx], temp));
      } else {
        YA(j, j) = ZP(cadd)(YA(j, j), ZP(cmul)(x[jx], temp));
        long ix = jx;
        for (int i = j + 1; i < n; ++i) {
          ix += incx;
          YA(i, j) = ZP(cadd)(YA(i, j), ZP(cmul)(x[ix], temp));
        }
      }
    }
    jx += incx;
  }
#undef YA
  return 0;
}
int ZP(syr)(int order, int uplo, int n, ZT alpha, const ZT *x, int incx, ZT *a, int lda) {
  return ZP(k_syr)(order == ZO_COL ? uplo : (uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER), n, alpha, x,
                   incx, a, lda);
}

#define YA(i, j) a[zo_index(order, (i), (j), lda)]
#define YW(i, j) w[zo_index(order, (i), (j), ldw)]
#define QA(i, j) (a + zo_index(order, (i), (j), lda))
#define QW(i, j) (w + zo_index(order, (i), (j), ldw))

/* lapack/sytf2.zig:17-522 (complex): unblocked Bunch-Kaufman (LAPACK
 * zsytf2); a zero or NaN pivot column records info and is left as it is. */
int ZP(sytf2)(int order, int uplo, int n, ZT *a, int lda, int *ipiv) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  int info = 0;
  const R alpha = ((R)1 + ZO_SQRT((R)17)) / (R)8;
  const int cl = order == ZO_COL ? 1 : lda, rl = order == ZO_COL ? lda : 1;
  if (uplo == ZO_UPPER) {
    int k = n - 1;
    while (k >= 0) {
      int kstep = 1, kp, imax = 0;
      const R absakk = ZP(cabs1)(YA(k, k));
      R colmax = 0;
      if (k > 0) {
        imax = ZP(iamax)(k, QA(0, k), cl);
        colmax = ZP(cabs1)(YA(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (R)0 || absakk != absakk) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          int jmax = imax + 1 + ZP(iamax)(k - imax, QA(imax, imax + 1), rl);
          R rowmax = ZP(cabs1)(YA(imax, jmax));
          if (imax > 0) {
            jmax = ZP(iamax)(imax, QA(0, imax), cl);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(YA(jmax, imax)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZP(cabs1)(YA(imax, imax)) >= alpha * rowmax) {
            kp = imax;
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k - kstep + 1;
        if (kp != kk) {
          ZP(swapv)(kp, QA(0, kk), cl, QA(0, kp), cl);
          ZP(swapv)(kk - kp - 1, QA(kp + 1, kk), cl, QA(kp, kp + 1), rl);
          ZT t = YA(kk, kk);
          YA(kk, kk) = YA(kp, kp);
          YA(kp, kp) = t;
          if (kstep == 2) {
            t = YA(k - 1, k);
            YA(k - 1, k) = YA(kp, k);
            YA(kp, k) = t;
          }
        }
        if (kstep == 1) {
          const ZT r1 = ZP(crdiv)((R)1, YA(k, k));
          ZP(syr)(order, uplo, k, ZP(c)(-r1.re, -r1.im), QA(0, k), cl, a, lda);
          ZP(scal)(k, r1, QA(0, k), cl);
        } else if (k > 1) {
          ZT d12 = YA(k - 1, k);
          const ZT d22 = ZP(cdiv)(YA(k - 1, k - 1), d12);
          const ZT d11 = ZP(cdiv)(YA(k, k), d12);
          const ZT t = ZP(crdiv)((R)1, ZP(sub1)(ZP(cmul)(d11, d22)));
          d12 = ZP(cdiv)(t, d12);
          for (int j = k - 2; j >= 0; --j) {
            const ZT wkm1 = ZP(cmul)(d12, ZP(csub)(ZP(cmul)(d11, YA(j, k - 1)), YA(j, k)));
            const ZT wk = ZP(cmul)(d12, ZP(csub)(ZP(cmul)(d22, YA(j, k)), YA(j, k - 1)));
            for (int i = j; i >= 0; --i)
              YA(i, j) = ZP(csub)(YA(i, j), ZP(cadd)(ZP(cmul)(YA(i, k), wk), ZP(cmul)(YA(i, k - 1), wkm1)));
            YA(j, k) = wk;
            YA(j, k - 1) = wkm1;
          }
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k - 1] = -(kp + 1);
      }
      k -= kstep;
    }
  } else {
    int k = 0;
    while (k < n) {
      int kstep = 1, kp, imax = 0;
      const R absakk = ZP(cabs1)(YA(k, k));
      R colmax = 0;
      if (k < n - 1) {
        imax = k + 1 + ZP(iamax)(n - k - 1, QA(k + 1, k), cl);
        colmax = ZP(cabs1)(YA(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (R)0 || absakk != absakk) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          int jmax = k + ZP(iamax)(imax - k, QA(imax, k), rl);
          R rowmax = ZP(cabs1)(YA(imax, jmax));
          if (imax < n - 1) {
            jmax = imax + 1 + ZP(iamax)(n - imax - 1, QA(imax + 1, imax), cl);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(YA(jmax, imax)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZP(cabs1)(YA(imax, imax)) >= alpha * rowmax) {
            kp = imax;
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k + kstep - 1;
        if (kp != kk) {
          if (kp < n - 1) ZP(swapv)(n - kp - 1, QA(kp + 1, kk), cl, QA(kp + 1, kp), cl);
          ZP(swapv)(kp - kk - 1, QA(kk + 1, kk), cl, QA(kp, kk + 1), rl);
          ZT t = YA(kk, kk);
          YA(kk, kk) = YA(kp, kp);
          YA(kp, kp) = t;
          if (kstep == 2) {
            t = YA(k + 1, k);
            YA(k + 1, k) = YA(kp, k);
            YA(kp, k) = t;
          }
        }
        if (kstep == 1) {
          if (k < n - 1) {
            const ZT d11 = ZP(crdiv)((R)1, YA(k, k));
            ZP(syr)(order, uplo, n - k - 1, ZP(c)(-d11.re, -d11.im), QA(k + 1, k), cl,
                    QA(k + 1, k + 1), lda);
            ZP(scal)(n - k - 1, d11, QA(k + 1, k), cl);
          }
        } else if (k < n - 2) {
          ZT d21 = YA(k + 1, k);
          const ZT d11 = ZP(cdiv)(YA(k + 1, k + 1), d21);
          const ZT d22 = ZP(cdiv)(YA(k, k), d21);
          const ZT t = ZP(crdiv)((R)1, ZP(sub1)(ZP(cmul)(d11, d22)));
          d21 = ZP(cdiv)(t, d21);
          for (int j = k + 2; j < n; ++j) {
            const ZT wk = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d11, YA(j, k)), YA(j, k + 1)));
            const ZT wkp1 = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d22, YA(j, k + 1)), YA(j, k)));
            for (int i = j; i < n; ++i)
              YA(i, j) = ZP(csub)(YA(i, j), ZP(cadd)(ZP(cmul)(YA(i, k), wk), ZP(cmul)(YA(i, k + 1), wkp1)));
            YA(j, k) = wk;
            YA(j, k + 1) = wkp1;
          }
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k + 1] = -(kp + 1);
      }
      k += kstep;
    }
  }
  return info;
}

/* lapack/lasyf.zig:17-896 (complex, LAPACK zlasyf with gemmtr): up to nb
 * columns with W = U12 D or L21 D built alongside, the rest of the triangle
 * updated by gemmtr, the later interchanges undone; *kb = columns factored. */
int ZP(lasyf)(int order, int uplo, int n, int nb, int *kb, ZT *a, int lda, int *ipiv, ZT *w,
              int ldw) {
  int info = 0;
  const R alpha = ((R)1 + ZO_SQRT((R)17)) / (R)8;
  const int cl = order == ZO_COL ? 1 : lda, rl = order == ZO_COL ? lda : 1;
  const int clw = order == ZO_COL ? 1 : ldw, rlw = order == ZO_COL ? ldw : 1;
  if (uplo == ZO_UPPER) {
    int k = n - 1, kw;
    while (1) {
      kw = nb + k - n;
      if ((k <= n - nb && nb < n) || k < 0) break;
      ZP(copy)(k + 1, QA(0, k), cl, QW(0, kw), clw);
      if (k < n - 1)
        ZP(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), ZP(mone), QA(0, k + 1), lda, QW(k, kw + 1),
                 rlw, ZP(one), QW(0, kw), clw);
      int kstep = 1, imax = 0, kp;
      const R absakk = ZP(cabs1)(YW(k, kw));
      R colmax = 0;
      if (k > 0) {
        imax = ZP(iamax)(k, QW(0, kw), clw);
        colmax = ZP(cabs1)(YW(imax, kw));
      }
      if (ZO_MAX(absakk, colmax) == (R)0) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          ZP(copy)(imax + 1, QA(0, imax), cl, QW(0, kw - 1), clw);
          ZP(copy)(k - imax, QA(imax, imax + 1), rl, QW(imax + 1, kw - 1), clw);
          if (k < n - 1)
            ZP(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), ZP(mone), QA(0, k + 1), lda,
                     QW(imax, kw + 1), rlw, ZP(one), QW(0, kw - 1), clw);
          int jmax = imax + 1 + ZP(iamax)(k - imax, QW(imax + 1, kw - 1), clw);
          R rowmax = ZP(cabs1)(YW(jmax, kw - 1));
          if (imax > 0) {
            jmax = ZP(iamax)(imax, QW(0, kw - 1), clw);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(YW(jmax, kw - 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZP(cabs1)(YW(imax, kw - 1)) >= alpha * rowmax) {
            kp = imax;
            ZP(copy)(k + 1, QW(0, kw - 1), clw, QW(0, kw), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k - kstep + 1, kkw = nb + kk - n;
        if (kp != kk) {
          YA(kp, kp) = YA(kk, kk);
          ZP(copy)(kk - kp - 1, QA(kp + 1, kk), cl, QA(kp, kp + 1), rl);
          if (kp > 0) ZP(copy)(kp, QA(0, kk), cl, QA(0, kp), cl);
          if (k < n - 1) ZP(swapv)(n - (k + 1), QA(kk, k + 1), rl, QA(kp, k + 1), rl);
          ZP(swapv)(n - kk, QW(kk, kkw), rlw, QW(kp, kkw), rlw);
        }
        if (kstep == 1) {
          ZP(copy)(k + 1, QW(0, kw), clw, QA(0, k), cl);
          const ZT r1 = ZP(crdiv)((R)1, YA(k, k));
          ZP(scal)(k, r1, QA(0, k), cl);
        } else {
          if (k > 1) {
            ZT d21 = YW(k - 1, kw);
            const ZT d11 = ZP(cdiv)(YW(k, kw), d21);
            const ZT d22 = ZP(cdiv)(YW(k - 1, kw - 1), d21);
            const ZT t = ZP(crdiv)((R)1, ZP(sub1)(ZP(cmul)(d11, d22)));
            d21 = ZP(cdiv)(t, d21);
            for (int j = 0; j < k - 1; ++j) {
              YA(j, k - 1) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d11, YW(j, kw - 1)), YW(j, kw)));
              YA(j, k) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d22, YW(j, kw)), YW(j, kw - 1)));
            }
          }
          YA(k - 1, k - 1) = YW(k - 1, kw - 1);
          YA(k - 1, k) = YW(k - 1, kw);
          YA(k, k) = YW(k, kw);
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k - 1] = -(kp + 1);
      }
      k -= kstep;
    }
    ZP(gemmtr)(order, ZO_UPPER, ZO_NOTRANS, ZO_TRANS, k + 1, n - (k + 1), ZP(mone), QA(0, k + 1),
               lda, QW(0, kw + 1), ldw, ZP(one), a, lda);
    int j = k + 1;
    while (j < n) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j += 1;
      }
      j += 1;
      if (jp - 1 != jj && j < n) ZP(swapv)(n - j, QA(jp - 1, j), rl, QA(jj, j), rl);
    }
    *kb = n - k - 1;
  } else {
    int k = 0;
    while (1) {
      if ((k >= nb - 1 && nb < n) || k > n - 1) break;
      ZP(copy)(n - k, QA(k, k), cl, QW(k, k), clw);
      ZP(gemv)(order, ZO_NOTRANS, n - k, k, ZP(mone), QA(k, 0), lda, QW(k, 0), rlw, ZP(one),
               QW(k, k), clw);
      int kstep = 1, imax = 0, kp;
      const R absakk = ZP(cabs1)(YW(k, k));
      R colmax = 0;
      if (k < n - 1) {
        imax = k + 1 + ZP(iamax)(n - k - 1, QW(k + 1, k), clw);
        colmax = ZP(cabs1)(YW(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (R)0) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          ZP(copy)(imax - k, QA(imax, k), rl, QW(k, k + 1), clw);
          ZP(copy)(n - imax, QA(imax, imax), cl, QW(imax, k + 1), clw);
          ZP(gemv)(order, ZO_NOTRANS, n - k, k, ZP(mone), QA(k, 0), lda, QW(imax, 0), rlw, ZP(one),
                   QW(k, k + 1), clw);
          int jmax = k + ZP(iamax)(imax - k, QW(k, k + 1), clw);
          R rowmax = ZP(cabs1)(YW(jmax, k + 1));
          if (imax < n - 1) {
            jmax = imax + 1 + ZP(iamax)(n - imax - 1, QW(imax + 1, k + 1), clw);
            rowmax = ZO_MAX(rowmax, ZP(cabs1)(YW(jmax, k + 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZP(cabs1)(YW(imax, k + 1)) >= alpha * rowmax) {
            kp = imax;
            ZP(copy)(n - k, QW(k, k + 1), clw, QW(k, k), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k + kstep - 1;
        if (kp != kk) {
          YA(kp, kp) = YA(kk, kk);
          ZP(copy)(kp - kk - 1, QA(kk + 1, kk), cl, QA(kp, kk + 1), rl);
          if (kp < n - 1) ZP(copy)(n - kp - 1, QA(kp + 1, kk), cl, QA(kp + 1, kp), cl);
          if (k > 0) ZP(swapv)(k, QA(kk, 0), rl, QA(kp, 0), rl);
          ZP(swapv)(kk + 1, QW(kk, 0), rlw, QW(kp, 0), rlw);
        }
        if (kstep == 1) {
          ZP(copy)(n - k, QW(k, k), clw, QA(k, k), cl);
          if (k < n - 1) {
            const ZT r1 = ZP(crdiv)((R)1, YA(k, k));
            ZP(scal)(n - k - 1, r1, QA(k + 1, k), cl);
          }
        } else {
          if (k < n - 2) {
            ZT d21 = YW(k + 1, k);
            const ZT d11 = ZP(cdiv)(YW(k + 1, k + 1), d21);
            const ZT d22 = ZP(cdiv)(YW(k, k), d21);
            const ZT t = ZP(crdiv)((R)1, ZP(sub1)(ZP(cmul)(d11, d22)));
            d21 = ZP(cdiv)(t, d21);
            for (int j = k + 2; j < n; ++j) {
              YA(j, k) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d11, YW(j, k)), YW(j, k + 1)));
              YA(j, k + 1) = ZP(cmul)(d21, ZP(csub)(ZP(cmul)(d22, YW(j, k + 1)), YW(j, k)));
            }
          }
          YA(k, k) = YW(k, k);
          YA(k + 1, k) = YW(k + 1, k);
          YA(k + 1, k + 1) = YW(k + 1, k + 1);
        }
      }
      if (kstep == 1) {
        ipiv[k] = kp + 1;
      } else {
        ipiv[k] = -(kp + 1);
        ipiv[k + 1] = -(kp + 1);
      }
      k += kstep;
    }
    ZP(gemmtr)(order, ZO_LOWER, ZO_NOTRANS, ZO_TRANS, n - k, k, ZP(mone), QA(k, 0), lda, QW(k, 0),
               ldw, ZP(one), QA(k, k), lda);
    int j = k - 1;
    while (j > 0) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j -= 1;
      }
      j -= 1;
      if (jp - 1 != jj && j >= 0) ZP(swapv)(j + 1, QA(jp - 1, 0), rl, QA(jj, 0), rl);
    }
    *kb = k;
  }
  return info;
}
#undef YA
#undef YW
#undef QA
#undef QW

/* lapack/sytrf.zig:17-187 (complex): blocks of nb = ilaenv("DSYTRF") = 64 by
 * lasyf while more than nb columns remain, the rest by sytf2 (LAPACK zsytrf). */
int ZP(sytrf)(int order, int uplo, int n, ZT *a, int lda, int *ipiv, ZT *work, int lwork) {
  if (n < 0 || lda < ZO_MAX(1, n) || (lwork < 1 && lwork != -1)) return ZO_EINVAL;
  int info = 0;
  int nb = zo_ilaenv(1, "DSYTRF", n, -1, -1, -1);
  work[0] = ZP(c)((R)ZO_MAX(1, n * nb), (R)0);
  if (lwork == -1) return info;
  int nbmin = 2;
  const int ldwork = order == ZO_COL ? n : nb;
  if (nb > 1 && nb < n && lwork < ldwork * nb) {
    nb = ZO_MAX(lwork / ldwork, 1);
    nbmin = ZO_MAX(2, zo_ilaenv(2, "DSYTRF", n, -1, -1, -1));
  }
  if (nb < nbmin) nb = n;
  if (uplo == ZO_UPPER) {
    int k = n - 1;
    while (k >= 0) {
      int kb, iinfo;
      if (k + 1 > nb) {
        iinfo = ZP(lasyf)(order, ZO_UPPER, k + 1, nb, &kb, a, lda, ipiv, work, ldwork);
      } else {
        iinfo = ZP(sytf2)(order, ZO_UPPER, k + 1, a, lda, ipiv);
        kb = k + 1;
      }
      if (info == 0 && iinfo > 0) info = iinfo;
      k -= kb;
    }
  } else {
    int k = 0;
    while (k < n) {
      int kb, iinfo;
      if (k <= n - nb - 1) {
        iinfo = ZP(lasyf)(order, ZO_LOWER, n - k, nb, &kb, a + zo_index(order, k, k, lda), lda,
                          ipiv + k, work, ldwork);
      } else {
        iinfo = ZP(sytf2)(order, ZO_LOWER, n - k, a + zo_index(order, k, k, lda), lda, ipiv + k);
        kb = n - k;
      }
      if (info == 0 && iinfo > 0) info = iinfo + k;
      for (int j = k; j < k + kb; ++j) ipiv[j] = ipiv[j] > 0 ? ipiv[j] + k : ipiv[j] - k;
      k += kb;
    }
  }
  return info;
}
