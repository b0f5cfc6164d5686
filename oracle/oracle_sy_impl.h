/*
 * oracle_sy_impl.h -- Bunch-Kaufman symmetric-indefinite factorization of the
 * zml oracle (TEST INFRASTRUCTURE): A = U D U^T or L D L^T with 1x1 and 2x2
 * pivot blocks (lapack/sytrf.zig, lasyf.zig, sytf2.zig) and the BLAS they
 * call that oracle_impl.h does not hold (blas/syr.zig, gemmtr.zig).
 *
 * Included once per element type after oracle_impl.h and oracle_qr_impl.h
 * (T, P(x) as there).  Each routine restates the cited Zig code in its loop
 * order and association (e.g. the 2x2 update subtracts the SUM of the two
 * products, sytf2.zig:222-236, where LAPACK's Fortran subtracts them in
 * turn).  ipiv follows LAPACK: k+1 for a 1x1 block at k, -(p+1) on both
 * columns of a 2x2 block whose interchange row is p.
 */

static inline int P(row_ld)(int order, int ld) { return order == ZO_COL ? ld : 1; } /* utils.zig:17-19 */

#define SA(i, j) a[P(idx)(order, (i), (j), lda)]
#define SW(i, j) w[P(idx)(order, (i), (j), ldw)]
#define SYA_(i, j) a[(long)(i) + (long)(j) * lda] /* column-major kernels */
#define SYB_(i, j) b[(long)(i) + (long)(j) * ldb]
#define SYC_(i, j) c[(long)(i) + (long)(j) * ldc]

/* blas/syr.zig:32-225 (k_syr): A := alpha x x^T + A on the uplo triangle;
 * column j skipped when x[j] == 0; row-major inverts uplo (14-17). */
static int P(k_syr)(int uplo, int n, T alpha, const T *x, int incx, T *a, int lda) {
  if (n < 0 || lda < ZO_MAX(1, n) || incx == 0) return ZO_EINVAL;
  if (n == 0 || alpha == (T)0) return 0;
  const long kx = incx < 0 ? (long)(-n + 1) * incx : 0;
  long jx = kx;
  for (int j = 0; j < n; ++j) {
    if (x[jx] != (T)0) {
      const T temp = x[jx] * alpha;
      if (uplo == ZO_UPPER) {
        long ix = kx;
        for (int i = 0; i < j; ++i) {
          SYA_(i, j) = SYA_(i, j) + x[ix] * temp;
          ix += incx;
        }
        SYA_(j, j) = SYA_(j, j) + x[jx] * temp;
      } else {
        SYA_(j, j) = SYA_(j, j) + x[jx] * temp;
        long ix = jx;
        for (int i = j + 1; i < n; ++i) {
          ix += incx;
          SYA_(i, j) = SYA_(i, j) + x[ix] * temp;
        }
      }
    }
    jx += incx;
  }
  return 0;
}
int P(syr)(int order, int uplo, int n, T alpha, const T *x, int incx, T *a, int lda) {
  if (order == ZO_COL) return P(k_syr)(uplo, n, alpha, x, incx, a, lda);
  return P(k_syr)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, n, alpha, x, incx, a, lda);
}

/* blas/gemmtr.zig:69-1032 (k_gemmtr): the uplo triangle of
 * C := alpha op(A) op(B) + beta C (C n x n, inner dimension k), gemm's four
 * loop forms with the row range cut to the triangle; row-major inverts uplo
 * and swaps the operands (gemmtr.zig:30-64). */
static int P(k_gemmtr)(int uplo, int transa, int transb, int n, int k, T alpha, const T *a,
                       int lda, const T *b, int ldb, T beta, T *c, int ldc) {
  const int nota = transa == ZO_NOTRANS || transa == ZO_CONJNOTRANS;
  const int notb = transb == ZO_NOTRANS || transb == ZO_CONJNOTRANS;
  const int nrowa = nota ? n : k, nrowb = notb ? k : n;
  if (n < 0 || k < 0 || lda < ZO_MAX(1, nrowa) || ldb < ZO_MAX(1, nrowb) || ldc < ZO_MAX(1, n))
    return ZO_EINVAL;
  if (n == 0) return 0;
  const int up = uplo == ZO_UPPER;
  if (alpha == (T)0) { /* 110-138 */
    for (int j = 0; j < n; ++j)
      for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i)
        SYC_(i, j) = beta == (T)0 ? (T)0 : SYC_(i, j) * beta;
    return 0;
  }
  if (nota) { /* axpy forms */
    for (int j = 0; j < n; ++j) {
      const int i0 = up ? 0 : j, i1 = up ? j + 1 : n;
      if (beta == (T)0) {
        for (int i = i0; i < i1; ++i) SYC_(i, j) = 0;
      } else if (beta != (T)1) {
        for (int i = i0; i < i1; ++i) SYC_(i, j) = SYC_(i, j) * beta;
      }
      for (int l = 0; l < k; ++l) {
        const T temp = alpha * (notb ? SYB_(l, j) : SYB_(j, l));
        for (int i = i0; i < i1; ++i) SYC_(i, j) = SYC_(i, j) + temp * SYA_(i, l);
      }
    }
  } else { /* dot forms */
    for (int j = 0; j < n; ++j)
      for (int i = up ? 0 : j; i < (up ? j + 1 : n); ++i) {
        T temp = 0;
        for (int l = 0; l < k; ++l) temp = temp + SYA_(l, i) * (notb ? SYB_(l, j) : SYB_(j, l));
        if (beta == (T)0) {
          SYC_(i, j) = alpha * temp;
        } else if (beta == (T)1) {
          SYC_(i, j) = SYC_(i, j) + alpha * temp;
        } else {
          SYC_(i, j) = SYC_(i, j) * beta;
          SYC_(i, j) = SYC_(i, j) + alpha * temp;
        }
      }
  }
  return 0;
}
int P(gemmtr)(int order, int uplo, int transa, int transb, int n, int k, T alpha, const T *a,
              int lda, const T *b, int ldb, T beta, T *c, int ldc) {
  if (order == ZO_COL)
    return P(k_gemmtr)(uplo, transa, transb, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  return P(k_gemmtr)(uplo == ZO_UPPER ? ZO_LOWER : ZO_UPPER, transb, transa, n, k, alpha, b, ldb,
                     a, lda, beta, c, ldc);
}

/* lapack/sytf2.zig:17-522: unblocked Bunch-Kaufman (LAPACK dsytf2), alpha =
 * (1 + sqrt(17)) / 8; a zero (or NaN) pivot column records info and is left
 * as it is. */
int P(sytf2)(int order, int uplo, int n, T *a, int lda, int *ipiv) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  int info = 0;
  const T alpha = ((T)1 + ZO_SQRT((T)17)) / (T)8;
  const int cl = P(col_ld)(order, lda), rl = P(row_ld)(order, lda);
  if (uplo == ZO_UPPER) { /* 30-296: k from n-1 down, steps of 1 or 2 */
    int k = n - 1;
    while (k >= 0) {
      int kstep = 1, kp;
      const T absakk = ZO_ABS(SA(k, k));
      int imax = 0;
      T colmax = 0;
      if (k > 0) {
        imax = P(iamax)(k, a + P(idx)(order, 0, k, lda), cl);
        colmax = ZO_ABS(SA(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (T)0 || absakk != absakk) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          int jmax = imax + 1 + P(iamax)(k - imax, a + P(idx)(order, imax, imax + 1, lda), rl);
          T rowmax = ZO_ABS(SA(imax, jmax));
          if (imax > 0) {
            jmax = P(iamax)(imax, a + P(idx)(order, 0, imax, lda), cl);
            rowmax = ZO_MAX(rowmax, ZO_ABS(SA(jmax, imax)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(SA(imax, imax)) >= alpha * rowmax) {
            kp = imax;
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k - kstep + 1;
        if (kp != kk) {
          P(swap)(kp, a + P(idx)(order, 0, kk, lda), cl, a + P(idx)(order, 0, kp, lda), cl);
          P(swap)(kk - kp - 1, a + P(idx)(order, kp + 1, kk, lda), cl,
                  a + P(idx)(order, kp, kp + 1, lda), rl);
          T t = SA(kk, kk);
          SA(kk, kk) = SA(kp, kp);
          SA(kp, kp) = t;
          if (kstep == 2) {
            t = SA(k - 1, k);
            SA(k - 1, k) = SA(kp, k);
            SA(kp, k) = t;
          }
        }
        if (kstep == 1) {
          const T r1 = (T)1 / SA(k, k);
          P(syr)(order, uplo, k, -r1, a + P(idx)(order, 0, k, lda), cl, a, lda);
          P(scal)(k, r1, a + P(idx)(order, 0, k, lda), cl);
        } else if (k > 1) {
          T d12 = SA(k - 1, k);
          const T d22 = SA(k - 1, k - 1) / d12;
          const T d11 = SA(k, k) / d12;
          const T t = (T)1 / (d11 * d22 - (T)1);
          d12 = t / d12;
          for (int j = k - 2; j >= 0; --j) {
            const T wkm1 = d12 * (d11 * SA(j, k - 1) - SA(j, k));
            const T wk = d12 * (d22 * SA(j, k) - SA(j, k - 1));
            for (int i = j; i >= 0; --i) SA(i, j) = SA(i, j) - (SA(i, k) * wk + SA(i, k - 1) * wkm1);
            SA(j, k) = wk;
            SA(j, k - 1) = wkm1;
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
  } else { /* 297-515: k from 0 up */
    int k = 0;
    while (k < n) {
      int kstep = 1, kp;
      const T absakk = ZO_ABS(SA(k, k));
      int imax = 0;
      T colmax = 0;
      if (k < n - 1) {
        imax = k + 1 + P(iamax)(n - k - 1, a + P(idx)(order, k + 1, k, lda), cl);
        colmax = ZO_ABS(SA(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (T)0 || absakk != absakk) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          int jmax = k + P(iamax)(imax - k, a + P(idx)(order, imax, k, lda), rl);
          T rowmax = ZO_ABS(SA(imax, jmax));
          if (imax < n - 1) {
            jmax = imax + 1 + P(iamax)(n - imax - 1, a + P(idx)(order, imax + 1, imax, lda), cl);
            rowmax = ZO_MAX(rowmax, ZO_ABS(SA(jmax, imax)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(SA(imax, imax)) >= alpha * rowmax) {
            kp = imax;
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k + kstep - 1;
        if (kp != kk) {
          if (kp < n - 1)
            P(swap)(n - kp - 1, a + P(idx)(order, kp + 1, kk, lda), cl,
                    a + P(idx)(order, kp + 1, kp, lda), cl);
          P(swap)(kp - kk - 1, a + P(idx)(order, kk + 1, kk, lda), cl,
                  a + P(idx)(order, kp, kk + 1, lda), rl);
          T t = SA(kk, kk);
          SA(kk, kk) = SA(kp, kp);
          SA(kp, kp) = t;
          if (kstep == 2) {
            t = SA(k + 1, k);
            SA(k + 1, k) = SA(kp, k);
            SA(kp, k) = t;
          }
        }
        if (kstep == 1) {
          if (k < n - 1) {
            const T d11 = (T)1 / SA(k, k);
            P(syr)(order, uplo, n - k - 1, -d11, a + P(idx)(order, k + 1, k, lda), cl,
                   a + P(idx)(order, k + 1, k + 1, lda), lda);
            P(scal)(n - k - 1, d11, a + P(idx)(order, k + 1, k, lda), cl);
          }
        } else if (k < n - 2) {
          T d21 = SA(k + 1, k);
          const T d11 = SA(k + 1, k + 1) / d21;
          const T d22 = SA(k, k) / d21;
          const T t = (T)1 / (d11 * d22 - (T)1);
          d21 = t / d21;
          for (int j = k + 2; j < n; ++j) {
            const T wk = d21 * (d11 * SA(j, k) - SA(j, k + 1));
            const T wkp1 = d21 * (d22 * SA(j, k + 1) - SA(j, k));
            for (int i = j; i < n; ++i) SA(i, j) = SA(i, j) - (SA(i, k) * wk + SA(i, k + 1) * wkp1);
            SA(j, k) = wk;
            SA(j, k + 1) = wkp1;
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

/* lapack/lasyf.zig:17-896 (LAPACK dlasyf, the trailing update by gemmtr):
 * factors up to nb columns (nb - 1 when the last step takes a 2x2 block) at
 * the bottom-right (upper) or top-left (lower) of A, builds W = U12 D or
 * L21 D alongside, updates the rest of the triangle with gemmtr and puts
 * U12 / L21 in standard form by undoing the later interchanges; *kb = the
 * columns factored. */
int P(lasyf)(int order, int uplo, int n, int nb, int *kb, T *a, int lda, int *ipiv, T *w,
             int ldw) {
  int info = 0;
  const T alpha = ((T)1 + ZO_SQRT((T)17)) / (T)8;
  const int cl = P(col_ld)(order, lda), rl = P(row_ld)(order, lda);
  const int clw = P(col_ld)(order, ldw), rlw = P(row_ld)(order, ldw);
#define IA(i, j) P(idx)(order, (i), (j), lda)
#define IW(i, j) P(idx)(order, (i), (j), ldw)
  if (uplo == ZO_UPPER) { /* 39-464 */
    int k = n - 1, kw;
    while (1) {
      kw = nb + k - n;
      if ((k <= n - nb && nb < n) || k < 0) break;
      P(copy)(k + 1, a + IA(0, k), cl, w + IW(0, kw), clw);
      if (k < n - 1)
        P(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), (T)-1, a + IA(0, k + 1), lda,
                w + IW(k, kw + 1), rlw, (T)1, w + IW(0, kw), clw);
      int kstep = 1, imax = 0, kp;
      const T absakk = ZO_ABS(SW(k, kw));
      T colmax = 0;
      if (k > 0) {
        imax = P(iamax)(k, w + IW(0, kw), clw);
        colmax = ZO_ABS(SW(imax, kw));
      }
      if (ZO_MAX(absakk, colmax) == (T)0) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          P(copy)(imax + 1, a + IA(0, imax), cl, w + IW(0, kw - 1), clw);
          P(copy)(k - imax, a + IA(imax, imax + 1), rl, w + IW(imax + 1, kw - 1), clw);
          if (k < n - 1)
            P(gemv)(order, ZO_NOTRANS, k + 1, n - (k + 1), (T)-1, a + IA(0, k + 1), lda,
                    w + IW(imax, kw + 1), rlw, (T)1, w + IW(0, kw - 1), clw);
          int jmax = imax + 1 + P(iamax)(k - imax, w + IW(imax + 1, kw - 1), clw);
          T rowmax = ZO_ABS(SW(jmax, kw - 1));
          if (imax > 0) {
            jmax = P(iamax)(imax, w + IW(0, kw - 1), clw);
            rowmax = ZO_MAX(rowmax, ZO_ABS(SW(jmax, kw - 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(SW(imax, kw - 1)) >= alpha * rowmax) {
            kp = imax;
            P(copy)(k + 1, w + IW(0, kw - 1), clw, w + IW(0, kw), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k - kstep + 1, kkw = nb + kk - n;
        if (kp != kk) {
          SA(kp, kp) = SA(kk, kk);
          P(copy)(kk - kp - 1, a + IA(kp + 1, kk), cl, a + IA(kp, kp + 1), rl);
          if (kp > 0) P(copy)(kp, a + IA(0, kk), cl, a + IA(0, kp), cl);
          if (k < n - 1) P(swap)(n - (k + 1), a + IA(kk, k + 1), rl, a + IA(kp, k + 1), rl);
          P(swap)(n - kk, w + IW(kk, kkw), rlw, w + IW(kp, kkw), rlw);
        }
        if (kstep == 1) {
          P(copy)(k + 1, w + IW(0, kw), clw, a + IA(0, k), cl);
          const T r1 = (T)1 / SA(k, k);
          P(scal)(k, r1, a + IA(0, k), cl);
        } else {
          if (k > 1) {
            T d21 = SW(k - 1, kw);
            const T d11 = SW(k, kw) / d21;
            const T d22 = SW(k - 1, kw - 1) / d21;
            const T t = (T)1 / (d11 * d22 - (T)1);
            d21 = t / d21;
            for (int j = 0; j < k - 1; ++j) {
              SA(j, k - 1) = d21 * (d11 * SW(j, kw - 1) - SW(j, kw));
              SA(j, k) = d21 * (d22 * SW(j, kw) - SW(j, kw - 1));
            }
          }
          SA(k - 1, k - 1) = SW(k - 1, kw - 1);
          SA(k - 1, k) = SW(k - 1, kw);
          SA(k, k) = SW(k, kw);
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
    P(gemmtr)(order, ZO_UPPER, ZO_NOTRANS, ZO_TRANS, k + 1, n - (k + 1), (T)-1, a + IA(0, k + 1),
              lda, w + IW(0, kw + 1), ldw, (T)1, a, lda);
    int j = k + 1;
    while (j < n) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j += 1;
      }
      j += 1;
      if (jp - 1 != jj && j < n) P(swap)(n - j, a + IA(jp - 1, j), rl, a + IA(jj, j), rl);
    }
    *kb = n - k - 1;
  } else { /* 465-889 */
    int k = 0;
    while (1) {
      if ((k >= nb - 1 && nb < n) || k > n - 1) break;
      P(copy)(n - k, a + IA(k, k), cl, w + IW(k, k), clw);
      P(gemv)(order, ZO_NOTRANS, n - k, k, (T)-1, a + IA(k, 0), lda, w + IW(k, 0), rlw, (T)1,
              w + IW(k, k), clw);
      int kstep = 1, imax = 0, kp;
      const T absakk = ZO_ABS(SW(k, k));
      T colmax = 0;
      if (k < n - 1) {
        imax = k + 1 + P(iamax)(n - k - 1, w + IW(k + 1, k), clw);
        colmax = ZO_ABS(SW(imax, k));
      }
      if (ZO_MAX(absakk, colmax) == (T)0) {
        if (info == 0) info = k + 1;
        kp = k;
      } else {
        if (absakk >= alpha * colmax) {
          kp = k;
        } else {
          P(copy)(imax - k, a + IA(imax, k), rl, w + IW(k, k + 1), clw);
          P(copy)(n - imax, a + IA(imax, imax), cl, w + IW(imax, k + 1), clw);
          P(gemv)(order, ZO_NOTRANS, n - k, k, (T)-1, a + IA(k, 0), lda, w + IW(imax, 0), rlw,
                  (T)1, w + IW(k, k + 1), clw);
          int jmax = k + P(iamax)(imax - k, w + IW(k, k + 1), clw);
          T rowmax = ZO_ABS(SW(jmax, k + 1));
          if (imax < n - 1) {
            jmax = imax + 1 + P(iamax)(n - imax - 1, w + IW(imax + 1, k + 1), clw);
            rowmax = ZO_MAX(rowmax, ZO_ABS(SW(jmax, k + 1)));
          }
          if (absakk >= alpha * (colmax * (colmax / rowmax))) {
            kp = k;
          } else if (ZO_ABS(SW(imax, k + 1)) >= alpha * rowmax) {
            kp = imax;
            P(copy)(n - k, w + IW(k, k + 1), clw, w + IW(k, k), clw);
          } else {
            kp = imax;
            kstep = 2;
          }
        }
        const int kk = k + kstep - 1;
        if (kp != kk) {
          SA(kp, kp) = SA(kk, kk);
          P(copy)(kp - kk - 1, a + IA(kk + 1, kk), cl, a + IA(kp, kk + 1), rl);
          if (kp < n - 1) P(copy)(n - kp - 1, a + IA(kp + 1, kk), cl, a + IA(kp + 1, kp), cl);
          if (k > 0) P(swap)(k, a + IA(kk, 0), rl, a + IA(kp, 0), rl);
          P(swap)(kk + 1, w + IW(kk, 0), rlw, w + IW(kp, 0), rlw);
        }
        if (kstep == 1) {
          P(copy)(n - k, w + IW(k, k), clw, a + IA(k, k), cl);
          if (k < n - 1) {
            const T r1 = (T)1 / SA(k, k);
            P(scal)(n - k - 1, r1, a + IA(k + 1, k), cl);
          }
        } else {
          if (k < n - 2) {
            T d21 = SW(k + 1, k);
            const T d11 = SW(k + 1, k + 1) / d21;
            const T d22 = SW(k, k) / d21;
            const T t = (T)1 / (d11 * d22 - (T)1);
            d21 = t / d21;
            for (int j = k + 2; j < n; ++j) {
              SA(j, k) = d21 * (d11 * SW(j, k) - SW(j, k + 1));
              SA(j, k + 1) = d21 * (d22 * SW(j, k + 1) - SW(j, k));
            }
          }
          SA(k, k) = SW(k, k);
          SA(k + 1, k) = SW(k + 1, k);
          SA(k + 1, k + 1) = SW(k + 1, k + 1);
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
    P(gemmtr)(order, ZO_LOWER, ZO_NOTRANS, ZO_TRANS, n - k, k, (T)-1, a + IA(k, 0), lda,
              w + IW(k, 0), ldw, (T)1, a + IA(k, k), lda);
    int j = k - 1;
    while (j > 0) {
      const int jj = j;
      int jp = ipiv[j];
      if (jp < 0) {
        jp = -jp;
        j -= 1;
      }
      j -= 1;
      if (jp - 1 != jj && j >= 0) P(swap)(j + 1, a + IA(jp - 1, 0), rl, a + IA(jj, 0), rl);
    }
    *kb = k;
  }
#undef IA
#undef IW
  return info;
}

/* lapack/sytrf.zig:17-187 (LAPACK dsytrf): blocks of nb = ilaenv = 64 by
 * lasyf while more than nb columns remain, the rest by sytf2; work holds W
 * (n x nb column-major, nb x n row-major); lwork = -1 queries n nb. */
int P(sytrf)(int order, int uplo, int n, T *a, int lda, int *ipiv, T *work, int lwork) {
  if (n < 0 || lda < ZO_MAX(1, n) || (lwork < 1 && lwork != -1)) return ZO_EINVAL;
  int info = 0;
  int nb = zo_ilaenv(1, "DSYTRF", n, -1, -1, -1);
  const int lwkopt = ZO_MAX(1, n * nb);
  work[0] = (T)lwkopt;
  if (lwork == -1) return info;
  int nbmin = 2;
  const int ldwork = order == ZO_COL ? n : nb;
  if (nb > 1 && nb < n && lwork < ldwork * nb) {
    nb = ZO_MAX(lwork / ldwork, 1);
    nbmin = ZO_MAX(2, zo_ilaenv(2, "DSYTRF", n, -1, -1, -1));
  }
  if (nb < nbmin) nb = n;
  if (uplo == ZO_UPPER) { /* 60-110 */
    int k = n - 1;
    while (k >= 0) {
      int kb, iinfo;
      if (k + 1 > nb) {
        iinfo = P(lasyf)(order, ZO_UPPER, k + 1, nb, &kb, a, lda, ipiv, work, ldwork);
      } else {
        iinfo = P(sytf2)(order, ZO_UPPER, k + 1, a, lda, ipiv);
        kb = k + 1;
      }
      if (info == 0 && iinfo > 0) info = iinfo;
      k -= kb;
    }
  } else { /* 111-176 */
    int k = 0;
    while (k < n) {
      int kb, iinfo;
      if (k <= n - nb - 1) {
        iinfo = P(lasyf)(order, ZO_LOWER, n - k, nb, &kb, a + P(idx)(order, k, k, lda), lda,
                         ipiv + k, work, ldwork);
      } else {
        iinfo = P(sytf2)(order, ZO_LOWER, n - k, a + P(idx)(order, k, k, lda), lda, ipiv + k);
        kb = n - k;
      }
      if (info == 0 && iinfo > 0) info = iinfo + k;
      for (int j = k; j < k + kb; ++j) ipiv[j] = ipiv[j] > 0 ? ipiv[j] + k : ipiv[j] - k;
      k += kb;
    }
  }
  return info;
}

#undef SA
#undef SW
#undef SYA_
#undef SYB_
#undef SYC_
