/* oracle_mt.h -- threaded drivers of the oracle's blocked getrf and potrf
 * (test infrastructure, binary64, column-major).
 *
 * The parity tests at the workload's sizes (n = 8192) need the oracle's
 * factors of the full matrix, which one scalar thread takes minutes to form.
 * These drivers run the same blocked loops as P(getrf) (lapack/getrf.zig:52-136)
 * and P(potrf) (lapack/potrf.zig:52-231) and call the same restated kernels;
 * they only split, over host threads, loops whose iterations the serial
 * restatement already computes independently:
 *   - the trailing gemm (NN, getrf.zig:125; NC / CN, potrf.zig:197 / :110):
 *     gemm.zig's loop nests compute every column of C on its own;
 *   - the left-side trsm of getrf.zig:107 and potrf.zig:127: trsm.zig's
 *     left-side branches solve every column of B on its own;
 *   - the right-side trsm of potrf.zig:215: every row of B on its own.
 * The panel (getrf2), the interchanges (laswp), syrk and potrf2 stay serial.
 * The results therefore equal P(getrf) / P(potrf) bit for bit.
 *
 * Included by zml_oracle.c inside its binary64 instantiation (T = double,
 * P(x) = zo_d_##x). */
#include <pthread.h>

typedef struct {
  void (*fn)(void *ctx, int lo, int hi);
  void *ctx;
  int lo, hi;
} zo_job;

static void *zo_job_run(void *p) {
  zo_job *j = (zo_job *)p;
  j->fn(j->ctx, j->lo, j->hi);
  return 0;
}

/* fn(ctx, lo, hi) over [0, count) in contiguous chunks, one per thread; the
 * calling thread runs the first chunk. */
static void zo_parallel(int count, int threads, void (*fn)(void *, int, int), void *ctx) {
  enum { kMax = 128 };
  if (count <= 0) return;
  if (threads < 1) threads = 1;
  if (threads > kMax) threads = kMax;
  if (threads > count) threads = count;
  const int chunk = (count + threads - 1) / threads;
  zo_job jobs[kMax];
  pthread_t th[kMax];
  int nj = 0;
  for (int lo = 0; lo < count; lo += chunk) {
    jobs[nj].fn = fn;
    jobs[nj].ctx = ctx;
    jobs[nj].lo = lo;
    jobs[nj].hi = ZO_MIN(count, lo + chunk);
    ++nj;
  }
  int started[kMax] = {0};
  for (int t = 1; t < nj; ++t) started[t] = pthread_create(&th[t], 0, zo_job_run, &jobs[t]) == 0;
  zo_job_run(&jobs[0]);
  for (int t = 1; t < nj; ++t) {
    if (started[t]) pthread_join(th[t], 0);
    else zo_job_run(&jobs[t]); /* no thread: run the chunk here */
  }
}

typedef struct {
  int ta, tb, m, k, side, uplo, trans, diag, n;
  const double *a;
  int lda;
  double *b;
  int ldb;
  double *c;
  int ldc;
  int by_row; /* trsm: split the rows of B (right side) instead of its columns */
} zo_mt_ctx;

/* C(:, lo:hi) -= op(A) op(B)(:, lo:hi)   (alpha = -1, beta = 1) */
static void zo_mt_gemm_cols(void *p, int lo, int hi) {
  const zo_mt_ctx *c = (const zo_mt_ctx *)p;
  /* op(B)(:, lo:hi): columns lo..hi of B for NN, its rows lo..hi for B^T */
  const double *b = c->tb == ZO_NOTRANS ? c->b + (long)lo * c->ldb : c->b + lo;
  P(gemm)(ZO_COL, c->ta, c->tb, c->m, hi - lo, c->k, -1.0, c->a, c->lda, b, c->ldb, 1.0,
          c->c + (long)lo * c->ldc, c->ldc);
}

static void zo_mt_trsm(void *p, int lo, int hi) {
  const zo_mt_ctx *c = (const zo_mt_ctx *)p;
  if (c->by_row)
    P(trsm)(ZO_COL, c->side, c->uplo, c->trans, c->diag, hi - lo, c->n, 1.0, c->a, c->lda,
            c->b + lo, c->ldb);
  else
    P(trsm)(ZO_COL, c->side, c->uplo, c->trans, c->diag, c->m, hi - lo, 1.0, c->a, c->lda,
            c->b + (long)lo * c->ldb, c->ldb);
}

/* P(getrf)'s result (column-major) on `threads` host threads.  margin
 * (optional, min(m, n) entries): each column's pivot gap, as recorded by
 * getrf2's one-column step. */
int P(getrf_mt)(int m, int n, double *a, int lda, int *ipiv, double *margin, int threads) {
  if (m < 0 || n < 0 || lda < ZO_MAX(1, m)) return ZO_EINVAL;
  int info = 0;
  if (m == 0 || n == 0) return info;
  const int nb = zo_ilaenv(1, "DGETRF", m, n, -1, -1);
  const int mn = ZO_MIN(m, n);
  P(margin_out) = margin;
  P(margin_ipiv) = ipiv;
  if (nb <= 1 || nb >= mn) {
    info = P(getrf2)(ZO_COL, m, n, a, lda, ipiv);
    P(margin_out) = 0;
    return info;
  }
  for (int j = 0; j < mn; j += nb) {
    const int jb = ZO_MIN(mn - j, nb);
    const int iinfo = P(getrf2)(ZO_COL, m - j, jb, a + j + (long)j * lda, lda, ipiv + j);
    if (info == 0 && iinfo > 0) info = iinfo + j;
    for (int i = j; i < ZO_MIN(m, j + jb); ++i) ipiv[i] = ipiv[i] + j;
    P(laswp)(ZO_COL, j, a, lda, j + 1, j + jb, ipiv, 1);
    if (j + jb < n) {
      const int nr = n - j - jb;
      P(laswp)(ZO_COL, nr, a + (long)(j + jb) * lda, lda, j + 1, j + jb, ipiv, 1);
      zo_mt_ctx t = {0};
      t.side = ZO_LEFT, t.uplo = ZO_LOWER, t.trans = ZO_NOTRANS, t.diag = ZO_UNIT;
      t.m = jb, t.a = a + j + (long)j * lda, t.lda = lda;
      t.b = a + j + (long)(j + jb) * lda, t.ldb = lda;
      zo_parallel(nr, threads, zo_mt_trsm, &t);
      if (j + jb < m) {
        zo_mt_ctx g = {0};
        g.ta = ZO_NOTRANS, g.tb = ZO_NOTRANS, g.m = m - j - jb, g.k = jb;
        g.a = a + (j + jb) + (long)j * lda, g.lda = lda;
        g.b = a + j + (long)(j + jb) * lda, g.ldb = lda;
        g.c = a + (j + jb) + (long)(j + jb) * lda, g.ldc = lda;
        zo_parallel(nr, threads, zo_mt_gemm_cols, &g);
      }
    }
  }
  P(margin_out) = 0;
  return info;
}

/* P(potrf)'s result (column-major) on `threads` host threads. */
int P(potrf_mt)(int uplo, int n, double *a, int lda, int threads) {
  if (n < 0 || lda < ZO_MAX(1, n)) return ZO_EINVAL;
  if (n == 0) return 0;
  const int nb = zo_ilaenv(1, "DPOTRF", n, -1, -1, -1);
  if (nb <= 1 || nb >= n) return P(potrf2)(ZO_COL, uplo, n, a, lda);
  int info = 0;
  for (int j = 0; j < n; j += nb) {
    const int jb = ZO_MIN(nb, n - j), nr = n - j - jb;
    if (uplo == ZO_UPPER) { /* potrf.zig:52-141 */
      P(syrk)(ZO_COL, ZO_UPPER, ZO_TRANS, jb, j, -1.0, a + (long)j * lda, lda, 1.0,
              a + j + (long)j * lda, lda);
      info = P(potrf2)(ZO_COL, ZO_UPPER, jb, a + j + (long)j * lda, lda);
      if (info != 0) return info + j;
      if (nr > 0) {
        zo_mt_ctx g = {0};
        g.ta = ZO_CONJTRANS, g.tb = ZO_NOTRANS, g.m = jb, g.k = j;
        g.a = a + (long)j * lda, g.lda = lda;
        g.b = a + (long)(j + jb) * lda, g.ldb = lda;
        g.c = a + j + (long)(j + jb) * lda, g.ldc = lda;
        zo_parallel(nr, threads, zo_mt_gemm_cols, &g);
        zo_mt_ctx t = {0};
        t.side = ZO_LEFT, t.uplo = ZO_UPPER, t.trans = ZO_CONJTRANS, t.diag = ZO_NONUNIT;
        t.m = jb, t.a = a + j + (long)j * lda, t.lda = lda;
        t.b = a + j + (long)(j + jb) * lda, t.ldb = lda;
        zo_parallel(nr, threads, zo_mt_trsm, &t);
      }
    } else { /* potrf.zig:144-231 */
      P(syrk)(ZO_COL, ZO_LOWER, ZO_NOTRANS, jb, j, -1.0, a + j, lda, 1.0, a + j + (long)j * lda,
              lda);
      info = P(potrf2)(ZO_COL, ZO_LOWER, jb, a + j + (long)j * lda, lda);
      if (info != 0) return info + j;
      if (nr > 0) {
        zo_mt_ctx g = {0};
        g.ta = ZO_NOTRANS, g.tb = ZO_CONJTRANS, g.m = nr, g.k = j;
        g.a = a + (j + jb), g.lda = lda;
        g.b = a + j, g.ldb = lda;
        g.c = a + (j + jb) + (long)j * lda, g.ldc = lda;
        zo_parallel(jb, threads, zo_mt_gemm_cols, &g);
        zo_mt_ctx t = {0};
        t.side = ZO_RIGHT, t.uplo = ZO_LOWER, t.trans = ZO_CONJTRANS, t.diag = ZO_NONUNIT;
        t.n = jb, t.a = a + j + (long)j * lda, t.lda = lda;
        t.b = a + (j + jb) + (long)j * lda, t.ldb = lda, t.by_row = 1;
        zo_parallel(nr, threads, zo_mt_trsm, &t);
      }
    }
  }
  return info;
}
