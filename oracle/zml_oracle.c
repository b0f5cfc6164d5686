/*
 * zml_oracle.c -- instantiates the type-generic oracle for binary64 and
 * binary32, real (oracle_impl.h, oracle_qr_impl.h, oracle_sy_impl.h) and complex
 * (oracle_z_impl.h) (TEST INFRASTRUCTURE; see zml_oracle.h).
 *
 * Build with -O2 -ffp-contract=off: Zig does not contract a*b+c into an FMA,
 * and gcc does so by default on aarch64.
 */
#include "zml_oracle.h"

#include <float.h>
#include <math.h>
#include <string.h>

#define ZO_ROW 101
#define ZO_COL 102
#define ZO_NOTRANS 111
#define ZO_TRANS 112
#define ZO_CONJTRANS 113
#define ZO_CONJNOTRANS 114
#define ZO_UPPER 121
#define ZO_LOWER 122
#define ZO_NONUNIT 131
#define ZO_UNIT 132
#define ZO_LEFT 141
#define ZO_RIGHT 142
#define ZO_MAX(a, b) ((a) > (b) ? (a) : (b))
#define ZO_MIN(a, b) ((a) < (b) ? (a) : (b))

static int zo_trsm_as_written = 1;
void zo_set_trsm_as_written(int on) { zo_trsm_as_written = on ? 1 : 0; }

/* linalg.zig:113-120 (Transpose.invert) */
static int zo_trans_invert(int t) {
  switch (t) {
    case ZO_NOTRANS: return ZO_TRANS;
    case ZO_TRANS: return ZO_NOTRANS;
    case ZO_CONJNOTRANS: return ZO_CONJTRANS;
    default: return ZO_CONJNOTRANS;
  }
}

/* lapack/ilaenv.zig:9-745, the entries this path reads: NB (ispec 1) = 64
 * for xGETRF, xPOTRF and xSYTRF, 32 for xGEQRF; NBMIN (ispec 2) = 8 for
 * xSYTRF, else 2; NX (ispec 3) = 128 for xGEQRF. */
int zo_ilaenv(int ispec, const char *name, int n1, int n2, int n3, int n4) {
  (void)n1; (void)n2; (void)n3; (void)n4;
  const char *c2 = name + 1, *c3 = name + 3;
  if (ispec == 1) {
    if (!strncmp(c2, "GE", 2) && !strncmp(c3, "TRF", 3)) return 64;
    if (!strncmp(c2, "PO", 2) && !strncmp(c3, "TRF", 3)) return 64;
    if (!strncmp(c2, "GE", 2) && !strncmp(c3, "QRF", 3)) return 32;
    if (!strncmp(c2, "OR", 2) && !strncmp(c3, "GQR", 3)) return 32;
    if (!strncmp(c2, "SY", 2) && !strncmp(c3, "TRF", 3)) return 64;
    if (!strncmp(c2, "HE", 2) && !strncmp(c3, "TRF", 3)) return 64; /* ilaenv.zig:255-261 */
    return 1;
  }
  if (ispec == 2) {
    if (!strncmp(c2, "SY", 2) && !strncmp(c3, "TRF", 3)) return 8; /* ilaenv.zig:406-412 */
    return 2;
  }
  if (ispec == 3) {
    if (!strncmp(c2, "GE", 2) && !strncmp(c3, "QRF", 3)) return 128;
    if (!strncmp(c2, "OR", 2) && !strncmp(c3, "GQR", 3)) return 128;
    return 0;
  }
  return -1;
}

/* ---- binary64 ---- */
#define T double
#define P(x) zo_d_##x
#define ZO_ABS fabs
#define ZO_SQRT sqrt
#define ZO_EPS DBL_EPSILON
#define ZO_TMIN DBL_MIN
#define ZO_TMAX DBL_MAX
#define ZO_COPYSIGN copysign
#define ZO_EMIN (-1022)
#define ZO_EMAX 1023
#define ZO_BITS 64
#include "oracle_impl.h"
#include "oracle_qr_impl.h"
#include "oracle_sy_impl.h"
#include "oracle_mt.h"
#undef T
#undef P
#undef ZO_ABS
#undef ZO_SQRT
#undef ZO_EPS
#undef ZO_TMIN
#undef ZO_TMAX
#undef ZO_COPYSIGN
#undef ZO_EMIN
#undef ZO_EMAX
#undef ZO_BITS

/* ---- binary32 ---- */
#define T float
#define P(x) zo_s_##x
#define ZO_ABS fabsf
#define ZO_SQRT sqrtf
#define ZO_EPS FLT_EPSILON
#define ZO_TMIN FLT_MIN
#define ZO_TMAX FLT_MAX
#define ZO_COPYSIGN copysignf
#define ZO_EMIN (-126)
#define ZO_EMAX 127
#define ZO_BITS 32
#include "oracle_impl.h"
#include "oracle_qr_impl.h"
#include "oracle_sy_impl.h"
#undef T
#undef P

#undef ZO_ABS
#undef ZO_SQRT
#undef ZO_EPS
#undef ZO_TMIN
#undef ZO_TMAX
#undef ZO_COPYSIGN
#undef ZO_EMIN
#undef ZO_EMAX
#undef ZO_BITS

/* ---- complex ------------------------------------------------------------- */
static int zo_cdiv_as_written = 0;
void zo_set_cdiv_as_written(int on) { zo_cdiv_as_written = on ? 1 : 0; }

/* linalg/utils.zig:4-6 */
static inline long zo_index(int order, int i, int j, int ld) {
  return order == ZO_COL ? (long)i + (long)j * ld : (long)i * ld + j;
}

#define R double
#define ZT zo_cf64
#define ZP(x) zo_z_##x
#define ZFMA fma
#define ZO_ABS fabs
#define ZO_SQRT sqrt
#define ZLAPY3 zo_d_lapy3
#define ZLAMCH zo_d_lamch
#define ZCOPYSIGN copysign
#define ZR_TMAX DBL_MAX
#define ZR_EMIN (-1022)
#define ZR_EMAX 1023
#define ZR_BITS 64
static inline double zo_z_lamch_s(void) { return zo_d_lamch('s'); }
#include "oracle_z_impl.h"
#undef R
#undef ZT
#undef ZP
#undef ZFMA
#undef ZO_ABS
#undef ZO_SQRT
#undef ZLAPY3
#undef ZLAMCH
#undef ZCOPYSIGN
#undef ZR_TMAX
#undef ZR_EMIN
#undef ZR_EMAX
#undef ZR_BITS

#define R float
#define ZT zo_cf32
#define ZP(x) zo_c_##x
#define ZFMA fmaf
#define ZO_ABS fabsf
#define ZO_SQRT sqrtf
#define ZLAPY3 zo_s_lapy3
#define ZLAMCH zo_s_lamch
#define ZCOPYSIGN copysignf
#define ZR_TMAX FLT_MAX
#define ZR_EMIN (-126)
#define ZR_EMAX 127
#define ZR_BITS 32
static inline float zo_c_lamch_s(void) { return zo_s_lamch('s'); }
#include "oracle_z_impl.h"
#undef R
#undef ZT
#undef ZP
#undef ZFMA
#undef ZO_ABS
#undef ZO_SQRT
#undef ZLAPY3
#undef ZLAMCH
#undef ZCOPYSIGN
#undef ZR_TMAX
#undef ZR_EMIN
#undef ZR_EMAX
#undef ZR_BITS

/* ---- seeded inputs ------------------------------------------------------ */
static unsigned long long zo_splitmix(unsigned long long *s) {
  unsigned long long z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double zo_u01(unsigned long long *s) { /* (0,1], 53 random bits */
  return ((double)(zo_splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}
void zo_fill_uniform(double *x, long long count, unsigned long long seed, double lo, double hi) {
  unsigned long long s = seed;
  for (long long i = 0; i < count; ++i) x[i] = lo + (hi - lo) * zo_u01(&s);
}
void zo_fill_normal(double *x, long long count, unsigned long long seed) {
  unsigned long long s = seed;
  const double two_pi = 6.283185307179586476925286766559;
  for (long long i = 0; i < count; i += 2) {
    double u1 = zo_u01(&s), u2 = zo_u01(&s);
    double r = sqrt(-2.0 * log(u1));
    x[i] = r * cos(two_pi * u2);
    if (i + 1 < count) x[i + 1] = r * sin(two_pi * u2);
  }
}
