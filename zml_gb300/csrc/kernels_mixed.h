// kernels_mixed.h -- mixed-precision factorization and iterative refinement.
#pragma once
#include "common.cuh"

namespace zg {

// kPrecBF16x3: each 16-bit operand split hi + lo, three BF16 products
// (hi*hi + hi*lo + lo*hi) accumulated in FP32 -- about 16 significant bits.
enum : int { kPrecFP16 = 0, kPrecBF16 = 1, kPrecFP32 = 2, kPrecBF16x3 = 3 };
enum : int { kModeIR = 0, kModeGMRES = 1 };
// Arithmetic of the preconditioner / correction solves with the FP32 factors.
enum : int { kApplyAuto = 0, kApplyF32 = 1, kApplyF64 = 2 };

struct MpirOpts {
  int prec = kPrecBF16;     // factor precision of the trailing updates
  int mode = kModeGMRES;    // refinement
  double tol = 0;           // stop when berr <= tol; 0 = iterate to stagnation
  int max_iter = 30;        // outer refinement steps
  int gmres_restart = 50;   // inner GMRES iterations per outer step
  // inner relative tolerance (preconditioned residual).  An outer step gains
  // about 1e4 at most with FP32-applied factors, so asking GMRES for 1e-4
  // instead of 1e-6 saves inner iterations without adding outer steps
  // (n = 16384 Gaussian: 3 outer / 15 inner steps instead of 3 / 20).
  double gmres_rtol = 1e-4;
  int apply = kApplyAuto;   // FP32 first, FP64 once refinement stops improving
  // when the low-precision factorization fails or refinement stops short of
  // the target, solve again with the plain FP64 factorization of A
  bool fallback = false;
};

struct MpirResult {
  int info = 0;             // info of the factorization whose solution is returned
  int iters = 0;            // outer refinement steps taken
  int inner_iters = 0;      // total GMRES iterations
  int converged = 0;        // berr reached FP64 level (or tol)
  int switched_f64 = 0;     // the solves moved to FP64 arithmetic
  int fp64_fallback = 0;    // the solution came from the FP64 factorization
  double berr = 0;          // final normwise backward error
  double factor_ms = 0;     // device time of the factorization
  double berr_history[32] = {0};
};

int getrf_lowp(int n, float *A, long lda, int *ipiv, int prec, Control *ctl, cudaStream_t s);
// Panels of getrf_lowp: tournament pivoting (on != 0) or partial (the default)
// pivoting; returns the previous setting.
int set_mixed_tournament(int on);
// Solves A X = B (device pointers, column-major) to FP64 accuracy: one
// low-precision factorization, then refinement of each right-hand side.
int gesv_mpir_dev(int n, int nrhs, const double *A, long lda, const double *B, long ldb,
                  double *X, long ldx, const MpirOpts &o, MpirResult *res, cudaStream_t s);
// The same solve with A in pinned host memory (column-major, ld ldh): A is
// copied into Ad (device, n x n, ld n) in column chunks while the
// factorization already runs on the chunks that have arrived; the factors
// and the solution equal gesv_mpir_dev's on the same A.  Only where
// mixed_streams_host(n, o) holds: n >= kChunkMinN and BF16x3 updates.
constexpr int kChunkMinN = 4096;
bool mixed_streams_host(int n, const MpirOpts &o);
int gesv_mpir_host(int n, int nrhs, const double *Ah, long ldh, double *Ad, const double *B,
                   long ldb, double *X, long ldx, const MpirOpts &o, MpirResult *res,
                   cudaStream_t s);
// SPD form: low-precision Cholesky (only the `lower` / upper triangle of A is
// read) and the same refinement.
int posv_mpir_dev(bool lower, int n, int nrhs, const double *A, long lda, const double *B,
                  long ldb, double *X, long ldx, const MpirOpts &o, MpirResult *res,
                  cudaStream_t s);
int potrf_lowp(int n, float *A, long lda, int prec, Control *ctl, cudaStream_t s);

// ---- precision selection -------------------------------------------------
// Classes of the precision ladder, cheapest first; the last is the plain FP64
// LU.  kClassPrec maps a refined class to its factor precision.
enum : int { kClassBF16 = 0, kClassFP16 = 1, kClassBF16x3 = 2, kClassFP32 = 3, kClassFP64 = 4,
             kNumClasses = 5 };
constexpr int kClassPrec[4] = {kPrecBF16, kPrecFP16, kPrecBF16x3, kPrecFP32};
constexpr int kSelFeatures = 16;

struct AutoResult {
  int info = 0;        // info of the returned attempt (FP64 getrf info for class 4)
  int predicted = -1;  // class the network chose (-1: none consulted)
  int used = -1;       // class of the returned solution
  int attempts = 0;    // factorizations performed, the probe included
  int converged = 0;   // backward error of every column <= 64 u
  int iters = 0;       // refinement steps of the returned attempt
  double berr = 0;     // its normwise backward error (max over columns)
  double ms = 0;       // wall time of the call
  float features[kSelFeatures] = {0};
  float proba[kNumClasses] = {0};
  int reserved = 0;
};

// A X = B (general A) to FP64 backward error by the ladder BF16 -> FP16 ->
// BF16x3 -> FP32 (GMRES-IR, at most max_iter steps each) -> FP64 LU.  The
// first attempt (BF16 factors) doubles as the probe: its first two
// refinement steps give features 12..15, and it continues from there when it
// is the class to try.  model (host, may be null): the selector network,
// mlp parameters followed by the 16 feature means and 16 scales; with it the
// ladder starts at the smallest class whose cumulative predicted probability
// reaches `confidence`; without it the ladder is walked from the bottom.
int gesv_auto_dev(int n, int nrhs, const double *A, long lda, const double *B, long ldb, double *X,
                  long ldx, const float *model, float confidence, int max_iter, AutoResult *r,
                  cudaStream_t s);
// Features 12..15 from the probe's refinement record and the condition
// estimate of its factors (0 when they failed).
void probe_features(const MpirResult &pr, double kappa, float *f);
// Steps of inverse iteration behind the probe's condition estimate.
constexpr int kCondSteps = 3;

}  // namespace zg
