// zblas.cu -- complex level-3 BLAS (gemm, herk, syrk; binary64 and binary32
// components) as real GEMMs on the CUDA cores.
//
// A complex product is four real products (zml's cfloat product,
// cfloat.zig:149-174), so a complex GEMM C += A B is one real GEMM of twice
// the rows and twice the depth: C viewed as a real 2m x n matrix (each
// complex row i becomes real rows 2i (re) and 2i+1 (im); this is just the
// interleaved storage read with leading dimension 2 ldc), B viewed the same
// way as a real 2k x n matrix, and A expanded into the real 2m x 2k matrix
// whose 2x2 block (i, l) is [[re, -im], [im, re]] of alpha op(A)(i, l).
// The expansion is the only extra pass (it writes 32 m k bytes); the product
// runs on the tuned FP64 / FP32 SIMT GEMM at its full rate, 8 m n k real
// flops, the 4-multiply cost of any complex GEMM.  herk and syrk form the full
// product op(A) op(A)^H (or ^T) in a scratch matrix and merge its triangle
// into C with alpha and beta.
#include "common.cuh"
#include "kernels.h"

namespace zg {

// op(A)(i, l) of an operand stored column-major, conjugated on request
template <typename C2>
__device__ __forceinline__ C2 op_at(const C2 *A, long lda, bool nota, bool cj, int i, int l) {
  C2 v = nota ? A[i + (long)l * lda] : A[l + (long)i * lda];
  if (cj) v.y = -v.y;
  return v;
}

// E (2m x 2k, column-major, leading dimension 2m) from alpha op(A), where
// op(A) is m x k: block (i, l) = [[re, -im], [im, re]] of alpha op(A)(i, l),
// the product formed as zml's cfloat product (fused).
template <typename R, typename C2>
__global__ void __launch_bounds__(256) cexpand_kernel(int m, int k, R ar, R ai, const C2 *A,
                                                      long lda, bool nota, bool cj, R *E) {
  const long total = (long)m * k, ld = 2L * m;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), l = (int)(e / m);
    const C2 v = op_at(A, lda, nota, cj, i, l);
    const R re = fma(ar, v.x, (-ai) * v.y), im = fma(ar, v.y, ai * v.x);
    R *c0 = E + (2L * l) * ld + 2L * i;
    c0[0] = re;
    c0[1] = im;
    c0[ld] = -im;
    c0[ld + 1] = re;
  }
}

// Y (k x n, leading dimension k) = op(B) of an operand stored column-major
template <typename C2>
__global__ void __launch_bounds__(256) cop_kernel(int k, int n, const C2 *B, long ldb, bool notb,
                                                  bool cj, C2 *Y) {
  const long total = (long)k * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int l = (int)(e % k), j = (int)(e / k);
    Y[e] = op_at(B, ldb, notb, cj, l, j);
  }
}

// C = beta C over an m x n block: zeros when beta == 0, so that NaNs in C do
// not survive (gemm.zig:111-140, 146-160)
template <typename R, typename C2>
__global__ void __launch_bounds__(256) cscale_kernel(int m, int n, R br, R bi, C2 *C, long ldc) {
  const long total = (long)m * n;
  const bool zero = br == R(0) && bi == R(0);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), j = (int)(e / m);
    C2 *p = C + i + (long)j * ldc;
    C2 c = *p, r;
    if (zero) {
      r.x = R(0);
      r.y = R(0);
    } else {
      r.x = fma(c.x, br, (-c.y) * bi);
      r.y = fma(c.x, bi, c.y * br);
    }
    *p = r;
  }
}

// The triangle of C (uplo) <- alpha T + beta C, T the full product or none
// (alpha == 0); herm: alpha, beta real and the diagonal keeps only its real
// part (herk.zig:121, 192-199, 229, 383-397).
template <typename R, typename C2>
__global__ void __launch_bounds__(256) ctri_merge_kernel(int n, bool lower, bool herm, R ar, R ai,
                                                         R br, R bi, const C2 *T, long ldt,
                                                         C2 *C, long ldc) {
  const long total = (long)n * n;
  const bool bzero = br == R(0) && bi == R(0), bone = br == R(1) && bi == R(0);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if (lower ? i < j : i > j) continue;
    C2 *p = C + i + (long)j * ldc;
    C2 c = *p, r;
    if (bzero) {
      r.x = R(0);
      r.y = R(0);
    } else if (bone) {
      r = c;
    } else {
      r.x = fma(c.x, br, (-c.y) * bi);
      r.y = fma(c.x, bi, c.y * br);
    }
    if (herm && i == j) {
      r.x = bzero ? R(0) : br * c.x;
      r.y = R(0);
    }
    if (T) {
      const C2 t = T[i + (long)j * ldt];
      if (herm && i == j) {
        r.x += ar * t.x;
      } else {
        r.x += fma(ar, t.x, (-ai) * t.y);
        r.y += fma(ar, t.y, ai * t.x);
      }
    }
    *p = r;
  }
}

static int grid_for(long total) {
  DeviceInfo di;
  if (device_info(&di) != 0) return 1;
  const long g = (total + 255) / 256;
  return (int)std::max(1L, std::min(g, (long)di.num_sms * 16));
}

template <typename R>
int zgemm_dev(int ta, int tb, int m, int n, int k, const R *alpha, const R *A, long lda,
              const R *B, long ldb, const R *beta, R *C, long ldc, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (m <= 0 || n <= 0) return 0;
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  const bool bone = beta[0] == R(1) && beta[1] == R(0);
  if ((azero || k == 0) && bone) return 0;
  C2 *Cc = reinterpret_cast<C2 *>(C);
  if (!bone) {
    const long tot = (long)m * n;
    ZG_LAUNCH(kTagOther, 0, 32.0 * tot, s,
              (cscale_kernel<R, C2><<<grid_for(tot), 256, 0, s>>>(m, n, beta[0], beta[1], Cc, ldc)));
  }
  if (azero || k == 0) return 0;
  const bool nota = ta == kNoTrans || ta == kConjNoTrans;
  const bool notb = tb == kNoTrans || tb == kConjNoTrans;
  const bool cja = ta == kConjNoTrans || ta == kConjTrans;
  const bool cjb = tb == kConjNoTrans || tb == kConjTrans;
  // FP64 products as exact slices on the tensor cores (as the FP64 LU's
  // updates), where they apply; they subtract, so the expansion carries -alpha
  bool slices = false;
  if constexpr (sizeof(R) == sizeof(double)) slices = fp64_updates_on_tensor_cores(2 * m, n);
  const R ar = slices ? -alpha[0] : alpha[0], ai = slices ? -alpha[1] : alpha[1];
  void *we;
  ZG_TRY(workspace(s, kSlotZExp, sizeof(R) * 4 * (size_t)m * k, &we));
  R *E = (R *)we;
  const long tot = (long)m * k;
  ZG_LAUNCH(kTagConvert, 0, 2.0 * sizeof(R) * tot + 4.0 * sizeof(R) * tot, s,
            (cexpand_kernel<R, C2><<<grid_for(tot), 256, 0, s>>>(
                m, k, ar, ai, reinterpret_cast<const C2 *>(A), lda, nota, cja, E)));
  const R *Bh = B;
  long ldbh = 2 * ldb;
  if (!(notb && !cjb)) {  // op(B) materialized, k x n
    void *wb;
    ZG_TRY(workspace(s, kSlotZOpB, sizeof(C2) * (size_t)k * n, &wb));
    const long tb2 = (long)k * n;
    ZG_LAUNCH(kTagConvert, 0, 4.0 * sizeof(R) * tb2, s,
              (cop_kernel<C2><<<grid_for(tb2), 256, 0, s>>>(
                  k, n, reinterpret_cast<const C2 *>(B), ldb, notb, cjb, (C2 *)wb)));
    Bh = (const R *)wb;
    ldbh = 2L * k;
  }
  if constexpr (sizeof(R) == sizeof(double)) {
    if (slices) {  // C (2m x n real) -= (-E) op(B), K in chunks of the slices' 256
      Control *ctl;
      ZG_TRY(control(s, &ctl));
      for (int kk = 0; kk < 2 * k; kk += 256) {
        const int kc = std::min(256, 2 * k - kk);
        ZG_TRY(dgemm_oz_sub(2 * m, n, kc, E + (long)kk * 2 * m, 2L * m, Bh + kk, ldbh, C, 2 * ldc,
                            false, &ctl->status, s));
      }
      return 0;
    }
  }
  return gemm_simt<R>(kNoTrans, kNoTrans, 2 * m, n, 2 * k, R(1), E, 2L * m, Bh, ldbh, R(1), C,
                      2 * ldc, 0, s);
}

template <typename R>
int zsyherk_dev(bool herm, int uplo, int trans, int n, int k, const R *alpha, const R *A, long lda,
                const R *beta, R *C, long ldc, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  if (n <= 0) return 0;
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  const bool bone = beta[0] == R(1) && beta[1] == R(0);
  if ((azero || k == 0) && bone) return 0;
  C2 *T = nullptr;
  if (!azero && k > 0) {
    // T = op(A) op(A)^H (herk) or op(A) op(A)^T (syrk), n x n
    void *wt;
    ZG_TRY(workspace(s, kSlotZTmp, sizeof(C2) * (size_t)n * n, &wt));
    T = (C2 *)wt;
    const R one[2] = {R(1), R(0)}, zero[2] = {R(0), R(0)};
    int ta, tb;
    if (trans == kNoTrans) {
      ta = kNoTrans;
      tb = herm ? kConjTrans : kTrans;
    } else {
      ta = herm ? kConjTrans : kTrans;
      tb = kNoTrans;
    }
    ZG_TRY(zgemm_dev<R>(ta, tb, n, n, k, one, A, lda, A, lda, zero, (R *)T, n, s));
  }
  const long tot = (long)n * n;
  ZG_LAUNCH(kTagOther, 0, 48.0 * tot, s,
            (ctri_merge_kernel<R, C2><<<grid_for(tot), 256, 0, s>>>(
                n, uplo == kLower, herm, alpha[0], herm ? R(0) : alpha[1], beta[0],
                herm ? R(0) : beta[1], T, n, reinterpret_cast<C2 *>(C), ldc)));
  return 0;
}

template int zgemm_dev<double>(int, int, int, int, int, const double *, const double *, long,
                               const double *, long, const double *, double *, long, cudaStream_t);
template int zgemm_dev<float>(int, int, int, int, int, const float *, const float *, long,
                              const float *, long, const float *, float *, long, cudaStream_t);
template int zsyherk_dev<double>(bool, int, int, int, int, const double *, const double *, long,
                                 const double *, double *, long, cudaStream_t);
template int zsyherk_dev<float>(bool, int, int, int, int, const float *, const float *, long,
                                const float *, float *, long, cudaStream_t);

}  // namespace zg
