// capi.cu -- the C ABI of libzml_gb300 (include/cblas.h, include/clapack.h).
//
// cblas_* keep the reference prototypes (reference include/cblas.h:216-253,
// implemented in src/cblas.zig:523-638) and its behaviour: row-major calls
// are mapped to column-major by the index swaps of blas/gemm.zig:48-65,
// trsm.zig:48-63 and syrk.zig:28-57; invalid arguments return silently
// (cblas.zig forwards to zml.linalg.blas.d*, which swallows the error).
//
// LAPACKE_* take the LAPACKE signatures the reference itself calls when
// linked against a system LAPACKE (lapack.zig:1169, 1575, 2103, 3012, 3466,
// 3948, 5121) and return LAPACKE's info: 0, -(index of the bad argument), or
// a positive numerical info.  Row-major matrices are transposed on the
// device, factored column-major and transposed back (the logical matrix is
// the same one zml factors with its row-major indexing).
//
// Every pointer may be host memory (staged through device workspaces) or
// device / managed memory (used in place).  Calls are synchronous.
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "kernels_batched.h"
#include "kernels_mixed.h"
#include "kernels_selector.h"
#include "kernels_tc.h"

using namespace zg;

namespace {

// The stream of the synchronous entries.  A blocking stream: its work starts
// after everything already queued on the legacy default stream (where
// PyTorch and most CUDA callers fill device buffers), so an operand passed
// as a device pointer is never read while the caller's copy into it is still
// running.
cudaStream_t lib_stream() {
  static thread_local cudaStream_t s = nullptr;
  static thread_local int dev = -1;
  int d = 0;
  cudaGetDevice(&d);
  if (!s || d != dev) {
    cudaStreamCreateWithFlags(&s, cudaStreamDefault);
    dev = d;
  }
  return s;
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): copies from it
// are asynchronous, so they can run beside kernels.
bool is_pinned_host(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// A column-major rows x cols operand that lives on the device for the call.
template <typename T> struct Staged {
  T *d = nullptr;
  long ld = 0;
  const T *host = nullptr;
  long host_ld = 0;
  int rows = 0, cols = 0;
  bool staged = false;

  int in(const T *p, long ldp, int r, int c, int slot, bool copy, cudaStream_t s) {
    rows = r; cols = c; host = p; host_ld = ldp;
    if (r <= 0 || c <= 0) return 0;
    if (is_device_ptr(p)) {
      d = const_cast<T *>(p);
      ld = ldp;
      return 0;
    }
    void *w;
    ZG_TRY(workspace(s, slot, sizeof(T) * (size_t)r * c, &w));
    d = (T *)w;
    ld = r;
    staged = true;
    if (copy)
      ZG_CUDA(cudaMemcpy2DAsync(d, sizeof(T) * r, p, sizeof(T) * ldp, sizeof(T) * r, c,
                                cudaMemcpyHostToDevice, s));
    return 0;
  }
  int out(cudaStream_t s) {
    if (staged && rows > 0 && cols > 0)
      ZG_CUDA(cudaMemcpy2DAsync(const_cast<T *>(host), sizeof(T) * host_ld, d, sizeof(T) * ld,
                                sizeof(T) * rows, cols, cudaMemcpyDeviceToHost, s));
    return 0;
  }
};

template <typename T> struct Buf {  // small host-or-device vector
  T *d = nullptr;
  T *host = nullptr;
  long n = 0;
  bool staged = false;
  int in(T *p, long cnt, int slot, bool copy, cudaStream_t s) {
    host = p; n = cnt;
    if (cnt <= 0) return 0;
    if (is_device_ptr(p)) { d = p; return 0; }
    void *w;
    ZG_TRY(workspace(s, slot, sizeof(T) * cnt, &w));
    d = (T *)w;
    staged = true;
    if (copy) ZG_CUDA(cudaMemcpyAsync(d, p, sizeof(T) * cnt, cudaMemcpyHostToDevice, s));
    return 0;
  }
  int out(cudaStream_t s) {
    if (staged && n > 0) ZG_CUDA(cudaMemcpyAsync(host, d, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
    return 0;
  }
};

int sync(cudaStream_t s) {
  ZG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

bool is_trans(int t) { return t == kNoTrans || t == kTrans || t == kConjTrans || t == kConjNoTrans; }
int trans_invert(int t) {
  switch (t) {
    case kNoTrans: return kTrans;
    case kTrans: return kNoTrans;
    case kConjNoTrans: return kConjTrans;
    default: return kConjNoTrans;
  }
}

// ---- BLAS level 3 ----------------------------------------------------------

template <typename T>
int gemm_any(int order, int ta, int tb, int m, int n, int k, T alpha, const T *a, int lda,
             const T *b, int ldb, T beta, T *c, int ldc) {
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if (!is_trans(ta) || !is_trans(tb)) return kErrInvalid;
  if (order == kRowMajor) {  // gemm.zig:48-65
    std::swap(ta, tb); std::swap(m, n); std::swap(a, b); std::swap(lda, ldb);
  }
  const bool nota = ta == kNoTrans || ta == kConjNoTrans;
  const bool notb = tb == kNoTrans || tb == kConjNoTrans;
  const int nrowa = nota ? m : k, ncola = nota ? k : m;
  const int nrowb = notb ? k : n, ncolb = notb ? n : k;
  if (m < 0 || n < 0 || k < 0 || lda < std::max(1, nrowa) || ldb < std::max(1, nrowb) ||
      ldc < std::max(1, m))
    return kErrInvalid;  // gemm.zig:101-102
  if (m == 0 || n == 0 || ((alpha == T(0) || k == 0) && beta == T(1))) return 0;
  cudaStream_t s = lib_stream();
  Staged<T> A, B, C;
  const bool use_ab = alpha != T(0) && k > 0;
  if (use_ab) {
    ZG_TRY(A.in(a, lda, nrowa, ncola, kSlotA, true, s));
    ZG_TRY(B.in(b, ldb, nrowb, ncolb, kSlotB, true, s));
  }
  ZG_TRY(C.in(c, ldc, m, n, kSlotC, beta != T(0), s));
  ZG_TRY(gemm_simt<T>(ta, tb, m, n, use_ab ? k : 0, alpha, A.d, A.ld ? A.ld : 1, B.d,
                      B.ld ? B.ld : 1, beta, C.d, C.ld, 0, s));
  ZG_TRY(C.out(s));
  return sync(s);
}

// Complex gemm (cblas_zgemm / cblas_cgemm, reference include/cblas.h:218-219;
// the checks and the row-major swap of blas/gemm.zig:14-66, 101-108).
// Scalars are {re, im} pairs of R, matrices interleaved pairs.
template <typename R>
int zgemm_any(int order, int ta, int tb, int m, int n, int k, const R *alpha, const R *a, int lda,
              const R *b, int ldb, const R *beta, R *c, int ldc) {
  using C2 = typename std::conditional<sizeof(R) == 8, double2, float2>::type;
  if (!alpha || !beta) return kErrInvalid;
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if (!is_trans(ta) || !is_trans(tb)) return kErrInvalid;
  if (order == kRowMajor) {
    std::swap(ta, tb); std::swap(m, n); std::swap(a, b); std::swap(lda, ldb);
  }
  const bool nota = ta == kNoTrans || ta == kConjNoTrans;
  const bool notb = tb == kNoTrans || tb == kConjNoTrans;
  const int nrowa = nota ? m : k, ncola = nota ? k : m;
  const int nrowb = notb ? k : n, ncolb = notb ? n : k;
  if (m < 0 || n < 0 || k < 0 || lda < std::max(1, nrowa) || ldb < std::max(1, nrowb) ||
      ldc < std::max(1, m))
    return kErrInvalid;
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  const bool bone = beta[0] == R(1) && beta[1] == R(0);
  if (m == 0 || n == 0 || ((azero || k == 0) && bone)) return 0;
  cudaStream_t s = lib_stream();
  Staged<C2> A, B, C;
  const bool use_ab = !azero && k > 0;
  if (use_ab) {
    ZG_TRY(A.in((const C2 *)a, lda, nrowa, ncola, kSlotA, true, s));
    ZG_TRY(B.in((const C2 *)b, ldb, nrowb, ncolb, kSlotB, true, s));
  }
  const bool bzero = beta[0] == R(0) && beta[1] == R(0);
  ZG_TRY(C.in((const C2 *)c, ldc, m, n, kSlotC, !bzero, s));
  ZG_TRY(zgemm_dev<R>(ta, tb, m, n, use_ab ? k : 0, alpha, (const R *)A.d, A.ld ? A.ld : 1,
                      (const R *)B.d, B.ld ? B.ld : 1, beta, (R *)C.d, C.ld, s));
  ZG_TRY(C.out(s));
  return sync(s);
}

// Complex herk (herm) and syrk (cblas_zherk / cblas_zsyrk and the c forms,
// reference include/cblas.h:224-225, 237-238): row-major inverts uplo and
// reverses (herk, herk.zig:14-58) or inverts (syrk, syrk.zig:15-58) the
// transpose; herk accepts no_trans / conj_trans, syrk no_trans / trans.
template <typename R>
int zsyherk_any(bool herm, int order, int uplo, int trans, int n, int k, const R *alpha,
                const R *a, int lda, const R *beta, R *c, int ldc) {
  using C2 = typename std::conditional<sizeof(R) == 8, double2, float2>::type;
  if (!alpha || !beta) return kErrInvalid;
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if (uplo != kUpper && uplo != kLower) return kErrInvalid;
  if (!is_trans(trans)) return kErrInvalid;
  if (order == kRowMajor) {
    uplo = uplo == kUpper ? kLower : kUpper;
    if (herm)
      trans = trans == kNoTrans ? kConjTrans
            : trans == kConjTrans ? kNoTrans
            : trans == kTrans ? kConjNoTrans : kTrans;
    else
      trans = trans_invert(trans);
  }
  const bool ok_trans = herm ? (trans == kNoTrans || trans == kConjTrans)
                             : (trans == kNoTrans || trans == kTrans);
  const int nrowa = trans == kNoTrans ? n : k;
  if (!ok_trans || n < 0 || k < 0 || lda < std::max(1, nrowa) || ldc < std::max(1, n))
    return kErrInvalid;
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  const bool bone = beta[0] == R(1) && beta[1] == R(0);
  if (n == 0 || ((azero || k == 0) && bone)) return 0;
  cudaStream_t s = lib_stream();
  Staged<C2> A, C;
  const bool use_a = !azero && k > 0;
  if (use_a) ZG_TRY(A.in((const C2 *)a, lda, nrowa, trans == kNoTrans ? k : n, kSlotA, true, s));
  // C: the whole n x n square is staged so that the other triangle survives
  ZG_TRY(C.in((const C2 *)c, ldc, n, n, kSlotC, true, s));
  const R a0[2] = {use_a ? alpha[0] : R(0), use_a ? alpha[1] : R(0)};
  ZG_TRY(zsyherk_dev<R>(herm, uplo, trans, n, use_a ? k : 0, a0, (const R *)A.d,
                        A.ld ? A.ld : 1, beta, (R *)C.d, C.ld, s));
  ZG_TRY(C.out(s));
  return sync(s);
}

// Complex trsm (cblas_ztrsm / cblas_ctrsm, reference include/cblas.h:252-253;
// the row-major mapping of trsm.zig:18-64).
template <typename R>
int ztrsm_any(int order, int side, int uplo, int ta, int diag, int m, int n, const R *alpha,
              const R *a, int lda, R *b, int ldb) {
  using C2 = typename Cx<R>::T;
  if (!alpha) return kErrInvalid;
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if ((side != kLeft && side != kRight) || (uplo != kUpper && uplo != kLower) || !is_trans(ta) ||
      (diag != kUnit && diag != kNonUnit))
    return kErrInvalid;
  if (order == kRowMajor) {
    side = side == kLeft ? kRight : kLeft;
    uplo = uplo == kUpper ? kLower : kUpper;
    std::swap(m, n);
  }
  const int nrowa = side == kLeft ? m : n;
  if (m < 0 || n < 0 || lda < std::max(1, nrowa) || ldb < std::max(1, m)) return kErrInvalid;
  if (m == 0 || n == 0) return 0;
  const bool azero = alpha[0] == R(0) && alpha[1] == R(0);
  cudaStream_t s = lib_stream();
  Staged<C2> A, B;
  if (!azero) ZG_TRY(A.in((const C2 *)a, lda, nrowa, nrowa, kSlotA, true, s));
  ZG_TRY(B.in((const C2 *)b, ldb, m, n, kSlotB, !azero, s));
  ZG_TRY(ztrsm_dev<R>(side, uplo, ta, diag, m, n, alpha, (const R *)A.d, A.ld ? A.ld : 1,
                      (R *)B.d, B.ld, s));
  ZG_TRY(B.out(s));
  return sync(s);
}

template <typename T>
int syrk_any(int order, int uplo, int trans, int n, int k, T alpha, const T *a, int lda, T beta,
             T *c, int ldc) {
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if (uplo != kUpper && uplo != kLower) return kErrInvalid;
  if (!is_trans(trans)) return kErrInvalid;
  if (order == kRowMajor) {  // syrk.zig:28-57
    uplo = uplo == kUpper ? kLower : kUpper;
    trans = trans_invert(trans);
  }
  const int nrowa = trans == kNoTrans ? n : k;
  if (trans == kConjNoTrans || trans == kConjTrans || n < 0 || k < 0 ||
      lda < std::max(1, nrowa) || ldc < std::max(1, n))
    return kErrInvalid;  // syrk.zig:82-84
  if (n == 0 || ((alpha == T(0) || k == 0) && beta == T(1))) return 0;
  cudaStream_t s = lib_stream();
  Staged<T> A, C;
  const bool use_a = alpha != T(0) && k > 0;
  if (use_a) ZG_TRY(A.in(a, lda, nrowa, trans == kNoTrans ? k : n, kSlotA, true, s));
  // C: the whole n x n square is staged so that the other triangle survives
  ZG_TRY(C.in(c, ldc, n, n, kSlotC, true, s));
  if (use_a)
    ZG_TRY(syrk_dev<T>(uplo, trans, n, k, alpha, A.d, A.ld, beta, C.d, C.ld, s));
  else
    ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, n, n, 0, T(0), C.d, C.ld, C.d, C.ld, beta, C.d, C.ld,
                        uplo == kLower ? 1 : 2, s));
  ZG_TRY(C.out(s));
  return sync(s);
}

template <typename T>
int trsm_any(int order, int side, int uplo, int ta, int diag, int m, int n, T alpha, const T *a,
             int lda, T *b, int ldb) {
  if (order != kRowMajor && order != kColMajor) return kErrInvalid;
  if ((side != kLeft && side != kRight) || (uplo != kUpper && uplo != kLower) || !is_trans(ta) ||
      (diag != kUnit && diag != kNonUnit))
    return kErrInvalid;
  if (order == kRowMajor) {  // trsm.zig:48-63
    side = side == kLeft ? kRight : kLeft;
    uplo = uplo == kUpper ? kLower : kUpper;
    std::swap(m, n);
  }
  const int nrowa = side == kLeft ? m : n;
  if (m < 0 || n < 0 || lda < std::max(1, nrowa) || ldb < std::max(1, m)) return kErrInvalid;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = lib_stream();
  Staged<T> A, B;
  if (alpha != T(0)) ZG_TRY(A.in(a, lda, nrowa, nrowa, kSlotA, true, s));
  ZG_TRY(B.in(b, ldb, m, n, kSlotB, alpha != T(0), s));
  ZG_TRY(trsm_dev<T>(side, uplo, ta, diag, m, n, alpha, A.d, A.ld, B.d, B.ld, s));
  ZG_TRY(B.out(s));
  return sync(s);
}

// ---- LAPACK ------------------------------------------------------------------

int lay_ok(int layout) { return layout == kRowMajor || layout == kColMajor; }

// Brings a (possibly row-major) r x c matrix to a column-major device copy.
template <typename T> struct ColMajor {
  Staged<T> st;     // the caller's storage as it is
  T *d = nullptr;   // column-major view
  long ld = 0;
  bool transposed = false;
  int in(int layout, const T *p, int ldp, int r, int c, int slot, int tslot, bool copy,
         cudaStream_t s) {
    if (layout == kColMajor) {
      ZG_TRY(st.in(p, ldp, r, c, slot, copy, s));
      d = st.d;
      ld = st.ld;
      return 0;
    }
    // row-major r x c == column-major c x r with leading dimension ldp
    ZG_TRY(st.in(p, ldp, c, r, slot, copy, s));
    void *w;
    ZG_TRY(workspace(s, tslot, sizeof(T) * (size_t)std::max(1, r) * std::max(1, c), &w));
    d = (T *)w;
    ld = std::max(1, r);
    transposed = true;
    if (copy) ZG_TRY(transpose_dev<T>(c, r, st.d, st.ld, d, ld, s));
    return 0;
  }
  int out(cudaStream_t s) {
    if (transposed) ZG_TRY(transpose_dev<T>(st.cols, st.rows, d, ld, st.d, st.ld, s));
    return st.out(s);
  }
};

char up(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

template <typename T> int getrf_any(int layout, int m, int n, T *a, int lda, int *ipiv) {
  if (!lay_ok(layout)) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, layout == kColMajor ? m : n)) return -5;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  Buf<int> P;
  ZG_TRY(A.in(layout, a, lda, m, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(P.in(ipiv, std::min(m, n), kSlotPiv, false, s));
  int info = 0;
  ZG_TRY(getrf_dev<T>(m, n, A.d, A.ld, P.d, &info, s));
  ZG_TRY(A.out(s));
  ZG_TRY(P.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename T>
int getrs_any(int layout, char trans, int n, int nrhs, const T *a, int lda, const int *ipiv, T *b,
              int ldb) {
  if (!lay_ok(layout)) return -1;
  trans = up(trans);
  if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -9;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A, B;
  Buf<int> P;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(P.in(const_cast<int *>(ipiv), n, kSlotPiv, true, s));
  ZG_TRY(getrs_dev<T>(trans == 'N' ? kNoTrans : kTrans, n, nrhs, A.d, A.ld, P.d, B.d, B.ld, s));
  ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return 0;
}

template <typename T>
int gesv_any(int layout, int n, int nrhs, T *a, int lda, int *ipiv, T *b, int ldb) {
  if (!lay_ok(layout)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A, B;
  Buf<int> P;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(P.in(ipiv, n, kSlotPiv, false, s));
  int info = 0;
  ZG_TRY(getrf_dev<T>(n, n, A.d, A.ld, P.d, &info, s));
  if (info == 0) ZG_TRY(getrs_dev<T>(kNoTrans, n, nrhs, A.d, A.ld, P.d, B.d, B.ld, s));
  ZG_TRY(A.out(s));
  ZG_TRY(P.out(s));
  if (info == 0) ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename T> int potrf_any(int layout, char uplo, int n, T *a, int lda) {
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  int info = 0;
  ZG_TRY(potrf_dev<T>(uplo == 'L' ? kLower : kUpper, n, A.d, A.ld, &info, s));
  ZG_TRY(A.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename T>
int potrs_any(int layout, char uplo, int n, int nrhs, const T *a, int lda, T *b, int ldb) {
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A, B;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(potrs_dev<T>(uplo == 'L' ? kLower : kUpper, n, nrhs, A.d, A.ld, B.d, B.ld, s));
  ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return 0;
}

template <typename T>
int posv_any(int layout, char uplo, int n, int nrhs, T *a, int lda, T *b, int ldb) {
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A, B;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  const int ul = uplo == 'L' ? kLower : kUpper;
  int info = 0;
  ZG_TRY(potrf_dev<T>(ul, n, A.d, A.ld, &info, s));
  if (info == 0) ZG_TRY(potrs_dev<T>(ul, n, nrhs, A.d, A.ld, B.d, B.ld, s));
  ZG_TRY(A.out(s));
  if (info == 0) ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return info;
}

// ---- complex LAPACK (LAPACKE_z* / LAPACKE_c*, lapack.zig cfloat branches,
// e.g. :1190 LAPACKE_zgetrf) --------------------------------------------------
// Matrices are interleaved (re, im) pairs of R; argument checks and return
// codes as the real wrappers above.
template <typename R> int zgetrf_any(int layout, int m, int n, R *a, int lda, int *ipiv) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, layout == kColMajor ? m : n)) return -5;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A;
  Buf<int> P;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, m, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(P.in(ipiv, std::min(m, n), kSlotPiv, false, s));
  int info = 0;
  ZG_TRY(zgetrf_dev<R>(m, n, (R *)A.d, A.ld, P.d, &info, s));
  ZG_TRY(A.out(s));
  ZG_TRY(P.out(s));
  ZG_TRY(sync(s));
  return info;
}

int ztrans_code(char t) { return t == 'N' ? kNoTrans : t == 'T' ? kTrans : kConjTrans; }

template <typename R> int zgeqrf_any(int layout, int m, int n, R *a, int lda, R *tau) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, layout == kColMajor ? m : n)) return -5;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A;
  Buf<C2> Tau;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, m, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(Tau.in((C2 *)tau, std::min(m, n), kSlotPiv, false, s));
  ZG_TRY(zgeqrf_dev<R>(m, n, (R *)A.d, A.ld, (R *)Tau.d, s));
  ZG_TRY(A.out(s));
  ZG_TRY(Tau.out(s));
  return sync(s);
}

template <typename R>
int zgetrs_any(int layout, char trans, int n, int nrhs, const R *a, int lda, const int *ipiv,
               R *b, int ldb) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  trans = up(trans);
  if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -9;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A, B;
  Buf<int> P;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, (const C2 *)b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(P.in(const_cast<int *>(ipiv), n, kSlotPiv, true, s));
  ZG_TRY(zgetrs_dev<R>(ztrans_code(trans), n, nrhs, (const R *)A.d, A.ld, P.d, (R *)B.d, B.ld,
                       s));
  ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return 0;
}

template <typename R>
int zgesv_any(int layout, int n, int nrhs, R *a, int lda, int *ipiv, R *b, int ldb) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A, B;
  Buf<int> P;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, (const C2 *)b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(P.in(ipiv, n, kSlotPiv, false, s));
  int info = 0;
  ZG_TRY(zgetrf_dev<R>(n, n, (R *)A.d, A.ld, P.d, &info, s));
  if (info == 0) ZG_TRY(zgetrs_dev<R>(kNoTrans, n, nrhs, (const R *)A.d, A.ld, P.d, (R *)B.d, B.ld, s));
  ZG_TRY(A.out(s));
  ZG_TRY(P.out(s));
  if (info == 0) ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename R> int zpotrf_any(int layout, char uplo, int n, R *a, int lda) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, n, n, kSlotA, kSlotAT, true, s));
  int info = 0;
  ZG_TRY(zpotrf_dev<R>(uplo == 'L' ? kLower : kUpper, n, (R *)A.d, A.ld, &info, s));
  ZG_TRY(A.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename R>
int zpotrs_any(int layout, char uplo, int n, int nrhs, const R *a, int lda, R *b, int ldb) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A, B;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, (const C2 *)b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(zpotrs_dev<R>(uplo == 'L' ? kLower : kUpper, n, nrhs, (const R *)A.d, A.ld, (R *)B.d,
                       B.ld, s));
  ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return 0;
}

template <typename R>
int zposv_any(int layout, char uplo, int n, int nrhs, R *a, int lda, R *b, int ldb) {
  using C2 = typename Cx<R>::T;
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<C2> A, B;
  ZG_TRY(A.in(layout, (const C2 *)a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, (const C2 *)b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  const int ul = uplo == 'L' ? kLower : kUpper;
  int info = 0;
  ZG_TRY(zpotrf_dev<R>(ul, n, (R *)A.d, A.ld, &info, s));
  if (info == 0) ZG_TRY(zpotrs_dev<R>(ul, n, nrhs, (const R *)A.d, A.ld, (R *)B.d, B.ld, s));
  ZG_TRY(A.out(s));
  if (info == 0) ZG_TRY(B.out(s));
  ZG_TRY(sync(s));
  return info;
}

// Bunch-Kaufman (LAPACKE_dsytrf / ssytrf, called from lapack.zig:4400-4409):
// the uplo triangle of the symmetric n x n matrix is overwritten with the
// block-diagonal D and the multipliers; ipiv as LAPACK's dsytrf.
template <typename T, bool HERM = false>
int sytrf_any(int layout, char uplo, int n, T *a, int lda, int *ipiv) {
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  Buf<int> P;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(P.in(ipiv, n, kSlotPiv, false, s));
  int info = 0;
  if constexpr (HERM)
    ZG_TRY(hetrf_dev<T>(uplo == 'U' ? kUpper : kLower, n, A.d, A.ld, P.d, &info, s));
  else
    ZG_TRY(sytrf_dev<T>(uplo == 'U' ? kUpper : kLower, n, A.d, A.ld, P.d, &info, s));
  ZG_TRY(A.out(s));
  ZG_TRY(P.out(s));
  ZG_TRY(sync(s));
  return info;
}

template <typename T> int geqrf_any(int layout, int m, int n, T *a, int lda, T *tau) {
  if (!lay_ok(layout)) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max(1, layout == kColMajor ? m : n)) return -5;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  Buf<T> Tau;
  ZG_TRY(A.in(layout, a, lda, m, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(Tau.in(tau, std::min(m, n), kSlotPiv, false, s));
  ZG_TRY(geqrf_dev<T>(m, n, A.d, A.ld, Tau.d, s));
  ZG_TRY(A.out(s));
  ZG_TRY(Tau.out(s));
  return sync(s);
}

template <typename T> int orgqr_any(int layout, int m, int n, int k, T *a, int lda, const T *tau) {
  if (!lay_ok(layout)) return -1;
  if (m < 0) return -2;
  if (n < 0 || n > m) return -3;
  if (k < 0 || k > n) return -4;
  if (lda < std::max(1, layout == kColMajor ? m : n)) return -6;
  if (n == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  Buf<T> Tau;
  ZG_TRY(A.in(layout, a, lda, m, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(Tau.in(const_cast<T *>(tau), k, kSlotPiv, true, s));
  ZG_TRY(orgqr_dev<T>(m, n, k, A.d, A.ld, Tau.d, s));
  ZG_TRY(A.out(s));
  return sync(s);
}

template <typename T>
int laswp_any(int layout, int n, T *a, int lda, int k1, int k2, const int *ipiv, int incx) {
  if (!lay_ok(layout)) return -1;
  if (n < 0) return -2;
  if (incx == 0) return -7;
  if (n == 0 || k2 < k1) return 0;
  // rows touched: k1..k2 and every pivot target
  int rmax = k2;
  for (int i = k1 - 1; i < k2; ++i) rmax = std::max(rmax, ipiv[(long)i * std::abs(incx)]);
  if (layout == kColMajor ? lda < std::max(1, rmax) : lda < std::max(1, n)) return -4;
  if (std::abs(incx) != 1) {
    set_last_error("laswp: |incx| != 1 is not supported");
    return kErrInvalid;
  }
  cudaStream_t s = lib_stream();
  ColMajor<T> A;
  Buf<int> P;
  ZG_TRY(A.in(layout, a, lda, rmax, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(P.in(const_cast<int *>(ipiv), k2, kSlotPiv, true, s));
  ZG_TRY(laswp_dev<T>(n, A.d, A.ld, k1, k2, P.d, incx, s));
  ZG_TRY(A.out(s));
  return sync(s);
}

int mpir_any(int layout, int n, int nrhs, const double *a, int lda, const double *b, int ldb,
             double *x, int ldx, const MpirOpts &o, MpirResult *res) {
  if (!lay_ok(layout)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -7;
  if (ldx < std::max(1, layout == kColMajor ? n : nrhs)) return -9;
  *res = MpirResult{};
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<double> A, B, X;
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(X.in(layout, x, ldx, n, nrhs, kSlotX, kSlotXT, false, s));
  if (layout == kColMajor && mixed_streams_host(n, o) && is_pinned_host(a)) {
    // A from page-locked memory: its copy overlaps the factorization
    void *w;
    ZG_TRY(workspace(s, kSlotA, sizeof(double) * (size_t)n * n, &w));
    ZG_TRY(gesv_mpir_host(n, nrhs, a, lda, (double *)w, B.d, B.ld, X.d, X.ld, o, res, s));
  } else {
    ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
    ZG_TRY(gesv_mpir_dev(n, nrhs, A.d, A.ld, B.d, B.ld, X.d, X.ld, o, res, s));
  }
  ZG_TRY(X.out(s));
  return sync(s);
}

int auto_any(int layout, int n, int nrhs, const double *a, int lda, const double *b, int ldb,
             double *x, int ldx, const float *model, float confidence, int max_iter,
             AutoResult *res) {
  if (!lay_ok(layout)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -7;
  if (ldx < std::max(1, layout == kColMajor ? n : nrhs)) return -9;
  if (model && !(confidence > 0.f && confidence <= 1.f)) return -11;
  *res = AutoResult{};
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<double> A, B, X;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(X.in(layout, x, ldx, n, nrhs, kSlotX, kSlotXT, false, s));
  ZG_TRY(gesv_auto_dev(n, nrhs, A.d, A.ld, B.d, B.ld, X.d, X.ld, model, confidence, max_iter, res,
                       s));
  ZG_TRY(X.out(s));
  return sync(s);
}

int posv_mpir_any(int layout, char uplo, int n, int nrhs, const double *a, int lda,
                  const double *b, int ldb, double *x, int ldx, const MpirOpts &o,
                  MpirResult *res) {
  if (!lay_ok(layout)) return -1;
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldb < std::max(1, layout == kColMajor ? n : nrhs)) return -8;
  if (ldx < std::max(1, layout == kColMajor ? n : nrhs)) return -10;
  *res = MpirResult{};
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = lib_stream();
  ColMajor<double> A, B, X;
  ZG_TRY(A.in(layout, a, lda, n, n, kSlotA, kSlotAT, true, s));
  ZG_TRY(B.in(layout, b, ldb, n, nrhs, kSlotB, kSlotBT, true, s));
  ZG_TRY(X.in(layout, x, ldx, n, nrhs, kSlotX, kSlotXT, false, s));
  ZG_TRY(posv_mpir_dev(uplo == 'L', n, nrhs, A.d, A.ld, B.d, B.ld, X.d, X.ld, o, res, s));
  ZG_TRY(X.out(s));
  return sync(s);
}

}  // namespace

static_assert(sizeof(MpirResult) == 6 * sizeof(int) + 34 * sizeof(double), "zml_mpir_result layout");

extern "C" {

// ---- CBLAS (include/cblas.h) ----
#define CBLAS_GEMM(P, T)                                                                          \
  void cblas_##P##gemm(int order, int ta, int tb, int m, int n, int k, T alpha, const T *a,        \
                       int lda, const T *b, int ldb, T beta, T *c, int ldc) {                      \
    gemm_any<T>(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);                      \
  }                                                                                                \
  void cblas_##P##syrk(int order, int uplo, int trans, int n, int k, T alpha, const T *a, int lda, \
                       T beta, T *c, int ldc) {                                                    \
    syrk_any<T>(order, uplo, trans, n, k, alpha, a, lda, beta, c, ldc);                            \
  }                                                                                                \
  void cblas_##P##trsm(int order, int side, int uplo, int ta, int diag, int m, int n, T alpha,     \
                       const T *a, int lda, T *b, int ldb) {                                       \
    trsm_any<T>(order, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb);                         \
  }
CBLAS_GEMM(d, double)
CBLAS_GEMM(s, float)
#undef CBLAS_GEMM

#define CBLAS_ZGEMM(P, R)                                                                          \
  void cblas_##P##gemm(int order, int ta, int tb, int m, int n, int k, const void *alpha,           \
                       const void *a, int lda, const void *b, int ldb, const void *beta, void *c,   \
                       int ldc) {                                                                   \
    zgemm_any<R>(order, ta, tb, m, n, k, (const R *)alpha, (const R *)a, lda, (const R *)b, ldb,    \
                 (const R *)beta, (R *)c, ldc);                                                     \
  }                                                                                                 \
  void cblas_##P##herk(int order, int uplo, int trans, int n, int k, R alpha, const void *a,        \
                       int lda, R beta, void *c, int ldc) {                                         \
    const R al[2] = {alpha, R(0)}, be[2] = {beta, R(0)};                                            \
    zsyherk_any<R>(true, order, uplo, trans, n, k, al, (const R *)a, lda, be, (R *)c, ldc);         \
  }                                                                                                 \
  void cblas_##P##syrk(int order, int uplo, int trans, int n, int k, const void *alpha,             \
                       const void *a, int lda, const void *beta, void *c, int ldc) {                \
    zsyherk_any<R>(false, order, uplo, trans, n, k, (const R *)alpha, (const R *)a, lda,            \
                   (const R *)beta, (R *)c, ldc);                                                   \
  }
CBLAS_ZGEMM(z, double)
CBLAS_ZGEMM(c, float)
#undef CBLAS_ZGEMM

#define ZLAPACK_FNS(P, R)                                                                        \
  void cblas_##P##trsm(int order, int side, int uplo, int ta, int diag, int m, int n,             \
                       const void *alpha, const void *a, int lda, void *b, int ldb) {             \
    ztrsm_any<R>(order, side, uplo, ta, diag, m, n, (const R *)alpha, (const R *)a, lda,         \
                 (R *)b, ldb);                                                                   \
  }                                                                                              \
  int LAPACKE_##P##getrf(int layout, int m, int n, void *a, int lda, int *ipiv) {                \
    return zgetrf_any<R>(layout, m, n, (R *)a, lda, ipiv);                                       \
  }                                                                                              \
  int LAPACKE_##P##getrs(int layout, char trans, int n, int nrhs, const void *a, int lda,        \
                         const int *ipiv, void *b, int ldb) {                                    \
    return zgetrs_any<R>(layout, trans, n, nrhs, (const R *)a, lda, ipiv, (R *)b, ldb);          \
  }                                                                                              \
  int LAPACKE_##P##gesv(int layout, int n, int nrhs, void *a, int lda, int *ipiv, void *b,       \
                        int ldb) {                                                               \
    return zgesv_any<R>(layout, n, nrhs, (R *)a, lda, ipiv, (R *)b, ldb);                        \
  }                                                                                              \
  int LAPACKE_##P##potrf(int layout, char uplo, int n, void *a, int lda) {                       \
    return zpotrf_any<R>(layout, uplo, n, (R *)a, lda);                                          \
  }                                                                                              \
  int LAPACKE_##P##potrs(int layout, char uplo, int n, int nrhs, const void *a, int lda,         \
                         void *b, int ldb) {                                                     \
    return zpotrs_any<R>(layout, uplo, n, nrhs, (const R *)a, lda, (R *)b, ldb);                 \
  }                                                                                              \
  int LAPACKE_##P##posv(int layout, char uplo, int n, int nrhs, void *a, int lda, void *b,       \
                        int ldb) {                                                               \
    return zposv_any<R>(layout, uplo, n, nrhs, (R *)a, lda, (R *)b, ldb);                        \
  }                                                                                              \
  int LAPACKE_##P##geqrf(int layout, int m, int n, void *a, int lda, void *tau) {                \
    return zgeqrf_any<R>(layout, m, n, (R *)a, lda, (R *)tau);                                   \
  }                                                                                              \
  int LAPACKE_##P##sytrf(int layout, char uplo, int n, void *a, int lda, int *ipiv) {            \
    using C2 = typename Cx<R>::T;                                                                \
    return sytrf_any<C2>(layout, uplo, n, (C2 *)a, lda, ipiv);                                   \
  }                                                                                              \
  int LAPACKE_##P##hetrf(int layout, char uplo, int n, void *a, int lda, int *ipiv) {            \
    using C2 = typename Cx<R>::T;                                                                \
    return sytrf_any<C2, true>(layout, uplo, n, (C2 *)a, lda, ipiv);                             \
  }
int LAPACKE_dsytrf(int layout, char uplo, int n, double *a, int lda, int *ipiv) {
  return sytrf_any<double>(layout, uplo, n, a, lda, ipiv);
}
int LAPACKE_ssytrf(int layout, char uplo, int n, float *a, int lda, int *ipiv) {
  return sytrf_any<float>(layout, uplo, n, a, lda, ipiv);
}
ZLAPACK_FNS(z, double)
ZLAPACK_FNS(c, float)
#undef ZLAPACK_FNS

// ---- LAPACKE-shaped (include/clapack.h) ----
#define LAPACKE_FNS(P, T)                                                                        \
  int LAPACKE_##P##getrf(int layout, int m, int n, T *a, int lda, int *ipiv) {                   \
    return getrf_any<T>(layout, m, n, a, lda, ipiv);                                             \
  }                                                                                               \
  int LAPACKE_##P##getrs(int layout, char trans, int n, int nrhs, const T *a, int lda,           \
                         const int *ipiv, T *b, int ldb) {                                       \
    return getrs_any<T>(layout, trans, n, nrhs, a, lda, ipiv, b, ldb);                           \
  }                                                                                               \
  int LAPACKE_##P##gesv(int layout, int n, int nrhs, T *a, int lda, int *ipiv, T *b, int ldb) {  \
    return gesv_any<T>(layout, n, nrhs, a, lda, ipiv, b, ldb);                                   \
  }                                                                                               \
  int LAPACKE_##P##potrf(int layout, char uplo, int n, T *a, int lda) {                          \
    return potrf_any<T>(layout, uplo, n, a, lda);                                                \
  }                                                                                               \
  int LAPACKE_##P##potrs(int layout, char uplo, int n, int nrhs, const T *a, int lda, T *b,      \
                         int ldb) {                                                              \
    return potrs_any<T>(layout, uplo, n, nrhs, a, lda, b, ldb);                                  \
  }                                                                                               \
  int LAPACKE_##P##posv(int layout, char uplo, int n, int nrhs, T *a, int lda, T *b, int ldb) {  \
    return posv_any<T>(layout, uplo, n, nrhs, a, lda, b, ldb);                                   \
  }
LAPACKE_FNS(d, double)
LAPACKE_FNS(s, float)

int LAPACKE_dgeqrf(int layout, int m, int n, double *a, int lda, double *tau) {
  return geqrf_any<double>(layout, m, n, a, lda, tau);
}
int LAPACKE_sgeqrf(int layout, int m, int n, float *a, int lda, float *tau) {
  return geqrf_any<float>(layout, m, n, a, lda, tau);
}
int zml_gpu_zgeqrf(int m, int n, void *dA, int ldda, void *dtau, void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, m)) return -4;
  return zgeqrf_dev<double>(m, n, (double *)dA, ldda, (double *)dtau, (cudaStream_t)stream);
}
int zml_gpu_dgeqrf(int m, int n, double *dA, int ldda, double *dtau, void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, m)) return -4;
  return geqrf_dev<double>(m, n, dA, ldda, dtau, (cudaStream_t)stream);
}
int LAPACKE_dorgqr(int layout, int m, int n, int k, double *a, int lda, const double *tau) {
  return orgqr_any<double>(layout, m, n, k, a, lda, tau);
}
int LAPACKE_sorgqr(int layout, int m, int n, int k, float *a, int lda, const float *tau) {
  return orgqr_any<float>(layout, m, n, k, a, lda, tau);
}
int zml_gpu_dorgqr(int m, int n, int k, double *dA, int ldda, const double *dtau, void *stream) {
  if (m < 0) return -1;
  if (n < 0 || n > m) return -2;
  if (k < 0 || k > n) return -3;
  if (ldda < std::max(1, m)) return -5;
  return orgqr_dev<double>(m, n, k, dA, ldda, dtau, (cudaStream_t)stream);
}

int LAPACKE_dlaswp(int layout, int n, double *a, int lda, int k1, int k2, const int *ipiv,
                   int incx) {
  return laswp_any<double>(layout, n, a, lda, k1, k2, ipiv, incx);
}
int LAPACKE_slaswp(int layout, int n, float *a, int lda, int k1, int k2, const int *ipiv,
                   int incx) {
  return laswp_any<float>(layout, n, a, lda, k1, k2, ipiv, incx);
}
#undef LAPACKE_FNS

// ---- device-pointer, stream-ordered extensions (column-major) ----
int zml_gpu_dgetrf(int m, int n, double *dA, int ldda, int *dipiv, int *info, void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, m)) return -4;
  int inf = 0;
  int r = getrf_dev<double>(m, n, dA, ldda, dipiv, &inf, (cudaStream_t)stream);
  if (info) *info = inf;
  return r;
}
int zml_gpu_dgetrs(char trans, int n, int nrhs, const double *dA, int ldda, const int *dipiv,
                   double *dB, int lddb, void *stream) {
  trans = up(trans);
  if (trans != 'N' && trans != 'T' && trans != 'C') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (ldda < std::max(1, n)) return -5;
  if (lddb < std::max(1, n)) return -8;
  return getrs_dev<double>(trans == 'N' ? kNoTrans : kTrans, n, nrhs, dA, ldda, dipiv, dB, lddb,
                           (cudaStream_t)stream);
}
int zml_gpu_dpotrf(char uplo, int n, double *dA, int ldda, int *info, void *stream) {
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, n)) return -4;
  int inf = 0;
  int r = potrf_dev<double>(uplo == 'L' ? kLower : kUpper, n, dA, ldda, &inf,
                            (cudaStream_t)stream);
  if (info) *info = inf;
  return r;
}
int zml_gpu_dpotrs(char uplo, int n, int nrhs, const double *dA, int ldda, double *dB, int lddb,
                   void *stream) {
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (ldda < std::max(1, n)) return -5;
  if (lddb < std::max(1, n)) return -7;
  return potrs_dev<double>(uplo == 'L' ? kLower : kUpper, n, nrhs, dA, ldda, dB, lddb,
                           (cudaStream_t)stream);
}
int zml_gpu_dgemm(int ta, int tb, int m, int n, int k, double alpha, const double *dA, int ldda,
                  const double *dB, int lddb, double beta, double *dC, int lddc, void *stream) {
  if (!is_trans(ta) || !is_trans(tb)) return kErrInvalid;
  return gemm_simt<double>(ta, tb, m, n, k, alpha, dA, ldda, dB, lddb, beta, dC, lddc, 0,
                           (cudaStream_t)stream);
}

// C <- alpha A B^T + beta C with 16-bit K-major A (m x k), B (n x k) on the
// tensor cores; prec 0 = fp16, 1 = bf16.
int zml_gpu_gemm_lowp(int prec, int m, int n, int k, float alpha, const void *dA, int lda,
                      const void *dB, int ldb, float beta, float *dC, int ldc, void *stream) {
  if (prec != 0 && prec != 1) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (lda < std::max(1, k) || lda % 8) return -7;
  if (ldb < std::max(1, k) || ldb % 8) return -9;
  if (ldc < std::max(1, m)) return -12;
  cudaStream_t s = (cudaStream_t)stream;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  ZG_TRY(gemm_tc(m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, prec, &ctl->status, s));
  return check_status(s, ctl, nullptr);
}

// Mixed-precision solve of A X = B to FP64 backward error (host or device
// pointers).  prec: 0 fp16, 1 bf16, 2 fp32 trailing updates; mode: 0 plain
// IR, 1 GMRES-IR; tol 0 = refine until the backward error stagnates.
int zml_dgesv_mpir(int layout, int n, int nrhs, const double *a, int lda, const double *b, int ldb,
                   double *x, int ldx, int prec, int mode, double tol, int max_iter,
                   MpirResult *res) {
  if (prec < 0 || prec > 3) return -10;
  if (mode != 0 && mode != 1) return -11;
  MpirOpts o;
  o.prec = prec;
  o.mode = mode;
  o.tol = tol;
  o.max_iter = max_iter > 0 ? max_iter : 30;
  o.fallback = true;
  MpirResult local;
  return mpir_any(layout, n, nrhs, a, lda, b, ldb, x, ldx, o, res ? res : &local);
}

// LAPACK dsgesv semantics: FP32 factorization + FP64 iterative refinement;
// if refinement does not reach FP64 accuracy within 30 steps the system is
// re-solved with the FP64 LU (iter < 0), leaving that LU in a and ipiv.
int LAPACKE_dsgesv(int layout, int n, int nrhs, double *a, int lda, int *ipiv, double *b, int ldb,
                   double *x, int ldx, int *iter) {
  MpirOpts o;
  o.prec = kPrecFP32;
  o.mode = kModeIR;
  o.max_iter = 30;
  MpirResult res;
  int r = mpir_any(layout, n, nrhs, a, lda, b, ldb, x, ldx, o, &res);
  if (r < 0) return r;
  if (iter) *iter = res.iters;
  if (res.info == 0 && res.converged) return 0;
  // fallback: FP64 LU of a, solution into x (X <- B first; either may be
  // host or device memory)
  if (iter) *iter = -1;
  if (layout == kColMajor) {
    ZG_CUDA(cudaMemcpy2D(x, sizeof(double) * ldx, b, sizeof(double) * ldb, sizeof(double) * n,
                         nrhs, cudaMemcpyDefault));
  } else {
    ZG_CUDA(cudaMemcpy2D(x, sizeof(double) * ldx, b, sizeof(double) * ldb,
                         sizeof(double) * nrhs, n, cudaMemcpyDefault));
  }
  return gesv_any<double>(layout, n, nrhs, a, lda, ipiv, x, ldx);
}

// Mixed-precision SPD solve (low-precision Cholesky + FP64 refinement), host
// or device pointers; only the `uplo` triangle of A is read.
int zml_dposv_mpir(int layout, char uplo, int n, int nrhs, const double *a, int lda,
                   const double *b, int ldb, double *x, int ldx, int prec, int mode, double tol,
                   int max_iter, MpirResult *res) {
  if (prec < 0 || prec > 3) return -11;
  if (mode != 0 && mode != 1) return -12;
  MpirOpts o;
  o.prec = prec;
  o.mode = mode;
  o.tol = tol;
  o.max_iter = max_iter > 0 ? max_iter : 30;
  o.fallback = true;
  MpirResult local;
  return posv_mpir_any(layout, uplo, n, nrhs, a, lda, b, ldb, x, ldx, o, res ? res : &local);
}

// LAPACK dsposv semantics: FP32 Cholesky + FP64 refinement; FP64 posv fallback
// (iter < 0, a holding its factor) when refinement does not converge.
int LAPACKE_dsposv(int layout, char uplo, int n, int nrhs, double *a, int lda, double *b, int ldb,
                   double *x, int ldx, int *iter) {
  MpirOpts o;
  o.prec = kPrecFP32;
  o.mode = kModeIR;
  o.max_iter = 30;
  MpirResult res;
  int r = posv_mpir_any(layout, uplo, n, nrhs, a, lda, b, ldb, x, ldx, o, &res);
  if (r < 0) return r;
  if (iter) *iter = res.iters;
  if (res.info == 0 && res.converged) return 0;
  if (iter) *iter = -1;
  if (layout == kColMajor) {
    ZG_CUDA(cudaMemcpy2D(x, sizeof(double) * ldx, b, sizeof(double) * ldb, sizeof(double) * n,
                         nrhs, cudaMemcpyDefault));
  } else {
    ZG_CUDA(cudaMemcpy2D(x, sizeof(double) * ldx, b, sizeof(double) * ldb,
                         sizeof(double) * nrhs, n, cudaMemcpyDefault));
  }
  return posv_any<double>(layout, uplo, n, nrhs, a, lda, x, ldx);
}

int zml_gpu_dposv_mpir(char uplo, int n, int nrhs, const double *dA, int ldda, const double *dB,
                       int lddb, double *dX, int lddx, int prec, int mode, double tol,
                       int max_iter, MpirResult *res, void *stream) {
  uplo = up(uplo);
  if (uplo != 'U' && uplo != 'L') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (ldda < std::max(1, n)) return -5;
  if (lddb < std::max(1, n)) return -7;
  if (lddx < std::max(1, n)) return -9;
  if (prec < 0 || prec > 3) return -10;
  if (mode != 0 && mode != 1) return -11;
  MpirOpts o;
  o.prec = prec;
  o.mode = mode;
  o.tol = tol;
  o.max_iter = max_iter > 0 ? max_iter : 30;
  o.fallback = true;
  MpirResult local;
  return posv_mpir_dev(uplo == 'L', n, nrhs, dA, ldda, dB, lddb, dX, lddx, o,
                       res ? res : &local, (cudaStream_t)stream);
}

int zml_gpu_dgesv_mpir(int n, int nrhs, const double *dA, int ldda, const double *dB, int lddb,
                       double *dX, int lddx, int prec, int mode, double tol, int max_iter,
                       MpirResult *res, void *stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (ldda < std::max(1, n)) return -4;
  if (lddb < std::max(1, n)) return -6;
  if (lddx < std::max(1, n)) return -8;
  if (prec < 0 || prec > 3) return -9;
  if (mode != 0 && mode != 1) return -10;
  MpirOpts o;
  o.prec = prec;
  o.mode = mode;
  o.tol = tol;
  o.max_iter = max_iter > 0 ? max_iter : 30;
  o.fallback = true;
  MpirResult local;
  return gesv_mpir_dev(n, nrhs, dA, ldda, dB, lddb, dX, lddx, o, res ? res : &local,
                       (cudaStream_t)stream);
}

// ---- batched small solves ----
int zml_gpu_batched_plan_create(void **plan, int count, const int *n, const int *spd, int nrhs,
                                int prec, int max_ir) {
  if (!plan) return -1;
  if (count < 0) return -2;
  if (!n && count > 0) return -3;
  if (nrhs < 1 || nrhs > 64) return -5;
  if (prec != 0 && prec != 1) return -6;
  for (int i = 0; i < count; ++i)
    if (n[i] < 1 || n[i] > 256) {
      set_last_error("batched: n[%d] = %d outside 1..256", i, n[i]);
      return kErrInvalid;
    }
  BatchPlan *p = nullptr;
  ZG_TRY(batched_plan_create(&p, count, n, spd, nrhs, prec, max_ir));
  *plan = p;
  return 0;
}
int zml_gpu_batched_execute(void *plan, double *dA, const double *dB, double *dX, int *dipiv,
                            int *dinfo, int *diters, void *stream) {
  if (!plan) return -1;
  return batched_plan_execute((BatchPlan *)plan, dA, dB, dX, dipiv, dinfo, diters,
                              (cudaStream_t)stream);
}
int zml_gpu_batched_run_graph(void *plan, double *dA, const double *dB, double *dX, int *dipiv,
                              int *dinfo, int *diters, void *stream) {
  if (!plan) return -1;
  return batched_plan_run_graph((BatchPlan *)plan, dA, dB, dX, dipiv, dinfo, diters,
                                (cudaStream_t)stream);
}
void zml_gpu_batched_plan_destroy(void *plan) { batched_plan_destroy((BatchPlan *)plan); }
int zml_gpu_batched_schedule(int prec, int *warps, int *edges, int cap, int set) {
  if (edges) batched_classes(edges, cap);
  return batched_schedule(prec, warps, cap, set != 0);
}
int zml_gpu_batched_autotune(int prec, int nrhs, int *chosen, double *ms, void *stream) {
  if (prec != 0 && prec != 1) return -1;
  if (nrhs < 1 || nrhs > 64) return -2;
  return batched_autotune(prec, nrhs, (cudaStream_t)stream, chosen, ms);
}

// ---- learned precision selector ----
int zml_gpu_selector_features(int n, const double *dA, int ldda, float *dfeat, void *stream) {
  if (n < 1) return -1;
  if (ldda < n) return -3;
  return selector_features(n, dA, ldda, dfeat, (cudaStream_t)stream);
}
int zml_gpu_mlp_num_params(void) { return selector_num_params(); }
long zml_gpu_mlp_work_floats(int batch) { return (long)mlp_work_floats(batch); }
int zml_gpu_mlp_forward(int batch, const float *dX, const float *dP, float *dLogits, float *dWork,
                        void *stream) {
  if (batch < 1) return -1;
  return mlp_forward(batch, dX, dP, dLogits, dWork, (cudaStream_t)stream);
}
int zml_gpu_mlp_gradients(int batch, const float *dX, const int *dy, const float *dP, float *dG,
                          float *dLoss, float *dWork, void *stream) {
  if (batch < 1) return -1;
  return mlp_gradients(batch, dX, dy, dP, dG, dLoss, dWork, (cudaStream_t)stream);
}
int zml_gpu_mlp_adam(float *dP, const float *dG, float *dM, float *dV, float lr, float beta1,
                     float beta2, float eps, int step, float weight_decay, void *stream) {
  if (step < 1) return -9;
  return mlp_adam(dP, dG, dM, dV, lr, beta1, beta2, eps, step, weight_decay, (cudaStream_t)stream);
}
int zml_gpu_selector_model_floats(void) { return selector_num_params() + 2 * kSelFeatures; }

// Solve with the precision ladder, started where the selector network
// predicts (model != NULL) or at the bottom (model == NULL).
int zml_dgesv_auto(int layout, int n, int nrhs, const double *a, int lda, const double *b, int ldb,
                   double *x, int ldx, const float *model, float confidence, int max_iter,
                   AutoResult *res) {
  AutoResult local;
  return auto_any(layout, n, nrhs, a, lda, b, ldb, x, ldx, model, confidence, max_iter,
                  res ? res : &local);
}
int zml_gpu_dgesv_auto(int n, int nrhs, const double *dA, int ldda, const double *dB, int lddb,
                       double *dX, int lddx, const float *model, float confidence, int max_iter,
                       AutoResult *res, void *stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (ldda < std::max(1, n)) return -4;
  if (lddb < std::max(1, n)) return -6;
  if (lddx < std::max(1, n)) return -8;
  if (model && !(confidence > 0.f && confidence <= 1.f)) return -10;
  AutoResult local;
  return gesv_auto_dev(n, nrhs, dA, ldda, dB, lddb, dX, lddx, model, confidence, max_iter,
                       res ? res : &local, (cudaStream_t)stream);
}

const char *zml_gpu_last_error(void) { return last_error(); }

int zml_gpu_set_spin_limit(long long tries) { return set_spin_limit(tries); }

int zml_gpu_mixed_panel(int tournament) { return set_mixed_tournament(tournament); }

int zml_gpu_fp64_updates(int mode) { return set_fp64_updates(mode); }
int zml_gpu_panel_rows(int rows) { return set_panel_rows(rows); }

int zml_gpu_dgemm_slices(int m, int n, int k, const double *dA, int ldda, const double *dB,
                         int lddb, double *dC, int lddc, int lower, void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (k < 0 || k > 256) return -3;
  if (ldda < std::max(1, m)) return -5;
  if (!lower && lddb < std::max(1, k)) return -7;
  if (lddc < std::max(1, m)) return -9;
  if (lower && m != n) return -10;
  cudaStream_t s = (cudaStream_t)stream;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  ZG_TRY(dgemm_oz_sub(m, n, k, dA, ldda, dB, lddb, dC, lddc, lower != 0, &ctl->status, s));
  return check_status(s, ctl, nullptr);
}

int zml_gpu_sgetrf_calu(int m, int n, float *dA, int ldda, int *dipiv, int *info, void *stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < std::max(1, m)) return -4;
  int inf = 0;
  ZG_TRY(getrf_dev<float>(m, n, dA, ldda, dipiv, &inf, (cudaStream_t)stream, true));
  if (info) *info = inf;
  return 0;
}

int zml_gpu_version(void) { return 1; }

}  // extern "C"
