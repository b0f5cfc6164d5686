// sytrf.cu -- Bunch-Kaufman symmetric-indefinite factorization on the GPU:
// A = U D U^T or L D L^T with 1x1 and 2x2 pivot blocks (LAPACK's dsytf2
// pivoting, as zml restates it in lapack/sytf2.zig:17-522).
//
// One step per pivot block, driven from device memory: a single-CTA kernel
// takes the step's column from the previous step (a four-word state: column,
// block size, skip, done), finds the pivot (|a_kk|, the column maximum, and
// when needed the maximum of row imax, with zml's iamax semantics: the first
// maximum wins, a NaN never displaces it, a NaN at the first position blocks
// the search), decides the 1x1 / 2x2 block, performs the symmetric
// interchange and writes ipiv / info and the state; the update of the
// remaining triangle and the block's columns read the state too.  The host
// only enqueues n steps -- those past the last column find `done` set and
// return -- so no step waits for a round trip to the host.  Every product and sum of the update is
// rounded on its own (__dmul_rn / __dadd_rn; the compiler may not contract
// them into an FMA), in the association sytf2.zig writes, so the result is
// the restated unblocked algorithm's, bit for bit.  zml's sytrf factors
// matrices above nb = 64 columns with the blocked lasyf, whose sums are
// grouped differently; against it the factors agree to rounding.
#include <climits>

#include "common.cuh"
#include "kernels.h"

namespace zg {

// Arithmetic of one step, as the restatement performs it.  Real: every
// product and sum rounded on its own (no FMA contraction).  Complex (double2 /
// float2 = (re, im)): zml's cfloat -- products re = fma(x.re, y.re,
// -x.im y.im), im = fma(x.re, y.im, x.im y.re) (operand order matters),
// component-wise sums, Smith's division with fused updates, 1 / z as
// (1 + 0i) / z, and pivot magnitudes |re| + |im|.
template <typename T> struct BkOps;
template <typename F> struct BkReal {
  using R = F;
  static __device__ __forceinline__ F mul(F a, F b) { return BkOps<F>::rmul(a, b); }
  static __device__ __forceinline__ F add(F a, F b) { return BkOps<F>::radd(a, b); }
  static __device__ __forceinline__ F sub(F a, F b) { return BkOps<F>::rsub(a, b); }
  static __device__ __forceinline__ F div(F a, F b) { return BkOps<F>::rdiv(a, b); }
  static __device__ __forceinline__ F inv(F a) { return F(1) / a; }
  static __device__ __forceinline__ F sub1(F a) { return sub(a, F(1)); }
  static __device__ __forceinline__ F neg(F a) { return -a; }
  static __device__ __forceinline__ F mag(F a) { return fabs(a); }
  static __device__ __forceinline__ bool is0(F a) { return a == F(0); }
  static __device__ __forceinline__ bool is1(F a) { return a == F(1); }
};
template <> struct BkOps<double> : BkReal<double> {
  static __device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
};
template <> struct BkOps<float> : BkReal<float> {
  static __device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
};
template <typename C, typename F> struct BkCplx {
  using R = F;
  using O = BkOps<F>;
  static __device__ __forceinline__ C mk(F re, F im) {
    C z;
    z.x = re;
    z.y = im;
    return z;
  }
  static __device__ __forceinline__ C mul(C a, C b) {
    return mk(fma(a.x, b.x, O::rmul(-a.y, b.y)), fma(a.x, b.y, O::rmul(a.y, b.x)));
  }
  static __device__ __forceinline__ C add(C a, C b) { return mk(O::radd(a.x, b.x), O::radd(a.y, b.y)); }
  static __device__ __forceinline__ C sub(C a, C b) { return mk(O::rsub(a.x, b.x), O::rsub(a.y, b.y)); }
  static __device__ __forceinline__ C div(C a, C b) {
    if (fabs(b.y) < fabs(b.x)) {
      const F t1 = O::rdiv(b.y, b.x);
      const F t2 = O::rdiv(F(1), fma(t1, b.y, b.x));
      return mk(O::rmul(fma(a.y, t1, a.x), t2), O::rmul(fma(-a.x, t1, a.y), t2));
    }
    const F t1 = O::rdiv(b.x, b.y);
    const F t2 = O::rdiv(F(1), fma(t1, b.x, b.y));
    return mk(O::rmul(fma(a.x, t1, a.y), t2), O::rmul(fma(a.y, t1, -a.x), t2));
  }
  static __device__ __forceinline__ C inv(C a) { return div(mk(F(1), F(0)), a); }
  static __device__ __forceinline__ C sub1(C a) { return mk(O::rsub(a.x, F(1)), a.y); }
  static __device__ __forceinline__ C neg(C a) { return mk(-a.x, -a.y); }
  static __device__ __forceinline__ F mag(C a) { return O::radd(fabs(a.x), fabs(a.y)); }
  static __device__ __forceinline__ bool is0(C a) { return a.x == F(0) && a.y == F(0); }
  static __device__ __forceinline__ bool is1(C a) { return a.x == F(1) && a.y == F(0); }
};
template <> struct BkOps<double2> : BkCplx<double2, double> {};
template <> struct BkOps<float2> : BkCplx<float2, float> {};

// the C macro max of the restatement: (a) > (b) ? (a) : (b)
template <typename T> __device__ __forceinline__ T cmax(T a, T b) { return a > b ? a : b; }

// zml's iamax over len magnitudes v(t), t = 0 .. len-1, by the whole CTA:
// the first maximum, NaN never chosen, a NaN first blocks (index 0).
template <typename T, typename F>
__device__ int cta_iamax(int len, F v, T *sv, int *si) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  T best = T(-1);
  int bi = INT_MAX;
  for (int q = t; q < len; q += blockDim.x) {
    const T a = v(q);
    if (a > best) {
      best = a;
      bi = q;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const T ov = __shfl_down_sync(0xffffffffu, best, off);
    const int oi = __shfl_down_sync(0xffffffffu, bi, off);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  __syncthreads();
  if (lane == 0) {
    sv[w] = best;
    si[w] = bi;
  }
  __syncthreads();
  if (t == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
      if (sv[q] > best || (sv[q] == best && si[q] < bi)) {
        best = sv[q];
        bi = si[q];
      }
    const T a0 = len > 0 ? v(0) : T(0);
    si[0] = (len <= 0 || a0 != a0 || bi == INT_MAX) ? 0 : bi;
  }
  __syncthreads();
  const int r = si[0];
  __syncthreads();
  return r;
}

// info: the first zero pivot column in the order the steps run (the upper
// factorization runs from the last column down), as sytf2.zig:67-68 sets it.
__device__ __forceinline__ void record_first(int *info, int v) { atomicCAS(info, 0, v); }

// The state of the factorization in device memory: st[0] = the current
// step's column k, st[1] = its block size, st[2] = 1 when the column is zero
// (or its diagonal NaN) and the step makes no update, st[3] = 1 once every
// column is done.
enum : int { kStK = 0, kStStep = 1, kStSkip = 2, kStDone = 3 };

// Thread 0's value of v for the whole CTA.  Every value a branch depends on
// goes through here, so the control flow around the CTA's barriers is the
// same in every thread even when the matrix changes under the kernel.
template <typename T> __device__ __forceinline__ T cta_bcast(T v, T *slot) {
  __syncthreads();
  if (threadIdx.x == 0) *slot = v;
  __syncthreads();
  return *slot;
}

// Step k (sytf2.zig:30-296 upper, 297-515 lower; HERM: hetf2.zig, the
// Hermitian form): the column after the previous step's block, pivot choice,
// interchange, ipiv, info.
template <typename T, bool HERM>
__global__ void __launch_bounds__(1024) sytf2_pivot_kernel(int n, T *A, long lda, bool upper,
                                                           typename BkOps<T>::R alpha, int *ipiv,
                                                           int *st, int *info) {
  using Ops = BkOps<T>;
  using R = typename Ops::R;
  using RO = BkOps<R>;
  __shared__ R sv[32];
  __shared__ int si[32];
  __shared__ R sb;
  auto a = [&](int i, int j) -> T & { return A[i + (long)j * lda]; };
  if (st[kStDone]) return;
  const int k = upper ? st[kStK] - st[kStStep] : st[kStK] + st[kStStep];
  if (upper ? k < 0 : k >= n) {
    __syncthreads();  // every thread has read the state
    if (threadIdx.x == 0) st[kStDone] = 1;
    return;
  }
  R akk_mag;
  if constexpr (HERM) akk_mag = fabs(a(k, k).x);  // the diagonal's real part
  else akk_mag = Ops::mag(a(k, k));
  const R absakk = cta_bcast(akk_mag, &sb);
  int imax = 0;
  R colmax = R(0);
  if (upper) {
    if (k > 0) {
      imax = cta_iamax<R>(k, [&](int q) { return Ops::mag(a(q, k)); }, sv, si);
      colmax = cta_bcast(Ops::mag(a(imax, k)), &sb);
    }
  } else if (k < n - 1) {
    imax = k + 1 + cta_iamax<R>(n - k - 1, [&](int q) { return Ops::mag(a(k + 1 + q, k)); }, sv, si);
    colmax = cta_bcast(Ops::mag(a(imax, k)), &sb);
  }
  int kp = k, kstep = 1, skip = 0;
  if (cmax(absakk, colmax) == R(0) || absakk != absakk) {
    skip = 1;
  } else if (!(absakk >= RO::mul(alpha, colmax))) {
    R rowmax;
    if (upper) {
      int jmax = imax + 1 +
                 cta_iamax<R>(k - imax, [&](int q) { return Ops::mag(a(imax, imax + 1 + q)); }, sv, si);
      rowmax = cta_bcast(Ops::mag(a(imax, jmax)), &sb);
      if (imax > 0) {
        jmax = cta_iamax<R>(imax, [&](int q) { return Ops::mag(a(q, imax)); }, sv, si);
        rowmax = cmax(rowmax, cta_bcast(Ops::mag(a(jmax, imax)), &sb));
      }
    } else {
      int jmax = k + cta_iamax<R>(imax - k, [&](int q) { return Ops::mag(a(imax, k + q)); }, sv, si);
      rowmax = cta_bcast(Ops::mag(a(imax, jmax)), &sb);
      if (imax < n - 1) {
        jmax = imax + 1 + cta_iamax<R>(n - imax - 1,
                                       [&](int q) { return Ops::mag(a(imax + 1 + q, imax)); }, sv, si);
        rowmax = cmax(rowmax, cta_bcast(Ops::mag(a(jmax, imax)), &sb));
      }
    }
    const R absimax = cta_bcast(Ops::mag(a(imax, imax)), &sb);
    if (absakk >= RO::mul(alpha, RO::mul(colmax, RO::div(colmax, rowmax)))) {
      kp = k;
    } else if (absimax >= RO::mul(alpha, rowmax)) {
      kp = imax;
    } else {
      kp = imax;
      kstep = 2;
    }
  }
  const int t = threadIdx.x;
  __syncthreads();  // every thread has read what the decision needs
  if (!skip) {
    const int kk = upper ? k - kstep + 1 : k + kstep - 1;
    // the entries that cross the diagonal are conjugated in the Hermitian form
    auto cr = [](T x) -> T {
      if constexpr (HERM) x.y = -x.y;
      return x;
    };
    if (kp != kk) {  // the interchange: disjoint pairs, all at once
      if (upper) {
        for (int i = t; i < kp; i += blockDim.x) {  // columns kk and kp above row kp
          const T x = a(i, kk);
          a(i, kk) = a(i, kp);
          a(i, kp) = x;
        }
        for (int q = t; q < kk - kp - 1; q += blockDim.x) {  // column kk below kp <-> row kp
          const T x = cr(a(kp + 1 + q, kk));
          a(kp + 1 + q, kk) = cr(a(kp, kp + 1 + q));
          a(kp, kp + 1 + q) = x;
        }
      } else {
        for (int q = t; q < n - kp - 1; q += blockDim.x) {  // columns kk and kp below row kp
          const T x = a(kp + 1 + q, kk);
          a(kp + 1 + q, kk) = a(kp + 1 + q, kp);
          a(kp + 1 + q, kp) = x;
        }
        for (int q = t; q < kp - kk - 1; q += blockDim.x) {  // column kk below kk <-> row kp
          const T x = cr(a(kk + 1 + q, kk));
          a(kk + 1 + q, kk) = cr(a(kp, kk + 1 + q));
          a(kp, kk + 1 + q) = x;
        }
      }
      if (t == 0) {
        if constexpr (HERM) {  // hetf2: a(kp, kk) conjugated, the diagonal kept real
          a(kp, kk) = cr(a(kp, kk));
          const R r1 = a(kk, kk).x;
          a(kk, kk) = Ops::mk(a(kp, kp).x, R(0));
          a(kp, kp) = Ops::mk(r1, R(0));
          if (kstep == 2) a(k, k).y = R(0);
        } else {
          T x = a(kk, kk);
          a(kk, kk) = a(kp, kp);
          a(kp, kp) = x;
        }
        if (kstep == 2) {
          const int r = upper ? k - 1 : k + 1;
          const T x = a(r, k);
          a(r, k) = a(kp, k);
          a(kp, k) = x;
        }
      }
    } else if constexpr (HERM) {
      if (t == 0) {  // the block's diagonal made real
        a(k, k).y = R(0);
        if (kstep == 2) {
          const int r = upper ? k - 1 : k + 1;
          a(r, r).y = R(0);
        }
      }
    }
  }
  if (t == 0) {
    if (skip) record_first(info, k + 1);
    if (kstep == 1) {
      ipiv[k] = kp + 1;
    } else {
      ipiv[k] = -(kp + 1);
      ipiv[upper ? k - 1 : k + 1] = -(kp + 1);
    }
    st[kStK] = k;
    st[kStStep] = kstep;
    st[kStSkip] = skip;
  }
}

// The update of step k.  1x1 (sytf2.zig:158-180 / 404-426): syr with
// alpha = -1/d on the triangle still to factor, a_ij += x_i (x_j (-1/d)),
// column j skipped where x_j == 0 (syr.zig:62, 142).  2x2 (185-236 /
// 430-482): the multipliers of column j from the original columns k, k-1
// (upper) or k, k+1 (lower), then a_ij -= a_ik wk + a_ik' wk'.  The columns
// of the block are rewritten afterwards by sytf2_store_kernel.  HERM
// (hetf2.zig): her with the real alpha -1/re(d), a_ij += x_i (conj(x_j)
// alpha), the diagonal kept real; 2x2 with d = |a_k',k| and conjugated
// multipliers, a_ij -= a_ik conj(wk) + a_ik' conj(wk').
template <typename T> struct HermScalars {
  typename BkOps<T>::R d, dk, dother;
  T dd;
};
// hetf2's 2x2 block scalars: d = |a(k2, k)|, dk = re a(k, k) / d, dother =
// re a(k2, k2) / d, dd = a(k2, k) / d, then d <- (1 / (dk dother - 1)) / d
template <typename T>
__device__ __forceinline__ HermScalars<T> herm_scalars(const T &akk, const T &a2k, const T &a22) {
  using R = typename BkOps<T>::R;
  using RO = BkOps<R>;
  HermScalars<T> h;
  R d = hypot(a2k.x, a2k.y);
  h.dother = RO::div(a22.x, d);
  h.dk = RO::div(akk.x, d);
  const R t = R(1) / RO::sub(RO::mul(h.dk, h.dother), R(1));
  h.dd = BkOps<T>::mk(RO::div(a2k.x, d), RO::div(a2k.y, d));
  h.d = RO::div(t, d);
  return h;
}
template <typename T>
__device__ __forceinline__ T cscale(const T &z, typename BkOps<T>::R s) {
  using RO = BkOps<typename BkOps<T>::R>;
  return BkOps<T>::mk(RO::mul(z.x, s), RO::mul(z.y, s));
}
template <typename T> __device__ __forceinline__ T cconj(T z) {
  z.y = -z.y;
  return z;
}
// wk (the multiplier of column k) and wo (of the block's other column) in
// column j of the Hermitian 2x2 step: wk = d (dother a_jk - dd a_jo),
// wo = d (dk a_jo - conj(dd) a_jk), in both triangles (hetf2.zig)
template <typename T>
__device__ __forceinline__ void herm_mult(const HermScalars<T> &h, const T &ajk, const T &ajo, T &wk,
                                          T &wo) {
  using Ops = BkOps<T>;
  wk = cscale(Ops::sub(cscale(ajk, h.dother), Ops::mul(h.dd, ajo)), h.d);
  wo = cscale(Ops::sub(cscale(ajo, h.dk), Ops::mul(cconj(h.dd), ajk)), h.d);
}

template <typename T, bool HERM>
__global__ void __launch_bounds__(256) sytf2_update_kernel(int n, T *A, long lda, bool upper,
                                                           const int *st) {
  using Ops = BkOps<T>;
  using R = typename Ops::R;
  auto a = [&](int i, int j) -> T & { return A[i + (long)j * lda]; };
  if (st[kStDone] || st[kStSkip]) return;
  const int k = st[kStK], kstep = st[kStStep];
  // the triangle to update: upper rows/cols [0, m), lower [k + kstep, n)
  const int m = upper ? k - kstep + 1 : n - k - kstep;
  const int o = upper ? 0 : k + kstep;
  const long tot = (long)m * m;
  if (kstep == 1) {
    if constexpr (HERM) {
      const R alpha = -(R(1) / a(k, k).x);
      for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot;
           e += (long)gridDim.x * blockDim.x) {
        const int i = o + (int)(e % m), j = o + (int)(e / m);
        if (upper ? i > j : i < j) continue;
        const T xj = a(j, k);
        if (Ops::is0(xj)) {
          if (i == j) a(j, j).y = R(0);
          continue;
        }
        const T temp = cscale(cconj(xj), alpha);
        if (i == j) a(j, j) = Ops::mk(BkOps<R>::add(a(j, j).x, Ops::mul(xj, temp).x), R(0));
        else a(i, j) = Ops::add(a(i, j), Ops::mul(a(i, k), temp));
      }
    } else {
      const T r1 = Ops::inv(a(k, k));
      const T nr1 = Ops::neg(r1);
      for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot;
           e += (long)gridDim.x * blockDim.x) {
        const int i = o + (int)(e % m), j = o + (int)(e / m);
        if (upper ? i > j : i < j) continue;
        const T xj = a(j, k);
        if (Ops::is0(xj)) continue;
        const T temp = Ops::mul(xj, nr1);
        a(i, j) = Ops::add(a(i, j), Ops::mul(a(i, k), temp));
      }
    }
  } else {
    const int k2 = upper ? k - 1 : k + 1;  // the block's other column
    if constexpr (HERM) {
      const HermScalars<T> h = herm_scalars(a(k, k), a(k2, k), a(k2, k2));
      for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot;
           e += (long)gridDim.x * blockDim.x) {
        const int i = o + (int)(e % m), j = o + (int)(e / m);
        if (upper ? i > j : i < j) continue;
        T wk, wo;
        herm_mult(h, a(j, k), a(j, k2), wk, wo);
        T v = Ops::sub(a(i, j),
                       Ops::add(Ops::mul(a(i, k), cconj(wk)), Ops::mul(a(i, k2), cconj(wo))));
        if (i == j) v.y = R(0);
        a(i, j) = v;
      }
    } else {
      T d = a(k2, k);  // d12 (upper) / d21 (lower)
      const T dkk = Ops::div(a(k2, k2), d);  // d22 (upper) / d11 (lower)
      const T dk = Ops::div(a(k, k), d);     // d11 (upper) / d22 (lower)
      const T t = Ops::inv(Ops::sub1(Ops::mul(upper ? dk : dkk, upper ? dkk : dk)));
      d = Ops::div(t, d);
      for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot;
           e += (long)gridDim.x * blockDim.x) {
        const int i = o + (int)(e % m), j = o + (int)(e / m);
        if (upper ? i > j : i < j) continue;
        T wk, wo;  // the multipliers of columns k and k2 in column j
        if (upper) {  // wkm1 = d12 (d11 a_j,k-1 - a_jk), wk = d12 (d22 a_jk - a_j,k-1)
          wo = Ops::mul(d, Ops::sub(Ops::mul(dk, a(j, k2)), a(j, k)));
          wk = Ops::mul(d, Ops::sub(Ops::mul(dkk, a(j, k)), a(j, k2)));
        } else {  // wk = d21 (d11 a_jk - a_j,k+1), wkp1 = d21 (d22 a_j,k+1 - a_jk)
          wk = Ops::mul(d, Ops::sub(Ops::mul(dkk, a(j, k)), a(j, k2)));
          wo = Ops::mul(d, Ops::sub(Ops::mul(dk, a(j, k2)), a(j, k)));
        }
        a(i, j) = Ops::sub(a(i, j), Ops::add(Ops::mul(a(i, k), wk), Ops::mul(a(i, k2), wo)));
      }
    }
  }
}

// The block's columns after the update: x / d (1x1) or the multipliers (2x2).
template <typename T, bool HERM>
__global__ void __launch_bounds__(256) sytf2_store_kernel(int n, T *A, long lda, bool upper,
                                                          const int *st) {
  using Ops = BkOps<T>;
  using R = typename Ops::R;
  auto a = [&](int i, int j) -> T & { return A[i + (long)j * lda]; };
  if (st[kStDone] || st[kStSkip]) return;
  const int k = st[kStK], kstep = st[kStStep];
  const int m = upper ? k - kstep + 1 : n - k - kstep;
  const int o = upper ? 0 : k + kstep;
  const int j0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (kstep == 1) {
    if constexpr (HERM) {  // x scaled by the real 1 / re(d), no early return
      const R r1 = R(1) / a(k, k).x;
      for (int j = j0; j < m; j += gridDim.x * blockDim.x) a(o + j, k) = cscale(a(o + j, k), r1);
    } else {
      const T r1 = Ops::inv(a(k, k));
      if (Ops::is1(r1)) return;  // scal returns early for alpha == 1 (scal.zig)
      for (int j = j0; j < m; j += gridDim.x * blockDim.x) a(o + j, k) = Ops::mul(a(o + j, k), r1);
    }
    return;
  }
  const int k2 = upper ? k - 1 : k + 1;
  if constexpr (HERM) {
    const HermScalars<T> h = herm_scalars(a(k, k), a(k2, k), a(k2, k2));
    for (int q = j0; q < m; q += gridDim.x * blockDim.x) {
      const int j = o + q;
      T wk, wo;
      herm_mult(h, a(j, k), a(j, k2), wk, wo);
      a(j, k) = wk;
      a(j, k2) = wo;
    }
    return;
  }
  T d = a(k2, k);
  const T dkk = Ops::div(a(k2, k2), d), dk = Ops::div(a(k, k), d);
  const T t = Ops::inv(Ops::sub1(Ops::mul(upper ? dk : dkk, upper ? dkk : dk)));
  d = Ops::div(t, d);
  for (int q = j0; q < m; q += gridDim.x * blockDim.x) {
    const int j = o + q;
    T wk, wo;
    if (upper) {
      wo = Ops::mul(d, Ops::sub(Ops::mul(dk, a(j, k2)), a(j, k)));
      wk = Ops::mul(d, Ops::sub(Ops::mul(dkk, a(j, k)), a(j, k2)));
    } else {
      wk = Ops::mul(d, Ops::sub(Ops::mul(dkk, a(j, k)), a(j, k2)));
      wo = Ops::mul(d, Ops::sub(Ops::mul(dk, a(j, k2)), a(j, k)));
    }
    a(j, k) = wk;
    a(j, k2) = wo;
  }
}

template <typename T, bool HERM>
static int bk_dev(int uplo, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  void *w;
  ZG_TRY(workspace(s, kSlotSytrf, sizeof(int) * 4, &w));
  int *st = (int *)w;
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const bool upper = uplo == kUpper;
  using R = typename BkOps<T>::R;
  const R alpha = (R(1) + std::sqrt(R(17))) / R(8);
  // the first step's column is n - 1 (upper) or 0 (lower)
  const int st0[4] = {upper ? n : -1, 1, 0, 0};
  ZG_CUDA(cudaMemcpyAsync(st, st0, sizeof st0, cudaMemcpyHostToDevice, s));
  const long tot = (long)n * n;
  const int grid = (int)std::max(1L, std::min((tot + 255) / 256, (long)di.num_sms * 8));
  // at most n steps (one per column when every block is 1x1)
  for (int it = 0; it < n; ++it) {
    ZG_LAUNCH(kTagPanel, 0, 0, s,
              (sytf2_pivot_kernel<T, HERM><<<1, 1024, 0, s>>>(n, A, lda, upper, alpha, ipiv, st,
                                                        &ctl->info)));
    ZG_LAUNCH(kTagPotf2, 0, 0, s,
              (sytf2_update_kernel<T, HERM><<<grid, 256, 0, s>>>(n, A, lda, upper, st)));
    ZG_LAUNCH(kTagPotf2, 0, 0, s,
              (sytf2_store_kernel<T, HERM><<<ceil_div(n, 256), 256, 0, s>>>(n, A, lda, upper, st)));
  }
  return check_status(s, ctl, info);
}

template <typename T>
int sytrf_dev(int uplo, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s) {
  return bk_dev<T, false>(uplo, n, A, lda, ipiv, info, s);
}
template <typename T>
int hetrf_dev(int uplo, int n, T *A, long lda, int *ipiv, int *info, cudaStream_t s) {
  return bk_dev<T, true>(uplo, n, A, lda, ipiv, info, s);
}

template int sytrf_dev<double>(int, int, double *, long, int *, int *, cudaStream_t);
template int sytrf_dev<float>(int, int, float *, long, int *, int *, cudaStream_t);
template int sytrf_dev<double2>(int, int, double2 *, long, int *, int *, cudaStream_t);
template int sytrf_dev<float2>(int, int, float2 *, long, int *, int *, cudaStream_t);
template int hetrf_dev<double2>(int, int, double2 *, long, int *, int *, cudaStream_t);
template int hetrf_dev<float2>(int, int, float2 *, long, int *, int *, cudaStream_t);

}  // namespace zg
