// zqr.cu -- complex Householder QR (zgeqrf / cgeqrf) on the GPU.
//
// Replaces the cfloat branch of zml's geqrf (lapack.zig:5138 LAPACKE_cgeqrf,
// :5152 LAPACKE_zgeqrf; kernel lapack/geqrf.zig:18-157) with its panel
// geqr2.zig:17-59 (larfg.zig:17-170, larf1f.zig:17-259), the triangular factor
// larft.zig:18-231 and the block reflector larfb.zig:20-178 applied as H^H
// (conj_trans, geqrf.zig:116), nb = 32.  The structure is the real QR's
// (qr.cu) in complex arithmetic:
//   * panel: one cooperative launch, a slab of rows per CTA in shared memory.
//     Per column k, one bounded grid barrier for the sum of |x_i|^2 below the
//     diagonal, after which every CTA forms larfg's reflector the same way:
//     beta = -sign(re alpha) lapy3(re alpha, im alpha, ||x||),
//     tau = ((beta - re alpha) / beta, -im alpha / beta),
//     v = x / (alpha - beta) (the quotient of complex numbers, Smith's method
//     with fused updates as zml's cfloat division), alpha <- beta; H = I when
//     x = 0 and alpha is real.  A second barrier for w = v^H A(k:, k+1:), then
//     A -= conj(tau) v w (geqr2 applies H^H, larf1f with conj(tau));
//   * T from the Gram matrix G = V^H V: T(0:j, j) = -tau_j T(0:j, 0:j) G(0:j, j),
//     T(j, j) = tau_j, the T of larft's recursion in another order;
//   * block reflector: C <- H^H C = C - V (T^H (V^H C)), three complex GEMMs on
//     the expanded real operand (zblas.cu).
// As in the real QR: the norm is a plain sum of squares (zml's nrm2 scales by
// Blue's thresholds, which only matters beyond 1e+150 or below 1e-150) and
// larfg's rescaling loop for |beta| < safmin / eps is not taken.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace zg {

namespace {

constexpr int kZqrNB = 32;

template <typename C2, typename R> __device__ __forceinline__ C2 qz(R re, R im) {
  C2 z;
  z.x = re;
  z.y = im;
  return z;
}
// zml's cfloat product (cfloat.zig:149-174) and Smith's division with fused
// updates (cfloat.zig:206-290)
template <typename C2> __device__ __forceinline__ C2 qz_mul(C2 a, C2 b) {
  return qz<C2>(fma(a.x, b.x, (-a.y) * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename C2> __device__ __forceinline__ C2 qz_conj(C2 a) { return qz<C2>(a.x, -a.y); }
template <typename C2> __device__ __forceinline__ C2 qz_div(C2 x, C2 y) {
  if (fabs(y.y) < fabs(y.x)) {
    const auto t1 = y.y / y.x;
    const auto t2 = decltype(t1)(1) / fma(t1, y.y, y.x);
    return qz<C2>(fma(x.y, t1, x.x) * t2, fma(-x.x, t1, x.y) * t2);
  }
  const auto t1 = y.x / y.y;
  const auto t2 = decltype(t1)(1) / fma(t1, y.x, y.y);
  return qz<C2>(fma(x.x, t1, x.y) * t2, fma(x.y, t1, -x.x) * t2);
}
template <typename C2> __device__ __forceinline__ C2 qz_add(C2 a, C2 b) {
  return qz<C2>(a.x + b.x, a.y + b.y);
}

template <typename C2> __device__ __forceinline__ C2 warp_sum(C2 a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
  }
  return a;
}

// The panel of nb <= 32 columns, m rows (column-major, lda), factored in
// place; tau (nb) and T (nb x nb, ld nb) out.  Exchange words: sums of squares
// [2][nblk] (re part), alpha [2], w [2][nblk][nb], Gram partials [nblk][nb][nb].
template <typename R, typename C2>
__global__ void __launch_bounds__(256) zqr_panel_kernel(int m, int nb, C2 *__restrict__ A, long lda,
                                                        C2 *__restrict__ tau, C2 *__restrict__ Tout,
                                                        Control *ctl, int RR, C2 *__restrict__ xchg) {
  extern __shared__ __align__(16) unsigned char zqsm_raw[];
  C2 *S = reinterpret_cast<C2 *>(zqsm_raw);  // S[c * RR + r]
  __shared__ R red[8];
  __shared__ C2 w_s[kZqrNB];
  __shared__ C2 sc_tau, sc_scale;
  __shared__ R sc_beta;
  const int b = blockIdx.x, nblk = gridDim.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int r0 = b * RR, rows = max(0, min(RR, m - r0));
  C2 *ssq_slot = xchg;                   // [2][nblk], .x used
  C2 *alpha_slot = ssq_slot + 2 * nblk;  // [2]
  C2 *w_slot = alpha_slot + 2;           // [2][nblk][nb]
  C2 *g_slot = w_slot + 2L * nblk * nb;  // [nblk][nb][nb]
  unsigned gen = 0;
  const C2 zero = qz<C2>(R(0), R(0)), one = qz<C2>(R(1), R(0));

  for (int e = tid; e < rows * nb; e += blockDim.x) {
    const int r = e % rows, c = e / rows;
    S[c * RR + r] = A[(r0 + r) + (long)c * lda];
  }
  __syncthreads();

  const int kmax = min(m, nb);
  for (int k = 0; k < kmax; ++k) {
    const int p = k & 1;
    // (1) |x|^2 of column k below the diagonal
    R acc = 0;
    for (int r = tid; r < rows; r += blockDim.x)
      if (r0 + r > k) {
        const C2 v = S[k * RR + r];
        acc = fma(v.x, v.x, acc);
        acc = fma(v.y, v.y, acc);
      }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (tid == 0) {
      R t = 0;
      for (int q = 0; q < 8; ++q) t += red[q];
      ssq_slot[p * nblk + b] = qz<C2>(t, R(0));
      if (k >= r0 && k < r0 + rows) alpha_slot[p] = S[k * RR + (k - r0)];
    }
    grid_barrier(ctl, nblk, gen);
    if (tid == 0) {
      R ss = 0;
      for (int q = 0; q < nblk; ++q) ss += __ldcg(&ssq_slot[p * nblk + q].x);
      C2 alpha;
      alpha.x = __ldcg(&alpha_slot[p].x);
      alpha.y = __ldcg(&alpha_slot[p].y);
      const R xnorm = sqrt(ss);
      C2 t = zero, scale = zero;
      R beta = alpha.x;
      if (!(xnorm == R(0) && alpha.y == R(0))) {
        // lapy3(re alpha, im alpha, xnorm) (lapack/lapy3.zig)
        const R ax = fabs(alpha.x), ay = fabs(alpha.y);
        const R w = fmax(ax, fmax(ay, xnorm));
        const R hyp = w == R(0) ? R(0)
                                : w * sqrt((ax / w) * (ax / w) + (ay / w) * (ay / w) +
                                           (xnorm / w) * (xnorm / w));
        beta = -copysign(hyp, alpha.x);
        t = qz<C2>((beta - alpha.x) / beta, (-alpha.y) / beta);
        scale = qz_div(one, qz<C2>(alpha.x - beta, alpha.y));
      }
      sc_tau = t;
      sc_scale = scale;
      sc_beta = beta;
      if (b == 0) tau[k] = t;
    }
    __syncthreads();
    const C2 tk = sc_tau, scale = sc_scale;
    const R beta = sc_beta;
    const bool active = !(tk.x == R(0) && tk.y == R(0));
    if (active) {
      for (int r = tid; r < rows; r += blockDim.x)
        if (r0 + r > k) S[k * RR + r] = qz_mul(S[k * RR + r], scale);
      if (tid == 0 && k >= r0 && k < r0 + rows) S[k * RR + (k - r0)] = qz<C2>(beta, R(0));
    }
    __syncthreads();
    if (!active || k == nb - 1) continue;
    // (2) w_j = v^H A(k:, j) with v(k) = 1
    const int ncol = nb - k - 1;
    for (int jj = warp; jj < ncol; jj += 8) {
      const int j = k + 1 + jj;
      C2 a2 = zero;
      for (int r = lane; r < rows; r += 32) {
        const int gi = r0 + r;
        if (gi < k) continue;
        const C2 v = gi == k ? one : S[k * RR + r];
        a2 = qz_add(a2, qz_mul(qz_conj(v), S[j * RR + r]));
      }
      a2 = warp_sum(a2);
      if (lane == 0) w_slot[((long)p * nblk + b) * nb + j] = a2;
    }
    grid_barrier(ctl, nblk, gen);
    for (int jj = tid; jj < ncol; jj += blockDim.x) {
      const int j = k + 1 + jj;
      C2 ws = zero;
      for (int q = 0; q < nblk; ++q) {
        const C2 *src = w_slot + ((long)p * nblk + q) * nb + j;
        ws = qz_add(ws, qz<C2>(__ldcg(&src->x), __ldcg(&src->y)));
      }
      w_s[j] = qz_mul(qz_conj(tk), ws);  // conj(tau) w_j
    }
    __syncthreads();
    const int lr = tid & 127, cph = tid >> 7;
    for (int r = lr; r < rows; r += 128) {
      const int gi = r0 + r;
      if (gi < k) continue;
      const C2 v = gi == k ? one : S[k * RR + r];
      for (int j = k + 1 + cph; j < nb; j += 2) {
        const C2 d = qz_mul(v, w_s[j]);
        C2 &s = S[j * RR + r];
        s = qz<C2>(s.x - d.x, s.y - d.y);
      }
    }
    __syncthreads();
  }

  // G = V^H V (upper part) and T
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e % nb, j = e / nb;
    C2 g = zero;
    if (i <= j)
      for (int r = 0; r < rows; ++r) {
        const int gi = r0 + r;
        const C2 vi = gi > i ? S[i * RR + r] : (gi == i ? one : zero);
        const C2 vj = gi > j ? S[j * RR + r] : (gi == j ? one : zero);
        g = qz_add(g, qz_mul(qz_conj(vi), vj));
      }
    g_slot[(long)b * nb * nb + e] = g;
  }
  grid_barrier(ctl, nblk, gen);
  if (b == 0) {
    C2 *G = reinterpret_cast<C2 *>(zqsm_raw);
    __syncthreads();
    for (int e = tid; e < rows * nb; e += blockDim.x) {
      const int r = e % rows, c = e / rows;
      A[(r0 + r) + (long)c * lda] = S[c * RR + r];
    }
    __syncthreads();
    for (int e = tid; e < nb * nb; e += blockDim.x) {
      C2 g = zero;
      for (int q = 0; q < nblk; ++q) {
        const C2 *src = g_slot + (long)q * nb * nb + e;
        g = qz_add(g, qz<C2>(__ldcg(&src->x), __ldcg(&src->y)));
      }
      G[e] = g;
    }
    __syncthreads();
    C2 *Ts = G + nb * nb;
    for (int e = tid; e < nb * nb; e += blockDim.x) Ts[e] = zero;
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
      const C2 tj = tau[j];
      if (tid < j) {
        C2 acc2 = zero;
        for (int l = tid; l < j; ++l) acc2 = qz_add(acc2, qz_mul(Ts[tid + l * nb], G[l + j * nb]));
        const C2 v = qz_mul(tj, acc2);
        Ts[tid + j * nb] = qz<C2>(-v.x, -v.y);
      }
      if (tid == j) Ts[j + j * nb] = tj;
      __syncthreads();
    }
    for (int e = tid; e < nb * nb; e += blockDim.x) Tout[e] = Ts[e];
    return;
  }
  for (int e = tid; e < rows * nb; e += blockDim.x) {
    const int r = e % rows, c = e / rows;
    A[(r0 + r) + (long)c * lda] = S[c * RR + r];
  }
}

// V (m x ib, ld m): the panel's reflectors with unit diagonal, zero above.
template <typename R, typename C2>
__global__ void zbuild_v_kernel(int m, int ib, const C2 *A, long lda, C2 *V) {
  const long total = (long)m * ib;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % m, j = e / m;
    V[e] = i > j ? A[i + (long)j * lda] : qz<C2>(R(i == j ? 1 : 0), R(0));
  }
}

template <typename R, typename C2>
int zqr_panel(int m, int nb, C2 *A, long lda, C2 *tau, C2 *Tout, C2 *xchg, Control *ctl,
              cudaStream_t s) {
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const size_t limit = di.smem_optin - 8192;
  int nblk = std::min(di.num_sms, ceil_div(m, 8));
  int RR = ceil_div(m, nblk);
  if ((size_t)RR * nb * sizeof(C2) > limit) {
    set_last_error("zgeqrf: panel %d x %d too tall for %d SMs", m, nb, di.num_sms);
    return kErrInvalid;
  }
  nblk = ceil_div(m, RR);
  const size_t smem = std::max((size_t)RR * nb, (size_t)2 * nb * nb) * sizeof(C2);
  ZG_TRY(smem_optin(zqr_panel_kernel<R, C2>, (int)limit));
  ZG_CUDA(cudaMemsetAsync(&ctl->barrier[0], 0, 2 * sizeof(unsigned), s));
  void *args[] = {&m, &nb, &A, &lda, &tau, &Tout, &ctl, &RR, &xchg};
  ZG_LAUNCH(kTagQR, 16.0 * m * nb * nb, 2.0 * sizeof(C2) * m * nb, s,
            ZG_CUDA(cudaLaunchCooperativeKernel((void *)zqr_panel_kernel<R, C2>, dim3(nblk),
                                                dim3(256), args, smem, s)));
  return 0;
}

}  // namespace

template <typename R> int zgeqrf_dev(int m, int n, R *Ar, long lda, R *taur, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  const int k = std::min(m, n);
  if (k <= 0) return 0;
  C2 *A = reinterpret_cast<C2 *>(Ar), *tau = reinterpret_cast<C2 *>(taur);
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const int nb = kZqrNB;
  // workspace: V (m x nb), T (nb x nb), W and T^H W (nb x n), the panel exchange
  const size_t nv = (size_t)m * nb, nt = (size_t)nb * nb, nw = (size_t)nb * n;
  const size_t nx = 2 * (size_t)di.num_sms + 2 + 2 * (size_t)di.num_sms * nb +
                    (size_t)di.num_sms * nb * nb;
  void *w;
  ZG_TRY(workspace(s, kSlotQR, sizeof(C2) * (nv + nt + 2 * nw + nx) + 1024, &w));
  C2 *V = (C2 *)w, *Tm = V + nv, *W = Tm + nt, *W2 = W + nw, *X = W2 + nw;
  const R one[2] = {R(1), R(0)}, zero[2] = {R(0), R(0)}, mone[2] = {R(-1), R(0)};
  for (int i = 0; i < k; i += nb) {
    const int ib = std::min(nb, k - i);
    const int mi = m - i;
    C2 *Ai = A + i + (long)i * lda;
    ZG_TRY((zqr_panel<R, C2>(mi, ib, Ai, lda, tau + i, Tm, X, ctl, s)));
    const int nc = n - i - ib;
    if (nc <= 0) continue;
    C2 *Cb = Ai + (long)ib * lda;
    ZG_LAUNCH(kTagQR, 0, sizeof(C2) * 2.0 * mi * ib, s,
              (zbuild_v_kernel<R, C2><<<std::min(ceil_div((long)mi * ib, 256), 152 * 8), 256, 0, s>>>(
                  mi, ib, Ai, lda, V)));
    // W = V^H C, W2 = T^H W, C -= V W2
    ZG_TRY(zgemm_dev<R>(kConjTrans, kNoTrans, ib, nc, mi, one, (const R *)V, mi, (const R *)Cb,
                        lda, zero, (R *)W, ib, s));
    ZG_TRY(zgemm_dev<R>(kConjTrans, kNoTrans, ib, nc, ib, one, (const R *)Tm, ib, (const R *)W,
                        ib, zero, (R *)W2, ib, s));
    ZG_TRY(zgemm_dev<R>(kNoTrans, kNoTrans, mi, nc, ib, mone, (const R *)V, mi, (const R *)W2,
                        ib, one, (R *)Cb, lda, s));
  }
  return check_status(s, ctl, nullptr);
}

template int zgeqrf_dev<double>(int, int, double *, long, double *, cudaStream_t);
template int zgeqrf_dev<float>(int, int, float *, long, float *, cudaStream_t);

}  // namespace zg
