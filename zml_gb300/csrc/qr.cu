// qr.cu -- Householder QR (geqrf) on the GPU, FP64 / FP32.
//
// Replaces zml's lapack/geqrf.zig:18-157 with its panel geqr2.zig:17-59
// (larfg.zig:17-170, larf1f.zig:17-259), the triangular factor larft.zig:18-231
// and the block reflector larfb.zig:20-178 (left, transpose, forward,
// columnwise), with zml's block size nb = 32 (ilaenv.zig:150-155).
//
// Panel: one cooperative launch.  Every CTA keeps a slab of the panel's rows
// in shared memory.  Per column k: (1) each CTA reduces the squares of its
// part of the column below the diagonal, the owner of row k publishes alpha;
// one bounded grid barrier; every CTA sums the partials in the same order and
// forms beta = -sign(alpha) sqrt(alpha^2 + ||x||^2), tau = (beta - alpha)/beta
// and v = x / (alpha - beta) exactly as larfg.zig:55-149 (v(0) = 1 implied);
// (2) the CTAs reduce w = v^T A(k:, k+1:) and, after a second barrier, apply
// A -= tau v w^T to their rows.  After the last column the CTAs reduce the
// Gram matrix G = V^T V and CTA 0 builds T column by column,
// T(0:j, j) = -tau_j T(0:j, 0:j) G(0:j, j), T(j, j) = tau_j -- the same T as
// larft's recursive (Elmroth-Gustavson) construction, in a different order.
// Differences from the reference: the norm is a plain sum of squares (zml's
// nrm2 scales by Blue's thresholds, which matters only beyond 1e+150 or below
// 1e-150), and larfg's rescaling loop for |beta| < safmin/eps is not taken.
//
// Block reflector: C <- (I - V T V^T)^T C = C - V (T^T (V^T C)) as three
// GEMMs (V^T C split along its long K so every SM works).
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace zg {

constexpr int kQrNB = 32;

template <typename T>
__global__ void __launch_bounds__(256) qr_panel_kernel(int m, int nb, T *__restrict__ A, long lda,
                                                       T *__restrict__ tau, T *__restrict__ Tout,
                                                       Control *ctl, int R, T *__restrict__ xchg) {
  extern __shared__ __align__(16) unsigned char qsm_raw[];
  T *S = reinterpret_cast<T *>(qsm_raw);  // S[c * R + r]
  __shared__ T red[8];
  __shared__ T w_s[kQrNB];
  __shared__ T sc[4];  // tau_k, scale, beta, xnorm
  const int b = blockIdx.x, nblk = gridDim.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int r0 = b * R, rows = max(0, min(R, m - r0));
  // exchange regions
  T *ssq_slot = xchg;                                  // [2][nblk]
  T *alpha_slot = ssq_slot + 2 * nblk;                 // [2]
  T *w_slot = alpha_slot + 2;                          // [2][nblk][nb]
  T *g_slot = w_slot + 2L * nblk * nb;                 // [nblk][nb][nb]
  unsigned gen = 0;

  for (int e = tid; e < rows * nb; e += blockDim.x) {
    const int r = e % rows, c = e / rows;
    S[c * R + r] = A[(r0 + r) + (long)c * lda];
  }
  __syncthreads();

  const int kmax = min(m, nb);
  for (int k = 0; k < kmax; ++k) {
    const int p = k & 1;
    // (1) squares of column k below the diagonal
    T acc = 0;
    for (int r = tid; r < rows; r += blockDim.x)
      if (r0 + r > k) acc += S[k * R + r] * S[k * R + r];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (tid == 0) {
      T t = 0;
      for (int q = 0; q < 8; ++q) t += red[q];
      ssq_slot[p * nblk + b] = t;
      if (k >= r0 && k < r0 + rows) alpha_slot[p] = S[k * R + (k - r0)];
    }
    grid_barrier(ctl, nblk, gen);
    if (tid == 0) {
      T ss = 0;
      for (int q = 0; q < nblk; ++q) ss += __ldcg(ssq_slot + p * nblk + q);
      const T alpha = __ldcg(alpha_slot + p);
      const T xnorm = sqrt(ss);
      T t = 0, scale = 0, beta = alpha;
      if (xnorm != T(0)) {
        // lapy3(alpha, 0, xnorm) of larfg.zig:55-64
        const T aa = fabs(alpha), w = fmax(aa, xnorm);
        const T hyp = w * sqrt((aa / w) * (aa / w) + (xnorm / w) * (xnorm / w));
        beta = -copysign(hyp, alpha);
        t = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      sc[0] = t;
      sc[1] = scale;
      sc[2] = beta;
      if (b == 0) tau[k] = t;
    }
    __syncthreads();
    const T tk = sc[0], scale = sc[1], beta = sc[2];
    if (tk != T(0)) {
      for (int r = tid; r < rows; r += blockDim.x)
        if (r0 + r > k) S[k * R + r] *= scale;
      if (tid == 0 && k >= r0 && k < r0 + rows) S[k * R + (k - r0)] = beta;
    }
    __syncthreads();
    if (tk == T(0) || k == nb - 1) continue;
    // (2) w = v^T A(k:, k+1:) with v(k) = 1
    const int ncol = nb - k - 1;
    for (int jj = warp; jj < ncol; jj += 8) {
      const int j = k + 1 + jj;
      T a2 = 0;
      for (int r = lane; r < rows; r += 32) {
        const int gi = r0 + r;
        if (gi < k) continue;
        const T v = gi == k ? T(1) : S[k * R + r];
        a2 += v * S[j * R + r];
      }
      for (int o = 16; o > 0; o >>= 1) a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      if (lane == 0) w_slot[((long)p * nblk + b) * nb + j] = a2;
    }
    grid_barrier(ctl, nblk, gen);
    for (int jj = tid; jj < ncol; jj += blockDim.x) {
      const int j = k + 1 + jj;
      T ws = 0;
      for (int q = 0; q < nblk; ++q) ws += __ldcg(w_slot + ((long)p * nblk + q) * nb + j);
      w_s[j] = ws;
    }
    __syncthreads();
    const int lr = tid & 127, cph = tid >> 7;
    for (int r = lr; r < rows; r += 128) {
      const int gi = r0 + r;
      if (gi < k) continue;
      const T v = gi == k ? T(1) : S[k * R + r];
      for (int j = k + 1 + cph; j < nb; j += 2) S[j * R + r] -= tk * v * w_s[j];
    }
    __syncthreads();
  }

  // Gram matrix of V (unit lower trapezoid) and the triangular factor T
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e % nb, j = e / nb;
    T g = 0;
    if (i <= j)
      for (int r = 0; r < rows; ++r) {
        const int gi = r0 + r;
        const T vi = gi > i ? S[i * R + r] : (gi == i ? T(1) : T(0));
        const T vj = gi > j ? S[j * R + r] : (gi == j ? T(1) : T(0));
        g += vi * vj;
      }
    g_slot[(long)b * nb * nb + e] = g;
  }
  grid_barrier(ctl, nblk, gen);
  if (b == 0) {
    T *G = reinterpret_cast<T *>(qsm_raw);  // the slab is dead in CTA 0 after write-back below
    __syncthreads();
    // CTA 0 writes its slab back first, then reuses the shared memory for G
    for (int e = tid; e < rows * nb; e += blockDim.x) {
      const int r = e % rows, c = e / rows;
      A[(r0 + r) + (long)c * lda] = S[c * R + r];
    }
    __syncthreads();
    for (int e = tid; e < nb * nb; e += blockDim.x) {
      T g = 0;
      for (int q = 0; q < nblk; ++q) g += __ldcg(g_slot + (long)q * nb * nb + e);
      G[e] = g;
    }
    __syncthreads();
    // T column by column: T(0:j, j) = -tau_j T(0:j, 0:j) G(0:j, j)
    T *Ts = G + nb * nb;
    for (int e = tid; e < nb * nb; e += blockDim.x) Ts[e] = 0;
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
      const T tj = tau[j];
      if (tid < j) {
        T acc2 = 0;
        for (int l = tid; l < j; ++l) acc2 += Ts[tid + l * nb] * G[l + j * nb];
        Ts[tid + j * nb] = -tj * acc2;
      }
      if (tid == j) Ts[j + j * nb] = tj;
      __syncthreads();
    }
    for (int e = tid; e < nb * nb; e += blockDim.x) Tout[e] = Ts[e];
    return;
  }
  for (int e = tid; e < rows * nb; e += blockDim.x) {
    const int r = e % rows, c = e / rows;
    A[(r0 + r) + (long)c * lda] = S[c * R + r];
  }
}

// V (m x ib, ld m): the panel's reflectors with unit diagonal, zero above.
template <typename T>
__global__ void build_v_kernel(int m, int ib, const T *A, long lda, T *V) {
  const long total = (long)m * ib;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % m, j = e / m;
    V[e] = i > j ? A[i + (long)j * lda] : (i == j ? T(1) : T(0));
  }
}

template <typename T>
static int qr_panel(int m, int nb, T *A, long lda, T *tau, T *Tout, T *xchg, Control *ctl,
                    cudaStream_t s) {
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const size_t limit = di.smem_optin - 8192;
  int nblk = std::min(di.num_sms, ceil_div(m, 8));
  int R = ceil_div(m, nblk);
  if ((size_t)R * nb * sizeof(T) > limit ||
      (size_t)2 * nb * nb * sizeof(T) > (size_t)R * nb * sizeof(T) + limit) {
    set_last_error("geqrf: panel %d x %d too tall for %d SMs", m, nb, di.num_sms);
    return kErrInvalid;
  }
  nblk = ceil_div(m, R);
  // CTA 0 reuses its shared memory for G and T (2 nb^2) at the end
  const size_t smem = std::max((size_t)R * nb, (size_t)2 * nb * nb) * sizeof(T);
  ZG_TRY(smem_optin(qr_panel_kernel<T>, (int)limit));
  ZG_CUDA(cudaMemsetAsync(&ctl->barrier[0], 0, 2 * sizeof(unsigned), s));
  void *args[] = {&m, &nb, &A, &lda, &tau, &Tout, &ctl, &R, &xchg};
  ZG_LAUNCH(kTagQR, 4.0 * m * nb * nb, 2.0 * sizeof(T) * m * nb, s,
            ZG_CUDA(cudaLaunchCooperativeKernel((void *)qr_panel_kernel<T>, dim3(nblk), dim3(256),
                                                args, smem, s)));
  return 0;
}

template <typename T> int geqrf_dev(int m, int n, T *A, long lda, T *tau, cudaStream_t s) {
  const int k = std::min(m, n);
  if (k <= 0) return 0;
  Control *ctl;
  ZG_TRY(control(s, &ctl));
  DeviceInfo di;
  ZG_TRY(device_info(&di));
  const int nb = kQrNB;
  const int splits = 8;
  // workspace: V (m x nb), T (nb x nb), W and T^T W (nb x n), split-K partials, exchange
  const size_t nv = (size_t)m * nb, nt = (size_t)nb * nb, nw = (size_t)nb * n;
  const size_t nx = 2 * (size_t)di.num_sms + 2 + 2 * (size_t)di.num_sms * nb +
                    (size_t)di.num_sms * nb * nb;
  void *w;
  ZG_TRY(workspace(s, kSlotQR, sizeof(T) * (nv + nt + 2 * nw + splits * nw + nx) + 1024, &w));
  T *V = (T *)w, *Tm = V + nv, *W = Tm + nt, *W2 = W + nw, *P = W2 + nw, *X = P + splits * nw;
  for (int i = 0; i < k; i += nb) {
    const int ib = std::min(nb, k - i);
    const int mi = m - i;
    T *Ai = A + i + (long)i * lda;
    ZG_TRY(qr_panel<T>(mi, ib, Ai, lda, tau + i, Tm, X, ctl, s));
    const int nc = n - i - ib;
    if (nc <= 0) continue;
    T *C = Ai + (long)ib * lda;
    ZG_LAUNCH(kTagQR, 0, sizeof(T) * 2.0 * mi * ib, s,
              build_v_kernel<T><<<std::min(ceil_div((long)mi * ib, 256), 152 * 8), 256, 0, s>>>(
                  mi, ib, Ai, lda, V));
    // W = V^T C (ib x nc), long K = mi split over the SMs
    ZG_TRY(gemm_simt_splitk<T>(kTrans, kNoTrans, ib, nc, mi, T(1), V, mi, C, lda, T(0), W, ib,
                               splits, P, s));
    // W2 = T^T W
    ZG_TRY(gemm_simt<T>(kTrans, kNoTrans, ib, nc, ib, T(1), Tm, ib, W, ib, T(0), W2, ib, 0, s));
    // C -= V W2
    ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, mi, nc, ib, T(-1), V, mi, W2, ib, T(1), C, lda, 0, s));
  }
  return check_status(s, ctl, nullptr);
}

template int geqrf_dev<double>(int, int, double *, long, double *, cudaStream_t);
template int geqrf_dev<float>(int, int, float *, long, float *, cudaStream_t);

// ---------------------------------------------------------------------------
// orgqr: the explicit first n columns of Q = H(0) H(1) ... H(k-1) (zml's
// lapack/orgqr.zig:18-194 with org2r.zig:18-102).  The reflectors are copied
// out of A, A's m x n block is set to the identity and the nb-blocks of
// reflectors are applied last to first as block reflectors from the left,
// C <- (I - V T V^T) C on the rows and columns the block touches (columns to
// the left of a block still hold identity columns that H leaves unchanged).
// T comes from the block's Gram matrix G = V^T V:
// T(0:j, j) = -tau_j T(0:j, 0:j) G(0:j, j), T(j, j) = tau_j (the T of
// larft.zig).  Unlike the reference there is no unblocked tail (org2r for the
// last nx = 128 columns): every block goes through the same three GEMMs.

// One CTA: T (ib x ib, ld ib, upper) from G (ib x ib, ld ib) and tau.
template <typename T>
__global__ void larft_gram_kernel(int ib, const T *__restrict__ G, const T *__restrict__ tau,
                                  T *__restrict__ Tm) {
  __shared__ T sT[kQrNB * kQrNB];
  __shared__ T sG[kQrNB * kQrNB];
  for (int e = threadIdx.x; e < ib * ib; e += blockDim.x) {
    sG[e] = G[e];
    sT[e] = T(0);
  }
  __syncthreads();
  for (int j = 0; j < ib; ++j) {
    const T tj = tau[j];
    T acc = T(0);
    const int r = threadIdx.x;
    if (r < j)
      for (int c = r; c < j; ++c) acc += sT[r + c * ib] * sG[c + j * ib];
    __syncthreads();
    if (r < j) sT[r + j * ib] = -tj * acc;
    if (r == j) sT[j + j * ib] = tj;
    __syncthreads();
  }
  for (int e = threadIdx.x; e < ib * ib; e += blockDim.x) Tm[e] = sT[e];
}

// A (m x n) <- the first n columns of the identity.
template <typename T> __global__ void set_identity_kernel(int m, int n, T *A, long lda) {
  const long total = (long)m * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % m, j = e / m;
    A[i + (long)j * lda] = i == j ? T(1) : T(0);
  }
}

template <typename T>
int orgqr_dev(int m, int n, int k, T *A, long lda, const T *tau, cudaStream_t s) {
  if (n <= 0) return 0;
  const int nb = kQrNB, splits = 8;
  // workspace: all k reflectors (m x k), G and T (nb x nb), W and T W (nb x n), split-K partials
  const size_t nv = (size_t)m * std::max(k, 1), nt = (size_t)nb * nb, nw = (size_t)nb * n;
  void *w;
  ZG_TRY(workspace(s, kSlotQR, sizeof(T) * (nv + 2 * nt + 2 * nw + splits * std::max(nw, nt)) + 1024,
                   &w));
  T *V = (T *)w, *G = V + nv, *Tm = G + nt, *W = Tm + nt, *W2 = W + nw, *P = W2 + nw;
  const int grid = 152 * 8;
  if (k > 0)
    ZG_LAUNCH(kTagQR, 0, sizeof(T) * 2.0 * m * k, s,
              build_v_kernel<T><<<(int)std::min<long>(ceil_div((long)m * k, 256), grid), 256, 0, s>>>(
                  m, k, A, lda, V));
  ZG_LAUNCH(kTagQR, 0, sizeof(T) * 1.0 * m * n, s,
            set_identity_kernel<T><<<(int)std::min<long>(ceil_div((long)m * n, 256), grid), 256, 0, s>>>(
                m, n, A, lda));
  const int last = k > 0 ? ((k - 1) / nb) * nb : -1;
  for (int i = last; i >= 0; i -= nb) {
    const int ib = std::min(nb, k - i), mi = m - i, nc = n - i;
    // V block: rows i.. of reflectors i..i+ib (unit diagonal at row i + j)
    const T *Vi = V + i + (long)i * m;
    T *C = A + i + (long)i * lda;
    ZG_TRY(gemm_simt_splitk<T>(kTrans, kNoTrans, ib, ib, mi, T(1), Vi, m, Vi, m, T(0), G, ib,
                               splits, P, s));
    ZG_LAUNCH(kTagQR, 0, 0, s, larft_gram_kernel<T><<<1, 64, 0, s>>>(ib, G, tau + i, Tm));
    // C <- C - V (T (V^T C))
    ZG_TRY(gemm_simt_splitk<T>(kTrans, kNoTrans, ib, nc, mi, T(1), Vi, m, C, lda, T(0), W, ib,
                               splits, P, s));
    ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, ib, nc, ib, T(1), Tm, ib, W, ib, T(0), W2, ib, 0, s));
    ZG_TRY(gemm_simt<T>(kNoTrans, kNoTrans, mi, nc, ib, T(-1), Vi, m, W2, ib, T(1), C, lda, 0, s));
  }
  ZG_CUDA(cudaGetLastError());
  return 0;
}

template int orgqr_dev<double>(int, int, int, double *, long, const double *, cudaStream_t);
template int orgqr_dev<float>(int, int, int, float *, long, const float *, cudaStream_t);

}  // namespace zg
