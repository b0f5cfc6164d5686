// selector.cu -- the learned precision selector: features and a small MLP.
//
// No counterpart in the reference (its path is FP64 only).  Given A, predict
// the lowest factorization precision (BF16 < FP16 < BF16x3 < FP32, FP64 LU as
// the last resort) whose refinement reaches FP64 backward error.
//
// Features (16 floats, all from device kernels): n and scale statistics of A
// computed here, plus the first backward error and the one-step contraction
// of refinement with the cheapest (BF16) factors, which the caller obtains
// from the mixed solver (a few-step estimate of kappa(A) * u_factor).
//
// MLP 16 -> 64 -> 64 -> 5 (ReLU), softmax cross-entropy.  Arithmetic "BF16
// with FP32 accumulation": every operand of a product (inputs, weights,
// activations, back-propagated errors) is rounded to BF16 (round to nearest
// even) and products are summed in FP32; the master weights and the Adam
// state are FP32.  Weight gradients are reduced over the batch in a fixed
// order (deterministic).
#include "common.cuh"
#include "kernels_selector.h"

namespace zg {

namespace {

__device__ __forceinline__ float bf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// ---- features ----------------------------------------------------------------
// Per-row pass: row 1-norm, |a_ii|, off-diagonal row sum, max |a_ij|, row
// sum of squares; per-column 1-norms via atomics; symmetry defect.
__global__ void row_stats_kernel(int n, const double *__restrict__ A, long lda, double *rows,
                                 double *cols, double *sym) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r1 = 0, mx = 0, ss = 0, sd = 0;
  for (int j = 0; j < n; ++j) {
    const double v = A[i + (long)j * lda];
    r1 += fabs(v);
    mx = fmax(mx, fabs(v));
    ss += v * v;
    const double t = A[j + (long)i * lda];
    sd += (v - t) * (v - t);
  }
  const double d = A[i + (long)i * lda];
  rows[5 * i + 0] = r1;
  rows[5 * i + 1] = fabs(d);
  rows[5 * i + 2] = r1 - fabs(d);
  rows[5 * i + 3] = mx;
  rows[5 * i + 4] = ss;
  sym[i] = sd;
  (void)cols;
}

__global__ void col_stats_kernel(int n, const double *__restrict__ A, long lda, double *cols) {
  const int j = blockIdx.x;
  __shared__ double sm[256];
  double c = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) c += fabs(A[i + (long)j * lda]);
  sm[threadIdx.x] = c;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) cols[j] = sm[0];
}

__device__ float lg(double v) { return (float)log10(fmax(v, 1e-300)); }

// One CTA: reduce the row/column statistics into features 0..13.
__global__ void features_finish_kernel(int n, const double *rows, const double *cols,
                                       const double *sym, float *f) {
  __shared__ double red[12][256];
  const int t = threadIdx.x;
  double rmax = 0, rmin = 1e300, cmax = 0, cmin = 1e300, fro = 0, emax = 0, sd = 0;
  double ddmin = 1e300, ddmean = 0, dpos = 0, dmax = 0, dmin = 1e300;
  for (int i = t; i < n; i += blockDim.x) {
    const double *r = rows + 5 * i;
    rmax = fmax(rmax, r[0]);
    rmin = fmin(rmin, r[0]);
    cmax = fmax(cmax, cols[i]);
    cmin = fmin(cmin, cols[i]);
    fro += r[4];
    emax = fmax(emax, r[3]);
    sd += sym[i];
    const double dd = r[1] / fmax(r[2], 1e-300);
    ddmin = fmin(ddmin, dd);
    ddmean += log10(fmax(dd, 1e-300));
    dmax = fmax(dmax, r[1]);
    dmin = fmin(dmin, r[1]);
  }
  double vals[12] = {rmax, -rmin, cmax, -cmin, fro, emax, sd, -ddmin, ddmean, dpos, dmax, -dmin};
  for (int q = 0; q < 12; ++q) red[q][t] = vals[q];
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (t < o)
      for (int q = 0; q < 12; ++q) {
        if (q == 4 || q == 6 || q == 8 || q == 9) red[q][t] += red[q][t + o];
        else red[q][t] = fmax(red[q][t], red[q][t + o]);
      }
    __syncthreads();
  }
  if (t == 0) {
    const double R = red[0][0], r0 = -red[1][0], Cc = red[2][0], c0 = -red[3][0];
    const double F = sqrt(red[4][0]), E = red[5][0], S = sqrt(red[6][0]);
    const double ddm = -red[7][0], ddavg = red[8][0] / n, Dx = red[10][0], Dn = -red[11][0];
    f[0] = (float)log2((double)n);
    f[1] = lg(F / sqrt((double)n));                // overall scale
    f[2] = lg(R / fmax(r0, 1e-300));               // row-scale spread
    f[3] = lg(Cc / fmax(c0, 1e-300));              // column-scale spread
    f[4] = lg(ddm);                                // worst diagonal dominance
    f[5] = (float)ddavg;                           // mean log diagonal dominance
    f[6] = (float)(S / fmax(F, 1e-300));           // asymmetry
    f[7] = lg(E * n / fmax(F, 1e-300));            // entry spread
    f[8] = lg(Dx / fmax(Dn, 1e-300));              // diagonal spread
    f[9] = lg(R / fmax(F, 1e-300));                // ||A||_inf / ||A||_F
    f[10] = lg(Dx / fmax(R, 1e-300));              // diagonal weight
    f[11] = lg(Cc / fmax(R, 1e-300));              // ||A||_1 / ||A||_inf
    f[12] = f[13] = f[14] = f[15] = 0.f;
  }
}

// ---- MLP ---------------------------------------------------------------------
// Parameter layout (FP32): W1[64][16] b1[64] W2[64][64] b2[64] W3[5][64] b3[5].
constexpr int kIn = 16, kH = 64, kOut = 5;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH,
              oW3 = oB2 + kH, oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;

// One thread per sample; weights in shared memory (rounded to BF16 once).
// Writes H1, H2 (post-ReLU, BF16-rounded) and logits Z for the backward pass.
__global__ void mlp_forward_kernel(int B, const float *__restrict__ X, const float *__restrict__ P,
                                   float *H1, float *H2, float *Z) {
  __shared__ float w[kParams];
  for (int e = threadIdx.x; e < kParams; e += blockDim.x) w[e] = bf(P[e]);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  float x[kIn], h1[kH], h2[kH];
#pragma unroll
  for (int k = 0; k < kIn; ++k) x[k] = bf(X[(long)s * kIn + k]);
  for (int o = 0; o < kH; ++o) {
    float a = 0;
#pragma unroll
    for (int k = 0; k < kIn; ++k) a = fmaf(w[oW1 + o * kIn + k], x[k], a);
    h1[o] = bf(fmaxf(a + w[oB1 + o], 0.f));
    H1[(long)s * kH + o] = h1[o];
  }
  for (int o = 0; o < kH; ++o) {
    float a = 0;
    for (int k = 0; k < kH; ++k) a = fmaf(w[oW2 + o * kH + k], h1[k], a);
    h2[o] = bf(fmaxf(a + w[oB2 + o], 0.f));
    H2[(long)s * kH + o] = h2[o];
  }
  for (int o = 0; o < kOut; ++o) {
    float a = 0;
    for (int k = 0; k < kH; ++k) a = fmaf(w[oW3 + o * kH + k], h2[k], a);
    Z[(long)s * kOut + o] = a + w[oB3 + o];
  }
}

// Per-sample errors: dZ = (softmax(Z) - onehot(y)) / B, dH2, dH1 (through the
// ReLUs), each rounded to BF16; also the per-sample loss.
__global__ void mlp_backward_errors_kernel(int B, const float *__restrict__ P,
                                           const float *__restrict__ H1, const float *__restrict__ H2,
                                           const float *__restrict__ Z, const int *__restrict__ y,
                                           float *dZ, float *dH2, float *dH1, float *loss) {
  __shared__ float w[kParams];
  for (int e = threadIdx.x; e < kParams; e += blockDim.x) w[e] = bf(P[e]);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  float z[kOut], m = -INFINITY;
  for (int o = 0; o < kOut; ++o) { z[o] = Z[(long)s * kOut + o]; m = fmaxf(m, z[o]); }
  float den = 0;
  for (int o = 0; o < kOut; ++o) den += expf(z[o] - m);
  const int lab = y[s];
  float dz[kOut];
  for (int o = 0; o < kOut; ++o) {
    const float p = expf(z[o] - m) / den;
    dz[o] = bf((p - (o == lab ? 1.f : 0.f)) / B);
    dZ[(long)s * kOut + o] = dz[o];
  }
  loss[s] = -(z[lab] - m - logf(den));
  float d2[kH];
  for (int k = 0; k < kH; ++k) {
    float a = 0;
    for (int o = 0; o < kOut; ++o) a = fmaf(w[oW3 + o * kH + k], dz[o], a);
    d2[k] = H2[(long)s * kH + k] > 0.f ? bf(a) : 0.f;
    dH2[(long)s * kH + k] = d2[k];
  }
  for (int k = 0; k < kH; ++k) {
    float a = 0;
    for (int o = 0; o < kH; ++o) a = fmaf(w[oW2 + o * kH + k], d2[o], a);
    dH1[(long)s * kH + k] = H1[(long)s * kH + k] > 0.f ? bf(a) : 0.f;
  }
}

// Weight gradients: one thread per parameter, summing over the batch in
// sample order (deterministic).
__global__ void mlp_grad_kernel(int B, const float *__restrict__ X, const float *__restrict__ H1,
                                const float *__restrict__ H2, const float *__restrict__ dZ,
                                const float *__restrict__ dH2, const float *__restrict__ dH1,
                                float *G) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  float acc = 0;
  if (p < oB1) {
    const int o = p / kIn, k = p % kIn;
    for (int s = 0; s < B; ++s) acc = fmaf(dH1[(long)s * kH + o], bf(X[(long)s * kIn + k]), acc);
  } else if (p < oW2) {
    const int o = p - oB1;
    for (int s = 0; s < B; ++s) acc += dH1[(long)s * kH + o];
  } else if (p < oB2) {
    const int o = (p - oW2) / kH, k = (p - oW2) % kH;
    for (int s = 0; s < B; ++s) acc = fmaf(dH2[(long)s * kH + o], H1[(long)s * kH + k], acc);
  } else if (p < oW3) {
    const int o = p - oB2;
    for (int s = 0; s < B; ++s) acc += dH2[(long)s * kH + o];
  } else if (p < oB3) {
    const int o = (p - oW3) / kH, k = (p - oW3) % kH;
    for (int s = 0; s < B; ++s) acc = fmaf(dZ[(long)s * kOut + o], H2[(long)s * kH + k], acc);
  } else {
    const int o = p - oB3;
    for (int s = 0; s < B; ++s) acc += dZ[(long)s * kOut + o];
  }
  G[p] = acc;
}

// Adam (FP32 master weights and moments); step t >= 1.
__global__ void adam_kernel(float *P, const float *G, float *M, float *V, float lr, float b1,
                            float b2, float eps, int t, float wd) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float g = G[p] + wd * P[p];
  M[p] = b1 * M[p] + (1 - b1) * g;
  V[p] = b2 * V[p] + (1 - b2) * g * g;
  const float mh = M[p] / (1 - powf(b1, (float)t)), vh = V[p] / (1 - powf(b2, (float)t));
  P[p] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

int selector_num_params() { return kParams; }

int selector_features(int n, const double *A, long lda, float *f_dev, cudaStream_t s) {
  if (n <= 0) return kErrInvalid;
  void *w;
  ZG_TRY(workspace(s, kSlotSel, sizeof(double) * (size_t)n * 7 + 1024, &w));
  double *rows = (double *)w, *cols = rows + 5L * n, *sym = cols + n;
  ZG_LAUNCH(kTagMLP, 0, 16.0 * n * n, s,
            row_stats_kernel<<<ceil_div(n, 128), 128, 0, s>>>(n, A, lda, rows, cols, sym));
  ZG_LAUNCH(kTagMLP, 0, 8.0 * n * n, s, col_stats_kernel<<<n, 256, 0, s>>>(n, A, lda, cols));
  ZG_LAUNCH(kTagMLP, 0, 0, s, features_finish_kernel<<<1, 256, 0, s>>>(n, rows, cols, sym, f_dev));
  return 0;
}

// Work buffer layout for batch B: H1, H2 (B*64), Z (B*5), dZ, dH2, dH1, loss (B).
size_t mlp_work_floats(int B) { return (size_t)B * (kH * 2 + kOut * 2 + kH * 2 + 1); }

int mlp_forward(int B, const float *X, const float *P, float *logits, float *work, cudaStream_t s) {
  float *H1 = work, *H2 = H1 + (size_t)B * kH, *Z = logits ? logits : H2 + (size_t)B * kH;
  ZG_LAUNCH(kTagMLP, 2.0 * B * (kIn * kH + kH * kH + kH * kOut), 0, s,
            mlp_forward_kernel<<<ceil_div(B, 128), 128, 0, s>>>(B, X, P, H1, H2, Z));
  return 0;
}

int mlp_gradients(int B, const float *X, const int *y, const float *P, float *G, float *loss,
                  float *work, cudaStream_t s) {
  float *H1 = work, *H2 = H1 + (size_t)B * kH, *Z = H2 + (size_t)B * kH;
  float *dZ = Z + (size_t)B * kOut, *dH2 = dZ + (size_t)B * kOut, *dH1 = dH2 + (size_t)B * kH;
  ZG_LAUNCH(kTagMLP, 2.0 * B * (kIn * kH + kH * kH + kH * kOut), 0, s,
            mlp_forward_kernel<<<ceil_div(B, 128), 128, 0, s>>>(B, X, P, H1, H2, Z));
  ZG_LAUNCH(kTagMLP, 2.0 * B * (kH * kH + kH * kOut), 0, s,
            mlp_backward_errors_kernel<<<ceil_div(B, 128), 128, 0, s>>>(B, P, H1, H2, Z, y, dZ, dH2,
                                                                        dH1, loss));
  ZG_LAUNCH(kTagMLP, 2.0 * B * kParams, 0, s,
            mlp_grad_kernel<<<ceil_div(kParams, 128), 128, 0, s>>>(B, X, H1, H2, dZ, dH2, dH1, G));
  return 0;
}

int mlp_adam(float *P, const float *G, float *M, float *V, float lr, float b1, float b2, float eps,
             int t, float wd, cudaStream_t s) {
  ZG_LAUNCH(kTagMLP, 10.0 * kParams, 0, s,
            adam_kernel<<<ceil_div(kParams, 128), 128, 0, s>>>(P, G, M, V, lr, b1, b2, eps, t, wd));
  return 0;
}

}  // namespace zg
