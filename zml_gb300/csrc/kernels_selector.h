// kernels_selector.h -- features and MLP kernels of the precision selector.
#pragma once
#include "common.cuh"

namespace zg {

int selector_num_params();
// Structural features f[0..11] of the n x n FP64 matrix A into f_dev (16
// floats; f[12..15] are left for the refinement probe).
int selector_features(int n, const double *A, long lda, float *f_dev, cudaStream_t s);
size_t mlp_work_floats(int B);
int mlp_forward(int B, const float *X, const float *P, float *logits, float *work, cudaStream_t s);
int mlp_gradients(int B, const float *X, const int *y, const float *P, float *G, float *loss,
                  float *work, cudaStream_t s);
int mlp_adam(float *P, const float *G, float *M, float *V, float lr, float b1, float b2, float eps,
             int t, float wd, cudaStream_t s);

}  // namespace zg
