// kernels_tc.h -- launchers of the tensor-core (tcgen05) kernels.
#pragma once
#include "common.cuh"

namespace zg {

// C (fp32, col-major, ldc) <- alpha * A * B^T + beta * C on tcgen05.
// A: M x K, B: N x K, 16-bit K-major (row stride lda / ldb elements, a
// multiple of 8); ab_type 0 = fp16, 1 = bf16.  `status` (device) collects
// timeout bits of the kernel's bounded waits; may be null.  tri = 1 computes
// only the 128 x 128 tiles on or below the diagonal (the SYRK form; the upper
// part of diagonal tiles is written too).
int gemm_tc(int M, int N, int K, float alpha, const void *A, long lda, const void *B, long ldb,
            float beta, float *C, long ldc, int ab_type, unsigned *status, cudaStream_t s,
            int tri = 0);

}  // namespace zg
