// kernels_batched.h -- batched small dense solves (one persistent launch).
#pragma once
#include "common.cuh"

namespace zg {

// One persistent CTA of kBatchWarps warps per SM.
constexpr int kBatchWarps = 16, kBatchThreads = 32 * kBatchWarps;

// Warp counts a matrix may be given: 1, 2, 4, 8, 16.
constexpr int kBatchWarpCounts = 5;

// The matrices factored by groups of `warps` warps: order[start .. start+len).
struct BatchQueue {
  int warps, start, len;
};

struct BatchArgs {
  const int *n, *spd;
  const long *a_off, *b_off, *p_off;
  int nrhs, max_ir;
  long vec_off;  // FP32 path: offset of a group's FP32 vector in its scratch
  double *A;
  const double *B;
  double *X, *R;
  int *ipiv, *info, *iters;
};

struct BatchPlan {
  int count = 0, nrhs = 1, fp32 = 0, max_ir = 10, nq = 0, grid = 0, nmax = 0;
  long a_elems = 0, b_elems = 0, p_elems = 0, scratch_per_group = 0;
  double flops = 0;
  void *dev = nullptr;
  int *d_n = nullptr, *d_spd = nullptr;
  long *d_aoff = nullptr, *d_boff = nullptr, *d_poff = nullptr;
  int *d_order = nullptr;
  BatchQueue *d_queues = nullptr;
  float *d_scratch = nullptr;
  double *d_R = nullptr;
  unsigned *d_queue = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  const void *graph_key[6] = {};
};

int batched_classes(int *edges, int cap);
int batched_schedule(int fp32, int *warps, int cap, bool set);
int batched_plan_create(BatchPlan **out, int count, const int *n, const int *spd, int nrhs,
                        int fp32, int max_ir);
void batched_plan_destroy(BatchPlan *p);
int batched_plan_execute(BatchPlan *p, double *A, const double *B, double *X, int *ipiv, int *info,
                         int *iters, cudaStream_t s);
int batched_autotune(int fp32, int nrhs, cudaStream_t s, int *chosen, double *ms_out);
int batched_plan_run_graph(BatchPlan *p, double *A, const double *B, double *X, int *ipiv,
                           int *info, int *iters, cudaStream_t s);

}  // namespace zg
