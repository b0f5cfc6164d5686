// gemm_tc.cu -- BF16 / FP16 tensor-core GEMM with FP32 accumulation (tcgen05).
//
// The low-precision trailing update of the mixed-precision LU and Cholesky
// (the form of getrf.zig:125 / potrf.zig:197 whose operands are rounded to
// 16 bits):
//
//     C (fp32, column-major) <- alpha * A * B^T + beta * C
//     A: M x K, B: N x K, both 16-bit and K-major (row stride ld >= K,
//     a multiple of 8 elements).
//
// One CTA computes a 128 x BN tile.  Warp 0 (one lane) streams 128 x 64 K
// slices of A and B into a STAGES-deep shared-memory ring (2 or 3 stages, so
// that two CTAs share an SM) with TMA (128-byte swizzle); warp 1 (one lane)
// issues tcgen05.mma (M=128, N=BN, K=16) into a TMEM accumulator and releases
// each stage with tcgen05.commit; all eight warps load their slice of the old
// C while the MMAs run, then drain TMEM (warps w and w+4 share accumulator
// rows 32(w%4)..32(w%4)+31 and split the columns) and apply the epilogue to C
// with column-major stores.
#include <cudaTypedefs.h>

#include "common.cuh"
#include "kernels.h"
#include "kernels_tc.h"
#include "tc_common.cuh"

namespace zg {

namespace {

constexpr int kBM = 128, kBK = 64;

template <int BN, int STAGES> struct TileCfg {
  static constexpr int a_bytes = kBM * kBK * 2;
  static constexpr int b_bytes = BN * kBK * 2;
  static constexpr int stage_bytes = a_bytes + b_bytes;
  static constexpr int smem_bytes = STAGES * stage_bytes + 1024 /*align*/ + 256 /*barriers*/;
  static_assert(2 * STAGES * 8 + 8 + 4 + 3 * 4 <= 256, "barrier area");
  static constexpr uint32_t tmem_cols = BN < 32 ? 32 : BN;
};

// 256 threads: warp 0 = TMA producer, warp 1 = MMA issuer; all eight warps
// drain TMEM, warps w and w+4 sharing lane quarter w%4 and splitting columns.
template <int BN, int STAGES>
__global__ void __launch_bounds__(256)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   int M, int N, int K, float alpha, float beta, float *__restrict__ C, long ldc,
                   int ab_type, unsigned *status, int tri) {
  using Cfg = TileCfg<BN, STAGES>;
  // SYRK form: tiles strictly above the diagonal are not needed
  if (tri && (int)(blockIdx.y * BN) >= (int)(blockIdx.x * kBM + kBM)) return;
  constexpr int kStages = STAGES;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * Cfg::stage_bytes);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  // stages the producer issued and the MMA issuer consumed, and whether any
  // wait of the CTA ran out (then the exit drains what is still in flight)
  int *issued = reinterpret_cast<int *>(tmem_slot + 1), *consumed = issued + 1, *bad = issued + 2;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int KT = (K + kBK - 1) / kBK;

  if (warp == 0 && lane == 0) {
    *issued = *consumed = *bad = 0;
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(done, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, Cfg::tmem_cols);
    tc::tmem_relinquish();
  }
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0 && lane == 0) {  // TMA producer
    int kt = 0;
    for (; kt < KT && ok; ++kt) {
      const int s = kt % kStages, round = kt / kStages;
      if (round > 0) ok = tc::mbar_wait(&empty[s], (round - 1) & 1, status);
      if (!ok) break;
      unsigned char *sa = smem + s * Cfg::stage_bytes;
      unsigned char *sb = sa + Cfg::a_bytes;
      tc::mbar_expect_tx(&full[s], Cfg::stage_bytes);
      tc::tma_load_2d(sa, &tmA, &full[s], kt * kBK, m0);
      tc::tma_load_2d(sb, &tmB, &full[s], kt * kBK, n0);
    }
    *issued = kt;
    if (!ok) *bad = 1;
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    const uint32_t idesc = tc::idesc_f16(kBM, BN, ab_type);
    int kt = 0;
    for (; kt < KT && ok; ++kt) {
      const int s = kt % kStages, round = kt / kStages;
      ok = tc::mbar_wait(&full[s], round & 1, status);
      if (!ok) break;
      tc::tc_fence_after();
      const unsigned char *sa = smem + s * Cfg::stage_bytes;
      const unsigned char *sb = sa + Cfg::a_bytes;
      const uint64_t adesc = tc::sdesc_sw128(sa), bdesc = tc::sdesc_sw128(sb);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk)  // +32 bytes along K per step
        tc::mma_f16(tmem, adesc + 2 * kk, bdesc + 2 * kk, idesc, (kt | kk) != 0);
      tc::mma_commit(&empty[s]);
    }
    *consumed = kt;
    if (!ok) *bad = 1;
    tc::mma_commit(done);
  }
  __syncwarp();

  // Epilogue.  Every warp first loads its part of the old C (beta != 0) into
  // registers, so those loads overlap the MMAs still in flight, then waits
  // for the accumulator and drains its 32 rows.  The old C is read through
  // L2 only (ld.global.cg): with the factorization's two streams, kernels of
  // the other stream may have rewritten C since this SM last cached it.
  const int quarter = warp & 3, half = warp >> 2;
  const int row = m0 + quarter * 32 + lane;
  constexpr int kCols = BN / 2, kChunks = kCols / 32;
  float old[kChunks][32];
  const bool pre = beta != 0.f && row < M && K > 0;
#pragma unroll
  for (int q = 0; q < kChunks; ++q) {
    const int c = half * kCols + q * 32;
    const float *base = C + row + (long)(n0 + c) * ldc;
    const int nc = min(32, N - (n0 + c));
#pragma unroll
    for (int j = 0; j < 32; ++j) old[q][j] = (pre && j < nc) ? __ldcg(base + (long)j * ldc) : 0.f;
  }
  const bool have = tc::mbar_wait(done, 0, status);
  if (!have) *bad = 1;
  tc::tc_fence_after();
  if (have && K > 0) {
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
#pragma unroll
    for (int q = 0; q < kChunks; ++q) {
      const int c = half * kCols + q * 32;
      float v[32];
      tc::tmem_ld32(trow + c, v);
      if (row < M) {
        float *base = C + row + (long)(n0 + c) * ldc;
        const int nc = min(32, N - (n0 + c));
        if (beta != 0.f) {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j < nc) __stcs(base + (long)j * ldc, fmaf(alpha, v[j], beta * old[q][j]));
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j < nc) __stcs(base + (long)j * ldc, alpha * v[j]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  // after a wait ran out: wait (bounded again) for the TMA copies issued but
  // never consumed and for the MMAs behind the final commit, so that neither
  // lands in shared memory or TMEM after the CTA has released them
  if (*bad && threadIdx.x == 0) {
    for (int kt = *consumed; kt < *issued; ++kt)
      tc::mbar_wait(&full[kt % kStages], (kt / kStages) & 1, status);
    tc::mbar_wait(done, 0, status);
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, Cfg::tmem_cols);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// K-major 16-bit operand: rows x K elements, row stride ld elements.
int make_map(CUtensorMap *m, const void *base, int rows, int K, long ld, int box_rows) {
  auto enc = get_encode();
  if (!enc) {
    set_last_error("cuTensorMapEncodeTiled unavailable");
    return kErrCuda;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 2) % 16) {
    set_last_error("gemm_tc: operand base/stride not 16-byte aligned");
    return kErrInvalid;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), gdim, gstride,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return kErrCuda;
  }
  return 0;
}

template <int BN, int STAGES>
int launch(int M, int N, int K, float alpha, const void *A, long lda, const void *B, long ldb,
           float beta, float *C, long ldc, int ab_type, unsigned *status, int tri, cudaStream_t s) {
  CUtensorMap ta, tb;
  ZG_TRY(make_map(&ta, A, M, K, lda, kBM));
  ZG_TRY(make_map(&tb, B, N, K, ldb, BN));
  using Cfg = TileCfg<BN, STAGES>;
  ZG_TRY(smem_optin(gemm_tc_kernel<BN, STAGES>, Cfg::smem_bytes));
  dim3 grid(ceil_div(M, kBM), ceil_div(N, BN));
  ZG_LAUNCH(kTagGemmTC, 2.0 * M * N * K, 2.0 * ((double)M + N) * K + (beta != 0.f ? 8.0 : 4.0) * M * N, s, gemm_tc_kernel<BN, STAGES><<<grid, 256, Cfg::smem_bytes, s>>>(ta, tb, M, N, K, alpha, beta, C,
                                                               ldc, ab_type, status, tri));
  ZG_CUDA(cudaGetLastError());
  return 0;
}

}  // namespace

int gemm_tc(int M, int N, int K, float alpha, const void *A, long lda, const void *B, long ldb,
            float beta, float *C, long ldc, int ab_type, unsigned *status, cudaStream_t s,
            int tri) {
  if (M <= 0 || N <= 0) return 0;
  if (K <= 0) return scale_dev<float>(M, N, beta, C, ldc, s);
  if (ab_type != 0 && ab_type != 1) return kErrInvalid;
  // short K: two stages; longer K (768 for the split-BF16 updates): three.
  // Either way two CTAs share an SM (128 registers x 256 threads each), so
  // one CTA's epilogue overlaps the other's main loop.
  if (K <= 256)
    return launch<128, 2>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ab_type, status, tri, s);
  return launch<128, 3>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ab_type, status, tri, s);
}

}  // namespace zg
