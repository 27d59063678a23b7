// fpa_batch_kernels.cu -- persistent kernel of one register class of the batched form
// (compiled once per class, GFPA_BATCH_CLASS = 0, 1, 2).
//
// Each CTA repeatedly takes the next task of its class from a device counter and runs it
// with all its warps; every lane group executes the same per-operation device code as the
// elementwise kernels, so batched results are bit-identical to them.
#include <cuda_runtime.h>
#include "fpa_ops.cuh"
#include "fpa_batch.h"

#ifndef GFPA_BATCH_CLASS
#define GFPA_BATCH_CLASS 0
#endif

namespace gfpa {

// One task body per (configuration, operation), out of line so the class kernel is a
// small dispatcher over separately compiled bodies.
template <int OP, int G, int K, int R>
__device__ __noinline__ void run_task(const BatchArgs A, uint32_t first, uint32_t count, uint32_t *smem) {
  Grp<G> g;
  constexpr int gpw = 32 / G;
  constexpr int words = OpWords<OP, G, K, R>::aligned();
  const int warp = (int)(threadIdx.x >> 5), nwarps = (int)(blockDim.x >> 5);
  const int gi = (int)((threadIdx.x & 31u) / G);
  uint32_t *ws = smem + (size_t)warp * A.warp_words + gi * words;
  const int stride = nwarps * gpw;
  // div / sqrt: every thread of the CTA (all on this task) runs the same number of
  // iterations and meets a CTA barrier after each, so the warps share the fetched code of
  // each phase (as in the elementwise kernel).  The barrier has one call site, after the
  // per-group branch: a warp's lanes must all reach the same barrier instruction.
  constexpr bool lockstep = OP == OP_DIV || OP == OP_SQRT;
  const uint32_t iters = lockstep ? (count + stride - 1) / stride : 0u;
  for (uint32_t it = 0, j = (uint32_t)(warp * gpw + gi); lockstep ? it < iters : j < count; it++, j += stride) {
    if (j < count) {
      const uint32_t idx = A.order[first + j];
      const fpa_batch_desc d = A.descs[idx];
      const int n = d.limbs, mode = d.mode;
      if (OP == OP_ADD || OP == OP_SUB)
        op_addsub<G, K, R>(g, ws, n, mode, OP == OP_SUB, A.a_exps[idx], A.a_limbs + d.a_off, A.b_exps[idx],
                        A.b_limbs + d.b_off, A.r_exps + idx, A.r_limbs + d.r_off);
      else if (OP == OP_MUL)
        op_mul<G, K, R>(g, ws, n, mode, A.a_exps[idx], A.a_limbs + d.a_off, A.b_exps[idx], A.b_limbs + d.b_off,
                     A.r_exps + idx, A.r_limbs + d.r_off);
      else if (OP == OP_DIV)
        op_div<G, K, R>(g, ws, n, mode, A.a_exps[idx], A.a_limbs + d.a_off, A.b_exps[idx], A.b_limbs + d.b_off,
                     A.r_exps + idx, A.r_limbs + d.r_off, A.err);
      else
        op_sqrt<G, K, R>(g, ws, n, mode, A.a_exps[idx], A.a_limbs + d.a_off, A.r_exps + idx, A.r_limbs + d.r_off, A.err);
      g.sync();
    }
    if (lockstep) __syncthreads();
  }
}

#define GFPA_TASK_OP(CFG, GG, KK, RR, OPV)                                       \
  case CFG * 5 + OPV:                                                            \
    if constexpr (gfpa_class_of(CFG, OPV) == CLS) run_task<OPV, GG, KK, RR>(A, t.first, t.count, smem); \
    break;
#define GFPA_TASK(CFG, GG, KK, RR)                                               \
  GFPA_TASK_OP(CFG, GG, KK, RR, OP_ADD) GFPA_TASK_OP(CFG, GG, KK, RR, OP_SUB)    \
  GFPA_TASK_OP(CFG, GG, KK, RR, OP_MUL) GFPA_TASK_OP(CFG, GG, KK, RR, OP_DIV)    \
  GFPA_TASK_OP(CFG, GG, KK, RR, OP_SQRT)
#define GFPA_TASKS_TILE4                                                         \
  GFPA_TASK(0, 4, 2, 1) GFPA_TASK(1, 8, 2, 1) GFPA_TASK(2, 8, 4, 1) GFPA_TASK(3, 16, 4, 1) \
  GFPA_TASK(4, 32, 4, 1) GFPA_TASK(10, 8, 4, 2) GFPA_TASK(11, 8, 4, 4) GFPA_TASK(12, 16, 4, 2) \
  GFPA_TASK(15, 4, 4, 8)

template <int CLS>
struct ClassShape {
  static constexpr int threads = CLS == 0 ? 256 : 128;
  static constexpr int min_blocks = CLS == 0 ? 4 : (CLS == 1 ? 4 : 2);
};

template <int CLS>
__global__ void __launch_bounds__(ClassShape<CLS>::threads, ClassShape<CLS>::min_blocks) k_batch(BatchArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint32_t s_task;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(A.counter, 1u);
    __syncthreads();
    const uint32_t ti = s_task;
    __syncthreads();
    if (ti >= A.ntasks) break;
    const BatchTask t = A.tasks[ti];
    if constexpr (CLS == 0) {
      switch (t.key) { GFPA_TASKS_TILE4 default: break; }
    } else if constexpr (CLS == 1) {
      switch (t.key) {
        GFPA_TASKS_TILE4 GFPA_TASK(5, 32, 8, 1) GFPA_TASK(7, 16, 8, 1) GFPA_TASK(13, 8, 8, 4) GFPA_TASK(14, 16, 8, 2)
        default: break;
      }
    } else {
      switch (t.key) { GFPA_TASK(6, 32, 16, 1) GFPA_TASK(8, 8, 16, 1) GFPA_TASK(9, 16, 16, 1) default: break; }
    }
  }
}

}  // namespace gfpa

#define GFPA_CAT2(a, b) a##b
#define GFPA_CAT(a, b) GFPA_CAT2(a, b)

extern "C" cudaError_t GFPA_CAT(gfpa_batch_prepare, GFPA_BATCH_CLASS)(size_t smem, int *blocks_per_sm) {
  auto k = gfpa::k_batch<GFPA_BATCH_CLASS>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k,
                                                       gfpa::ClassShape<GFPA_BATCH_CLASS>::threads, smem);
}

extern "C" cudaError_t GFPA_CAT(gfpa_batch_launch, GFPA_BATCH_CLASS)(const BatchArgs *a, int grid, size_t smem,
                                                                      cudaStream_t st) {
  gfpa::k_batch<GFPA_BATCH_CLASS><<<grid, gfpa::ClassShape<GFPA_BATCH_CLASS>::threads, smem, st>>>(*a);
  return cudaGetLastError();
}
