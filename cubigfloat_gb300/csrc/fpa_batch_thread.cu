// fpa_batch_thread.cu -- the one-thread class of the batched form: mul, div and sqrt of 8 to
// 128 limbs, one operation per thread (tmul_op / tdiv / tsqrt of fpa_thread_newton.cuh).
//
// A task is up to 32 operations of one (operation, limb count), so the 32 lanes of a warp
// follow one instruction stream; rounding modes and operands differ per lane.  The persistent
// kernel's CTAs are one warp each and take tasks from a device counter.  Operations whose
// first pass defers them (near-halfway products, near-exact quotients and roots) are
// appended to a list that a second launch finishes with the exact correction, 32 at a time,
// as in the elementwise kernels.
//
// Each CTA keeps one workspace (shared memory) and one slab (global memory) sized for the
// largest of the three operations at 128 limbs.  mul lays its operands out differently from
// div and sqrt, so a lane clears its columns whenever the operation it runs changes; that
// restores the zero guard limbs the product tiles rely on.  Limb counts may also change from
// task to task: the staging of every operand clears the 16 guard limbs above it.
#include <cuda_runtime.h>
#include "fpa_thread_newton.cuh"
#include "fpa_batch.h"

namespace gfpa {

constexpr int BN = 128;                                   // largest limb count of the class
constexpr int kWords = TSpace<BN>::words > MSpace<BN>::words ? TSpace<BN>::words : MSpace<BN>::words;
constexpr int kSlab = TSpace<BN>::slab > MSpace<BN>::slab ? TSpace<BN>::slab : MSpace<BN>::slab;

__device__ __forceinline__ void clear_columns(uint32_t *w, uint32_t *slab) {
  for (int j = 0; j < kWords; j++) w[TS * j] = 0u;
  for (int j = 0; j < kSlab; j++) slab[TS * j] = 0u;
}

// Runs operation idx of the batch on this thread; 1 when the first pass defers it.
__device__ __forceinline__ int run_thread_op(const ThreadBatchArgs &A, uint32_t idx, bool exact, uint32_t *w,
                                             uint32_t *slab, int &last_op) {
  const fpa_batch_desc d = A.b.descs[idx];
  const int op = d.op, n = d.limbs;
  if (op != last_op) { clear_columns(w, slab); last_op = op; }
  const uint32_t *a = A.b.a_limbs + d.a_off, *b = A.b.b_limbs + d.b_off;
  uint32_t *r = A.b.r_limbs + d.r_off;
  if (op == OP_MUL)
    return tmul_op(w, slab + TS * MSpace<BN>::SB, slab + TS * MSpace<BN>::GQ, n,
                   d.mode, A.b.a_exps[idx], a, A.b.b_exps[idx], b, A.b.r_exps + idx, r, exact);
  if (op == OP_DIV)
    return tdiv<BN>(w, slab, n, d.mode, A.b.a_exps[idx], a, A.b.b_exps[idx], b, A.b.r_exps + idx, r, exact, A.b.err);
  return tsqrt<BN>(w, slab, n, d.mode, A.b.a_exps[idx], a, A.b.r_exps + idx, r, exact, A.b.err);
}

__global__ void __launch_bounds__(32, 1) k_batch_thread(ThreadBatchArgs A, int pass) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x;
  uint32_t *w = smem + lane;
  uint32_t *slab = A.slabs + (size_t)blockIdx.x * 32 * kSlab + lane;
  int last_op = -1;                                       // forces the first clear
  if (pass == 0) {
    for (;;) {
      uint32_t ti = 0;
      if (lane == 0) ti = atomicAdd(A.b.counter, 1u);
      ti = __shfl_sync(0xFFFFFFFFu, ti, 0);
      if (ti >= A.b.ntasks) break;
      const BatchTask t = A.b.tasks[ti];
      const int hard = lane < t.count ? run_thread_op(A, A.b.order[t.first + lane], false, w, slab, last_op) : 0;
      const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hard != 0);
      if (mask) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(A.hard_count, (uint32_t)__popc(mask));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (hard) A.hard_idx[base + __popc(mask & ((1u << lane) - 1u))] = A.b.order[t.first + lane];
      }
    }
  } else {
    const uint32_t cnt = *A.hard_count;
    for (uint32_t j = blockIdx.x * 32 + lane; j < cnt; j += gridDim.x * 32)
      run_thread_op(A, A.hard_idx[j], true, w, slab, last_op);
  }
}

}  // namespace gfpa

size_t gfpa_batch_thread_smem() { return (size_t)32 * gfpa::kWords * sizeof(uint32_t); }
size_t gfpa_batch_thread_slab_bytes(int grid) { return (size_t)grid * 32 * gfpa::kSlab * sizeof(uint32_t); }

cudaError_t gfpa_batch_thread_prepare(int *blocks_per_sm) {
  const size_t smem = gfpa_batch_thread_smem();
  cudaError_t e = cudaFuncSetAttribute(gfpa::k_batch_thread, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gfpa::k_batch_thread, 32, smem);
}

cudaError_t gfpa_batch_thread_launch(const ThreadBatchArgs *a, int grid, cudaStream_t st) {
  const size_t smem = gfpa_batch_thread_smem();
  cudaError_t e = cudaMemsetAsync(a->hard_count, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  gfpa::k_batch_thread<<<grid, 32, smem, st>>>(*a, 0);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  gfpa::k_batch_thread<<<grid, 32, smem, st>>>(*a, 1);
  return cudaGetLastError();
}
