// fpa_thread_newton.cu -- elementwise mul, div and sqrt with one thread per operation
// (configurations 18 and 19: up to 128 and up to 64 limbs).
//
// A CTA is one warp; each thread runs whole operations (tdiv / tsqrt of
// fpa_thread_newton.cuh) in its columns of the warp's shared-memory workspace and of the
// CTA's operand slab.  Each thread first clears its workspace and slab columns, which sets
// the zero guard limbs the product tiles rely on.  Warps take 32 operations at a time from
// a counter, so a warp that shares its SM sub-partition with another takes fewer.  An
// operation whose extra-limb quotient or root lies within the rounding margin needs the
// exact correction, a full n x n product on one thread: done inline it would keep the other
// 31 threads of its warp waiting, and with a few percent of such operations most warps
// would carry one.  So the first pass only appends their indices to a list (one atomic per
// warp) and writes nothing for them, and a second pass runs the listed operations again
// with the exact correction, 32 at a time.  The counters, the list (4 bytes per operation)
// and the slabs are stream-ordered scratch from the library's memory pool, so concurrent
// calls on different streams never share them.
#include <cuda_runtime.h>
#include "fpa_thread_newton.cuh"
#include "fpa_launch.h"

namespace gfpa {

// One warp per CTA, and at least one CTA per SM requested from the compiler: shared memory
// already limits a div/sqrt kernel to 9 warps per SM, and with this bound ptxas gives it the
// registers it can use there (191-197 instead of 128; measured at 4096 bits: div 5.49 ->
// 5.30 ms, sqrt 6.9 -> 5.7 ms per 2^20 operations).
template <int OP, int N>
__global__ void __launch_bounds__(32, 1) k_tnewton(ElementwiseArgs args, uint32_t *ctl, uint32_t *hard_idx,
                                                uint32_t *slabs, int pass) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x;
  uint32_t *w = smem + lane;                          // this thread's columns
  uint32_t *slab = slabs + (size_t)blockIdx.x * 32 * TSpace<N>::slab + lane;
  for (int j = 0; j < TSpace<N>::words; j++) w[TS * j] = 0u;
  for (int j = 0; j < TSpace<N>::slab; j++) slab[TS * j] = 0u;
  const int n = (int)args.n;
  auto run = [&](uint64_t i, bool exact) -> int {
    const uint64_t off = i * (uint64_t)n;
    if (OP == OP_DIV)
      return tdiv<N>(w, slab, n, args.mode, args.a_exps[i], args.a_limbs + off, args.b_exps[i], args.b_limbs + off,
                     args.r_exps + i, args.r_limbs + off, exact, args.err);
    return tsqrt<N>(w, slab, n, args.mode, args.a_exps[i], args.a_limbs + off, args.r_exps + i, args.r_limbs + off, exact,
                    args.err);
  };
  if (pass == 0) {
    unsigned long long *next = reinterpret_cast<unsigned long long *>(ctl + 2);
    for (;;) {                                        // the same trip count on every thread of the warp
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(next, 32ull);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= args.count) break;
      const uint64_t i = base + lane;
      const int hard = (i < args.count) ? run(i, false) : 0;
      const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hard != 0);
      if (mask) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(ctl, (uint32_t)__popc(mask));
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (hard) hard_idx[b + __popc(mask & ((1u << lane) - 1u))] = (uint32_t)i;
      }
    }
  } else {
    const uint64_t total = (uint64_t)gridDim.x * 32;
    const uint64_t cnt = *ctl;
    for (uint64_t j = (uint64_t)blockIdx.x * 32 + lane; j < cnt; j += total) run(hard_idx[j], true);
  }
}

template <int OP, int N>
static cudaError_t launch_tnewton(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  constexpr size_t smem = (size_t)32 * TSpace<N>::words * sizeof(uint32_t);
  static_assert(smem <= 227 * 1024, "one warp's workspace must fit a CTA");
  auto kern = k_tnewton<OP, N>;
  static int per_sm = 0;
  if (!per_sm) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, 32, smem);
    if (e != cudaSuccess) return e;
    per_sm = blocks > 0 ? blocks : 1;
  }
  const uint64_t need = (args.count + 31) / 32, cap = (uint64_t)sms * (uint64_t)per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  cudaMemPool_t pool;
  if (!gfpa_scratch_pool(&pool)) return cudaErrorMemoryAllocation;
  // control words (hard count, then the 64-bit operation counter), the hard-operation list
  // (count words), then one operand slab per CTA
  const size_t list_bytes = ((size_t)(args.count + 4) * sizeof(uint32_t) + 255) & ~(size_t)255;
  const size_t slab_bytes = (size_t)grid * 32 * TSpace<N>::slab * sizeof(uint32_t);
  uint32_t *list = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync((void **)&list, list_bytes + slab_bytes, pool, stream);
  if (e != cudaSuccess) return e;
  uint32_t *slabs = list + list_bytes / sizeof(uint32_t);
  e = cudaMemsetAsync(list, 0, 4 * sizeof(uint32_t), stream);
  if (e == cudaSuccess) {
    kern<<<grid, 32, smem, stream>>>(args, list, list + 4, slabs, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    kern<<<grid, 32, smem, stream>>>(args, list, list + 4, slabs, 1);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(list, stream);
  return e != cudaSuccess ? e : ef;
}

template <int N>
__global__ void __launch_bounds__(32) k_tmul(ElementwiseArgs args, uint32_t *ctl, uint32_t *hard_idx, uint32_t *slabs,
                                             int pass) {
  using S = MSpace<N>;
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x;
  uint32_t *A = smem + lane;
  uint32_t *slab = slabs + (size_t)blockIdx.x * 32 * S::slab + lane;
  for (int j = 0; j < S::words; j++) A[TS * j] = 0u;
  for (int j = 0; j < S::slab; j++) slab[TS * j] = 0u;
  uint32_t *B = slab + TS * S::SB, *Q = slab + TS * S::GQ;
  const int n = (int)args.n;
  auto run = [&](uint64_t i, bool exact) -> int {
    const uint64_t off = i * (uint64_t)n;
    return tmul_op(A, B, Q, n, args.mode, args.a_exps[i], args.a_limbs + off, args.b_exps[i], args.b_limbs + off,
                   args.r_exps + i, args.r_limbs + off, exact);
  };
  if (pass == 0) {
    unsigned long long *next = reinterpret_cast<unsigned long long *>(ctl + 2);
    for (;;) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(next, 32ull);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= args.count) break;
      const uint64_t i = base + lane;
      const int hard = (i < args.count) ? run(i, false) : 0;
      const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hard != 0);
      if (mask) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(ctl, (uint32_t)__popc(mask));
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (hard) hard_idx[b + __popc(mask & ((1u << lane) - 1u))] = (uint32_t)i;
      }
    }
  } else {
    const uint64_t total = (uint64_t)gridDim.x * 32;
    const uint64_t cnt = *ctl;
    for (uint64_t j = (uint64_t)blockIdx.x * 32 + lane; j < cnt; j += total) run(hard_idx[j], true);
  }
}

template <int N>
static cudaError_t launch_tmul(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  using S = MSpace<N>;
  constexpr size_t smem = (size_t)32 * S::words * sizeof(uint32_t);
  auto kern = k_tmul<N>;
  static int per_sm = 0;
  if (!per_sm) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, 32, smem);
    if (e != cudaSuccess) return e;
    per_sm = blocks > 0 ? blocks : 1;
  }
  const uint64_t need = (args.count + 31) / 32, cap = (uint64_t)sms * (uint64_t)per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  cudaMemPool_t pool;
  if (!gfpa_scratch_pool(&pool)) return cudaErrorMemoryAllocation;
  const size_t list_bytes = ((size_t)(args.count + 4) * sizeof(uint32_t) + 255) & ~(size_t)255;
  const size_t slab_bytes = (size_t)grid * 32 * S::slab * sizeof(uint32_t);
  uint32_t *list = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync((void **)&list, list_bytes + slab_bytes, pool, stream);
  if (e != cudaSuccess) return e;
  uint32_t *slabs = list + list_bytes / sizeof(uint32_t);
  e = cudaMemsetAsync(list, 0, 4 * sizeof(uint32_t), stream);
  if (e == cudaSuccess) {
    kern<<<grid, 32, smem, stream>>>(args, list, list + 4, slabs, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    kern<<<grid, 32, smem, stream>>>(args, list, list + 4, slabs, 1);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(list, stream);
  return e != cudaSuccess ? e : ef;
}

template <int N>
static cudaError_t launch_cfg(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  if ((int)args->n > N) return cudaErrorInvalidValue;
  if ((int)args->n < TSpace<N>::min_limbs) {           // small numbers: the lane-group kernels
    const int c = gfpa_default_cfg(args->n < 4 ? 4 : args->n);
    return c < 0 ? cudaErrorInvalidValue : gfpa_launch(c, op, args, stream, sms);
  }
  switch (op) {
    case OP_MUL: return launch_tmul<N>(*args, stream, sms);
    case OP_DIV: return launch_tnewton<OP_DIV, N>(*args, stream, sms);
    case OP_SQRT: return launch_tnewton<OP_SQRT, N>(*args, stream, sms);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gfpa

extern "C" cudaError_t gfpa_launch_cfg18(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  return gfpa::launch_cfg<128>(op, args, stream, sms);
}
extern "C" cudaError_t gfpa_launch_cfg19(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  return gfpa::launch_cfg<64>(op, args, stream, sms);
}
