// fpa_thread_kernels.cu -- add/sub with one thread per operation, for small precisions.
//
// At a few hundred to a couple of thousand bits add/sub move far more bytes than they
// compute, so their bound is HBM.  A lane group per operation spends too many instructions
// per byte there; here each thread runs one whole operation (the same device code as the
// lane-group kernels, with a group of one lane) and each warp moves the limbs of its 32
// consecutive operations through shared memory with coalesced loads and stores.
//
// Configurations 16 and 17 (capacity 32 and 64 limbs) are add/sub only.
#include <cuda_runtime.h>
#include "fpa_ops.cuh"
#include "fpa_launch.h"

namespace gfpa {

// Words of one warp's shared slice: two buffers, each holding operand rows a and b of `row`
// words for 32 operations (the result is written over a's row), the add/sub integer of
// every thread (NMAX + 5 words: NMAX + 3 used, odd stride), and the 32 result exponents.
template <int NMAX>
struct ThreadSpace {
  __host__ __device__ static constexpr int xstride() { return NMAX + 5; }
  __host__ __device__ static int row(int n) { return n | 1; }   // odd: conflict-free rows
  __host__ __device__ static int buffer(int n) { return 2 * 32 * row(n); }
  __host__ __device__ static int words(int n) { return 2 * buffer(n) + 32 * xstride() + 32; }
};

// Asynchronous copy of chunk `c` (32 operations from index 32c) into buffer `buf`: word w
// of the chunk's contiguous limbs is limb w % n of operation w / n.
__device__ __forceinline__ void stage_chunk(uint32_t *buf, int row, const ElementwiseArgs &args, uint64_t c, int lane) {
  const int n = (int)args.n;
  const uint64_t base = c * 32;
  const int cnt = (int)min((uint64_t)32, args.count - base);
  const int words = cnt * n;
  const uint32_t *ga = args.a_limbs + base * n, *gb = args.b_limbs + base * n;
  uint32_t *sa = buf, *sb = buf + 32 * row;
  int op = lane / n, limb = lane % n;
  for (int w = lane; w < words; w += 32) {
    cp_async4(sa + op * row + limb, ga + w);
    cp_async4(sb + op * row + limb, gb + w);
    limb += 32;
    while (limb >= n) { limb -= n; op++; }
  }
}

template <int OP, int NMAX>
__global__ void __launch_bounds__(128, 4) k_addsub_thread(ElementwiseArgs args, int warp_words) {
  extern __shared__ __align__(16) uint32_t smem[];
  Grp<1> g;
  const int n = (int)args.n, row = ThreadSpace<NMAX>::row(n), bw = ThreadSpace<NMAX>::buffer(n);
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
  uint32_t *ws = smem + (size_t)warp * warp_words;
  uint32_t *X = ws + 2 * bw + lane * ThreadSpace<NMAX>::xstride();
  uint32_t *rexp = ws + 2 * bw + 32 * ThreadSpace<NMAX>::xstride();
  const uint64_t nchunks = (args.count + 31) / 32;
  const uint64_t stride = (uint64_t)gridDim.x * (blockDim.x >> 5);
  uint64_t c = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  uint32_t ae = 0, be = 0;
  if (c < nchunks) {
    stage_chunk(ws, row, args, c, lane);
    if (c * 32 + lane < args.count) { ae = args.a_exps[c * 32 + lane]; be = args.b_exps[c * 32 + lane]; }
  }
  cp_async_commit();
  int cur = 0;
  for (; c < nchunks; c += stride) {
    const uint64_t nx = c + stride;
    uint32_t nae = 0, nbe = 0;
    if (nx < nchunks) {
      stage_chunk(ws + (cur ^ 1) * bw, row, args, nx, lane);
      if (nx * 32 + lane < args.count) { nae = args.a_exps[nx * 32 + lane]; nbe = args.b_exps[nx * 32 + lane]; }
    }
    cp_async_commit();
    cp_async_wait<1>();                            // this chunk's operands have landed
    __syncwarp();
    const uint64_t base = c * 32;
    const int cnt = (int)min((uint64_t)32, args.count - base);
    uint32_t *sa = ws + cur * bw, *sb = sa + 32 * row;
    if (lane < cnt) {
      uint32_t *ra = sa + lane * row;              // the result overwrites a's row
      op_addsub_staged<1>(g, X, n, args.mode, OP == OP_SUB, ae, ra, be, sb + lane * row, rexp + lane, ra);
      args.r_exps[base + lane] = rexp[lane];
    }
    __syncwarp();
    // coalesced copy-out of the operations that produced limbs (class results leave the
    // destination limbs untouched)
    {
      uint32_t *gr = args.r_limbs + base * n;
      int op = lane / n, limb = lane % n;
      for (int w = lane; w < cnt * n; w += 32) {
        if (rexp[op] > CLS_SNAN) gr[w] = sa[op * row + limb];
        limb += 32;
        while (limb >= n) { limb -= n; op++; }
      }
    }
    __syncwarp();                                  // the buffer is refilled two chunks on
    ae = nae; be = nbe; cur ^= 1;
  }
  cp_async_wait<0>();
}

template <int OP, int NMAX>
static cudaError_t launch_thread(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  if ((int)args.n > NMAX) return cudaErrorInvalidValue;
  const int n = (int)args.n;
  const int ww = (ThreadSpace<NMAX>::words(n) + 3) & ~3;
  const int warps = 4;
  const size_t smem = (size_t)warps * ww * 4;
  auto kern = k_addsub_thread<OP, NMAX>;
  // the attribute is raised to the largest slice (n = NMAX) once; CTAs per SM per n cached
  static int configured = 0;
  static int per_sm_of[NMAX + 1] = {0};
  cudaError_t e;
  if (!configured) {
    const size_t most = (size_t)warps * ((ThreadSpace<NMAX>::words(NMAX) + 3) & ~3) * 4;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most)) != cudaSuccess)
      return e;
    configured = 1;
  }
  if (per_sm_of[n] == 0) {
    int b = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 32 * warps, smem)) != cudaSuccess) return e;
    per_sm_of[n] = b < 1 ? 1 : b;
  }
  const int per_sm = per_sm_of[n];
  const uint64_t need = (args.count + 32 * warps - 1) / (32 * warps);
  const uint64_t cap = (uint64_t)sms * per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  kern<<<grid, 32 * warps, smem, stream>>>(args, ww);
  return cudaGetLastError();
}

}  // namespace gfpa

#define GFPA_THREAD_CFG(NAME, NMAX)                                                        \
  extern "C" cudaError_t NAME(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) { \
    switch (op) {                                                                          \
      case gfpa::OP_ADD: return gfpa::launch_thread<gfpa::OP_ADD, NMAX>(*args, stream, sms);       \
      case gfpa::OP_SUB: return gfpa::launch_thread<gfpa::OP_SUB, NMAX>(*args, stream, sms);       \
    }                                                                                      \
    return cudaErrorInvalidValue;                                                          \
  }
GFPA_THREAD_CFG(gfpa_launch_cfg16, 32)
GFPA_THREAD_CFG(gfpa_launch_cfg17, 64)
