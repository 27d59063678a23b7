// fpa_kernels.cu -- elementwise fpa kernels for one lane-group configuration.
//
// This file is compiled once per configuration (GFPA_CFG selects G lanes per operation,
// K limbs per product tile and R column-block pairs per lane, capacity N = G*K*R limbs)
// so the configurations build in parallel.  Each object exports gfpa_launch_cfg<i>() used by the host dispatcher.
#include <cuda_runtime.h>
#include "fpa_ops.cuh"
#include "fpa_addsub_regs.cuh"
#include "fpa_launch.h"

#ifndef GFPA_CFG
#define GFPA_CFG 4
#endif

#if GFPA_CFG == 0
#define CFG_G 4
#define CFG_K 2
#define CFG_R 1
#elif GFPA_CFG == 1
#define CFG_G 8
#define CFG_K 2
#define CFG_R 1
#elif GFPA_CFG == 2
#define CFG_G 8
#define CFG_K 4
#define CFG_R 1
#elif GFPA_CFG == 3
#define CFG_G 16
#define CFG_K 4
#define CFG_R 1
#elif GFPA_CFG == 4
#define CFG_G 32
#define CFG_K 4
#define CFG_R 1
#elif GFPA_CFG == 5
#define CFG_G 32
#define CFG_K 8
#define CFG_R 1
#elif GFPA_CFG == 6
#define CFG_G 32
#define CFG_K 16
#define CFG_R 1
#elif GFPA_CFG == 7
#define CFG_G 16
#define CFG_K 8
#define CFG_R 1
#elif GFPA_CFG == 8
#define CFG_G 8
#define CFG_K 16
#define CFG_R 1
#elif GFPA_CFG == 9
#define CFG_G 16
#define CFG_K 16
#define CFG_R 1
#elif GFPA_CFG == 10
#define CFG_G 8
#define CFG_K 4
#define CFG_R 2
#elif GFPA_CFG == 11
#define CFG_G 8
#define CFG_K 4
#define CFG_R 4
#elif GFPA_CFG == 12
#define CFG_G 16
#define CFG_K 4
#define CFG_R 2
#elif GFPA_CFG == 13
#define CFG_G 8
#define CFG_K 8
#define CFG_R 4
#elif GFPA_CFG == 14
#define CFG_G 16
#define CFG_K 8
#define CFG_R 2
#elif GFPA_CFG == 15
#define CFG_G 4
#define CFG_K 4
#define CFG_R 8
#else
#error "unknown GFPA_CFG"
#endif

#define GFPA_CAT2(a, b) a##b
#define GFPA_CAT(a, b) GFPA_CAT2(a, b)
#define GFPA_LAUNCH_NAME GFPA_CAT(gfpa_launch_cfg, GFPA_CFG)

namespace gfpa {

template <int OP, int G, int K, int R>
using Words = PipeWords<OP, G, K, R>;

// Register budgets (blocks of 128 threads per SM): 64 registers per thread for add/sub/mul
// with tiles up to 4 limbs, 128 for 8-limb tiles and for div/sqrt (whose Newton loops keep
// more state live), 255 for 16-limb tiles (a 16x16 tile holds 48 accumulators + 48 operands).
#ifndef GFPA_NEWTON_MINBLOCKS
#define GFPA_NEWTON_MINBLOCKS 4
#endif
template <int OP, int K>
struct MinBlocks {
  static constexpr int v = (K >= 16) ? 2
                           : ((OP == OP_DIV || OP == OP_SQRT || OP == OP_FMA) ? (K >= 8 ? 4 : GFPA_NEWTON_MINBLOCKS)
                                                                               : (K >= 8 ? 4 : 8));
};

// add/sub: HBM-bound, so each group double-buffers its operands: the copies of its next
// operation (cp.async) are in flight while it computes the current one.
template <int OP, int G, int K, int R>
__device__ __forceinline__ void addsub_pipelined(const Grp<G> &g, uint32_t *ws, const ElementwiseArgs &args,
                                                 uint64_t i, uint64_t stride) {
  constexpr int N = G * K * R;
  const int n = (int)args.n;
  uint32_t *X = ws + 4 * N;
  const bool vec = (n & 3) == 0 && ((((uintptr_t)args.a_limbs) | ((uintptr_t)args.b_limbs)) & 15) == 0;
  uint32_t ae = 0, be = 0;
  if (i < args.count) {
    grp_stage_async<G>(g, ws, args.a_limbs + i * n, n, vec);
    grp_stage_async<G>(g, ws + N, args.b_limbs + i * n, n, vec);
    ae = args.a_exps[i]; be = args.b_exps[i];
  }
  cp_async_commit();
  int cur = 0;
  for (; i < args.count; i += stride) {
    const uint64_t nx = i + stride;
    uint32_t nae = 0, nbe = 0;
    if (nx < args.count) {
      uint32_t *nb = ws + (cur ^ 1) * 2 * N;
      grp_stage_async<G>(g, nb, args.a_limbs + nx * n, n, vec);
      grp_stage_async<G>(g, nb + N, args.b_limbs + nx * n, n, vec);
      nae = args.a_exps[nx]; nbe = args.b_exps[nx];
    }
    cp_async_commit();
    cp_async_wait<1>();                          // this operation's operands have landed
    g.sync();
    const uint32_t *sa = ws + cur * 2 * N;
    op_addsub_staged<G>(g, X, n, args.mode, OP == OP_SUB, ae, sa, be, sa + N, args.r_exps + i,
                        args.r_limbs + i * n);
    g.sync();                                    // the buffer is refilled two operations on
    ae = nae; be = nbe; cur ^= 1;
  }
  cp_async_wait<0>();
}

// mul: the same double buffering; the zero padding around the staged operands is the same
// for every operation of a launch, so it is written once.
// KARA: the instantiation with the Karatsuba split (launched from its threshold up).
template <int G, int K, int R, bool KARA>
__device__ __forceinline__ void mul_pipelined(const Grp<G> &g, uint32_t *ws, const ElementwiseArgs &args, uint64_t i,
                                              uint64_t stride) {
  constexpr int N = G * K * R;
  const int n = (int)args.n;
  const int NK = ((n + K - 1) / K) * K;
  MulScratch<G, K, R> s; s.carve(ws);
  uint32_t *P = ws + MulScratch<G, K, R>::words();
  uint32_t *xa[2] = {s.sa, P + 2 * N + 4};
  uint32_t *yb[2] = {s.sb, xa[1] + N};
  uint32_t *kws = KARA ? yb[1] + N + 2 * K : nullptr;   // Karatsuba staging
  for (int j = g.lane; j < NK; j += G)
    if (j >= n) { xa[0][j] = 0u; xa[1][j] = 0u; }
  for (int j = g.lane; j < NK + 2 * K; j += G)
    if (j < K || j >= K + n) { yb[0][j] = 0u; yb[1][j] = 0u; }
  const bool va = (n & 3) == 0 && (((uintptr_t)args.a_limbs) & 15) == 0;
  const bool vb = va && (K & 3) == 0 && (((uintptr_t)args.b_limbs) & 15) == 0;
  uint32_t ae = 0, be = 0;
  if (i < args.count) {
    grp_stage_async<G>(g, xa[0], args.a_limbs + i * n, n, va);
    grp_stage_async<G>(g, yb[0] + K, args.b_limbs + i * n, n, vb);
    ae = args.a_exps[i]; be = args.b_exps[i];
  }
  cp_async_commit();
  int cur = 0;
  for (; i < args.count; i += stride) {
    const uint64_t nx = i + stride;
    uint32_t nae = 0, nbe = 0;
    if (nx < args.count) {
      grp_stage_async<G>(g, xa[cur ^ 1], args.a_limbs + nx * n, n, va);
      grp_stage_async<G>(g, yb[cur ^ 1] + K, args.b_limbs + nx * n, n, vb);
      nae = args.a_exps[nx]; nbe = args.b_exps[nx];
    }
    cp_async_commit();
    cp_async_wait<1>();                          // this operation's operands have landed
    g.sync();
    s.sa = xa[cur]; s.sb = yb[cur];
    op_mul_staged<G, K, R>(g, s, P, n, args.mode, ae, be, args.r_exps + i, args.r_limbs + i * n, kws);
    g.sync();                                    // the buffer is refilled two operations on
    ae = nae; be = nbe; cur ^= 1;
  }
  cp_async_wait<0>();
}

// sqrt may run CTAs of up to 8 warps (its lockstep warps then share the fetched code eight
// at a time), with the same registers per thread as four-warp CTAs.
template <int OP, int K>
struct CtaBounds {
  static constexpr int threads = OP == OP_SQRT ? 256 : 128;
  static constexpr int min_blocks = OP == OP_SQRT ? (MinBlocks<OP, K>::v + 1) / 2 : MinBlocks<OP, K>::v;
};

template <int OP, int G, int K, int R>
__global__ void __launch_bounds__(CtaBounds<OP, K>::threads, CtaBounds<OP, K>::min_blocks)
    k_elementwise(ElementwiseArgs args) {
  extern __shared__ __align__(16) uint32_t smem[];
  Grp<G> g;
  const uint32_t gpc = blockDim.x / G, gi = threadIdx.x / G;
  uint32_t *ws = smem + gi * Words<OP, G, K, R>::aligned();
  const int n = (int)args.n;
  if constexpr (OP == OP_ADD || OP == OP_SUB) {
    addsub_pipelined<OP, G, K, R>(g, ws, args, (uint64_t)blockIdx.x * gpc + gi, (uint64_t)gridDim.x * gpc);
    return;
  }
  if constexpr (OP == OP_MUL || OP == OP_MUL_KARA) {
    mul_pipelined<G, K, R, OP == OP_MUL_KARA>(g, ws, args, (uint64_t)blockIdx.x * gpc + gi,
                                               (uint64_t)gridDim.x * gpc);
    return;
  }
  // div / sqrt / fma.  Every thread of the CTA runs the same number of iterations and meets
  // a CTA barrier after each: the warps then go through an operation's phases together and
  // share the fetched code of each phase (div and sqrt are 130-190 KB of code, and with the
  // warps spread over the phases instruction-fetch stalls led; measured on 8x4x4 at 4096
  // bits: div +16 %, sqrt +8 %).
  const uint64_t total = (uint64_t)gridDim.x * gpc;
  const uint64_t iters = (args.count + total - 1) / total;
  for (uint64_t it = 0; it < iters; it++) {
    const uint64_t i = it * total + (uint64_t)blockIdx.x * gpc + gi;
    if (i < args.count) {
      const uint64_t off = i * (uint64_t)n;
      const uint32_t a_exp = args.a_exps[i];
      const uint32_t b_exp = (OP == OP_SQRT) ? 0u : args.b_exps[i];
      if (OP == OP_DIV)
        op_div<G, K, R>(g, ws, n, args.mode, a_exp, args.a_limbs + off, b_exp, args.b_limbs + off,
                        args.r_exps + i, args.r_limbs + off, args.err);
      else if (OP == OP_SQRT)
        op_sqrt<G, K, R>(g, ws, n, args.mode, a_exp, args.a_limbs + off, args.r_exps + i, args.r_limbs + off,
                         args.err);
      else
        op_fma<G, K, R>(g, ws, n, args.mode, a_exp, args.a_limbs + off, b_exp, args.b_limbs + off, args.c_exps[i],
                        args.c_limbs + off, args.r_exps + i, args.r_limbs + off);
      g.sync();   // the group's shared slice is reused by its next instance
    }
    __syncthreads();
  }
}

template <int OP>
static cudaError_t launch_op(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  constexpr int G = CFG_G, K = CFG_K, R = CFG_R;
  if constexpr (OP == OP_ADD || OP == OP_SUB) {
    if ((int)args.n <= G * K) return launch_addsub_regk<OP, G, K>(args, stream, sms);
  }
  if constexpr (OP == OP_MUL && KaratsubaCfg<G, K, R>::on) {
    if (args.n >= 4 && args.n >= args.kara_min) return launch_op<OP_MUL_KARA>(args, stream, sms);
  }
  constexpr size_t warp_bytes = (size_t)(32 / G) * Words<OP, G, K, R>::aligned() * sizeof(uint32_t);
  constexpr size_t cta_max = 227 * 1024;
  if constexpr (warp_bytes > cta_max) return cudaErrorInvalidConfiguration;
  // CTA of 4, 2 or 1 warps (sqrt: up to 8, CtaBounds): a smaller CTA is taken only when it
  // keeps at least a quarter more warps resident on an SM (shared memory is granted per CTA,
  // so where a larger CTA's worth does not fit once more, a smaller CTA may still fit;
  // measured, small CTAs are otherwise slower).
  static int configured = 0, warps = 1, per_sm = 1;
  auto kern = k_elementwise<OP, G, K, R>;
  if (!configured) {
    const int wtop = CtaBounds<OP, K>::threads / 32;
    int wmax = 1;
    while (wmax * 2 <= wtop && warp_bytes * wmax * 2 <= cta_max) wmax *= 2;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(wmax * warp_bytes));
    if (e != cudaSuccess) return e;
    int best = 0;
    for (int w = wmax; w >= 1; w >>= 1) {
      int blocks = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, 32 * w, w * warp_bytes);
      if (e != cudaSuccess) return e;
      if (4 * blocks * w >= 5 * best && blocks * w > best) { best = blocks * w; warps = w; per_sm = blocks; }
    }
    if (per_sm < 1) per_sm = 1;
    configured = 1;
  }
  const int threads = 32 * warps, gpc = threads / G;
  const size_t smem = (size_t)warps * warp_bytes;
  const uint64_t need = (args.count + gpc - 1) / gpc;
  const uint64_t cap = (uint64_t)sms * (uint64_t)per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  kern<<<grid, threads, smem, stream>>>(args);
  return cudaGetLastError();
}

}  // namespace gfpa

extern "C" cudaError_t GFPA_LAUNCH_NAME(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  using namespace gfpa;
  switch (op) {
    case OP_ADD: return launch_op<OP_ADD>(*args, stream, sms);
    case OP_SUB: return launch_op<OP_SUB>(*args, stream, sms);
    case OP_MUL: return launch_op<OP_MUL>(*args, stream, sms);
    case OP_DIV: return launch_op<OP_DIV>(*args, stream, sms);
    case OP_SQRT: return launch_op<OP_SQRT>(*args, stream, sms);
#if GFPA_CFG <= 6
    case OP_FMA: return launch_op<OP_FMA>(*args, stream, sms);   // default configurations only
#endif
  }
  return cudaErrorInvalidValue;
}
