// fpa_chain.cu -- fused operation chains that keep their intermediates on chip.
//
//   dot:          acc_d = RN(acc_d + RN(x_{d,i} * y_{d,i})) for i = 0 .. len-1, in order
//   newton sqrt:  y <- RN(RN(y + RN(x / y)) * 0.5), `iters` times
//
// Every step is rounded exactly as the separate fpa_mul / fpa_add / fpa_div calls would
// round it (the same per-operation device code runs, with shared-memory operands), but
// the accumulator and the temporaries never leave the lane group's shared memory, and a
// whole chain is one launch.  The multiplication by 0.5 is an exact exponent decrement
// with the multiply's special-value and range rules (fpa_warp_mul.h:1-12, 124-128).
#include <cuda_runtime.h>
#include "../../include/fpa_gb300.h"
#include "fpa_ops.cuh"
#include "fpa_launch.h"
#include "fpa_batch.h"

namespace gfpa {

struct ChainArgs {
  uint64_t count;
  uint32_t n, len;                 // len: dot length or Newton iterations
  int mode;
  uint32_t *r_exps, *r_limbs;
  const uint32_t *x_exps, *x_limbs, *y_exps, *y_limbs;
  uint32_t *err;
};

template <int G, int K, int R>
struct ChainSpace {
  static constexpr int N = G * K * R;
  __host__ __device__ static constexpr int cmax(int a, int b) { return a > b ? a : b; }
  static constexpr int ws_dot = cmax(OpWords<OP_MUL, G, K, R>::aligned(), OpWords<OP_ADD, G, K, R>::aligned());
  static constexpr int ws_newton = cmax(OpWords<OP_DIV, G, K, R>::aligned(), OpWords<OP_ADD, G, K, R>::aligned());
  static constexpr int value = N + 8;                   // one number: exponent word + limbs, aligned
  __host__ __device__ static constexpr int dot() { return ws_dot + 2 * value; }
  __host__ __device__ static constexpr int newton() { return ws_newton + 3 * value; }
};

// y <- y * 0.5 in place (exponent word of a shared-memory number)
__device__ __forceinline__ uint32_t half_of(uint32_t e) {
  const uint32_t c = classify(e);
  if (c > 1u) return c_action[2][c * 9 + CLS_POS_VALUE];       // class x +value
  const long long ex = (long long)(e >> 1) - BIAS - 1;
  if ((long long)BIAS + ex < 5) return CLS_POS_TINY - (e & 1u);
  return e - 2u;
}

template <int G, int K, int R>
__global__ void __launch_bounds__(128, 4) k_dot(ChainArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  Grp<G> g;
  constexpr int W = ChainSpace<G, K, R>::dot(), V = ChainSpace<G, K, R>::value;
  const uint32_t gpc = blockDim.x / G, gi = threadIdx.x / G;
  uint32_t *ws = smem + gi * W;
  uint32_t *acc = ws + ChainSpace<G, K, R>::ws_dot, *tmp = acc + V;   // [0] = exponent, [4..] = limbs
  const int n = (int)A.n;
  for (uint64_t d = (uint64_t)blockIdx.x * gpc + gi; d < A.count; d += (uint64_t)gridDim.x * gpc) {
    if (g.lane == 0) acc[0] = CLS_ZERO;
    g.sync();
    for (uint32_t i = 0; i < A.len; i++) {
      const uint64_t k = d * A.len + i, off = k * (uint64_t)n;
      op_mul<G, K, R>(g, ws, n, A.mode, A.x_exps[k], A.x_limbs + off, A.y_exps[k], A.y_limbs + off, tmp, tmp + 4);
      g.sync();
      // every lane reads both exponent words before the sum may write acc[0] (a sum that is
      // a copy of one operand writes it without meeting a collective first)
      const uint32_t acc_e = acc[0], tmp_e = tmp[0];
      g.sync();
      op_addsub<G, K, R>(g, ws, n, A.mode, 0, acc_e, acc + 4, tmp_e, tmp + 4, acc, acc + 4);
      g.sync();
    }
    for (int i = g.lane; i < n; i += G) A.r_limbs[d * n + i] = acc[4 + i];
    if (g.lane == 0) A.r_exps[d] = acc[0];
    g.sync();
  }
}

template <int G, int K, int R>
__global__ void __launch_bounds__(128, 4) k_newton_sqrt(ChainArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  Grp<G> g;
  constexpr int W = ChainSpace<G, K, R>::newton(), V = ChainSpace<G, K, R>::value;
  const uint32_t gpc = blockDim.x / G, gi = threadIdx.x / G;
  uint32_t *ws = smem + gi * W;
  uint32_t *y = ws + ChainSpace<G, K, R>::ws_newton, *t = y + V, *s = t + V;
  const int n = (int)A.n;
  // every thread of the CTA runs the same number of iterations and meets a CTA barrier after
  // each Newton step, so the warps go through the division's phases together (shared
  // instruction fetch, as in the elementwise div kernel)
  const uint64_t total = (uint64_t)gridDim.x * gpc, rounds = (A.count + total - 1) / total;
  for (uint64_t q = 0; q < rounds; q++) {
    const uint64_t d = q * total + (uint64_t)blockIdx.x * gpc + gi;
    const bool act = d < A.count;
    const uint64_t off = d * (uint64_t)n;
    uint32_t xe = 0;
    if (act) {
      for (int i = g.lane; i < n; i += G) y[4 + i] = A.y_limbs[off + i];
      if (g.lane == 0) y[0] = A.y_exps[d];
      g.sync();
      xe = A.x_exps[d];
    }
    for (uint32_t it = 0; it < A.len; it++) {
      if (act) {
        op_div<G, K, R>(g, ws, n, A.mode, xe, A.x_limbs + off, y[0], y + 4, t, t + 4, A.err);    // t = x / y
        g.sync();
        op_addsub<G, K, R>(g, ws, n, A.mode, 0, y[0], y + 4, t[0], t + 4, s, s + 4);           // s = y + t
        g.sync();
        for (int i = g.lane; i < n; i += G) y[4 + i] = s[4 + i];                            // y = s * 0.5
        if (g.lane == 0) y[0] = half_of(s[0]);
        g.sync();
      }
      __syncthreads();
    }
    if (act) {
      for (int i = g.lane; i < n; i += G) A.r_limbs[off + i] = y[4 + i];
      if (g.lane == 0) A.r_exps[d] = y[0];
      g.sync();
    }
  }
}

template <int G, int K, int R>
cudaError_t launch_chain(int kind, const ChainArgs &A, cudaStream_t st, int sms) {
  constexpr int gpc = 128 / G;
  const size_t smem = (size_t)gpc * (kind == 0 ? ChainSpace<G, K, R>::dot() : ChainSpace<G, K, R>::newton()) * 4;
  auto kern = kind == 0 ? k_dot<G, K, R> : k_newton_sqrt<G, K, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 128, smem)) != cudaSuccess) return e;
  if (per < 1) per = 1;
  const uint64_t need = (A.count + gpc - 1) / gpc, cap = (uint64_t)per * sms;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  kern<<<grid, 128, smem, st>>>(A);
  return cudaGetLastError();
}

cudaError_t dispatch_chain(int kind, int cfg, const ChainArgs &A, cudaStream_t st, int sms) {
  switch (cfg) {
    case 0: return launch_chain<4, 2, 1>(kind, A, st, sms);
    case 1: return launch_chain<8, 2, 1>(kind, A, st, sms);
    case 2: return launch_chain<8, 4, 1>(kind, A, st, sms);
    case 3: return launch_chain<16, 4, 1>(kind, A, st, sms);
    case 4: return launch_chain<32, 4, 1>(kind, A, st, sms);
    case 5: return launch_chain<32, 8, 1>(kind, A, st, sms);
    case 6: return launch_chain<32, 16, 1>(kind, A, st, sms);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gfpa

using namespace gfpa;

static fpa_result run_chain(int kind, uint32_t precision, uint64_t count, uint32_t len, int mode, uint32_t *r_exps,
                            uint32_t *r_limbs, const uint32_t *x_exps, const uint32_t *x_limbs,
                            const uint32_t *y_exps, const uint32_t *y_limbs, void *stream) {
  if (precision < 32 || precision > 32u * GFPA_MAX_LIMBS || precision % 32) return fpa_invalid_precisions;
  if (mode < 0 || mode > 4) return fpa_math_error;
  if (count == 0) return fpa_success;
  int sms;
  uint32_t *err;
  if (!gfpa_context(&sms, &err)) return fpa_device_error;
  ChainArgs A;
  A.count = count; A.n = precision / 32; A.len = len; A.mode = mode;
  A.r_exps = r_exps; A.r_limbs = r_limbs; A.x_exps = x_exps; A.x_limbs = x_limbs;
  A.y_exps = y_exps; A.y_limbs = y_limbs; A.err = err;
  const int cfg = gfpa_default_cfg(A.n < 4 ? 4 : A.n);
  if (cfg < 0) return fpa_invalid_precisions;
  return dispatch_chain(kind, cfg, A, (cudaStream_t)stream, sms) == cudaSuccess ? fpa_success : fpa_device_error;
}

extern "C" fpa_result fpa_gb300_dot(uint32_t precision, uint64_t count, uint32_t len, fpa_rounding_mode mode,
                                    uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *x_exps,
                                    const uint32_t *x_limbs, const uint32_t *y_exps, const uint32_t *y_limbs,
                                    void *stream) {
  if (len == 0) return fpa_invalid_counts;
  return run_chain(0, precision, count, len, (int)mode, r_exps, r_limbs, x_exps, x_limbs, y_exps, y_limbs, stream);
}

extern "C" fpa_result fpa_gb300_newton_sqrt(uint32_t precision, uint64_t count, uint32_t iters,
                                            fpa_rounding_mode mode, uint32_t *y_exps, uint32_t *y_limbs,
                                            const uint32_t *x_exps, const uint32_t *x_limbs, void *stream) {
  return run_chain(1, precision, count, iters, (int)mode, y_exps, y_limbs, x_exps, x_limbs, y_exps, y_limbs,
                   stream);
}
