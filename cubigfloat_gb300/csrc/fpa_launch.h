// fpa_launch.h -- internal host/device interface between the C-ABI layer and the kernels.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

// One elementwise launch: `count` instances of `n` limbs each, contiguous per instance
// (instance i's limbs at i*n), exponent words in separate arrays.  All pointers are device
// pointers.  b_* are ignored for sqrt; c_* are read by fma only (op 5, which the default
// configurations 0..6 run).  `err` is a device word the kernels OR error bits
// into (1: div correction did not converge, 2: sqrt correction did not converge).
struct ElementwiseArgs {
  uint64_t count;
  uint32_t n;
  int mode;
  uint32_t *r_exps, *r_limbs;
  const uint32_t *a_exps, *a_limbs;
  const uint32_t *b_exps, *b_limbs;
  uint32_t *err;
  const uint32_t *c_exps = nullptr, *c_limbs = nullptr;   // third operand (fma only)
  uint32_t kara_min = 0xFFFFFFFFu;   // mul: Karatsuba split from this many limbs (tile >= 8)
};

#define GFPA_NUM_CFGS 20
#define GFPA_OP_FMA 5        // elementwise operation code of fma (after add, sub, mul, div, sqrt)
#define GFPA_NUM_DEFAULT_CFGS 7
#define GFPA_MAX_LIMBS 512
#ifndef GFPA_KARATSUBA_DEFAULT
#define GFPA_KARATSUBA_DEFAULT 0xFFFFFFFFu   // mul: Karatsuba split from this many limbs
#endif

// Lane-group configurations (G lanes x K limbs per tile x R block pairs per lane, capacity
// G*K*R limbs).  0..6 are the defaults in increasing capacity; 7..15 put two to eight
// operations in one warp (fewer lanes per operation, wider tiles or several block pairs
// per lane), which the autotuner can choose (mostly for div/sqrt); 16 to 19 are elementwise
// only: 16 runs add/sub and mul, one thread per operation on shared-memory rows for 8, 16
// and 32 limbs and lane groups otherwise; 17 runs add/sub on four lanes x 16 limbs in
// registers (fpa_addsub_narrow.cu); 18 and 19 run mul, div and sqrt with one thread per
// operation and 8x8-limb product tiles, up to 128 and 64 limbs (fpa_thread_newton.cu).
static const int gfpa_cfg_G[GFPA_NUM_CFGS] = {4, 8, 8, 16, 32, 32, 32, 16, 8, 16, 8, 8, 16, 8, 16, 4, 4, 4, 1, 1};
static const int gfpa_cfg_K[GFPA_NUM_CFGS] = {2, 2, 4, 4, 4, 8, 16, 8, 16, 16, 4, 4, 4, 8, 8, 4, 8, 16, 8, 8};
static const int gfpa_cfg_R[GFPA_NUM_CFGS] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 4, 2, 4, 2, 8, 1, 1, 16, 8};
static inline int gfpa_cfg_capacity(int c) { return gfpa_cfg_G[c] * gfpa_cfg_K[c] * gfpa_cfg_R[c]; }
// configurations 16 to 19 have elementwise kernels only
static inline bool gfpa_cfg_elementwise_only(int c) { return c >= 16; }
static inline bool gfpa_cfg_supports(int c, int op) {
  if (c >= 18) return op == 2 || op == 3 || op == 4;
  return c < 16 || op <= 1 || (c == 16 && op == 2);
}
// the current device's memory pool for stream-ordered scratch (fpa_api.cu)
bool gfpa_scratch_pool(cudaMemPool_t *pool);

extern "C" {
cudaError_t gfpa_launch_cfg0(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg1(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg2(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg3(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg4(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg5(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg6(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg7(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg8(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg9(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg10(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg11(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg12(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg13(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg14(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg15(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg16(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg17(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg18(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
cudaError_t gfpa_launch_cfg19(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms);
}

// smallest default configuration whose capacity holds n limbs
static inline int gfpa_default_cfg(uint32_t n) {
  for (int c = 0; c < GFPA_NUM_DEFAULT_CFGS; c++)
    if ((uint32_t)gfpa_cfg_capacity(c) >= n) return c;
  return -1;
}

static inline cudaError_t gfpa_launch(int cfg, int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  switch (cfg) {
    case 0: return gfpa_launch_cfg0(op, args, stream, sms);
    case 1: return gfpa_launch_cfg1(op, args, stream, sms);
    case 2: return gfpa_launch_cfg2(op, args, stream, sms);
    case 3: return gfpa_launch_cfg3(op, args, stream, sms);
    case 4: return gfpa_launch_cfg4(op, args, stream, sms);
    case 5: return gfpa_launch_cfg5(op, args, stream, sms);
    case 6: return gfpa_launch_cfg6(op, args, stream, sms);
    case 7: return gfpa_launch_cfg7(op, args, stream, sms);
    case 8: return gfpa_launch_cfg8(op, args, stream, sms);
    case 9: return gfpa_launch_cfg9(op, args, stream, sms);
    case 10: return gfpa_launch_cfg10(op, args, stream, sms);
    case 11: return gfpa_launch_cfg11(op, args, stream, sms);
    case 12: return gfpa_launch_cfg12(op, args, stream, sms);
    case 13: return gfpa_launch_cfg13(op, args, stream, sms);
    case 14: return gfpa_launch_cfg14(op, args, stream, sms);
    case 15: return gfpa_launch_cfg15(op, args, stream, sms);
    case 16: return gfpa_launch_cfg16(op, args, stream, sms);
    case 17: return gfpa_launch_cfg17(op, args, stream, sms);
    case 18: return gfpa_launch_cfg18(op, args, stream, sms);
    case 19: return gfpa_launch_cfg19(op, args, stream, sms);
  }
  return cudaErrorInvalidValue;
}
