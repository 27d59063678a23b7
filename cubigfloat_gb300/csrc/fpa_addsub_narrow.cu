// fpa_addsub_narrow.cu -- add/sub-only configurations with narrow lane groups.
//
// add/sub move more bytes than they compute, so their bound is HBM, and the part of their
// work that does not depend on the limb count (classes, exponents, the rounding decision)
// is done by every lane of a group.  A group of four lanes holding eight or sixteen limbs
// each puts eight operations in a warp, so that work is spread over more operations than
// with the general configurations' eight- to thirty-two-lane groups.  These configurations
// (16: 4 lanes x 8 limbs, 17: 4 lanes x 16 limbs) run add/sub only, with the operands in
// registers (op_addsub_regk).
#include <cuda_runtime.h>
#include "fpa_addsub_regs.cuh"

#define GFPA_NARROW_CFG(NAME, G, K)                                                               \
  extern "C" cudaError_t NAME(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) { \
    if ((int)args->n > (G) * (K)) return cudaErrorInvalidValue;                                   \
    switch (op) {                                                                                 \
      case gfpa::OP_ADD: return gfpa::launch_addsub_regk<gfpa::OP_ADD, G, K>(*args, stream, sms);  \
      case gfpa::OP_SUB: return gfpa::launch_addsub_regk<gfpa::OP_SUB, G, K>(*args, stream, sms);  \
    }                                                                                             \
    return cudaErrorInvalidValue;                                                                 \
  }
GFPA_NARROW_CFG(gfpa_launch_cfg16, 4, 8)
GFPA_NARROW_CFG(gfpa_launch_cfg17, 4, 16)
