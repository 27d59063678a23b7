// fpa_addsub_narrow.cu -- add/sub-only configurations with narrow lane groups.
//
// add/sub move more bytes than they compute, so their bound is HBM, and the part of their
// work that does not depend on the limb count (classes, exponents, the rounding decision)
// is done by every lane of a group.  A group of four lanes holding eight or sixteen limbs
// each puts eight operations in a warp, so that work is spread over more operations than
// with the general configurations' eight- to thirty-two-lane groups.  Configuration 17 runs
// add/sub on four lanes x 16 limbs with the operands in registers (op_addsub_regk);
// configuration 16 runs add/sub and mul on one thread per operation for 8, 16 and 32 limbs
// (below) and on lane groups otherwise.
#include <cuda_runtime.h>
#include "fpa_addsub_regs.cuh"
#include "fpa_addsub_rows.cuh"

#define GFPA_NARROW_CFG(NAME, G, K)                                                               \
  extern "C" cudaError_t NAME(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) { \
    if ((int)args->n > (G) * (K)) return cudaErrorInvalidValue;                                   \
    switch (op) {                                                                                 \
      case gfpa::OP_ADD: return gfpa::launch_addsub_regk<gfpa::OP_ADD, G, K>(*args, stream, sms);  \
      case gfpa::OP_SUB: return gfpa::launch_addsub_regk<gfpa::OP_SUB, G, K>(*args, stream, sms);  \
    }                                                                                             \
    return cudaErrorInvalidValue;                                                                 \
  }
GFPA_NARROW_CFG(gfpa_launch_cfg17, 4, 16)

// Configuration 16: numbers of exactly 8, 16 or 32 limbs take one thread per operation on
// shared-memory rows (fpa_addsub_rows.cuh, add/sub and mul); other sizes up to 32 limbs the
// four-lane register add/sub with 8 limbs per lane, and the 8x4x1 lane-group mul.
template <int OP>
static cudaError_t launch_cfg16(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  switch (args.n) {
    case 8: return gfpa::launch_rows<OP, 8>(args, stream, sms);
    case 16: return gfpa::launch_rows<OP, 16>(args, stream, sms);
    case 32: return gfpa::launch_rows<OP, 32>(args, stream, sms);
  }
  if (args.n > 32) return cudaErrorInvalidValue;
  if constexpr (OP == gfpa::OP_MUL) return gfpa_launch_cfg2(OP, &args, stream, sms);
  else return gfpa::launch_addsub_regk<OP, 4, 8>(args, stream, sms);
}

extern "C" cudaError_t gfpa_launch_cfg16(int op, const ElementwiseArgs *args, cudaStream_t stream, int sms) {
  switch (op) {
    case gfpa::OP_ADD: return launch_cfg16<gfpa::OP_ADD>(*args, stream, sms);
    case gfpa::OP_SUB: return launch_cfg16<gfpa::OP_SUB>(*args, stream, sms);
    case gfpa::OP_MUL: return launch_cfg16<gfpa::OP_MUL>(*args, stream, sms);
  }
  return cudaErrorInvalidValue;
}
