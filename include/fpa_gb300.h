/*
 * fpa_gb300.h -- additions to the fpa.h API in the GB300 library.
 *
 * None of these exist in the reference; they sit beside the drop-in fpa.h entry points:
 *   - stream-ordered and raw-device-pointer forms of the elementwise operations,
 *   - a device error word for the bounded correction loops,
 *   - the lane-group configuration table used by the autotuner.
 * Streams are passed as `void *` (a cudaStream_t, or NULL for the legacy default stream)
 * so that this header needs no CUDA include.
 */
#ifndef FPA_GB300_H
#define FPA_GB300_H

#include <stdint.h>
#include "fpa.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { fpa_op_add = 0, fpa_op_sub = 1, fpa_op_mul = 2, fpa_op_div = 3, fpa_op_sqrt = 4 } fpa_op;

/* r = a <op> b elementwise on raw device arrays of `count` numbers of `precision` bits
 * (limbs contiguous per number).  b_* are ignored for sqrt.  Asynchronous on `stream`. */
fpa_result fpa_gb300_elementwise(fpa_op op, uint32_t precision, uint64_t count, fpa_rounding_mode mode,
                                 uint32_t *r_exps, uint32_t *r_limbs,
                                 const uint32_t *a_exps, const uint32_t *a_limbs,
                                 const uint32_t *b_exps, const uint32_t *b_limbs, void *stream);

/* fpa_add/sub/mul/div/sqrt on a caller-chosen stream (b ignored for sqrt) */
fpa_result fpa_op_async(fpa_op op, fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode, void *stream);

/* whole-array copies ordered on `stream` (pinned host memory makes them asynchronous) */
fpa_result fpa_copy_array_to_device_async(fpa_t fpa, const uint32_t *exps, const uint32_t *limbs, void *stream);
fpa_result fpa_copy_array_to_host_async(fpa_t fpa, uint32_t *exps, uint32_t *limbs, void *stream);

/* Error bits raised by kernels since the previous call, then cleared (synchronizes the
 * device): 1 = a division's correction loop hit its bound, 2 = same for sqrt. */
uint32_t fpa_gb300_device_errors(void);

/* Lane-group configurations: configuration c runs one number per `lanes` threads with
 * product tiles of `tile_limbs` limbs and holds up to lanes*tile_limbs limbs. */
int fpa_gb300_num_configs(void);
fpa_result fpa_gb300_config_shape(int cfg, uint32_t *lanes, uint32_t *tile_limbs);
/* choose the configuration used for numbers of `limbs` limbs (-1 = built-in default) */
fpa_result fpa_gb300_set_config(uint32_t limbs, int cfg);
int fpa_gb300_get_config(uint32_t limbs);

/* Measured integer multiply-add throughput of the current GPU (mad.lo.u32 and mad.hi.u32
 * per second over all SMs): the roofline denominator for the multiply-bound operations. */
fpa_result fpa_gb300_measure_imad_peak(double *mad_lo_per_s, double *mad_hi_per_s);

const char *fpa_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif
