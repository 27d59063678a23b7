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

/* ---- batched form: many operations of mixed type and precision in one submission ----
 *
 * Each descriptor names one operation on numbers of `limbs` limbs (1..512); operand and
 * result limbs live in caller-owned device pools at the given limb offsets, and exponent
 * word i of the r/a/b exponent arrays belongs to descriptor i.  The plan sorts the
 * operations into per-configuration tasks, picks each one's lane-group configuration from
 * the autotuned table, and runs them with persistent kernels (one per register class,
 * concurrent) that pull tasks from device work queues. */
typedef struct {
  uint8_t op;          /* fpa_op */
  uint8_t mode;        /* fpa_rounding_mode */
  uint16_t limbs;      /* precision / 32 */
  uint32_t reserved;
  uint64_t r_off, a_off, b_off;   /* limb offsets into the pools (b ignored for sqrt) */
} fpa_batch_desc;

typedef struct fpa_batch_s *fpa_batch_t;

/* Build a plan for `count` host descriptors (copied to the device). */
fpa_result fpa_batch_create(fpa_batch_t *batch, const fpa_batch_desc *descs, uint64_t count);
/* Run the plan on `stream` (asynchronous). */
fpa_result fpa_batch_run(fpa_batch_t batch, uint32_t *r_exps, uint32_t *r_limbs,
                         const uint32_t *a_exps, const uint32_t *a_limbs,
                         const uint32_t *b_exps, const uint32_t *b_limbs, void *stream);
/* Capture one run (with these pointers) as a CUDA graph, then replay it with
 * fpa_batch_graph_launch: one launch submits every task of the batch. */
fpa_result fpa_batch_capture(fpa_batch_t batch, uint32_t *r_exps, uint32_t *r_limbs,
                             const uint32_t *a_exps, const uint32_t *a_limbs,
                             const uint32_t *b_exps, const uint32_t *b_limbs);
fpa_result fpa_batch_graph_launch(fpa_batch_t batch, void *stream);
/* number of tasks per register class (3 classes) and kernels per run, for inspection */
fpa_result fpa_batch_info(fpa_batch_t batch, uint32_t *tasks_per_class, uint32_t *kernels);
fpa_result fpa_batch_destroy(fpa_batch_t batch);

/* Autotuned configuration table: the configuration used for `op` on numbers of `limbs`
 * limbs (-1 = built-in default), settable per operation. */
fpa_result fpa_gb300_set_op_config(fpa_op op, uint32_t limbs, int cfg);
int fpa_gb300_get_op_config(fpa_op op, uint32_t limbs);

/* Measured integer multiply-add throughput of the current GPU (mad.lo.u32 and mad.hi.u32
 * per second over all SMs): the roofline denominator for the multiply-bound operations. */
fpa_result fpa_gb300_measure_imad_peak(double *mad_lo_per_s, double *mad_hi_per_s);

const char *fpa_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif
