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

/* Error bits raised by kernels on the current device since the previous call, then
 * cleared (synchronizes the device): 1 = a division's correction loop hit its bound, 2 =
 * same for sqrt.  The library keeps one such word (and its SM count) per device, made on
 * the first call that finds the device current. */
uint32_t fpa_gb300_device_errors(void);

/* r = RND(a*b + c) with a single rounding (no counterpart in the reference, whose API has
 * no fused operation).  All four arrays share count and precision; argument checks follow
 * fpa_dispatch.h:175-183.  Special values: the class of the exact product from the mul
 * table (fpa_warp_mul.h:1-12), combined with c by the add table (fpa_warp_add_sub.h:15-24). */
fpa_result fpa_gb300_fma(fpa_t r, fpa_t a, fpa_t b, fpa_t c, fpa_rounding_mode mode);

/* Lane-group configurations: configuration c runs one number per `lanes` threads with
 * product tiles of `tile_limbs` limbs, `pairs` column-block pairs per lane, and holds up
 * to lanes*tile_limbs*pairs limbs. */
int fpa_gb300_num_configs(void);
fpa_result fpa_gb300_config_shape(int cfg, uint32_t *lanes, uint32_t *tile_limbs, uint32_t *pairs);
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
 * concurrent) that pull tasks from device work queues.  mul, div and sqrt of 8 to 128 limbs
 * whose tuned configuration runs one thread per operation form one more class (tasks of up
 * to 32 operations of one operation and limb count), whose device scratch the batch owns. */
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
/* number of tasks per lane-group register class (3 entries) and class kernels per run
 * (the one-thread class counts as one), for inspection */
fpa_result fpa_batch_info(fpa_batch_t batch, uint32_t *tasks_per_class, uint32_t *kernels);
fpa_result fpa_batch_destroy(fpa_batch_t batch);

/* ---- fused chains (intermediates stay in on-chip shared memory, one launch) ----------
 *
 * Dot products: r_d = RN(... RN(RN(x_{d,0} y_{d,0}) + RN(x_{d,1} y_{d,1})) ...), every
 * product and every addition rounded in `mode`, accumulated in order from zero.  Element i
 * of dot d is number d*len + i of the x and y arrays (device). */
fpa_result fpa_gb300_dot(uint32_t precision, uint64_t count, uint32_t len, fpa_rounding_mode mode,
                         uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *x_exps, const uint32_t *x_limbs,
                         const uint32_t *y_exps, const uint32_t *y_limbs, void *stream);
/* Newton square root: `iters` times y <- RN(RN(y + RN(x / y)) * 0.5), y updated in place
 * (y holds the starting values on entry). */
fpa_result fpa_gb300_newton_sqrt(uint32_t precision, uint64_t count, uint32_t iters, fpa_rounding_mode mode,
                                 uint32_t *y_exps, uint32_t *y_limbs, const uint32_t *x_exps,
                                 const uint32_t *x_limbs, void *stream);

/* ---- served form: a request loop with continuous batching ----------------------------
 *
 * Jobs (one precision, `count` operations of mixed type) are submitted from any thread;
 * a server thread keeps up to `max_inflight` batches on the GPU, each in a slot whose
 * device arena is `hbm_budget_bytes / max_inflight` (allocated once, at creation).  When a
 * slot frees, pending jobs are admitted in arrival order while they fit its arena, so jobs
 * arriving while others run join the next batch and overlap with the batches in flight.
 * `batching = 0` serves each job alone with plain per-operation-type launches (the
 * comparison point).  Host arrays passed to submit must stay valid until the job is done;
 * results are written to r_exps / r_limbs (host) on completion. */
typedef struct {
  uint64_t hbm_budget_bytes;
  uint32_t max_inflight;
  uint32_t max_batch_ops;   /* 0 = no limit beyond the arena */
  int batching;             /* 1 = continuous batching, 0 = plain per-job launches */
} fpa_server_config;

typedef struct fpa_server_s *fpa_server_t;

fpa_result fpa_server_create(fpa_server_t *server, const fpa_server_config *config);
/* Returns a job id > 0, or minus an fpa_result code (e.g. -fpa_invalid_counts when the job
 * is larger than one slot's share of the budget). modes may be NULL (ties to even);
 * b_exps/b_limbs may be NULL when every operation is a sqrt. */
int64_t fpa_server_submit(fpa_server_t server, uint32_t precision, uint32_t count, const uint8_t *ops,
                          const uint8_t *modes, const uint32_t *a_exps, const uint32_t *a_limbs,
                          const uint32_t *b_exps, const uint32_t *b_limbs, uint32_t *r_exps, uint32_t *r_limbs);
/* Wait for a job (timeout_ms < 0: no limit); fpa_success once its results are written. */
fpa_result fpa_server_wait(fpa_server_t server, int64_t job, int64_t timeout_ms);
/* Nanoseconds since server creation at submission, admission to a batch, completion. */
fpa_result fpa_server_job_times(fpa_server_t server, int64_t job, uint64_t *t_submit, uint64_t *t_admit,
                                uint64_t *t_done);
/* Forget a finished job. */
fpa_result fpa_server_release(fpa_server_t server, int64_t job);
/* stats[6]: jobs done, operations done, batches launched, peak resident bytes, failed jobs,
 * budget bytes. */
fpa_result fpa_server_stats(fpa_server_t server, uint64_t *stats);
/* Finish pending work and free everything. */
fpa_result fpa_server_destroy(fpa_server_t server);

/* Device-resident results (no counterpart in the reference).  A server created with a
 * resident store keeps the results of jobs submitted with `keep` on the device until they
 * are released, and a later job of the same precision and count may take either operand
 * from such a result (`a_from` / `b_from` = its job id, the host operand pointers are then
 * ignored).  The operand is copied device to device; while its source is still in flight
 * the copy waits for it on the GPU, so a chain of jobs never returns to the host between
 * steps.  A job waits in the queue until its sources are launched.  Batching servers only.
 * The store is one device allocation of `resident_bytes`, made at creation; a job whose
 * kept result does not fit is refused with -fpa_invalid_counts.  A source cannot be released
 * while jobs that read it are pending. */
typedef struct {
  int64_t a_from;     /* > 0: operand a is that job's kept result */
  int64_t b_from;     /* > 0: operand b is that job's kept result */
  uint32_t keep;      /* 1: keep this job's result on the device */
  uint32_t copy_out;  /* 1: also write the result to r_exps / r_limbs (0: they may be NULL) */
} fpa_server_job_opts;
fpa_result fpa_server_create_resident(fpa_server_t *server, const fpa_server_config *config,
                                      uint64_t resident_bytes);
/* fpa_server_submit with options (opts = NULL: the defaults of fpa_server_submit). */
int64_t fpa_server_submit_ex(fpa_server_t server, uint32_t precision, uint32_t count, const uint8_t *ops,
                             const uint8_t *modes, const uint32_t *a_exps, const uint32_t *a_limbs,
                             const uint32_t *b_exps, const uint32_t *b_limbs, uint32_t *r_exps, uint32_t *r_limbs,
                             const fpa_server_job_opts *opts);
/* Copy a kept result to host memory (waits for the job). */
fpa_result fpa_server_read(fpa_server_t server, int64_t job, uint32_t *r_exps, uint32_t *r_limbs);
/* Cost account (no counterpart in the reference): ns[4] = nanoseconds summed over all batches
 * of the server thread's packing and planning, the host-to-device copies (with kept-result
 * operands), the kernels (with the copies into the resident store), and the device-to-host
 * copy, the last three from CUDA events on each batch's stream. */
fpa_result fpa_server_costs(fpa_server_t server, uint64_t *ns);

/* Batched run without any memory allocation.  No counterpart in the reference.
 *
 * For callers that must not allocate GPU memory at the point where they compute: a serving
 * loop whose latency budget cannot absorb cudaMalloc / cudaFree (which may synchronize the
 * device and wait on other work), and host applications that hand all device memory to
 * their own allocator up front and treat any later allocation by a library as a failure.
 * Inputs and outputs are the caller's device arrays.  The batch's working memory is one
 * fixed device array sized for FPA_NOALLOC_MAX_OPS operations, which every GPU that loads
 * the library holds until the process exits; more operations than that return
 * fpa_invalid_counts.  The first call on each device looks up that array's device address
 * (with that device current) and should come before any stream capture.  All calls share
 * the array and it keeps the last call's contents: each call clears its task counters and
 * error word itself, and calls that overlap on the GPU race on the array, so order them
 * (one stream, or an event between streams).  A device reset is not supported (the looked-
 * up address is kept).  Error bits of the bounded correction loops are read with
 * fpa_batch_noalloc_errors (which synchronizes `stream`). */
#define FPA_NOALLOC_MAX_OPS 4096
fpa_result fpa_batch_run_noalloc(const fpa_batch_desc *descs, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                                 const uint32_t *a_exps, const uint32_t *a_limbs,
                                 const uint32_t *b_exps, const uint32_t *b_limbs, void *stream);
uint32_t fpa_batch_noalloc_errors(void *stream);

/* Autotuned configuration table: the configuration used for `op` on numbers of `limbs`
 * limbs (-1 = built-in default), settable per operation. */
fpa_result fpa_gb300_set_op_config(fpa_op op, uint32_t limbs, int cfg);
int fpa_gb300_get_op_config(fpa_op op, uint32_t limbs);
/* Time every configuration that can hold `limbs` (and is at most 4x too large) on `sample`
 * random operations of `op`, return the fastest and its rate (the table is not changed). */
fpa_result fpa_gb300_autotune(fpa_op op, uint32_t limbs, uint32_t sample, int *best_cfg, double *ops_per_s);
/* Load a table file of lines "op first_limbs last_limbs cfg" ('#' starts a comment).  The
 * library loads tuned_configs.txt from the package directory (or the file named by the
 * environment variable FPA_GB300_TUNING) when it is loaded. */
fpa_result fpa_gb300_load_tuning(const char *path);

/* Karatsuba split for fpa_mul (and the mul launches of fpa_gb300_elementwise): numbers of at
 * least `limbs` limbs whose configuration holds at least 256 limbs on tiles of at least
 * 8 limbs take one Karatsuba level (three half-size products) instead of the schoolbook
 * product; 0 = never.  The
 * result is the same either way (the product is exact).  The default is the threshold
 * measured fastest on GB300. */
fpa_result fpa_gb300_set_karatsuba_limbs(uint32_t limbs);
uint32_t fpa_gb300_get_karatsuba_limbs(void);

/* Measured integer multiply-add throughput of the current GPU (mad.lo.u32 and mad.hi.u32
 * per second over all SMs): the roofline denominator for the multiply-bound operations. */
fpa_result fpa_gb300_measure_imad_peak(double *mad_lo_per_s, double *mad_hi_per_s);
/* Measured limb-product throughput of the current GPU: 32x32-bit products accumulated into
 * 96-bit columns per second over all SMs, issued as the product kernels issue them
 * (mad.lo.cc, madc.hi.cc, addc per product) -- the roofline denominator for mul/div/sqrt. */
fpa_result fpa_gb300_measure_product_peak(double *products_per_s);

const char *fpa_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif
