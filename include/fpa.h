/*
 * fpa.h -- drop-in C API of the GB300 fpa library (libfpa_gb300.so).
 *
 * Same names, enum values, struct layout and argument meaning as cuBigFloat's public
 * header (fpa.h:8-63 of the reference), so existing callers recompile and link against
 * this library unchanged.  Each entry point below names the reference declaration it
 * replaces.
 *
 * Arrays of `count` binary floating-point numbers of one precision live in device memory.
 * Host layout used by fpa_copy_array_to_device/host: one exponent word per number and
 * precision/32 little-endian 32-bit limbs per number, numbers stored one after another.
 *
 * Differences from the reference, all additive:
 *   - precision may be any multiple of 32 bits from 32 to 16384 (the reference accepts
 *     1024..8192 in steps of 1024, fpa_management.h:2-3);
 *   - errors from the CUDA runtime are returned as fpa_device_error instead of printing
 *     and exiting the process (fpa.cu:34);
 *   - results are correctly rounded in all five modes, also where the reference's kernels
 *     are not: exact ties after mul's one-bit normalisation (fpa_warp_mul.h:115-121), a
 *     mul result whose high half is all ones (:99-105), 0 - b (fpa_warp_add_sub.h:357-379)
 *     and sqrt rounding up into the next binade (fpa_warp_sqrt.h:238-242);
 *   - fpa_set stores the rounded limbs (the reference's kernel never stores them,
 *     fpa_warp_set.h:134-199), and at precision 32 the conversions round a wider integer or
 *     double mantissa to nearest, ties to even.
 */
#ifndef FPA_H
#define FPA_H

#include <stdint.h>

#define GPU_FPA

/* fpa.h:8-10 */
typedef enum {
  fpa_round_truncate,
  fpa_round_up,
  fpa_round_down,
  fpa_round_ties_to_even,
  fpa_round_ties_away_from_zero
} fpa_rounding_mode;

/* fpa.h:12-17; fpa_device_error is an addition (value 4) */
typedef enum {
  fpa_success,
  fpa_math_error,
  fpa_invalid_precisions,
  fpa_invalid_counts,
  fpa_device_error
} fpa_result;

/* fpa.h:19-26 (the -DGPU layout, which is the only implemented one) */
struct fpa_s {
  uint32_t count;
  uint32_t precision;
  uint32_t *gpu_exps;
  uint32_t *gpu_limbs;
};

typedef struct fpa_s fpa_t[1];   /* fpa.h:36 */
typedef struct fpa_s *fpa_ptr;   /* fpa.h:37 */

#ifdef __cplusplus
extern "C" {
#endif

/* fpa.h:43 -- allocate count numbers of `precision` bits on the current device */
fpa_result fpa_init(fpa_t fpa, uint32_t count, uint32_t precision);
/* fpa.h:44 */
fpa_result fpa_clear(fpa_t fpa);

/* fpa.h:46-47 -- synchronous copies of a whole array (host arrays as described above) */
fpa_result fpa_copy_array_to_device(fpa_t fpa, uint32_t *exps, uint32_t *limbs);
fpa_result fpa_copy_array_to_host(fpa_t fpa, uint32_t *exps, uint32_t *limbs);

/* fpa.h:49-53 -- conversions into the format */
fpa_result fpa_set_ui(fpa_t r, uint64_t *ui);
fpa_result fpa_set_si(fpa_t r, int64_t *si);
fpa_result fpa_set_float(fpa_t r, float *floats);
fpa_result fpa_set_double(fpa_t r, double *doubles);
fpa_result fpa_set(fpa_t r, fpa_t x, fpa_rounding_mode mode);

/* fpa.h:55-56 -- r is a device array of count int32 values */
fpa_result fpa_sgn(int32_t *r, fpa_t x);
fpa_result fpa_cmp(int32_t *r, fpa_t a, fpa_t b);

/* fpa.h:58-63 -- elementwise arithmetic, asynchronous on the legacy default stream */
fpa_result fpa_neg(fpa_t r, fpa_t a);
fpa_result fpa_add(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode);
fpa_result fpa_sub(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode);
fpa_result fpa_mul(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode);
fpa_result fpa_div(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode);
fpa_result fpa_sqrt(fpa_t r, fpa_t x, fpa_rounding_mode mode);

#ifdef __cplusplus
}
#endif

#endif
