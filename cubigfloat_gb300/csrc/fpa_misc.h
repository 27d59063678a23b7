// fpa_misc.h -- launchers for the non-arithmetic fpa entry points (fpa_misc.cu)
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

cudaError_t gfpa_misc_set_int(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *d_vals,
                              int is_signed, cudaStream_t st);
cudaError_t gfpa_misc_set_fp(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *d_vals,
                             int is_double, cudaStream_t st);
cudaError_t gfpa_misc_set_prec(uint32_t *r_exps, uint32_t *r_limbs, uint32_t nr, const uint32_t *x_exps,
                               const uint32_t *x_limbs, uint32_t nx, uint64_t count, int mode, cudaStream_t st);
cudaError_t gfpa_misc_sgn(int32_t *r, const uint32_t *x_exps, uint64_t count, cudaStream_t st);
cudaError_t gfpa_misc_cmp(int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                          const uint32_t *b_limbs, uint32_t n, uint64_t count, cudaStream_t st);
cudaError_t gfpa_misc_neg(uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps, const uint32_t *a_limbs,
                          uint32_t n, uint64_t count, cudaStream_t st);
