// fpa_misc.cu -- conversions, sign, compare and negation (the non-arithmetic fpa.h entry
// points).  These are not on the arithmetic hot path; each number is handled by one
// thread, walking its limbs.
//
// Reference semantics: fpa_warp_set.h:1-132 (set_ui/si/float/double), fpa_warp_set.h:134-199
// (precision change), fpa_threaded.h:1-93 (sgn, cmp), fpa_warp_add_sub.h:3-13,284-308 (neg).
#include <cuda_runtime.h>
#include <stdint.h>
#include "fpa_misc.h"

namespace gfpa_misc {

constexpr uint32_t BIAS = 0x3FFFFFF3u;
constexpr int CMP_VALUES = 25, CMP_ERR = 26;

// fpa_threaded.h:1-11 (NaN compares as error -> 0)
__constant__ int8_t c_sgn[9] = {+1, -1, 0, -1, +1, -1, +1, CMP_ERR, CMP_ERR};
// fpa_threaded.h:13-24, rows = class of a, columns = class of b
__constant__ int8_t c_cmp[81] = {
  CMP_VALUES, +1, +1, +1, +1, +1, -1, CMP_ERR, CMP_ERR,
  -1, CMP_VALUES, -1, -1, -1, +1, -1, CMP_ERR, CMP_ERR,
  -1, +1, 0, +1, -1, +1, -1, CMP_ERR, CMP_ERR,
  -1, +1, -1, CMP_ERR, -1, +1, -1, CMP_ERR, CMP_ERR,
  -1, +1, +1, +1, CMP_ERR, +1, -1, CMP_ERR, CMP_ERR,
  -1, -1, -1, -1, -1, CMP_ERR, -1, CMP_ERR, CMP_ERR,
  +1, +1, +1, +1, +1, +1, CMP_ERR, CMP_ERR, CMP_ERR,
  CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR,
  CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR, CMP_ERR,
};
// fpa_warp_add_sub.h:3-13
__constant__ uint8_t c_neg[9] = {0, 1, 2, 4, 3, 6, 5, 7, 8};

__device__ __forceinline__ uint32_t classify(uint32_t e) { return e <= 8u ? e : (e & 1u); }

// Writes an unsigned 64-bit magnitude (nonzero) times 2^extra_exp as a normalized number.
// Two or more limbs hold it exactly.  At one limb (precision 32) the 32 bits below the limb
// are rounded to nearest, ties to even, as mpfr_set_ui / mpfr_set_d do with MPFR_RNDN (the
// reference's precisions, 1024 bits and up, never round here).  Returns the exponent word
// for a positive value.
__device__ uint32_t put_u64(uint32_t *r, uint32_t n, uint64_t v, int extra_exp) {
  int s = __clzll((long long)v);
  v <<= s;
  long long e = 64 - s + extra_exp;
  uint32_t hi = (uint32_t)(v >> 32);
  const uint32_t lo = (uint32_t)v;
  if (n == 1) {
    if ((lo >> 31) && ((lo << 1) | (hi & 1u))) {       // above one half, or a tie on an odd limb
      hi++;
      if (hi == 0) { hi = 0x80000000u; e++; }         // 0.11..1 + ulp = 1.0
    }
    r[0] = hi;
  } else {
    for (uint32_t i = 0; i + 2 < n; i++) r[i] = 0;
    r[n - 1] = hi;
    r[n - 2] = lo;
  }
  return (uint32_t)(2 * ((long long)BIAS + e));
}

__global__ void k_set_int(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *vals, int is_signed) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint64_t u = ((const uint64_t *)vals)[i];
  uint32_t sign = 0;
  if (is_signed && (int64_t)u < 0) { sign = 1; u = 0 - u; }
  if (u == 0) { r_exps[i] = 2u; return; }
  r_exps[i] = put_u64(r_limbs + i * n, n, u, 0) + sign;
}

// IEEE binary32 / binary64 decode: value = (-1)^s * m * 2^q with integer m
__global__ void k_set_fp(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *vals, int is_double) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint64_t bits, m;
  int ef, q, mbits;
  uint32_t sign;
  if (is_double) {
    bits = ((const uint64_t *)vals)[i];
    sign = (uint32_t)(bits >> 63); ef = (int)((bits >> 52) & 0x7FF); m = bits & ((1ull << 52) - 1);
    mbits = 52;
    if (ef == 0x7FF) { r_exps[i] = m ? 7u : (sign ? 5u : 6u); return; }
    if (ef == 0) q = -1074; else { m |= 1ull << 52; q = ef - 1075; }
  } else {
    uint32_t b = ((const uint32_t *)vals)[i];
    sign = b >> 31; ef = (int)((b >> 23) & 0xFF); m = b & ((1u << 23) - 1);
    mbits = 23;
    if (ef == 0xFF) { r_exps[i] = m ? 7u : (sign ? 5u : 6u); return; }
    if (ef == 0) q = -149; else { m |= 1ull << 23; q = ef - 150; }
  }
  (void)mbits;
  if (m == 0) { r_exps[i] = 2u; return; }
  r_exps[i] = put_u64(r_limbs + i * n, n, m, q) + sign;
}

__device__ __forceinline__ bool round_up(int mode, uint32_t sign, uint32_t lsb, uint32_t rbit, uint32_t sticky) {
  switch (mode) {
    case 1: return sign == 0 && (rbit | sticky);
    case 2: return sign != 0 && (rbit | sticky);
    case 3: return rbit && (sticky | lsb);
    case 4: return rbit;
    default: return false;
  }
}

// precision change with rounding (fpa_set)
__global__ void k_set_prec(uint32_t *r_exps, uint32_t *r_limbs, uint32_t nr, const uint32_t *x_exps,
                           const uint32_t *x_limbs, uint32_t nx, uint64_t count, int mode) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t xe = x_exps[i];
  if (classify(xe) > 1u) { r_exps[i] = xe; return; }
  const uint32_t *x = x_limbs + i * nx;
  uint32_t *r = r_limbs + i * nr;
  if (nr >= nx) {
    for (uint32_t j = 0; j < nr - nx; j++) r[j] = 0;
    for (uint32_t j = 0; j < nx; j++) r[nr - nx + j] = x[j];
    r_exps[i] = xe;
    return;
  }
  const uint32_t drop = nx - nr;
  uint32_t rbit = x[drop - 1] >> 31, sticky = x[drop - 1] & 0x7FFFFFFFu;
  for (uint32_t j = 0; j + 1 < drop; j++) sticky |= x[j];
  uint32_t sign = xe & 1u;
  long long e = (long long)(xe >> 1) - BIAS;
  bool up = round_up(mode, sign, x[drop] & 1u, rbit, sticky != 0);
  uint32_t carry = up ? 1u : 0u;
  for (uint32_t j = 0; j < nr; j++) { uint32_t v = x[drop + j] + carry; carry = carry && v == 0; r[j] = v; }
  if (carry) { r[nr - 1] = 0x80000000u; e++; }
  if ((long long)BIAS + e > 0x7FFFFFFFLL) { r_exps[i] = 6u - sign; return; }
  r_exps[i] = (uint32_t)(2 * ((long long)BIAS + e)) + sign;
}

__global__ void k_sgn(int32_t *r, const uint32_t *x_exps, uint64_t count) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int a = c_sgn[classify(x_exps[i])];
  r[i] = (a == CMP_ERR) ? 0 : a;
}

__global__ void k_cmp(int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                      const uint32_t *b_limbs, uint32_t n, uint64_t count) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t ae = a_exps[i], be = b_exps[i];
  int act = c_cmp[classify(ae) * 9 + classify(be)];
  if (act == CMP_ERR) { r[i] = 0; return; }
  if (act != CMP_VALUES) { r[i] = act; return; }
  int sgn = (ae & 1u) ? -1 : 1, c = 0;
  if ((ae >> 1) != (be >> 1)) c = (ae >> 1) > (be >> 1) ? 1 : -1;
  else {
    const uint32_t *a = a_limbs + i * n, *b = b_limbs + i * n;
    for (int j = (int)n - 1; j >= 0; j--)
      if (a[j] != b[j]) { c = a[j] > b[j] ? 1 : -1; break; }
  }
  r[i] = sgn * c;
}

__global__ void k_neg(uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps, const uint32_t *a_limbs,
                      uint32_t n, uint64_t count) {
  uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31u;
  if (w >= count) return;
  uint32_t ae = a_exps[w];
  if (ae <= 8u) { if (lane == 0) r_exps[w] = c_neg[ae]; return; }
  for (uint32_t j = lane; j < n; j += 32) r_limbs[w * n + j] = a_limbs[w * n + j];
  if (lane == 0) r_exps[w] = ae ^ 1u;
}

static unsigned blocks_for(uint64_t threads) { return (unsigned)((threads + 255) / 256); }

}  // namespace gfpa_misc

using namespace gfpa_misc;

cudaError_t gfpa_misc_set_int(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *d_vals,
                              int is_signed, cudaStream_t st) {
  if (count) k_set_int<<<blocks_for(count), 256, 0, st>>>(r_exps, r_limbs, n, count, d_vals, is_signed);
  return cudaGetLastError();
}
cudaError_t gfpa_misc_set_fp(uint32_t *r_exps, uint32_t *r_limbs, uint32_t n, uint64_t count, const void *d_vals,
                             int is_double, cudaStream_t st) {
  if (count) k_set_fp<<<blocks_for(count), 256, 0, st>>>(r_exps, r_limbs, n, count, d_vals, is_double);
  return cudaGetLastError();
}
cudaError_t gfpa_misc_set_prec(uint32_t *r_exps, uint32_t *r_limbs, uint32_t nr, const uint32_t *x_exps,
                               const uint32_t *x_limbs, uint32_t nx, uint64_t count, int mode, cudaStream_t st) {
  if (count) k_set_prec<<<blocks_for(count), 256, 0, st>>>(r_exps, r_limbs, nr, x_exps, x_limbs, nx, count, mode);
  return cudaGetLastError();
}
cudaError_t gfpa_misc_sgn(int32_t *r, const uint32_t *x_exps, uint64_t count, cudaStream_t st) {
  if (count) k_sgn<<<blocks_for(count), 256, 0, st>>>(r, x_exps, count);
  return cudaGetLastError();
}
cudaError_t gfpa_misc_cmp(int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                          const uint32_t *b_limbs, uint32_t n, uint64_t count, cudaStream_t st) {
  if (count) k_cmp<<<blocks_for(count), 256, 0, st>>>(r, a_exps, a_limbs, b_exps, b_limbs, n, count);
  return cudaGetLastError();
}
cudaError_t gfpa_misc_neg(uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps, const uint32_t *a_limbs,
                          uint32_t n, uint64_t count, cudaStream_t st) {
  if (count) k_neg<<<blocks_for(count * 32), 256, 0, st>>>(r_exps, r_limbs, a_exps, a_limbs, n, count);
  return cudaGetLastError();
}
