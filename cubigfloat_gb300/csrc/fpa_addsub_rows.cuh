// fpa_addsub_rows.cuh -- add/sub and mul with one thread per operation on shared-memory
// rows, for numbers of exactly N = 8, 16 or 32 limbs (256, 512 and 1024 bits).
//
// A lane group repeats an operation's scalar work (classes, exponents, the rounding
// decision) on every lane, which leaves a few-hundred-bit add/sub bound by integer issue,
// not by HBM.  Here one thread runs one whole operation:
//   - each warp stages its 32 consecutive operations with 16-byte cp.async copies into
//     rows of N+4 words (the stride keeps eight threads' 16-byte row reads on distinct
//     banks), double-buffered so the next 32 operations' copies are in flight;
//   - the thread reads the larger operand with 16-byte loads and the aligned smaller one
//     at shifted word offsets straight from its row, forms the aligned sum in registers
//     with compile-time indices, and rounds it;
//   - the result mantissa goes back over the thread's row, and the warp stores the rows
//     with coalesced 16-byte stores.
// Same semantics and result as op_addsub_staged / op_addsub_regk: X = BIG*2^64 +- T,
// T = floor(SMALL*2^(64-d)) in N+3 limbs, bits of SMALL below X limb 0 as sticky (and one
// unit borrowed for an effective subtraction, as the ones' complement with a carry in of
// 1 - sticky), one rounding.  Reference: fpa_warp_add_sub.h:310-380 (dispatch), :41-125
// (same-sign add), :127-282 (effective subtraction); range checks as there.
#pragma once
#include <cuda_runtime.h>
#include "fpa_ops.cuh"
#include "fpa_launch.h"

namespace gfpa {

template <int N>
struct RowSpace {
  static constexpr int S = N + 4;                   // row stride (words, 16-byte multiple)
  static constexpr int buf = 2 * 32 * S + 64;       // rows of a, rows of b, exponents of a and b
  static constexpr int words = 2 * buf;             // two buffers
};

// One operation by one thread.  ra / rb: the operands' rows; the result mantissa is
// written over ra (class results write no limbs).  Returns the result's exponent word.
template <int N>
__device__ __forceinline__ uint32_t row_addsub(uint32_t *ra, const uint32_t *rb, uint32_t a_exp, uint32_t b_exp,
                                               int mode, int is_sub) {
  const uint32_t act = c_action[is_sub][classify(a_exp) * 9 + classify(b_exp)];
  if (act == ACT_COPY_A) return a_exp;                          // the limbs are already in ra
  if (act == ACT_COPY_B || act == ACT_NEG_B) {                  // b, or 0 - b = -b
#pragma unroll
    for (int s = 0; s < N; s += 4)
      *reinterpret_cast<uint4 *>(ra + s) = *reinterpret_cast<const uint4 *>(rb + s);
    return act == ACT_COPY_B ? b_exp : (b_exp ^ 1u);
  }
  if (act != ACT_ADD && act != ACT_SUB) return act;
  const uint32_t sa = a_exp & 1u, sb = (b_exp & 1u) ^ (uint32_t)is_sub;
  const uint32_t wa = a_exp >> 1, wb = b_exp >> 1;              // BIAS + e
  const bool eff_sub = sa != sb;
  bool a_big = wa > wb;
  if (wa == wb) {                                               // compare the mantissas
    int s = N - 1;
    while (s >= 0 && ra[s] == rb[s]) s--;
    if (s < 0) {
      if (eff_sub) return CLS_ZERO;                             // exact cancellation
      a_big = true;
    } else {
      a_big = ra[s] > rb[s];
    }
  }
  const uint32_t *big = a_big ? ra : rb, *sml = a_big ? rb : ra;
  const uint32_t sign = a_big ? sa : sb;
  const uint32_t wbig = a_big ? wa : wb, diff = a_big ? wa - wb : wb - wa;
  const uint32_t cap = 32u * N + 64u;
  const int d = (int)(diff > cap ? cap : diff);
  const int dw = d >> 5, db = d & 31;

  uint32_t bg[N];
#pragma unroll
  for (int s = 0; s < N; s += 4) {
    const uint4 v = *reinterpret_cast<const uint4 *>(big + s);
    bg[s] = v.x; bg[s + 1] = v.y; bg[s + 2] = v.z; bg[s + 3] = v.w;
  }
  // SMALL limbs dw-2 .. dw+N (0 outside the number)
  uint32_t w[N + 3];
#pragma unroll
  for (int j = 0; j < N + 3; j++) {
    const int k = j - 2 + dw;
    const uint32_t kc = min((uint32_t)k, (uint32_t)(N - 1));   // in the row whatever k is
    const uint32_t v = sml[kc];
    w[j] = (uint32_t)k < (uint32_t)N ? v : 0u;
  }
  // bits of SMALL below X limb 0 (d > 64): sticky, and one unit less for a subtraction
  uint32_t lost = 0;
  if (d > 64) {
    const int cut = d - 64, full = cut >> 5, part = cut & 31;
    uint32_t lv = 0;
    for (int k = 0; k < full && k < N; k++) lv |= sml[k];
    if (part && full < N) lv |= sml[full] & ((1u << part) - 1u);
    lost = lv != 0u ? 1u : 0u;
  }
  // X = BIG*2^64 + (T ^ msk) + (1 - lost for a subtraction), N+3 limbs
  const uint32_t msk = eff_sub ? 0xFFFFFFFFu : 0u;
  uint32_t x[N + 3];
  uint64_t acc = eff_sub ? (uint64_t)(1u - lost) : 0ull;
#pragma unroll
  for (int j = 0; j < N + 3; j++) {
    const uint32_t tj = (j < N + 2) ? __funnelshift_r(w[j], w[j + 1], db) : 0u;
    const uint32_t bj = (j >= 2 && j < N + 2) ? bg[j - 2] : 0u;
    acc += (uint64_t)bj + (tj ^ msk);
    x[j] = (uint32_t)acc;
    acc >>= 32;
  }
  if (eff_sub) x[N + 2] = 0u;                                   // the complement's wrap-around

  uint32_t mant[N], rbit = 0, st = 0;
  int L;
  if (x[N + 2] != 0u || (x[N + 1] >> 30) != 0u) {
    // no cancellation, a carry, or one bit of cancellation: the mantissa starts at bit 63,
    // 64 or 65 of X
    L = x[N + 2] ? 32 * (N + 2) + 32 - (int)clz32(x[N + 2]) : 32 * (N + 1) + 32 - (int)clz32(x[N + 1]);
    const int lo = L - 32 * N, lb = lo & 31;
    const bool w2 = (lo >> 5) == 2;
#pragma unroll
    for (int i = 0; i < N; i++) {
      const uint32_t p = w2 ? x[i + 2] : x[i + 1], q = w2 ? x[i + 3] : x[i + 2];
      mant[i] = __funnelshift_r(p, q, lb);
    }
    const int rp = lo - 1, rq = rp & 31;                        // rp in [62, 64]
    const uint32_t xr = (rp >> 5) == 2 ? x[2] : x[1];
    rbit = (xr >> rq) & 1u;
    st = (x[0] | ((rp >> 5) == 2 ? x[1] : 0u) | (xr & ((1u << rq) - 1u)) | lost) != 0u ? 1u : 0u;
  } else {
    // deep cancellation (an effective subtraction with d <= 1): X has no bits below bit 63,
    // so the result is exact.  X goes through the row to be read at a shifted offset.
    int top = -1;
#pragma unroll
    for (int j = 0; j < N + 2; j++) if (x[j]) top = j;
    if (top < 0) return CLS_ZERO;
#pragma unroll
    for (int j = 0; j < N + 3; j++) ra[j] = x[j];               // the row holds N+4 words
    const uint32_t xt = ra[top];
    L = 32 * top + 32 - (int)clz32(xt);
    const int lo = L - 32 * N, lw = lo >> 5, lb = lo & 31;      // lo < 63, may be negative
#pragma unroll
    for (int i = 0; i < N; i++) {
      const int k = i + lw;
      const uint32_t p = (uint32_t)k < (uint32_t)(N + 3) ? ra[min((uint32_t)k, (uint32_t)(N + 2))] : 0u;
      const uint32_t q = (uint32_t)(k + 1) < (uint32_t)(N + 3) ? ra[min((uint32_t)(k + 1), (uint32_t)(N + 2))] : 0u;
      mant[i] = __funnelshift_r(p, q, lb);
    }
  }
  // round: add one unit, carrying through the limbs
  uint32_t c = round_up(mode, sign, mant[0] & 1u, rbit, st) ? 1u : 0u;
#pragma unroll
  for (int i = 0; i < N; i++) {
    const uint32_t v = mant[i] + c;
    c = (c && v == 0u) ? 1u : 0u;
    mant[i] = v;
  }
  const int ovf = (int)c;                                       // 0.11..1 + ulp = 1.0
  if (ovf) mant[N - 1] = 0x80000000u;
  const long long be = (long long)wbig - 32LL * N - 64 + L + ovf;   // BIAS + e
  if (!eff_sub && be > 0x7FFFFFFFLL) return CLS_POS_INF - sign;
  if (eff_sub && be < 5) return CLS_POS_TINY - sign;
#pragma unroll
  for (int s = 0; s < N; s += 4)
    *reinterpret_cast<uint4 *>(ra + s) = make_uint4(mant[s], mant[s + 1], mant[s + 2], mant[s + 3]);
  return (uint32_t)(2 * be) + sign;
}

// mul of two rows by one thread: product scanning over the 2N-1 columns with a 96-bit
// (lo, hi, top) accumulator and compile-time indices; the limbs below the top N+2 of the
// product only feed the sticky bit.  The product of two normalised mantissas has its top
// bit at 64N-1 or 64N-2, so the mantissa is the top N limbs shifted by 0 or 1 bit.
// Reference: fpa_warp_mul.h:41-139 (one rounding; TINY when BIAS+e < 5, INF when
// BIAS+e > 0x7FFFFFFF, :124-128).
template <int N>
__device__ __forceinline__ uint32_t row_mul(uint32_t *ra, const uint32_t *rb, uint32_t a_exp, uint32_t b_exp,
                                            int mode) {
  const uint32_t act = c_action[2][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_MUL) return act;
  uint32_t a[N], b[N];
#pragma unroll
  for (int s = 0; s < N; s += 4) {
    const uint4 u = *reinterpret_cast<const uint4 *>(ra + s), v = *reinterpret_cast<const uint4 *>(rb + s);
    a[s] = u.x; a[s + 1] = u.y; a[s + 2] = u.z; a[s + 3] = u.w;
    b[s] = v.x; b[s + 1] = v.y; b[s + 2] = v.z; b[s + 3] = v.w;
  }
  uint32_t top[N + 2], low = 0, lo = 0, hi = 0, tp = 0;   // top[k] = product limb N-2+k
#pragma unroll
  for (int c = 0; c < 2 * N - 1; c++) {
#pragma unroll
    for (int i = (c < N ? 0 : c - N + 1); i <= (c < N ? c : N - 1); i++) mac3(lo, hi, tp, a[i], b[c - i]);
    if (c < N - 2) low |= lo;
    else top[c - (N - 2)] = lo;
    lo = hi; hi = tp; tp = 0;
  }
  top[N + 1] = lo;                                          // limb 2N-1
  const uint32_t sign = (a_exp ^ b_exp) & 1u;
  const bool full = (top[N + 1] >> 31) != 0u;               // top bit at 64N-1
  uint32_t mant[N];
#pragma unroll
  for (int i = 0; i < N; i++) mant[i] = full ? top[i + 2] : ((top[i + 2] << 1) | (top[i + 1] >> 31));
  // round bit: product bit 32N-1 (full) or 32N-2; sticky: everything below it
  const uint32_t rl = top[1];                               // limb N-1
  const uint32_t rbit = full ? (rl >> 31) : ((rl >> 30) & 1u);
  const uint32_t st = ((full ? (rl & 0x7FFFFFFFu) : (rl & 0x3FFFFFFFu)) | top[0] | low) != 0u ? 1u : 0u;
  uint32_t cy = round_up(mode, sign, mant[0] & 1u, rbit, st) ? 1u : 0u;
#pragma unroll
  for (int i = 0; i < N; i++) {
    const uint32_t v = mant[i] + cy;
    cy = (cy && v == 0u) ? 1u : 0u;
    mant[i] = v;
  }
  if (cy) mant[N - 1] = 0x80000000u;                        // 0.11..1 + ulp = 1.0
  const int L = full ? 64 * N : 64 * N - 1;
  const long long e = (long long)(a_exp >> 1) + (long long)(b_exp >> 1) - 2LL * BIAS - 64LL * N + L + (int)cy;
  if ((long long)BIAS + e < 5) return CLS_POS_TINY - sign;
  if ((long long)BIAS + e > 0x7FFFFFFFLL) return CLS_POS_INF - sign;
#pragma unroll
  for (int s = 0; s < N; s += 4)
    *reinterpret_cast<uint4 *>(ra + s) = make_uint4(mant[s], mant[s + 1], mant[s + 2], mant[s + 3]);
  return exp_word(e, sign);
}

// Copies of one warp's 32 operations from index `base` (cnt of them): limbs of a and b into
// rows, exponents beside them.  Unit u of the contiguous limbs is chunk r of operation o;
// (o, r) advance by 32 units per step without a division.
template <int N>
__device__ __forceinline__ void rows_stage(uint32_t *buf, const ElementwiseArgs &args, uint64_t base, int cnt,
                                           int lane, bool vec) {
  constexpr int S = RowSpace<N>::S;
  uint32_t *ra = buf, *rb = buf + 32 * S, *ea = buf + 64 * S, *eb = ea + 32;
  if (lane < cnt) {
    cp_async4(ea + lane, args.a_exps + base + lane);
    cp_async4(eb + lane, args.b_exps + base + lane);
  }
  const uint32_t *ga = args.a_limbs + base * N, *gb = args.b_limbs + base * N;
  if (vec) {
    constexpr int q = N / 4, d32 = 32 / q, m32 = 32 % q;
    int o = lane / q, r = lane % q;
    for (int u = lane; u < cnt * q; u += 32) {
      cp_async16(ra + o * S + 4 * r, ga + 4 * u);
      cp_async16(rb + o * S + 4 * r, gb + 4 * u);
      o += d32; r += m32;
      if (r >= q) { r -= q; o++; }
    }
  } else {
    constexpr int d32 = 32 / N, m32 = 32 % N;
    int o = lane / N, r = lane % N;
    for (int u = lane; u < cnt * N; u += 32) {
      cp_async4(ra + o * S + r, ga + u);
      cp_async4(rb + o * S + r, gb + u);
      o += d32; r += m32;
      if (r >= N) { r -= N; o++; }
    }
  }
}

template <int OP, int N>
__global__ void __launch_bounds__(128, 4) k_rows(ElementwiseArgs args) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int S = RowSpace<N>::S;
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
  uint32_t *wb = smem + (size_t)warp * RowSpace<N>::words;
  const bool vec = ((((uintptr_t)args.a_limbs) | ((uintptr_t)args.b_limbs) | ((uintptr_t)args.r_limbs)) & 15) == 0;
  const uint64_t nchunks = (args.count + 31) / 32;
  const uint64_t stride = (uint64_t)gridDim.x * (blockDim.x >> 5);
  uint64_t c = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (c < nchunks) rows_stage<N>(wb, args, c * 32, (int)min((uint64_t)32, args.count - c * 32), lane, vec);
  cp_async_commit();
  int cur = 0;
  for (; c < nchunks; c += stride) {
    const uint64_t nx = c + stride;
    if (nx < nchunks)
      rows_stage<N>(wb + (cur ^ 1) * RowSpace<N>::buf, args, nx * 32, (int)min((uint64_t)32, args.count - nx * 32),
                    lane, vec);
    cp_async_commit();
    cp_async_wait<1>();                                          // this chunk's copies have landed
    __syncwarp();
    uint32_t *buf = wb + cur * RowSpace<N>::buf;
    uint32_t *ra = buf, *rb = buf + 32 * S, *ea = buf + 64 * S, *eb = ea + 32;
    const uint64_t base = c * 32;
    const int cnt = (int)min((uint64_t)32, args.count - base);
    uint32_t rexp = 0;
    if (lane < cnt) {
      rexp = OP == OP_MUL ? row_mul<N>(ra + lane * S, rb + lane * S, ea[lane], eb[lane], args.mode)
                          : row_addsub<N>(ra + lane * S, rb + lane * S, ea[lane], eb[lane], args.mode, OP == OP_SUB);
      args.r_exps[base + lane] = rexp;
    }
    ea[lane] = rexp;                                             // read back by the copy-out below
    __syncwarp();
    // coalesced copy-out of the operations that produced limbs
    uint32_t *gr = args.r_limbs + base * N;
    if (vec) {
      constexpr int q = N / 4, d32 = 32 / q, m32 = 32 % q;
      int o = lane / q, r = lane % q;
      for (int u = lane; u < cnt * q; u += 32) {
        if (ea[o] > CLS_SNAN)
          __stcs(reinterpret_cast<uint4 *>(gr) + u, *reinterpret_cast<const uint4 *>(ra + o * S + 4 * r));
        o += d32; r += m32;
        if (r >= q) { r -= q; o++; }
      }
    } else {
      constexpr int d32 = 32 / N, m32 = 32 % N;
      int o = lane / N, r = lane % N;
      for (int u = lane; u < cnt * N; u += 32) {
        if (ea[o] > CLS_SNAN) gr[u] = ra[o * S + r];
        o += d32; r += m32;
        if (r >= N) { r -= N; o++; }
      }
    }
    __syncwarp();                                                // the buffer is refilled two chunks on
    cur ^= 1;
  }
  cp_async_wait<0>();
}

template <int OP, int N>
static cudaError_t launch_rows(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  constexpr int warps = 4;
  constexpr size_t smem = (size_t)warps * RowSpace<N>::words * sizeof(uint32_t);
  static int per_sm = 0;
  auto kern = k_rows<OP, N>;
  if (per_sm == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int b = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 32 * warps, smem)) != cudaSuccess) return e;
    per_sm = b < 1 ? 1 : b;
  }
  const uint64_t need = (args.count + 32 * warps - 1) / (32 * warps), cap = (uint64_t)sms * per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  kern<<<grid, 32 * warps, smem, stream>>>(args);
  return cudaGetLastError();
}

}  // namespace gfpa
