// fpa_device.cuh -- device-side building blocks for the GB300 fpa kernels.
//
// Number format (cuBigFloat fpa_internal.h:1-17, tests.c:114-159): one exponent word per
// instance (0..8 = class codes, otherwise bit 0 = sign and bits 31..1 = BIAS + e) and n
// little-endian 32-bit limbs with the top bit of limb n-1 set; value = +-M * 2^(e - 32n).
//
// Execution model: one *lane group* of G lanes (G in {4,8,16,32}, a slice of one warp)
// owns one operation at a time.  Operands are staged in the group's slice of shared
// memory; big-integer steps (products, adds, compares, rounding) are cooperative over
// the group, with carries resolved across lanes by ballot-based carry lookahead.
// Products use product scanning: the column blocks of K limbs are paired (t, t+M) so that
// every pair holds the same number of K x K tiles, each lane owns R such pairs (t = lane,
// lane+G, ...), and each column is accumulated in a 96-bit (lo, hi, top) register triple
// fed by mad.lo.cc / madc.hi.cc.  A group's capacity is N = G*K*R limbs (G*R <= 32).
#pragma once
#include <stdint.h>

namespace gfpa {

constexpr uint32_t BIAS = 0x3FFFFFF3u;

enum : uint32_t {
  CLS_POS_VALUE = 0, CLS_NEG_VALUE = 1, CLS_ZERO = 2, CLS_NEG_TINY = 3, CLS_POS_TINY = 4,
  CLS_NEG_INF = 5, CLS_POS_INF = 6, CLS_NAN = 7, CLS_SNAN = 8
};
enum : uint32_t {
  ACT_MUL = 16, ACT_DIV = 17, ACT_SQRT = 18, ACT_ADD = 20, ACT_SUB = 21,
  ACT_COPY_A = 22, ACT_COPY_B = 23, ACT_NEG_B = 24
};
enum : int { OP_ADD = 0, OP_SUB = 1, OP_MUL = 2, OP_DIV = 3, OP_SQRT = 4, OP_FMA = 5 };

// Special-value tables, rows = class of a, columns = class of b.  Same entries as the
// reference's tables (fpa_warp_add_sub.h:15-39, fpa_warp_mul.h:1-12, fpa_warp_div.h:1-12,
// fpa_warp_sqrt.h:1-11) so special operands give the same class results.
static __constant__ uint8_t c_action[4][81] = {
  { // add
    ACT_ADD, ACT_SUB, ACT_COPY_A, ACT_COPY_A, ACT_COPY_A, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    ACT_SUB, ACT_ADD, ACT_COPY_A, ACT_COPY_A, ACT_COPY_A, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    ACT_COPY_B, ACT_COPY_B, CLS_ZERO, CLS_NEG_TINY, CLS_POS_TINY, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    ACT_COPY_B, ACT_COPY_B, CLS_NEG_TINY, CLS_NEG_TINY, CLS_NAN, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    ACT_COPY_B, ACT_COPY_B, CLS_POS_TINY, CLS_NAN, CLS_POS_TINY, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_NAN, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN },
  { // sub
    ACT_SUB, ACT_ADD, ACT_COPY_A, ACT_COPY_A, ACT_COPY_A, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    ACT_ADD, ACT_SUB, ACT_COPY_A, ACT_COPY_A, ACT_COPY_A, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    ACT_NEG_B, ACT_NEG_B, CLS_ZERO, CLS_POS_TINY, CLS_NEG_TINY, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    ACT_NEG_B, ACT_NEG_B, CLS_NEG_TINY, CLS_NAN, CLS_NEG_INF, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    ACT_NEG_B, ACT_NEG_B, CLS_POS_TINY, CLS_POS_TINY, CLS_NAN, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NEG_INF, CLS_NAN, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_POS_INF, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN },
  { // mul
    ACT_MUL, ACT_MUL, CLS_ZERO, CLS_NEG_TINY, CLS_POS_TINY, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    ACT_MUL, ACT_MUL, CLS_ZERO, CLS_POS_TINY, CLS_NEG_TINY, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    CLS_ZERO, CLS_ZERO, CLS_ZERO, CLS_ZERO, CLS_ZERO, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_NEG_TINY, CLS_POS_TINY, CLS_ZERO, CLS_POS_TINY, CLS_NEG_TINY, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_POS_TINY, CLS_NEG_TINY, CLS_ZERO, CLS_NEG_TINY, CLS_POS_TINY, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_NAN, CLS_NAN, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_SNAN,
    CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN,
    CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN },
  { // div
    ACT_DIV, ACT_DIV, CLS_NAN, CLS_NEG_INF, CLS_POS_INF, CLS_NEG_TINY, CLS_POS_TINY, CLS_NAN, CLS_SNAN,
    ACT_DIV, ACT_DIV, CLS_NAN, CLS_POS_INF, CLS_NEG_INF, CLS_POS_TINY, CLS_NEG_TINY, CLS_NAN, CLS_SNAN,
    CLS_ZERO, CLS_ZERO, CLS_NAN, CLS_ZERO, CLS_ZERO, CLS_ZERO, CLS_ZERO, CLS_NAN, CLS_SNAN,
    CLS_NEG_TINY, CLS_POS_TINY, CLS_NAN, CLS_NAN, CLS_NAN, CLS_POS_TINY, CLS_NEG_TINY, CLS_NAN, CLS_SNAN,
    CLS_POS_TINY, CLS_NEG_TINY, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NEG_TINY, CLS_POS_TINY, CLS_NAN, CLS_SNAN,
    CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_POS_INF, CLS_NEG_INF, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_NAN, CLS_SNAN,
    CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN, CLS_SNAN },
};
static __constant__ uint8_t c_sqrt_action[9] = {
  ACT_SQRT, CLS_NAN, CLS_ZERO, CLS_NAN, CLS_POS_TINY, CLS_NAN, CLS_POS_INF, CLS_NAN, CLS_SNAN };

__device__ __forceinline__ uint32_t classify(uint32_t e) { return e <= CLS_SNAN ? e : (e & 1u); }

// Round-away decision from the bits below the kept mantissa (fpa_internal.h:62-88,
// restated on a round bit and a sticky flag).
__device__ __forceinline__ bool round_up(int mode, uint32_t sign, uint32_t lsb, uint32_t rbit, uint32_t sticky) {
  switch (mode) {
    case 1: return sign == 0 && (rbit | sticky) != 0;
    case 2: return sign != 0 && (rbit | sticky) != 0;
    case 3: return rbit != 0 && (sticky | lsb) != 0;
    case 4: return rbit != 0;
    default: return false;
  }
}

// ---------------------------------------------------------------------------------------
// lane group
template <int G>
struct Grp {
  uint32_t lane, base, mask;
  __device__ __forceinline__ Grp() {
    uint32_t wl = threadIdx.x & 31u;
    base = wl & ~(uint32_t)(G - 1);
    lane = wl - base;
    mask = (G == 32) ? 0xFFFFFFFFu : (((1u << G) - 1u) << base);
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ uint32_t ballot(bool p) const {
    uint32_t b = __ballot_sync(mask, p);
    return (G == 32) ? b : ((b >> base) & ((1u << G) - 1u));
  }
  __device__ __forceinline__ uint32_t bcast(uint32_t v, int src) const { return __shfl_sync(mask, v, src, G); }
  __device__ __forceinline__ uint32_t rmin(uint32_t v) const { return __reduce_min_sync(mask, v); }
  __device__ __forceinline__ uint32_t rmax(uint32_t v) const { return __reduce_max_sync(mask, v); }
  __device__ __forceinline__ uint32_t ror(uint32_t v) const { return __reduce_or_sync(mask, v); }
};

// carry lookahead over the G lanes: bit i of the result = carry into lane i.
// gm = lanes that generate a carry, pm = lanes that propagate one (and do not generate).
template <int G>
__device__ __forceinline__ uint64_t lookahead(uint32_t gm, uint32_t pm, uint32_t cin, uint32_t &cout) {
  uint64_t A = (uint64_t)(gm | pm), B = (uint64_t)gm;
  uint64_t S = A + B + (uint64_t)cin;
  cout = (uint32_t)(S >> G) & 1u;
  return S ^ A ^ B;
}

struct Zero { __device__ __forceinline__ uint32_t operator()(int) const { return 0; } };
struct Ptr {
  const uint32_t *p; int len;
  __device__ __forceinline__ uint32_t operator()(int i) const { return (i >= 0 && i < len) ? p[i] : 0u; }
};
// limbs of (p[0..len) << bits) for bits in [0, 31]
struct ShlBits {
  const uint32_t *p; int len; int bits;
  __device__ __forceinline__ uint32_t operator()(int i) const {
    uint32_t v = (i >= 0 && i < len) ? p[i] : 0u;
    if (bits == 0) return v;
    uint32_t w = (i - 1 >= 0 && i - 1 < len) ? p[i - 1] : 0u;
    return (v << bits) | (w >> (32 - bits));
  }
};
// limbs of floor(p[0..len) * 2^shift) for any signed shift (in bits)
struct Shifted {
  const uint32_t *p; int len; int shift;
  __device__ __forceinline__ uint32_t operator()(int i) const {
    int bp = 32 * i - shift;                     // bit position in p of this limb's bit 0
    int q = bp >> 5, r = bp & 31;                // arithmetic shift: floor
    uint32_t lo = (q >= 0 && q < len) ? p[q] : 0u;
    if (r == 0) return lo;
    uint32_t hi = (q + 1 >= 0 && q + 1 < len) ? p[q + 1] : 0u;
    return (lo >> r) | (hi << (32 - r));
  }
};

// dst[0..len) = x + y + cin (x, y functors of the limb index); returns the carry out.
// Blocked: lane t owns limbs [t*c, t*c+c).  dst may alias the storage read by x/y only
// at the same index.
template <int G, class X, class Y>
__device__ __forceinline__ uint32_t grp_add(const Grp<G> &g, uint32_t *dst, X x, Y y, int len, uint32_t cin) {
  int c = (len + G - 1) / G, lo = min(len, (int)g.lane * c), hi = min(len, lo + c);
  uint32_t carry = 0, all1 = 1;
  for (int i = lo; i < hi; i++) {
    uint64_t t = (uint64_t)x(i) + y(i) + carry;
    uint32_t v = (uint32_t)t;
    dst[i] = v; carry = (uint32_t)(t >> 32); all1 &= (v == 0xFFFFFFFFu);
  }
  uint32_t gm = g.ballot(carry != 0), pm = g.ballot(all1 && carry == 0), cout;
  uint64_t cv = lookahead<G>(gm, pm, cin, cout);
  if ((cv >> g.lane) & 1u)
    for (int i = lo; i < hi; i++) { uint32_t v = dst[i] + 1u; dst[i] = v; if (v) break; }
  g.sync();
  return cout;
}

// dst[0..len) = x - y - bin; returns the borrow out.
template <int G, class X, class Y>
__device__ __forceinline__ uint32_t grp_sub(const Grp<G> &g, uint32_t *dst, X x, Y y, int len, uint32_t bin) {
  int c = (len + G - 1) / G, lo = min(len, (int)g.lane * c), hi = min(len, lo + c);
  uint32_t borrow = 0, all0 = 1;
  for (int i = lo; i < hi; i++) {
    uint32_t xv = x(i), yv = y(i);
    uint32_t v = xv - yv - borrow;
    borrow = (xv < yv) || (xv == yv && borrow) ? 1u : 0u;
    dst[i] = v; all0 &= (v == 0u);
  }
  uint32_t gm = g.ballot(borrow != 0), pm = g.ballot(all0 && borrow == 0), bout;
  uint64_t cv = lookahead<G>(gm, pm, bin, bout);
  if ((cv >> g.lane) & 1u)
    for (int i = lo; i < hi; i++) { uint32_t v = dst[i]; dst[i] = v - 1u; if (v) break; }
  g.sync();
  return bout;
}

// compare two numbers given as functors over [0, len): -1, 0, 1 (group-uniform).
// Each lane reduces 2*(index+1) + (x > y) at its highest differing limb, so the one
// reduction yields both the top differing limb and the sign, and no lane reads the
// operands after it (a caller may overwrite them right away).
template <int G, class X, class Y>
__device__ __forceinline__ int grp_cmp(const Grp<G> &g, X x, Y y, int len) {
  uint32_t key = 0;
  for (int i = g.lane; i < len; i += G) {
    const uint32_t xv = x(i), yv = y(i);
    if (xv != yv) key = 2u * ((uint32_t)i + 1u) + (xv > yv ? 1u : 0u);
  }
  key = g.rmax(key);
  return key == 0 ? 0 : ((key & 1u) ? 1 : -1);
}

template <int G, class X>
__device__ __forceinline__ bool grp_is_zero(const Grp<G> &g, X x, int len) {
  uint32_t o = 0;
  for (int i = g.lane; i < len; i += G) o |= x(i);
  return g.ror(o) == 0;
}

template <int G, class X>
__device__ __forceinline__ void grp_copy(const Grp<G> &g, uint32_t *dst, X x, int len) {
  for (int i = g.lane; i < len; i += G) dst[i] = x(i);
  g.sync();
}

__device__ __forceinline__ uint32_t clz32(uint32_t v) { return (uint32_t)__clz((int)v); }

// ---------------------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async): add/sub stage the next operation's
// operands while they compute the current one, so loads stay in flight.
__device__ __forceinline__ void cp_async4(uint32_t *dst, const uint32_t *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t *dst, const uint32_t *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// wait until at most PENDING of this thread's committed groups are still in flight
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory"); }

// the group copies n limbs src -> dst asynchronously; vec: 16-byte pieces (n % 4 == 0 and
// both addresses 16-byte aligned)
template <int G>
__device__ __forceinline__ void grp_stage_async(const Grp<G> &g, uint32_t *dst, const uint32_t *src, int n, bool vec) {
  if (vec) {
    for (int c = g.lane; c < (n >> 2); c += G) cp_async16(dst + 4 * c, src + 4 * c);
  } else {
    for (int i = g.lane; i < n; i += G) cp_async4(dst + i, src + i);
  }
}

// ---------------------------------------------------------------------------------------
// Rounding of a nonnegative integer X[0..xlen) (shared memory) to n limbs.
// grp_round decides the rounding (group-uniform); store_limbs then writes the rounded
// limbs straight from X, so X must stay unchanged until the store.  Returns false when
// X == 0.  L = bit length of X; ovf = 1 when rounding carried into a new binade.
struct Rounded {
  const uint32_t *X; int xlen;
  int lo;          // bit index in X of the mantissa's bit 0
  int L, ovf;
  int up;          // add one unit in the last place
  uint32_t f;      // lowest limb that is not all ones (the one the increment stops at)
};

template <int G>
__device__ bool grp_round(const Grp<G> &g, const uint32_t *X, int xlen, int n, uint32_t sticky_in,
                          int mode, uint32_t sign, Rounded &out) {
  uint32_t top = 0;
  for (int i = g.lane; i < xlen; i += G) if (X[i]) top = (uint32_t)i + 1u;
  top = g.rmax(top);
  if (top == 0) return false;
  const int h = (int)top - 1;
  const int L = 32 * h + 32 - (int)clz32(X[h]);
  const int lo = L - 32 * n;
  const Shifted src{X, xlen, -lo};
  const int rp = lo - 1;                             // round bit position
  uint32_t rbit = 0, st = 0;
  if (rp >= 0) {
    rbit = (X[rp >> 5] >> (rp & 31)) & 1u;
    const int full = rp >> 5;                        // limbs fully below the round limb
    for (int i = g.lane; i < full; i += G) st |= X[i];
    if (g.lane == 0 && (rp & 31)) st |= X[full] & ((1u << (rp & 31)) - 1u);
  }
  st = g.ror(st) | sticky_in;
  const uint32_t lsb = src(0) & 1u;
  const int up = round_up(mode, sign, lsb, rbit, st != 0) ? 1 : 0;
  uint32_t f = (uint32_t)n;
  if (up) {
    for (int i = g.lane; i < n; i += G)
      if (src(i) != 0xFFFFFFFFu) { f = (uint32_t)i; break; }
    f = g.rmin(f);
  }
  out.X = X; out.xlen = xlen; out.lo = lo; out.L = L;
  out.up = up; out.f = f; out.ovf = (up && f == (uint32_t)n) ? 1 : 0;   // 0.11..1 + ulp = 1.0
  return true;
}

template <int G>
__device__ __forceinline__ void store_limbs(const Grp<G> &g, uint32_t *dst, int n, const Rounded &r) {
  const Shifted src{r.X, r.xlen, -r.lo};
  for (int i = g.lane; i < n; i += G) {
    uint32_t v = src(i);
    if (r.up) v = (i < (int)r.f) ? 0u : (i == (int)r.f ? v + 1u : v);
    if (r.ovf && i == n - 1) v = 0x80000000u;
    dst[i] = v;
  }
}

// ---------------------------------------------------------------------------------------
// Products of up to N = G*K*R limbs per operand.
//
// Layout of the per-group product scratch (32-bit words):
//   sa   : N          operand x, zero padded to Mp*K
//   sb   : N + 2K     operand y at offset K, K zero limbs below and above
//   snap : G*3K       per-lane snapshot of the first block's column sums (reused per pair)
//   ov   : 4GR        the two limbs above each column block's K limbs (2 per block)
// A block's own K limbs go straight to the product buffer P; limbs at or above the product
// length are never stored, so P needs room for the product only.
template <int G, int K, int R>
struct MulScratch {
  static_assert(G * R <= 32, "the block carry lookahead covers at most 64 column blocks");
  static constexpr int N = G * K * R;
  uint32_t *sa, *sb, *snap, *ov;
  __host__ __device__ static constexpr int words() { return N + (N + 2 * K) + G * 3 * K + 4 * G * R; }
  __device__ __forceinline__ void carve(uint32_t *p) {
    sa = p; sb = sa + N; snap = sb + N + 2 * K; ov = snap + G * 3 * K;
  }
};

__device__ __forceinline__ void mac3(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a, uint32_t b) {
  asm volatile("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
               "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
               "addc.u32 %2, %2, 0;"
               : "+r"(lo), "+r"(hi), "+r"(tp) : "r"(a), "r"(b));
}

// (lo,hi,tp)[c] columns -> K+2 limbs
template <int K>
__device__ __forceinline__ void columns_to_limbs(const uint32_t *lo, const uint32_t *hi, const uint32_t *tp, uint32_t *L) {
  uint64_t carry = 0;
#pragma unroll
  for (int j = 0; j < K + 2; j++) {
    uint64_t s = carry;
    if (j < K) s += lo[j];
    if (j >= 1 && j - 1 < K) s += hi[j - 1];
    if (j >= 2 && j - 2 < K) s += tp[j - 2];
    L[j] = (uint32_t)s; carry = s >> 32;
  }
}

template <int G, int K, int R>
__device__ __forceinline__ void blocks_final_sum_inl(const Grp<G> g, uint32_t *P, int outlen, int Mp,
                                                     const MulScratch<G, K, R> s);

// A column block's K+2 limbs: the low K to P at K*cb (those below the product length), the
// top two to ov[2cb..2cb+2).
template <int K>
__device__ __forceinline__ void emit_block(uint32_t *P, uint32_t *ov, int cb, int outlen, const uint32_t *L) {
#pragma unroll
  for (int j = 0; j < K; j++)
    if (K * cb + j < outlen) P[K * cb + j] = L[j];
  ov[2 * cb] = L[K];
  ov[2 * cb + 1] = L[K + 1];
}

// Product P[0..lx+ly) of x (staged in s.sa, Mp = ceil(lx/K) blocks, zero padded) and y
// (staged in s.sb at offset K, Mb = ceil(ly/K) <= Mp blocks, K zero limbs on each side).
// Pair t < Mp is column blocks t and t+Mp; lane l runs pairs l, l+G, ... in turn.  Block t
// holds min(t, Mb)+1 tiles and block t+Mp holds max(0, Mb-t), so every pair is exactly
// Mb+1 tile steps (for a square, Mp+1).  The first block's column sums are snapshotted at
// the pair's switch step (or after the loop when there is no second block) and the second
// block is acc - snapshot.
template <int G, int K, int R>
__device__ __forceinline__ void grp_mul_staged(const Grp<G> g, uint32_t *P, int lx, int ly, const MulScratch<G, K, R> s) {
  static_assert(K >= 2, "a column block must be at least 2 limbs wide");
  const int Mp = (lx + K - 1) / K, Mb = (ly + K - 1) / K;
  uint32_t *sn = s.snap + g.lane * 3 * K;
#pragma unroll 1
  for (int pr = 0; pr < R; pr++) {
    if (pr * G >= Mp) break;                     // uniform over the group
    const int t = (int)g.lane + pr * G;
    const bool act = t < Mp;
    const int n1 = (t < Mb ? t : Mb) + 1;        // tiles of block t
    const int I0 = t > Mb ? t - Mb : 0;
    uint32_t lo[K], hi[K], tp[K];
#pragma unroll
    for (int c = 0; c < K; c++) { lo[c] = 0; hi[c] = 0; tp[c] = 0; }
    if (act) {
      for (int st = 0; st <= Mb; st++) {
        const bool first = st < n1;
        const int I = first ? I0 + st : t + Mp - Mb + (st - n1);
        const int cb = first ? t : t + Mp;
        if (st == n1) {
#pragma unroll
          for (int c = 0; c < K; c++) { sn[c] = lo[c]; sn[K + c] = hi[c]; sn[2 * K + c] = tp[c]; }
        }
        uint32_t a[K], w[2 * K];
        const uint32_t *ap = s.sa + K * I;
        const uint32_t *wp = s.sb + K * (cb - I);      // w[m] = y[K(cb-I) - K + m]
        if constexpr (K % 4 == 0) {
#pragma unroll
          for (int i = 0; i < K; i += 4) {
            uint4 v = *reinterpret_cast<const uint4 *>(ap + i);
            a[i] = v.x; a[i + 1] = v.y; a[i + 2] = v.z; a[i + 3] = v.w;
          }
#pragma unroll
          for (int i = 0; i < 2 * K; i += 4) {
            uint4 v = *reinterpret_cast<const uint4 *>(wp + i);
            w[i] = v.x; w[i + 1] = v.y; w[i + 2] = v.z; w[i + 3] = v.w;
          }
        } else {
#pragma unroll
          for (int i = 0; i < K; i++) a[i] = ap[i];
#pragma unroll
          for (int i = 1; i < 2 * K; i++) w[i] = wp[i];
        }
        // column c of this block gets a[i] * y[K(cb-I) + c - i] = a[i] * w[K + c - i]
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
          for (int c = 0; c < K; c++) mac3(lo[c], hi[c], tp[c], a[i], w[K + c - i]);
      }
      // acc = blocks t + (t+Mp); snapshot = block t.  Emit both as K+2 limbs.
      if (n1 > Mb) {                             // no second block: snapshot = everything
#pragma unroll
        for (int c = 0; c < K; c++) { sn[c] = lo[c]; sn[K + c] = hi[c]; sn[2 * K + c] = tp[c]; }
      }
      uint32_t L[K + 2];
      // second block = acc - snapshot (exact: each column sum < 2^96)
#pragma unroll
      for (int c = 0; c < K; c++) {
        uint32_t a0 = sn[c], a1 = sn[K + c], a2 = sn[2 * K + c];
        asm("sub.cc.u32 %0, %0, %3;\n\tsubc.cc.u32 %1, %1, %4;\n\tsubc.u32 %2, %2, %5;"
            : "+r"(lo[c]), "+r"(hi[c]), "+r"(tp[c]) : "r"(a0), "r"(a1), "r"(a2));
      }
      const int outlen = lx + ly;
      columns_to_limbs<K>(lo, hi, tp, L);
      emit_block<K>(P, s.ov, t + Mp, outlen, L);
#pragma unroll
      for (int c = 0; c < K; c++) { lo[c] = sn[c]; hi[c] = sn[K + c]; tp[c] = sn[2 * K + c]; }
      columns_to_limbs<K>(lo, hi, tp, L);
      emit_block<K>(P, s.ov, t, outlen, L);
    }
  }
  g.sync();
  blocks_final_sum_inl<G, K, R>(g, P, lx + ly, Mp, s);
}

// square product of operands staged for m limbs each
template <int G, int K, int R>
__device__ __forceinline__ void grp_mulsq_staged(const Grp<G> g, uint32_t *P, int m, const MulScratch<G, K, R> s) {
  grp_mul_staged<G, K, R>(g, P, m, m, s);
}


// P[0..lx+ly) = x[0..lx) * y[0..ly) for functor operands (lx, ly <= G*K*R, any order): the
// longer one is staged as the block operand.
// Out-of-line product core for the operations that call it many times (div, sqrt): one
// copy of the unrolled tile loop keeps their code inside the instruction cache.
template <int G, int K, int R>
__device__ __noinline__ void grp_mul_call(const Grp<G> g, uint32_t *P, int lx, int ly, const MulScratch<G, K, R> s) {
  grp_mul_staged<G, K, R>(g, P, lx, ly, s);
}

template <int G, int K, int R, class X, class Y>
__device__ __forceinline__ void grp_mul(const Grp<G> &g, uint32_t *P, X x, int lx, Y y, int ly,
                                        const MulScratch<G, K, R> &s) {
  const bool swap = ly > lx;
  const int la = swap ? ly : lx, lb = swap ? lx : ly;
  const int Ma = (la + K - 1) / K, Mb = (lb + K - 1) / K;
  for (int i = g.lane; i < Ma * K; i += G) s.sa[i] = (i < la) ? (swap ? y(i) : x(i)) : 0u;
  for (int i = g.lane; i < Mb * K + 2 * K; i += G) {
    const int j = i - K;
    s.sb[i] = (j >= 0 && j < lb) ? (swap ? x(j) : y(j)) : 0u;
  }
  g.sync();
  grp_mul_call<G, K, R>(g, P, la, lb, s);
}

// Sum of the per-block partials into P[0..outlen): block cb = its K limbs (already in P)
// + the two limbs above block cb-1 (ov).  Each block is summed in place without its carry
// in; the carries between the 2*Mp <= 64 blocks come from one 64-bit lookahead over the
// generate / propagate ballots, and the (rare) blocks that receive one are incremented.
template <int G, int K, int R>
__device__ __forceinline__ void blocks_final_sum_inl(const Grp<G> g, uint32_t *P, int outlen, int Mp,
                                                     const MulScratch<G, K, R> s) {
  uint64_t Gm = 0, Pm = 0;
#pragma unroll
  for (int pr = 0; pr < R; pr++) {
    if (pr * G >= Mp) break;                     // uniform over the group
    const int t = (int)g.lane + pr * G;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int cb = t + half * Mp;
      uint32_t gen = 0, prop = 0;
      if (t < Mp) {
        uint32_t c0 = 0, c1 = 0;
        if (cb > 0) { c0 = s.ov[2 * (cb - 1)]; c1 = s.ov[2 * (cb - 1) + 1]; }
        uint64_t carry = 0;
        uint32_t all1 = 1u;
#pragma unroll
        for (int j = 0; j < K; j++) {
          const int idx = K * cb + j;
          const uint32_t pv = idx < outlen ? P[idx] : 0u;
          const uint64_t sum = (uint64_t)pv + carry + (j == 0 ? c0 : 0u) + (j == 1 ? c1 : 0u);
          const uint32_t v = (uint32_t)sum;
          carry = sum >> 32;
          all1 &= (v == 0xFFFFFFFFu);
          if (idx < outlen) P[idx] = v;
        }
        gen = (uint32_t)(carry != 0);
        prop = all1 && carry == 0;
      }
      const uint32_t bg = g.ballot(gen), bp = g.ballot(prop);
      const int sh = pr * G + half * Mp;         // bit of lane l = block l + sh
      if (sh < 64) { Gm |= (uint64_t)bg << sh; Pm |= (uint64_t)bp << sh; }
    }
  }
  const uint64_t A = Gm | Pm, B = Gm;
  const uint64_t cv = (A + B) ^ A ^ B;           // bit cb = carry into block cb
#pragma unroll
  for (int pr = 0; pr < R; pr++) {
    if (pr * G >= Mp) break;
    const int t = (int)g.lane + pr * G;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int cb = t + half * Mp;
      if (t < Mp && ((cv >> cb) & 1u)) {
        for (int j = 0; j < K; j++) {
          const int idx = K * cb + j;
          if (idx >= outlen) break;
          const uint32_t v = P[idx] + 1u;
          P[idx] = v;
          if (v) break;
        }
      }
    }
  }
  g.sync();
}

// P[0..2m) = x[0..m) * y[0..m) with x, y functors (any storage); m <= G*K*R
template <int G, int K, int R, class X, class Y>
__device__ __forceinline__ void grp_mulsq(const Grp<G> &g, uint32_t *P, X x, Y y, int m, const MulScratch<G, K, R> &s) {
  grp_mul<G, K, R>(g, P, x, m, y, m, s);
}

}  // namespace gfpa
