// fpa_thread_newton.cuh -- div and sqrt with one thread per operation.
//
// The lane-group div/sqrt (op_div / op_sqrt in fpa_ops.cuh) spend most of their time outside
// the limb products: staging operands, summing column blocks, syncing the group, and
// products whose column blocks leave some lanes idle.  Here every thread of a warp runs a
// whole operation of its own, so there is no cross-lane traffic, no sync and no idle lane;
// the 32 operations of a warp share one limb count and follow the same instruction stream.
//
// The method is that of op_div / op_sqrt: a Newton iteration for the reciprocal (div) or the
// reciprocal square root (sqrt) over levels 1 -> 2 -> 3 -> 5 -> ... -> h (the one-thread
// register levels up to SMALL_LEVEL limbs first), then one Karp-Markstein step that yields
// one limb more than the result, rounding decided from that extra limb when it lies at
// least 2^20 units from a rounding boundary, and otherwise the bounded exact correction.
// What differs is which limbs each product forms.  Every product here is restricted to the
// limbs that its consumer reads, plus GUARD limbs below them: the low columns of
// T = B_k' Y_k and of the Newton corrections, of q0 = A_top Y_h and of the final correction
// D Y_h are never formed (a dropped carry changes a kept limb by at most one unit), and the
// Karp-Markstein remainder D = A 2^96 - q0 B is a middle product of its dlen limbs, its
// sign read from its top bit (|D| stays about 31 bits below 2^(32 dlen)).  The integer
// steps are restated exactly by tests/test_km_error_bound.py, which checks that the
// extra-limb quotient and root stay within a few units of the exact values at every size,
// far inside the 2^20-unit margin; the exact correction is unchanged.  A 4096-bit division
// forms about 12K limb products this way, against 21.8K with whole products.
//
// Products are column-block product scans with an 8x8 register tile (96-bit column sums
// fed by mac3) and no bounds checks: tprod (one output block per pass, the tile loop
// unrolled twice so that the next tile's operands load while the current one multiplies,
// and tiles that would multiply zero guard limbs skip them), tprod2 (two output blocks per
// pass, mul's) and tsqr (a square on its symmetric half).  Every buffer a product reads
// sits in zero guard limbs, so the tiles may read past either end: an operand needs zeros
// in the 8 limbs below it and from its length to 8 limbs past its length rounded up to 8,
// and 8 more readable limbs beyond each of those (the next tile's loads and tprod2's wider
// window read them without using them).  The layouts below provide that, and
// tests/test_tile_products_host.py holds the three routines to it.
//
// Storage.  A thread's limb j of a buffer is at base[32*j] (the warp's 32 threads
// interleaved limb by limb, so the 32 threads reading one limb index touch 32 consecutive
// words).  Workspace (shared memory): two slots of N/2+8 limbs with zero guards, holding the
// Newton iterate and the residual, then q0 / S0.  Slab (global memory, one per CTA, laid
// out the same way): B and A (div) or Xh = floor(A 2^(32-odd)) (sqrt), staged once per
// operation from the caller's natural layout so that every later operand read is one
// coalesced warp load; the next iterate (copied back to shared memory at the end of each
// level), sqrt's V1 and the remainder D, which are only read as a product's first factor;
// and the extra-limb result Q' / S'.  Every product thus has its second factor, the one
// whose window moves with each tile, in shared memory, and a warp's workspace (23.5 KB at
// N = 128) leaves room for 9 warps per SM.
//
// Operands a, b and the result r are the caller's arrays in the natural layout (number i's
// limbs contiguous).  Reference semantics as op_div / op_sqrt: fpa_warp_div.h:127-201,
// fpa_warp_sqrt.h:195-254.
#pragma once
#include <type_traits>
#include "fpa_ops.cuh"

namespace gfpa {

constexpr int TS = 32;      // distance between a thread's consecutive limbs
constexpr int GUARD = 2;    // limbs formed below the lowest limb a short product keeps

template <int N>
struct TSpace {
  static constexpr int SLOT = N / 2 + 8;                       // limbs per slot (multiple of 8)
  // workspace (shared memory), in limbs: 8 readable + 8 zero | slot 0 | 8 zero | slot 2 |
  // 8 zero + 8 readable.  Slot 0 holds the Newton iterate, slot 2 the residual, then q0 / S0.
  static constexpr int Z0 = 16, Z2 = Z0 + SLOT + 8;
  static constexpr int words = Z2 + SLOT + 16;
  // slab (global memory), in limbs: 16 zero | B | 16 zero | A or Xh | 16 zero | Q' or S' |
  // slot 1 (the next iterate, sqrt's V1, then the remainder D: each read only as a product's
  // first factor) | 8 zero + 8 readable
  static constexpr int SB = 16, SA = SB + N + 16, SQ = SA + N + 16, S1 = SQ + N + 16;
  static constexpr int slab = S1 + SLOT + 16;
  static constexpr int min_limbs = 8;                          // smaller numbers keep the lane-group path
};

// Copies n limbs of a natural-layout number to a slab column (limb j at dst[TS*j]) and
// clears the 16 limbs above them, the zero guard that a buffer staged for a larger limb
// count may have left nonzero (a CTA of the batched form runs tasks of several sizes).
__device__ __forceinline__ void stage_limbs(uint32_t *dst, const uint32_t *src, int n) {
  for (int j = n; j < n + 16; j++) dst[TS * j] = 0u;
  if ((((uintptr_t)src) & 15) == 0 && (n & 3) == 0) {
    for (int j = 0; j < n; j += 4) {
      const uint4 v = *reinterpret_cast<const uint4 *>(src + j);
      dst[TS * j] = v.x; dst[TS * (j + 1)] = v.y; dst[TS * (j + 2)] = v.z; dst[TS * (j + 3)] = v.w;
    }
  } else {
    for (int j = 0; j < n; j++) dst[TS * j] = src[j];
  }
}

// ---- operand views ------------------------------------------------------------------------
struct PV {                     // a zero-guarded buffer: limb i at p[TS*i], read unchecked
  const uint32_t *p;
  __device__ __forceinline__ uint32_t get(int i) const { return p[TS * i]; }
};
struct VW {                     // any buffer: 0 outside [0, len)
  const uint32_t *p; int len;
  __device__ __forceinline__ uint32_t get(int i) const { return ((unsigned)i < (unsigned)len) ? p[TS * i] : 0u; }
};

__device__ __forceinline__ int rup8(int v) { return (v + 7) & ~7; }
// first 8-limb output block of a product restricted to its limbs from `keep` up
__device__ __forceinline__ int blk(int keep) { return max(0, keep - GUARD) >> 3; }
// zeros from limb len of a slot up to 8 limbs past len rounded up (the rest is a zero guard)
__device__ __forceinline__ void zero_tail(uint32_t *p, int len) {
  const int e = rup8(len) + 8;
  for (int i = len; i < e; i++) p[TS * i] = 0u;
}

// ---- product: output blocks [cb_lo, cb_hi) of x * y, 8 limbs at a time, lowest first -----
// Output block cb gathers x-block i times the y window y[8(cb-i)-8 .. 8(cb-i)+7] for every i
// with 0 <= cb-i <= My (My = y's block count), into 96-bit (lo, hi, top) column sums fed by
// mac3; the two limbs above a block carry into the next one (none into block cb_lo).
// sink(cb, L) receives limbs 8cb .. 8cb+7 in L[0..7].
//
// A block's first tile reads its window's upper half from y's zero guard when cb >= My, and
// its last tile (i = cb) reads the lower half from the guard below y; the 28 products of
// such a half are skipped (MASK 1 keeps column c of row r only for c < r, MASK 2 only for
// c >= r).  Measured at 4096 bits: div 5.30 -> 5.16 ms and sqrt 5.71 -> 5.51 ms per 2^20
// operations.  When x's last block holds 1 to 4 limbs, its rows 4..7 are zero guard: a
// tile of that block that is not an edge tile skips them (MASK 5).  (Loading the next block's first tile during the current block cost div and
// sqrt registers they lack; mul's short product runs on tprod2 below.)

// one 8x8 tile: column c gathers a[r] * w[OFF + 8 + c - r]
template <int MASK, int OFF = 0, int W>
__device__ __forceinline__ void tile_mac(uint32_t (&lo)[8], uint32_t (&hi)[8], uint32_t (&tp)[8], const uint32_t (&a)[8],
                                         const uint32_t (&w)[W]) {
#pragma unroll
  for (int r = 0; r < 8; r++)
#pragma unroll
    for (int c = 0; c < 8; c++)
      if (MASK == 0 || (MASK == 1 && c < r) || (MASK == 2 && c >= r) || (MASK == 3 && 2 * r < c) ||
          (MASK == 4 && 2 * r - c < 8) || (MASK == 5 && r < 4))
        mac3(lo[c], hi[c], tp[c], a[r], w[OFF + 8 + c - r]);
}

template <class X, class Y, class Sink>
__device__ __forceinline__ void tprod(const X &x, int lx, const Y &y, int ly, int cb_lo, int cb_hi, Sink &&sink) {
  const int Mx = (lx + 7) >> 3, My = (ly + 7) >> 3;
  const int Mo = min(Mx + My, cb_hi);
  const bool half_rows = (lx & 7) != 0 && (lx & 7) <= 4;           // x's last block: rows 4..7 zero
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int cb = cb_lo; cb < Mo; cb++) {
    uint32_t lo[8], hi[8], tp[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { lo[c] = 0u; hi[c] = 0u; tp[c] = 0u; }
    lo[0] = c0; lo[1] = c1;
    const int i0 = max(0, cb - My), i1 = min(cb, Mx - 1);
    uint32_t a[8], w[16];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = x.get(8 * i0 + r);
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = y.get(8 * (cb - i0) - 8 + m);
    // the next tile's operands load ahead of the math
    auto step = [&](int i, auto mask) {
      uint32_t an[8], wn[8];
#pragma unroll
      for (int r = 0; r < 8; r++) an[r] = x.get(8 * (i + 1) + r);
#pragma unroll
      for (int m = 0; m < 8; m++) wn[m] = y.get(8 * (cb - i - 2) + m);
      tile_mac<decltype(mask)::value>(lo, hi, tp, a, w);
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = an[r];
#pragma unroll
      for (int m = 0; m < 8; m++) { w[8 + m] = w[m]; w[m] = wn[m]; }
    };
    int i = i0;
    if (cb >= My) step(i++, std::integral_constant<int, 1>{});   // upper window half in the guard
    const int iend = i1 == cb ? i1 : i1 + 1;                       // i = cb: lower half in the guard
    const bool rows4 = half_rows && iend == Mx && i < iend;        // the loop ends on x's last block
#pragma unroll 2
    for (; i < iend - (rows4 ? 1 : 0); i++) step(i, std::integral_constant<int, 0>{});
    if (rows4) step(i++, std::integral_constant<int, 5>{});
    if (i1 == cb) tile_mac<2>(lo, hi, tp, a, w);
    uint32_t L[10];
    columns_to_limbs<8>(lo, hi, tp, L);
    sink(cb, L);
    c0 = L[8]; c1 = L[9];
  }
}

// ---- product, two output blocks per pass --------------------------------------------------
// The result of tprod, with blocks cb and cb+1 formed together: tile i of block cb+1 reads
// the y window 8 limbs above that of block cb, so one 24-limb window
// u = y[8(cb-i)-8 .. 8(cb-i)+15] serves both, each new 8 y limbs feed 128 products, and the
// two blocks' column sums are independent chains.  Block cb's first tile when cb >= My and
// block cb+1's last tile (i = cb+1) run alone, on their nonzero half; tiles of both blocks
// run whole.  Block cb+1 takes block cb's carry after its sums are formed.  A last unpaired
// block runs with whole tiles.  Measured at 4096 bits: mul's short product 2.03 -> 1.86 ms
// per 2^20 operations; div and sqrt (230 instead of about 200 registers, 8 warps per SM
// instead of 9) 5.15 -> 5.97 and 5.36 -> 6.41 ms, so they keep tprod.
template <class X, class Y, class Sink>
__device__ __forceinline__ void tprod2(const X &x, int lx, const Y &y, int ly, int cb_lo, int cb_hi, Sink &&sink) {
  const int Mx = (lx + 7) >> 3, My = (ly + 7) >> 3;
  const int Mo = min(Mx + My, cb_hi);
  uint32_t c0 = 0u, c1 = 0u;
  int cb = cb_lo;
  using I0 = std::integral_constant<int, 0>;
#pragma unroll 1
  for (; cb + 1 < Mo; cb += 2) {
    uint32_t lo[8], hi[8], tp[8], lo2[8], hi2[8], tp2[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { lo[c] = 0u; hi[c] = 0u; tp[c] = 0u; lo2[c] = 0u; hi2[c] = 0u; tp2[c] = 0u; }
    lo[0] = c0; lo[1] = c1;
    const int i0a = max(0, cb - My), i1a = min(cb, Mx - 1);
    const int i0b = max(0, cb + 1 - My), i1b = min(cb + 1, Mx - 1);
    uint32_t a[8], u[24];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = x.get(8 * i0a + r);
#pragma unroll
    for (int m = 0; m < 24; m++) u[m] = y.get(8 * (cb - i0a) - 8 + m);
    // kind 0: both blocks, 1: block cb alone (upper half of its window in the guard)
    auto step = [&](int i, auto kind) {
      uint32_t an[8], un[8];
#pragma unroll
      for (int r = 0; r < 8; r++) an[r] = x.get(8 * (i + 1) + r);
#pragma unroll
      for (int m = 0; m < 8; m++) un[m] = y.get(8 * (cb - i - 2) + m);
      constexpr int K = decltype(kind)::value;
      if constexpr (K == 0) {
        tile_mac<0, 0>(lo, hi, tp, a, u);
        tile_mac<0, 8>(lo2, hi2, tp2, a, u);
      } else {
        tile_mac<1, 0>(lo, hi, tp, a, u);
      }
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = an[r];
#pragma unroll
      for (int m = 23; m >= 8; m--) u[m] = u[m - 8];
#pragma unroll
      for (int m = 0; m < 8; m++) u[m] = un[m];
    };
    int i = i0a;
    if (i0a < i0b) step(i++, std::integral_constant<int, 1>{});
#pragma unroll 2
    for (; i <= i1a; i++) step(i, I0{});
    // block cb+1 alone at i = cb+1 (lower half of its window in the guard; no next tile to load)
    if (i1b > i1a) tile_mac<2, 8>(lo2, hi2, tp2, a, u);
    uint32_t L[10];
    columns_to_limbs<8>(lo, hi, tp, L);
    sink(cb, L);
    mac3(lo2[0], hi2[0], tp2[0], L[8], 1u);
    mac3(lo2[1], hi2[1], tp2[1], L[9], 1u);
    columns_to_limbs<8>(lo2, hi2, tp2, L);
    sink(cb + 1, L);
    c0 = L[8]; c1 = L[9];
  }
  if (cb < Mo) {
    uint32_t lo[8], hi[8], tp[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { lo[c] = 0u; hi[c] = 0u; tp[c] = 0u; }
    lo[0] = c0; lo[1] = c1;
    const int i0 = max(0, cb - My), i1 = min(cb, Mx - 1);
    uint32_t a[8], w[16];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = x.get(8 * i0 + r);
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = y.get(8 * (cb - i0) - 8 + m);
#pragma unroll 1
    for (int i = i0; i <= i1; i++) {
      uint32_t an[8], wn[8];
#pragma unroll
      for (int r = 0; r < 8; r++) an[r] = x.get(8 * (i + 1) + r);
#pragma unroll
      for (int m = 0; m < 8; m++) wn[m] = y.get(8 * (cb - i - 2) + m);
      tile_mac<0>(lo, hi, tp, a, w);
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = an[r];
#pragma unroll
      for (int m = 0; m < 8; m++) { w[8 + m] = w[m]; w[m] = wn[m]; }
    }
    uint32_t L[10];
    columns_to_limbs<8>(lo, hi, tp, L);
    sink(cb, L);
  }
}

// ---- square: output blocks [0, cb_hi) of x * x -------------------------------------------
// The tiles of tprod(x, x) pair limbs a (x-block i) and b = 8(cb-i) + c - r.  In block cb,
// the tiles with i < floor(cb/2) hold only pairs a < b and are summed once, then doubled;
// those with i > cb/2 hold only their mirror images (a > b) and are skipped.  The tile
// i = floor(cb/2) holds both and a = b: MASK 3 (even cb) or 4 (odd cb) keeps its a < b
// pairs before the doubling, the squares x_a^2 are added after it, then the carry from the
// block below.  About half of tprod's products.
template <class X, class Sink>
__device__ __forceinline__ void tsqr(const X &x, int lx, int cb_hi, Sink &&sink) {
  const int Mx = (lx + 7) >> 3;
  const int Mo = min(2 * Mx, cb_hi);
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int cb = 0; cb < Mo; cb++) {
    uint32_t lo[8], hi[8], tp[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { lo[c] = 0u; hi[c] = 0u; tp[c] = 0u; }
    const int i0 = max(0, cb - Mx), id = cb >> 1;
    uint32_t a[8], w[16];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = x.get(8 * i0 + r);
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = x.get(8 * (cb - i0) - 8 + m);
    auto step = [&](int i, auto mask) {
      uint32_t an[8], wn[8];
#pragma unroll
      for (int r = 0; r < 8; r++) an[r] = x.get(8 * (i + 1) + r);
#pragma unroll
      for (int m = 0; m < 8; m++) wn[m] = x.get(8 * (cb - i - 2) + m);
      tile_mac<decltype(mask)::value>(lo, hi, tp, a, w);
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = an[r];
#pragma unroll
      for (int m = 0; m < 8; m++) { w[8 + m] = w[m]; w[m] = wn[m]; }
    };
    int i = i0;
    if (i < id && cb >= Mx) step(i++, std::integral_constant<int, 1>{});   // upper window half in the guard
#pragma unroll 2
    for (; i < id; i++) step(i, std::integral_constant<int, 0>{});
    if (cb & 1) tile_mac<4>(lo, hi, tp, a, w);
    else tile_mac<3>(lo, hi, tp, a, w);
#pragma unroll
    for (int c = 0; c < 8; c++) {                     // double the (top, hi, lo) column sums
      tp[c] = (tp[c] << 1) | (hi[c] >> 31);
      hi[c] = (hi[c] << 1) | (lo[c] >> 31);
      lo[c] <<= 1;
    }
    if (cb & 1) {                                     // x_a^2 lands in column 2a - 8cb
#pragma unroll
      for (int r = 4; r < 8; r++) mac3(lo[2 * r - 8], hi[2 * r - 8], tp[2 * r - 8], a[r], a[r]);
    } else {
#pragma unroll
      for (int r = 0; r < 4; r++) mac3(lo[2 * r], hi[2 * r], tp[2 * r], a[r], a[r]);
    }
    mac3(lo[0], hi[0], tp[0], c0, 1u);
    mac3(lo[1], hi[1], tp[1], c1, 1u);
    uint32_t L[10];
    columns_to_limbs<8>(lo, hi, tp, L);
    sink(cb, L);
    c0 = L[8]; c1 = L[9];
  }
}

// ---- rounding: X (xlen limbs, stride TS) to n limbs, written to r (natural layout) --------
// X must have at least 32n+1 significant bits.  sticky_in: a nonzero part lies below X.
// Returns X's bit length; ovf = 1 when rounding up carried into a new binade (the stored
// mantissa is then 0.1000...).  Same decision as grp_round / store_limbs.
__device__ __forceinline__ int tround_store(const uint32_t *X, int xlen, int n, uint32_t sticky_in, int mode,
                                            uint32_t sign, uint32_t *r, int &ovf) {
  int h = xlen - 1;
  while (h > 0 && X[TS * h] == 0u) h--;
  const int L = 32 * h + 32 - (int)clz32(X[TS * h]);
  const int lo = L - 32 * n;                         // bit of X that becomes the mantissa's bit 0
  const int rp = lo - 1, rq = rp >> 5, rs = rp & 31;
  const uint32_t rbit = (X[TS * rq] >> rs) & 1u;
  uint32_t st = sticky_in | (rs ? (X[TS * rq] & ((1u << rs) - 1u)) : 0u);
  for (int i = 0; i < rq; i++) st |= X[TS * i];
  const int q = lo >> 5, s = lo & 31;
  const uint32_t lsb = (X[TS * q] >> s) & 1u;
  uint32_t carry = round_up(mode, sign, lsb, rbit, st) ? 1u : 0u;
  uint32_t cur = X[TS * q];
  auto limb = [&](int i) {                           // mantissa limb i, rounded
    const uint32_t nxt = (q + i + 1 < xlen) ? X[TS * (q + i + 1)] : 0u;
    uint32_t v = s ? ((cur >> s) | (nxt << (32 - s))) : cur;
    v += carry;
    carry = (carry && v == 0u) ? 1u : 0u;
    cur = nxt;
    return v;
  };
  if ((((uintptr_t)r) & 15) == 0 && (n & 3) == 0) {  // 16-byte stores: a quarter of the transactions
    for (int i = 0; i < n; i += 4) {
      const uint32_t v0 = limb(i), v1 = limb(i + 1), v2 = limb(i + 2), v3 = limb(i + 3);
      *reinterpret_cast<uint4 *>(r + i) = make_uint4(v0, v1, v2, v3);
    }
  } else {
    for (int i = 0; i < n; i++) r[i] = limb(i);
  }
  ovf = (int)carry;
  if (carry) {                                       // 0.11..1 + ulp = 1.0
    for (int i = 0; i < n - 1; i++) r[i] = 0u;
    r[n - 1] = 0x80000000u;
  }
  return L;
}

// ---- div ---------------------------------------------------------------------------------
// Returns 0 when the result is written, 1 when the extra-limb quotient lies within the
// rounding margin and `exact` is false: the operation then needs the exact correction
// (the caller runs it again with exact = true; nothing has been written).
// w: this thread's workspace (zero-initialised guards); slab: its slab column.
template <int N>
__device__ int tdiv(uint32_t *w, uint32_t *slab, int n, int mode, uint32_t a_exp, const uint32_t *a, uint32_t b_exp,
                    const uint32_t *b, uint32_t *r_exp, uint32_t *r, bool exact, uint32_t *err) {
  using S = TSpace<N>;
  const uint32_t act = c_action[3][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_DIV) { *r_exp = act; return 0; }
  uint32_t *SA = slab + TS * S::SA, *SB = slab + TS * S::SB, *Q = slab + TS * S::SQ;
  stage_limbs(SA, a, n);
  stage_limbs(SB, b, n);
  int lv[24];
  const int nl = newton_levels(n, lv);
  const int l0 = small_levels_end(lv, nl, true);
  uint32_t *Y = w + TS * S::Z0, *Y2 = slab + TS * S::S1, *E = w + TS * S::Z2;
  {
    const uint64_t y = 0xFFFFFFFFFFFFFFFFull / (uint64_t)SB[TS * (n - 1)];   // level 1: floor((2^64-1)/B_top)
    uint32_t v[SMALL_LEVEL + 1], bt[SMALL_LEVEL];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) v[i] = 0u;
    v[0] = (uint32_t)y; v[1] = (uint32_t)(y >> 32);
#pragma unroll
    for (int i = 0; i < SMALL_LEVEL; i++) bt[i] = (n - SMALL_LEVEL + i >= 0) ? SB[TS * (n - SMALL_LEVEL + i)] : 0u;
    small_levels<false>(bt, lv, l0, v);
    const int k = lv[l0 - 1];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) if (i <= k) Y[TS * i] = v[i];
    zero_tail(Y, k + 1);
  }
  for (int li = l0; li < nl - 1; li++) {
    const int k = lv[li - 1], kp = lv[li], L = k + kp, lt = kp - k + 3;
    // T = B_k' Y_k ~ 2^(32L): E = its limbs k-1 .. kp+1, T[L] = 1 when T >= 2^(32L)
    uint32_t tL = 0u;
    tprod(PV{SB + TS * (n - kp)}, kp, PV{Y}, k + 1, blk(k - 1), L / 8 + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int j = 8 * cb + q - (k - 1);
        if (j >= 0 && j < lt) E[TS * j] = o[q];
        if (8 * cb + q == L) tL = o[q];
      }
    });
    const bool neg = tL != 0u;
    if (!neg)                                        // |2^(32L) - T| ~ complement (one unit low)
      for (int j = 0; j < lt; j++) E[TS * j] = ~E[TS * j];
    zero_tail(E, lt);
    // Y_k' = Y_k 2^(32(k'-k)) +- M,  M = (Y_k |E|) >> 32(k+1),  over k'+1 limbs
    uint32_t cy = 0u;
    int next = 0;                                    // next limb of Y_k' to form
    auto put = [&](int i, uint32_t mv) {
      const uint32_t ys = (i >= kp - k) ? Y[TS * (i - (kp - k))] : 0u;
      uint32_t v;
      if (neg) { v = ys - mv - cy; cy = (ys < mv || (ys == mv && cy)) ? 1u : 0u; }
      else { const uint64_t t = (uint64_t)ys + mv + cy; v = (uint32_t)t; cy = (uint32_t)(t >> 32); }
      Y2[TS * i] = v;
    };
    tprod(PV{Y}, k + 1, PV{E}, lt, blk(k + 1), (k + 1 + lt + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - (k + 1);
        if (i >= 0 && i < lt) { put(i, o[q]); next = i + 1; }
      }
    });
    for (int i = next; i <= kp; i++) put(i, 0u);
    for (int i = 0; i <= kp; i++) Y[TS * i] = Y2[TS * i];       // back to shared memory
    zero_tail(Y, kp + 1);
  }
  // Karp-Markstein step with one limb more than the result (op_div): h = the last Newton
  // level, m = n+2-h.  q0 = floor(A_top Y / 2^(32(h+1))), A_top = the top m+1 limbs of A.
  const int h = lv[nl - 2], m = n + 2 - h;
  uint32_t *q0 = E, *D = Y2;
  tprod(PV{SA + TS * (n - m - 1)}, m + 1, PV{Y}, h + 1, blk(h + 1), (h + m + 9) / 8,
        [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const int j = 8 * cb + q - (h + 1);
            if (j >= 0 && j <= m) q0[TS * j] = o[q];
          }
        });
  zero_tail(q0, m + 1);
  // D = A 2^96 - floor(q0 B / 2^(32(n-h-1))) mod 2^(32 dlen): the product's limbs sh .. sh+dlen-1
  const int dlen = m + 2, sh = n - h - 1;
  uint32_t bw = 0u;
  tprod(PV{q0}, m + 1, PV{SB}, n, blk(sh), (sh + dlen + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q - sh;
      if (i >= 0 && i < dlen) {
        const uint32_t xa = i >= 3 ? SA[TS * (i - 3)] : 0u, xq = o[q];
        D[TS * i] = xa - xq - bw;
        bw = (xa < xq || (xa == xq && bw)) ? 1u : 0u;
      }
    }
  });
  const bool dneg = (D[TS * (dlen - 1)] >> 31) != 0u;
  if (dneg) {                                        // D = -D (mod 2^(32 dlen))
    uint32_t c = 1u;
    for (int i = 0; i < dlen; i++) { const uint32_t v = ~D[TS * i] + c; c = (c && v == 0u) ? 1u : 0u; D[TS * i] = v; }
  }
  zero_tail(D, dlen);
  // Q' = q0 2^(32(h-1)) +- floor(D Y / 2^(32(h+2))),  n+2 limbs, into the slab
  uint32_t cq = 0u;
  int nextq = 0;
  auto putq = [&](int i, uint32_t c) {
    const uint32_t qv = (i >= h - 1) ? q0[TS * (i - (h - 1))] : 0u;
    uint32_t v;
    if (dneg) { v = qv - c - cq; cq = (qv < c || (qv == c && cq)) ? 1u : 0u; }
    else { const uint64_t t = (uint64_t)qv + c + cq; v = (uint32_t)t; cq = (uint32_t)(t >> 32); }
    Q[TS * i] = v;
  };
  tprod(PV{D}, dlen, PV{Y}, h + 1, blk(h + 2), (dlen + h + 8) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q - (h + 2);
      if (i >= 0 && i < n + 2) { putq(i, o[q]); nextq = i + 1; }
    }
  });
  for (int i = nextq; i < n + 2; i++) putq(i, 0u);
  const uint32_t sign = (a_exp ^ b_exp) & 1u;
  {
    const uint32_t qtop = Q[TS * (n + 1)], q0w = Q[0];
    const uint32_t u = qtop ? q0w : (q0w & 0x7FFFFFFFu), umax = qtop ? 0xFFFFFFFFu : 0x7FFFFFFFu;
    if (u >= (1u << 20) && u <= umax - (1u << 20)) {
      int ovf;
      const int Lb = tround_store(Q, n + 2, n, 1u, mode, sign, r, ovf);
      const long long e = (long long)(a_exp >> 1) - (long long)(b_exp >> 1) - 32LL * n - 32 + Lb + ovf;
      if ((long long)BIAS + e < 10) *r_exp = CLS_POS_TINY - sign;
      else if ((long long)BIAS + e >= 0x7FFFFFFFLL) *r_exp = CLS_POS_INF - sign;
      else *r_exp = exp_word(e, sign);
      return 0;
    }
  }
  if (!exact) return 1;
  // exact correction: Qc = floor(Q'/2^32) (n+1 limbs, from limb 1 of Q'),
  // Rm = (A 2^(32n) - Qc B) mod 2^(32(n+2)) over slots 0 and 2 (the guard limbs between
  // them are cleared again at the end)
  uint32_t *Qc = Q + TS, *Rm = w + TS * S::Z0;
  const uint32_t qt = Qc[TS * n];
  uint32_t c1 = 0u, b2 = 0u;
  auto putr = [&](int i, uint32_t p) {
    // P2 = Qc[0..n) B + (qt B) 2^(32n): add the small multiple, then subtract from A 2^(32n)
    uint32_t smv = 0u;                               // (qt B) 2^(32n), qt in {0, 1, 2, 4}
    if (i >= n && qt) {
      const int t = i - n;
      const uint32_t v = t < n ? SB[TS * t] : 0u, wv = (t >= 1 && t - 1 < n) ? SB[TS * (t - 1)] : 0u;
      smv = qt == 1 ? v : (qt == 2 ? ((v << 1) | (wv >> 31)) : ((v << 2) | (wv >> 30)));
    }
    const uint64_t t = (uint64_t)p + smv + c1;
    const uint32_t pv = (uint32_t)t;
    c1 = (uint32_t)(t >> 32);
    const uint32_t av = (i >= n && i - n < n) ? SA[TS * (i - n)] : 0u;
    const uint32_t v = av - pv - b2;
    b2 = (av < pv || (av == pv && b2)) ? 1u : 0u;
    Rm[TS * i] = v;
  };
  int nextr = 0;
  tprod(VW{Qc, n}, n, VW{SB, n}, n, 0, (n + 2 + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q;
      if (i < n + 2) { putr(i, o[q]); nextr = i + 1; }
    }
  });
  for (int i = nextr; i < n + 2; i++) putr(i, 0u);
  // 0 <= Rm < B, Qc stepped alongside (bounded; a hit bound sets the error word)
  int guard = 0;
  while ((Rm[TS * (n + 1)] >> 31) != 0u && guard < 64) {
    uint32_t bq = 1u;
    for (int i = 0; i <= n && bq; i++) { const uint32_t v = Qc[TS * i]; Qc[TS * i] = v - 1u; bq = v == 0u; }
    uint32_t c = 0u;
    for (int i = 0; i < n + 2; i++) {
      const uint64_t t = (uint64_t)Rm[TS * i] + (i < n ? SB[TS * i] : 0u) + c;
      Rm[TS * i] = (uint32_t)t; c = (uint32_t)(t >> 32);
    }
    guard++;
  }
  for (;;) {
    int cmp = 0;
    for (int i = n + 1; i >= 0 && cmp == 0; i--) {
      const uint32_t x = Rm[TS * i], y = i < n ? SB[TS * i] : 0u;
      if (x != y) cmp = x > y ? 1 : -1;
    }
    if (cmp < 0 || guard >= 64) break;
    uint32_t cq2 = 1u;
    for (int i = 0; i <= n && cq2; i++) { const uint32_t v = Qc[TS * i] + 1u; Qc[TS * i] = v; cq2 = v == 0u; }
    uint32_t bb = 0u;
    for (int i = 0; i < n + 2; i++) {
      const uint32_t x = Rm[TS * i], y = i < n ? SB[TS * i] : 0u;
      Rm[TS * i] = x - y - bb;
      bb = (x < y || (x == y && bb)) ? 1u : 0u;
    }
    guard++;
  }
  if (guard >= 64) atomicOr(err, 1u);
  // round bit: 2Rm >= B;  sticky: Rm != 0 and 2Rm != B (2Rm == B is impossible here)
  int c2 = 0;
  uint32_t nz = 0u;
  for (int i = n + 1; i >= 0; i--) {
    const uint32_t x = (Rm[TS * i] << 1) | (i > 0 ? (Rm[TS * (i - 1)] >> 31) : 0u), y = i < n ? SB[TS * i] : 0u;
    nz |= Rm[TS * i];
    if (c2 == 0 && x != y) c2 = x > y ? 1 : -1;
  }
  for (int i = S::SLOT; i < S::SLOT + 8; i++) Rm[TS * i] = 0u;   // the guard limbs between slots 0 and 2
  const uint32_t rb = c2 >= 0 ? 1u : 0u, sticky = (nz != 0u && c2 != 0) ? 1u : 0u;
  // X = 2Qc + rb, n+2 limbs, formed in place one limb below Qc (limb i of X over limb i of Q')
  uint32_t *X = Q;
  for (int i = 0; i < n + 2; i++) {
    const uint32_t qi = i <= n ? Qc[TS * i] : 0u, qm = i > 0 ? Qc[TS * (i - 1)] : 0u;
    X[TS * i] = (qi << 1) | (i > 0 ? (qm >> 31) : rb);
  }
  int ovf;
  const int Lb = tround_store(X, n + 2, n, sticky, mode, sign, r, ovf);
  const long long e = (long long)(a_exp >> 1) - (long long)(b_exp >> 1) - 32LL * n - 1 + Lb + ovf;
  if ((long long)BIAS + e < 10) *r_exp = CLS_POS_TINY - sign;
  else if ((long long)BIAS + e >= 0x7FFFFFFFLL) *r_exp = CLS_POS_INF - sign;
  else *r_exp = exp_word(e, sign);
  return 0;
}

// ---- sqrt --------------------------------------------------------------------------------
// Same return convention as tdiv.  Steps of op_sqrt: A_ext = A 2^(32n - odd), Xh = its top
// n+1 limbs, Newton on 1/sqrt with three products per level, the Karp-Markstein step with
// one limb more, the exact correction with R = A_ext - S^2.
template <int N>
__device__ int tsqrt(uint32_t *w, uint32_t *slab, int n, int mode, uint32_t a_exp, const uint32_t *a, uint32_t *r_exp,
                     uint32_t *r, bool exact, uint32_t *err) {
  using S = TSpace<N>;
  const uint32_t act = c_sqrt_action[classify(a_exp)];
  if (act != ACT_SQRT) { *r_exp = act; return 0; }
  const long long e = (long long)(a_exp >> 1) - BIAS;
  const int odd = (int)(e & 1);
  const long long eh = (e + odd) / 2;
  uint32_t *X = slab + TS * S::SA, *Sq = slab + TS * S::SQ;
  // Xh = floor(A * 2^(32 - odd)), n+1 limbs, staged in the slab
  {
    uint32_t prev = 0u;
    for (int j = 0; j < n; j++) {
      const uint32_t cur = a[j];
      X[TS * j] = odd ? ((prev >> 1) | (cur << 31)) : prev;
      prev = cur;
    }
    X[TS * n] = odd ? (prev >> 1) : prev;
    for (int j = n + 1; j < n + 16; j++) X[TS * j] = 0u;     // the zero guard above Xh
  }
  int lv[24];
  const int nl = newton_levels(n, lv);
  const int l0 = small_levels_end(lv, nl, true);
  uint32_t *Z = w + TS * S::Z0, *Z2 = slab + TS * S::S1, *E = w + TS * S::Z2;
  {
    const uint64_t x1 = (uint64_t)X[TS * n] << 32;
    const uint64_t s1 = isqrt64(x1);
    const uint64_t z = 0xFFFFFFFFFFFFFFFFull / s1;
    uint32_t v[SMALL_LEVEL + 1], xt[SMALL_LEVEL];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) v[i] = 0u;
    v[0] = (uint32_t)z; v[1] = (uint32_t)(z >> 32);
#pragma unroll
    for (int i = 0; i < SMALL_LEVEL; i++) xt[i] = (n + 1 - SMALL_LEVEL + i >= 0) ? X[TS * (n + 1 - SMALL_LEVEL + i)] : 0u;
    small_levels<true>(xt, lv, l0, v);
    const int k = lv[l0 - 1];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) if (i <= k) Z[TS * i] = v[i];
    zero_tail(Z, k + 1);
  }
  for (int li = l0; li < nl - 1; li++) {
    const int k = lv[li - 1], kp = lv[li];
    const int j = k > 2 ? k - 2 : 0, l1 = kp + k + 1 - j, L = kp + 2 * k - j, lt = kp - k + 3, off = 2 * k - 1 - j;
    uint32_t *V1s = Z2;
    // V1 = X_k' Z_k, its limbs j .. j+l1-1
    tprod(PV{X + TS * (n + 1 - kp)}, kp, PV{Z}, k + 1, blk(j), (j + l1 + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - j;
        if (i >= 0 && i < l1) V1s[TS * i] = o[q];
      }
    });
    zero_tail(V1s, l1);
    // W = (V1 >> 32j) Z_k ~ 2^(32L): E = its limbs off .. off+lt-1, W[L] = 1 when W >= 2^(32L)
    uint32_t wL = 0u;
    tprod(PV{V1s}, l1, PV{Z}, k + 1, blk(off), L / 8 + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - off;
        if (i >= 0 && i < lt) E[TS * i] = o[q];
        if (8 * cb + q == L) wL = o[q];
      }
    });
    const bool neg = wL != 0u;
    if (!neg)
      for (int i = 0; i < lt; i++) E[TS * i] = ~E[TS * i];
    zero_tail(E, lt);
    // Z_k' = Z_k 2^(32(k'-k)) +- M,  M = (Z_k |E|) >> (32(k+1)+1),  over k'+1 limbs (into V1s' slot)
    uint32_t cy = 0u, prev = 0u;
    int next = 0;
    auto put = [&](int i, uint32_t mv) {
      const uint32_t zs = (i >= kp - k) ? Z[TS * (i - (kp - k))] : 0u;
      uint32_t v;
      if (neg) { v = zs - mv - cy; cy = (zs < mv || (zs == mv && cy)) ? 1u : 0u; }
      else { const uint64_t t = (uint64_t)zs + mv + cy; v = (uint32_t)t; cy = (uint32_t)(t >> 32); }
      Z2[TS * i] = v;
    };
    // M[i] = (P[k+1+i] >> 1) | (P[k+2+i] << 31): formed when P[k+2+i] arrives (the limbs of
    // the last block past the product's end are 0)
    tprod(PV{Z}, k + 1, PV{E}, lt, blk(k + 1), 1 << 20, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - (k + 2);
        if (i >= 0 && i <= kp) { put(i, (prev >> 1) | (o[q] << 31)); next = i + 1; }
        prev = o[q];
      }
    });
    for (int i = next; i <= kp; i++) put(i, i == next ? (prev >> 1) : 0u);
    for (int i = 0; i <= kp; i++) Z[TS * i] = Z2[TS * i];       // back to shared memory
    zero_tail(Z, kp + 1);
  }
  // Karp-Markstein with one limb more (op_sqrt): S0 = floor(Xt Z / 2^(32(h+1))),
  // Xt = the top m+1 limbs of Xh
  const int h = lv[nl - 2], m = n + 2 - h;
  uint32_t *S0 = E, *D = Z2;
  tprod(PV{X + TS * (n - m)}, m + 1, PV{Z}, h + 1, blk(h + 1), (h + m + 9) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q - (h + 1);
      if (i >= 0 && i <= m) S0[TS * i] = o[q];
    }
  });
  zero_tail(S0, m + 1);
  // D = Xh 2^96 - S0^2 2^(32(2h-n)) mod 2^(32 dlen): the square's limbs below dlen - ssh
  const int dlen = m + 3, ssh = 2 * h - n;
  uint32_t bw = 0u;
  auto putd = [&](int i, uint32_t ss) {
    const uint32_t xs = i >= 3 ? X[TS * (i - 3)] : 0u;
    D[TS * i] = xs - ss - bw;
    bw = (xs < ss || (xs == ss && bw)) ? 1u : 0u;
  };
  for (int i = 0; i < ssh; i++) putd(i, 0u);
  tsqr(PV{S0}, m + 1, (dlen - ssh + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q + ssh;
      if (i < dlen) putd(i, o[q]);
    }
  });
  const bool dneg = (D[TS * (dlen - 1)] >> 31) != 0u;
  if (dneg) {
    uint32_t c = 1u;
    for (int i = 0; i < dlen; i++) { const uint32_t v = ~D[TS * i] + c; c = (c && v == 0u) ? 1u : 0u; D[TS * i] = v; }
  }
  zero_tail(D, dlen);
  // S' = S0 2^(32(h-1)) +- floor(D Z / 2^(32(h+3)+1)),  n+2 limbs, into the slab
  uint32_t cs = 0u, prev = 0u;
  int nexts = 0;
  auto puts = [&](int i, uint32_t c) {
    const uint32_t sv = (i >= h - 1) ? S0[TS * (i - (h - 1))] : 0u;
    uint32_t v;
    if (dneg) { v = sv - c - cs; cs = (sv < c || (sv == c && cs)) ? 1u : 0u; }
    else { const uint64_t t = (uint64_t)sv + c + cs; v = (uint32_t)t; cs = (uint32_t)(t >> 32); }
    Sq[TS * i] = v;
  };
  const int plen = dlen + h + 1;
  tprod(PV{D}, dlen, PV{Z}, h + 1, blk(h + 3), 1 << 20, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int pj = 8 * cb + q;
      const int i = pj - (h + 4);
      if (pj < plen) {
        if (i >= 0 && i < n + 2) { puts(i, (prev >> 1) | (o[q] << 31)); nexts = i + 1; }
        prev = o[q];
      }
    }
  });
  for (int i = nexts; i < n + 2; i++) {              // product limbs past its end are 0
    const int pj = i + h + 4;
    puts(i, pj == plen ? (prev >> 1) : 0u);
  }
  {
    const uint32_t u = Sq[0] & 0x7FFFFFFFu;
    if (Sq[TS * (n + 1)] == 0u && u >= (1u << 20) && u <= 0x7FFFFFFFu - (1u << 20)) {
      int ovf;
      const int Lb = tround_store(Sq, n + 1, n, 1u, mode, 0u, r, ovf);
      *r_exp = exp_word(eh - 32LL * n - 32 + Lb + ovf, 0u);
      return 0;
    }
  }
  if (!exact) return 1;
  // exact correction: Sc = floor(S'/2^32) (n+1 limbs), Rm = (A_ext - Sc^2) mod 2^(32(n+2))
  // over slots 0 and 2
  uint32_t *Sc = Sq + TS, *Rm = w + TS * S::Z0;
  const VW xh{X, n + 1};
  const uint32_t stop = Sc[TS * n];
  uint32_t c1 = 0u, b2 = 0u;
  auto putr = [&](int i, uint32_t p) {
    uint32_t smv = 0u;                               // (2 stop Sc) 2^(32n)
    if (i >= n && stop) {
      const int t = i - n;
      const uint32_t v = (t < n) ? Sc[TS * t] : 0u, wv = (t >= 1 && t - 1 < n) ? Sc[TS * (t - 1)] : 0u;
      smv = (v << 1) | (wv >> 31);
    }
    const uint64_t tt = (uint64_t)p + smv + c1;
    const uint32_t pv = (uint32_t)tt;
    c1 = (uint32_t)(tt >> 32);
    const uint32_t av = (i >= n - 1) ? xh.get(i - (n - 1)) : 0u;
    const uint32_t v = av - pv - b2;
    b2 = (av < pv || (av == pv && b2)) ? 1u : 0u;
    Rm[TS * i] = v;
  };
  int nextr = 0;
  const VW sl{Sc, n};
  tsqr(sl, n, (n + 2 + 7) / 8, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q;
      if (i < n + 2) { putr(i, o[q]); nextr = i + 1; }
    }
  });
  for (int i = nextr; i < n + 2; i++) putr(i, 0u);
  // 0 <= Rm <= 2Sc, Sc stepped alongside (bounded; a hit bound sets the error word)
  int guard = 0;
  while ((Rm[TS * (n + 1)] >> 31) != 0u && guard < 64) {            // Rm += 2Sc - 1, Sc -= 1
    uint32_t c = 0u;
    for (int i = 0; i < n + 2; i++) {
      const uint32_t v = (i <= n ? Sc[TS * i] : 0u), wv = (i >= 1 && i - 1 <= n) ? Sc[TS * (i - 1)] : 0u;
      const uint32_t s2 = (v << 1) | (wv >> 31);
      const uint64_t t = (uint64_t)Rm[TS * i] + s2 + c;
      Rm[TS * i] = (uint32_t)t; c = (uint32_t)(t >> 32);
    }
    uint32_t bq = 1u;
    for (int i = 0; i < n + 2 && bq; i++) { const uint32_t v = Rm[TS * i]; Rm[TS * i] = v - 1u; bq = v == 0u; }
    bq = 1u;
    for (int i = 0; i <= n && bq; i++) { const uint32_t v = Sc[TS * i]; Sc[TS * i] = v - 1u; bq = v == 0u; }
    guard++;
  }
  for (;;) {                                          // Rm -= 2Sc + 1, Sc += 1 while Rm > 2Sc
    int cmp = 0;
    for (int i = n + 1; i >= 0 && cmp == 0; i--) {
      const uint32_t v = (i <= n ? Sc[TS * i] : 0u), wv = (i >= 1 && i - 1 <= n) ? Sc[TS * (i - 1)] : 0u;
      const uint32_t x = Rm[TS * i], y = (v << 1) | (wv >> 31);
      if (x != y) cmp = x > y ? 1 : -1;
    }
    if (cmp <= 0 || guard >= 64) break;
    uint32_t bb = 1u;
    for (int i = 0; i < n + 2; i++) {
      const uint32_t v = (i <= n ? Sc[TS * i] : 0u), wv = (i >= 1 && i - 1 <= n) ? Sc[TS * (i - 1)] : 0u;
      const uint32_t x = Rm[TS * i], y = (v << 1) | (wv >> 31);
      Rm[TS * i] = x - y - bb;
      bb = (x < y || (x == y && bb)) ? 1u : 0u;
    }
    uint32_t cq2 = 1u;
    for (int i = 0; i <= n && cq2; i++) { const uint32_t v = Sc[TS * i] + 1u; Sc[TS * i] = v; cq2 = v == 0u; }
    guard++;
  }
  if (guard >= 64) atomicOr(err, 2u);
  // round bit: Rm > Sc;  sticky: Rm != 0
  int c2 = 0;
  uint32_t nz = 0u;
  for (int i = n + 1; i >= 0; i--) {
    const uint32_t x = Rm[TS * i], y = i <= n ? Sc[TS * i] : 0u;
    nz |= x;
    if (c2 == 0 && x != y) c2 = x > y ? 1 : -1;
  }
  for (int i = S::SLOT; i < S::SLOT + 8; i++) Rm[TS * i] = 0u;   // the guard limbs between slots 0 and 2
  const uint32_t rb = c2 > 0 ? 1u : 0u, sticky = nz != 0u ? 1u : 0u;
  uint32_t *Xr = Sq;                                  // 2Sc + rb in place one limb below Sc
  for (int i = 0; i < n + 2; i++) {
    const uint32_t si = i <= n ? Sc[TS * i] : 0u, sm = i > 0 ? Sc[TS * (i - 1)] : 0u;
    Xr[TS * i] = (si << 1) | (i > 0 ? (sm >> 31) : rb);
  }
  int ovf;
  const int Lb = tround_store(Xr, n + 2, n, sticky, mode, 0u, r, ovf);
  *r_exp = exp_word(eh - 32LL * n - 1 + Lb + ovf, 0u);
  return 0;
}


// mul (tmul_op): A in this thread's shared-memory columns (read as the product's first
// factor: 8 limbs per tile), B and the product limbs that feed the rounding in its slab
// column.  Measured on GB300 at 4096 bits: A and B both in shared memory allow 5 warps per
// SM (3.88 ms per 2^20 operations), both in the slab leave the operand reads to L2
// (3.10 ms); this split holds 11 warps per SM (2.37 ms).  Limb offsets per thread:
template <int N>
struct MSpace {
  static constexpr int words = N + 16;                  // shared memory: A, then zeros
  static constexpr int SB = 16, GQ = N + 32;            // slab: 16 zero | B | 16 zero | Q
  static constexpr int slab = GQ + N + 8;
};

// ---- mul ---------------------------------------------------------------------------------
// One thread per multiplication.  The product of two normalised n-limb mantissas has its
// top bit at 64n-1 or 64n-2, so the result is product limbs n-1 .. 2n-1 shifted by 0 or 1
// bit and rounded at bit 31 or 30 of limb n-1.  The first pass forms only the output
// blocks from c0 = 8*blk(n-1) up (a short product: about n^2/2 + 8n of the n^2 limb
// products), without the carry from the columns below c0, which is less than c0+1 units
// of limb c0+1.  When the bits between limb c0+1 and the round bit are neither within
// 2^16 units of zero nor of all ones, that carry cannot reach the round bit or make the
// bits below it zero, so the round bit is exact and sticky is 1.  Otherwise (exact ties
// and near-ties, about 2^-170 of random operands) the operation returns 1 and is run again
// with exact = true, which forms the whole product.  Same results as op_mul / row_mul:
// reference fpa_warp_mul.h:41-139 (TINY when BIAS+e < 5, INF when BIAS+e > 0x7FFFFFFF).
// A and B are zero-guarded buffers (A read as the first factor, B as the second); the
// product limbs n-1 .. 2n-1 go to Q (n+1 limbs).
__device__ __forceinline__ int tmul_op(uint32_t *A, uint32_t *B, uint32_t *Q, int n, int mode, uint32_t a_exp,
                                       const uint32_t *a, uint32_t b_exp, const uint32_t *b, uint32_t *r_exp,
                                       uint32_t *r, bool exact) {
  const uint32_t act = c_action[2][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_MUL) { *r_exp = act; return 0; }
  stage_limbs(A, a, n);
  stage_limbs(B, b, n);
  const int cb0 = exact ? 0 : blk(n - 1), c0 = 8 * cb0;
  uint32_t low = 0u;                                   // exact: OR of limbs 0 .. n-2
  uint32_t l1 = 0u, midz = 0u, mido = 0xFFFFFFFFu;     // short: limb c0+1; OR / AND of limbs c0+2 .. n-2
  tprod2(PV{A}, n, PV{B}, n, cb0, 1 << 20, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int p = 8 * cb + q;
      if (p < n - 1) {
        low |= o[q];
        if (p == c0 + 1) l1 = o[q];
        else if (p > c0 + 1) { midz |= o[q]; mido &= o[q]; }
      } else if (p < 2 * n) {
        Q[TS * (p - (n - 1))] = o[q];
      }
    }
  });
  const uint32_t full = Q[TS * n] >> 31;               // top bit at 64n-1
  const uint32_t below = full ? 0x7FFFFFFFu : 0x3FFFFFFFu;
  const uint32_t rl = Q[0] & below;                    // limb n-1's bits below the round bit
  uint32_t sticky = low != 0u;
  if (!exact && c0 > 0) {
    const bool near0 = midz == 0u && l1 < (1u << 16) && rl == 0u;
    const bool near1 = mido == 0xFFFFFFFFu && l1 >= 0xFFFF0000u && rl == below;
    if (near0 || near1) return 1;
    sticky = 1u;
  }
  const uint32_t sign = (a_exp ^ b_exp) & 1u;
  int ovf;
  const int Lb = tround_store(Q, n + 1, n, sticky, mode, sign, r, ovf);
  const long long e = (long long)(a_exp >> 1) + (long long)(b_exp >> 1) - 2LL * BIAS - 32LL * n - 32 + Lb + ovf;
  if ((long long)BIAS + e < 5) *r_exp = CLS_POS_TINY - sign;
  else if ((long long)BIAS + e > 0x7FFFFFFFLL) *r_exp = CLS_POS_INF - sign;
  else *r_exp = exp_word(e, sign);
  return 0;
}

}  // namespace gfpa
