// fpa_thread_newton.cuh -- div and sqrt with one thread per operation.
//
// The lane-group div/sqrt (op_div / op_sqrt in fpa_ops.cuh) spend most of their time outside
// the limb products: staging operands, summing column blocks, syncing the group, and
// products whose column blocks leave some lanes idle (a 66-limb operand is 17 blocks of 4).
// Here every thread of a warp runs a whole operation of its own, so there is no cross-lane
// traffic, no sync and no idle lane; the 32 operations of a warp share one limb count and
// follow the same instruction stream.
//
// The integer steps are those of op_div / op_sqrt, unchanged: the same Newton level
// schedule (newton_levels, the one-thread small levels up to SMALL_LEVEL limbs), the same
// truncations of every product and residual, the same Karp-Markstein last step with one
// extra limb, the same 2^20-unit rounding margin and the same bounded exact correction.
// The iterates, the extra-limb quotient / root and every result are therefore the same
// integers, which the error analysis of those steps covers.  Only the data movement is
// new: each product's limbs come out lowest first, 8 at a time (tmul), and go straight into
// the step that uses them, so the full products are never stored.
//
// Storage: a thread's buffers live in its warp's shared-memory workspace with the warp's
// 32 threads interleaved limb by limb (limb j of a buffer at p[32*j]), so the 32 threads
// reading the same limb index touch 32 consecutive words.  Per thread, with N the largest
// limb count served: regions R0 and R1 of N/2+8 limbs (Newton iterates, then the
// Karp-Markstein remainder) and R3 of N+8 limbs (raw residual limbs, then the extra-limb
// result with the half-size quotient / root placed at its final offset), 2N+24 words.
//
// Operands a, b and the result r are the caller's arrays in the natural layout (number i's
// limbs contiguous).  A thread reading its own number touches one 32-byte sector per limb
// read across the warp's 32 numbers, and the products read the operands many times, so
// each operation first copies its operands once into a slab in global memory laid out
// like the workspace (limb j of this thread at slab[32*j]): A and B for div, Xh =
// floor(A * 2^(32-odd)) for sqrt.  Every later operand read is then one coalesced 128-byte
// warp load, and sqrt's shifted operand costs no shifts.  Reference semantics as op_div /
// op_sqrt: fpa_warp_div.h:127-201, fpa_warp_sqrt.h:195-254.
#pragma once
#include "fpa_ops.cuh"

namespace gfpa {

constexpr int TS = 32;   // distance between a thread's consecutive limbs in the workspace

template <int N>
struct TSpace {
  static constexpr int H = N / 2 + 8;        // R0, R1
  static constexpr int Q = N + 8;            // R3
  static constexpr int words = 2 * H + Q;    // per thread
  static constexpr int slab = 2 * N + 8;     // operand slab words per thread (global memory)
  static constexpr int min_limbs = 8;        // smaller numbers keep the lane-group path
};

// Copies n limbs of a natural-layout number to a slab column (limb j at dst[TS*j]).
__device__ __forceinline__ void stage_limbs(uint32_t *dst, const uint32_t *src, int n) {
  if ((((uintptr_t)src) & 15) == 0 && (n & 3) == 0) {
    for (int j = 0; j < n; j += 4) {
      const uint4 v = *reinterpret_cast<const uint4 *>(src + j);
      dst[TS * j] = v.x; dst[TS * (j + 1)] = v.y; dst[TS * (j + 2)] = v.z; dst[TS * (j + 3)] = v.w;
    }
  } else {
    for (int j = 0; j < n; j++) dst[TS * j] = src[j];
  }
}

// ---- operand views: limb i of a number, 0 outside [0, len) ---------------------------
struct VW {                     // a workspace buffer or a slab column
  const uint32_t *p; int len;
  __device__ __forceinline__ uint32_t get(int i) const { return ((unsigned)i < (unsigned)len) ? p[TS * i] : 0u; }
};
// the Newton residual magnitude (ResidualMag) read from raw product limbs T[off ...] that
// were stored from index 0: limb i is T[i] (or ~T[i] when the product was below 2^(32L)),
// 0 at and above limb `lim` (= L - off) and outside [0, len)
struct VResid {
  const uint32_t *T; int lim, len; uint32_t neg;
  __device__ __forceinline__ uint32_t get(int i) const {
    if ((unsigned)i >= (unsigned)len || i >= lim) return 0u;
    const uint32_t v = T[TS * i];
    return neg ? v : ~v;
  }
};

// ---- product: limbs of x * y lowest first, 8 at a time ----------------------------------
// Column-block product scanning with an 8x8 register tile: output block cb gathers
// x-block i times the y window y[8(cb-i)-8 .. 8(cb-i)+7] for every i with
// 0 <= cb-i <= My (My = y's block count), into
// 96-bit (lo, hi, top) column sums fed by mac3; the two limbs above a block carry into the
// next one.  sink(cb, L) receives limbs 8cb .. 8cb+7 in L[0..7]; blocks stop once
// `out_limbs` limbs have been produced (the higher limbs are not computed).
template <class X, class Y, class Sink>
__device__ __forceinline__ void tmul(const X &x, int lx, const Y &y, int ly, int out_limbs, Sink &&sink) {
  const int Mx = (lx + 7) >> 3, My = (ly + 7) >> 3;
  const int Mo = min(Mx + My, (out_limbs + 7) >> 3);
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int cb = 0; cb < Mo; cb++) {
    uint32_t lo[8], hi[8], tp[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { lo[c] = 0u; hi[c] = 0u; tp[c] = 0u; }
    lo[0] = c0; lo[1] = c1;
    // the window spans y-blocks cb-i and cb-i-1, so x-block i reaches output blocks i .. i+My
    const int i0 = max(0, cb - My), i1 = min(cb, Mx - 1);
    uint32_t a[8], w[16];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = x.get(8 * i0 + r);
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = y.get(8 * (cb - i0) - 8 + m);
#pragma unroll 1
    for (int i = i0; i <= i1; i++) {
      uint32_t an[8], wn[8];              // the next tile's operands, loaded ahead of the math
#pragma unroll
      for (int r = 0; r < 8; r++) an[r] = x.get(8 * (i + 1) + r);
#pragma unroll
      for (int m = 0; m < 8; m++) wn[m] = y.get(8 * (cb - i - 2) + m);
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) mac3(lo[c], hi[c], tp[c], a[r], w[8 + c - r]);
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = an[r];
#pragma unroll
      for (int m = 0; m < 8; m++) { w[8 + m] = w[m]; w[m] = wn[m]; }
    }
    uint32_t L[10];
    columns_to_limbs<8>(lo, hi, tp, L);
    sink(cb, L);
    c0 = L[8]; c1 = L[9];
  }
}

// ---- rounding: X (workspace, xlen limbs) to n limbs, written to r (natural layout) -------
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
  for (int i = 0; i < n; i++) {
    const uint32_t nxt = (q + i + 1 < xlen) ? X[TS * (q + i + 1)] : 0u;
    uint32_t v = s ? ((cur >> s) | (nxt << (32 - s))) : cur;
    v += carry;
    carry = (carry && v == 0u) ? 1u : 0u;
    r[i] = v;
    cur = nxt;
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
template <int N>
__device__ int tdiv(uint32_t *w, uint32_t *slab, int n, int mode, uint32_t a_exp, const uint32_t *a, uint32_t b_exp,
                    const uint32_t *b, uint32_t *r_exp, uint32_t *r, bool exact, uint32_t *err) {
  constexpr int H = TSpace<N>::H;
  const uint32_t act = c_action[3][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_DIV) { *r_exp = act; return 0; }
  uint32_t *R0 = w, *R1 = w + TS * H, *R3 = w + TS * 2 * H;
  uint32_t *SA = slab, *SB = slab + TS * n;          // A and B, limb j at [TS*j]
  stage_limbs(SA, a, n);
  stage_limbs(SB, b, n);
  int lv[24];
  const int nl = newton_levels(n, lv);
  const int l0 = small_levels_end(lv, nl, true);
  uint32_t *Y = R0, *Y2 = R1;
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
  }
  for (int li = l0; li < nl - 1; li++) {
    const int k = lv[li - 1], kp = lv[li], L = k + kp, lt = kp - k + 3;
    // T = B_k' * Y_k: keep limbs k-1 .. L (the lower ones reach them only through carries)
    tmul(VW{SB + TS * (n - kp), kp}, kp, VW{Y, k + 1}, k + 1, L + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int j = 8 * cb + q - (k - 1);
        if (j >= 0 && j <= L - (k - 1)) R3[TS * j] = o[q];
      }
    });
    const uint32_t neg = R3[TS * (L - (k - 1))] != 0u;
    // Y_k' = Y_k * 2^(32(k'-k)) +- M,  M = (Y_k * |E|) >> 32(k+1),  over k'+1 limbs
    uint32_t cy = 0u;
    int next = 0;                                    // next limb of Y_k' to form
    auto put = [&](int i, uint32_t m) {
      const uint32_t ys = (i >= kp - k) ? Y[TS * (i - (kp - k))] : 0u;
      uint32_t v;
      if (neg) { v = ys - m - cy; cy = (ys < m || (ys == m && cy)) ? 1u : 0u; }
      else { const uint64_t t = (uint64_t)ys + m + cy; v = (uint32_t)t; cy = (uint32_t)(t >> 32); }
      Y2[TS * i] = v;
    };
    tmul(VW{Y, k + 1}, k + 1, VResid{R3, L - (k - 1), lt, neg}, lt, k + 1 + lt, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - (k + 1);
        if (i >= 0 && i < lt && i <= kp) { put(i, o[q]); next = i + 1; }
      }
    });
    for (int i = next; i <= kp; i++) put(i, 0u);
    uint32_t *t = Y; Y = Y2; Y2 = t;
  }
  // Karp-Markstein step with one limb more than the result (op_div): h = the last Newton
  // level, m = n+2-h; q0 is placed at limb h-1 of R3 so that Q' forms in place.
  const int h = lv[nl - 2], m = n + 2 - h;
  uint32_t *D = Y2, *Q = R3;
  tmul(VW{SA + TS * (n - m - 1), m + 1}, m + 1, VW{Y, h + 1}, h + 1, h + 2 + m, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int j = 8 * cb + q - (h + 1);
      if (j >= 0 && j <= m) Q[TS * (h - 1 + j)] = o[q];
    }
  });
  // D = |A 2^96 - floor(q0 B / 2^(32(n-h-1)))| over n+4 limbs, its low m+2 limbs kept
  const int dl = n + 4, dlen = m + 2, sh = n - h - 1;
  uint32_t bw = 0u;
  tmul(VW{Q + TS * (h - 1), m + 1}, m + 1, VW{SB, n}, n, n + m + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q - sh;
      if (i >= 0 && i < dl) {
        const uint32_t xa = (i >= 3 && i - 3 < n) ? SA[TS * (i - 3)] : 0u, xq = o[q];
        const uint32_t v = xa - xq - bw;
        bw = (xa < xq || (xa == xq && bw)) ? 1u : 0u;
        if (i < dlen) D[TS * i] = v;
      }
    }
  });
  const bool dneg = bw != 0u;
  if (dneg) {                                        // D = -D (mod 2^(32 dlen))
    uint32_t c = 1u;
    for (int i = 0; i < dlen; i++) { const uint32_t v = ~D[TS * i] + c; c = (c && v == 0u) ? 1u : 0u; D[TS * i] = v; }
  }
  // Q' = q0 2^(32(h-1)) +- floor(D Y / 2^(32(h+2))),  n+2 limbs
  uint32_t cq = 0u;
  int nextq = 0;
  auto putq = [&](int i, uint32_t c) {
    const uint32_t qv = (i >= h - 1) ? Q[TS * i] : 0u;
    uint32_t v;
    if (dneg) { v = qv - c - cq; cq = (qv < c || (qv == c && cq)) ? 1u : 0u; }
    else { const uint64_t t = (uint64_t)qv + c + cq; v = (uint32_t)t; cq = (uint32_t)(t >> 32); }
    Q[TS * i] = v;
  };
  tmul(VW{D, dlen}, dlen, VW{Y, h + 1}, h + 1, dlen + h + 1, [&](int cb, const uint32_t (&o)[10]) {
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
  // exact correction: Q = floor(Q'/2^32) (n+1 limbs, at limb 1 of R3),
  // Rm = (A 2^(32n) - Q B) mod 2^(32(n+2)) over R0..R1
  uint32_t *Qc = Q + TS, *Rm = R0;
  const uint32_t qt = Qc[TS * n];
  uint32_t c1 = 0u, b2 = 0u;
  auto putr = [&](int i, uint32_t p) {
    // P2 = Q[0..n) B + (qt B) 2^(32n): add the small multiple, then subtract from A 2^(32n)
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
  tmul(VW{Qc, n}, n, VW{SB, n}, n, n + 2, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q;
      if (i < n + 2) { putr(i, o[q]); nextr = i + 1; }
    }
  });
  for (int i = nextr; i < n + 2; i++) putr(i, 0u);
  // 0 <= Rm < B, Q stepped alongside (bounded; a hit bound sets the error word)
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
  const uint32_t rb = c2 >= 0 ? 1u : 0u, sticky = (nz != 0u && c2 != 0) ? 1u : 0u;
  // X = 2Q + rb, n+2 limbs, formed in place one limb below Q (limb i of X over limb i of R3)
  uint32_t *X = R3;
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
// n+1 limbs (read from A on the fly), Newton on 1/sqrt with three products per level, the
// Karp-Markstein step with one limb more, the exact correction with R = A_ext - S^2.
template <int N>
__device__ int tsqrt(uint32_t *w, uint32_t *slab, int n, int mode, uint32_t a_exp, const uint32_t *a, uint32_t *r_exp,
                     uint32_t *r, bool exact, uint32_t *err) {
  constexpr int H = TSpace<N>::H;
  const uint32_t act = c_sqrt_action[classify(a_exp)];
  if (act != ACT_SQRT) { *r_exp = act; return 0; }
  uint32_t *R0 = w, *R1 = w + TS * H, *R3 = w + TS * 2 * H;
  const long long e = (long long)(a_exp >> 1) - BIAS;
  const int odd = (int)(e & 1);
  const long long eh = (e + odd) / 2;
  // Xh = floor(A * 2^(32 - odd)), n+1 limbs, staged in the slab
  {
    uint32_t prev = 0u;
    for (int j = 0; j < n; j++) {
      const uint32_t cur = a[j];
      slab[TS * j] = odd ? ((prev >> 1) | (cur << 31)) : prev;
      prev = cur;
    }
    slab[TS * n] = odd ? (prev >> 1) : prev;
  }
  const VW xh{slab, n + 1};
  int lv[24];
  const int nl = newton_levels(n, lv);
  const int l0 = small_levels_end(lv, nl, true);
  uint32_t *Z = R0, *Z2 = R1;
  {
    const uint64_t x1 = (uint64_t)xh.get(n) << 32;
    const uint64_t s1 = isqrt64(x1);
    const uint64_t z = 0xFFFFFFFFFFFFFFFFull / s1;
    uint32_t v[SMALL_LEVEL + 1], xt[SMALL_LEVEL];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) v[i] = 0u;
    v[0] = (uint32_t)z; v[1] = (uint32_t)(z >> 32);
#pragma unroll
    for (int i = 0; i < SMALL_LEVEL; i++) xt[i] = xh.get(n + 1 - SMALL_LEVEL + i);
    small_levels<true>(xt, lv, l0, v);
    const int k = lv[l0 - 1];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) if (i <= k) Z[TS * i] = v[i];
  }
  constexpr int WOFF = N / 2 + 4;                    // Wraw at R3 + WOFF (V1s below it)
  for (int li = l0; li < nl - 1; li++) {
    const int k = lv[li - 1], kp = lv[li];
    const int j = k > 2 ? k - 2 : 0, l1 = kp + k + 1 - j, L = kp + 2 * k - j, lt = kp - k + 3;
    uint32_t *V1s = R3, *Wr = R3 + TS * WOFF;
    // V1 = X_k' Z_k, kept from limb j up
    tmul(VW{slab + TS * (n + 1 - kp), kp}, kp, VW{Z, k + 1}, k + 1, kp + k + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - j;
        if (i >= 0 && i < l1) V1s[TS * i] = o[q];
      }
    });
    // W = (V1 >> 32j) Z_k, kept from limb 2k-1-j to L
    const int off = 2 * k - 1 - j;
    tmul(VW{V1s, l1}, l1, VW{Z, k + 1}, k + 1, L + 1, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - off;
        if (i >= 0 && i <= L - off) Wr[TS * i] = o[q];
      }
    });
    const uint32_t neg = Wr[TS * (L - off)] != 0u;
    // Z_k' = Z_k 2^(32(k'-k)) +- M,  M = (Z_k |E|) >> (32(k+1)+1),  over k'+1 limbs
    uint32_t cy = 0u, prev = 0u;
    int next = 0;
    auto put = [&](int i, uint32_t m) {
      const uint32_t zs = (i >= kp - k) ? Z[TS * (i - (kp - k))] : 0u;
      uint32_t v;
      if (neg) { v = zs - m - cy; cy = (zs < m || (zs == m && cy)) ? 1u : 0u; }
      else { const uint64_t t = (uint64_t)zs + m + cy; v = (uint32_t)t; cy = (uint32_t)(t >> 32); }
      Z2[TS * i] = v;
    };
    // M[i] = (P[k+1+i] >> 1) | (P[k+2+i] << 31): formed when P[k+2+i] arrives (the limbs of
    // the last block past the product's end are 0)
    tmul(VW{Z, k + 1}, k + 1, VResid{Wr, L - off, lt, neg}, lt, k + 1 + lt, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = 8 * cb + q - (k + 2);
        if (i >= 0 && i <= kp) { put(i, (prev >> 1) | (o[q] << 31)); next = i + 1; }
        prev = o[q];
      }
    });
    for (int i = next; i <= kp; i++) put(i, i == next ? (prev >> 1) : 0u);
    uint32_t *t = Z; Z = Z2; Z2 = t;
  }
  // Karp-Markstein with one limb more (op_sqrt): S0 = floor(Xt Z / 2^(32(h+1))), placed at
  // limb h-1 of R3 so that S' forms in place
  const int h = lv[nl - 2], m = n + 2 - h;
  uint32_t *D = Z2, *S = R3;
  tmul(VW{slab + TS * (n - m), m + 1}, m + 1, VW{Z, h + 1}, h + 1, h + 2 + m, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q - (h + 1);
      if (i >= 0 && i <= m) S[TS * (h - 1 + i)] = o[q];
    }
  });
  // D = |Xh 2^96 - S0^2 2^(32(2h-n))| over n+6 limbs, its low m+3 limbs kept
  const int dl = n + 6, dlen = m + 3, ssh = 2 * h - n;
  uint32_t bw = 0u;
  auto putd = [&](int i, uint32_t ss) {
    const uint32_t xs = xh.get(i - 3);
    const uint32_t v = xs - ss - bw;
    bw = (xs < ss || (xs == ss && bw)) ? 1u : 0u;
    if (i < dlen) D[TS * i] = v;
  };
  for (int i = 0; i < ssh && i < dl; i++) putd(i, 0u);
  const VW s0{S + TS * (h - 1), m + 1};
  tmul(s0, m + 1, s0, m + 1, 2 * m + 2, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q + ssh;
      if (i < dl && 8 * cb + q < 2 * m + 2) putd(i, o[q]);
    }
  });
  for (int i = 2 * m + 2 + ssh; i < dl; i++) putd(i, 0u);
  const bool dneg = bw != 0u;
  if (dneg) {
    uint32_t c = 1u;
    for (int i = 0; i < dlen; i++) { const uint32_t v = ~D[TS * i] + c; c = (c && v == 0u) ? 1u : 0u; D[TS * i] = v; }
  }
  // S' = S0 2^(32(h-1)) +- floor(D Z / 2^(32(h+3)+1)),  n+2 limbs
  uint32_t cs = 0u, prev = 0u;
  int nexts = 0;
  auto puts = [&](int i, uint32_t c) {
    const uint32_t sv = (i >= h - 1) ? S[TS * i] : 0u;
    uint32_t v;
    if (dneg) { v = sv - c - cs; cs = (sv < c || (sv == c && cs)) ? 1u : 0u; }
    else { const uint64_t t = (uint64_t)sv + c + cs; v = (uint32_t)t; cs = (uint32_t)(t >> 32); }
    S[TS * i] = v;
  };
  const int plen = dlen + h + 1;
  tmul(VW{D, dlen}, dlen, VW{Z, h + 1}, h + 1, plen, [&](int cb, const uint32_t (&o)[10]) {
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
  for (int i = nexts; i < n + 2; i++) {              // V1 limbs past its end are 0
    const int pj = i + h + 4;
    puts(i, pj == plen ? (prev >> 1) : 0u);
  }
  {
    const uint32_t u = S[0] & 0x7FFFFFFFu;
    if (S[TS * (n + 1)] == 0u && u >= (1u << 20) && u <= 0x7FFFFFFFu - (1u << 20)) {
      int ovf;
      const int Lb = tround_store(S, n + 1, n, 1u, mode, 0u, r, ovf);
      *r_exp = exp_word(eh - 32LL * n - 32 + Lb + ovf, 0u);
      return 0;
    }
  }
  if (!exact) return 1;
  // exact correction: S = floor(S'/2^32) (n+1 limbs), Rm = (A_ext - S^2) mod 2^(32(n+2))
  uint32_t *Sc = S + TS, *Rm = R0;
  const uint32_t stop = Sc[TS * n];
  uint32_t c1 = 0u, b2 = 0u;
  auto putr = [&](int i, uint32_t p) {
    uint32_t smv = 0u;                               // (2 stop S) 2^(32n)
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
  tmul(sl, n, sl, n, n + 2, [&](int cb, const uint32_t (&o)[10]) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = 8 * cb + q;
      if (i < n + 2) { putr(i, o[q]); nextr = i + 1; }
    }
  });
  for (int i = nextr; i < n + 2; i++) putr(i, 0u);
  // 0 <= Rm <= 2S, S stepped alongside (bounded; a hit bound sets the error word)
  int guard = 0;
  while ((Rm[TS * (n + 1)] >> 31) != 0u && guard < 64) {            // Rm += 2S - 1, S -= 1
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
  for (;;) {                                          // Rm -= 2S + 1, S += 1 while Rm > 2S
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
  // round bit: Rm > S;  sticky: Rm != 0
  int c2 = 0;
  uint32_t nz = 0u;
  for (int i = n + 1; i >= 0; i--) {
    const uint32_t x = Rm[TS * i], y = i <= n ? Sc[TS * i] : 0u;
    nz |= x;
    if (c2 == 0 && x != y) c2 = x > y ? 1 : -1;
  }
  const uint32_t rb = c2 > 0 ? 1u : 0u, sticky = nz != 0u ? 1u : 0u;
  uint32_t *X = R3;                                   // 2S + rb in place one limb below S
  for (int i = 0; i < n + 2; i++) {
    const uint32_t si = i <= n ? Sc[TS * i] : 0u, sm = i > 0 ? Sc[TS * (i - 1)] : 0u;
    X[TS * i] = (si << 1) | (i > 0 ? (sm >> 31) : rb);
  }
  int ovf;
  const int Lb = tround_store(X, n + 2, n, sticky, mode, 0u, r, ovf);
  *r_exp = exp_word(eh - 32LL * n - 1 + Lb + ovf, 0u);
  return 0;
}

}  // namespace gfpa
