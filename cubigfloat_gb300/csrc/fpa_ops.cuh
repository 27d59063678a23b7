// fpa_ops.cuh -- one fpa operation (add/sub/mul/div/sqrt) executed by one lane group.
//
// Every operation computes its mantissa result exactly (or exactly enough: an integer
// part plus an exact sticky flag) and rounds once with grp_round, so the result is the
// correctly rounded value for the requested mode.  Special operands follow the action
// tables of fpa_device.cuh; exponent range limits follow the reference kernels cited
// at each operation.
#pragma once
#include "fpa_device.cuh"

namespace gfpa {

// Configurations that carry the Karatsuba split of mul, and the elementwise kernel
// instantiation that runs it (an operation code of the kernels only).
template <int G, int K, int R>
struct KaratsubaCfg { static constexpr bool on = K >= 8 && G * K * R >= 256; };
constexpr int OP_MUL_KARA = 6;

// Workspace words per group, beyond MulScratch.  N = G*K*R is the group's limb capacity.
template <int G, int K, int R>
struct OpSpace {
  static constexpr int N = G * K * R;
  __host__ __device__ static constexpr int addsub() { return 3 * N + 8; }   // staged a, b + X
  __host__ __device__ static constexpr int mul() { return 2 * N + 4; }
  __host__ __device__ static constexpr int div() { return (N / 2 + 8) * 2 + (N + 8) + (2 * N + 8) + (N + 8); }
  __host__ __device__ static constexpr int sqrt() { return (N + 4) + (N / 2 + 8) * 2 + (N + 8) * 3 + (2 * N + 8); }
  __host__ __device__ static constexpr int fma() { return (2 * N + 4) + (3 * N + 8); }      // P + sum window
  __host__ __device__ static constexpr int max_all() {
    int a = addsub(), b = mul(), c = div(), d = sqrt();
    int m = a > b ? a : b; m = m > c ? m : c; m = m > d ? m : d;
    return m;
  }
  __host__ __device__ static constexpr int words() { return MulScratch<G, K, R>::words() + max_all(); }
};

// Shared-memory words one group needs for operation OP (16-byte aligned slice size).
template <int OP, int G, int K, int R>
struct OpWords {
  __host__ __device__ static constexpr int v() {
    return (OP == OP_ADD || OP == OP_SUB) ? OpSpace<G, K, R>::addsub()
           : MulScratch<G, K, R>::words() + ((OP == OP_MUL || OP == OP_MUL_KARA) ? OpSpace<G, K, R>::mul()
                                          : OP == OP_DIV ? OpSpace<G, K, R>::div()
                                          : OP == OP_SQRT ? OpSpace<G, K, R>::sqrt() : OpSpace<G, K, R>::fma());
  }
  __host__ __device__ static constexpr int aligned() { return (v() + 3) & ~3; }
};

// The elementwise kernels double-buffer the operands of add/sub and mul (the next
// operation's copies are in flight while the group computes): one more staged pair each;
// the Karatsuba mul instantiation also carries the split's staging (N + K words).
template <int OP, int G, int K, int R>
struct PipeWords {
  static constexpr int N = G * K * R;
  __host__ __device__ static constexpr int v() {
    return OpWords<OP, G, K, R>::v() + ((OP == OP_ADD || OP == OP_SUB) ? 2 * N
                                        : OP == OP_MUL ? 2 * N + 2 * K : (OP == OP_MUL_KARA ? 3 * N + 3 * K : 0));
  }
  __host__ __device__ static constexpr int aligned() { return (v() + 3) & ~3; }
};

// Rounded mantissa + exponent for one instance, written by the group.
template <int G>
__device__ __forceinline__ void write_value(const Grp<G> &g, uint32_t *r_exp, uint32_t *r, int n,
                                            const Rounded &res, uint32_t exp_word) {
  store_limbs<G>(g, r, n, res);
  if (g.lane == 0) *r_exp = exp_word;
}

template <int G>
__device__ __forceinline__ void write_class(const Grp<G> &g, uint32_t *r_exp, uint32_t cls) {
  if (g.lane == 0) *r_exp = cls;
}

template <int G>
__device__ __forceinline__ void copy_value(const Grp<G> &g, uint32_t *r_exp, uint32_t *r, int n,
                                           uint32_t exp_word, const uint32_t *src) {
  for (int i = g.lane; i < n; i += G) r[i] = src[i];
  if (g.lane == 0) *r_exp = exp_word;
}

// exponent word from an unbiased exponent (range already checked)
__device__ __forceinline__ uint32_t exp_word(long long e, uint32_t sign) {
  return (uint32_t)(2 * ((long long)BIAS + e)) + sign;
}

// ---------------------------------------------------------------------------------------
// add / sub.  Reference: fpa_warp_add_sub.h:310-380 (dispatch), :41-125 (same-sign add),
// :127-282 (effective subtraction).  The aligned sum is formed exactly in n+3 limbs:
//   X = BIG * 2^64 +- floor(SMALL * 2^(64-d))
// Bits of SMALL shifted out below the window only matter as a sticky flag; for an
// effective subtraction one extra unit is subtracted so that the true value lies in
// (X, X+1) (d > 64 implies at most one bit of cancellation, so 63 guard bits remain).
// Range: effective add -> +-INF when BIAS+e > 0x7FFFFFFF (:118-119); effective
// subtraction -> +-TINY when BIAS+e < 5 (:226-227, :272-273).
template <int G>
__device__ void op_addsub_staged(const Grp<G> &g, uint32_t *X, int n, int mode, int is_sub,
                                 uint32_t a_exp, const uint32_t *sA, uint32_t b_exp, const uint32_t *sB,
                                 uint32_t *r_exp, uint32_t *r) {
  const uint32_t act = c_action[is_sub][classify(a_exp) * 9 + classify(b_exp)];
  if (act == ACT_COPY_A) { copy_value<G>(g, r_exp, r, n, a_exp, sA); return; }
  if (act == ACT_COPY_B) { copy_value<G>(g, r_exp, r, n, b_exp, sB); return; }
  if (act == ACT_NEG_B) { copy_value<G>(g, r_exp, r, n, b_exp ^ 1u, sB); return; }   // 0 - b = -b
  if (act != ACT_ADD && act != ACT_SUB) { write_class<G>(g, r_exp, act); return; }
  const uint32_t sa = a_exp & 1u, sb = (b_exp & 1u) ^ (uint32_t)is_sub;
  const long long ea = (long long)(a_exp >> 1) - BIAS, eb = (long long)(b_exp >> 1) - BIAS;
  const bool eff_sub = sa != sb;
  bool a_big;
  if (ea != eb) a_big = ea > eb;
  else {
    int c = grp_cmp<G>(g, Ptr{sA, n}, Ptr{sB, n}, n);
    if (c == 0 && eff_sub) { write_class<G>(g, r_exp, CLS_ZERO); return; }   // exact cancellation
    a_big = c >= 0;
  }
  const uint32_t *big = a_big ? sA : sB, *sml = a_big ? sB : sA;
  const uint32_t sign = a_big ? sa : sb;
  const long long ebig = a_big ? ea : eb, esml = a_big ? eb : ea;
  const long long cap = 32LL * n + 64;
  const int d = (int)((ebig - esml) > cap ? cap : (ebig - esml));
  // sticky from SMALL's bits below position d - 64
  uint32_t lost = 0;
  if (d > 64) {
    const int cut = d - 64, full = cut >> 5;
    for (int i = g.lane; i < full && i < n; i += G) lost |= sml[i];
    if (g.lane == 0 && (cut & 31) && full < n) lost |= sml[full] & ((1u << (cut & 31)) - 1u);
    lost = g.ror(lost) != 0;
  }
  const int xl = n + 3;
  Shifted bigs{big, n, 64}, smls{sml, n, 64 - d};
  if (eff_sub) grp_sub<G>(g, X, bigs, smls, xl, lost);
  else grp_add<G>(g, X, bigs, smls, xl, 0u);
  Rounded res;
  if (!grp_round<G>(g, X, xl, n, lost, mode, sign, res)) { write_class<G>(g, r_exp, CLS_ZERO); return; }
  const long long e = ebig - 32LL * n - 64 + res.L + res.ovf;
  if (!eff_sub && (long long)BIAS + e > 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sign); return; }
  if (eff_sub && (long long)BIAS + e < 5) { write_class<G>(g, r_exp, CLS_POS_TINY - sign); return; }
  write_value<G>(g, r_exp, r, n, res, exp_word(e, sign));
}

// add/sub with operands anywhere: copies and class results straight from the operands,
// otherwise the operands are staged in the workspace first (they are read several times).
template <int G, int K, int R>
__device__ void op_addsub(const Grp<G> &g, uint32_t *ws, int n, int mode, int is_sub,
                          uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b,
                          uint32_t *r_exp, uint32_t *r) {
  constexpr int N = G * K * R;
  const uint32_t act = c_action[is_sub][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_ADD && act != ACT_SUB) {
    op_addsub_staged<G>(g, ws, n, mode, is_sub, a_exp, a, b_exp, b, r_exp, r);
    return;
  }
  uint32_t *sA = ws, *sB = sA + N, *X = sB + N;     // no product scratch needed
  for (int i = g.lane; i < n; i += G) { sA[i] = a[i]; sB[i] = b[i]; }
  g.sync();
  op_addsub_staged<G>(g, X, n, mode, is_sub, a_exp, sA, b_exp, sB, r_exp, r);
}

// ---------------------------------------------------------------------------------------
// Karatsuba split of a staged square product (x in s.sa, y in s.sb + K, n limbs each):
//   P[0..2n) = z0 + z1 2^(32h) + z2 2^(64h),  h = ceil(n/2),
//   z0 = x0 y0,  z2 = x1 y1,  z1 = (x0 + x1)(y0 + y1) - z0 - z2.
// The three half products run on tiles of K/2 limbs, so all G lanes stay busy on h limbs
// (with K-limb tiles half of them would idle).  The sums x0 + x1 = cx 2^(32h) + sx and
// y0 + y1 = cy 2^(32h) + sy are kept to h limbs: cx sy + cy sx + cx cy 2^(32h) is added
// at 2^(32h) afterwards, so every half product is h x h.  kws: N + K words (the half
// products' staging); z1 is formed in s.sb once x and y have been read, and s.sb's low K
// zero limbs are restored at the end.
template <int G, int K, int R>
__device__ __noinline__ void grp_mul_karatsuba(const Grp<G> g, uint32_t *P, int n, const MulScratch<G, K, R> s,
                                               uint32_t *kws) {
  constexpr int KS = K / 2, N = G * K * R;
  static_assert(KS >= 4, "Karatsuba halves use tiles of at least 4 limbs");
  MulScratch<G, KS, R> s2;
  s2.sa = kws; s2.sb = kws + N / 2; s2.snap = s.snap; s2.ov = s.ov;
  const int h = (n + 1) / 2, u = n - h;
  const uint32_t *x = s.sa, *y = s.sb + K;
  grp_mul<G, KS, R>(g, P, Ptr{x, h}, h, Ptr{y, h}, h, s2);                    // z0 -> P[0, 2h)
  grp_mul<G, KS, R>(g, P + 2 * h, Ptr{x + h, u}, u, Ptr{y + h, u}, u, s2);    // z2 -> P[2h, 2n)
  // sx, sy staged in place for the middle product (KS zero limbs below sy, zeros above both)
  const uint32_t cx = grp_add<G>(g, s2.sa, Ptr{x, h}, Ptr{x + h, u}, h, 0u);
  const uint32_t cy = grp_add<G>(g, s2.sb + KS, Ptr{y, h}, Ptr{y + h, u}, h, 0u);
  const int M = (h + KS - 1) / KS;
  for (int i = g.lane; i < M * KS + 2 * KS; i += G) {
    if (i >= h && i < M * KS) s2.sa[i] = 0u;
    if (i < KS || i >= KS + h) s2.sb[i] = 0u;
  }
  g.sync();
  uint32_t *Z1 = s.sb;                                                         // 2h+2 <= n+3 limbs
  grp_mul_call<G, KS, R>(g, Z1, h, h, s2);                                     // sx sy -> Z1[0, 2h)
  if (g.lane == 0) { Z1[2 * h] = cx & cy; Z1[2 * h + 1] = 0u; }
  g.sync();
  if (cx) grp_add<G>(g, Z1 + h, Ptr{Z1 + h, h + 2}, Ptr{s2.sb + KS, h}, h + 2, 0u);
  if (cy) grp_add<G>(g, Z1 + h, Ptr{Z1 + h, h + 2}, Ptr{s2.sa, h}, h + 2, 0u);
  grp_sub<G>(g, Z1, Ptr{Z1, 2 * h + 2}, Ptr{P, 2 * h}, 2 * h + 2, 0u);          // - z0
  grp_sub<G>(g, Z1, Ptr{Z1, 2 * h + 2}, Ptr{P + 2 * h, 2 * u}, 2 * h + 2, 0u);  // - z2
  grp_add<G>(g, P + h, Ptr{P + h, 2 * n - h}, Ptr{Z1, 2 * h + 2}, 2 * n - h, 0u);
  for (int i = g.lane; i < K; i += G) s.sb[i] = 0u;
  g.sync();
}

// ---------------------------------------------------------------------------------------
// mul.  Reference: fpa_warp_mul.h:41-139.  Exact 2n-limb product, one rounding.
// Range (:124-128): TINY when BIAS+e < 5, INF when BIAS+e > 0x7FFFFFFF.
// kws != nullptr: the product takes the Karatsuba split (N + K words of staging), compiled
// into the configurations that hold at least 256 limbs on tiles of at least 8 limbs (the
// split only pays at large sizes; out of line so that the schoolbook path keeps its
// registers).
template <int G, int K, int R>
__device__ __forceinline__ void op_mul_staged(const Grp<G> &g, const MulScratch<G, K, R> &s, uint32_t *P, int n,
                                              int mode, uint32_t a_exp, uint32_t b_exp, uint32_t *r_exp,
                                              uint32_t *r, uint32_t *kws = nullptr) {
  const uint32_t act = c_action[2][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_MUL) { write_class<G>(g, r_exp, act); return; }
  if constexpr (KaratsubaCfg<G, K, R>::on) {
    if (kws) grp_mul_karatsuba<G, K, R>(g, P, n, s, kws);
    else grp_mulsq_staged<G, K, R>(g, P, n, s);
  } else {
    grp_mulsq_staged<G, K, R>(g, P, n, s);
  }
  const uint32_t sign = (a_exp ^ b_exp) & 1u;
  Rounded res;
  grp_round<G>(g, P, 2 * n, n, 0u, mode, sign, res);
  const long long e = (long long)(a_exp >> 1) + (long long)(b_exp >> 1) - 2LL * BIAS - 64LL * n + res.L + res.ovf;
  if ((long long)BIAS + e < 5) { write_class<G>(g, r_exp, CLS_POS_TINY - sign); return; }
  if ((long long)BIAS + e > 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sign); return; }
  write_value<G>(g, r_exp, r, n, res, exp_word(e, sign));
}

template <int G, int K, int R>
__device__ void op_mul(const Grp<G> &g, uint32_t *ws, int n, int mode,
                       uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b,
                       uint32_t *r_exp, uint32_t *r) {
  const uint32_t act = c_action[2][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_MUL) { write_class<G>(g, r_exp, act); return; }
  MulScratch<G, K, R> s; s.carve(ws);
  uint32_t *P = ws + MulScratch<G, K, R>::words();
  const int Mp = (n + K - 1) / K, NK = Mp * K;
  for (int i = g.lane; i < NK; i += G) s.sa[i] = (i < n) ? a[i] : 0u;
  for (int i = g.lane; i < NK + 2 * K; i += G) { int j = i - K; s.sb[i] = (j >= 0 && j < n) ? b[j] : 0u; }
  g.sync();
  op_mul_staged<G, K, R>(g, s, P, n, mode, a_exp, b_exp, r_exp, r);
}

// ---------------------------------------------------------------------------------------
// fma: r = RND(a*b + c) with one rounding (no counterpart in the reference).  Special
// values: the mul table gives the class of the exact product, the add table combines it
// with c.  A product that is a value with c = 0 or tiny rounds like fpa_mul; otherwise the
// exact 2n-limb product and c are summed exactly in a window of at most 3n+4 limbs (an
// operand lying wholly more than 64 bits below the other's lowest bit matters only as a
// sticky / borrow and is moved up to just below that guard) and rounded once.  Results
// outside the exponent range become +-INF (BIAS+e > 0x7FFFFFFF) or +-TINY (BIAS+e < 5).
template <int G>
__device__ __forceinline__ int grp_bitlen(const Grp<G> &g, const uint32_t *X, int len) {
  uint32_t top = 0;
  for (int i = g.lane; i < len; i += G) if (X[i]) top = (uint32_t)i + 1u;
  top = g.rmax(top);
  return top == 0 ? 0 : 32 * ((int)top - 1) + 32 - (int)clz32(X[top - 1]);
}

template <int G, int K, int R>
__device__ void op_fma(const Grp<G> &g, uint32_t *ws, int n, int mode, uint32_t a_exp, const uint32_t *a,
                       uint32_t b_exp, const uint32_t *b, uint32_t c_exp, const uint32_t *c, uint32_t *r_exp,
                       uint32_t *r) {
  constexpr int N = G * K * R;
  const uint32_t pm = c_action[2][classify(a_exp) * 9 + classify(b_exp)];
  const uint32_t sp = (a_exp ^ b_exp) & 1u;
  const uint32_t pcls = pm == ACT_MUL ? sp : pm;          // class of the exact product
  const uint32_t act = c_action[0][pcls * 9 + classify(c_exp)];
  if (act == ACT_COPY_B) { copy_value<G>(g, r_exp, r, n, c_exp, c); return; }
  if (act != ACT_COPY_A && act != ACT_ADD && act != ACT_SUB) { write_class<G>(g, r_exp, act); return; }
  MulScratch<G, K, R> s; s.carve(ws);
  uint32_t *P = ws + MulScratch<G, K, R>::words(), *X = P + (2 * N + 4);
  const int Mp = (n + K - 1) / K, NK = Mp * K;
  for (int i = g.lane; i < NK; i += G) s.sa[i] = (i < n) ? a[i] : 0u;
  for (int i = g.lane; i < NK + 2 * K; i += G) { int j = i - K; s.sb[i] = (j >= 0 && j < n) ? b[j] : 0u; }
  g.sync();
  grp_mulsq_staged<G, K, R>(g, P, n, s);
  long long lowP = (long long)(a_exp >> 1) + (long long)(b_exp >> 1) - 2LL * BIAS - 64LL * n;   // a*b = P*2^lowP
  if (act == ACT_COPY_A) {                                 // c is zero or tiny: the rounded product
    Rounded res;
    grp_round<G>(g, P, 2 * n, n, 0u, mode, sp, res);
    const long long e = lowP + res.L + res.ovf;
    if ((long long)BIAS + e < 5) { write_class<G>(g, r_exp, CLS_POS_TINY - sp); return; }
    if ((long long)BIAS + e > 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sp); return; }
    write_value<G>(g, r_exp, r, n, res, exp_word(e, sp));
    return;
  }
  const uint32_t sc = c_exp & 1u;
  const long long ec = (long long)(c_exp >> 1) - BIAS;
  long long lowC = ec - 32LL * n, topC = ec;                // c = C*2^lowC, C normalized
  long long topP = lowP + grp_bitlen<G>(g, P, 2 * n);
  if (topC < lowP - 64) { lowC = lowP - 64 - 32LL * n; topC = lowC + 32LL * n; }
  else if (topP < lowC - 64) { const long long sh = (lowC - 64 - 64LL * n) - lowP; lowP += sh; topP += sh; }
  const long long lo = lowP < lowC ? lowP : lowC, hi = topP > topC ? topP : topC;
  const int xl = (int)((hi - lo) >> 5) + 2;                // <= 3n + 4
  const Shifted xp{P, 2 * n, (int)(lowP - lo)}, xc{c, n, (int)(lowC - lo)};
  uint32_t sign = sp;
  if (sp == sc) grp_add<G>(g, X, xp, xc, xl, 0u);
  else {
    const int cmp = grp_cmp<G>(g, xp, xc, xl);
    if (cmp == 0) { write_class<G>(g, r_exp, CLS_ZERO); return; }   // exact cancellation
    if (cmp > 0) grp_sub<G>(g, X, xp, xc, xl, 0u);
    else { grp_sub<G>(g, X, xc, xp, xl, 0u); sign = sc; }
  }
  Rounded res;
  grp_round<G>(g, X, xl, n, 0u, mode, sign, res);
  const long long e = lo + res.L + res.ovf;
  if ((long long)BIAS + e > 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sign); return; }
  if ((long long)BIAS + e < 5) { write_class<G>(g, r_exp, CLS_POS_TINY - sign); return; }
  write_value<G>(g, r_exp, r, n, res, exp_word(e, sign));
}

// ---------------------------------------------------------------------------------------
// Newton level schedule: levels k_0 = 1 < k_1 < ... < k_last = n with
// k_{j+1} <= 2 k_j - 1 (except 1 -> 2), so the quadratic error term stays below one ulp.
__device__ __forceinline__ int newton_levels(int n, int *lv) {
  int tmp[24], c = 0;
  int k = n;
  tmp[c++] = k;
  while (k > 1) {
    int p = (k + 2) / 2;
    if (p >= k) p = k - 1;
    k = p;
    tmp[c++] = k;
  }
  for (int i = 0; i < c; i++) lv[i] = tmp[c - 1 - i];
  return c;
}

// m * p as limbs (len+1 limbs) for a small multiplier m in {0, 1, 2, 4}
struct SmallMul {
  const uint32_t *p; int len; uint32_t m;
  __device__ __forceinline__ uint32_t operator()(int i) const {
    uint32_t v = (i >= 0 && i < len) ? p[i] : 0u, w = (i - 1 >= 0 && i - 1 < len) ? p[i - 1] : 0u;
    switch (m) {
      case 0: return 0u;
      case 1: return v;
      case 2: return (v << 1) | (w >> 31);
      default: return (v << 2) | (w >> 30);   // 4
    }
  }
};

// Newton residual magnitude read straight from a product T ~ 2^(32L):
// |E| = |2^(32L) - T|, returned as limbs of |E| >> 32*off (i < len).  When T >= 2^(32L)
// (neg) the low limbs of T are |E| itself; otherwise |E| = ~T + 1 and the +1 is dropped
// (an error of one unit at 2^(32*off), far below the precision the step needs).
struct ResidualMag {
  const uint32_t *T; int off, L, len; uint32_t neg;
  __device__ __forceinline__ uint32_t operator()(int i) const {
    if (i < 0 || i >= len) return 0u;
    const int idx = off + i;
    if (idx >= L) return 0u;
    const uint32_t v = T[idx];
    return neg ? v : ~v;
  }
};

// ---------------------------------------------------------------------------------------
// The small Newton levels (k' <= SMALL_LEVEL limbs) of div and sqrt, run by one lane in
// registers.  Group products cost a roughly fixed latency (staging, block sums, syncs)
// however small they are, which made each of these levels as slow as a 17-limb one; here
// every (k, k') pair is its own instantiation with compile-time sizes.  The steps and
// truncations are exactly those of the group levels in op_div / op_sqrt, so the iterates
// are the same integers.  Levels: k' = 2 comes from k = 1, otherwise k = floor((k'+2)/2).
constexpr int SMALL_LEVEL = 9;

// t = a * b (one thread)
template <int LA, int LB>
__device__ __forceinline__ void mul_regs(const uint32_t (&a)[LA], const uint32_t (&b)[LB], uint32_t (&t)[LA + LB]) {
#pragma unroll
  for (int i = 0; i < LA + LB; i++) t[i] = 0u;
#pragma unroll
  for (int i = 0; i < LA; i++) {
    uint32_t carry = 0;
#pragma unroll
    for (int j = 0; j < LB; j++) {
      const uint64_t x = (uint64_t)a[i] * b[j] + t[i + j] + carry;
      t[i + j] = (uint32_t)x; carry = (uint32_t)(x >> 32);
    }
    t[i + LB] = carry;
  }
}

// y' = y * 2^(32(kp-k)) +- (m >> sh) over kp+1 limbs (sh in {0, 1} bits; m of LM limbs,
// read from limb MO up)
template <int k, int kp, int LM, int MO>
__device__ __forceinline__ void level_update(const uint32_t (&y)[k + 1], const uint32_t (&m)[LM], int sh, bool neg,
                                             uint32_t (&out)[SMALL_LEVEL + 1]) {
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i <= SMALL_LEVEL; i++) {
    if (i > kp) { out[i] = 0u; continue; }
    const uint32_t ys = (i >= kp - k) ? y[i - (kp - k)] : 0u;
    const uint32_t lo = (MO + i < LM) ? m[MO + i] : 0u, hi = (MO + i + 1 < LM) ? m[MO + i + 1] : 0u;
    const uint32_t mv = sh ? ((lo >> 1) | (hi << 31)) : lo;
    if (!neg) { const uint64_t v = (uint64_t)ys + mv + c; out[i] = (uint32_t)v; c = (uint32_t)(v >> 32); }
    else { const uint64_t v = (uint64_t)ys - mv - c; out[i] = (uint32_t)v; c = (uint32_t)(v >> 63); }
  }
}

// div level k -> kp: T = B_kp * Y, E from T, Y' = Y 2^(32(kp-k)) +- (Y |E|) >> 32(k+1)
template <int k, int kp>
__device__ __forceinline__ void div_level_regs(const uint32_t (&bt)[SMALL_LEVEL], uint32_t (&y)[SMALL_LEVEL + 1]) {
  constexpr int L = k + kp, lt = kp - k + 3;
  uint32_t bk[kp], yk[k + 1], t[kp + k + 1], em[lt], p[k + 1 + lt];
#pragma unroll
  for (int i = 0; i < kp; i++) bk[i] = bt[SMALL_LEVEL - kp + i];
#pragma unroll
  for (int i = 0; i <= k; i++) yk[i] = y[i];
  mul_regs<kp, k + 1>(bk, yk, t);
  const bool neg = t[L] != 0u;
#pragma unroll
  for (int i = 0; i < lt; i++) em[i] = (k - 1 + i < L) ? (neg ? t[k - 1 + i] : ~t[k - 1 + i]) : 0u;
  mul_regs<k + 1, lt>(yk, em, p);
  level_update<k, kp, k + 1 + lt, k + 1>(yk, p, 0, neg, y);
}

// sqrt level k -> kp: V = (X_kp Z) Z without the low j = k-2 limbs of X_kp Z,
// E = 2^(32(kp+2k)) - V, Z' = Z 2^(32(kp-k)) +- (Z |E|) >> (32(k+1)+1)
template <int k, int kp>
__device__ __forceinline__ void sqrt_level_regs(const uint32_t (&xt)[SMALL_LEVEL], uint32_t (&z)[SMALL_LEVEL + 1]) {
  constexpr int j = k > 2 ? k - 2 : 0, l1 = kp + k + 1 - j, L = kp + 2 * k - j, lt = kp - k + 3;
  uint32_t xk[kp], zk[k + 1], v1[kp + k + 1], t1[l1], w[l1 + k + 1], em[lt], p[k + 1 + lt];
#pragma unroll
  for (int i = 0; i < kp; i++) xk[i] = xt[SMALL_LEVEL - kp + i];
#pragma unroll
  for (int i = 0; i <= k; i++) zk[i] = z[i];
  mul_regs<kp, k + 1>(xk, zk, v1);
#pragma unroll
  for (int i = 0; i < l1; i++) t1[i] = v1[j + i];
  mul_regs<l1, k + 1>(t1, zk, w);
  const bool neg = w[L] != 0u;
#pragma unroll
  for (int i = 0; i < lt; i++) {
    const int idx = 2 * k - 1 - j + i;
    em[i] = (idx < L) ? (neg ? w[idx] : ~w[idx]) : 0u;
  }
  mul_regs<k + 1, lt>(zk, em, p);
  level_update<k, kp, k + 1 + lt, k + 1>(zk, p, 1, neg, z);
}

// Runs levels lv[1 .. end) (all k' <= SMALL_LEVEL) on the calling lane; v holds level 1's
// two limbs on entry and the last level's limbs on return.
template <bool SQRT>
__device__ __noinline__ void small_levels(const uint32_t (&top)[SMALL_LEVEL], const int *lv, int end,
                                          uint32_t (&v)[SMALL_LEVEL + 1]) {
  for (int li = 1; li < end; li++) {
    switch (lv[li]) {
#define GFPA_SMALL_LEVEL(K_, KP_) \
      case KP_: if (SQRT) sqrt_level_regs<K_, KP_>(top, v); else div_level_regs<K_, KP_>(top, v); break;
      GFPA_SMALL_LEVEL(1, 2) GFPA_SMALL_LEVEL(2, 3) GFPA_SMALL_LEVEL(3, 4) GFPA_SMALL_LEVEL(3, 5)
      GFPA_SMALL_LEVEL(4, 6) GFPA_SMALL_LEVEL(4, 7) GFPA_SMALL_LEVEL(5, 8) GFPA_SMALL_LEVEL(5, 9)
#undef GFPA_SMALL_LEVEL
      default: break;
    }
  }
}

// first level index the group runs: the small ones go to small_levels
__device__ __forceinline__ int small_levels_end(const int *lv, int nl, bool km) {
  const int last = km ? nl - 1 : nl;
  int e = 1;
  while (e < last && lv[e] <= SMALL_LEVEL) e++;
  return e;
}

// ---------------------------------------------------------------------------------------
// div.  Reference: fpa_warp_div.h:127-201.
//   1. Y ~ 2^(64n)/B by Newton: Y_k' = Y_k*2^(32(k'-k)) + Y_k*E/2^(64k),
//      E = 2^(32(k+k')) - B_k' * Y_k   (B_k' = top k' limbs of B).
//   2. Q from Y: for n >= 4 the last Newton level is replaced by one Karp-Markstein step
//      (q0 = A*Y_h to half precision, Q = q0 + Y_h * (A - q0*B)) that yields one limb more
//      than the result; when those 32 extra bits are clear of a rounding boundary they
//      decide the rounding directly.  Otherwise (and for n < 4, Q = floor(A*Y / 2^(32n)))
//      one exact correction: R = A*2^(32n) - Q*B is formed from the low n+2 limbs and Q is
//      stepped until 0 <= R < B.
//   3. X = 2Q + [2R >= B], sticky = R != 0 (2R == B is impossible for a quotient of two
//      precision-p numbers), rounded once.
// Range (:189-193): TINY when BIAS+e < 10, INF when BIAS+e >= 0x7FFFFFFF.
template <int G, int K, int R>
__device__ void op_div(const Grp<G> &g, uint32_t *ws, int n, int mode,
                       uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b,
                       uint32_t *r_exp, uint32_t *r, uint32_t *err) {
  constexpr int N = G * K * R;
  const uint32_t act = c_action[3][classify(a_exp) * 9 + classify(b_exp)];
  if (act != ACT_DIV) { write_class<G>(g, r_exp, act); return; }
  MulScratch<G, K, R> s; s.carve(ws);
  // the operands are read where they lie (a, b): only the quotient's state is staged
  // With the Karp-Markstein last step Y never exceeds h+1 <= n/2+2 limbs and T never holds
  // more than n+3 (n < 4 takes the full-level path, whose 2n+2-limb A*Y fits N+8 there).
  uint32_t *Y = ws + MulScratch<G, K, R>::words(), *Y2 = Y + (N / 2 + 8);
  uint32_t *T = Y2 + (N / 2 + 8), *P2 = T + (N + 8);
  uint32_t *Q = P2 + (2 * N + 8);
  uint32_t *Rm = T;                  // T is dead once Q is formed
  uint32_t *X = P2;                  // P2 (Q*B) is dead once Rm is formed
  int lv[24];
  const int nl = newton_levels(n, lv);
  const bool km = n >= 4;                      // last level replaced by one Karp-Markstein step
  const int l0 = small_levels_end(lv, nl, km);
  if (g.lane == 0) {
    uint64_t y = 0xFFFFFFFFFFFFFFFFull / (uint64_t)b[n - 1];   // level 1: floor((2^64-1)/B_top)
    uint32_t v[SMALL_LEVEL + 1], bt[SMALL_LEVEL];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) v[i] = 0u;
    v[0] = (uint32_t)y; v[1] = (uint32_t)(y >> 32);
#pragma unroll
    for (int i = 0; i < SMALL_LEVEL; i++) bt[i] = (n - SMALL_LEVEL + i >= 0) ? b[n - SMALL_LEVEL + i] : 0u;
    small_levels<false>(bt, lv, l0, v);
    const int k = lv[l0 - 1];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) if (i <= k) Y[i] = v[i];
  }
  g.sync();
  for (int li = l0; li < (km ? nl - 1 : nl); li++) {
    const int k = lv[li - 1], kp = lv[li];
    const uint32_t *Bk = b + (n - kp);
    // T = B_k' * Y_k   (k' x (k+1) limbs)
    grp_mul<G, K, R>(g, T, Ptr{Bk, kp}, kp, Ptr{Y, k + 1}, k + 1, s);
    // M = (Y_k * (|E| >> 32(k-1))) >> 32(k+1)
    const int L = k + kp, lt = kp - k + 3;
    const uint32_t neg = T[L] != 0u;
    grp_mul<G, K, R>(g, P2, Ptr{Y, k + 1}, k + 1, ResidualMag{T, k - 1, L, lt, neg}, lt, s);
    // Y_k' = Y_k * 2^(32(k'-k)) +- M   (E <= 0 means Y_k was too large)
    Shifted ysh{Y, k + 1, 32 * (kp - k)};
    Ptr M{P2 + (k + 1), lt};
    if (neg) grp_sub<G>(g, Y2, ysh, M, kp + 1, 0u);
    else grp_add<G>(g, Y2, ysh, M, kp + 1, 0u);
    uint32_t *tmp = Y; Y = Y2; Y2 = tmp;
  }
  if (km) {
    // Karp-Markstein with one limb more than the result needs: with Y = Y_h (h = the level
    // below n, a = A/2^(32n), y = 2^(32n)/B) and m = n+2-h,
    //   q0 = floor(At * Y / 2^(32(h+1))) ~ a y 2^(32m), At = top m+1 limbs of A,
    //   D  = (A 2^(32(n+1)) - q0 B 2^(32(h-1))) / 2^(32(n-2))   (|D| < 2^(32(m+2))),
    //   Q' = q0 2^(32(h-1)) + floor(D Y / 2^(32(h+2)))  ~ (A/B) 2^(32(n+1)),  n+2 limbs.
    // m is chosen so that the error of Y_h and the quadratic term stay within a few units
    // of Q' (at most 9 over every size 4..512 in an exact integer simulation of these
    // steps).  When the bits of Q' below the result's last place lie at least 2^20 units
    // away from 0 and from one half, they decide the rounding on their own (round bit =
    // their top bit, sticky = 1); otherwise floor(Q'/2^32) takes the exact correction.
    const int h = lv[nl - 2], m = n + 2 - h;
    grp_mul<G, K, R>(g, T, Ptr{a + (n - m - 1), m + 1}, m + 1, Ptr{Y, h + 1}, h + 1, s);
    uint32_t *q0 = Y2;                         // m+1 limbs
    grp_copy<G>(g, q0, Ptr{T + (h + 1), m + 1}, m + 1);
    grp_mul<G, K, R>(g, P2, Ptr{q0, m + 1}, m + 1, Ptr{b, n}, n, s);
    const int dl = n + 4;
    const Shifted xa{a, n, 96}, xq{P2, n + m + 1, -32 * (n - h - 1)};
    const bool dneg = grp_cmp<G>(g, xa, xq, dl) < 0;
    if (dneg) grp_sub<G>(g, T, xq, xa, dl, 0u);
    else grp_sub<G>(g, T, xa, xq, dl, 0u);
    const int dlen = m + 2;                    // <= n/2 + 4: within the group's capacity
    grp_mul<G, K, R>(g, P2, Ptr{T, dlen}, dlen, Ptr{Y, h + 1}, h + 1, s);
    const Shifted qs{q0, m + 1, 32 * (h - 1)}, cs{P2, dlen + h + 1, -32 * (h + 2)};
    if (dneg) grp_sub<G>(g, Q, qs, cs, n + 2, 0u);
    else grp_add<G>(g, Q, qs, cs, n + 2, 0u);
    // Q' lies in (2^(32n+31), 2^(32n+33)): 32 bits below the last place when Q'[n+1] = 0,
    // else 33 (their top bit in Q'[1]); u = those bits without their top bit
    const uint32_t qtop = Q[n + 1], u = qtop ? Q[0] : (Q[0] & 0x7FFFFFFFu);
    const uint32_t umax = qtop ? 0xFFFFFFFFu : 0x7FFFFFFFu;
    if (u >= (1u << 20) && u <= umax - (1u << 20)) {
      const uint32_t sign = (a_exp ^ b_exp) & 1u;
      Rounded res;
      grp_round<G>(g, Q, n + 2, n, 1u, mode, sign, res);
      const long long e = (long long)(a_exp >> 1) - (long long)(b_exp >> 1) - 32LL * n - 32 + res.L + res.ovf;
      if ((long long)BIAS + e < 10) { write_class<G>(g, r_exp, CLS_POS_TINY - sign); return; }
      if ((long long)BIAS + e >= 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sign); return; }
      write_value<G>(g, r_exp, r, n, res, exp_word(e, sign));
      return;
    }
    Q += 1;                                    // floor(Q'/2^32): n+1 limbs, within one unit
  } else {
    // Q = floor(A * Y / 2^(32n)),  n+1 limbs;  Y = ytop*2^(32n) + Ylow
    const uint32_t ytop = Y[n];
    grp_mulsq<G, K, R>(g, T, Ptr{a, n}, Ptr{Y, n}, n, s);
    if (g.lane == 0) { T[2 * n] = 0; T[2 * n + 1] = 0; }
    g.sync();
    grp_add<G>(g, T + n, Ptr{T + n, n + 2}, SmallMul{a, n, ytop}, n + 2, 0u);
    grp_copy<G>(g, Q, Ptr{T + n, n + 2}, n + 1);
  }
  // Rm = (A * 2^(32n) - Q * B) mod 2^(32(n+2))
  const uint32_t qtop = Q[n];
  grp_mulsq<G, K, R>(g, P2, Ptr{Q, n}, Ptr{b, n}, n, s);
  if (g.lane == 0) { P2[2 * n] = 0; P2[2 * n + 1] = 0; P2[2 * n + 2] = 0; }
  g.sync();
  grp_add<G>(g, P2 + n, Ptr{P2 + n, n + 3}, SmallMul{b, n, qtop}, n + 3, 0u);
  grp_sub<G>(g, Rm, Shifted{a, n, 32 * n}, Ptr{P2, 2 * n + 3}, n + 2, 0u);
  // exact correction: 0 <= Rm < B
  int guard = 0;
  while ((Rm[n + 1] >> 31) != 0 && guard < 64) {
    grp_sub<G>(g, Q, Ptr{Q, n + 1}, Zero{}, n + 1, 1u);
    grp_add<G>(g, Rm, Ptr{Rm, n + 2}, Ptr{b, n}, n + 2, 0u);
    guard++;
  }
  while (grp_cmp<G>(g, Ptr{Rm, n + 2}, Ptr{b, n}, n + 2) >= 0 && guard < 64) {
    grp_add<G>(g, Q, Ptr{Q, n + 1}, Zero{}, n + 1, 1u);
    grp_sub<G>(g, Rm, Ptr{Rm, n + 2}, Ptr{b, n}, n + 2, 0u);
    guard++;
  }
  if (guard >= 64 && g.lane == 0) atomicOr(err, 1u);
  const int c2 = grp_cmp<G>(g, ShlBits{Rm, n + 2, 1}, Ptr{b, n}, n + 2);
  const uint32_t rb = c2 >= 0 ? 1u : 0u;
  const uint32_t sticky = (!grp_is_zero<G>(g, Ptr{Rm, n + 2}, n + 2) && c2 != 0) ? 1u : 0u;
  // X = 2Q + rb  (n+2 limbs)
  grp_add<G>(g, X, ShlBits{Q, n + 1, 1}, Zero{}, n + 2, rb);
  const uint32_t sign = (a_exp ^ b_exp) & 1u;
  Rounded res;
  grp_round<G>(g, X, n + 2, n, sticky, mode, sign, res);
  const long long e = (long long)(a_exp >> 1) - (long long)(b_exp >> 1) - 32LL * n - 1 + res.L + res.ovf;
  if ((long long)BIAS + e < 10) { write_class<G>(g, r_exp, CLS_POS_TINY - sign); return; }
  if ((long long)BIAS + e >= 0x7FFFFFFFLL) { write_class<G>(g, r_exp, CLS_POS_INF - sign); return; }
  write_value<G>(g, r_exp, r, n, res, exp_word(e, sign));
}

// integer square root of a 64-bit value (bitwise, exact)
__device__ __forceinline__ uint64_t isqrt64(uint64_t x) {
  uint64_t r = 0, bit = 1ull << 62;
  while (bit > x) bit >>= 2;
  while (bit) {
    if (x >= r + bit) { x -= r + bit; r = (r >> 1) + bit; }
    else r >>= 1;
    bit >>= 2;
  }
  return r;
}

// ---------------------------------------------------------------------------------------
// sqrt.  Reference: fpa_warp_sqrt.h:195-254 (odd exponents are made even, :218-223).
//   A_ext = A * 2^(32n) (even e) or A * 2^(32n-1) (odd e), S* = sqrt(A_ext) in [2^(32n-1), 2^(32n)).
//   1. Z ~ 2^(32k)/sqrt(x) by Newton on 1/sqrt: Z_k' = Z_k*2^(32(k'-k)) + Z_k*E/2^(96k+1),
//      E = 2^(32(k'+2k)) - (X_k' * Z_k) * Z_k   (X_k' = top k' limbs of A_ext; the low
//      limbs of the inner product that cannot reach the limbs of E used are dropped).
//   2. S from Z: for n >= 4 the last Newton level is replaced by one Karp-Markstein step
//      (S0 = sqrt(x) to half precision from Z, S = S0 + Z (A_ext - S0^2) / 2), otherwise
//      S = floor(A * Z / 2^(32n [+1])); then one exact correction with R = A_ext - S^2
//      until 0 <= R <= 2S.
//   3. X = 2S + [R > S], sticky = R != 0, rounded once (positive).
template <int G, int K, int R>
__device__ void op_sqrt(const Grp<G> &g, uint32_t *ws, int n, int mode,
                        uint32_t a_exp, const uint32_t *a, uint32_t *r_exp, uint32_t *r, uint32_t *err) {
  constexpr int N = G * K * R;
  const uint32_t act = c_sqrt_action[classify(a_exp)];
  if (act != ACT_SQRT) { write_class<G>(g, r_exp, act); return; }
  MulScratch<G, K, R> s; s.carve(ws);
  // A_ext = A * 2^(32n - odd) has 2n limbs of which the low n-1 are zero: only its top n+1
  // limbs Xh = A * 2^(32 - odd) are kept (A_ext limb i = Xh[i - (n-1)]).
  // With the Karp-Markstein last step Z never exceeds h+1 <= n/2+2 limbs and the Newton
  // products stay below 3n/4+8 limbs (n < 4 takes the full-level path).
  uint32_t *Xh = ws + MulScratch<G, K, R>::words();
  uint32_t *Z = Xh + (N + 4), *Z2 = Z + (N / 2 + 8);
  uint32_t *W = Z2 + (N / 2 + 8);    // T2 (<= 3n/4+8 limbs), later S0^2 (2m+2 <= n+3) and the rounded integer
  uint32_t *V1 = W + (N + 8), *P = V1 + (2 * N + 8), *S = P + (N + 8);
  uint32_t *Rm = P;                  // P (Z*E, then |D|) is dead once S is formed
  uint32_t *E = W;                   // W is dead once S is formed
  const long long e = (long long)(a_exp >> 1) - BIAS;
  const int odd = (int)(e & 1);
  const long long eh = (e + odd) / 2;          // exact: e + odd is even
  grp_copy<G>(g, Xh, Shifted{a, n, 32 - odd}, n + 1);
  int lv[24];
  const int nl = newton_levels(n, lv);
  const bool km = n >= 4;                      // last level replaced by one Karp-Markstein step
  const int l0 = small_levels_end(lv, nl, km);
  if (g.lane == 0) {
    uint64_t x1 = (uint64_t)Xh[n] << 32;                   // top limb of A_ext, in [2^30, 2^32)
    uint64_t s1 = isqrt64(x1);                             // in [2^31, 2^32)
    uint64_t z = 0xFFFFFFFFFFFFFFFFull / s1;               // level 1: ~ 2^32 / sqrt(x)
    uint32_t v[SMALL_LEVEL + 1], xt[SMALL_LEVEL];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) v[i] = 0u;
    v[0] = (uint32_t)z; v[1] = (uint32_t)(z >> 32);
#pragma unroll
    for (int i = 0; i < SMALL_LEVEL; i++) xt[i] = (n + 1 - SMALL_LEVEL + i >= 0) ? Xh[n + 1 - SMALL_LEVEL + i] : 0u;
    small_levels<true>(xt, lv, l0, v);
    const int k = lv[l0 - 1];
#pragma unroll
    for (int i = 0; i <= SMALL_LEVEL; i++) if (i <= k) Z[i] = v[i];
  }
  g.sync();
  for (int li = l0; li < (km ? nl - 1 : nl); li++) {
    const int k = lv[li - 1], kp = lv[li];
    // V = X_k' Z_k^2 as (X_k' Z_k) Z_k: the low j = k-2 limbs of T1 = X_k' Z_k only reach V
    // below limb 2k-1, the lowest limb of E that is read, so T2 = (T1 >> 32j) Z_k = V / 2^(32j)
    const uint32_t *Xk = Xh + (n + 1 - kp);             // top k' limbs of A_ext (k' <= n)
    grp_mul<G, K, R>(g, V1, Ptr{Xk, kp}, kp, Ptr{Z, k + 1}, k + 1, s);
    const int j = k > 2 ? k - 2 : 0, l1 = kp + k + 1 - j;
    grp_mul<G, K, R>(g, W, Ptr{V1 + j, l1}, l1, Ptr{Z, k + 1}, k + 1, s);
    // M = (Z_k * (|E| >> 32(2k-1))) >> (32(k+1) + 1),  E = 2^(32(k'+2k)) - V
    const int L = kp + 2 * k - j, lt = kp - k + 3;    // L: limb of 2^(32(k'+2k)) in T2
    const uint32_t neg = W[L] != 0u;
    grp_mul<G, K, R>(g, P, Ptr{Z, k + 1}, k + 1, ResidualMag{W, 2 * k - 1 - j, L, lt, neg}, lt, s);
    Shifted zsh{Z, k + 1, 32 * (kp - k)};
    Shifted M{P, k + 1 + lt, -(32 * (k + 1) + 1)};
    if (neg) grp_sub<G>(g, Z2, zsh, M, kp + 1, 0u);
    else grp_add<G>(g, Z2, zsh, M, kp + 1, 0u);
    uint32_t *tmp = Z; Z = Z2; Z2 = tmp;
  }
  if (km) {
    // Karp-Markstein with one limb more than the result needs: with Z = Z_h (h = the level
    // below n, x = A_ext / 2^(64n)) and m = n+2-h,
    //   S0 = floor(Xt * Z / 2^(32(h+1))) ~ sqrt(x) 2^(32m), Xt = top m+1 limbs of A_ext,
    //   D  = (A_ext 2^64 - S0^2 2^(64(h-1))) / 2^(32(n-2))   (|D| < 2^(32(m+3))),
    //   S' = S0 2^(32(h-1)) + floor(D Z / 2^(32(h+3)+1))  ~ sqrt(A_ext) 2^32,  n+2 limbs.
    // m is chosen so that Z_h's error and the quadratic term stay within a few units of S'
    // (at most 3 over every size 4..512 in an exact integer simulation of these steps).
    // When the 32 bits of S' below the result's last place lie at least 2^20 units away
    // from 0 and from one half, they decide the rounding on their own (round bit = their
    // top bit, sticky = 1); otherwise floor(S'/2^32) takes the exact correction.
    const int h = lv[nl - 2], m = n + 2 - h;
    grp_mul<G, K, R>(g, V1, Ptr{Xh + (n - m), m + 1}, m + 1, Ptr{Z, h + 1}, h + 1, s);
    uint32_t *S0 = Z2;                         // m+1 limbs
    grp_copy<G>(g, S0, Ptr{V1 + (h + 1), m + 1}, m + 1);
    grp_mulsq<G, K, R>(g, W, Ptr{S0, m + 1}, Ptr{S0, m + 1}, m + 1, s);
    const int dl = n + 6;
    const Shifted xs{Xh, n + 1, 96}, ss{W, 2 * m + 2, 32 * (2 * h - n)};
    const bool dneg = grp_cmp<G>(g, xs, ss, dl) < 0;
    if (dneg) grp_sub<G>(g, P, ss, xs, dl, 0u);
    else grp_sub<G>(g, P, xs, ss, dl, 0u);
    const int dlen = m + 3;                    // <= n/2 + 5: within the group's capacity
    grp_mul<G, K, R>(g, V1, Ptr{P, dlen}, dlen, Ptr{Z, h + 1}, h + 1, s);
    const Shifted s0s{S0, m + 1, 32 * (h - 1)}, cs{V1, dlen + h + 1, -(32 * (h + 3) + 1)};
    if (dneg) grp_sub<G>(g, S, s0s, cs, n + 2, 0u);
    else grp_add<G>(g, S, s0s, cs, n + 2, 0u);
    // S' lies in [2^(32n+31), 2^(32n+32)) up to its error: 32 bits below the last place
    const uint32_t u = S[0] & 0x7FFFFFFFu;
    if (S[n + 1] == 0u && u >= (1u << 20) && u <= 0x7FFFFFFFu - (1u << 20)) {
      Rounded res;
      grp_round<G>(g, S, n + 1, n, 1u, mode, 0u, res);
      write_value<G>(g, r_exp, r, n, res, exp_word(eh - 32LL * n - 32 + res.L + res.ovf, 0u));
      return;
    }
    S += 1;                                    // floor(S'/2^32): n+1 limbs, within one unit
  } else {
    // S = floor(A * Z / 2^(32n + odd))   (n+1 limbs)
    const uint32_t ztop = Z[n];
    grp_mulsq<G, K, R>(g, V1, Ptr{a, n}, Ptr{Z, n}, n, s);
    if (g.lane == 0) { V1[2 * n] = 0; V1[2 * n + 1] = 0; }
    g.sync();
    grp_add<G>(g, V1 + n, Ptr{V1 + n, n + 2}, SmallMul{a, n, ztop}, n + 2, 0u);
    grp_copy<G>(g, S, Shifted{V1, 2 * n + 2, -(32 * n + odd)}, n + 1);
  }
  // Rm = (A_ext - S^2) mod 2^(32(n+2)),  S = stop*2^(32n) + Slow
  const uint32_t stop = S[n];
  grp_mulsq<G, K, R>(g, V1, Ptr{S, n}, Ptr{S, n}, n, s);
  if (g.lane == 0) { V1[2 * n] = 0; V1[2 * n + 1] = 0; V1[2 * n + 2] = 0; }
  g.sync();
  grp_add<G>(g, V1 + n, Ptr{V1 + n, n + 3}, SmallMul{S, n, 2u * stop}, n + 3, 0u);
  if (stop) {
    const uint32_t ss = stop * stop;
    grp_add<G>(g, V1 + 2 * n, Ptr{V1 + 2 * n, 3}, Ptr{&ss, 1}, 3, 0u);
  }
  grp_sub<G>(g, Rm, Shifted{Xh, n + 1, 32 * (n - 1)}, Ptr{V1, 2 * n + 3}, n + 2, 0u);
  // exact correction: 0 <= Rm <= 2S
  int guard = 0;
  // the sign limb is read through a shuffle: every lane reads it before the shuffle, so the
  // lane that owns it cannot overwrite it in the loop body while another lane still reads it
  while ((g.bcast(Rm[n + 1], 0) >> 31) != 0 && guard < 64) {       // Rm += 2S - 1, S -= 1
    grp_add<G>(g, Rm, Ptr{Rm, n + 2}, ShlBits{S, n + 1, 1}, n + 2, 0u);
    grp_sub<G>(g, Rm, Ptr{Rm, n + 2}, Zero{}, n + 2, 1u);
    grp_sub<G>(g, S, Ptr{S, n + 1}, Zero{}, n + 1, 1u);
    guard++;
  }
  while (grp_cmp<G>(g, Ptr{Rm, n + 2}, ShlBits{S, n + 1, 1}, n + 2) > 0 && guard < 64) {   // Rm -= 2S + 1, S += 1
    grp_sub<G>(g, Rm, Ptr{Rm, n + 2}, ShlBits{S, n + 1, 1}, n + 2, 1u);
    grp_add<G>(g, S, Ptr{S, n + 1}, Zero{}, n + 1, 1u);
    guard++;
  }
  if (guard >= 64 && g.lane == 0) atomicOr(err, 2u);
  const uint32_t rb = grp_cmp<G>(g, Ptr{Rm, n + 2}, Ptr{S, n + 1}, n + 2) > 0 ? 1u : 0u;
  const uint32_t sticky = grp_is_zero<G>(g, Ptr{Rm, n + 2}, n + 2) ? 0u : 1u;
  grp_add<G>(g, E, ShlBits{S, n + 1, 1}, Zero{}, n + 2, rb);
  Rounded res;
  grp_round<G>(g, E, n + 2, n, sticky, mode, 0u, res);
  const long long er = eh - 32LL * n - 1 + res.L + res.ovf;
  write_value<G>(g, r_exp, r, n, res, exp_word(er, 0u));
}

}  // namespace gfpa
