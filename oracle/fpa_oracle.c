/*
 * fpa_oracle.c -- CPU oracle for cuBigFloat's add/sub/mul/div/sqrt (TEST INFRASTRUCTURE).
 *
 * Restates, in plain C with exact integer arithmetic, what the reference's warp
 * kernels compute.  Every mantissa operation is done exactly (full products, exact
 * long division, exact integer square root) and then rounded once, so the results
 * are the correctly rounded ones that MPFR produces.  The special-value semantics
 * (action tables, class codes, exponent range limits) follow the reference file
 * and line cited beside each piece.  Where the reference's GPU kernels disagree
 * with correct rounding, this oracle follows MPFR (the reference's own test
 * oracle, tests.c:423-485), see `mul_round_divergence` notes below.
 *
 * Only tests/, smoke() and bench.py's CPU-baseline leg use this file.
 */
#include "fpa_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define BIAS 0x3FFFFFF3LL            /* fpa_internal.h:1 */

enum {                                /* fpa_internal.h:9-17 */
  C_POS_VALUE = 0, C_NEG_VALUE = 1, C_ZERO = 2, C_NEG_TINY = 3, C_POS_TINY = 4,
  C_NEG_INF = 5, C_POS_INF = 6, C_NAN = 7, C_SNAN = 8
};
enum {                                /* fpa_internal.h:19-32 (action codes) */
  A_MUL = 16, A_DIV = 17, A_SQRT = 18, A_ADD = 20, A_SUB = 21,
  A_COPY_A = 22, A_COPY_B = 23, A_NEG_B = 24
};

/* ---- special-value action tables -------------------------------------------
 * Rows = class of a, columns = class of b, in class-code order
 * (+value, -value, zero, -tiny, +tiny, -inf, +inf, nan, snan).
 * The entries are the reference's; a table of IEEE-like special cases has to hold
 * the same values to give the same results. */

/* fpa_warp_add_sub.h:15-26 */
static const uint8_t add_table[81] = {
  A_ADD,      A_SUB,      A_COPY_A,   A_COPY_A,   A_COPY_A,   C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  A_SUB,      A_ADD,      A_COPY_A,   A_COPY_A,   A_COPY_A,   C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  A_COPY_B,   A_COPY_B,   C_ZERO,     C_NEG_TINY, C_POS_TINY, C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  A_COPY_B,   A_COPY_B,   C_NEG_TINY, C_NEG_TINY, C_NAN,      C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  A_COPY_B,   A_COPY_B,   C_POS_TINY, C_NAN,      C_POS_TINY, C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NAN,      C_NAN, C_SNAN,
  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_NAN,      C_POS_INF,  C_NAN, C_SNAN,
  C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN, C_SNAN,
};

/* fpa_warp_add_sub.h:28-39 */
static const uint8_t sub_table[81] = {
  A_SUB,      A_ADD,      A_COPY_A,   A_COPY_A,   A_COPY_A,   C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  A_ADD,      A_SUB,      A_COPY_A,   A_COPY_A,   A_COPY_A,   C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  A_NEG_B,    A_NEG_B,    C_ZERO,     C_POS_TINY, C_NEG_TINY, C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  A_NEG_B,    A_NEG_B,    C_NEG_TINY, C_NAN,      C_NEG_INF,  C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  A_NEG_B,    A_NEG_B,    C_POS_TINY, C_POS_TINY, C_NAN,      C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NEG_INF,  C_NAN,      C_NEG_INF,  C_NAN, C_SNAN,
  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_POS_INF,  C_NAN,      C_NAN, C_SNAN,
  C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN, C_SNAN,
};

/* fpa_warp_mul.h:1-12 */
static const uint8_t mul_table[81] = {
  A_MUL,      A_MUL,      C_ZERO,     C_NEG_TINY, C_POS_TINY, C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  A_MUL,      A_MUL,      C_ZERO,     C_POS_TINY, C_NEG_TINY, C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  C_ZERO,     C_ZERO,     C_ZERO,     C_ZERO,     C_ZERO,     C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_NEG_TINY, C_POS_TINY, C_ZERO,     C_POS_TINY, C_NEG_TINY, C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_POS_TINY, C_NEG_TINY, C_ZERO,     C_NEG_TINY, C_POS_TINY, C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_NEG_INF,  C_POS_INF,  C_NAN,      C_NAN,      C_NAN,      C_POS_INF,  C_NEG_INF,  C_NAN, C_SNAN,
  C_POS_INF,  C_NEG_INF,  C_NAN,      C_NAN,      C_NAN,      C_NEG_INF,  C_POS_INF,  C_NAN, C_SNAN,
  C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN, C_SNAN,
};

/* fpa_warp_div.h:1-12 */
static const uint8_t div_table[81] = {
  A_DIV,      A_DIV,      C_NAN,      C_NEG_INF,  C_POS_INF,  C_NEG_TINY, C_POS_TINY, C_NAN, C_SNAN,
  A_DIV,      A_DIV,      C_NAN,      C_POS_INF,  C_NEG_INF,  C_POS_TINY, C_NEG_TINY, C_NAN, C_SNAN,
  C_ZERO,     C_ZERO,     C_NAN,      C_ZERO,     C_ZERO,     C_ZERO,     C_ZERO,     C_NAN, C_SNAN,
  C_NEG_TINY, C_POS_TINY, C_NAN,      C_NAN,      C_NAN,      C_POS_TINY, C_NEG_TINY, C_NAN, C_SNAN,
  C_POS_TINY, C_NEG_TINY, C_NAN,      C_NAN,      C_NAN,      C_NEG_TINY, C_POS_TINY, C_NAN, C_SNAN,
  C_POS_INF,  C_NEG_INF,  C_NAN,      C_POS_INF,  C_NEG_INF,  C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_NEG_INF,  C_POS_INF,  C_NAN,      C_NEG_INF,  C_POS_INF,  C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN,      C_NAN, C_SNAN,
  C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN,     C_SNAN, C_SNAN,
};

/* fpa_warp_sqrt.h:1-11 */
static const uint8_t sqrt_table[9] = {
  A_SQRT, C_NAN, C_ZERO, C_NAN, C_POS_TINY, C_NAN, C_POS_INF, C_NAN, C_SNAN,
};

/* fpa_internal.h:52-60 */
static inline uint32_t classify(uint32_t e) { return e <= C_SNAN ? e : (e & 1u); }

/* ---- exact big-integer helpers (little-endian uint32 limbs) ---------------- */

static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

static int bitlen(const uint32_t *x, int len) {
  for (int i = len - 1; i >= 0; i--)
    if (x[i]) return 32 * i + 32 - clz32(x[i]);
  return 0;
}

static inline int getbit(const uint32_t *x, int len, int bit) {
  if (bit < 0 || bit >= 32 * len) return 0;
  return (x[bit >> 5] >> (bit & 31)) & 1;
}

static int any_below(const uint32_t *x, int len, int bit) {   /* any set bit with index < bit */
  if (bit <= 0) return 0;
  int w = bit >> 5, b = bit & 31;
  if (w >= len) { w = len; b = 0; }
  for (int i = 0; i < w; i++) if (x[i]) return 1;
  if (b && (x[w] & ((1u << b) - 1))) return 1;
  return 0;
}

/* dst[0..dlen) = (src << shift) truncated */
static void shl_into(uint32_t *dst, int dlen, const uint32_t *src, int slen, int shift) {
  memset(dst, 0, sizeof(uint32_t) * dlen);
  int ws = shift >> 5, bs = shift & 31;
  for (int i = 0; i < slen; i++) {
    int k = i + ws;
    if (k < dlen) dst[k] |= src[i] << bs;
    if (bs && k + 1 < dlen) dst[k + 1] |= src[i] >> (32 - bs);
  }
}

/* dst[0..n) = (x >> lo) truncated to n limbs, lo >= 0 */
static void shr_into(uint32_t *dst, int n, const uint32_t *x, int len, int lo) {
  int ws = lo >> 5, bs = lo & 31;
  for (int i = 0; i < n; i++) {
    int k = i + ws;
    uint32_t v = k < len ? x[k] >> bs : 0;
    if (bs && k + 1 < len) v |= x[k + 1] << (32 - bs);
    dst[i] = v;
  }
}

static uint32_t add_into(uint32_t *x, int len, const uint32_t *y, int ylen) {  /* x += y */
  uint64_t c = 0;
  for (int i = 0; i < len; i++) {
    c += (uint64_t)x[i] + (i < ylen ? y[i] : 0);
    x[i] = (uint32_t)c; c >>= 32;
  }
  return (uint32_t)c;
}

static uint32_t sub_into(uint32_t *x, int len, const uint32_t *y, int ylen) {  /* x -= y, returns borrow */
  int64_t c = 0;
  for (int i = 0; i < len; i++) {
    c += (int64_t)x[i] - (int64_t)(i < ylen ? y[i] : 0);
    x[i] = (uint32_t)c; c >>= 32;   /* arithmetic shift: 0 or -1 */
  }
  return c ? 1u : 0u;
}

static int cmp_n(const uint32_t *x, const uint32_t *y, int len) {
  for (int i = len - 1; i >= 0; i--)
    if (x[i] != y[i]) return x[i] > y[i] ? 1 : -1;
  return 0;
}

/* p[0..na+nb) = a * b (schoolbook, operand scanning) */
static void mul_full(uint32_t *p, const uint32_t *a, int na, const uint32_t *b, int nb) {
  memset(p, 0, sizeof(uint32_t) * (na + nb));
  for (int i = 0; i < na; i++) {
    uint64_t c = 0, ai = a[i];
    if (!ai) continue;
    for (int j = 0; j < nb; j++) {
      c += ai * b[j] + p[i + j];
      p[i + j] = (uint32_t)c; c >>= 32;
    }
    p[i + nb] = (uint32_t)c;
  }
}

/* Knuth algorithm D: q[0..m-nv+1) = u / v, r[0..nv) = u % v; v[nv-1] != 0, m >= nv */
static void divmod(uint32_t *q, uint32_t *r, const uint32_t *u, int m, const uint32_t *v, int nv) {
  if (nv == 1) {
    uint64_t rem = 0;
    for (int i = m - 1; i >= 0; i--) {
      uint64_t cur = (rem << 32) | u[i];
      q[i] = (uint32_t)(cur / v[0]); rem = cur % v[0];
    }
    r[0] = (uint32_t)rem;
    return;
  }
  int s = clz32(v[nv - 1]);
  uint32_t *vn = (uint32_t *)malloc(sizeof(uint32_t) * nv);
  uint32_t *un = (uint32_t *)malloc(sizeof(uint32_t) * (m + 1));
  for (int i = nv - 1; i > 0; i--) vn[i] = s ? (v[i] << s) | (v[i - 1] >> (32 - s)) : v[i];
  vn[0] = v[0] << s;
  un[m] = s ? u[m - 1] >> (32 - s) : 0;
  for (int i = m - 1; i > 0; i--) un[i] = s ? (u[i] << s) | (u[i - 1] >> (32 - s)) : u[i];
  un[0] = u[0] << s;
  const uint64_t B = 1ull << 32;
  for (int j = m - nv; j >= 0; j--) {
    uint64_t num = ((uint64_t)un[j + nv] << 32) | un[j + nv - 1];
    uint64_t qhat = num / vn[nv - 1], rhat = num % vn[nv - 1];
    while (qhat >= B || qhat * vn[nv - 2] > ((rhat << 32) | un[j + nv - 2])) {
      qhat--; rhat += vn[nv - 1];
      if (rhat >= B) break;
    }
    int64_t borrow = 0; uint64_t carry = 0;
    for (int i = 0; i < nv; i++) {
      uint64_t p = qhat * vn[i] + carry;
      carry = p >> 32;
      int64_t t = (int64_t)un[i + j] - (int64_t)(uint32_t)p + borrow;
      un[i + j] = (uint32_t)t; borrow = t >> 32;
    }
    int64_t t = (int64_t)un[j + nv] - (int64_t)carry + borrow;
    un[j + nv] = (uint32_t)t;
    if (t < 0) {            /* add back */
      qhat--;
      uint64_t c = 0;
      for (int i = 0; i < nv; i++) {
        c += (uint64_t)un[i + j] + vn[i];
        un[i + j] = (uint32_t)c; c >>= 32;
      }
      un[j + nv] += (uint32_t)c;
    }
    q[j] = (uint32_t)qhat;
  }
  for (int i = 0; i < nv; i++) r[i] = s ? (un[i] >> s) | (un[i + 1] << (32 - s)) : un[i];
  free(vn); free(un);
}

/* s[0..xl/2+1) = floor(sqrt(x)), returns 1 if x is not a perfect square */
static int isqrt(uint32_t *s, const uint32_t *x, int xl) {
  int L = bitlen(x, xl);
  int sl = xl / 2 + 2;
  memset(s, 0, sizeof(uint32_t) * sl);
  if (L == 0) return 0;
  /* initial upper bound from the top bits: T = x >> 2h, s0 = (floor(sqrt(T)) + 2) << h */
  int h = L > 52 ? (L - 51) / 2 : 0;
  uint32_t t2[2];
  shr_into(t2, 2, x, xl, 2 * h);
  double T = (double)(((uint64_t)t2[1] << 32) | t2[0]);
  uint64_t r0 = (uint64_t)sqrt(T) + 2;
  uint32_t r0l[2] = { (uint32_t)r0, (uint32_t)(r0 >> 32) };
  shl_into(s, sl, r0l, 2, h);
  uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * (xl + 2));
  uint32_t *r = (uint32_t *)malloc(sizeof(uint32_t) * (sl + 1));
  uint32_t *t = (uint32_t *)malloc(sizeof(uint32_t) * (xl + 2));
  for (;;) {     /* Newton from above: t = (s + x/s) / 2 until it stops decreasing */
    int sn = sl; while (sn > 1 && s[sn - 1] == 0) sn--;
    if (xl < sn) { memset(q, 0, sizeof(uint32_t) * (xl + 2)); }
    else divmod(q, r, x, xl, s, sn);
    int ql = xl >= sn ? xl - sn + 1 : 1;
    memset(t, 0, sizeof(uint32_t) * (xl + 2));
    memcpy(t, s, sizeof(uint32_t) * sl);
    add_into(t, xl + 2, q, ql);
    shr_into(t, xl + 1, t, xl + 2, 1);     /* in place: reads index k+1 >= writes index k */
    /* compare t with s over max(sl, xl+1) limbs */
    int len = xl + 1 > sl ? xl + 1 : sl;
    int c = 0;
    for (int i = len - 1; i >= 0; i--) {
      uint32_t tv = i < xl + 1 ? t[i] : 0, sv = i < sl ? s[i] : 0;
      if (tv != sv) { c = tv > sv ? 1 : -1; break; }
    }
    if (c >= 0) break;
    memcpy(s, t, sizeof(uint32_t) * sl);
  }
  /* remainder test */
  uint32_t *sq = (uint32_t *)malloc(sizeof(uint32_t) * 2 * sl);
  mul_full(sq, s, sl, s, sl);
  int inexact = 0;
  for (int i = 0; i < 2 * sl; i++) {
    uint32_t xv = i < xl ? x[i] : 0;
    if (xv != sq[i]) { inexact = 1; break; }
  }
  free(sq); free(q); free(r); free(t);
  return inexact;
}

/* ---- rounding (fpa_internal.h:62-88 restated on bits) --------------------- */

static int round_up(int mode, int sign, int lsb, int rbit, int sticky) {
  switch (mode) {
    case 0: return 0;                                 /* truncate */
    case 1: return !sign && (rbit || sticky);         /* toward +inf */
    case 2: return sign && (rbit || sticky);          /* toward -inf */
    case 3: return rbit && (sticky || lsb);           /* ties to even */
    case 4: return rbit;                              /* ties away from zero */
  }
  return 0;
}

/* Round X * 2^E0 (+ a positive amount below every bit of X when sticky_in) to n
 * limbs.  Writes the normalized mantissa to M, returns the exponent e so that the
 * rounded value is 0.M * 2^e. X must be nonzero. */
static int64_t round_pack(uint32_t n, int mode, int sign, const uint32_t *X, int xlen,
                          int64_t E0, int sticky_in, uint32_t *M) {
  int L = bitlen(X, xlen);
  int P = 32 * (int)n;
  int64_t e = E0 + L;
  int rbit = 0, sticky = sticky_in;
  if (L > P) {
    int lo = L - P;
    shr_into(M, n, X, xlen, lo);
    rbit = getbit(X, xlen, lo - 1);
    sticky |= any_below(X, xlen, lo - 1);
  } else {
    shl_into(M, n, X, xlen, P - L);
  }
  if (round_up(mode, sign, M[0] & 1, rbit, sticky)) {
    uint32_t one = 1;
    if (add_into(M, n, &one, 1)) {          /* 0.111..1 + ulp = 1.0 */
      memset(M, 0, sizeof(uint32_t) * n);
      M[n - 1] = 0x80000000u;
      e++;
    }
  }
  return e;
}

static uint32_t encode(int64_t e, int sign) { return (uint32_t)(2 * (BIAS + e) + sign); }

/* ---- operations ------------------------------------------------------------ */

/* fpa_warp_add_sub.h:41-125 (same-sign add), :127-282 (effective subtract),
 * dispatch :310-380.  Range limits: effective add -> +/-INF when BIAS+e > 0x7FFFFFFF
 * (:118-119), effective subtract -> +/-TINY when BIAS+e < 5 (:226-227, :272-273). */
static void op_addsub(int is_sub, uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
                      uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b) {
  uint32_t action = (is_sub ? sub_table : add_table)[classify(a_exp) * 9 + classify(b_exp)];
  switch (action) {
    case A_COPY_A: *r_exp = a_exp; memcpy(r_limbs, a, 4 * n); return;
    case A_COPY_B: *r_exp = b_exp; memcpy(r_limbs, b, 4 * n); return;
    case A_NEG_B:
      /* 0 - b = -b.  The reference's sub dispatcher (fpa_warp_add_sub.h:357-379) has no
       * case for this action and stores the action code (24) as the exponent word; the
       * oracle gives the value MPFR gives. */
      *r_exp = b_exp ^ 1u; memcpy(r_limbs, b, 4 * n); return;
    case A_ADD: case A_SUB: break;
    default: *r_exp = action; return;
  }
  int sa = a_exp & 1, sb = (b_exp & 1) ^ (is_sub ? 1 : 0);
  int64_t ea = (int64_t)(a_exp >> 1) - BIAS, eb = (int64_t)(b_exp >> 1) - BIAS;
  const uint32_t *big = a, *small = b;
  int sbig = sa, ssmall = sb;
  int64_t ebig = ea, esmall = eb;
  if (eb > ea || (eb == ea && cmp_n(b, a, n) > 0)) {
    big = b; small = a; sbig = sb; ssmall = sa; ebig = eb; esmall = ea;
  }
  int64_t d = ebig - esmall;
  int64_t cap = 32LL * n + 64;
  int dc = (int)(d > cap ? cap : d);
  int xl = (int)n + (dc >> 5) + 2;
  uint32_t *X = (uint32_t *)calloc(xl, sizeof(uint32_t));
  shl_into(X, xl, big, n, dc);
  int effective_sub = sbig != ssmall;
  if (effective_sub) sub_into(X, xl, small, n);
  else add_into(X, xl, small, n);
  if (bitlen(X, xl) == 0) { *r_exp = C_ZERO; free(X); return; }   /* exact cancellation */
  uint32_t *M = (uint32_t *)malloc(4 * n);
  int64_t e = round_pack(n, mode, sbig, X, xl, ebig - dc - 32LL * n, 0, M);
  if (!effective_sub && BIAS + e > 0x7FFFFFFFLL) *r_exp = C_POS_INF - sbig;
  else if (effective_sub && BIAS + e < 5) *r_exp = C_POS_TINY - sbig;
  else { *r_exp = encode(e, sbig); memcpy(r_limbs, M, 4 * n); }
  free(M); free(X);
}

/* fpa_warp_mul.h:41-139.  Range limits (:124-128): TINY when BIAS+e < 5, INF when
 * BIAS+e > 0x7FFFFFFF.  Rounding is exact; the reference's kernel reads the parity
 * bit before its one-bit normalisation shift (:115-121) and treats a 0x7FFF..F high
 * half as a carry into the next binade regardless of the next bit (:99-105), which
 * can differ from MPFR on exact ties and on those all-ones products. */
static void op_mul(uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
                   uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b) {
  uint32_t action = mul_table[classify(a_exp) * 9 + classify(b_exp)];
  if (action != A_MUL) { *r_exp = action; return; }
  int sign = (a_exp ^ b_exp) & 1;
  int64_t ea = (int64_t)(a_exp >> 1) - BIAS, eb = (int64_t)(b_exp >> 1) - BIAS;
  uint32_t *P = (uint32_t *)malloc(8 * n), *M = (uint32_t *)malloc(4 * n);
  mul_full(P, a, n, b, n);
  int64_t e = round_pack(n, mode, sign, P, 2 * n, ea + eb - 64LL * n, 0, M);
  if (BIAS + e < 5) *r_exp = C_POS_TINY - sign;
  else if (BIAS + e > 0x7FFFFFFFLL) *r_exp = C_POS_INF - sign;
  else { *r_exp = encode(e, sign); memcpy(r_limbs, M, 4 * n); }
  free(P); free(M);
}

/* fpa_warp_div.h:127-201.  Range limits (:189-193): TINY when BIAS+e < 10, INF when
 * BIAS+e >= 0x7FFFFFFF. */
static void op_div(uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
                   uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b) {
  uint32_t action = div_table[classify(a_exp) * 9 + classify(b_exp)];
  if (action != A_DIV) { *r_exp = action; return; }
  int sign = (a_exp ^ b_exp) & 1;
  int64_t ea = (int64_t)(a_exp >> 1) - BIAS, eb = (int64_t)(b_exp >> 1) - BIAS;
  /* Q = floor(A * 2^(32n+64) / B): 32n+64 or 32n+65 bits, so round bit and sticky
   * come from Q's low bits and the remainder. */
  uint32_t *U = (uint32_t *)calloc(2 * n + 2, 4);
  for (uint32_t i = 0; i < n; i++) U[n + 2 + i] = a[i];
  uint32_t *Q = (uint32_t *)calloc(n + 3, 4), *R = (uint32_t *)calloc(n, 4), *M = (uint32_t *)malloc(4 * n);
  divmod(Q, R, U, 2 * n + 2, b, n);
  int rem = bitlen(R, n) != 0;
  int64_t e = round_pack(n, mode, sign, Q, n + 3, ea - eb - 32LL * n - 64, rem, M);
  if (BIAS + e < 10) *r_exp = C_POS_TINY - sign;
  else if (BIAS + e >= 0x7FFFFFFFLL) *r_exp = C_POS_INF - sign;
  else { *r_exp = encode(e, sign); memcpy(r_limbs, M, 4 * n); }
  free(U); free(Q); free(R); free(M);
}

/* fpa_warp_sqrt.h:195-254: odd exponents are made even (:218-223); the result is
 * always a positive value in range.  The reference adds 1 instead of 2 to the
 * exponent word when the root rounds up to the next binade (:238-242); the oracle
 * gives the value MPFR gives. */
static void op_sqrt(uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
                    uint32_t a_exp, const uint32_t *a) {
  uint32_t action = sqrt_table[classify(a_exp)];
  if (action != A_SQRT) { *r_exp = action; return; }
  int64_t ea = (int64_t)(a_exp >> 1) - BIAS;
  int64_t t = ea - 32LL * n;                      /* value = A * 2^t */
  int k = 32 * (int)n + 128;
  if (((t - k) & 1) != 0) k++;
  int xl = (int)n + (k >> 5) + 1;
  uint32_t *X = (uint32_t *)calloc(xl, 4);
  shl_into(X, xl, a, n, k);
  int sl = xl / 2 + 2;
  uint32_t *S = (uint32_t *)calloc(sl, 4), *M = (uint32_t *)malloc(4 * n);
  int inexact = isqrt(S, X, xl);
  int64_t e = round_pack(n, mode, 0, S, sl, (t - k) / 2, inexact, M);
  *r_exp = encode(e, 0);
  memcpy(r_limbs, M, 4 * n);
  free(X); free(S); free(M);
}

/* Fused multiply-add r = RND(a*b + c) with one rounding.  The reference has no FMA; its
 * special values follow the existing tables: the class of the exact product is the mul
 * table's (fpa_warp_mul.h:1-12), then the add table (fpa_warp_add_sub.h:15-24) combines
 * it with c.  A product that is a value and c = 0 / tiny rounds like fpa_mul; the sum of
 * two values is exact before its single rounding, and a result outside the exponent range
 * becomes +-INF (BIAS+e > 0x7FFFFFFF) or +-TINY (BIAS+e < 5). */
static void op_fma(uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
                   uint32_t a_exp, const uint32_t *a, uint32_t b_exp, const uint32_t *b,
                   uint32_t c_exp, const uint32_t *c) {
  uint32_t pm = mul_table[classify(a_exp) * 9 + classify(b_exp)];
  int sp = (int)((a_exp ^ b_exp) & 1u);
  uint32_t pcls = pm == A_MUL ? (uint32_t)sp : pm;       /* class of the exact product */
  uint32_t action = add_table[pcls * 9 + classify(c_exp)];
  if (action == A_COPY_B) { *r_exp = c_exp; memcpy(r_limbs, c, 4 * n); return; }
  if (action != A_COPY_A && action != A_ADD && action != A_SUB) { *r_exp = action; return; }
  int64_t ea = (int64_t)(a_exp >> 1) - BIAS, eb = (int64_t)(b_exp >> 1) - BIAS;
  uint32_t *P = (uint32_t *)calloc(2 * n, 4), *M = (uint32_t *)malloc(4 * n);
  mul_full(P, a, n, b, n);
  int64_t lowP = ea + eb - 64LL * n;                     /* product = P * 2^lowP */
  if (action == A_COPY_A) {                              /* c is zero or tiny: rounded product */
    int64_t e = round_pack(n, mode, sp, P, 2 * n, lowP, 0, M);
    if (BIAS + e < 5) *r_exp = C_POS_TINY - sp;
    else if (BIAS + e > 0x7FFFFFFFLL) *r_exp = C_POS_INF - sp;
    else { *r_exp = encode(e, sp); memcpy(r_limbs, M, 4 * n); }
    free(P); free(M);
    return;
  }
  int sc = (int)(c_exp & 1u);
  int64_t ec = (int64_t)(c_exp >> 1) - BIAS, lowC = ec - 32LL * n;   /* c = C * 2^lowC */
  int64_t topP = lowP + bitlen(P, 2 * n), topC = ec;
  /* an operand entirely more than 64 bits below the other's lowest bit only matters as a
   * sticky / borrow: move it up to just below that 64-bit guard (exact for rounding) */
  if (topC < lowP - 64) { lowC = lowP - 64 - 32LL * n; topC = lowC + 32LL * n; }
  else if (topP < lowC - 64) { int64_t sh = (lowC - 64 - 64LL * n) - lowP; lowP += sh; topP += sh; }
  int64_t lo = lowP < lowC ? lowP : lowC, hi = topP > topC ? topP : topC;
  int xl = (int)((hi - lo) >> 5) + 2;
  uint32_t *X1 = (uint32_t *)calloc(xl, 4), *X2 = (uint32_t *)calloc(xl, 4);
  shl_into(X1, xl, P, 2 * n, (int)(lowP - lo));
  shl_into(X2, xl, c, n, (int)(lowC - lo));
  int sign;
  if (sp == sc) { add_into(X1, xl, X2, xl); sign = sp; }
  else {
    int cmp = cmp_n(X1, X2, xl);
    if (cmp == 0) { *r_exp = C_ZERO; free(P); free(M); free(X1); free(X2); return; }
    if (cmp > 0) { sub_into(X1, xl, X2, xl); sign = sp; }
    else { sub_into(X2, xl, X1, xl); memcpy(X1, X2, 4 * (size_t)xl); sign = sc; }
  }
  int64_t e = round_pack(n, mode, sign, X1, xl, lo, 0, M);
  if (BIAS + e > 0x7FFFFFFFLL) *r_exp = C_POS_INF - sign;
  else if (BIAS + e < 5) *r_exp = C_POS_TINY - sign;
  else { *r_exp = encode(e, sign); memcpy(r_limbs, M, 4 * n); }
  free(P); free(M); free(X1); free(X2);
}

int oracle_fma_batch(uint32_t n, int mode, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                     const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                     const uint32_t *b_limbs, const uint32_t *c_exps, const uint32_t *c_limbs) {
  if (n == 0 || n > 4096 || mode < 0 || mode > 4) return -1;
  for (uint32_t i = 0; i < count; i++)
    op_fma(n, mode, r_exps + i, r_limbs + (size_t)i * n, a_exps[i], a_limbs + (size_t)i * n, b_exps[i],
           b_limbs + (size_t)i * n, c_exps[i], c_limbs + (size_t)i * n);
  return 0;
}

int oracle_op(int op, uint32_t n, int mode, uint32_t *r_exp, uint32_t *r_limbs,
              uint32_t a_exp, const uint32_t *a_limbs, uint32_t b_exp, const uint32_t *b_limbs) {
  if (n == 0 || n > 4096 || mode < 0 || mode > 4) return -1;
  switch (op) {
    case ORACLE_ADD: op_addsub(0, n, mode, r_exp, r_limbs, a_exp, a_limbs, b_exp, b_limbs); return 0;
    case ORACLE_SUB: op_addsub(1, n, mode, r_exp, r_limbs, a_exp, a_limbs, b_exp, b_limbs); return 0;
    case ORACLE_MUL: op_mul(n, mode, r_exp, r_limbs, a_exp, a_limbs, b_exp, b_limbs); return 0;
    case ORACLE_DIV: op_div(n, mode, r_exp, r_limbs, a_exp, a_limbs, b_exp, b_limbs); return 0;
    case ORACLE_SQRT: op_sqrt(n, mode, r_exp, r_limbs, a_exp, a_limbs); return 0;
  }
  return -1;
}

/* ---- conversions, sign, compare, negation (the non-arithmetic fpa.h entry points) ----
 *
 * fpa_set_ui/si/float/double (fpa_warp_set.h:1-132, dispatch fpa_dispatch.h:8-86): the
 * value is stored exactly whenever it fits the precision, which is always the case at the
 * reference's precisions (>= 1024 bits).  The precision-32 numbers of this library hold
 * only 32 bits, so a wider integer or double mantissa is rounded to nearest, ties to even
 * (what mpfr_set_ui / mpfr_set_d give with MPFR_RNDN).  Zero (either sign) is the ZERO
 * class, every NaN (quiet or signalling, any payload) the NAN class, infinities the INF
 * classes (fpa_warp_set.h:89-96). */
static void put_int(uint32_t n, uint64_t mag, int sign, int64_t e0, uint32_t *r_exp, uint32_t *r_limbs) {
  if (mag == 0) { *r_exp = C_ZERO; return; }
  uint32_t X[2] = { (uint32_t)mag, (uint32_t)(mag >> 32) };
  uint32_t *M = (uint32_t *)calloc(n, 4);
  int64_t e = round_pack(n, 3, sign, X, 2, e0, 0, M);
  memcpy(r_limbs, M, 4 * (size_t)n);
  *r_exp = encode(e, sign);
  free(M);
}

int oracle_set_ui(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *vals) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) put_int(n, vals[i], 0, 0, r_exps + i, r_limbs + (size_t)i * n);
  return 0;
}

/* fpa_warp_set.h:34-41 (INT64_MIN has magnitude 2^63) */
int oracle_set_si(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const int64_t *vals) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) {
    const int neg = vals[i] < 0;
    const uint64_t mag = neg ? (uint64_t)0 - (uint64_t)vals[i] : (uint64_t)vals[i];
    put_int(n, mag, neg, 0, r_exps + i, r_limbs + (size_t)i * n);
  }
  return 0;
}

/* IEEE binary32 / binary64 from their bit patterns: (-1)^s * m * 2^q with integer m
 * (fpa_warp_set.h:74-132 uses frexp/ldexp for the same decomposition). */
static void put_ieee(uint32_t n, uint64_t bits, int is_double, uint32_t *r_exp, uint32_t *r_limbs) {
  const int mbits = is_double ? 52 : 23, ebits = is_double ? 11 : 8;
  const int sign = (int)((bits >> (mbits + ebits)) & 1u);
  const int ef = (int)((bits >> mbits) & ((1u << ebits) - 1u));
  uint64_t m = bits & ((1ull << mbits) - 1u);
  const int bias = (1 << (ebits - 1)) - 1;
  if (ef == (1 << ebits) - 1) { *r_exp = m ? C_NAN : (sign ? C_NEG_INF : C_POS_INF); return; }
  int64_t q;
  if (ef == 0) q = 1 - bias - mbits;
  else { m |= 1ull << mbits; q = ef - bias - mbits; }
  put_int(n, m, sign, q, r_exp, r_limbs);
}

int oracle_set_float(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *bits) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) put_ieee(n, bits[i], 0, r_exps + i, r_limbs + (size_t)i * n);
  return 0;
}

int oracle_set_double(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *bits) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) put_ieee(n, bits[i], 1, r_exps + i, r_limbs + (size_t)i * n);
  return 0;
}

/* fpa_set: change of precision with rounding in `mode` (fpa_warp_set.h:134-199 decides the
 * rounding but never stores the limbs; here the rounded value is stored).  Class operands
 * are copied; rounding up past the largest exponent gives +/-INF (the mul limit,
 * fpa_warp_mul.h:124-128). */
int oracle_set_prec(uint32_t nr, uint32_t nx, int mode, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                    const uint32_t *x_exps, const uint32_t *x_limbs) {
  if (nr == 0 || nr > 4096 || nx == 0 || nx > 4096 || mode < 0 || mode > 4) return -1;
  uint32_t *M = (uint32_t *)calloc(nr, 4);
  for (uint32_t i = 0; i < count; i++) {
    const uint32_t xe = x_exps[i];
    if (classify(xe) > C_NEG_VALUE) { r_exps[i] = xe; continue; }
    const int sign = (int)(xe & 1u);
    const int64_t ex = (int64_t)(xe >> 1) - BIAS;
    const int64_t e = round_pack(nr, mode, sign, x_limbs + (size_t)i * nx, (int)nx, ex - 32LL * nx, 0, M);
    if (BIAS + e > 0x7FFFFFFFLL) { r_exps[i] = C_POS_INF - sign; continue; }
    r_exps[i] = encode(e, sign);
    memcpy(r_limbs + (size_t)i * nr, M, 4 * (size_t)nr);
  }
  free(M);
  return 0;
}

/* fpa_threaded.h:1-11 (sgn) and :13-24 (cmp): class tables; a NaN operand (the tables'
 * error entry) gives 0, as in fpa_threaded.h:34-37.  CMP_V = compare the values. */
enum { CMP_V = 25, CMP_E = 26 };
static const int8_t sgn_table[9] = { +1, -1, 0, -1, +1, -1, +1, CMP_E, CMP_E };
static const int8_t cmp_table[81] = {
  CMP_V, +1,    +1,    +1,    +1,    +1,    -1,    CMP_E, CMP_E,
  -1,    CMP_V, -1,    -1,    -1,    +1,    -1,    CMP_E, CMP_E,
  -1,    +1,    0,     +1,    -1,    +1,    -1,    CMP_E, CMP_E,
  -1,    +1,    -1,    CMP_E, -1,    +1,    -1,    CMP_E, CMP_E,
  -1,    +1,    +1,    +1,    CMP_E, +1,    -1,    CMP_E, CMP_E,
  -1,    -1,    -1,    -1,    -1,    CMP_E, -1,    CMP_E, CMP_E,
  +1,    +1,    +1,    +1,    +1,    +1,    CMP_E, CMP_E, CMP_E,
  CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E,
  CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E, CMP_E,
};
/* fpa_warp_add_sub.h:3-13: the class of -x for each class of x */
static const uint8_t neg_table[9] = { 0, 1, C_ZERO, C_POS_TINY, C_NEG_TINY, C_POS_INF, C_NEG_INF, C_NAN, C_SNAN };

int oracle_sgn(uint32_t count, int32_t *r, const uint32_t *x_exps) {
  for (uint32_t i = 0; i < count; i++) {
    const int a = sgn_table[classify(x_exps[i])];
    r[i] = a == CMP_E ? 0 : a;
  }
  return 0;
}

/* values of one sign: the exponent words order them, then the limbs from the top
 * (fpa_threaded.h:52-89) */
int oracle_cmp(uint32_t n, uint32_t count, int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs,
               const uint32_t *b_exps, const uint32_t *b_limbs) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) {
    const uint32_t ae = a_exps[i], be = b_exps[i];
    const int act = cmp_table[classify(ae) * 9 + classify(be)];
    if (act == CMP_E) { r[i] = 0; continue; }
    if (act != CMP_V) { r[i] = act; continue; }
    const int sgn = (ae & 1u) ? -1 : 1;
    int c = ae > be ? 1 : (ae < be ? -1 : cmp_n(a_limbs + (size_t)i * n, b_limbs + (size_t)i * n, (int)n));
    r[i] = sgn * c;
  }
  return 0;
}

/* fpa_warp_neg (fpa_warp_add_sub.h:284-308): values flip the sign bit and copy the limbs */
int oracle_neg(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
               const uint32_t *a_limbs) {
  if (n == 0 || n > 4096) return -1;
  for (uint32_t i = 0; i < count; i++) {
    const uint32_t ae = a_exps[i];
    if (ae <= C_SNAN) { r_exps[i] = neg_table[ae]; continue; }
    r_exps[i] = ae ^ 1u;
    memcpy(r_limbs + (size_t)i * n, a_limbs + (size_t)i * n, 4 * (size_t)n);
  }
  return 0;
}

/* ---- threaded batch runners ------------------------------------------------ */

typedef struct {
  int kind;                       /* 0 = uniform batch, 1 = mixed */
  int op; uint32_t n; int mode;
  uint32_t begin, end;
  uint32_t *r_exps, *r_limbs;
  const uint32_t *a_exps, *a_limbs, *b_exps, *b_limbs;
  const uint8_t *ops, *modes; const uint16_t *ns;
  const uint64_t *r_off, *a_off, *b_off;
} job_t;

static void *worker(void *p) {
  job_t *j = (job_t *)p;
  for (uint32_t i = j->begin; i < j->end; i++) {
    if (j->kind == 0) {
      uint64_t o = (uint64_t)i * j->n;
      oracle_op(j->op, j->n, j->mode, j->r_exps + i, j->r_limbs + o,
                j->a_exps[i], j->a_limbs + o,
                j->b_exps ? j->b_exps[i] : 0, j->b_limbs ? j->b_limbs + o : j->a_limbs + o);
    } else {
      int op = j->ops[i];
      oracle_op(op, j->ns[i], j->modes[i], j->r_exps + i, j->r_limbs + j->r_off[i],
                j->a_exps[i], j->a_limbs + j->a_off[i],
                op == ORACLE_SQRT ? 0 : j->b_exps[i],
                op == ORACLE_SQRT ? j->a_limbs + j->a_off[i] : j->b_limbs + j->b_off[i]);
    }
  }
  return NULL;
}

static int run_jobs(job_t proto, uint32_t count, int threads) {
  if (threads < 1) threads = 1;
  if ((uint32_t)threads > count) threads = count ? (int)count : 1;
  job_t *jobs = (job_t *)malloc(sizeof(job_t) * threads);
  pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  for (int t = 0; t < threads; t++) {
    jobs[t] = proto;
    jobs[t].begin = (uint32_t)((uint64_t)count * t / threads);
    jobs[t].end = (uint32_t)((uint64_t)count * (t + 1) / threads);
  }
  if (threads == 1) worker(&jobs[0]);
  else {
    for (int t = 0; t < threads; t++) pthread_create(&tids[t], NULL, worker, &jobs[t]);
    for (int t = 0; t < threads; t++) pthread_join(tids[t], NULL);
  }
  free(jobs); free(tids);
  return 0;
}

int oracle_batch(int op, uint32_t n, int mode, uint32_t count,
                 uint32_t *r_exps, uint32_t *r_limbs,
                 const uint32_t *a_exps, const uint32_t *a_limbs,
                 const uint32_t *b_exps, const uint32_t *b_limbs, int threads) {
  if (op < 0 || op > 4 || n == 0 || n > 4096 || mode < 0 || mode > 4) return -1;
  job_t p; memset(&p, 0, sizeof p);
  p.kind = 0; p.op = op; p.n = n; p.mode = mode;
  p.r_exps = r_exps; p.r_limbs = r_limbs; p.a_exps = a_exps; p.a_limbs = a_limbs;
  p.b_exps = b_exps; p.b_limbs = b_limbs;
  return run_jobs(p, count, threads);
}

int oracle_mixed(uint32_t count, const uint8_t *ops, const uint16_t *limbs_n, const uint8_t *modes,
                 uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *r_off,
                 const uint32_t *a_exps, const uint32_t *a_limbs, const uint64_t *a_off,
                 const uint32_t *b_exps, const uint32_t *b_limbs, const uint64_t *b_off,
                 int threads) {
  job_t p; memset(&p, 0, sizeof p);
  p.kind = 1; p.ops = ops; p.ns = limbs_n; p.modes = modes;
  p.r_exps = r_exps; p.r_limbs = r_limbs; p.r_off = r_off;
  p.a_exps = a_exps; p.a_limbs = a_limbs; p.a_off = a_off;
  p.b_exps = b_exps; p.b_limbs = b_limbs; p.b_off = b_off;
  return run_jobs(p, count, threads);
}
