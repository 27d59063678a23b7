/*
 * mpfr_gold.c -- MPFR gold values for the fpa encoding (test fixture generator).
 *
 * The reference validates its kernels against MPFR (tests.c:423-485), converting
 * between its limb encoding and mpfr_t as in tests.c:114-159.  This file does the
 * same conversion with mpfr_set_z_2exp / mpfr_get_z_2exp.  MPFR and GMP headers are
 * not installed in this image, so the few entry points used are declared here with
 * the layouts of MPFR 4.x / GMP 6.x on LP64 Linux.
 *
 * Used only to generate and check the committed golden fixtures under tests/golden/.
 */
#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;
typedef struct { mpfr_prec_t prec; mpfr_sign_t sign; mpfr_exp_t exp; void *d; } mpfr_s;
typedef struct { int alloc; int size; void *d; } mpz_s;
enum { RNDN = 0, RNDZ = 1, RNDU = 2, RNDD = 3, RNDA = 4 };

void mpfr_init2(mpfr_s *, mpfr_prec_t);
void mpfr_clear(mpfr_s *);
void mpfr_set_prec(mpfr_s *, mpfr_prec_t);
int mpfr_set_z_2exp(mpfr_s *, const mpz_s *, mpfr_exp_t, int);
mpfr_exp_t mpfr_get_z_2exp(mpz_s *, const mpfr_s *);
int mpfr_add(mpfr_s *, const mpfr_s *, const mpfr_s *, int);
int mpfr_sub(mpfr_s *, const mpfr_s *, const mpfr_s *, int);
int mpfr_mul(mpfr_s *, const mpfr_s *, const mpfr_s *, int);
int mpfr_div(mpfr_s *, const mpfr_s *, const mpfr_s *, int);
int mpfr_sqrt(mpfr_s *, const mpfr_s *, int);
int mpfr_fma(mpfr_s *, const mpfr_s *, const mpfr_s *, const mpfr_s *, int);
int mpfr_prec_round(mpfr_s *, mpfr_prec_t, int);
int mpfr_zero_p(const mpfr_s *);
int mpfr_nan_p(const mpfr_s *);
int mpfr_inf_p(const mpfr_s *);
int mpfr_set_ui(mpfr_s *, unsigned long, int);
int mpfr_set_si(mpfr_s *, long, int);
int mpfr_set_d(mpfr_s *, double, int);
int mpfr_set_flt(mpfr_s *, float, int);
int mpfr_set(mpfr_s *, const mpfr_s *, int);
int mpfr_sgn(const mpfr_s *);
int mpfr_cmp(const mpfr_s *, const mpfr_s *);
int mpfr_neg(mpfr_s *, const mpfr_s *, int);
int mpfr_signbit(const mpfr_s *);
void mpfr_set_nan(mpfr_s *);
void mpfr_set_inf(mpfr_s *, int);
void mpfr_set_zero(mpfr_s *, int);
const char *mpfr_get_version(void);
void __gmpz_init(mpz_s *);
void __gmpz_clear(mpz_s *);
void __gmpz_import(mpz_s *, size_t, int, size_t, int, size_t, const void *);
void *__gmpz_export(void *, size_t *, int, size_t, int, size_t, const mpz_s *);

#define BIAS 0x3FFFFFF3LL

const char *gold_version(void) { return mpfr_get_version(); }

/* fpa value -> mpfr (tests.c:114-134 convention: value = M * 2^(e - 32n)) */
static void to_mpfr(mpfr_s *x, uint32_t exp, const uint32_t *limbs, uint32_t n) {
  mpz_s z;
  __gmpz_init(&z);
  __gmpz_import(&z, n, -1, 4, 0, 0, limbs);
  if (exp & 1) z.size = -z.size;
  mpfr_set_z_2exp(x, &z, (mpfr_exp_t)((int64_t)(exp >> 1) - BIAS - 32LL * n), RNDZ);
  __gmpz_clear(&z);
}

/* mpfr -> fpa value (tests.c:136-159).  Returns 0 on success, -1 when the value is
 * not a finite number. */
static int from_mpfr(uint32_t *exp, uint32_t *limbs, uint32_t n, const mpfr_s *x) {
  if (mpfr_nan_p(x) || mpfr_inf_p(x)) return -1;
  if (mpfr_zero_p(x)) { *exp = 2; return 0; }
  mpz_s z;
  __gmpz_init(&z);
  mpfr_exp_t e2 = mpfr_get_z_2exp(&z, x);
  int sign = z.size < 0;
  if (sign) z.size = -z.size;
  size_t words = 0;
  uint32_t *tmp = (uint32_t *)calloc(n + 2, 4);
  __gmpz_export(tmp, &words, -1, 4, 0, 0, &z);
  /* significand of a precision-32n mpfr_t is exactly 32n bits */
  memcpy(limbs, tmp, 4 * n);
  free(tmp);
  __gmpz_clear(&z);
  *exp = (uint32_t)(2 * (BIAS + (int64_t)e2 + 32LL * n) + sign);
  return words == n ? 0 : -2;
}

static int apply(int op, mpfr_s *r, const mpfr_s *a, const mpfr_s *b, const mpfr_s *c, int rnd) {
  switch (op) {
    case 5: return mpfr_fma(r, a, b, c, rnd);
    case 0: return mpfr_add(r, a, b, rnd);
    case 1: return mpfr_sub(r, a, b, rnd);
    case 2: return mpfr_mul(r, a, b, rnd);
    case 3: return mpfr_div(r, a, b, rnd);
    case 4: return mpfr_sqrt(r, a, rnd);
  }
  return 0;
}

/* op: 0 add, 1 sub, 2 mul, 3 div, 4 sqrt, 5 fma (a*b + c).  mode: fpa_rounding_mode
 * (fpa.h:8-10); ties-away is computed as a (p+1)-bit truncation followed by rounding away
 * from zero when the extra bit is set. Inputs must be finite nonzero values. */
int gold_batch3(int op, uint32_t n, int mode, uint32_t count,
                uint32_t *r_exps, uint32_t *r_limbs,
                const uint32_t *a_exps, const uint32_t *a_limbs,
                const uint32_t *b_exps, const uint32_t *b_limbs,
                const uint32_t *c_exps, const uint32_t *c_limbs) {
  static const int map[4] = { RNDZ, RNDU, RNDD, RNDN };
  mpfr_s a, b, c, r;
  mpfr_prec_t p = 32L * n;
  mpfr_init2(&a, p); mpfr_init2(&b, p); mpfr_init2(&c, p); mpfr_init2(&r, p);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    to_mpfr(&a, a_exps[i], a_limbs + (size_t)i * n, n);
    if (op != 4) to_mpfr(&b, b_exps[i], b_limbs + (size_t)i * n, n);
    if (op == 5) to_mpfr(&c, c_exps[i], c_limbs + (size_t)i * n, n);
    if (mode == 4) {
      mpfr_set_prec(&r, p + 1);
      apply(op, &r, &a, &b, &c, RNDZ);
      mpz_s z; __gmpz_init(&z);
      if (!mpfr_zero_p(&r) && !mpfr_nan_p(&r) && !mpfr_inf_p(&r)) {
        mpfr_get_z_2exp(&z, &r);
        uint32_t low = 0; size_t w = 0;
        uint32_t *tmp = (uint32_t *)calloc(n + 3, 4);
        int neg = z.size < 0; if (neg) z.size = -z.size;
        __gmpz_export(tmp, &w, -1, 4, 0, 0, &z);
        low = tmp[0] & 1u;
        free(tmp);
        mpfr_prec_round(&r, p, low ? RNDA : RNDZ);
      } else {
        mpfr_prec_round(&r, p, RNDZ);
      }
      __gmpz_clear(&z);
    } else {
      mpfr_set_prec(&r, p);
      apply(op, &r, &a, &b, &c, map[mode]);
    }
    if (from_mpfr(r_exps + i, r_limbs + (size_t)i * n, n, &r) != 0) bad++;
  }
  mpfr_clear(&a); mpfr_clear(&b); mpfr_clear(&c); mpfr_clear(&r);
  return bad;
}

int gold_batch(int op, uint32_t n, int mode, uint32_t count,
               uint32_t *r_exps, uint32_t *r_limbs,
               const uint32_t *a_exps, const uint32_t *a_limbs,
               const uint32_t *b_exps, const uint32_t *b_limbs) {
  return gold_batch3(op, n, mode, count, r_exps, r_limbs, a_exps, a_limbs, b_exps, b_limbs, NULL, NULL);
}


/* ---- conversions, precision change, sign, compare, negation ------------------------ */

/* like from_mpfr, with MPFR's special values mapped to the fpa classes: NaN -> NAN (7),
 * -inf / +inf -> NEG_INF (5) / POS_INF (6), zero of either sign -> ZERO (2) */
static int from_mpfr_any(uint32_t *exp, uint32_t *limbs, uint32_t n, const mpfr_s *x) {
  if (mpfr_nan_p(x)) { *exp = 7; return 0; }
  if (mpfr_inf_p(x)) { *exp = mpfr_signbit(x) ? 5 : 6; return 0; }
  return from_mpfr(exp, limbs, n, x);
}

/* fpa number -> mpfr, with the classes MPFR can represent (ZERO, INF, NAN); returns -1 for
 * the TINY classes and SNAN, which have no MPFR counterpart */
static int to_mpfr_any(mpfr_s *x, uint32_t exp, const uint32_t *limbs, uint32_t n) {
  if (exp > 8) { to_mpfr(x, exp, limbs, n); return 0; }
  switch (exp) {
    case 2: mpfr_set_zero(x, 1); return 0;
    case 5: mpfr_set_inf(x, -1); return 0;
    case 6: mpfr_set_inf(x, 1); return 0;
    case 7: mpfr_set_nan(x); return 0;
  }
  return -1;
}

/* kind: 0 = mpfr_set_ui (uint64), 1 = mpfr_set_si (int64), 2 = mpfr_set_flt (float bits),
 * 3 = mpfr_set_d (double bits); precision 32n, round to nearest (ties to even). */
int gold_set(int kind, uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const void *vals) {
  mpfr_s r;
  mpfr_init2(&r, 32L * n);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    switch (kind) {
      case 0: mpfr_set_ui(&r, (unsigned long)((const uint64_t *)vals)[i], RNDN); break;
      case 1: mpfr_set_si(&r, (long)((const int64_t *)vals)[i], RNDN); break;
      case 2: mpfr_set_flt(&r, ((const float *)vals)[i], RNDN); break;
      default: mpfr_set_d(&r, ((const double *)vals)[i], RNDN); break;
    }
    if (from_mpfr_any(r_exps + i, r_limbs + (size_t)i * n, n, &r) != 0) bad++;
  }
  mpfr_clear(&r);
  return bad;
}

/* mpfr_set from precision 32nx to 32nr in `mode` (fpa_rounding_mode; ties-away as in
 * gold_batch3).  Inputs must be values. */
int gold_set_prec(uint32_t nr, uint32_t nx, int mode, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                  const uint32_t *x_exps, const uint32_t *x_limbs) {
  static const int map[4] = { RNDZ, RNDU, RNDD, RNDN };
  mpfr_s x, r;
  const mpfr_prec_t p = 32L * nr;
  mpfr_init2(&x, 32L * nx); mpfr_init2(&r, p);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    to_mpfr(&x, x_exps[i], x_limbs + (size_t)i * nx, nx);
    if (mode == 4) {
      mpfr_set_prec(&r, p + 1);
      mpfr_set(&r, &x, RNDZ);
      mpz_s z; __gmpz_init(&z);
      mpfr_get_z_2exp(&z, &r);
      int neg = z.size < 0; if (neg) z.size = -z.size;
      uint32_t *tmp = (uint32_t *)calloc(nr + 3, 4); size_t w = 0;
      __gmpz_export(tmp, &w, -1, 4, 0, 0, &z);
      const uint32_t low = tmp[0] & 1u;
      free(tmp);
      __gmpz_clear(&z);
      mpfr_prec_round(&r, p, low ? RNDA : RNDZ);
    } else {
      mpfr_set_prec(&r, p);
      mpfr_set(&r, &x, map[mode]);
    }
    if (from_mpfr_any(r_exps + i, r_limbs + (size_t)i * nr, nr, &r) != 0) bad++;
  }
  mpfr_clear(&x); mpfr_clear(&r);
  return bad;
}

/* mpfr_sgn, mpfr_cmp (NaN -> 0) and mpfr_neg on fpa numbers that are values or the
 * ZERO / INF / NAN classes; returns the number of inputs MPFR cannot represent. */
int gold_sgn(uint32_t n, uint32_t count, int32_t *r, const uint32_t *x_exps, const uint32_t *x_limbs) {
  mpfr_s x;
  mpfr_init2(&x, 32L * n);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    if (to_mpfr_any(&x, x_exps[i], x_limbs + (size_t)i * n, n) != 0) { bad++; continue; }
    r[i] = mpfr_nan_p(&x) ? 0 : mpfr_sgn(&x);
    r[i] = r[i] > 0 ? 1 : (r[i] < 0 ? -1 : 0);
  }
  mpfr_clear(&x);
  return bad;
}

int gold_cmp(uint32_t n, uint32_t count, int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs,
             const uint32_t *b_exps, const uint32_t *b_limbs) {
  mpfr_s a, b;
  mpfr_init2(&a, 32L * n); mpfr_init2(&b, 32L * n);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    if (to_mpfr_any(&a, a_exps[i], a_limbs + (size_t)i * n, n) != 0 ||
        to_mpfr_any(&b, b_exps[i], b_limbs + (size_t)i * n, n) != 0) { bad++; continue; }
    const int c = mpfr_cmp(&a, &b);
    r[i] = c > 0 ? 1 : (c < 0 ? -1 : 0);
  }
  mpfr_clear(&a); mpfr_clear(&b);
  return bad;
}

int gold_neg(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
             const uint32_t *a_limbs) {
  mpfr_s a, r;
  mpfr_init2(&a, 32L * n); mpfr_init2(&r, 32L * n);
  int bad = 0;
  for (uint32_t i = 0; i < count; i++) {
    if (to_mpfr_any(&a, a_exps[i], a_limbs + (size_t)i * n, n) != 0) { bad++; continue; }
    mpfr_neg(&r, &a, RNDN);
    if (from_mpfr_any(r_exps + i, r_limbs + (size_t)i * n, n, &r) != 0) bad++;
  }
  mpfr_clear(&a); mpfr_clear(&r);
  return bad;
}
