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
