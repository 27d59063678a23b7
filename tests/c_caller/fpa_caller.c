/*
 * fpa_caller.c -- a plain C caller of the drop-in fpa.h API, built by the tests with
 *   gcc fpa_caller.c -I include -L cubigfloat_gb300/_build -lfpa_gb300
 * and no CUDA headers.  It follows the flow of the reference's own test driver
 * (fpa_test.c:283-306): fpa_init -> fpa_copy_array_to_device -> fpa_add / sub / mul / div /
 * sqrt -> fpa_copy_array_to_host -> fpa_clear.
 *
 *   fpa_caller IN OUT
 * IN : little-endian uint32 words op (0 add, 1 sub, 2 mul, 3 div, 4 sqrt), count,
 *      precision, mode, then a's exponent words and limbs, then b's (absent for sqrt)
 * OUT: the result's exponent words, then its limbs
 * Exit status: 0, or the first fpa_result that was not fpa_success (10 + code), or 2 for
 * a file error.
 */
#include <stdio.h>
#include <stdlib.h>
#include "fpa.h"

static int read_words(FILE *f, uint32_t *p, size_t n) { return fread(p, 4, n, f) == n; }

#define CHECK(call)                                                                  \
  do {                                                                               \
    fpa_result rc_ = (call);                                                         \
    if (rc_ != fpa_success) { fprintf(stderr, "%s -> %d\n", #call, (int)rc_); return 10 + (int)rc_; } \
  } while (0)

int main(int argc, char **argv) {
  uint32_t hdr[4], op, count, precision, n;
  fpa_rounding_mode mode;
  FILE *in, *out;
  uint32_t *a_exps, *a_limbs, *b_exps = NULL, *b_limbs = NULL, *r_exps, *r_limbs;
  fpa_t r, a, b;

  if (argc != 3 || !(in = fopen(argv[1], "rb"))) return 2;
  if (!read_words(in, hdr, 4)) return 2;
  op = hdr[0]; count = hdr[1]; precision = hdr[2]; mode = (fpa_rounding_mode)hdr[3];
  n = precision / 32;
  a_exps = (uint32_t *)malloc(4 * (size_t)count);
  a_limbs = (uint32_t *)malloc(4 * (size_t)count * n);
  r_exps = (uint32_t *)calloc(count, 4);
  r_limbs = (uint32_t *)calloc((size_t)count * n, 4);
  if (!read_words(in, a_exps, count) || !read_words(in, a_limbs, (size_t)count * n)) return 2;
  if (op != 4) {
    b_exps = (uint32_t *)malloc(4 * (size_t)count);
    b_limbs = (uint32_t *)malloc(4 * (size_t)count * n);
    if (!read_words(in, b_exps, count) || !read_words(in, b_limbs, (size_t)count * n)) return 2;
  }
  fclose(in);

  CHECK(fpa_init(r, count, precision));
  CHECK(fpa_init(a, count, precision));
  CHECK(fpa_init(b, count, precision));
  CHECK(fpa_copy_array_to_device(a, a_exps, a_limbs));
  if (op != 4) CHECK(fpa_copy_array_to_device(b, b_exps, b_limbs));
  switch (op) {
    case 0: CHECK(fpa_add(r, a, b, mode)); break;
    case 1: CHECK(fpa_sub(r, a, b, mode)); break;
    case 2: CHECK(fpa_mul(r, a, b, mode)); break;
    case 3: CHECK(fpa_div(r, a, b, mode)); break;
    case 4: CHECK(fpa_sqrt(r, a, mode)); break;
    default: return 2;
  }
  CHECK(fpa_copy_array_to_host(r, r_exps, r_limbs));
  CHECK(fpa_clear(r));
  CHECK(fpa_clear(a));
  CHECK(fpa_clear(b));

  if (!(out = fopen(argv[2], "wb"))) return 2;
  if (fwrite(r_exps, 4, count, out) != count || fwrite(r_limbs, 4, (size_t)count * n, out) != (size_t)count * n)
    return 2;
  fclose(out);
  free(a_exps); free(a_limbs); free(b_exps); free(b_limbs); free(r_exps); free(r_limbs);
  return 0;
}
