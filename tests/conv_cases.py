"""Seeded inputs for the conversion, precision-change, sign, compare and negation tests.

Each generator mixes fixed edge values with seeded random ones:
- integers: 0, 1, the 32-bit boundaries, INT64_MIN / INT64_MAX / UINT64_MAX, 2^63, and
  values whose bits below the top 32 are exactly one half (ties, both parities), just above
  or just below it (what rounds at precision 32);
- floats and doubles: +-0, +-1, +-inf, NaNs (quiet, signalling, negative, with payloads),
  the smallest and largest subnormals and normals, ties at 32 bits, random bit patterns;
- numbers: random values, pairs with equal exponents or equal values, all-ones mantissas
  (rounding carries into a new binade) and the special classes.
"""
import numpy as np

from cubigfloat_gb300 import workloads as W

SIZES = (1, 2, 32, 128, 512)
CLASSES = np.array([W.CLS_ZERO, W.CLS_NEG_TINY, W.CLS_POS_TINY, W.CLS_NEG_INF, W.CLS_POS_INF, W.CLS_NAN,
                    W.CLS_SNAN], dtype=np.uint32)
# the classes MPFR has a counterpart for (zero, infinities, NaN)
MPFR_CLASSES = np.array([W.CLS_ZERO, W.CLS_NEG_INF, W.CLS_POS_INF, W.CLS_NAN], dtype=np.uint32)


def _u64(rng, count):
    """random 64-bit values of random bit length"""
    v = rng.integers(0, 1 << 63, size=count, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, size=count,
                                                                                              dtype=np.uint64)
    bits = rng.integers(1, 65, size=count)
    mask = np.array([(1 << int(b)) - 1 for b in bits], dtype=np.uint64)
    return v & mask


def uint_values(seed, count=96):
    fixed = [0, 1, 2, 3, 0xFFFFFFFF, 0x100000000, 0x100000001, 0x1FFFFFFFF, 0xFFFFFFFF80000000,
             0xFFFFFFFE80000000, 0x7FFFFFFF80000000, 0x8000000080000001, 0x800000007FFFFFFF, 1 << 63,
             (1 << 64) - 1, (1 << 63) - 1, 0x1234567880000000, 0x1234567980000000]
    rng = np.random.default_rng(seed)
    return np.concatenate([np.array(fixed, dtype=np.uint64), _u64(rng, count - len(fixed))])


def int_values(seed, count=96):
    u = uint_values(seed, count)
    i64 = u.view(np.int64).copy()
    rng = np.random.default_rng(seed + 1)
    flip = rng.integers(0, 2, size=count).astype(bool)
    flip[:18] = False
    i64[flip] = -np.abs(i64[flip])
    fixed = np.array([-1, -(1 << 32), -(1 << 32) - 1, -0x1234567880000000, -0x1234567980000000,
                      -(2 ** 63 - 1)], dtype=np.int64)
    i64[18:18 + fixed.size] = fixed
    i64[0] = np.iinfo(np.int64).min
    return i64


def float_bits(seed, count=96):
    fixed = [0x00000000, 0x80000000, 0x3F800000, 0xBF800000, 0x7F800000, 0xFF800000, 0x7FC00000, 0xFFC00000,
             0x7F800001, 0x7FA5A5A5, 0xFFFFFFFF, 0x00000001, 0x807FFFFF, 0x00800000, 0x7F7FFFFF, 0xFF7FFFFF,
             0x00400000, 0x3FFFFFFF]
    rng = np.random.default_rng(seed)
    r = rng.integers(0, 1 << 32, size=count - len(fixed), dtype=np.uint64).astype(np.uint32)
    r[:8] &= np.uint32(0x807FFFFF)                 # subnormals
    return np.concatenate([np.array(fixed, dtype=np.uint32), r])


def double_bits(seed, count=96):
    fixed = [0x0000000000000000, 0x8000000000000000, 0x3FF0000000000000, 0xBFF0000000000000, 0x7FF0000000000000,
             0xFFF0000000000000, 0x7FF8000000000000, 0xFFF8000000000000, 0x7FF0000000000001, 0x7FF4A5A5A5A5A5A5,
             0x0000000000000001, 0x800FFFFFFFFFFFFF, 0x0010000000000000, 0x7FEFFFFFFFFFFFFF, 0xFFEFFFFFFFFFFFFF,
             # 53-bit mantissas whose 21 bits below the top 32 are one half: ties (even, odd), above, below
             0x3FF0000000100000, 0x3FF0000000300000, 0x3FF0000000100001, 0x3FF00000000FFFFF, 0x3FFFFFFFFFF00000,
             0xC1DFFFFFFFF00000]
    rng = np.random.default_rng(seed)
    r = rng.integers(0, 1 << 63, size=count - len(fixed), dtype=np.uint64) * np.uint64(2)
    r[:8] &= np.uint64(0x800FFFFFFFFFFFFF)          # subnormals
    r[8:16] = (r[8:16] & np.uint64(0xFFFFFFFFFFE00000)) | np.uint64(0x100000)   # ties at 32 bits
    return np.concatenate([np.array(fixed, dtype=np.uint64), r])


def numbers(seed, n, count=64, classes=CLASSES):
    """Values (random, all-ones, one-bit) followed by one number of each class in `classes`."""
    rng = np.random.default_rng(seed)
    e, l = W.uniform(rng, count, n, -300, 300)
    l[:4] = 0xFFFFFFFF
    l[4:8] = 0
    l[4:8, n - 1] = 0x80000000
    k = classes.size
    e = np.concatenate([e, classes])
    l = np.concatenate([l, np.zeros((k, n), dtype=np.uint32)])
    return e, l


def compare_pairs(seed, n, count=96, classes=CLASSES):
    """Pairs (a, b): random, equal values, opposite signs of one magnitude, equal exponent
    words with limbs differing in one place, plus every (class or value) x (class or value)."""
    rng = np.random.default_rng(seed)
    ae, al = W.uniform(rng, count, n, -20, 20)
    be, bl = W.uniform(rng, count, n, -20, 20)
    q = count // 4
    be[:q], bl[:q] = ae[:q], al[:q]                              # equal
    be[q:2 * q], bl[q:2 * q] = ae[q:2 * q] ^ np.uint32(1), al[q:2 * q]   # opposite sign
    be[2 * q:3 * q], bl[2 * q:3 * q] = ae[2 * q:3 * q], al[2 * q:3 * q].copy()
    pos = rng.integers(0, n, size=q)
    bl[np.arange(2 * q, 3 * q), pos] ^= rng.integers(1, 1 << 32, size=q, dtype=np.uint64).astype(np.uint32)
    bl[:, n - 1] |= np.uint32(0x80000000)
    ve = np.array([W.exp_word(1, 0), W.exp_word(1, 1)], dtype=np.uint32)
    es = np.concatenate([ve, classes])
    gi, gj = np.meshgrid(np.arange(es.size), np.arange(es.size), indexing="ij")
    ce, de = es[gi.ravel()], es[gj.ravel()]
    cl = np.zeros((ce.size, n), dtype=np.uint32)
    cl[:, n - 1] = 0xC0000000
    return (np.concatenate([ae, ce]), np.concatenate([al, cl]), np.concatenate([be, de]),
            np.concatenate([bl, cl.copy()]))


PREC_PAIRS = ((1, 2), (2, 1), (32, 1), (1, 32), (33, 32), (4, 3), (128, 32), (32, 128), (512, 128), (128, 512),
              (512, 1), (3, 3))


def prec_sources(seed, nx, nr, count=64):
    """Numbers of nx limbs to be rounded to nr: random, all-ones (carry into a new binade),
    dropped part exactly one half (ties) or one half +- one unit."""
    rng = np.random.default_rng(seed)
    e, l = W.uniform(rng, count, nx, -300, 300)
    if nr < nx:
        d = nx - nr                                        # dropped limbs
        l[:4] = 0xFFFFFFFF
        for i, (lo, top) in enumerate(((0, 0x80000000), (0, 0x80000000), (1, 0x80000000), (0xFFFFFFFF, 0x7FFFFFFF))):
            r = 4 + i
            l[r, :d] = lo
            l[r, d - 1] = top
        l[5, d] ^= np.uint32(1)                           # the other parity of the tie
    return e, l
