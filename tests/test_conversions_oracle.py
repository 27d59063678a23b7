"""CPU: the oracle's conversions (fpa_set_ui/si/float/double), precision change (fpa_set),
sgn, cmp and neg against MPFR 4.2.1 (committed fixtures and live) and against the
reference's class tables (fpa_threaded.h:1-24, fpa_warp_add_sub.h:3-13) for the classes
MPFR has no counterpart for (the TINY classes and SNAN)."""
import os

import numpy as np
import pytest

import conv_cases as CC
import gold
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "conv", "conv_mpfr.npz")
KINDS = ("ui", "si", "float", "double")


@pytest.fixture(scope="module")
def fx():
    z = np.load(FIXTURE)
    return {k: z[k] for k in z.files}


def _inputs(fx, kind):
    v = fx[f"set_{kind}_in"]
    return v


@pytest.mark.parametrize("n", (1, 2, 32, 128))
@pytest.mark.parametrize("kind", KINDS)
def test_set_values_match_mpfr_fixture(fx, kind, n):
    e, l = oracle.set_values(kind, n, _inputs(fx, kind))
    bad = mismatches(fx[f"set_{kind}_n{n}_exps"], fx[f"set_{kind}_n{n}_limbs"], e, l)
    assert bad.size == 0, (kind, n, bad[:5], _inputs(fx, kind)[bad[:5]])


def test_set_rounds_to_nearest_even_at_32_bits(fx):
    """At one limb a 64-bit integer or a double mantissa is rounded to nearest, ties to
    even (mpfr_set_ui / mpfr_set_d with MPFR_RNDN); the cases below are exact ties."""
    e, l = oracle.set_values("ui", 1, [0xFFFFFFFF80000000, 0xFFFFFFFE80000000, 0x9234567880000000,
                                       0x9234567980000000, 0x1234567880000000])
    assert list(l[:, 0]) == [0x80000000, 0xFFFFFFFE, 0x92345678, 0x9234567A, 0x91A2B3C4]
    assert list(W.decode_exp(e)[0]) == [65, 64, 64, 64, 61]


def test_set_classes_and_signs():
    nan_bits = np.array([0x7FC00000, 0xFFC00000, 0x7F800001, 0x7FA5A5A5], dtype=np.uint32).view(np.float32)
    e, _ = oracle.set_values("float", 4, nan_bits)
    assert (e == W.CLS_NAN).all()
    e, _ = oracle.set_values("double", 4, [0.0, -0.0, np.inf, -np.inf])
    assert list(e) == [W.CLS_ZERO, W.CLS_ZERO, W.CLS_POS_INF, W.CLS_NEG_INF]
    e, l = oracle.set_values("si", 2, [np.iinfo(np.int64).min, -1])
    assert list(W.decode_exp(e)[1]) == [1, 1]
    assert l[0, 1] == 0x80000000 and W.decode_exp(e)[0][0] == 64


@pytest.mark.parametrize("pair", [p for p in CC.PREC_PAIRS if max(p) <= 128], ids=str)
def test_set_prec_matches_mpfr_fixture(fx, pair):
    nx, nr = pair
    xe, xl = fx[f"prec_{nx}_{nr}_in_exps"], fx[f"prec_{nx}_{nr}_in_limbs"]
    for mode in range(5):
        e, l = oracle.set_prec(nr, nx, mode, xe, xl)
        bad = mismatches(fx[f"prec_{nx}_{nr}_exps"][mode], fx[f"prec_{nx}_{nr}_limbs"][mode], e, l)
        assert bad.size == 0, (pair, mode, bad[:5])


@pytest.mark.parametrize("n", (1, 2, 32, 128))
def test_sgn_cmp_neg_match_mpfr_fixture(fx, n):
    xe, xl = fx[f"num_n{n}_exps"], fx[f"num_n{n}_limbs"]
    assert (oracle.sgn(xe) == fx[f"sgn_n{n}"]).all()
    e, l = oracle.neg(n, xe, xl)
    assert mismatches(fx[f"neg_n{n}_exps"], fx[f"neg_n{n}_limbs"], e, l).size == 0
    r = oracle.cmp(n, fx[f"cmp_n{n}_a_exps"], fx[f"cmp_n{n}_a_limbs"], fx[f"cmp_n{n}_b_exps"],
                   fx[f"cmp_n{n}_b_limbs"])
    assert (r == fx[f"cmp_n{n}"]).all()


@pytest.mark.skipif(not gold.available(), reason="libmpfr not installed")
@pytest.mark.parametrize("n", CC.SIZES)
def test_conversions_match_mpfr_live(n):
    gens = {"ui": CC.uint_values(11 + n), "si": CC.int_values(12 + n), "float": CC.float_bits(13 + n).view(np.float32),
            "double": CC.double_bits(14 + n).view(np.float64)}
    for kind, v in gens.items():
        g = gold.set_values(kind, n, v)
        o = oracle.set_values(kind, n, v)
        bad = mismatches(g[0], g[1], o[0], o[1])
        assert bad.size == 0, (kind, n, v[bad[:5]])
    xe, xl = CC.numbers(70 + n, n, classes=CC.MPFR_CLASSES)
    assert (oracle.sgn(xe) == gold.sgn(n, xe, xl)).all()
    g, o = gold.neg(n, xe, xl), oracle.neg(n, xe, xl)
    assert mismatches(g[0], g[1], o[0], o[1]).size == 0
    ae, al, be, bl = CC.compare_pairs(80 + n, n, classes=CC.MPFR_CLASSES)
    assert (oracle.cmp(n, ae, al, be, bl) == gold.cmp(n, ae, al, be, bl)).all()


@pytest.mark.skipif(not gold.available(), reason="libmpfr not installed")
@pytest.mark.parametrize("pair", CC.PREC_PAIRS, ids=str)
def test_set_prec_matches_mpfr_live(pair):
    nx, nr = pair
    xe, xl = CC.prec_sources(90 + nx + nr, nx, nr)
    for mode in range(5):
        g = gold.set_prec(nr, nx, mode, xe, xl)
        o = oracle.set_prec(nr, nx, mode, xe, xl)
        bad = mismatches(g[0], g[1], o[0], o[1])
        assert bad.size == 0, (pair, mode, bad[:5])


def test_class_tables_beyond_mpfr():
    """TINY and SNAN entries of the reference's tables (fpa_threaded.h:1-24,
    fpa_warp_add_sub.h:3-13), which MPFR cannot check."""
    T, t, Z, NT = W.CLS_POS_TINY, W.CLS_NEG_TINY, W.CLS_ZERO, W.CLS_NAN
    assert list(oracle.sgn([T, t, W.CLS_SNAN, W.CLS_NAN])) == [1, -1, 0, 0]
    n = 2
    one = W.exp_word(1, 0)
    pairs = [(T, Z, 1), (t, Z, -1), (Z, T, -1), (Z, t, 1), (T, T, 0), (t, t, 0), (T, t, 1), (t, T, -1),
             (one, T, 1), (T, one, -1), (W.exp_word(1, 1), t, -1), (W.CLS_POS_INF, T, 1), (W.CLS_SNAN, one, 0),
             (W.CLS_NEG_INF, W.CLS_NEG_INF, 0), (NT, NT, 0)]
    ae = np.array([p[0] for p in pairs], np.uint32)
    be = np.array([p[1] for p in pairs], np.uint32)
    lim = np.zeros((len(pairs), n), np.uint32)
    lim[:, -1] = 0x80000000
    assert list(oracle.cmp(n, ae, lim, be, lim)) == [p[2] for p in pairs]
    e, _ = oracle.neg(n, CC.CLASSES, np.zeros((CC.CLASSES.size, n), np.uint32))
    assert list(e) == [Z, T, t, W.CLS_POS_INF, W.CLS_NEG_INF, W.CLS_NAN, W.CLS_SNAN]


def test_set_prec_overflow_and_classes():
    """Rounding up at the largest exponent gives +-INF; class operands are copied."""
    nx, nr = 2, 1
    xe = np.array([W.exp_word(0x7FFFFFFF - W.BIAS, 0), W.exp_word(0x7FFFFFFF - W.BIAS, 1)], np.uint32)
    xl = np.full((2, nx), 0xFFFFFFFF, np.uint32)
    e, _ = oracle.set_prec(nr, nx, 4, xe, xl)
    assert list(e) == [W.CLS_POS_INF, W.CLS_NEG_INF]
    e, _ = oracle.set_prec(nr, nx, 0, xe, xl)
    assert list(e) == list(xe)
    e, _ = oracle.set_prec(nr, nx, 3, CC.CLASSES, np.zeros((CC.CLASSES.size, nx), np.uint32))
    assert (e == CC.CLASSES).all()
