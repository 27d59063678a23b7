"""CPU: the oracle against MPFR (golden fixtures and live) and the reference's special-value
semantics."""
import numpy as np
import pytest

import gold
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import OPS, describe, golden_files, load_golden, mismatches


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1])
def test_oracle_matches_golden(path):
    z = load_golden(path)
    op, n = int(z["op"]), int(z["n"])
    for mode in range(5):
        e, l = oracle.run(op, n, mode, z["a_exps"], z["a_limbs"], z["b_exps"], z["b_limbs"])
        bad = mismatches(z["r_exps"][mode], z["r_limbs"][mode], e, l)
        assert bad.size == 0, describe(bad[0], z["a_exps"], z["a_limbs"], z["b_exps"], z["b_limbs"],
                                       z["r_exps"][mode], z["r_limbs"][mode], e, l)


def test_golden_inventory():
    files = golden_files()
    assert len(files) == 35
    for op in OPS:
        assert any(f"/{op}_n128.npz" in f for f in files)


@pytest.mark.skipif(not gold.available(), reason="libmpfr not installed")
@pytest.mark.parametrize("n", [2, 5, 32, 100])
@pytest.mark.parametrize("op", range(5))
def test_oracle_matches_mpfr_live(op, n):
    rng = np.random.default_rng(7 * n + op)
    ae, al = W.uniform(rng, 64, n, -300, 300, signs=(op != 4))
    be, bl = W.uniform(rng, 64, n, -300, 300)
    if op != 4:   # overlapping exponents stress cancellation
        ae[:16] = be[:16] ^ np.uint32(rng.integers(0, 2))
    for mode in range(5):
        g = gold.run(op, n, mode, ae, al, be, bl)
        o = oracle.run(op, n, mode, ae, al, be, bl)
        bad = mismatches(g[0], g[1], o[0], o[1])
        assert bad.size == 0, describe(bad[0], ae, al, be, bl, g[0], g[1], o[0], o[1])


def _one(op, n, mode, a, b=None):
    ae, al = a
    be, bl = b if b is not None else (ae, al)
    e, l = oracle.run(op, n, mode, np.array([ae], np.uint32), al[None, :], np.array([be], np.uint32), bl[None, :])
    return int(e[0]), l[0]


def test_special_tables():
    n = 4
    exps, limbs = W.specials(n)
    one, neg_one, zero = (exps[0], limbs[0]), (exps[1], limbs[1]), (W.CLS_ZERO, limbs[4])
    pinf, ninf, nan = (W.CLS_POS_INF, limbs[4]), (W.CLS_NEG_INF, limbs[4]), (W.CLS_NAN, limbs[4])
    ptiny, ntiny = (W.CLS_POS_TINY, limbs[4]), (W.CLS_NEG_TINY, limbs[4])
    # fpa_warp_add_sub.h:15-26
    assert _one(0, n, 3, pinf, ninf)[0] == W.CLS_NAN
    assert _one(0, n, 3, one, zero)[0] == one[0]
    assert _one(0, n, 3, ptiny, ntiny)[0] == W.CLS_NAN
    # fpa_warp_add_sub.h:28-39, including its -tiny - (+tiny) entry
    assert _one(1, n, 3, ntiny, ptiny)[0] == W.CLS_NEG_INF
    # sub(0, b) = -b (the reference leaves this action unhandled)
    e, l = _one(1, n, 3, zero, one)
    assert e == neg_one[0] and (l == one[1]).all()
    # fpa_warp_mul.h:1-12
    assert _one(2, n, 3, zero, pinf)[0] == W.CLS_NAN
    assert _one(2, n, 3, neg_one, ptiny)[0] == W.CLS_NEG_TINY
    # fpa_warp_div.h:1-12
    assert _one(3, n, 3, one, zero)[0] == W.CLS_NAN
    assert _one(3, n, 3, one, pinf)[0] == W.CLS_POS_TINY
    assert _one(3, n, 3, zero, one)[0] == W.CLS_ZERO
    # fpa_warp_sqrt.h:1-11
    assert _one(4, n, 3, neg_one)[0] == W.CLS_NAN
    assert _one(4, n, 3, ptiny)[0] == W.CLS_POS_TINY
    assert _one(4, n, 3, nan)[0] == W.CLS_NAN


def test_exact_cancellation_is_zero():
    n = 8
    rng = np.random.default_rng(3)
    ae, al = W.uniform(rng, 4, n, -10, 10)
    for mode in range(5):
        e, _ = oracle.run(1, n, mode, ae, al, ae, al)
        assert (e == W.CLS_ZERO).all()


def test_range_limits():
    """Exponent range limits of the reference kernels (fpa_warp_mul.h:124-128,
    fpa_warp_div.h:189-193, fpa_warp_add_sub.h:118-119)."""
    n = 2
    m = np.zeros((1, n), np.uint32); m[0, -1] = 0x80000000
    big = np.array([W.exp_word(0x7FFFFFFF - W.BIAS, 0)], np.uint32)     # largest exponent field
    small = np.array([W.exp_word(5 - W.BIAS, 0)], np.uint32)            # smallest value exponent
    assert oracle.run(2, n, 3, big, m, big, m)[0][0] == W.CLS_POS_INF
    assert oracle.run(2, n, 3, small, m, small, m)[0][0] == W.CLS_POS_TINY
    assert oracle.run(0, n, 3, big, m, big, m)[0][0] == W.CLS_POS_INF
    assert oracle.run(3, n, 3, small, m, big, m)[0][0] == W.CLS_POS_TINY


def test_threaded_batch_equals_serial():
    n = 16
    rng = np.random.default_rng(11)
    ae, al = W.uniform(rng, 200, n, -50, 50)
    be, bl = W.uniform(rng, 200, n, -50, 50)
    for op in range(5):
        s = oracle.run(op, n, 3, ae & ~np.uint32(op == 4), al, be, bl, threads=1)
        t = oracle.run(op, n, 3, ae & ~np.uint32(op == 4), al, be, bl, threads=4)
        assert (s[0] == t[0]).all() and (s[1] == t[1]).all()
