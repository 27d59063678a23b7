"""One-thread-per-operation row kernels (configuration 16) for 8, 16 and 32 limbs: mul
bit-exact against the oracle in every rounding mode, on random operands, near-halfway
products, all-ones mantissas (rounding into the next binade), products at the TINY / INF
limits of the exponent range and the special classes; and the lane-group fallback of
configuration 16 at other sizes."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import describe, mismatches

pytestmark = pytest.mark.gpu

BIAS = W.BIAS


def mul_cases(rng, n):
    ae, al = W.uniform(rng, 300, n, -300, 300)
    be, bl = W.uniform(rng, 300, n, -300, 300)
    extra_a, extra_b = [], []
    for _ in range(40):
        A, B = W.mul_near_half(rng, n)
        extra_a.append((W.exp_word(int(rng.integers(-9, 9)), int(rng.integers(0, 2))), W.int_to_limbs(A, n)))
        extra_b.append((W.exp_word(int(rng.integers(-9, 9)), int(rng.integers(0, 2))), W.int_to_limbs(B, n)))
    ones = np.full(n, 0xFFFFFFFF, np.uint32)
    extra_a += [(W.exp_word(3, 0), ones), (W.exp_word(-2, 1), ones)]
    extra_b += [(W.exp_word(5, 0), ones), (W.exp_word(7, 0), ones)]
    # exponent words near the range limits: BIAS + e close to 5 (TINY) and to 2^31 (INF)
    for wa, wb in ((5, BIAS + 2), (5, BIAS + 1), (5, BIAS), (6, BIAS), (BIAS + 1, 6), (0x7FFFFFF0, BIAS + 20),
                   (0x7FFFFFF0, BIAS - 20), (0x7FFFFFFF, BIAS + 1), (0x7FFFFFFF, BIAS)):
        for sa, sb in ((0, 0), (1, 0)):
            extra_a.append((np.uint32(2 * wa + sa), W.uniform(rng, 1, n, 0, 0)[1][0]))
            extra_b.append((np.uint32(2 * wb + sb), W.uniform(rng, 1, n, 0, 0)[1][0]))
    se, sl = W.specials(n)
    for i in range(len(se)):
        for j in range(len(se)):
            extra_a.append((se[i], sl[i])); extra_b.append((se[j], sl[j]))
    ae = np.concatenate([ae, np.array([e for e, _ in extra_a], np.uint32)])
    al = np.concatenate([al, np.stack([l for _, l in extra_a])])
    be = np.concatenate([be, np.array([e for e, _ in extra_b], np.uint32)])
    bl = np.concatenate([bl, np.stack([l for _, l in extra_b])])
    return ae, al, be, bl


@pytest.fixture(scope="module", autouse=True)
def device_errors_clear():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


@pytest.mark.parametrize("n", [8, 16, 32, 7, 31])
def test_row_mul_matches_oracle(n):
    rng = np.random.default_rng(900 + n)
    ae, al, be, bl = mul_cases(rng, n)
    count = len(ae)
    assert fpa.set_op_config(2, n, 16) == 0
    try:
        A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
        assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0
        for mode in range(5):
            assert fpa.fpa_mul(R, A, B, mode) == 0
            got = R.to_host()
            exp = oracle.run(2, n, mode, ae, al, be, bl)
            bad = mismatches(exp[0], exp[1], got[0], got[1])
            assert bad.size == 0, f"n={n} mode={mode}: {bad.size} mismatches\n" + \
                describe(bad[0], ae, al, be, bl, exp[0], exp[1], got[0], got[1])
    finally:
        fpa.set_op_config(2, n, -1)
