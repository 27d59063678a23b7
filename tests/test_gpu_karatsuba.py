"""fpa_mul with the Karatsuba split (one level, three half-size products on half-width
tiles): bit-identical to the schoolbook product and to the oracle on every configuration
that carries it (at least 256 limbs on tiles of at least 8), for odd and even sizes up to the capacity, including
mantissas whose half sums carry (all ones) and whose low halves are zero."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches

pytestmark = pytest.mark.gpu


def operands(rng, n, count):
    ae, al = W.uniform(rng, count, n, -300, 300)
    be, bl = W.uniform(rng, count, n, -300, 300)
    al[0] = 0xFFFFFFFF; bl[0] = 0xFFFFFFFF                     # both half sums carry
    al[1] = 0; al[1, -1] = 0x80000000; bl[1] = 0xFFFFFFFF        # x0 = 0
    h = (n + 1) // 2
    al[2, :h] = 0xFFFFFFFF; bl[2, h:] = 0xFFFFFFFF; bl[2, -1] |= 0x80000000
    return ae, al, be, bl


def run_mul(n, mode, ae, al, be, bl):
    count = len(ae)
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0
    assert fpa.fpa_mul(R, A, B, mode) == 0
    return R.to_host()


@pytest.fixture(scope="module", autouse=True)
def restore_threshold():
    old = fpa.get_karatsuba_limbs()
    fpa.device_errors()
    yield
    fpa.set_karatsuba_limbs(old)
    assert fpa.device_errors() == 0


@pytest.mark.parametrize("cfg", [c for c in range(16)])
def test_karatsuba_every_configuration(cfg):
    lanes, tile, pairs = fpa.configs()[cfg]
    cap = lanes * tile * pairs
    if tile < 8 or cap < 256:
        pytest.skip("the split is compiled into configurations of >= 256 limbs on tiles of >= 8")
    rng = np.random.default_rng(700 + cfg)
    for n in sorted({4, 5, 8, 9, cap // 2 - 1, cap // 2, cap // 2 + 1, cap - 1, cap}):
        if n < 4 or n > min(cap, 512):
            continue
        ae, al, be, bl = operands(rng, n, 40)
        assert fpa.set_op_config(2, n, cfg) == 0
        try:
            for mode in (3, int(rng.integers(0, 5))):
                fpa.set_karatsuba_limbs(0)
                plain = run_mul(n, mode, ae, al, be, bl)
                fpa.set_karatsuba_limbs(4)
                kara = run_mul(n, mode, ae, al, be, bl)
                assert np.array_equal(plain[0], kara[0]) and np.array_equal(plain[1], kara[1]), (cfg, n, mode)
                exp = oracle.run(2, n, mode, ae, al, be, bl)
                assert mismatches(exp[0], exp[1], kara[0], kara[1]).size == 0, (cfg, n, mode)
        finally:
            fpa.set_op_config(2, n, -1)


def test_karatsuba_threshold_api():
    fpa.set_karatsuba_limbs(0)
    assert fpa.get_karatsuba_limbs() == 0
    fpa.set_karatsuba_limbs(256)
    assert fpa.get_karatsuba_limbs() == 256
    # results at the default sizes of the split are exact
    rng = np.random.default_rng(5)
    for n in (256, 384, 512):
        ae, al, be, bl = operands(rng, n, 64)
        got = run_mul(n, 3, ae, al, be, bl)
        exp = oracle.run(2, n, 3, ae, al, be, bl)
        assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0, n
