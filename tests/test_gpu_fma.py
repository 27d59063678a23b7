"""GPU: fpa_gb300_fma (r = RND(a*b + c), one rounding) through the C ABI against the oracle
(itself checked against MPFR's mpfr_fma on CPU), every rounding mode, bit-exact."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from fma_cases import fma_cases, special_cases
from helpers import mismatches

pytestmark = pytest.mark.gpu


def gpu_fma(n, mode, ae, al, be, bl, ce, cl):
    count = len(ae)
    arrs = []
    for e, l in ((ae, al), (be, bl), (ce, cl)):
        X = fpa.FpaArray(count, 32 * n)
        assert X.to_device(e, l) == fpa.fpa_success
        arrs.append(X)
    R = fpa.FpaArray(count, 32 * n)
    assert fpa.fpa_fma(R, *arrs, mode) == fpa.fpa_success
    return R.to_host()


@pytest.mark.parametrize("n", [1, 2, 5, 8, 16, 31, 32, 33, 64, 100, 128, 160, 256, 512])
def test_fma_matches_oracle(n):
    ae, al, be, bl, ce, cl = fma_cases(500 + n, n, count=192)
    for mode in range(5):
        exp = oracle.run_fma(n, mode, ae, al, be, bl, ce, cl)
        got = gpu_fma(n, mode, ae, al, be, bl, ce, cl)
        bad = mismatches(exp[0], exp[1], got[0], got[1])
        assert bad.size == 0, (n, mode, bad[:5], [hex(x) for x in exp[0][bad[:3]]], [hex(x) for x in got[0][bad[:3]]])


def test_fma_specials():
    n = 8
    ae, al, be, bl, ce, cl = special_cases(n)
    exp = oracle.run_fma(n, 3, ae, al, be, bl, ce, cl)
    got = gpu_fma(n, 3, ae, al, be, bl, ce, cl)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0


def test_fma_argument_checks():
    a, b, c, r = (fpa.FpaArray(4, 1024) for _ in range(4))
    d = fpa.FpaArray(5, 1024)
    assert fpa.fpa_fma(r, a, b, d, 3) == fpa.fpa_invalid_counts
    e = fpa.FpaArray(4, 2048)
    assert fpa.fpa_fma(r, a, b, e, 3) == fpa.fpa_invalid_precisions
    assert fpa.device_errors() == 0
