"""CPU: the oracle's single-rounding fma (no counterpart in the reference) against MPFR's
mpfr_fma, including cancellation and wide exponent gaps, and its special-value rules."""
import numpy as np
import pytest

import gold
import oracle
from fma_cases import fma_cases, special_cases
from helpers import mismatches


@pytest.mark.skipif(not gold.available(), reason="libmpfr not installed")
@pytest.mark.parametrize("n", [1, 3, 8, 32, 33, 128])
def test_oracle_fma_matches_mpfr(n):
    ae, al, be, bl, ce, cl = fma_cases(100 + n, n)
    for mode in range(5):
        g = gold.run_fma(n, mode, ae, al, be, bl, ce, cl)
        o = oracle.run_fma(n, mode, ae, al, be, bl, ce, cl)
        bad = mismatches(g[0], g[1], o[0], o[1])
        assert bad.size == 0, (n, mode, bad[:5])


def test_oracle_fma_specials():
    """A special operand anywhere: the result is the add table applied to the class of the
    exact product (the mul table's) and c."""
    n = 4
    ae, al, be, bl, ce, cl = special_cases(n)
    e, _ = oracle.run_fma(n, 3, ae, al, be, bl, ce, cl)
    pe, pl = oracle.run(2, n, 3, ae, al, be, bl)
    cls = (ae <= 8) | (be <= 8)                      # the product is a class
    s, _ = oracle.run(0, n, 3, pe[cls], pl[cls], ce[cls], cl[cls])
    assert np.array_equal(e[cls], s)
    assert cls.sum() > 0 and (~cls).sum() > 0
