"""GPU: our results against the reference's own kernels (its fpa.cu compiled for sm_103a,
loaded from oracle/_ref/ref_fpa.cubin) on the same inputs.  They must be identical
wherever the reference agrees with MPFR; every difference must be a case where the
reference's result differs from the correctly rounded (oracle/MPFR) one."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches
from test_gpu_parity import gpu_run

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not oracle.ref_gpu_available(), reason="reference cubin not built")]

OPNAMES = ["add", "sub", "mul", "div", "sqrt"]


def compare_three(op, n, mode, ae, al, be, bl):
    ours = gpu_run(op, n, mode, ae, al, be, bl)
    ref = oracle.ref_gpu_run(OPNAMES[op], n, mode, ae, al, be, bl)
    exact = oracle.run(op, n, mode, ae, al, be, bl)
    assert mismatches(exact[0], exact[1], ours[0], ours[1]).size == 0
    diff = mismatches(ref[0], ref[1], ours[0], ours[1])
    ref_wrong = mismatches(exact[0], exact[1], ref[0], ref[1])
    # every place where we differ from the reference is a place where the reference is not
    # correctly rounded
    assert set(diff.tolist()) <= set(ref_wrong.tolist())
    return diff.size


@pytest.mark.parametrize("n", [32, 64, 128, 256])
@pytest.mark.parametrize("op", [2, 3, 4], ids=["mul", "div", "sqrt"])
def test_identical_to_reference_on_random(op, n):
    rng = np.random.default_rng(77 + n + op)
    ae, al = W.uniform(rng, 2048, n, -1000, 1000, signs=(op != 4))
    be, bl = W.uniform(rng, 2048, n, -1000, 1000)
    assert compare_three(op, n, 3, ae, al, be, bl) == 0


@pytest.mark.parametrize("n", [32, 128])
def test_reference_test_pattern(n):
    """The reference's own test distribution (tests.c:803-925) for mul/div/sqrt."""
    rng = np.random.default_rng(5 * n)
    ae, al = W.reference_style(rng, 512, n)
    be, bl = W.reference_style(rng, 512, n)
    for op in (2, 3):
        assert compare_three(op, n, 3, ae, al, be, bl) == 0
    assert compare_three(4, n, 3, ae & ~np.uint32(1), al, be, bl) == 0


def test_near_halfway_divergences_are_reference_rounding_errors():
    """Exact-tie products: the reference reads the parity bit before its one-bit
    normalisation (fpa_warp_mul.h:115-121), so some ties round the wrong way there."""
    n = 32
    rng = np.random.default_rng(3)
    pairs = [W.mul_near_half(rng, n) for _ in range(256)]
    al = np.stack([W.int_to_limbs(a, n) for a, _ in pairs]); bl = np.stack([W.int_to_limbs(b, n) for _, b in pairs])
    ae = W.exp_word(rng.integers(-9, 9, 256), rng.integers(0, 2, 256))
    be = W.exp_word(rng.integers(-9, 9, 256), rng.integers(0, 2, 256))
    ndiff = compare_three(2, n, 3, ae, al, be, bl)
    print("tie cases where the reference kernel is not correctly rounded:", ndiff)
