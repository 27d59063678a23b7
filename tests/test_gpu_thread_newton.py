"""GPU: mul, div and sqrt with one thread per operation (configurations 18 and 19,
fpa_thread_newton.cu) forced through the per-operation table, bit-exact against the oracle
in every rounding mode at sizes from 8 to 128 limbs, on operand sets with near-halfway
products and near-exact quotients and squares (the operations the second, exact pass
finishes), in place (r = a), at ragged counts (partial warps, one operation), and identical
to the lane-group kernels on the 4096-bit workload."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def device_errors_clear():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


def operands(op, n, count, seed, hard_frac=0.2):
    (ae, al), (be, bl) = W.workload_4096({2: "mul", 3: "div", 4: "sqrt"}[op], seed, count=count, n=n,
                                         hard_frac=hard_frac, pool=16)
    return ae, al, be, bl


def run(op, n, mode, ae, al, be, bl, cfg, inplace=False):
    assert fpa.set_op_config(op, n, cfg) == 0
    try:
        A = fpa.FpaArray(len(ae), 32 * n)
        B = fpa.FpaArray(len(ae), 32 * n)
        assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0
        R = A if inplace else fpa.FpaArray(len(ae), 32 * n)
        rc = {2: fpa.fpa_mul, 3: fpa.fpa_div}[op](R, A, B, mode) if op != 4 else fpa.fpa_sqrt(R, A, mode)
        assert rc == 0
        return R.to_host()
    finally:
        fpa.set_op_config(op, n, -1)


@pytest.mark.parametrize("n", [8, 9, 11, 16, 31, 33, 48, 64, 65, 96, 127, 128])
@pytest.mark.parametrize("op", [2, 3, 4], ids=["mul", "div", "sqrt"])
def test_one_thread_every_mode(op, n):
    ae, al, be, bl = operands(op, n, 600, 40 + n)
    for cfg in ([18, 19] if n <= 64 else [18]):
        for mode in range(5):
            got = run(op, n, mode, ae, al, be, bl, cfg)
            exp = oracle.run(op, n, mode, ae, al, be, bl, threads=8)
            bad = mismatches(exp[0], exp[1], got[0], got[1])
            assert bad.size == 0, (op, n, cfg, mode, bad.size, int(bad[0]))


@pytest.mark.parametrize("count", [1, 2, 31, 33, 95, 1000])
@pytest.mark.parametrize("op", [2, 3, 4], ids=["mul", "div", "sqrt"])
def test_one_thread_ragged_counts_and_in_place(op, count):
    n = 128
    ae, al, be, bl = operands(op, n, count, 900 + count, hard_frac=0.3)
    exp = oracle.run(op, n, 3, ae, al, be, bl, threads=8)
    for inplace in (False, True):
        got = run(op, n, 3, ae, al, be, bl, 18, inplace=inplace)
        assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0, (op, count, inplace)


@pytest.mark.parametrize("op", [2, 3, 4], ids=["mul", "div", "sqrt"])
def test_one_thread_equals_lane_groups_at_4096_bits(op):
    n = 128
    ae, al, be, bl = operands(op, n, 1 << 15, 77, hard_frac=0.05)
    group_cfg = {2: 7, 3: 11, 4: 12}[op]
    a = run(op, n, 3, ae, al, be, bl, group_cfg)
    b = run(op, n, 3, ae, al, be, bl, 18)
    assert mismatches(a[0], a[1], b[0], b[1]).size == 0


def test_all_hard_operations():
    """Every operation needs the exact pass: exact and near ties of mul, a = b exactly
    (quotient 1) and perfect squares."""
    n, count = 64, 256
    rng = np.random.default_rng(3)
    mp = [W.mul_near_half(rng, n) for _ in range(count)]
    ml = np.stack([W.int_to_limbs(A, n) for A, _ in mp])
    nl = np.stack([W.int_to_limbs(B, n) for _, B in mp])
    me = W.exp_word(rng.integers(-9, 9, count), rng.integers(0, 2, count))
    for mode in range(5):
        got = run(2, n, mode, me, ml, me, nl, 18)
        exp = oracle.run(2, n, mode, me, ml, me, nl)
        assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0, mode
    be, bl = W.uniform(rng, count, n, -50, 50)
    ae, al = be.copy(), bl.copy()
    got = run(3, n, 3, ae, al, be, bl, 18)
    exp = oracle.run(3, n, 3, ae, al, be, bl)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0
    sq = [W.sqrt_near_exact(rng, n) for _ in range(count)]
    sl = np.stack([W.int_to_limbs(A, n) for A, _ in sq])
    se = W.exp_word(2 * rng.integers(-9, 9, count) + np.array([p for _, p in sq]), 0)
    for mode in range(5):
        got = run(4, n, mode, se, sl, se, sl, 18)
        exp = oracle.run(4, n, mode, se, sl)
        assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0, mode
