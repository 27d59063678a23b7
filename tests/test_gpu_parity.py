"""GPU parity: the CUDA path through the fpa.h C-ABI against MPFR (golden fixtures) and the
oracle, for every operation and rounding mode, bit-exact."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import describe, golden_files, load_golden, mismatches

pytestmark = pytest.mark.gpu

FNS = [fpa.fpa_add, fpa.fpa_sub, fpa.fpa_mul, fpa.fpa_div, None]


def gpu_run(op, n, mode, ae, al, be=None, bl=None, inplace=False):
    count = len(ae)
    A = fpa.FpaArray(count, 32 * n)
    assert A.to_device(ae, al) == fpa.fpa_success
    if op != 4:
        B = fpa.FpaArray(count, 32 * n)
        assert B.to_device(be, bl) == fpa.fpa_success
    R = A if inplace else fpa.FpaArray(count, 32 * n)
    if op == 4:
        rc = fpa.fpa_sqrt(R, A, mode)
    else:
        rc = FNS[op](R, A, B, mode)
    assert rc == fpa.fpa_success
    return R.to_host()


def check(op, n, mode, ae, al, be, bl, expect=None, **kw):
    if expect is None:
        expect = oracle.run(op, n, mode, ae, al, be, bl)
    got = gpu_run(op, n, mode, ae, al, be, bl, **kw)
    bad = mismatches(expect[0], expect[1], got[0], got[1])
    assert bad.size == 0, f"op={op} n={n} mode={mode} {bad.size} mismatches\n" + describe(
        bad[0], ae, al, be if be is not None else ae, bl if bl is not None else al, expect[0], expect[1], got[0], got[1])


@pytest.fixture(scope="module", autouse=True)
def device_errors_clear():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1])
def test_gpu_matches_mpfr_golden(path):
    z = load_golden(path)
    op, n = int(z["op"]), int(z["n"])
    for mode in range(5):
        check(op, n, mode, z["a_exps"], z["a_limbs"], z["b_exps"], z["b_limbs"],
              expect=(z["r_exps"][mode], z["r_limbs"][mode]))


SIZES = [1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 32, 33, 48, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256, 257,
         384, 511, 512]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("op", range(5), ids=["add", "sub", "mul", "div", "sqrt"])
def test_gpu_matches_oracle(op, n):
    rng = np.random.default_rng(1000 * op + n)
    count = 96 if n <= 128 else 24
    ae, al = W.uniform(rng, count, n, -100, 100, signs=(op != 4))
    be, bl = W.uniform(rng, count, n, -100, 100)
    re_, rl = W.reference_style(rng, count // 2, n)
    if op == 4:
        re_ &= ~np.uint32(1)
    ae = np.concatenate([ae, re_]); al = np.concatenate([al, rl])
    rb, rbl = W.reference_style(rng, count // 2, n)
    be = np.concatenate([be, rb]); bl = np.concatenate([bl, rbl])
    if op in (0, 1):   # close exponents: cancellation and carries
        ae[: count // 4] = (be[: count // 4] & ~np.uint32(1)) | (ae[: count // 4] & np.uint32(1))
    for mode in range(5):
        check(op, n, mode, ae, al, be, bl)


@pytest.mark.parametrize("n", [1, 4, 32, 128, 512])
@pytest.mark.parametrize("op", range(5), ids=["add", "sub", "mul", "div", "sqrt"])
def test_gpu_special_values(op, n):
    exps, limbs = W.specials(n)
    k = len(exps)
    ae = np.repeat(exps, k); al = np.repeat(limbs, k, axis=0)
    be = np.tile(exps, k); bl = np.tile(limbs, (k, 1))
    for mode in (0, 3):
        check(op, n, mode, ae, al, be, bl)


@pytest.mark.parametrize("n", [32, 128])
def test_gpu_near_halfway(n):
    rng = np.random.default_rng(n)
    for op, make in ((2, W.mul_near_half), (3, W.div_near_exact)):
        pairs = [make(rng, n) for _ in range(48)]
        al = np.stack([W.int_to_limbs(a, n) for a, _ in pairs]); bl = np.stack([W.int_to_limbs(b, n) for _, b in pairs])
        ae = W.exp_word(rng.integers(-9, 9, 48), rng.integers(0, 2, 48))
        be = W.exp_word(rng.integers(-9, 9, 48), rng.integers(0, 2, 48))
        for mode in range(5):
            check(op, n, mode, ae, al, be, bl)
    sq = [W.sqrt_near_exact(rng, n) for _ in range(48)]
    al = np.stack([W.int_to_limbs(a, n) for a, _ in sq])
    ae = W.exp_word(np.array([2 * int(rng.integers(-9, 9)) + par for _, par in sq]), 0)
    for mode in range(5):
        check(4, n, mode, ae, al, ae, al)


def test_gpu_all_ones_mantissas():
    """Results that round up into the next binade (fpa_warp_mul.h:99-105,
    fpa_warp_div.h:178-183, fpa_warp_sqrt.h:238-242)."""
    n = 8
    ones = np.full((4, n), 0xFFFFFFFF, np.uint32)
    top = np.zeros((4, n), np.uint32); top[:, -1] = 0x80000000
    ae = W.exp_word(np.array([0, 2, -4, 6]), np.array([0, 1, 0, 1]))
    for mode in range(5):
        for op in range(4):
            check(op, n, mode, ae, ones, ae, ones)
            check(op, n, mode, ae, ones, ae, top)
        check(4, n, mode, ae & ~np.uint32(1), ones, ae, ones)


def test_gpu_inplace_and_edge_counts():
    n = 32
    rng = np.random.default_rng(5)
    ae, al = W.uniform(rng, 33, n, -20, 20)
    be, bl = W.uniform(rng, 33, n, -20, 20)
    for op in range(4):
        check(op, n, 3, ae, al, be, bl, inplace=True)
    check(2, n, 3, ae[:1], al[:1], be[:1], bl[:1])
    A = fpa.FpaArray(0, 1024)
    assert fpa.fpa_mul(A, A, A, 3) == fpa.fpa_success


def test_gpu_larger_batch_uniform():
    """A few thousand instances per config: exercises the grid-stride loop."""
    rng = np.random.default_rng(9)
    for n in (32, 128):
        ae, al = W.uniform(rng, 5000, n, -64, 64)
        be, bl = W.uniform(rng, 5000, n, -64, 64)
        for op in range(4):
            check(op, n, 3, ae, al, be, bl)
