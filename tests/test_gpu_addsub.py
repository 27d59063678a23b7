"""add/sub on every lane-group configuration, with structured operands that reach each
branch of the alignment and rounding: exponent differences at and around every word
boundary, the 64 guard bits and the precision cap; deep and exact cancellation; carries
through all-ones mantissas; exact ties.  Bit-exact against the oracle in every rounding
mode, through the fpa.h C-ABI."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import describe, mismatches

pytestmark = pytest.mark.gpu


def addsub_cases(rng, n):
    """(a_exps, a_limbs, b_exps, b_limbs) for one precision of n limbs."""
    p = 32 * n
    shifts = sorted({0, 1, 2, 3, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 129,
                     p - 33, p - 32, p - 1, p, p + 1, p + 31, p + 32, p + 62, p + 63, p + 64, p + 65, p + 66,
                     p + 200} - {-1})
    shifts = [d for d in shifts if d >= 0]
    ae_l, al_l, be_l, bl_l = [], [], [], []

    def add(ea, sa, ma, eb, sb, mb):
        ae_l.append(W.exp_word(ea, sa)); al_l.append(W.int_to_limbs(ma, n))
        be_l.append(W.exp_word(eb, sb)); bl_l.append(W.int_to_limbs(mb, n))

    top = 1 << (p - 1)
    ones = (1 << p) - 1

    def rand_m():
        return top | (int.from_bytes(rng.bytes(4 * n), "little") & (top - 1))

    for d in shifts:
        for _ in range(3):
            ea = int(rng.integers(-40, 40))
            ma, mb = rand_m(), rand_m()
            sa, sb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
            add(ea, sa, ma, ea - d, sb, mb)              # |a| > |b|
            add(ea - d, sa, mb, ea, sb, ma)              # |b| > |a|
        # carries through an all-ones mantissa; borrows through a power of two
        add(3, 0, ones, 3 - d, 0, rand_m())
        add(3, 0, top, 3 - d, 1, rand_m())
        add(3, 1, top, 3 - d, 0, ones)
        # exact ties below the last place: b = 1/2 ulp of a (d = p + 1), and neighbours
        add(5, int(rng.integers(0, 2)), rand_m(), 5 - d, int(rng.integers(0, 2)), top)
    # deep cancellation: equal exponents, b shares the top k limbs of a
    for k in range(n + 1):
        ma = rand_m()
        keep = ma >> (32 * (n - k)) << (32 * (n - k)) if k < n else ma
        mb = keep | (int.from_bytes(rng.bytes(4 * n), "little") & ((1 << (32 * (n - k))) - 1)) if k < n else ma
        mb |= top
        for (sa, sb) in ((0, 1), (1, 0), (0, 0)):
            add(7, sa, ma, 7, sb, mb)
            add(7, sa, ma, 6, sb, mb)                    # d = 1 with the top bits cancelling
    # d = 1 and 2 with b close to 2a: cancellation to a few bits
    for _ in range(8):
        ma = rand_m()
        mb = ((ma << 1) & ones) | 1
        mb |= top
        add(0, 0, ma, -1, 1, mb)
        add(0, 1, ma, -2, 0, mb)
    ae = np.array(ae_l, dtype=np.uint32); be = np.array(be_l, dtype=np.uint32)
    return ae, np.array(al_l, dtype=np.uint32), be, np.array(bl_l, dtype=np.uint32)


def run_cfg(cfg, n, op, mode, ae, al, be, bl):
    count = len(ae)
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0
    fn = fpa.fpa_add if op == 0 else fpa.fpa_sub
    assert fn(R, A, B, mode) == 0
    return R.to_host()


def sizes_for(cfg):
    lanes, tile, pairs = fpa.configs()[cfg]
    gk = lanes * tile
    cap = gk * pairs
    out = {1, 2, 3, 4, 5, 8, 16, gk // 2, gk // 2 + 1, gk - 1, gk, gk + 1, cap - 1, cap}
    return sorted(x for x in out if 1 <= x <= min(cap, 512))


@pytest.fixture(scope="module", autouse=True)
def device_errors_clear():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


@pytest.mark.parametrize("cfg", range(18))
def test_addsub_structured_every_configuration(cfg):
    rng = np.random.default_rng(500 + cfg)
    for n in sizes_for(cfg):
        ae, al, be, bl = addsub_cases(rng, n)
        for op in (0, 1):
            assert fpa.set_op_config(op, n, cfg) == 0
            try:
                for mode in range(5):
                    got = run_cfg(cfg, n, op, mode, ae, al, be, bl)
                    exp = oracle.run(op, n, mode, ae, al, be, bl)
                    bad = mismatches(exp[0], exp[1], got[0], got[1])
                    assert bad.size == 0, f"cfg={cfg} op={op} n={n} mode={mode}: {bad.size} mismatches\n" + \
                        describe(bad[0], ae, al, be, bl, exp[0], exp[1], got[0], got[1])
            finally:
                assert fpa.set_op_config(op, n, -1) == 0


@pytest.mark.parametrize("n", [8, 32, 64, 128, 512])
def test_addsub_unaligned_operands(n):
    """Operands and results at word offsets that are not 16-byte aligned take the scalar
    loads and stores of the register path."""
    import torch
    rng = np.random.default_rng(n)
    ae, al = W.uniform(rng, 257, n, -70, 70)
    be, bl = W.uniform(rng, 257, n, -70, 70)
    for op in (0, 1):
        exp = oracle.run(op, n, 3, ae, al, be, bl)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
        # limbs at an offset of one word inside a larger buffer
        big_a = torch.zeros(257 * n + 1, dtype=torch.int32, device="cuda"); big_a[1:] = dev(al.reshape(-1))
        big_b = torch.zeros(257 * n + 1, dtype=torch.int32, device="cuda"); big_b[1:] = dev(bl.reshape(-1))
        big_r = torch.zeros(257 * n + 1, dtype=torch.int32, device="cuda")
        d_ae, d_be = dev(ae), dev(be)
        d_re = torch.zeros(257, dtype=torch.int32, device="cuda")
        rc = fpa.elementwise(op, 32 * n, 257, 3, d_re.data_ptr(), big_r.data_ptr() + 4, d_ae.data_ptr(),
                             big_a.data_ptr() + 4, d_be.data_ptr(), big_b.data_ptr() + 4)
        assert rc == 0
        torch.cuda.synchronize()
        got_e = d_re.cpu().numpy().view(np.uint32)
        got_l = big_r[1:].cpu().numpy().view(np.uint32).reshape(257, n)
        assert mismatches(exp[0], exp[1], got_e, got_l).size == 0, (op, n)
