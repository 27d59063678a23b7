"""GPU: fused chains (the dot and Newton sqrt shapes at small sizes) against the same operation sequence
run step by step in the oracle: dot products acc = RN(acc + RN(x*y)) and Newton square
roots y = RN(RN(y + RN(x/y)) * 0.5)."""
import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint32)


def oracle_dot(n, mode, xe, xl, ye, yl, count, length):
    xl = xl.reshape(count, length, n); yl = yl.reshape(count, length, n)
    xe = xe.reshape(count, length); ye = ye.reshape(count, length)
    acc_e = np.full(count, W.CLS_ZERO, np.uint32)
    acc_l = np.zeros((count, n), np.uint32)
    for i in range(length):
        te, tl = oracle.run(2, n, mode, xe[:, i], xl[:, i], ye[:, i], yl[:, i])
        acc_e, acc_l = oracle.run(0, n, mode, acc_e, acc_l, te, tl)
    return acc_e, acc_l


def half(e):
    """exact y * 0.5 on exponent words (values only in these tests)"""
    return np.where(e > 8, e - 2, e).astype(np.uint32)


@pytest.mark.parametrize("n,mode", [(64, 3), (64, 1), (8, 3), (100, 4)])
def test_fused_dot_matches_stepwise(n, mode):
    rng = np.random.default_rng(n + mode)
    count, length = 48, 40
    xe, xl = W.uniform(rng, count * length, n, -30, 30)
    ye, yl = W.uniform(rng, count * length, n, -30, 30)
    re_ = torch.zeros(count, dtype=torch.int32, device="cuda")
    rl = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    dxe, dxl, dye, dyl = dev(xe), dev(xl), dev(ye), dev(yl)
    assert fpa.dot(32 * n, count, length, mode, re_.data_ptr(), rl.data_ptr(), dxe.data_ptr(), dxl.data_ptr(),
                   dye.data_ptr(), dyl.data_ptr()) == 0
    torch.cuda.synchronize()
    exp = oracle_dot(n, mode, xe, xl, ye, yl, count, length)
    got = host(re_), host(rl).reshape(count, n)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0


@pytest.mark.parametrize("n", [32, 256])
def test_fused_newton_sqrt_matches_stepwise(n):
    rng = np.random.default_rng(n)
    count, iters, mode = 64, 8, 3
    xl = rng.integers(0, 1 << 32, size=(count, n), dtype=np.uint64).astype(np.uint32)
    xl[:, -1] |= np.uint32(0x80000000)
    xe = W.exp_word(np.ones(count, dtype=np.int64), 0)             # x in [1, 2)
    y0 = np.zeros((count, n), np.uint32); y0[:, -1] = 0xC0000000    # y0 = 1.5
    ye0 = W.exp_word(np.ones(count, dtype=np.int64), 0)
    dye, dyl = dev(ye0), dev(y0)
    dxe, dxl = dev(xe), dev(xl)
    assert fpa.newton_sqrt(32 * n, count, iters, mode, dye.data_ptr(), dyl.data_ptr(), dxe.data_ptr(),
                           dxl.data_ptr()) == 0
    torch.cuda.synchronize()
    ye, yl = ye0.copy(), y0.copy()
    for _ in range(iters):
        te, tl = oracle.run(3, n, mode, xe, xl, ye, yl)
        se, sl = oracle.run(0, n, mode, ye, yl, te, tl)
        ye, yl = half(se), sl
    got = host(dye), host(dyl).reshape(count, n)
    assert mismatches(ye, yl, got[0], got[1]).size == 0
    assert fpa.device_errors() == 0
