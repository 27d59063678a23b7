"""The div/sqrt/fma kernels run every thread of a CTA for the same number of iterations
with a CTA barrier after each (lockstep).  Operation counts that leave the last iteration
partly or almost empty (1, 2, a group count plus one, odd sizes) must give the oracle's
results, in the elementwise kernels, the batched form and the Newton chain."""
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


@pytest.mark.parametrize("n", [4, 9, 32, 128, 257])
@pytest.mark.parametrize("count", [1, 2, 17, 65, 1000])
def test_div_sqrt_tail_counts(n, count):
    rng = np.random.default_rng(31 * n + count)
    ae, al = W.uniform(rng, count, n, -50, 50)
    be, bl = W.uniform(rng, count, n, -50, 50)
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0
    assert fpa.fpa_div(R, A, B, 3) == 0
    got = R.to_host()
    exp = oracle.run(3, n, 3, ae, al, be, bl)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0
    a2 = ae & ~np.uint32(1)
    assert A.to_device(a2, al) == 0
    assert fpa.fpa_sqrt(R, A, 3) == 0
    got = R.to_host()
    exp = oracle.run(4, n, 3, a2, al)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0


@pytest.mark.parametrize("count", [1, 3, 33])
def test_fma_tail_counts(count):
    n = 32
    rng = np.random.default_rng(count)
    ae, al = W.uniform(rng, count, n, -50, 50)
    be, bl = W.uniform(rng, count, n, -50, 50)
    ce, cl = W.uniform(rng, count, n, -80, 80)
    A, B, C, R = (fpa.FpaArray(count, 32 * n) for _ in range(4))
    assert A.to_device(ae, al) == 0 and B.to_device(be, bl) == 0 and C.to_device(ce, cl) == 0
    assert fpa.fpa_fma(R, A, B, C, 3) == 0
    got = R.to_host()
    exp = oracle.run_fma(n, 3, ae, al, be, bl, ce, cl)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0


@pytest.mark.parametrize("count", [1, 5, 40])
def test_batch_div_sqrt_tail_counts(count):
    torch = pytest.importorskip("torch")
    for op in (3, 4):
        ops = np.full(count, op, np.uint8)
        limbs = np.full(count, 96, np.uint16)
        descs, ae, al, be, bl, total = W.mixed(50 + op + count, count, ops=ops, limbs=limbs)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
        d = [dev(x) for x in (ae, al, be, bl)]
        d_re = torch.zeros(count, dtype=torch.int32, device="cuda")
        d_rl = torch.zeros(total, dtype=torch.int32, device="cuda")
        b = fpa.Batch(descs)
        assert b.run(d_re.data_ptr(), d_rl.data_ptr(), *(x.data_ptr() for x in d)) == 0
        torch.cuda.synchronize()
        b.destroy()
        off = descs["a_off"]
        exp_e, exp_l = oracle.run_mixed(descs["op"], descs["limbs"], descs["mode"], ae, al, off, be, bl, off, off,
                                        total)
        ge, gl = d_re.cpu().numpy().view(np.uint32), d_rl.cpu().numpy().view(np.uint32)
        assert (ge == exp_e).all()
        for i in np.nonzero(exp_e > 8)[0]:
            o = int(off[i])
            assert (gl[o:o + 96] == exp_l[o:o + 96]).all()
