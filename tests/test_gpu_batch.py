"""GPU: the batched form (mixed operations and precisions in one submission) against the
oracle and against the elementwise kernels; CUDA-graph capture and replay; configuration
table overrides (every lane-group configuration is exercised)."""
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


def host_u32(t):
    return t.cpu().numpy().view(np.uint32)


def run_batch(descs, ae, al, be, bl, total, graph=False):
    d_ae, d_al, d_be, d_bl = dev(ae), dev(al), dev(be), dev(bl)
    d_re = torch.zeros(len(descs), dtype=torch.int32, device="cuda")
    d_rl = torch.zeros(max(total, 1), dtype=torch.int32, device="cuda")
    b = fpa.Batch(descs)
    ptrs = (d_re.data_ptr(), d_rl.data_ptr(), d_ae.data_ptr(), d_al.data_ptr(), d_be.data_ptr(), d_bl.data_ptr())
    if graph:
        assert b.capture(*ptrs) == 0
        assert b.graph_launch() == 0
        torch.cuda.synchronize()
        first = (host_u32(d_re).copy(), host_u32(d_rl).copy())
        d_re.zero_(); d_rl.zero_()
        assert b.graph_launch() == 0
    else:
        assert b.run(*ptrs) == 0
    torch.cuda.synchronize()
    out = host_u32(d_re).copy(), host_u32(d_rl).copy()
    info = b.info()
    b.destroy()
    if graph:
        assert np.array_equal(first[0], out[0]) and np.array_equal(first[1], out[1])
    return out, info


def check_mixed(descs, ae, al, be, bl, total, got):
    off = descs["a_off"]
    exp_e, exp_l = oracle.run_mixed(descs["op"], descs["limbs"], descs["mode"], ae, al, off, be, bl, off, off,
                                    total, threads=8)
    ge, gl = got
    bad = ge != exp_e
    for i in np.nonzero(exp_e > 8)[0]:
        o, n = int(off[i]), int(descs["limbs"][i])
        if not np.array_equal(gl[o:o + n], exp_l[o:o + n]):
            bad[i] = True
    idx = np.nonzero(bad)[0]
    assert idx.size == 0, f"{idx.size} mismatches, first: op={descs['op'][idx[0]]} limbs={descs['limbs'][idx[0]]}"


@pytest.fixture(scope="module", autouse=True)
def clean_errors():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


def test_mixed_batch_matches_oracle():
    descs, ae, al, be, bl, total = W.mixed(11, 3000, min_bits=32, max_bits=16384)
    rng = np.random.default_rng(4)
    descs["mode"] = rng.integers(0, 5, size=len(descs))
    got, info = run_batch(descs, ae, al, be, bl, total)
    tasks, kernels = info
    # the three lane-group classes and the one-thread class (mul/div/sqrt of 8-128 limbs)
    assert kernels == 4 and all(t > 0 for t in tasks)
    check_mixed(descs, ae, al, be, bl, total, got)


def test_batch_graph_replay_identical():
    descs, ae, al, be, bl, total = W.mixed(12, 1500)
    got, _ = run_batch(descs, ae, al, be, bl, total, graph=True)
    check_mixed(descs, ae, al, be, bl, total, got)


def test_batch_equals_elementwise():
    """Same device code: a uniform slice run through the batch equals fpa_mul/fpa_div."""
    n, count = 128, 256
    for op in (2, 3, 4):
        ops = np.full(count, op, np.uint8)
        limbs = np.full(count, n, np.uint16)
        descs, ae, al, be, bl, total = W.mixed(20 + op, count, ops=ops, limbs=limbs)
        got, _ = run_batch(descs, ae, al, be, bl, total)
        A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
        A.to_device(ae, al.reshape(count, n)); B.to_device(be, bl.reshape(count, n))
        fn = {2: fpa.fpa_mul, 3: fpa.fpa_div}.get(op)
        rc = fn(R, A, B, 3) if fn else fpa.fpa_sqrt(R, A, 3)
        assert rc == 0
        re_, rl = R.to_host()
        assert mismatches(re_, rl, got[0], got[1].reshape(count, n)).size == 0


def test_batch_rejects_bad_descriptors():
    descs, *_ = W.mixed(1, 4)
    bad = descs.copy(); bad["limbs"][0] = 0
    with pytest.raises(fpa.FpaError):
        fpa.Batch(bad)
    bad = descs.copy(); bad["op"][1] = 9
    with pytest.raises(fpa.FpaError):
        fpa.Batch(bad)
    empty = fpa.Batch(descs[:0])
    assert empty.run(0, 0, 0, 0) == 0
    empty.destroy()


def config_runs(cfg, op):
    """16: add/sub/mul, 17: add/sub, 18 and 19: mul/div/sqrt, the others every operation"""
    if cfg >= 18:
        return op in (2, 3, 4)
    return cfg < 16 or op <= (2 if cfg == 16 else 1)


@pytest.mark.parametrize("cfg", range(20))
def test_every_configuration(cfg):
    """Force each configuration through the per-op table and check exactness at a few
    sizes it can hold (with several block pairs per lane: sizes that need one, two and all
    of a lane's pairs)."""
    lanes, tile, pairs = fpa.configs()[cfg]
    cap = lanes * tile * pairs
    rng = np.random.default_rng(cfg)
    for n in sorted({1, 3, lanes * tile + 1, cap // 2 + 1, cap - 1, cap} - {0}):
        if n < 1 or n > min(cap, 512):
            continue
        ae, al = W.uniform(rng, 64, n, -200, 200)
        be, bl = W.uniform(rng, 64, n, -200, 200)
        for op in range(5):
            if not config_runs(cfg, op):
                assert fpa.set_op_config(op, n, cfg) != 0
                continue
            assert fpa.set_op_config(op, n, cfg) == 0
            a2 = ae & ~np.uint32(1) if op == 4 else ae
            A, B, R = fpa.FpaArray(64, 32 * n), fpa.FpaArray(64, 32 * n), fpa.FpaArray(64, 32 * n)
            A.to_device(a2, al); B.to_device(be, bl)
            fn = [fpa.fpa_add, fpa.fpa_sub, fpa.fpa_mul, fpa.fpa_div, None][op]
            rc = fn(R, A, B, 3) if fn else fpa.fpa_sqrt(R, A, 3)
            assert rc == 0
            got = R.to_host()
            exp = oracle.run(op, n, 3, a2, al, be, bl)
            assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0, (cfg, op, n)
            assert fpa.set_op_config(op, n, -1) == 0
