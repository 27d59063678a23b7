"""GPU: the served form.  Jobs of different precisions submitted concurrently are all
correctly rounded (oracle), a job's result is the same alone and in the mix, plain and
batched serving agree, and the HBM budget bounds admission."""
import threading

import numpy as np
import pytest

import cubigfloat_gb300 as fpa
import oracle
from cubigfloat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def oracle_job(job):
    precision, ops, modes, ae, al, be, bl = job
    n = precision // 32
    off = np.arange(len(ops), dtype=np.uint64) * n
    return oracle.run_mixed(ops, np.full(len(ops), n, np.uint16), modes, ae, al, off, be, bl, off, off,
                            len(ops) * n, threads=8)


def same(exp, got):
    ee, el = exp
    ge, gl = got
    if not np.array_equal(ee, ge):
        return False
    n = el.size // max(1, ee.size)
    for i in np.nonzero(ee > 8)[0]:
        if not np.array_equal(el[i * n:(i + 1) * n], gl[i * n:(i + 1) * n]):
            return False
    return True


@pytest.fixture(scope="module", autouse=True)
def clean_errors():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


def run_jobs(server, jobs, threads=1):
    out = [None] * len(jobs)

    def worker(idx):
        for i in idx:
            out[i] = server.submit(*jobs[i])

    chunks = [list(range(t, len(jobs), threads)) for t in range(threads)]
    ts = [threading.Thread(target=worker, args=(c,)) for c in chunks]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for jid, _ in out:
        assert server.wait(jid, 60000) == 0
    return out


def test_served_jobs_are_correctly_rounded():
    rng = np.random.default_rng(1)
    jobs = [W.served_job(rng, max_ops=256) for _ in range(40)]
    srv = fpa.Server(hbm_budget_bytes=256 << 20, max_inflight=3)
    out = run_jobs(srv, jobs, threads=4)
    for job, (jid, res) in zip(jobs, out):
        assert same(oracle_job(job), res)
        t_sub, t_adm, t_done = srv.times(jid)
        assert t_sub <= t_adm <= t_done
    st = srv.stats()
    assert st["jobs"] == 40 and st["failed"] == 0 and st["peak_bytes"] <= st["budget_bytes"]
    srv.destroy()


def test_alone_equals_in_mix():
    rng = np.random.default_rng(2)
    probe = W.served_job(rng, precision=4096, size=300)
    srv = fpa.Server(hbm_budget_bytes=256 << 20, max_inflight=4)
    jid, alone = srv.submit(*probe)
    assert srv.wait(jid, 60000) == 0
    alone = (alone[0].copy(), alone[1].copy())
    others = [W.served_job(rng, max_ops=512) for _ in range(30)]
    mix = others[:15] + [probe] + others[15:]
    out = run_jobs(srv, mix, threads=3)
    in_mix = out[15][1]
    assert np.array_equal(alone[0], in_mix[0]) and np.array_equal(alone[1], in_mix[1])
    assert same(oracle_job(probe), alone)
    assert srv.stats()["batches"] < len(mix) + 1      # jobs were batched together
    srv.destroy()


def test_plain_and_batched_agree():
    rng = np.random.default_rng(3)
    jobs = [W.served_job(rng, max_ops=128) for _ in range(12)]
    a = fpa.Server(hbm_budget_bytes=128 << 20, batching=True)
    b = fpa.Server(hbm_budget_bytes=128 << 20, batching=False)
    ra = run_jobs(a, jobs)
    rb = run_jobs(b, jobs)
    for (_, x), (_, y) in zip(ra, rb):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
    assert b.stats()["batches"] == len(jobs)
    a.destroy(); b.destroy()


def test_budget_rejects_oversized_job():
    rng = np.random.default_rng(4)
    srv = fpa.Server(hbm_budget_bytes=1 << 20, max_inflight=2)     # 512 KB per slot
    big = W.served_job(rng, precision=16384, size=400)              # ~2.5 MB
    with pytest.raises(fpa.FpaError):
        srv.submit(*big)
    small = W.served_job(rng, precision=512, size=10)
    jid, res = srv.submit(*small)
    assert srv.wait(jid, 60000) == 0 and same(oracle_job(small), res)
    srv.destroy()


def test_device_resident_chain_matches_oracle():
    """A chain of jobs whose operands are earlier jobs' kept results: x = a*b (kept, not
    copied out), y = x + c (kept), z = y / a (copied out).  z is submitted right behind y, so
    its source is still in flight when it is admitted (the copy waits on the GPU).  x cannot
    be released while y is pending.  Every kept result read back, and z, equals the oracle's
    step-by-step values, and the cost account has all four parts."""
    n, count = 64, 300
    prec = 32 * n
    rng = np.random.default_rng(77)
    ae, al = W.uniform(rng, count, n, -40, 40)
    be, bl = W.uniform(rng, count, n, -40, 40)
    ce, cl = W.uniform(rng, count, n, -40, 40)
    modes = rng.integers(0, 5, size=count).astype(np.uint8)
    off = np.arange(count, dtype=np.uint64) * n
    lim = np.full(count, n, np.uint16)
    step = lambda op, xe, xl, ye, yl: oracle.run_mixed(np.full(count, op, np.uint8), lim, modes, xe, xl, off,
                                                       ye, yl, off, off, count * n, threads=8)
    xe, xl = step(2, ae, al.ravel(), be, bl.ravel())
    ye, yl = step(0, xe, xl, ce, cl.ravel())
    ze, zl = step(3, ye, yl, ae, al.ravel())
    srv = fpa.Server(hbm_budget_bytes=256 << 20, max_inflight=2, resident_bytes=64 << 20)
    try:
        j1, _ = srv.submit(prec, np.full(count, 2, np.uint8), modes, ae, al, be, bl, keep=True, copy_out=False)
        assert srv.wait(j1, 60000) == 0
        j2, _ = srv.submit(prec, np.zeros(count, np.uint8), modes, None, None, ce, cl, a_from=j1, keep=True,
                           copy_out=False)
        assert srv.release(j1) != 0                  # y, which reads x, is still pending
        j3, (re3, rl3) = srv.submit(prec, np.full(count, 3, np.uint8), modes, None, None, ae, al, a_from=j2)
        assert srv.wait(j3, 60000) == 0
        assert same((xe, xl), srv.read(j1))
        assert same((ye, yl), srv.read(j2))
        assert same((ze, zl), (re3, rl3))
        assert srv.release(j3) == 0 and srv.release(j2) == 0 and srv.release(j1) == 0
        c = srv.costs()
        assert all(v > 0 for v in c.values()), c
    finally:
        srv.destroy()


def test_resident_store_full_is_refused():
    n, count = 32, 1000
    rng = np.random.default_rng(3)
    ae, al = W.uniform(rng, count, n, -5, 5)
    srv = fpa.Server(hbm_budget_bytes=64 << 20, max_inflight=1, resident_bytes=1 << 16)
    try:
        with pytest.raises(fpa.FpaError):
            srv.submit(32 * n, np.full(count, 4, np.uint8), None, ae & ~np.uint32(1), al, keep=True)
    finally:
        srv.destroy()
