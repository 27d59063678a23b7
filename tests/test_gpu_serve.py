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
