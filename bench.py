"""Benchmark: bit-exact 4096-bit fpa mul/div/sqrt throughput on GB300.

Workload (the reference metric's configuration, 4096-bit mul/div/sqrt): 2^20 operands of
128 limbs per operation, seeded synthetic data, mantissas uniform, exponents in
[-1000, 1000], 5% near-halfway (mul) / near-exact (div, sqrt) cases, ties-to-even.
One step = fpa_mul + fpa_div + fpa_sqrt over the whole batch (3 * 2^20 operations).
Inputs (541 MB per operand array) are larger than L2, so no flush is needed.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]

--impl reference times the reference path's CPU implementation (the oracle's C
restatement) on the host cores over a bounded sample of the same workload.
Under torchrun each rank runs an independent replica (the operation shards trivially by
index with no exchange); rank 0 prints one JSON line.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_LIMBS = 128
COUNT = 1 << 20
OPS = ("mul", "div", "sqrt")
OP_CODE = {"add": 0, "sub": 1, "mul": 2, "div": 3, "sqrt": 4}
# algorithmic 32x32->64 limb products per operation (schoolbook-equivalent):
# mul n^2, div n^2, sqrt n^2/2; two integer multiply-adds (lo, hi) per product
PRODUCTS = {"mul": N_LIMBS ** 2, "div": N_LIMBS ** 2, "sqrt": N_LIMBS ** 2 // 2}
METRIC = "bit-exact mul/div/sqrt ops/s at 4096 bits (2^20 operands each)"
CPU_SAMPLE = {"mul": 131072, "div": 131072, "sqrt": 32768}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--count", type=int, default=COUNT)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 1024-bit, mixed-batch, chained and served measurements")
    ap.add_argument("--quick-extras", action="store_true", help="smaller extra workloads")
    ap.add_argument("--extras", default=",".join(EXTRAS), help="comma-separated extra workloads to run")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(ms, device):
    """The slowest replica's time: every rank contributes its own timed region, all get the
    maximum (a collective on `device`; "cuda" under NCCL, "cpu" under gloo)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, ops_per_step, steps, max_ms):
    """Whole-job throughput of `world` replicas that each ran `steps` steps of `ops_per_step`
    operations, the slowest taking `max_ms`."""
    return world * ops_per_step * steps / (max_ms / 1e3)


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def make_inputs(count, seed=20240):
    from cubigfloat_gb300 import workloads as W
    data = {}
    for i, op in enumerate(OPS):
        data[op] = W.workload_4096(op, seed + i, count=count, n=N_LIMBS)
    return data


def cpu_leg(data, gpu_results, threads):
    """Oracle (C restatement, all host threads) on a bounded sample of the same operands;
    also checks the GPU results on that sample."""
    import oracle
    total_ops, total_s, exact = 0, 0.0, True
    per = {}
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        k = min(CPU_SAMPLE[op], len(ae))
        t0 = time.perf_counter()
        re_, rl = oracle.run(OP_CODE[op], N_LIMBS, 3, ae[:k], al[:k], be[:k], bl[:k], threads=threads)
        dt = time.perf_counter() - t0
        total_ops += k
        total_s += dt
        per[op] = k / dt
        if gpu_results is not None:
            ge, gl = gpu_results[op]
            val = re_ > 8
            ok = np.array_equal(ge[:k], re_) and np.array_equal(gl[:k][val], rl[val])
            exact = exact and ok
    return {"value": total_ops / total_s, "unit": "ops/s", "cores": threads, "kind": "port",
            "sample": "first {} mul, {} div, {} sqrt operands of the same 4096-bit workload, ties-to-even".format(
                CPU_SAMPLE["mul"], CPU_SAMPLE["div"], CPU_SAMPLE["sqrt"]),
            "per_op_ops_s": {k: round(v, 1) for k, v in per.items()},
            "gpu_sample_bit_exact": exact if gpu_results is not None else None}


def mpfr_leg(data, threads):
    """MPFR 4.2.1 (the reference's test oracle) on the host, single thread, same sample."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    try:
        import gold
        if not gold.available():
            return None
    except Exception:
        return None
    per, tot_ops, tot_s = {}, 0, 0.0
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        k = min(CPU_SAMPLE[op], len(ae))
        t0 = time.perf_counter()
        gold.run(OP_CODE[op], N_LIMBS, 3, ae[:k], al[:k], be[:k], bl[:k])
        dt = time.perf_counter() - t0
        per[op] = k / dt
        tot_ops += k
        tot_s += dt
    return {"value": tot_ops / tot_s, "unit": "ops/s", "cores": 1, "kind": "mpfr",
            "per_op_ops_s": {k: round(v, 1) for k, v in per.items()}, "version": gold.version()}


def load_traffic():
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    count = min(args.count, max(CPU_SAMPLE.values()))
    data = make_inputs(count)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_leg(data, None, threads)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_leg(data, None, threads)["value"])
    v = float(np.median(vals))
    cb = cpu_leg(data, None, threads)
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "ops/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "4096-bit mul/div/sqrt, 2^20 operands each", "limbs": N_LIMBS, "sample_ops":
                       sum(min(CPU_SAMPLE[o], count) for o in OPS), "mode": "ties_to_even"},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def hbm_peak():
    """Measured copy bandwidth of this GPU model (GB/s) and where it came from."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (STREAM-style copy)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (no measured copy bandwidth on this machine)"


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _timed(torch, fn, reps=3):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def extra_add_mul_1024(fpa, torch, count=1 << 22):
    """1024-bit add and mul (the 1024-bit workload's shape: uniform mantissas, e in [-64, 64],
    random signs) over 2^22 pairs so that the operands (554 MB each) exceed L2; add is
    HBM-bound, so its roofline is bytes moved per second against the copy bandwidth."""
    from cubigfloat_gb300 import workloads as W
    n = 32
    (ae, al), (be, bl) = W.workload_1024(11, count=count, n=n)
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    A.to_device(ae, al)
    B.to_device(be, bl)
    out = {}
    peak, src = hbm_peak()
    for name, fn in (("add", fpa.fpa_add), ("mul", fpa.fpa_mul)):
        ms = _timed(torch, lambda: fn(R, A, B, fpa.fpa_round_ties_to_even))
        rec = {"ops_s": count / (ms / 1e3), "ms": ms}
        if name == "add":
            gbs = 3 * count * (4 + 4 * n) / (ms / 1e3) / 1e9
            rec.update({"hbm_gbs": gbs, "hbm_peak_gbs": peak, "hbm_frac": gbs / peak, "peak_source": src})
        out[name] = rec
    del A, B, R
    return {"workload": f"1024-bit add and mul, {count} pairs, ties-to-even", **out}


def extra_batched(fpa, torch, count):
    """Mixed batch: `count` ops 30/20/30/10/10 add/sub/mul/div/sqrt, precision log-uniform in
    256..16384 bits, one CUDA-graph launch of the persistent class kernels, against plain
    per-(op, precision) elementwise launches over the same operands regrouped contiguously;
    both results must be bit-identical."""
    from cubigfloat_gb300 import workloads as W
    descs, ae, al, be, bl, total = W.mixed(303, count)
    d_ae, d_al, d_be, d_bl = (_dev(torch, x) for x in (ae, al, be, bl))
    d_re = torch.zeros(count, dtype=torch.int32, device="cuda")
    d_rl = torch.zeros(total, dtype=torch.int32, device="cuda")
    b = fpa.Batch(descs)
    ptrs = (d_re.data_ptr(), d_rl.data_ptr(), d_ae.data_ptr(), d_al.data_ptr(), d_be.data_ptr(), d_bl.data_ptr())
    ms_run = _timed(torch, lambda: b.run(*ptrs))
    assert b.capture(*ptrs) == 0
    ms_graph = _timed(torch, lambda: b.graph_launch())
    # plain: group (op, limbs) contiguously, one elementwise launch per group
    order = np.lexsort((descs["limbs"], descs["op"]))
    ops_s, lim_s = descs["op"][order], descs["limbs"][order]
    starts = np.flatnonzero(np.r_[True, (ops_s[1:] != ops_s[:-1]) | (lim_s[1:] != lim_s[:-1])])
    ends = np.r_[starts[1:], count]
    lens = lim_s.astype(np.int64)
    a_sel = np.repeat(descs["a_off"][order].astype(np.int64), lens) + (
        np.arange(lens.sum()) - np.repeat(np.cumsum(lens) - lens, lens))
    b_sel = np.repeat(descs["b_off"][order].astype(np.int64), lens) + (
        np.arange(lens.sum()) - np.repeat(np.cumsum(lens) - lens, lens))
    r_sel = np.repeat(descs["r_off"][order].astype(np.int64), lens) + (
        np.arange(lens.sum()) - np.repeat(np.cumsum(lens) - lens, lens))
    g_al, g_bl = _dev(torch, al[a_sel]), _dev(torch, bl[b_sel])
    g_ae, g_be = _dev(torch, ae[order]), _dev(torch, be[order])
    g_re = torch.zeros(count, dtype=torch.int32, device="cuda")
    g_rl = torch.zeros(int(lens.sum()), dtype=torch.int32, device="cuda")
    limb_pos = np.r_[0, np.cumsum(lens)]
    groups = [(int(ops_s[s]), int(lim_s[s]), int(e - s), int(limb_pos[s]), int(s)) for s, e in zip(starts, ends)]

    def plain():
        for op, n, c, lo, eo in groups:
            rc = fpa.elementwise(op, 32 * n, c, 3, g_re.data_ptr() + 4 * eo, g_rl.data_ptr() + 4 * lo,
                                 g_ae.data_ptr() + 4 * eo, g_al.data_ptr() + 4 * lo, g_be.data_ptr() + 4 * eo,
                                 g_bl.data_ptr() + 4 * lo)
            assert rc == 0, rc
    ms_plain = _timed(torch, plain)
    re_b, rl_b = d_re.cpu().numpy(), d_rl.cpu().numpy()
    re_p, rl_p = g_re.cpu().numpy(), g_rl.cpu().numpy()
    same_e = np.array_equal(re_b[order], re_p)
    valued = np.repeat(re_p > 8, lens)             # limbs are defined for ordinary values only
    same_l = np.array_equal(rl_b[r_sel][valued], rl_p[valued])
    tasks, _ = b.info()
    b.destroy()
    return {"workload": f"{count} mixed ops (add/sub/mul/div/sqrt 30/20/30/10/10), 256..16384 bits log-uniform",
            "ops_s_graph": count / (ms_graph / 1e3), "ms_graph": ms_graph, "ms_run": ms_run,
            "ops_s_plain_launches": count / (ms_plain / 1e3), "ms_plain": ms_plain, "plain_launches": len(groups),
            "speedup_vs_plain": ms_plain / ms_graph, "tasks_per_class": tasks,
            "bit_identical_to_plain": bool(same_e and same_l)}


def extra_chains(fpa, torch, dots=10000, length=1024, newtons=10000):
    """Dot products (acc += x*y, each step rounded, 2048 bits) and Newton sqrt
    (y <- (y + x/y)/2, 8 iterations at 8192 bits, x in [1, 2)), one launch each."""
    from cubigfloat_gb300 import workloads as W
    rng = np.random.default_rng(4)
    n = 64
    xe, xl = W.uniform(rng, dots * length, n, -64, 64)
    ye, yl = W.uniform(rng, dots * length, n, -64, 64)
    dxe, dxl, dye, dyl = (_dev(torch, x) for x in (xe, xl, ye, yl))
    del xl, yl
    re_ = torch.zeros(dots, dtype=torch.int32, device="cuda")
    rl = torch.zeros(dots * n, dtype=torch.int32, device="cuda")
    ms_dot = _timed(torch, lambda: fpa.dot(2048, dots, length, 3, re_.data_ptr(), rl.data_ptr(), dxe.data_ptr(),
                                           dxl.data_ptr(), dye.data_ptr(), dyl.data_ptr()), reps=2)
    del dxe, dxl, dye, dyl
    torch.cuda.empty_cache()
    n2 = 256
    xl2 = rng.integers(0, 1 << 32, size=(newtons, n2), dtype=np.uint64).astype(np.uint32)
    xl2[:, -1] |= np.uint32(0x80000000)
    xe2 = W.exp_word(np.ones(newtons, dtype=np.int64), 0)
    y0 = np.zeros((newtons, n2), np.uint32)
    y0[:, -1] = 0xC0000000
    dxe2, dxl2 = _dev(torch, xe2), _dev(torch, xl2)
    dye2, dyl2 = _dev(torch, xe2), _dev(torch, y0)
    d_y0 = _dev(torch, y0)

    def newton():
        dyl2.copy_(d_y0)
        dye2.copy_(dxe2)
        assert fpa.newton_sqrt(8192, newtons, 8, 3, dye2.data_ptr(), dyl2.data_ptr(), dxe2.data_ptr(),
                               dxl2.data_ptr()) == 0
    ms_newton = _timed(torch, newton, reps=2)
    return {"dot": {"workload": f"{dots} dot products of length {length} at 2048 bits",
                    "ms": ms_dot, "mul_add_steps_s": dots * length / (ms_dot / 1e3)},
            "newton_sqrt": {"workload": f"{newtons} Newton sqrt(x), 8 iterations at 8192 bits",
                            "ms": ms_newton, "iterations_s": newtons * 8 / (ms_newton / 1e3)}}


def extra_served(fpa, njobs=400, rates=(1000.0, 4000.0, 16000.0, None)):
    """Served request stream: jobs of 1..4096 ops at one precision from {512, 1024, 4096,
    16384} bits, Poisson arrivals at each rate (None = all jobs at once), through the
    continuous-batching request loop and through plain per-job launches."""
    from cubigfloat_gb300 import workloads as W
    rng = np.random.default_rng(5)
    jobs = [W.served_job(rng) for _ in range(njobs)]
    total_ops = sum(len(j[1]) for j in jobs)
    out = {"workload": f"{njobs} jobs, {total_ops} ops, sizes log-uniform 1..4096, op mix 30/20/30/10/10"}
    for rate in rates:
        arr = (W.poisson_arrivals(np.random.default_rng(int(rate or 0)), njobs, rate) if rate
               else np.zeros(njobs))
        rec = {}
        for batching in (True, False):
            srv = fpa.Server(hbm_budget_bytes=2 << 30, max_inflight=4, batching=batching)
            ids = []
            t0 = time.perf_counter()
            for j, ta in zip(jobs, arr):
                d = ta - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                ids.append(srv.submit(*j)[0])
            for i in ids:
                assert srv.wait(i, 300000) == 0
            tt = [srv.times(i) for i in ids]
            lat = np.array([(t[2] - t[0]) / 1e6 for t in tt])
            span = (max(t[2] for t in tt) - min(t[0] for t in tt)) / 1e9
            st = srv.stats()
            rec["batched" if batching else "plain"] = {
                "ops_s": total_ops / span, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "batches": int(st["batches"]),
                "peak_bytes": int(st["peak_bytes"])}
            srv.destroy()
        rec["throughput_vs_plain"] = rec["batched"]["ops_s"] / rec["plain"]["ops_s"]
        out["burst" if rate is None else f"poisson_{int(rate)}_jobs_s"] = rec
    return out


EXTRAS = ("add_mul_1024", "batched_mixed", "chains", "served")


def run_extras(fpa, torch, quick, only=EXTRAS):
    out = {}
    for name, fn in (("add_mul_1024", lambda: extra_add_mul_1024(fpa, torch, 1 << 20 if quick else 1 << 22)),
                     ("batched_mixed", lambda: extra_batched(fpa, torch, 100000 if quick else 1000000)),
                     ("chains", lambda: extra_chains(fpa, torch, dots=1000 if quick else 10000,
                                                     newtons=1000 if quick else 10000)),
                     ("served", lambda: extra_served(fpa, njobs=100 if quick else 400))):
        if name not in only:
            continue
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:                      # reported, never hidden
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 1)
        torch.cuda.empty_cache()
    assert fpa.device_errors() == 0
    return out


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        dist.barrier()
    import cubigfloat_gb300 as fpa

    count = args.count
    data = make_inputs(count, seed=20240 + 17 * rank)
    n = N_LIMBS
    prec = 32 * n
    arrs = {}
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        A, B, R = fpa.FpaArray(count, prec), fpa.FpaArray(count, prec), fpa.FpaArray(count, prec)
        assert A.to_device(ae, al) == 0
        assert B.to_device(be, bl) == 0
        arrs[op] = (A, B, R)
    fns = {"mul": fpa.fpa_mul, "div": fpa.fpa_div, "sqrt": lambda r, a, b, m: fpa.fpa_sqrt(r, a, m)}
    mode = fpa.fpa_round_ties_to_even
    stream = torch.cuda.current_stream()   # the legacy default stream: the library launches there

    def step(ev=None):
        for op in OPS:
            A, B, R = arrs[op]
            if ev is not None:
                ev[op][0].record(stream)
            rc = fns[op](R, A, B, mode)
            if ev is not None:
                ev[op][1].record(stream)
            assert rc == 0, (op, rc)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    lo, hi = fpa.measure_imad_peak()
    clocks = Clocks(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    evs = [{op: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for op in OPS}
           for _ in range(args.steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(args.steps):
        step(evs[s])
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    total_ms = e0.elapsed_time(e1)
    per_op_ms = {op: float(np.mean([evs[s][op][0].elapsed_time(evs[s][op][1]) for s in range(args.steps)]))
                 for op in OPS}
    if world > 1:
        total_ms = max_over_ranks(total_ms, "cuda")
    ops_per_step = len(OPS) * count
    value = job_rate(world, ops_per_step, args.steps, total_ms)
    assert fpa.device_errors() == 0

    # e2e: the C-ABI with host buffers (pinned), copies inside the timed region
    pinned = {}
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        pa = [torch.from_numpy(x).pin_memory() for x in (ae, al, be, bl)]
        pr = [torch.empty(count, dtype=torch.int32).pin_memory(), torch.empty(count * n, dtype=torch.int32).pin_memory()]
        pinned[op] = (pa, pr)
    lib = fpa.lib()
    vp = ctypes.c_void_p

    def e2e_step():
        for op in OPS:
            A, B, R = arrs[op]
            pa, pr = pinned[op]
            assert lib.fpa_copy_array_to_device(A.ref, vp(pa[0].data_ptr()), vp(pa[1].data_ptr())) == 0
            if op != "sqrt":
                assert lib.fpa_copy_array_to_device(B.ref, vp(pa[2].data_ptr()), vp(pa[3].data_ptr())) == 0
            assert fns[op](R, A, B, mode) == 0
            assert lib.fpa_copy_array_to_host(R.ref, vp(pr[0].data_ptr()), vp(pr[1].data_ptr())) == 0

    # The same through the stream-ordered calls of the C ABI: operand copies, the operation
    # and the result copy of each operation on three streams (host-to-device, compute,
    # device-to-host), so that one operation's copies overlap another's compute.
    s_in, s_op, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    done = {op: None for op in OPS}        # compute of the previous step (its inputs are free after)
    drained = {op: None for op in OPS}     # result copy of the previous step (its output is free after)

    def e2e_step_streams():
        for op in OPS:
            A, B, R = arrs[op]
            pa, pr = pinned[op]
            if done[op] is not None:
                s_in.wait_event(done[op])
            assert lib.fpa_copy_array_to_device_async(A.ref, vp(pa[0].data_ptr()), vp(pa[1].data_ptr()),
                                                      vp(s_in.cuda_stream)) == 0
            if op != "sqrt":
                assert lib.fpa_copy_array_to_device_async(B.ref, vp(pa[2].data_ptr()), vp(pa[3].data_ptr()),
                                                          vp(s_in.cuda_stream)) == 0
            e_in = torch.cuda.Event()
            e_in.record(s_in)
            s_op.wait_event(e_in)
            if drained[op] is not None:
                s_op.wait_event(drained[op])
            assert lib.fpa_op_async(OP_CODE[op], R.ref, A.ref, (A if op == "sqrt" else B).ref, mode,
                                    vp(s_op.cuda_stream)) == 0
            done[op] = torch.cuda.Event()
            done[op].record(s_op)
            s_out.wait_event(done[op])
            assert lib.fpa_copy_array_to_host_async(R.ref, vp(pr[0].data_ptr()), vp(pr[1].data_ptr()),
                                                    vp(s_out.cuda_stream)) == 0
            drained[op] = torch.cuda.Event()
            drained[op].record(s_out)

    def timed_e2e(step_fn, start_stream, end_stream):
        step_fn()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(start_stream)
        if start_stream is not stream:
            for st in (s_in, s_op, s_out):
                st.wait_event(g0)
        for _ in range(args.steps):
            step_fn()
        if end_stream is not stream:
            for st in (s_in, s_op):
                end_stream.wait_stream(st)
        g1.record(end_stream)
        torch.cuda.synchronize()
        ms = g0.elapsed_time(g1)
        if world > 1:
            ms = max_over_ranks(ms, "cuda")
        return ms

    e2e_sync_ms = timed_e2e(e2e_step, stream, stream)
    e2e_ms = timed_e2e(e2e_step_streams, s_in, s_out)
    h2d = sum((2 if op != "sqrt" else 1) * count * (4 + 4 * n) for op in OPS)
    d2h = len(OPS) * count * (4 + 4 * n)
    e2e_val = job_rate(world, ops_per_step, args.steps, e2e_ms)
    e2e_sync_val = job_rate(world, ops_per_step, args.steps, e2e_sync_ms)

    gpu_results = None
    if rank == 0 and not args.no_cpu:
        gpu_results = {}
        for op in OPS:
            pa, pr = pinned[op]
            gpu_results[op] = (pr[0].numpy().view(np.uint32), pr[1].numpy().view(np.uint32).reshape(count, n))
    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    dom = max(OPS, key=lambda o: per_op_ms[o])
    alg_imad = 2 * PRODUCTS[dom] * count
    achieved = alg_imad / (per_op_ms[dom] / 1e3) / 1e12
    traffic = load_traffic().get(f"{dom}_n{n}")
    roofline = {"bound": "int-multiply", "kernel": f"k_elementwise<{dom}>, 4096-bit",
                "achieved": round(achieved, 3), "peak": round(lo / 1e12, 3), "unit": "T IMAD/s",
                "frac": round(achieved / (lo / 1e12), 4),
                "peak_source": "measured live: mad.lo.u32 over all SMs (fpa_gb300_measure_imad_peak)",
                "mad_hi_peak": round(hi / 1e12, 3),
                "traffic": traffic,
                "per_op": {op: {"ms": round(per_op_ms[op], 3), "ops_s": round(count / (per_op_ms[op] / 1e3), 1),
                                "imad_frac": round(2 * PRODUCTS[op] * count / (per_op_ms[op] / 1e3) / lo, 4)}
                           for op in OPS}}
    extras = None
    if not args.no_extras and world == 1:
        extras = run_extras(fpa, torch, args.quick_extras, args.extras.split(","))
    cpu = None
    if not args.no_cpu:
        cpu = cpu_leg(data, gpu_results, os.cpu_count() or 1)
        m = mpfr_leg(data, 1)
        if m is not None:
            cpu["mpfr_single_thread"] = m
    line = {"metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "4096-bit mul/div/sqrt, 2^20 operands each", "limbs": n, "operands_per_op": count,
                       "near_halfway_frac": 0.05, "mode": "ties_to_even", "step": "fpa_mul+fpa_div+fpa_sqrt",
                       "l2": "inputs 541 MB per operand array, larger than L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "e2e": {"value": e2e_val, "unit": "ops/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "fpa_copy_array_to_device_async + fpa_op_async + fpa_copy_array_to_host_async "
                           "(pinned host buffers; copy-in, compute and copy-out on three streams)",
                    "sync": {"value": e2e_sync_val, "unit": "ops/s",
                             "api": "fpa_copy_array_to_device + fpa_mul/div/sqrt + fpa_copy_array_to_host "
                                    "(the fpa.h calls, one after another)"}},
            "gpu_launches": len(OPS) * args.steps,
            "extras": extras}
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
