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
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


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
        data[op] = W.config2(op, seed + i, count=count, n=N_LIMBS)
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
            "config": {"workload": "4096-bit mul/div/sqrt (config 2)", "limbs": N_LIMBS, "sample_ops":
                       sum(min(CPU_SAMPLE[o], count) for o in OPS), "mode": "ties_to_even"},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


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
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ops_per_step = len(OPS) * count
    value = world * ops_per_step * args.steps / (total_ms / 1e3)
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

    e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    if world > 1:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    h2d = sum((2 if op != "sqrt" else 1) * count * (4 + 4 * n) for op in OPS)
    d2h = len(OPS) * count * (4 + 4 * n)
    e2e_val = world * ops_per_step * args.steps / (e2e_ms / 1e3)

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
    cpu = None
    if not args.no_cpu:
        cpu = cpu_leg(data, gpu_results, os.cpu_count() or 1)
        m = mpfr_leg(data, 1)
        if m is not None:
            cpu["mpfr_single_thread"] = m
    line = {"metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "4096-bit mul/div/sqrt (config 2)", "limbs": n, "operands_per_op": count,
                       "near_halfway_frac": 0.05, "mode": "ties_to_even", "step": "fpa_mul+fpa_div+fpa_sqrt",
                       "l2": "inputs 541 MB per operand array, larger than L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "e2e": {"value": e2e_val, "unit": "ops/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "fpa_copy_array_to_device + fpa_mul/div/sqrt + fpa_copy_array_to_host (pinned)"},
            "gpu_launches": len(OPS) * args.steps}
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
