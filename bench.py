"""Benchmark: bit-exact 4096-bit fpa mul/div/sqrt throughput on GB300.

Workload (the reference metric's configuration, 4096-bit mul/div/sqrt): 2^20 operands of
128 limbs per operation, seeded synthetic data, mantissas uniform, exponents in
[-1000, 1000], 5% near-halfway (mul) / near-exact (div, sqrt) cases, ties-to-even.
One step = fpa_mul + fpa_div + fpa_sqrt over the whole batch (3 * 2^20 operations).
Inputs (541 MB per operand array) are larger than L2, so no flush is needed.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]

After the timed region every result of the step is checked bit-exact against the oracle
(the exact-integer C restatement, on all host cores), which also gives the CPU baseline;
MPFR runs on a sample beside it.  The other workloads (1024-bit add/mul, the 10^6-op mixed
batch, the chains, the served stream, the reference's own kernels) are measured and
checked in `extras`.

--impl reference times the reference path's CPU implementation (the oracle's C
restatement; the reference itself has none) on the host cores over a bounded sample of the
same workload, one third each mul, div and sqrt like the GPU step.
Under torchrun each rank runs an independent replica (the operation shards trivially by
index with no exchange); rank 0 prints one JSON line.
"""
import argparse
import ctypes
import hashlib
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
REF_SAMPLE = 32768          # reference arm: operands per operation per step (mul:div:sqrt = 1:1:1)
MPFR_SAMPLE = 16384         # MPFR: operands per operation (1:1:1), split over the host cores


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


def canonical(e, l):
    """Result arrays with the limbs of class results zeroed (those limbs are unspecified)."""
    e = np.ascontiguousarray(e, dtype=np.uint32)
    l = np.array(l, dtype=np.uint32).reshape(e.size, -1)
    l[e <= 8] = 0
    return e, l


def sha256_of(e, l):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(e, dtype=np.uint32).tobytes())
    h.update(np.ascontiguousarray(l, dtype=np.uint32).tobytes())
    return h.hexdigest()


def equal_mix_rate(rates):
    """ops/s of a step doing the same number of each operation, from per-operation rates"""
    return len(rates) / sum(1.0 / r for r in rates)


def cpu_leg(data, gpu_results, threads, count=None):
    """The oracle (exact-integer C restatement, `threads` host threads) over the first `count`
    operands of each operation (all by default) -- the CPU baseline at the GPU step's 1:1:1
    mix -- and, when GPU results are given, the bit-exact check of every one of them."""
    import oracle
    per, secs, exact, shas = {}, {}, {}, {}
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        k = len(ae) if count is None else min(count, len(ae))
        t0 = time.perf_counter()
        re_, rl = oracle.run(OP_CODE[op], N_LIMBS, 3, ae[:k], al[:k], be[:k], bl[:k], threads=threads)
        dt = time.perf_counter() - t0
        per[op], secs[op] = k / dt, dt
        if gpu_results is not None:
            ge, gl = canonical(gpu_results[op][0][:k], gpu_results[op][1][:k])
            oe, ol = canonical(re_, rl)
            exact[op] = bool(np.array_equal(ge, oe) and np.array_equal(gl, ol))
            shas[op] = sha256_of(oe, ol) if exact[op] else {"oracle": sha256_of(oe, ol), "gpu": sha256_of(ge, gl)}
    k = len(data[OPS[0]][0][0]) if count is None else count
    cpu = {"value": equal_mix_rate(list(per.values())), "unit": "ops/s", "cores": threads, "kind": "port",
           "sample": ("all 2^20 operands of each of mul, div, sqrt" if count is None else
                      f"the first {k} operands of each of mul, div, sqrt") +
                     " of the same 4096-bit workload, ties-to-even, one third each (the GPU step's mix)",
           "seconds": round(sum(secs.values()), 2),
           "per_op_ops_s": {o: round(v, 1) for o, v in per.items()}}
    check = None
    if gpu_results is not None:
        check = {"ok": all(exact.values()), "checked_ops": 3 * k, "of_ops": 3 * len(data[OPS[0]][0][0]),
                 "against": "oracle (exact integers; pinned to MPFR 4.2.1)", "per_op": exact,
                 "sha256": shas}
    return cpu, check


def mpfr_leg(data, gpu_results, threads, count=MPFR_SAMPLE):
    """MPFR 4.2.1 (the reference's test oracle) on the host cores: the first `count` operands
    of each operation split into `threads` chunks run concurrently; also checks the GPU
    results on that sample against MPFR."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    try:
        import gold
        if not gold.available():
            return None
    except Exception:
        return None
    from concurrent.futures import ThreadPoolExecutor
    per, exact = {}, True
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        k = min(count, len(ae))
        bounds = np.linspace(0, k, threads + 1).astype(int)
        parts = [(lo, hi) for lo, hi in zip(bounds[:-1], bounds[1:]) if hi > lo]
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=len(parts)) as ex:
            res = list(ex.map(lambda lh: gold.run(OP_CODE[op], N_LIMBS, 3, ae[lh[0]:lh[1]], al[lh[0]:lh[1]],
                                                  be[lh[0]:lh[1]], bl[lh[0]:lh[1]]), parts))
        per[op] = k / (time.perf_counter() - t0)
        if gpu_results is not None:
            me, ml = canonical(np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res]))
            ge, gl = canonical(gpu_results[op][0][:k], gpu_results[op][1][:k])
            exact = exact and bool(np.array_equal(me, ge) and np.array_equal(ml, gl))
    return {"value": equal_mix_rate(list(per.values())), "unit": "ops/s", "cores": threads, "kind": "mpfr",
            "sample": f"the first {count} operands of each of mul, div, sqrt, one third each",
            "per_op_ops_s": {o: round(v, 1) for o, v in per.items()}, "version": gold.version(),
            "gpu_sample_bit_exact_vs_mpfr": exact if gpu_results is not None else None}


# The one-thread kernels (configuration 18: k_tmul, k_tnewton in fpa_thread_newton.cu) form
# fewer limb products than the schoolbook basis counts: mul a short product above the
# rounding limb, div and sqrt Newton levels and a Karp-Markstein step whose products are
# restricted to the limbs that are read, sqrt's square on its symmetric half.
# tile_products() mirrors their 8x8-tile block ranges (tprod: output blocks [cb_lo, cb_hi)
# of an lx x ly product, block cb spanning x blocks max(0, cb-My) .. min(cb, Mx-1); 64
# products a tile, 28 or 36 for an edge tile whose window is half zero guard, 32 for a tile of
# x's last block when it holds 1 to 4 limbs; tprod2, mul's: two
# blocks per pass; tsqr: the tiles below the diagonal), so that the roofline can also report
# how busy the multiplier is on the products the first pass executes (deferred operations
# excluded).
KERNELS = {"mul": "k_tmul<128>", "div": "k_tnewton<3 (div), 128>", "sqrt": "k_tnewton<4 (sqrt), 128>"}


def _tprod(lx, ly, cb_lo, cb_hi):
    mx, my = (lx + 7) // 8, (ly + 7) // 8
    half_rows = 0 < lx % 8 <= 4
    total = 0
    for cb in range(cb_lo, min(mx + my, cb_hi)):
        i0, i1 = max(0, cb - my), min(cb, mx - 1)
        # a first tile in the guard keeps 28 products, a last tile 36
        total += 64 * (i1 - i0 + 1) - (36 if cb >= my else 0) - (28 if i1 == cb else 0)
        iend, i = (i1 if i1 == cb else i1 + 1), i0 + (1 if cb >= my else 0)
        if half_rows and iend == mx and i < iend:      # x's last block, rows 4..7 zero
            total -= 32
    return total


def _levels(n):
    out, k = [n], n
    while k > 1:
        p = (k + 2) // 2
        k = k - 1 if p >= k else p
        out.append(k)
    return out[::-1]


def _tprod2(lx, ly, cb_lo, cb_hi):
    """Limb products of tprod2 (two output blocks per pass): 128 per tile of both blocks, 28
    and 36 for the lone half tiles, 64 per tile of a last unpaired block."""
    mx, my = (lx + 7) // 8, (ly + 7) // 8
    mo, cb, total = min(mx + my, cb_hi), cb_lo, 0
    while cb + 1 < mo:
        i0a, i1a = max(0, cb - my), min(cb, mx - 1)
        i0b, i1b = max(0, cb + 1 - my), min(cb + 1, mx - 1)
        total += (28 if i0a < i0b else 0) + 128 * (i1a - i0b + 1) + (36 if i1b > i1a else 0)
        cb += 2
    if cb < mo:
        total += 64 * (min(cb, mx - 1) - max(0, cb - my) + 1)
    return total


def _tsqr(lx, cb_hi):
    """Limb products of tsqr (x*x, output blocks [0, cb_hi)): the tiles below the diagonal
    tile once (doubled afterwards), the diagonal tile's a < b pairs (16 for even blocks, 48
    for odd) and its 4 squares."""
    mx = (lx + 7) // 8
    total = 0
    for cb in range(0, min(2 * mx, cb_hi)):
        i0, d = max(0, cb - mx), cb // 2
        total += 64 * (d - i0) - (36 if (cb >= mx and i0 < d) else 0) + (52 if cb & 1 else 20)
    return total


def tile_products(op, n):
    """Limb products the first pass of one operation at n limbs executes in its tile products
    (the one-thread register levels below them are not counted)."""
    blk = lambda keep: max(0, keep - 2) // 8
    big = 1 << 20
    if op == "mul":
        return _tprod2(n, n, blk(n - 1), big)
    lv = _levels(n)
    e = 1
    while e < len(lv) - 1 and lv[e] <= 9:          # one-thread register levels
        e += 1
    prods = 0
    for li in range(e, len(lv) - 1):
        k, kp = lv[li - 1], lv[li]
        lt = kp - k + 3
        if op == "div":
            prods += _tprod(kp, k + 1, blk(k - 1), (k + kp) // 8 + 1)
            prods += _tprod(k + 1, lt, blk(k + 1), (k + 1 + lt + 7) // 8)
        else:
            j = k - 2 if k > 2 else 0
            l1, L, off = kp + k + 1 - j, kp + 2 * k - j, 2 * k - 1 - j
            prods += _tprod(kp, k + 1, blk(j), (j + l1 + 7) // 8)
            prods += _tprod(l1, k + 1, blk(off), L // 8 + 1)
            prods += _tprod(k + 1, lt, blk(k + 1), big)
    h = lv[-2]
    m = n + 2 - h
    if op == "div":
        dlen, sh = m + 2, n - h - 1
        prods += _tprod(m + 1, h + 1, blk(h + 1), (h + m + 9) // 8)
        prods += _tprod(m + 1, n, blk(sh), (sh + dlen + 7) // 8)
        prods += _tprod(dlen, h + 1, blk(h + 2), (dlen + h + 8) // 8)
    else:
        dlen, ssh = m + 3, 2 * h - n
        prods += _tprod(m + 1, h + 1, blk(h + 1), (h + m + 9) // 8)
        prods += _tsqr(m + 1, (dlen - ssh + 7) // 8)
        prods += _tprod(dlen, h + 1, blk(h + 3), big)
    return prods


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
    count = min(args.count, REF_SAMPLE)
    data = make_inputs(count)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_leg(data, None, threads, count)
    steps = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cb, _ = cpu_leg(data, None, threads, count)
        steps.append((time.perf_counter() - t0, cb))
    ms_step = float(np.median([t for t, _ in steps])) * 1e3
    v = len(OPS) * count / (ms_step / 1e3)
    cb = dict(steps[-1][1])
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "ops/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "4096-bit mul/div/sqrt, 2^20 operands each", "limbs": N_LIMBS,
                       "step": f"the first {count} operands of each of mul, div, sqrt (1:1:1, as the GPU step)",
                       "sample_ops": len(OPS) * count, "mode": "ties_to_even"},
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


def extra_add_mul_1024(fpa, torch, roofline_count=1 << 22, count=65536):
    """1024-bit add and mul (uniform mantissas, e in [-64, 64], random signs, ties-to-even).
    At the stated 65,536 pairs the operands (8.6 MB) sit in L2 and a launch takes a few
    microseconds, so that case is timed over back-to-back launches and every result is
    checked bit-exact against the oracle; the HBM roofline of add is measured over 2^22
    pairs (554 MB per operand array, larger than L2)."""
    import oracle
    from cubigfloat_gb300 import workloads as W
    n = 32
    peak, src = hbm_peak()
    out = {}
    (ae, al), (be, bl) = W.workload_1024(11, count=count, n=n)
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    A.to_device(ae, al)
    B.to_device(be, bl)
    stated = {}
    for name, fn in (("add", fpa.fpa_add), ("mul", fpa.fpa_mul)):
        ms = _timed(torch, lambda: fn(R, A, B, fpa.fpa_round_ties_to_even), reps=200)
        ge, gl = canonical(*R.to_host())
        oe, ol = canonical(*oracle.run(OP_CODE[name], n, 3, ae, al, be, bl, threads=os.cpu_count() or 1))
        ok = bool(np.array_equal(ge, oe) and np.array_equal(gl, ol))
        stated[name] = {"ops_s": count / (ms / 1e3), "us_per_launch": ms * 1e3,
                        "bit_exact": {"ok": ok, "checked_ops": count, "sha256": sha256_of(oe, ol)}}
    out["stated_65536_pairs"] = stated
    del A, B, R
    (ae, al), (be, bl) = W.workload_1024(11, count=roofline_count, n=n)
    A, B, R = (fpa.FpaArray(roofline_count, 32 * n), fpa.FpaArray(roofline_count, 32 * n),
               fpa.FpaArray(roofline_count, 32 * n))
    A.to_device(ae, al)
    B.to_device(be, bl)
    for name, fn in (("add", fpa.fpa_add), ("mul", fpa.fpa_mul)):
        ms = _timed(torch, lambda: fn(R, A, B, fpa.fpa_round_ties_to_even))
        rec = {"ops_s": roofline_count / (ms / 1e3), "ms": ms}
        if name == "add":
            gbs = 3 * roofline_count * (4 + 4 * n) / (ms / 1e3) / 1e9
            rec.update({"hbm_gbs": gbs, "hbm_peak_gbs": peak, "hbm_frac": gbs / peak, "peak_source": src})
        out[f"{name}_{roofline_count}_pairs"] = rec
    del A, B, R
    return {"workload": f"1024-bit add and mul, {count} pairs (checked) and {roofline_count} pairs (roofline), "
                        "ties-to-even", **out}


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
    re_b, rl_b = d_re.cpu().numpy().view(np.uint32), d_rl.cpu().numpy().view(np.uint32)
    re_p, rl_p = g_re.cpu().numpy().view(np.uint32), g_rl.cpu().numpy().view(np.uint32)
    same_e = np.array_equal(re_b[order], re_p)
    valued = np.repeat(re_p > 8, lens)             # limbs are defined for ordinary values only
    same_l = np.array_equal(rl_b[r_sel][valued], rl_p[valued])
    tasks, _ = b.info()
    b.destroy()
    # every result of the graph-launched batch against the oracle (checker, all host cores)
    import oracle
    t0 = time.perf_counter()
    oe, ol = oracle.run_mixed(descs["op"], descs["limbs"], descs["mode"], ae, al, descs["a_off"], be, bl,
                              descs["b_off"], descs["r_off"], total, threads=os.cpu_count() or 1)
    check_s = time.perf_counter() - t0
    r_all = np.repeat(descs["r_off"].astype(np.int64), descs["limbs"].astype(np.int64)) + (
        np.arange(int(descs["limbs"].astype(np.int64).sum())) -
        np.repeat(np.cumsum(descs["limbs"].astype(np.int64)) - descs["limbs"].astype(np.int64),
                  descs["limbs"].astype(np.int64)))
    val_all = np.repeat(oe > 8, descs["limbs"].astype(np.int64))
    ok_e = np.array_equal(re_b, oe)
    ok_l = np.array_equal(rl_b[r_all][val_all], ol[r_all][val_all])
    ol_c = ol[r_all].copy()
    ol_c[~val_all] = 0
    return {"workload": f"{count} mixed ops (add/sub/mul/div/sqrt 30/20/30/10/10), 256..16384 bits log-uniform",
            "ops_s_graph": count / (ms_graph / 1e3), "ms_graph": ms_graph, "ms_run": ms_run,
            "ops_s_plain_launches": count / (ms_plain / 1e3), "ms_plain": ms_plain, "plain_launches": len(groups),
            "speedup_vs_plain": ms_plain / ms_graph, "tasks_per_class": tasks,
            "bit_identical_to_plain": bool(same_e and same_l),
            "bit_exact": {"ok": bool(ok_e and ok_l), "checked_ops": count, "against": "oracle",
                          "check_s": round(check_s, 1), "sha256": sha256_of(oe, ol_c)}}


def _stepwise_dot(oracle, n, xe, xl, ye, yl, count, length, threads):
    """acc = RN(acc + RN(x*y)) in order, every step a separate oracle operation"""
    from cubigfloat_gb300 import workloads as W
    xl = xl.reshape(count, length, n)
    yl = yl.reshape(count, length, n)
    xe = xe.reshape(count, length)
    ye = ye.reshape(count, length)
    acc_e = np.full(count, W.CLS_ZERO, np.uint32)
    acc_l = np.zeros((count, n), np.uint32)
    for i in range(length):
        te, tl = oracle.run(2, n, 3, xe[:, i], xl[:, i], ye[:, i], yl[:, i], threads=threads)
        acc_e, acc_l = oracle.run(0, n, 3, acc_e, acc_l, te, tl, threads=threads)
    return acc_e, acc_l


def _stepwise_newton(oracle, n, xe, xl, ye, yl, iters, threads):
    """y <- RN(RN(y + RN(x/y)) * 0.5), every step a separate oracle operation (the halving is
    exact: the exponent word of a value drops by 2)"""
    for _ in range(iters):
        qe, ql = oracle.run(3, n, 3, xe, xl, ye, yl, threads=threads)
        se, sl = oracle.run(0, n, 3, ye, yl, qe, ql, threads=threads)
        ye, yl = np.where(se > 8, se - 2, se).astype(np.uint32), sl
    return ye, yl


def extra_chains(fpa, torch, dots=10000, length=1024, newtons=10000, check_dots=100):
    """Dot products (acc += x*y, each step rounded, 2048 bits) and Newton sqrt
    (y <- (y + x/y)/2, 8 iterations at 8192 bits, x in [1, 2)), one launch each; the first
    `check_dots` dot products and every Newton chain are checked against the same operation
    sequence run step by step in the oracle."""
    import oracle
    from cubigfloat_gb300 import workloads as W
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(4)
    n = 64
    xe, xl = W.uniform(rng, dots * length, n, -64, 64)
    ye, yl = W.uniform(rng, dots * length, n, -64, 64)
    dxe, dxl, dye, dyl = (_dev(torch, x) for x in (xe, xl, ye, yl))
    re_ = torch.zeros(dots, dtype=torch.int32, device="cuda")
    rl = torch.zeros(dots * n, dtype=torch.int32, device="cuda")
    ms_dot = _timed(torch, lambda: fpa.dot(2048, dots, length, 3, re_.data_ptr(), rl.data_ptr(), dxe.data_ptr(),
                                           dxl.data_ptr(), dye.data_ptr(), dyl.data_ptr()), reps=2)
    del dxe, dxl, dye, dyl
    torch.cuda.empty_cache()
    k = min(check_dots, dots)
    t0 = time.perf_counter()
    oe, ol = canonical(*_stepwise_dot(oracle, n, xe[:k * length], xl[:k * length], ye[:k * length],
                                      yl[:k * length], k, length, threads))
    ge, gl = canonical(re_.cpu().numpy().view(np.uint32)[:k], rl.cpu().numpy().view(np.uint32)[:k * n])
    dot_check = {"ok": bool(np.array_equal(oe, ge) and np.array_equal(ol, gl)), "checked_chains": k,
                 "of_chains": dots, "against": "oracle, step by step", "sha256": sha256_of(oe, ol),
                 "check_s": round(time.perf_counter() - t0, 1)}
    del xl, yl
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
    t0 = time.perf_counter()
    oe, ol = canonical(*_stepwise_newton(oracle, n2, xe2, xl2, xe2.copy(), y0, 8, threads))
    ge, gl = canonical(dye2.cpu().numpy().view(np.uint32), dyl2.cpu().numpy().view(np.uint32))
    newton_check = {"ok": bool(np.array_equal(oe, ge) and np.array_equal(ol, gl)), "checked_chains": newtons,
                    "of_chains": newtons, "against": "oracle, step by step", "sha256": sha256_of(oe, ol),
                    "check_s": round(time.perf_counter() - t0, 1)}
    return {"dot": {"workload": f"{dots} dot products of length {length} at 2048 bits",
                    "ms": ms_dot, "mul_add_steps_s": dots * length / (ms_dot / 1e3), "bit_exact": dot_check},
            "newton_sqrt": {"workload": f"{newtons} Newton sqrt(x), 8 iterations at 8192 bits",
                            "ms": ms_newton, "iterations_s": newtons * 8 / (ms_newton / 1e3),
                            "bit_exact": newton_check}}


def extra_reference_gpu(per_op_ms_ours, count=1 << 20):
    """The reference's own kernels (its fpa.cu compiled for sm_103a, launched as its host
    dispatcher does: one warp per number, 128-thread blocks) timed on this GPU with driver
    events over the same 4096-bit operands as the timed step, and over 1024-bit add/mul;
    beside each, our kernel's time on the same work."""
    import oracle
    if not oracle.ref_gpu_available():
        return {"unavailable": "the reference's kernels were not compiled (no reference sources where built)"}
    data = make_inputs(count)
    out = {"launch": "reference fpa_kernel_warp_<op>_<size>, <<<ceil(32*count/128), 128>>>, repeat 3, mean"}
    for op in OPS:
        (ae, al), (be, bl) = data[op]
        _, _, ms = oracle.ref_gpu_run(op, N_LIMBS, 3, ae, al, None if op == "sqrt" else be,
                                      None if op == "sqrt" else bl, repeat=3)
        rec = {"ms": round(ms, 3), "ops_s": count / (ms / 1e3)}
        if op in per_op_ms_ours:
            rec["ours_ms"] = round(per_op_ms_ours[op], 3)
            rec["speedup_ours_over_reference"] = round(ms / per_op_ms_ours[op], 2)
        out[f"{op}_4096"] = rec
    del data
    from cubigfloat_gb300 import workloads as W
    (ae, al), (be, bl) = W.workload_1024(11, count=count, n=32)
    for op in ("add", "mul"):
        _, _, ms = oracle.ref_gpu_run(op, 32, 3, ae, al, be, bl, repeat=3)
        out[f"{op}_1024"] = {"ms": round(ms, 3), "ops_s": count / (ms / 1e3)}
    return out


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
                "peak_bytes": int(st["peak_bytes"]),
                "submit_span_ms": round((max(t[0] for t in tt) - min(t[0] for t in tt)) / 1e6, 3)}
            if batching:
                c = srv.costs()
                rec["batched"]["cost_ms"] = {k[:-3]: round(v / 1e6, 3) for k, v in c.items()}
                rec["batched"]["span_ms"] = round(span * 1e3, 3)
            srv.destroy()
        rec["offered_ops_s"] = total_ops / max(float(arr[-1]), 1e-9) if rate else None
        rec["throughput_vs_plain"] = rec["batched"]["ops_s"] / rec["plain"]["ops_s"]
        out["burst" if rate is None else f"poisson_{int(rate)}_jobs_s"] = rec
    out["batch_graph_same_ops"] = _served_as_one_batch(fpa, jobs, total_ops)
    out["burst_vs_batch_graph"] = out["burst"]["batched"]["ops_s"] / out["batch_graph_same_ops"]["ops_s"]
    out["resident_chain"] = _resident_chain(fpa)
    return out


def _served_as_one_batch(fpa, jobs, total_ops):
    """The served stream's operations as one fpa_batch, operands already on the device, timed
    as a graph launch: the device-side bound the served stream is compared with."""
    import torch
    rows, off = [], 0
    for precision, ops, modes, ae, al, be, bl in jobs:
        n = precision // 32
        for i in range(len(ops)):
            rows.append((ops[i], modes[i], n, off + i * n))
        off += len(ops) * n
    descs = np.zeros(len(rows), dtype=fpa.BATCH_DESC)
    descs["op"] = [r[0] for r in rows]
    descs["mode"] = [r[1] for r in rows]
    descs["limbs"] = [r[2] for r in rows]
    descs["a_off"] = descs["b_off"] = descs["r_off"] = [r[3] for r in rows]
    cat = lambda k: np.concatenate([j[k] for j in jobs])
    d_ae, d_al, d_be, d_bl = (_dev(torch, cat(k)) for k in (3, 4, 5, 6))
    d_re = torch.zeros(len(rows), dtype=torch.int32, device="cuda")
    d_rl = torch.zeros(off, dtype=torch.int32, device="cuda")
    b = fpa.Batch(descs)
    assert b.capture(d_re.data_ptr(), d_rl.data_ptr(), d_ae.data_ptr(), d_al.data_ptr(), d_be.data_ptr(),
                     d_bl.data_ptr()) == 0
    ms = _timed(torch, lambda: b.graph_launch())
    b.destroy()
    return {"ops_s": total_ops / (ms / 1e3), "ms": round(ms, 3)}


def _resident_chain(fpa, steps=8, count=4096, precision=4096):
    """A chain y <- RN(y * x) repeated `steps` times on one job of `count` operations: each
    step a served job reading the previous step's kept result on the device (submitted all at
    once), against the same chain with a host round trip per step (wait, then resubmit with
    the result).  Both end with the same values."""
    from cubigfloat_gb300 import workloads as W
    rng = np.random.default_rng(8)
    n = precision // 32
    xe, xl = W.uniform(rng, count, n, -2, 2)
    ye, yl = W.uniform(rng, count, n, -2, 2)
    ops = np.full(count, 2, np.uint8)
    out = {"workload": f"{steps} chained mul jobs of {count} ops at {precision} bits"}
    srv = fpa.Server(hbm_budget_bytes=1 << 30, max_inflight=2, resident_bytes=256 << 20)
    try:
        t0 = time.perf_counter()
        prev, _ = srv.submit(precision, ops, None, ye, yl.ravel(), xe, xl.ravel(), keep=True, copy_out=False)
        ids = [prev]
        for k in range(1, steps):
            last = k == steps - 1
            prev, res = srv.submit(precision, ops, None, None, None, xe, xl.ravel(), a_from=prev, keep=not last,
                                   copy_out=last)
            ids.append(prev)
        assert srv.wait(prev, 60000) == 0
        dev_ms = (time.perf_counter() - t0) * 1e3
        dev_res = res
        t0 = time.perf_counter()
        ce, cl = ye, yl.ravel()
        for k in range(steps):
            jid, (ce, cl) = srv.submit(precision, ops, None, ce, cl, xe, xl.ravel())
            assert srv.wait(jid, 60000) == 0
        host_ms = (time.perf_counter() - t0) * 1e3
        out.update({"device_resident_ms": round(dev_ms, 3), "host_round_trip_ms": round(host_ms, 3),
                    "same_result": bool(np.array_equal(dev_res[0], ce) and np.array_equal(dev_res[1], cl))})
    finally:
        srv.destroy()
    return out


EXTRAS = ("add_mul_1024", "batched_mixed", "chains", "served", "reference_gpu")


def run_extras(fpa, torch, quick, only=EXTRAS, per_op_ms=None):
    out = {}
    for name, fn in (("add_mul_1024", lambda: extra_add_mul_1024(fpa, torch, 1 << 20 if quick else 1 << 22)),
                     ("batched_mixed", lambda: extra_batched(fpa, torch, 100000 if quick else 1000000)),
                     ("chains", lambda: extra_chains(fpa, torch, dots=1000 if quick else 10000,
                                                     newtons=1000 if quick else 10000,
                                                     check_dots=20 if quick else 100)),
                     ("served", lambda: extra_served(fpa, njobs=100 if quick else 400)),
                     ("reference_gpu", lambda: extra_reference_gpu(per_op_ms or {}, 1 << 18 if quick else 1 << 20))):
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
    prod_peak = fpa.measure_product_peak()
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

    # roofline of the dominant kernel: algorithmic limb products (schoolbook-equivalent:
    # mul n^2, div n^2, sqrt n^2/2 per operation) per CUDA-event second, against the measured
    # limb-product rate of the kernels' own instruction triple
    dom = max(OPS, key=lambda o: per_op_ms[o])
    achieved = PRODUCTS[dom] * count / (per_op_ms[dom] / 1e3) / 1e12
    traffic = load_traffic().get(f"{dom}_n{n}")
    roofline = {"bound": "int-multiply", "kernel": f"{KERNELS[dom]}, 4096-bit (first pass and the deferred "
                                                  "operations' exact pass, one fpa call)",
                "achieved": round(achieved, 4), "peak": round(prod_peak / 1e12, 4), "unit": "T limb products/s",
                "frac": round(achieved / (prod_peak / 1e12), 4),
                "peak_source": "measured live on this GPU: mad.lo.cc + madc.hi.cc + addc per 32x32-bit limb "
                               "product into 96-bit columns, 8-column register tiles on every SM "
                               "(fpa_gb300_measure_product_peak)",
                "basis": f"{PRODUCTS[dom]} limb products per {dom} at {n} limbs x {count} operations per launch",
                "isolated_instruction_peaks": {"mad_lo_T_per_s": round(lo / 1e12, 3), "mad_hi_T_per_s": round(hi / 1e12, 3)},
                "traffic": traffic,
                "per_op": {op: {"ms": round(per_op_ms[op], 3), "ops_s": round(count / (per_op_ms[op] / 1e3), 1),
                                "product_frac": round(PRODUCTS[op] * count / (per_op_ms[op] / 1e3) / prod_peak, 4),
                                "executed_products_per_op": tile_products(op, n),
                                "executed_frac": round(tile_products(op, n) * count / (per_op_ms[op] / 1e3) / prod_peak,
                                                       4)}
                           for op in OPS}}
    cpu, bit_exact = None, None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu, bit_exact = cpu_leg(data, gpu_results, threads)
        m = mpfr_leg(data, gpu_results, threads)
        if m is not None:
            cpu["mpfr"] = m
    extras = None
    if not args.no_extras and world == 1:
        extras = run_extras(fpa, torch, args.quick_extras, args.extras.split(","), per_op_ms)
    line = {"metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "4096-bit mul/div/sqrt, 2^20 operands each", "limbs": n, "operands_per_op": count,
                       "near_halfway_frac": 0.05, "mode": "ties_to_even", "step": "fpa_mul+fpa_div+fpa_sqrt",
                       "l2": "inputs 541 MB per operand array, larger than L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "bit_exact": bit_exact, "clocks": clk,
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
