"""Autotune the lane-group configuration table on the current GPU.

    python -m cubigfloat_gb300.tune [--sample N] [--out PATH] [--ops 0,1]

For every operation and every limb count on a grid from 1 to 512, fpa_gb300_autotune times
each configuration that can hold the limb count and keeps the fastest; each grid winner
covers the limb counts down to the previous grid point.  The result is written as
"op first_limbs last_limbs cfg" lines (default: tuned_configs.txt beside this file, which
the library loads at start-up).
"""
import argparse
import ctypes
import os

import cubigfloat_gb300 as fpa

GRID = [1, 2, 3, 4, 6, 8, 12, 16, 20, 24, 28, 32, 40, 48, 56, 64, 80, 96, 112, 128, 160, 192, 224, 256,
        320, 384, 448, 512]
OP_NAMES = ["add", "sub", "mul", "div", "sqrt"]
DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned_configs.txt")


def tune(sample=1 << 17, ops=range(5), grid=GRID, log=print):
    L = fpa.lib()
    table = []
    for op in ops:
        prev = 0
        # add/sub/mul: configuration 16 has kernels for exactly 8, 16 and 32 limbs, so the
        # sizes just below them get grid points of their own
        for n in (sorted(set(grid) | {7, 15, 31}) if op in (0, 1, 2) else grid):
            best, rate = ctypes.c_int(-1), ctypes.c_double(0)
            s = sample if n <= 64 else max(4096, sample * 64 // n)       # about the same limbs per point
            if op in (0, 1):       # add/sub are bound by HBM: operands and results well beyond L2
                s = max(s, (1 << 28) // (12 * (n + 1)))
            rc = L.fpa_gb300_autotune(op, n, s, ctypes.byref(best), ctypes.byref(rate))
            if rc != fpa.fpa_success:
                raise fpa.FpaError(f"fpa_gb300_autotune({op}, {n}) -> {rc}")
            table.append((op, prev + 1, n, best.value, rate.value))
            log(f"{OP_NAMES[op]:4s} limbs {prev + 1:3d}..{n:3d}: cfg {best.value} {fpa.configs()[best.value]} "
                f"{rate.value / 1e6:10.2f} M ops/s")
            prev = n
    return table


def read(path=DEFAULT_OUT):
    """The (op, first, last, cfg, rate) rows of a table file."""
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            head, _, tail = line.partition("#")
            op, lo, hi, cfg = (int(x) for x in head.split())
            rate = float(tail.split()[-1]) * 1e6 if tail.strip() else 0.0
            rows.append((op, lo, hi, cfg, rate))
    return rows


def write(table, path=DEFAULT_OUT):
    table = sorted(table, key=lambda r: (r[0], r[1]))
    with open(path, "w") as f:
        f.write("# op first_limbs last_limbs cfg   (autotuned on GB300 by cubigfloat_gb300.tune; "
                "rates in M ops/s at the last limb count)\n")
        for op, lo, hi, cfg, rate in table:
            f.write(f"{op} {lo} {hi} {cfg}   # {OP_NAMES[op]} {rate / 1e6:.2f}\n")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--sample", type=int, default=1 << 17)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--ops", default="0,1,2,3,4", help="operations to tune; the rows of the others are "
                    "kept from the current table")
    a = ap.parse_args()
    ops = sorted({int(x) for x in a.ops.split(",")})
    table = tune(a.sample, ops)
    if len(ops) < 5 and os.path.exists(DEFAULT_OUT):
        table += [r for r in read(DEFAULT_OUT) if r[0] not in ops]
    write(table, a.out)
    print("wrote", a.out)
