"""Builds tests/c_caller/fpa_caller.c, a plain C program against include/fpa.h linked with
libfpa_gb300.so (gcc, no CUDA headers), and runs it on operands written to a file."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "fpa_caller.c")
LIBDIR = os.path.join(ROOT, "cubigfloat_gb300", "_build")


def build(out_dir):
    exe = os.path.join(str(out_dir), "fpa_caller")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", SRC, "-I", os.path.join(ROOT, "include"),
                    "-L", LIBDIR, "-lfpa_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", exe], check=True)
    return exe


def run(exe, work_dir, op, n, mode, ae, al, be=None, bl=None):
    """One fpa.h operation through the C program; returns (r_exps, r_limbs)."""
    count = len(ae)
    fin, fout = os.path.join(str(work_dir), "in.bin"), os.path.join(str(work_dir), "out.bin")
    with open(fin, "wb") as f:
        np.array([op, count, 32 * n, mode], dtype=np.uint32).tofile(f)
        np.ascontiguousarray(ae, dtype=np.uint32).tofile(f)
        np.ascontiguousarray(al, dtype=np.uint32).tofile(f)
        if op != 4:
            np.ascontiguousarray(be, dtype=np.uint32).tofile(f)
            np.ascontiguousarray(bl, dtype=np.uint32).tofile(f)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr)
    out = np.fromfile(fout, dtype=np.uint32)
    os.remove(fin)
    os.remove(fout)
    return out[:count], out[count:].reshape(count, n)
