"""Build the GB300 fpa library in-tree: cubigfloat_gb300/_build/libfpa_gb300.so.

nvcc compiles each lane-group configuration of the elementwise kernels as its own object
(in parallel), plus the C-ABI layer and the conversion kernels, for sm_103a only.
"""
import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfpa_gb300.so")
NUM_CFGS = 16

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_digest():
    h = hashlib.sha256()
    for root in (CSRC, os.path.join(HERE, "..", "include")):
        for name in sorted(os.listdir(root)):
            if name.endswith((".cuh", ".h")):
                with open(os.path.join(root, name), "rb") as f:
                    h.update(name.encode() + f.read())
    return h.hexdigest()


def _units():
    units = []
    for c in range(NUM_CFGS):
        units.append(("fpa_kernels.cu", [f"-DGFPA_CFG={c}"], f"fpa_kernels_cfg{c}.o"))
    units.append(("fpa_addsub_narrow.cu", [], "fpa_addsub_narrow.o"))
    units.append(("fpa_misc.cu", [], "fpa_misc.o"))
    units.append(("fpa_api.cu", [], "fpa_api.o"))
    units.append(("fpa_probe.cu", [], "fpa_probe.o"))
    units.append(("fpa_batch.cu", [], "fpa_batch.o"))
    units.append(("fpa_chain.cu", [], "fpa_chain.o"))
    units.append(("fpa_tune.cu", [], "fpa_tune.o"))
    units.append(("fpa_batch_noalloc.cu", [], "fpa_batch_noalloc.o"))
    for c in range(3):
        units.append(("fpa_batch_kernels.cu", [f"-DGFPA_BATCH_CLASS={c}"], f"fpa_batch_kernels_cls{c}.o"))
    units.append(("fpa_serve.cu", [], "fpa_serve.o"))
    units.append(("fpa_thread_newton.cu", [], "fpa_thread_newton.o"))
    units.append(("fpa_batch_thread.cu", [], "fpa_batch_thread.o"))
    return [u for u in units if os.path.exists(os.path.join(CSRC, u[0]))]


def _stamp(src, defs):
    h = hashlib.sha256()
    with open(os.path.join(CSRC, src), "rb") as f:
        h.update(f.read())
    h.update(" ".join(defs + NVCC_FLAGS).encode())
    h.update(_headers_digest().encode())
    return h.hexdigest()


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    units = _units()

    def compile_one(u):
        src, defs, obj = u
        obj_path = os.path.join(OUT, obj)
        stamp_path = obj_path + ".stamp"
        stamp = _stamp(src, defs)
        if os.path.exists(obj_path) and os.path.exists(stamp_path):
            with open(stamp_path) as f:
                if f.read() == stamp:
                    return obj_path, False
        cmd = [nvcc] + NVCC_FLAGS + defs + ["-c", os.path.join(CSRC, src), "-o", obj_path]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src} {defs}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        with open(stamp_path, "w") as f:
            f.write(stamp)
        return obj_path, True

    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(compile_one, units))
    objs = [r[0] for r in results]
    changed = any(r[1] for r in results)
    if changed or not os.path.exists(LIB):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
