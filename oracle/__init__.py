"""CPU oracle for the fpa add/sub/mul/div/sqrt path -- TEST INFRASTRUCTURE ONLY.

Wraps fpa_oracle.c (a plain-C restatement of the reference kernels' semantics with exact
integer arithmetic, see that file's header).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, as the checker; the product library never does.

Parity of this oracle is pinned against MPFR 4.2.1 (the reference's own test oracle,
tests.c:423-485) through the golden fixtures in tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "fpa_oracle.c")

ADD, SUB, MUL, DIV, SQRT = range(5)
_lib = None


def build():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.oracle_batch.restype = i32
        L.oracle_batch.argtypes = [i32, u32, i32, u32, vp, vp, vp, vp, vp, vp, i32]
        L.oracle_mixed.restype = i32
        L.oracle_mixed.argtypes = [u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32]
        L.oracle_fma_batch.restype = i32
        L.oracle_fma_batch.argtypes = [u32, i32, u32, vp, vp, vp, vp, vp, vp, vp, vp]
        for name in ("oracle_set_ui", "oracle_set_si", "oracle_set_float", "oracle_set_double"):
            getattr(L, name).restype = i32
            getattr(L, name).argtypes = [u32, u32, vp, vp, vp]
        L.oracle_set_prec.restype = i32
        L.oracle_set_prec.argtypes = [u32, u32, i32, u32, vp, vp, vp, vp]
        L.oracle_sgn.restype = i32
        L.oracle_sgn.argtypes = [u32, vp, vp]
        L.oracle_cmp.restype = i32
        L.oracle_cmp.argtypes = [u32, u32, vp, vp, vp, vp, vp]
        L.oracle_neg.restype = i32
        L.oracle_neg.argtypes = [u32, u32, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def run(op, n, mode, a_exps, a_limbs, b_exps=None, b_limbs=None, threads=1):
    """Elementwise op over count instances; returns (r_exps, r_limbs[count, n]).
    Result limbs of special (class) results are left zero."""
    a_exps = np.ascontiguousarray(a_exps, dtype=np.uint32)
    a_limbs = np.ascontiguousarray(a_limbs, dtype=np.uint32).reshape(-1, n)
    count = a_exps.size
    if op != SQRT:
        b_exps = np.ascontiguousarray(b_exps, dtype=np.uint32)
        b_limbs = np.ascontiguousarray(b_limbs, dtype=np.uint32).reshape(-1, n)
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    rc = lib().oracle_batch(op, n, mode, count, _p(r_exps), _p(r_limbs), _p(a_exps), _p(a_limbs),
                            _p(b_exps) if op != SQRT else None, _p(b_limbs) if op != SQRT else None, threads)
    if rc != 0:
        raise ValueError(f"oracle_batch rc={rc}")
    return r_exps, r_limbs


def run_fma(n, mode, a_exps, a_limbs, b_exps, b_limbs, c_exps, c_limbs):
    """r = RND(a*b + c) with one rounding over count instances; returns (r_exps, r_limbs)."""
    arr = [np.ascontiguousarray(x, dtype=np.uint32) for x in (a_exps, a_limbs, b_exps, b_limbs, c_exps, c_limbs)]
    count = arr[0].size
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    rc = lib().oracle_fma_batch(n, mode, count, _p(r_exps), _p(r_limbs), *[_p(x) for x in arr])
    if rc != 0:
        raise ValueError(f"oracle_fma_batch rc={rc}")
    return r_exps, r_limbs


def run_mixed(ops, ns, modes, a_exps, a_limbs, a_off, b_exps, b_limbs, b_off, r_off, r_total, threads=1):
    """Heterogeneous batch (flat limb arrays with per-instance offsets)."""
    count = len(ops)
    ops = np.ascontiguousarray(ops, dtype=np.uint8)
    ns = np.ascontiguousarray(ns, dtype=np.uint16)
    modes = np.ascontiguousarray(modes, dtype=np.uint8)
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros(r_total, dtype=np.uint32)
    arrs = [np.ascontiguousarray(x, dtype=t) for x, t in
            ((a_exps, np.uint32), (a_limbs, np.uint32), (a_off, np.uint64),
             (b_exps, np.uint32), (b_limbs, np.uint32), (b_off, np.uint64), (r_off, np.uint64))]
    rc = lib().oracle_mixed(count, _p(ops), _p(ns), _p(modes), _p(r_exps), _p(r_limbs), _p(arrs[6]),
                            _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]), _p(arrs[4]), _p(arrs[5]), threads)
    if rc != 0:
        raise ValueError(f"oracle_mixed rc={rc}")
    return r_exps, r_limbs


# ---- conversions, sign, compare, negation ------------------------------------------
_SET_KIND = {"ui": ("oracle_set_ui", np.uint64), "si": ("oracle_set_si", np.int64),
             "float": ("oracle_set_float", np.float32), "double": ("oracle_set_double", np.float64)}


def set_values(kind, n, values):
    """fpa_set_ui / si / float / double of `values` at n limbs; returns (r_exps, r_limbs).
    Class results leave their limbs zero."""
    name, dt = _SET_KIND[kind]
    v = np.ascontiguousarray(values, dtype=dt)
    if kind in ("float", "double"):
        v = v.view(np.uint32 if kind == "float" else np.uint64)
    count = v.size
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    if getattr(lib(), name)(n, count, _p(r_exps), _p(r_limbs), _p(v)) != 0:
        raise ValueError(f"{name} failed")
    return r_exps, r_limbs


def set_prec(nr, nx, mode, x_exps, x_limbs):
    """fpa_set: numbers of nx limbs rounded to nr limbs in `mode`."""
    x_exps = np.ascontiguousarray(x_exps, dtype=np.uint32)
    x_limbs = np.ascontiguousarray(x_limbs, dtype=np.uint32).reshape(-1, nx)
    count = x_exps.size
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, nr), dtype=np.uint32)
    if lib().oracle_set_prec(nr, nx, mode, count, _p(r_exps), _p(r_limbs), _p(x_exps), _p(x_limbs)) != 0:
        raise ValueError("oracle_set_prec failed")
    return r_exps, r_limbs


def sgn(x_exps):
    x_exps = np.ascontiguousarray(x_exps, dtype=np.uint32)
    r = np.zeros(x_exps.size, dtype=np.int32)
    lib().oracle_sgn(x_exps.size, _p(r), _p(x_exps))
    return r


def cmp(n, a_exps, a_limbs, b_exps, b_limbs):
    arr = [np.ascontiguousarray(x, dtype=np.uint32) for x in (a_exps, a_limbs, b_exps, b_limbs)]
    r = np.zeros(arr[0].size, dtype=np.int32)
    if lib().oracle_cmp(n, arr[0].size, _p(r), *[_p(x) for x in arr]) != 0:
        raise ValueError("oracle_cmp failed")
    return r


def neg(n, a_exps, a_limbs):
    a_exps = np.ascontiguousarray(a_exps, dtype=np.uint32)
    a_limbs = np.ascontiguousarray(a_limbs, dtype=np.uint32).reshape(-1, n)
    r_exps = np.zeros(a_exps.size, dtype=np.uint32)
    r_limbs = np.zeros((a_exps.size, n), dtype=np.uint32)
    if lib().oracle_neg(n, a_exps.size, _p(r_exps), _p(r_limbs), _p(a_exps), _p(a_limbs)) != 0:
        raise ValueError("oracle_neg failed")
    return r_exps, r_limbs


# ---- the reference's own kernels (compiled from its sources, test use only) ----------
REF_DIR = os.path.join(HERE, "_ref")
REF_CUBIN = os.path.join(REF_DIR, "ref_fpa.cubin")


def build_ref(reference_root=None):
    """Compile the reference's device code (its single translation unit fpa.cu) for sm_103a
    into oracle/_ref/ref_fpa.cubin.  Runs only where the reference sources are present; the
    cubin is loaded by tests through the CUDA driver API to compare against the reference's
    own GPU output.  The sources are looked for in $FPA_REFERENCE_ROOT, else in a directory
    named `reference` beside the repository.  Returns the cubin path or None."""
    if reference_root is None:
        reference_root = os.environ.get("FPA_REFERENCE_ROOT",
                                        os.path.join(os.path.dirname(HERE), os.pardir, "reference"))
    src = os.path.join(reference_root, "fpa.cu")
    if not os.path.exists(src):
        return REF_CUBIN if os.path.exists(REF_CUBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if os.path.exists(REF_CUBIN) and os.path.getmtime(REF_CUBIN) >= os.path.getmtime(src):
        return REF_CUBIN
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-DGPU", "-O3",
                    "-o", REF_CUBIN, src], check=True, capture_output=True)
    return REF_CUBIN


RUNNER_SRC = os.path.join(HERE, "ref_runner.c")
RUNNER_LIB = os.path.join(BUILD, "libref_runner.so")
_runner = None


def ref_gpu_available():
    return os.path.exists(REF_CUBIN)


def _runner_lib():
    global _runner
    if _runner is None:
        os.makedirs(BUILD, exist_ok=True)
        if not os.path.exists(RUNNER_LIB) or os.path.getmtime(RUNNER_LIB) < os.path.getmtime(RUNNER_SRC):
            subprocess.run(["gcc", "-O2", "-shared", "-fPIC", RUNNER_SRC, "-o", RUNNER_LIB, "-ldl"], check=True)
        L = ctypes.CDLL(RUNNER_LIB)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.ref_load.restype = i32
        L.ref_load.argtypes = [ctypes.c_char_p]
        L.ref_run.restype = i32
        L.ref_run.argtypes = [ctypes.c_char_p, u32, u32, i32, vp, vp, vp, vp, vp, vp, i32,
                              ctypes.POINTER(ctypes.c_float)]
        rc = L.ref_load(REF_CUBIN.encode())
        if rc != 0:
            raise RuntimeError(f"ref_load failed rc={rc}")
        _runner = L
    return _runner


def ref_gpu_run(op, n, mode, a_exps, a_limbs, b_exps=None, b_limbs=None, repeat=1):
    """Run the reference's own kernel for `op` ("add".."sqrt") on the GPU.
    Returns (r_exps, r_limbs, ms_per_launch)."""
    L = _runner_lib()
    a_exps = np.ascontiguousarray(a_exps, dtype=np.uint32)
    a_limbs = np.ascontiguousarray(a_limbs, dtype=np.uint32).reshape(-1, n)
    count = a_exps.size
    if op != "sqrt":
        b_exps = np.ascontiguousarray(b_exps, dtype=np.uint32)
        b_limbs = np.ascontiguousarray(b_limbs, dtype=np.uint32).reshape(-1, n)
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    ms = ctypes.c_float()
    rc = L.ref_run(op.encode(), 32 * n, count, mode, _p(r_exps), _p(r_limbs), _p(a_exps), _p(a_limbs),
                   _p(b_exps) if op != "sqrt" else None, _p(b_limbs) if op != "sqrt" else None,
                   repeat, ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError(f"ref_run({op}) rc={rc}")
    return r_exps, r_limbs, ms.value
