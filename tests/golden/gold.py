"""MPFR gold values for fpa operands (test infrastructure).

Builds mpfr_gold.c against the system libmpfr.so.6 / libgmp.so.10 (no headers needed) and
computes correctly rounded results the way the reference's test harness does
(tests.c:114-159 conversion, tests.c:55-73 rounding map; ties-away via a (p+1)-bit
truncation).  `available()` is False where libmpfr is not installed.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "mpfr_gold.so")
SRC = os.path.join(HERE, "mpfr_gold.c")
_lib = None
_err = None


def _build():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", SRC, "-o", LIB, "-l:libmpfr.so.6", "-l:libgmp.so.10"],
                   check=True, capture_output=True)


def lib():
    global _lib, _err
    if _lib is None and _err is None:
        try:
            _build()
            L = ctypes.CDLL(LIB)
            vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
            L.gold_batch.restype = i32
            L.gold_batch.argtypes = [i32, u32, i32, u32, vp, vp, vp, vp, vp, vp]
            L.gold_batch3.restype = i32
            L.gold_batch3.argtypes = [i32, u32, i32, u32, vp, vp, vp, vp, vp, vp, vp, vp]
            L.gold_version.restype = ctypes.c_char_p
            _lib = L
        except Exception as e:  # libmpfr absent
            _err = e
    return _lib


def available():
    return lib() is not None


def version():
    return lib().gold_version().decode()


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def run(op, n, mode, a_exps, a_limbs, b_exps=None, b_limbs=None):
    """op 0..4 = add, sub, mul, div, sqrt; inputs must be finite nonzero values."""
    a_exps = np.ascontiguousarray(a_exps, dtype=np.uint32)
    a_limbs = np.ascontiguousarray(a_limbs, dtype=np.uint32).reshape(-1, n)
    count = a_exps.size
    if op != 4:
        b_exps = np.ascontiguousarray(b_exps, dtype=np.uint32)
        b_limbs = np.ascontiguousarray(b_limbs, dtype=np.uint32).reshape(-1, n)
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    bad = lib().gold_batch(op, n, mode, count, _p(r_exps), _p(r_limbs), _p(a_exps), _p(a_limbs),
                           _p(b_exps) if op != 4 else None, _p(b_limbs) if op != 4 else None)
    if bad:
        raise ValueError(f"{bad} MPFR results were not finite")
    return r_exps, r_limbs


def run_fma(n, mode, a_exps, a_limbs, b_exps, b_limbs, c_exps, c_limbs):
    """MPFR's correctly rounded a*b + c (mpfr_fma); inputs must be finite nonzero values."""
    arr = [np.ascontiguousarray(x, dtype=np.uint32) for x in (a_exps, a_limbs, b_exps, b_limbs, c_exps, c_limbs)]
    count = arr[0].size
    r_exps = np.zeros(count, dtype=np.uint32)
    r_limbs = np.zeros((count, n), dtype=np.uint32)
    bad = lib().gold_batch3(5, n, mode, count, _p(r_exps), _p(r_limbs), *[_p(x) for x in arr])
    if bad:
        raise ValueError(f"{bad} MPFR results were not finite")
    return r_exps, r_limbs
