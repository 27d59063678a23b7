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
            L.gold_set.restype = i32
            L.gold_set.argtypes = [i32, u32, u32, vp, vp, vp]
            L.gold_set_prec.restype = i32
            L.gold_set_prec.argtypes = [u32, u32, i32, u32, vp, vp, vp, vp]
            L.gold_sgn.restype = i32
            L.gold_sgn.argtypes = [u32, u32, vp, vp, vp]
            L.gold_cmp.restype = i32
            L.gold_cmp.argtypes = [u32, u32, vp, vp, vp, vp, vp]
            L.gold_neg.restype = i32
            L.gold_neg.argtypes = [u32, u32, vp, vp, vp, vp]
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


_SET_KIND = {"ui": (0, np.uint64), "si": (1, np.int64), "float": (2, np.float32), "double": (3, np.float64)}


def set_values(kind, n, values):
    """mpfr_set_ui / set_si / set_flt / set_d at precision 32n, round to nearest; class
    results (zero, inf, NaN) as the fpa class codes with zero limbs."""
    k, dt = _SET_KIND[kind]
    v = np.ascontiguousarray(values, dtype=dt)
    r_exps = np.zeros(v.size, dtype=np.uint32)
    r_limbs = np.zeros((v.size, n), dtype=np.uint32)
    bad = lib().gold_set(k, n, v.size, _p(r_exps), _p(r_limbs), _p(v))
    if bad:
        raise ValueError(f"{bad} conversions failed")
    return r_exps, r_limbs


def set_prec(nr, nx, mode, x_exps, x_limbs):
    """mpfr_set from 32nx to 32nr bits in `mode` (inputs must be values)."""
    x_exps = np.ascontiguousarray(x_exps, dtype=np.uint32)
    x_limbs = np.ascontiguousarray(x_limbs, dtype=np.uint32).reshape(-1, nx)
    r_exps = np.zeros(x_exps.size, dtype=np.uint32)
    r_limbs = np.zeros((x_exps.size, nr), dtype=np.uint32)
    bad = lib().gold_set_prec(nr, nx, mode, x_exps.size, _p(r_exps), _p(r_limbs), _p(x_exps), _p(x_limbs))
    if bad:
        raise ValueError(f"{bad} precision changes failed")
    return r_exps, r_limbs


def sgn(n, x_exps, x_limbs):
    x_exps = np.ascontiguousarray(x_exps, dtype=np.uint32)
    x_limbs = np.ascontiguousarray(x_limbs, dtype=np.uint32)
    r = np.zeros(x_exps.size, dtype=np.int32)
    if lib().gold_sgn(n, x_exps.size, _p(r), _p(x_exps), _p(x_limbs)):
        raise ValueError("gold_sgn: input without an MPFR counterpart")
    return r


def cmp(n, a_exps, a_limbs, b_exps, b_limbs):
    arr = [np.ascontiguousarray(x, dtype=np.uint32) for x in (a_exps, a_limbs, b_exps, b_limbs)]
    r = np.zeros(arr[0].size, dtype=np.int32)
    if lib().gold_cmp(n, arr[0].size, _p(r), *[_p(x) for x in arr]):
        raise ValueError("gold_cmp: input without an MPFR counterpart")
    return r


def neg(n, a_exps, a_limbs):
    a_exps = np.ascontiguousarray(a_exps, dtype=np.uint32)
    a_limbs = np.ascontiguousarray(a_limbs, dtype=np.uint32).reshape(-1, n)
    r_exps = np.zeros(a_exps.size, dtype=np.uint32)
    r_limbs = np.zeros((a_exps.size, n), dtype=np.uint32)
    if lib().gold_neg(n, a_exps.size, _p(r_exps), _p(r_limbs), _p(a_exps), _p(a_limbs)):
        raise ValueError("gold_neg: input without an MPFR counterpart")
    return r_exps, r_limbs
