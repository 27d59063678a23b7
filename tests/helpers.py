"""Shared helpers for the parity tests."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fixtures")
OPS = ["add", "sub", "mul", "div", "sqrt"]


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def mismatches(exp_e, exp_l, got_e, got_l):
    """Indices where two result sets differ: exponent words always, limbs only for values
    (class results leave limbs unspecified, as in the reference, tests.c:431)."""
    exp_e = np.asarray(exp_e); got_e = np.asarray(got_e)
    bad = exp_e != got_e
    val = exp_e > 8
    n = exp_l.shape[-1]
    bad |= val & np.any(np.asarray(exp_l).reshape(-1, n) != np.asarray(got_l).reshape(-1, n), axis=1)
    return np.nonzero(bad)[0]


def describe(i, a_e, a_l, b_e, b_l, exp_e, exp_l, got_e, got_l):
    def f(e, l):
        return f"exp=0x{int(e):08x} limbs[top]=0x{int(l[-1]):08x} limbs[0]=0x{int(l[0]):08x}"
    return (f"case {i}: a {f(a_e[i], a_l[i])}\n b {f(b_e[i], b_l[i])}\n"
            f" expected {f(exp_e[i], exp_l[i])}\n got      {f(got_e[i], got_l[i])}")
