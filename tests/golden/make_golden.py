"""Generate the committed golden fixtures: MPFR 4.2.1 results for seeded operands.

Run from the repository root:  python tests/golden/make_golden.py
Writes tests/golden/fixtures/<op>_n<limbs>.npz with the operands (a_*, b_*) and, for each
rounding mode m = 0..4, the MPFR result (r_exps[m], r_limbs[m]).  Operand sets per file:
uniform mantissas, the reference test generator's limb pattern (tests.c:173-181) and the
near-halfway / near-exact constructions of the 4096-bit workload.

Also writes tests/golden/conv/conv_mpfr.npz: mpfr_set_ui / set_si / set_flt / set_d
(round to nearest), mpfr_set between precisions in all five modes, and mpfr_sgn /
mpfr_cmp / mpfr_neg, on the seeded inputs of tests/conv_cases.py.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import conv_cases as CC  # noqa: E402
import gold  # noqa: E402
from cubigfloat_gb300 import workloads as W  # noqa: E402

OPS = ["add", "sub", "mul", "div", "sqrt"]
SIZES = {1: 24, 8: 24, 32: 24, 33: 24, 64: 16, 128: 16, 160: 6}
OUT = os.path.join(ROOT, "tests", "golden", "fixtures")
CONV_OUT = os.path.join(ROOT, "tests", "golden", "conv", "conv_mpfr.npz")
CONV_SIZES = (1, 2, 32, 128)


def operands(op, n, count, seed):
    rng = np.random.default_rng(seed)
    k1 = count // 2
    k2 = count // 4
    k3 = count - k1 - k2
    ae, al = W.uniform(rng, k1, n, -200, 200)
    be, bl = W.uniform(rng, k1, n, -200, 200)
    re_a, rl_a = W.reference_style(rng, k2, n)
    re_b, rl_b = W.reference_style(rng, k2, n)
    he_a = np.zeros(k3, np.uint32); hl_a = np.zeros((k3, n), np.uint32)
    he_b = np.zeros(k3, np.uint32); hl_b = np.zeros((k3, n), np.uint32)
    for i in range(k3):
        if op in ("mul", "add", "sub"):
            A, B = W.mul_near_half(rng, n)
        elif op == "div":
            A, B = W.div_near_exact(rng, n)
        else:
            A, par = W.sqrt_near_exact(rng, n)
            B = A
        hl_a[i] = W.int_to_limbs(A, n); hl_b[i] = W.int_to_limbs(B, n)
        ea = int(rng.integers(-20, 20)); eb = int(rng.integers(-20, 20))
        if op == "sqrt":
            ea = 2 * (ea // 2) + par
        he_a[i] = W.exp_word(ea, 0 if op == "sqrt" else int(rng.integers(0, 2)))
        he_b[i] = W.exp_word(eb, int(rng.integers(0, 2)))
    a_exps = np.concatenate([ae, re_a, he_a]); a_limbs = np.concatenate([al, rl_a, hl_a])
    b_exps = np.concatenate([be, re_b, he_b]); b_limbs = np.concatenate([bl, rl_b, hl_b])
    if op == "sqrt":
        a_exps = a_exps & ~np.uint32(1)
    return a_exps, a_limbs, b_exps, b_limbs


def main():
    os.makedirs(OUT, exist_ok=True)
    for oi, op in enumerate(OPS):
        for n, count in SIZES.items():
            a_exps, a_limbs, b_exps, b_limbs = operands(op, n, count, seed=1000 * oi + n)
            r_e, r_l = [], []
            for mode in range(5):
                e, l = gold.run(oi, n, mode, a_exps, a_limbs, b_exps, b_limbs)
                l[e <= 8] = 0
                r_e.append(e); r_l.append(l)
            np.savez_compressed(os.path.join(OUT, f"{op}_n{n}.npz"), op=oi, n=n,
                                a_exps=a_exps, a_limbs=a_limbs, b_exps=b_exps, b_limbs=b_limbs,
                                r_exps=np.stack(r_e), r_limbs=np.stack(r_l),
                                mpfr_version=gold.version())
    print("wrote", len(os.listdir(OUT)), "fixtures to", OUT)
    conversions()


def conversions():
    """MPFR results for the conversion, precision-change, sign, compare and negation cases."""
    z = {"mpfr_version": gold.version()}
    inputs = {"ui": CC.uint_values(1), "si": CC.int_values(2), "float": CC.float_bits(3).view(np.float32),
              "double": CC.double_bits(4).view(np.float64)}
    for kind, v in inputs.items():
        z[f"set_{kind}_in"] = v
        for n in CONV_SIZES:
            e, l = gold.set_values(kind, n, v)
            z[f"set_{kind}_n{n}_exps"], z[f"set_{kind}_n{n}_limbs"] = e, l
    for nx, nr in CC.PREC_PAIRS:
        if max(nx, nr) > 128:
            continue
        xe, xl = CC.prec_sources(10 * nx + nr, nx, nr)
        z[f"prec_{nx}_{nr}_in_exps"], z[f"prec_{nx}_{nr}_in_limbs"] = xe, xl
        outs = [gold.set_prec(nr, nx, m, xe, xl) for m in range(5)]
        z[f"prec_{nx}_{nr}_exps"] = np.stack([o[0] for o in outs])
        z[f"prec_{nx}_{nr}_limbs"] = np.stack([o[1] for o in outs])
    for n in CONV_SIZES:
        xe, xl = CC.numbers(50 + n, n, classes=CC.MPFR_CLASSES)
        z[f"num_n{n}_exps"], z[f"num_n{n}_limbs"] = xe, xl
        z[f"sgn_n{n}"] = gold.sgn(n, xe, xl)
        ne, nl = gold.neg(n, xe, xl)
        z[f"neg_n{n}_exps"], z[f"neg_n{n}_limbs"] = ne, nl
        ae, al, be, bl = CC.compare_pairs(60 + n, n, classes=CC.MPFR_CLASSES)
        z[f"cmp_n{n}_a_exps"], z[f"cmp_n{n}_a_limbs"] = ae, al
        z[f"cmp_n{n}_b_exps"], z[f"cmp_n{n}_b_limbs"] = be, bl
        z[f"cmp_n{n}"] = gold.cmp(n, ae, al, be, bl)
    os.makedirs(os.path.dirname(CONV_OUT), exist_ok=True)
    np.savez_compressed(CONV_OUT, **z)
    print("wrote", CONV_OUT)


if __name__ == "__main__":
    if sys.argv[1:] == ["--conversions"]:
        conversions()
    else:
        main()
