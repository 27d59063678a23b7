"""Operand sets for the fma tests (seeded): uniform values, exact and near cancellation of
a*b by c, c far above and far below the product, and every special class combination."""
import numpy as np

import oracle
from cubigfloat_gb300 import workloads as W

CLASSES = [2, 3, 4, 5, 6, 7, 8]          # ZERO, -TINY, +TINY, -INF, +INF, NAN, SNAN


def fma_cases(seed, n, count=96):
    rng = np.random.default_rng(seed)
    ae, al = W.uniform(rng, count, n, -60, 60)
    be, bl = W.uniform(rng, count, n, -60, 60)
    ce, cl = W.uniform(rng, count, n, -120, 120)
    q = count // 6
    # c = -RN(a*b): cancellation down to the product's rounding error; every 2nd one nudged
    pe, pl = oracle.run(2, n, 3, ae[:2 * q], al[:2 * q], be[:2 * q], bl[:2 * q])
    ce[:2 * q] = pe ^ np.uint32(1)
    cl[:2 * q] = pl
    cl[:q, 0] ^= np.uint32(1)
    # c = +RN(a*b) (doubling, carries into a new binade)
    pe2, pl2 = oracle.run(2, n, 0, ae[2 * q:3 * q], al[2 * q:3 * q], be[2 * q:3 * q], bl[2 * q:3 * q])
    ce[2 * q:3 * q] = pe2
    cl[2 * q:3 * q] = pl2
    # c far below / far above the product (only a sticky bit / the product is the sticky bit)
    ce[3 * q:4 * q] = W.exp_word(rng.integers(-3000, -2000, q), rng.integers(0, 2, q))
    ce[4 * q:5 * q] = W.exp_word(rng.integers(2000, 3000, q), rng.integers(0, 2, q))
    return ae, al, be, bl, ce, cl


def special_cases(n):
    """Every (class or value) x (class or value) x (class or value) combination."""
    vals_e = [W.exp_word(1, 0), W.exp_word(1, 1)] + CLASSES
    lim = np.zeros(n, dtype=np.uint32)
    lim[n - 1] = 0xC0000000
    es = np.array(vals_e, dtype=np.uint32)
    grid = np.array(np.meshgrid(np.arange(len(es)), np.arange(len(es)), np.arange(len(es)), indexing="ij")).reshape(3, -1)
    ae, be, ce = es[grid[0]], es[grid[1]], es[grid[2]]
    al = np.tile(lim, (ae.size, 1))
    return ae, al, be, al.copy(), ce, al.copy()
