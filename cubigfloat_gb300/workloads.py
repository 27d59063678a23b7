"""Seeded synthetic operands for the fpa benchmark configurations and tests.

Numbers use the fpa encoding: exponent word 2*(BIAS + e) + sign (classes 0..8 are
reserved) and n little-endian 32-bit limbs with the top bit set, value = M * 2^(e - 32n).
All generators take a seed and are deterministic across machines (numpy PCG64).
"""
import numpy as np

BIAS = 0x3FFFFFF3
CLS_ZERO, CLS_NEG_TINY, CLS_POS_TINY, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN = 2, 3, 4, 5, 6, 7, 8


def exp_word(e, sign):
    return (2 * (BIAS + np.asarray(e, dtype=np.int64)) + np.asarray(sign, dtype=np.int64)).astype(np.uint32)


def decode_exp(w):
    w = np.asarray(w, dtype=np.int64)
    return (w >> 1) - BIAS, w & 1


def int_to_limbs(x, n):
    return np.frombuffer(int(x).to_bytes(4 * n, "little"), dtype=np.uint32).copy()


def limbs_to_int(limbs):
    return int.from_bytes(np.ascontiguousarray(limbs, dtype=np.uint32).tobytes(), "little")


def uniform(rng, count, n, emin, emax, signs=True):
    """Uniform random mantissas (top bit set), exponents uniform in [emin, emax]."""
    limbs = rng.integers(0, 1 << 32, size=(count, n), dtype=np.uint64).astype(np.uint32)
    limbs[:, n - 1] |= np.uint32(0x80000000)
    e = rng.integers(emin, emax + 1, size=count)
    s = rng.integers(0, 2, size=count) if signs else np.zeros(count, dtype=np.int64)
    return exp_word(e, s), limbs


def reference_style(rng, count, n, shift_frac=5 / 8):
    """The reference test generator's pattern (tests.c:173-181, 815-830): limbs drawn from
    {0, 1, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF}, normalised, exponent offset drawn as the
    difference of two uniform values below 5/8 of the precision, random sign."""
    vals = np.array([0, 1, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF], dtype=np.uint32)
    raw = vals[rng.integers(0, 5, size=(count, n))]
    exps = np.zeros(count, dtype=np.uint32)
    limbs = np.zeros((count, n), dtype=np.uint32)
    p = 32 * n
    span = max(1, int(p * shift_frac))
    for i in range(count):
        m = limbs_to_int(raw[i])
        if m == 0:
            m = 1 << (p - 1)
        L = m.bit_length()
        m <<= p - L
        e = L - p + int(rng.integers(0, span)) - int(rng.integers(0, span))
        limbs[i] = int_to_limbs(m, n)
        exps[i] = 2 * (BIAS + e) + int(rng.integers(0, 2))
    return exps, limbs


# ---- near-halfway constructions (the 4096-bit workload's 5% hard cases) ---------------

def _rand_bits(rng, bits):
    """random integer with exactly `bits` significant bits"""
    nb = (bits + 31) // 32
    words = rng.integers(0, 1 << 32, size=nb, dtype=np.uint64)
    x = 0
    for w in words[::-1]:
        x = (x << 32) | int(w)
    x &= (1 << bits) - 1
    return x | (1 << (bits - 1))


def mul_near_half(rng, n):
    """Mantissas A, B (p = 32n bits) whose exact product has its bits below the rounding
    position equal to 10...0 (an exact tie) or 10...0 +- 1."""
    p = 32 * n
    delta = int(rng.integers(-1, 2))
    for _ in range(1000):
        A = _rand_bits(rng, p) | 1
        if rng.integers(0, 2):
            # product of 2p-1 bits: tail = low p-1 bits
            mod = 1 << (p - 1)
            T = (1 << (p - 2)) + delta
            B = (1 << (p - 1)) + (T * pow(A, -1, mod)) % mod
            want = 2 * p - 1
        else:
            # product of 2p bits: tail = low p bits
            mod = 1 << p
            T = (1 << (p - 1)) + delta
            B = (T * pow(A, -1, mod)) % mod
            want = 2 * p
        if B >> (p - 1) == 1 and (A * B).bit_length() == want:
            return A, B
    raise RuntimeError("no near-halfway pair found")


def div_near_exact(rng, n):
    """a = q*b +- 1 ulp with q and b of p/2 bits: the quotient sits within ~2^-p ulp of a
    representable value."""
    p = 32 * n
    h = max(1, p // 2 - 1)
    while True:
        q = _rand_bits(rng, h)
        b = _rand_bits(rng, h) | 1
        qb = q * b
        A = qb << (p - qb.bit_length())
        A += int(rng.integers(-1, 2))
        if A.bit_length() == p:
            return A, b << (p - b.bit_length())


def sqrt_near_exact(rng, n):
    """x = s^2 +- 1 ulp with s of at most p/2 bits (the reference's pattern, tests.c:894-906).
    Returns the mantissa and the exponent parity that makes s^2 an exact square."""
    p = 32 * n
    s = _rand_bits(rng, max(1, p // 2 - 1))
    sq = s * s
    A = (sq << (p - sq.bit_length())) + int(rng.integers(-1, 2))
    if A.bit_length() != p:
        A = sq << (p - sq.bit_length())
    # x = A * 2^(e - p) = sq * 2^(e - L): exact square when e - L is even
    return A, sq.bit_length() & 1


def workload_4096(op, seed, count=1 << 20, n=128, hard_frac=0.05, pool=256):
    """4096-bit mul/div/sqrt operands: uniform mantissas, e in [-1000, 1000]; nonzero
    divisors, positive sqrt arguments; `hard_frac` of the instances are near-halfway
    (mul) or near-exact (div, sqrt) cases drawn from a pool of distinct constructions
    (each placed with its own random exponents and signs)."""
    rng = np.random.default_rng(seed)
    a_exps, a_limbs = uniform(rng, count, n, -1000, 1000, signs=(op != "sqrt"))
    b_exps, b_limbs = uniform(rng, count, n, -1000, 1000, signs=True)
    nh = int(count * hard_frac)
    if nh:
        idx = rng.choice(count, size=nh, replace=False)
        npool = min(pool, nh)
        make = {"mul": mul_near_half, "div": div_near_exact, "sqrt": sqrt_near_exact}[op]
        cases = [make(rng, n) for _ in range(npool)]
        pa = np.stack([int_to_limbs(A, n) for A, _ in cases])
        pick = np.arange(nh) % npool
        a_limbs[idx] = pa[pick]
        if op == "sqrt":
            parity = np.array([par for _, par in cases], dtype=np.int64)[pick]   # exponent parity for s^2
            e = 2 * rng.integers(-500, 500, size=nh) + parity
            a_exps[idx] = exp_word(e, 0)
        else:
            b_limbs[idx] = np.stack([int_to_limbs(B, n) for _, B in cases])[pick]
    return (a_exps, a_limbs), (b_exps, b_limbs)


def workload_1024(seed, count=65536, n=32):
    """1024-bit add/mul operands: uniform mantissas, e in [-64, 64], random signs."""
    rng = np.random.default_rng(seed)
    a = uniform(rng, count, n, -64, 64)
    b = uniform(rng, count, n, -64, 64)
    return a, b


MIX_OPS = np.array([0, 1, 2, 3, 4])            # add, sub, mul, div, sqrt
MIX_P = np.array([0.3, 0.2, 0.3, 0.1, 0.1])


def mixed(seed, count, min_bits=256, max_bits=16384, mode=3, hard_frac=0.05, ops=None, limbs=None):
    """Mixed batch (10^6-op workload): op drawn 30/20/30/10/10 from add/sub/mul/div/sqrt, precision
    log-uniform in [min_bits, max_bits] rounded to whole limbs, operands as in the 4096-bit workload
    (uniform mantissas, e in [-1000, 1000], positive sqrt arguments, `hard_frac`
    near-halfway/near-exact cases, one construction per (op, limbs) pair).
    Returns (descs, a_exps, a_limbs_flat, b_exps, b_limbs_flat, r_total) with descs in the
    fpa_batch_desc layout."""
    from cubigfloat_gb300 import BATCH_DESC
    rng = np.random.default_rng(seed)
    if ops is None:
        ops = rng.choice(MIX_OPS, size=count, p=MIX_P).astype(np.uint8)
    if limbs is None:
        bits = 2.0 ** rng.uniform(np.log2(min_bits), np.log2(max_bits), size=count)
        limbs = np.clip(np.rint(bits / 32), 1, 512).astype(np.uint16)
    ops = np.asarray(ops, dtype=np.uint8)
    limbs = np.asarray(limbs, dtype=np.uint16)
    off = np.zeros(count + 1, dtype=np.uint64)
    np.cumsum(limbs, out=off[1:])
    total = int(off[-1])
    a_limbs = rng.integers(0, 1 << 32, size=total, dtype=np.uint64).astype(np.uint32)
    b_limbs = rng.integers(0, 1 << 32, size=total, dtype=np.uint64).astype(np.uint32)
    tops = (off[1:] - 1).astype(np.int64)
    a_limbs[tops] |= np.uint32(0x80000000)
    b_limbs[tops] |= np.uint32(0x80000000)
    ea = rng.integers(-1000, 1001, size=count)
    eb = rng.integers(-1000, 1001, size=count)
    sa = np.where(ops == 4, 0, rng.integers(0, 2, size=count))
    a_exps = exp_word(ea, sa)
    b_exps = exp_word(eb, rng.integers(0, 2, size=count))
    nh = int(count * hard_frac)
    if nh:
        idx = rng.choice(count, size=nh, replace=False)
        made = {}
        for i in idx:
            op, n = int(ops[i]), int(limbs[i])
            if op == 4:
                kind = "sqrt"
            elif op == 3:
                kind = "div"
            else:
                kind = "mul"
            key = (kind, n)
            if key not in made:
                made[key] = {"mul": mul_near_half, "div": div_near_exact, "sqrt": sqrt_near_exact}[kind](rng, n)
            A, B = made[key]
            o = int(off[i])
            a_limbs[o:o + n] = int_to_limbs(A, n)
            if kind == "sqrt":
                a_exps[i] = exp_word(2 * int(rng.integers(-500, 500)) + B, 0)
            else:
                b_limbs[o:o + n] = int_to_limbs(B, n)
    descs = np.zeros(count, dtype=BATCH_DESC)
    descs["op"] = ops
    descs["mode"] = mode
    descs["limbs"] = limbs
    descs["r_off"] = off[:-1]
    descs["a_off"] = off[:-1]
    descs["b_off"] = off[:-1]
    return descs, a_exps, a_limbs, b_exps, b_limbs, total


SERVED_PRECISIONS = (512, 1024, 4096, 16384)


def served_job(rng, precision=None, size=None, max_ops=4096):
    """One served request: a precision from {512, 1024, 4096, 16384} bits, a size
    log-uniform in [1, max_ops], ops drawn 30/20/30/10/10, operands as in the 4096-bit workload without
    the hard cases.  Returns (precision, ops, modes, a_exps, a_limbs, b_exps, b_limbs)."""
    if precision is None:
        precision = int(rng.choice(SERVED_PRECISIONS))
    if size is None:
        size = int(np.clip(np.rint(2.0 ** rng.uniform(0, np.log2(max_ops))), 1, max_ops))
    n = precision // 32
    ops = rng.choice(MIX_OPS, size=size, p=MIX_P).astype(np.uint8)
    ae, al = uniform(rng, size, n, -1000, 1000)
    be, bl = uniform(rng, size, n, -1000, 1000)
    ae = np.where(ops == 4, ae & ~np.uint32(1), ae).astype(np.uint32)
    modes = np.full(size, 3, np.uint8)
    return precision, ops, modes, ae, al.reshape(-1), be, bl.reshape(-1)


def reference_style_bulk(rng, count, n, signs=True, shift_frac=5 / 8):
    """The reference test generator's pattern (tests.c:173-181, 815-830) for large counts,
    vectorised: limbs drawn from {0, 1, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF}, normalised
    (an all-zero draw becomes 2^(p-1)), exponent offset drawn as the difference of two
    uniform values below 5/8 of the precision, random sign when `signs`."""
    vals = np.array([0, 1, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF], dtype=np.uint32)
    raw = vals[rng.integers(0, 5, size=(count, n))]
    p = 32 * n
    nz = raw != 0
    top = np.where(nz.any(axis=1), n - 1 - np.argmax(nz[:, ::-1], axis=1), -1)      # highest nonzero limb
    raw[top < 0, n - 1] = 0x80000000
    top[top < 0] = n - 1
    tl = raw[np.arange(count), top].astype(np.uint64)
    L = 32 * top + np.floor(np.log2(np.maximum(tl, 1).astype(np.float64))).astype(np.int64) + 1
    sh = p - L                                           # left shift that sets the top bit
    q, r = sh // 32, (sh % 32).astype(np.uint64)
    idx = np.arange(n)[None, :] - q[:, None]             # source limb of each destination limb
    lo_idx = idx - 1
    get = lambda ix: np.where((ix >= 0) & (ix < n), raw[np.arange(count)[:, None], np.clip(ix, 0, n - 1)], 0)
    hi = get(idx).astype(np.uint64)
    lo = get(lo_idx).astype(np.uint64)
    rr = r[:, None]
    limbs = ((hi << rr) | np.where(rr > 0, lo >> (np.uint64(32) - rr), np.uint64(0))) & np.uint64(0xFFFFFFFF)
    limbs = limbs.astype(np.uint32)
    span = max(1, int(p * shift_frac))
    e = L - p + rng.integers(0, span, size=count) - rng.integers(0, span, size=count)
    s = rng.integers(0, 2, size=count) if signs else np.zeros(count, dtype=np.int64)
    return exp_word(e, s), limbs


def poisson_arrivals(rng, njobs, rate_per_s):
    """Arrival times (seconds from start) of a Poisson process."""
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=njobs))


def specials(n):
    """One operand of each class plus +-1.0 and +-0.75, for special-value tables."""
    one = np.zeros(n, dtype=np.uint32)
    one[n - 1] = 0x80000000
    tq = np.zeros(n, dtype=np.uint32)
    tq[n - 1] = 0xC0000000
    exps = [exp_word(1, 0), exp_word(1, 1), exp_word(0, 0), exp_word(0, 1),
            CLS_ZERO, CLS_NEG_TINY, CLS_POS_TINY, CLS_NEG_INF, CLS_POS_INF, CLS_NAN, CLS_SNAN]
    limbs = [one, one, tq, tq] + [np.zeros(n, dtype=np.uint32)] * 7
    return np.array(exps, dtype=np.uint32), np.stack(limbs)
