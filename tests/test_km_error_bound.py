"""The error bound behind div/sqrt's rounding shortcut, checked on the CPU.

op_div and op_sqrt (cubigfloat_gb300/csrc/fpa_ops.cuh) finish with a Karp-Markstein step
that yields one limb more than the result: Q' ~ (A/B) 2^(32(n+1)) and S' ~ sqrt(A_ext) 2^32.
Rounding is decided from Q' / S' alone when their 32 guard bits lie at least 2^20 units
away from a rounding boundary, which is sound only if |Q' - exact| and |S' - exact| stay far
below 2^20.  This test restates the device's integer steps exactly (the Newton levels with
their truncations, the residual read from the product, the Karp-Markstein step with the
remainder kept from limb n-2 up) in Python integers, and checks on every size class
(including the worst case n = 2h-1, where the level below n is half of it) that
  - the remainder D fits the limbs the device multiplies (m+2 for div, m+3 for sqrt), and
  - the error is a few units (the device code comments quote <= 9 and <= 3).

The one-thread kernels (tdiv / tsqrt in fpa_thread_newton.cuh) take the same steps with
products restricted to the limbs their consumers read (short and middle products, formed
in 8-limb output blocks from GUARD limbs below the lowest kept limb, no carry into the
first block), and read the sign of the Karp-Markstein remainder from its top bit.  Their
model below restates those integer steps exactly and checks the same two properties, plus
that the remainder keeps its top bit free (the sign test needs |D| < 2^(32 dlen - 1))."""
import math
import random

import pytest

M32 = (1 << 32) - 1


def levels(n):
    """newton_levels in fpa_ops.cuh: k' -> k = (k'+2)/2 (k' = 2 from k = 1), bottom-up."""
    out, k = [n], n
    while k > 1:
        p = (k + 2) // 2
        if p >= k:
            p = k - 1
        k = p
        out.append(k)
    return out[::-1]


def residual(T, off, L, lt, neg):
    """ResidualMag: lt limbs of T from limb off, below limb L, complemented unless neg."""
    v = 0
    for i in range(lt):
        idx = off + i
        w = 0 if idx >= L else (T >> (32 * idx)) & M32
        if idx < L and not neg:
            w = ~w & M32
        v |= w << (32 * i)
    return v


def div_extra_limb(A, B, n):
    lv = levels(n)
    Y = (2 ** 64 - 1) // (B >> (32 * (n - 1)))
    for li in range(1, len(lv) - 1):
        k, kp = lv[li - 1], lv[li]
        T = (B >> (32 * (n - kp))) * Y
        L, lt = k + kp, kp - k + 3
        neg = (T >> (32 * L)) != 0
        M = ((Y * residual(T, k - 1, L, lt, neg)) >> (32 * (k + 1))) & ((1 << (32 * lt)) - 1)
        Ys = Y << (32 * (kp - k))
        Y = (Ys - M if neg else Ys + M) & ((1 << (32 * (kp + 1))) - 1)
    h = lv[-2]
    m = n + 2 - h
    q0 = ((A >> (32 * (n - m - 1))) * Y >> (32 * (h + 1))) & ((1 << (32 * (m + 1))) - 1)
    D = (A << 96) - ((q0 * B) >> (32 * (n - h - 1)))
    assert abs(D) < 1 << (32 * (m + 2)), "D exceeds the m+2 limbs the device multiplies"
    C = (abs(D) * Y) >> (32 * (h + 2))
    return (q0 << (32 * (h - 1))) + (-C if D < 0 else C)


def sqrt_extra_limb(Xh, n):
    lv = levels(n)
    Z = (2 ** 64 - 1) // math.isqrt((Xh >> (32 * n)) << 32)
    for li in range(1, len(lv) - 1):
        k, kp = lv[li - 1], lv[li]
        V1 = (Xh >> (32 * (n + 1 - kp))) * Z
        j = k - 2 if k > 2 else 0
        l1 = kp + k + 1 - j
        W = ((V1 >> (32 * j)) & ((1 << (32 * l1)) - 1)) * Z
        L, lt = kp + 2 * k - j, kp - k + 3
        neg = (W >> (32 * L)) != 0
        M = ((Z * residual(W, 2 * k - 1 - j, L, lt, neg)) >> (32 * (k + 1) + 1)) & ((1 << (32 * (kp + 1))) - 1)
        Zs = Z << (32 * (kp - k))
        Z = (Zs - M if neg else Zs + M) & ((1 << (32 * (kp + 1))) - 1)
    h = lv[-2]
    m = n + 2 - h
    S0 = ((Xh >> (32 * (n - m))) * Z >> (32 * (h + 1))) & ((1 << (32 * (m + 1))) - 1)
    D = (Xh << 96) - ((S0 * S0) << (32 * (2 * h - n)))
    assert abs(D) < 1 << (32 * (m + 3)), "D exceeds the m+3 limbs the device multiplies"
    C = (abs(D) * Z) >> (32 * (h + 3) + 1)
    return (S0 << (32 * (h - 1))) + (-C if D < 0 else C)


SIZES = [4, 5, 6, 7, 8, 9, 10, 16, 17, 18, 33, 65, 127, 128, 129, 257, 512]


@pytest.mark.parametrize("n", SIZES)
def test_extra_limb_error_is_a_few_units(n):
    rng = random.Random(n)
    top = 1 << (32 * n - 1)
    worst_div = worst_sqrt = 0
    for t in range(12):
        A = top | rng.getrandbits(32 * n - 1)
        B = top | rng.getrandbits(32 * n - 1)
        if t % 3 == 1:
            B = (1 << (32 * n)) - 1 - rng.getrandbits(20)        # divisor near the top of the binade
        if t % 3 == 2:
            B = top + rng.getrandbits(20)                         # and near the bottom
        Q = div_extra_limb(A, B, n)
        worst_div = max(worst_div, abs(Q - (A << (32 * (n + 1))) // B))
        odd = rng.getrandbits(1)
        Xh = A << (32 - odd)
        S = sqrt_extra_limb(Xh, n)
        worst_sqrt = max(worst_sqrt, abs(S - math.isqrt(Xh << (32 * (n - 1) + 64))))
    assert worst_div <= 16 and worst_sqrt <= 16, (worst_div, worst_sqrt)


# ---- the one-thread kernels: products restricted to the limbs their consumers read ---------
GUARD = 2


def blk(keep):
    """First 8-limb output block of a product kept from limb `keep` (fpa_thread_newton.cuh blk)."""
    return max(0, keep - GUARD) // 8


def tprod(x, lx, y, ly, cb_lo, cb_hi):
    """tprod: output blocks [cb_lo, cb_hi) of x * y, i.e. the sum of x_i y_j 2^(32(i+j)) over
    columns 8 cb_lo <= i + j < 8 cb_hi, carries out of the top block dropped."""
    c_lo, c_hi = 8 * cb_lo, 8 * min(cb_hi, (lx + ly + 7) // 8)
    s = 0
    for i in range(lx):
        xi = (x >> (32 * i)) & M32
        j0, j1 = max(0, c_lo - i), min(ly, c_hi - i)
        if xi and j0 < j1:
            s += (xi * ((y >> (32 * j0)) & ((1 << (32 * (j1 - j0))) - 1))) << (32 * (i + j0))
    return s & ((1 << (32 * c_hi)) - 1)


def limb(v, i):
    return (v >> (32 * i)) & M32


SMALL_LEVEL = 9


def small_levels_end(lv):
    """small_levels_end(lv, nl, true) in fpa_ops.cuh: the levels up to SMALL_LEVEL limbs run
    on one thread in registers, with the whole-product steps of div_extra_limb."""
    e = 1
    while e < len(lv) - 1 and lv[e] <= SMALL_LEVEL:
        e += 1
    return e


def div_level_whole(Y, B, n, k, kp):
    T = (B >> (32 * (n - kp))) * Y
    L, lt = k + kp, kp - k + 3
    neg = (T >> (32 * L)) != 0
    M = ((Y * residual(T, k - 1, L, lt, neg)) >> (32 * (k + 1))) & ((1 << (32 * lt)) - 1)
    Ys = Y << (32 * (kp - k))
    return (Ys - M if neg else Ys + M) & ((1 << (32 * (kp + 1))) - 1)


def sqrt_level_whole(Z, Xh, n, k, kp):
    V1 = (Xh >> (32 * (n + 1 - kp))) * Z
    j = k - 2 if k > 2 else 0
    l1 = kp + k + 1 - j
    W = ((V1 >> (32 * j)) & ((1 << (32 * l1)) - 1)) * Z
    L, lt = kp + 2 * k - j, kp - k + 3
    neg = (W >> (32 * L)) != 0
    M = ((Z * residual(W, 2 * k - 1 - j, L, lt, neg)) >> (32 * (k + 1) + 1)) & ((1 << (32 * (kp + 1))) - 1)
    Zs = Z << (32 * (kp - k))
    return (Zs - M if neg else Zs + M) & ((1 << (32 * (kp + 1))) - 1)


def tdiv_extra_limb(A, B, n):
    lv = levels(n)
    l0 = small_levels_end(lv)
    Y = (2 ** 64 - 1) // (B >> (32 * (n - 1)))
    for li in range(1, l0):
        Y = div_level_whole(Y, B, n, lv[li - 1], lv[li])
    for li in range(l0, len(lv) - 1):
        k, kp = lv[li - 1], lv[li]
        L, lt = k + kp, kp - k + 3
        T = tprod(B >> (32 * (n - kp)), kp, Y, k + 1, blk(k - 1), L // 8 + 1)
        neg = limb(T, L) != 0
        E = (T >> (32 * (k - 1))) & ((1 << (32 * lt)) - 1)
        if not neg:
            E ^= (1 << (32 * lt)) - 1
        P = tprod(Y, k + 1, E, lt, blk(k + 1), (k + 1 + lt + 7) // 8)
        M = (P >> (32 * (k + 1))) & ((1 << (32 * lt)) - 1)
        Ys = Y << (32 * (kp - k))
        Y = (Ys - M if neg else Ys + M) & ((1 << (32 * (kp + 1))) - 1)
    h = lv[-2]
    m = n + 2 - h
    q0 = (tprod(A >> (32 * (h - 3)), m + 1, Y, h + 1, blk(h + 1), (h + m + 9) // 8) >> (32 * (h + 1))) \
        & ((1 << (32 * (m + 1))) - 1)
    dlen, sh = m + 2, n - h - 1
    P = tprod(q0, m + 1, B, n, blk(sh), (sh + dlen + 7) // 8)
    Dm = ((A << 96) - (P >> (32 * sh))) & ((1 << (32 * dlen)) - 1)
    dneg = Dm >> (32 * dlen - 1)
    D = (1 << (32 * dlen)) - Dm if dneg else Dm
    exact_d = (A << 96) - ((q0 * B) >> (32 * sh))
    assert abs(exact_d) < 1 << (32 * dlen - 1), "the remainder's top bit is not free"
    C = tprod(D, dlen, Y, h + 1, blk(h + 2), (dlen + h + 8) // 8) >> (32 * (h + 2))
    return (q0 << (32 * (h - 1))) + (-C if dneg else C)


def tsqrt_extra_limb(Xh, n):
    lv = levels(n)
    l0 = small_levels_end(lv)
    Z = (2 ** 64 - 1) // math.isqrt((Xh >> (32 * n)) << 32)
    for li in range(1, l0):
        Z = sqrt_level_whole(Z, Xh, n, lv[li - 1], lv[li])
    for li in range(l0, len(lv) - 1):
        k, kp = lv[li - 1], lv[li]
        j = k - 2 if k > 2 else 0
        l1, L, lt, off = kp + k + 1 - j, kp + 2 * k - j, kp - k + 3, 2 * k - 1 - j
        V1 = tprod(Xh >> (32 * (n + 1 - kp)), kp, Z, k + 1, blk(j), (j + l1 + 7) // 8)
        V1s = (V1 >> (32 * j)) & ((1 << (32 * l1)) - 1)
        W = tprod(V1s, l1, Z, k + 1, blk(off), L // 8 + 1)
        neg = limb(W, L) != 0
        E = (W >> (32 * off)) & ((1 << (32 * lt)) - 1)
        if not neg:
            E ^= (1 << (32 * lt)) - 1
        P = tprod(Z, k + 1, E, lt, blk(k + 1), 1 << 20)
        M = (P >> (32 * (k + 1) + 1)) & ((1 << (32 * (kp + 1))) - 1)
        Zs = Z << (32 * (kp - k))
        Z = (Zs - M if neg else Zs + M) & ((1 << (32 * (kp + 1))) - 1)
    h = lv[-2]
    m = n + 2 - h
    S0 = (tprod(Xh >> (32 * (n - m)), m + 1, Z, h + 1, blk(h + 1), (h + m + 9) // 8) >> (32 * (h + 1))) \
        & ((1 << (32 * (m + 1))) - 1)
    dlen, ssh = m + 3, 2 * h - n
    sq = tprod(S0, m + 1, S0, m + 1, 0, (dlen - ssh + 7) // 8)
    Dm = ((Xh << 96) - (sq << (32 * ssh))) & ((1 << (32 * dlen)) - 1)
    dneg = Dm >> (32 * dlen - 1)
    D = (1 << (32 * dlen)) - Dm if dneg else Dm
    exact_d = (Xh << 96) - ((S0 * S0) << (32 * ssh))
    assert abs(exact_d) < 1 << (32 * dlen - 1), "the remainder's top bit is not free"
    C = tprod(D, dlen, Z, h + 1, blk(h + 3), 1 << 20) >> (32 * (h + 3) + 1)
    return (S0 << (32 * (h - 1))) + (-C if dneg else C)


THREAD_SIZES = [8, 9, 10, 11, 13, 16, 17, 18, 31, 32, 33, 48, 63, 64, 65, 96, 97, 127, 128]


@pytest.mark.parametrize("n", THREAD_SIZES)
def test_thread_extra_limb_error_is_a_few_units(n):
    rng = random.Random(1000 + n)
    top, full = 1 << (32 * n - 1), (1 << (32 * n)) - 1
    pairs = [(top | rng.getrandbits(32 * n - 1), top | rng.getrandbits(32 * n - 1)) for _ in range(10)]
    pairs += [(full, top), (top, full), (full, full), (top, top), (full - 1, full), (top + 1, full),
              (full, (1 << (32 * n)) - 1 - rng.getrandbits(20)), (top | rng.getrandbits(32 * n - 1), top + 1)]
    worst_div = worst_sqrt = 0
    for A, B in pairs:
        Q = tdiv_extra_limb(A, B, n)
        worst_div = max(worst_div, abs(Q - (A << (32 * (n + 1))) // B))
        for odd in (0, 1):
            Xh = A << (32 - odd)
            S = tsqrt_extra_limb(Xh, n)
            worst_sqrt = max(worst_sqrt, abs(S - math.isqrt(Xh << (32 * (n - 1) + 64))))
    assert worst_div <= 16 and worst_sqrt <= 16, (worst_div, worst_sqrt)
