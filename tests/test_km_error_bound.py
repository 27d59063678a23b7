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
  - the error is a few units (the device code comments quote <= 9 and <= 3)."""
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
