"""The one-lane Newton levels of div and sqrt (small_levels in cubigfloat_gb300/csrc/fpa_ops.cuh)
must produce the same iterates as the group levels they replace.  The device code of
small_levels and newton_levels is compiled for the host (its qualifiers stripped) and its
iterates are compared with the group levels' integer steps restated in Python (the same
restatement the error-bound test uses)."""
import math
import os
import random
import re
import shutil
import subprocess

import pytest

from test_km_error_bound import levels, residual

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OPS = os.path.join(ROOT, "cubigfloat_gb300", "csrc", "fpa_ops.cuh")
SMALL = 9
M32 = (1 << 32) - 1

HOST_MAIN = r"""
using namespace gfpa;
int main() {
  int mode, n;
  while (scanf("%d %d", &mode, &n) == 2) {
    uint32_t top[SMALL_LEVEL]; unsigned long long first;
    for (int i = 0; i < SMALL_LEVEL; i++) { unsigned x; if (scanf("%u", &x) != 1) return 1; top[i] = x; }
    if (scanf("%llu", &first) != 1) return 1;
    int lv[24]; const int nl = newton_levels(n, lv);
    const int end = small_levels_end(lv, nl, n >= 4);
    uint32_t v[SMALL_LEVEL + 1] = {0}; v[0] = (uint32_t)first; v[1] = (uint32_t)(first >> 32);
    if (mode) small_levels<true>(top, lv, end, v); else small_levels<false>(top, lv, end, v);
    printf("%d", lv[end - 1]);
    for (int i = 0; i <= SMALL_LEVEL; i++) printf(" %u", v[i]);
    printf("\n");
  }
  return 0;
}
"""


def host_source():
    src = open(OPS).read()
    a = src.index("__device__ __forceinline__ int newton_levels")
    b = src.index("\n}\n", a) + 3
    c = src.index("constexpr int SMALL_LEVEL")
    d = src.index("// ---------------------------------------------------------------------------------------\n// div.", c)
    body = src[a:b] + src[c:d]
    body = re.sub(r"__device__\s+__forceinline__", "static inline", body)
    body = re.sub(r"__device__\s+__noinline__", "static", body)
    return "#include <cstdint>\n#include <cstdio>\nnamespace gfpa {\n" + body + "}\n" + HOST_MAIN


def group_div_levels(B, n, upto):
    lv = levels(n)
    Y = (2 ** 64 - 1) // (B >> (32 * (n - 1)))
    for li in range(1, upto):
        k, kp = lv[li - 1], lv[li]
        T = (B >> (32 * (n - kp))) * Y
        L, lt = k + kp, kp - k + 3
        neg = (T >> (32 * L)) != 0
        M = ((Y * residual(T, k - 1, L, lt, neg)) >> (32 * (k + 1))) & ((1 << (32 * lt)) - 1)
        Ys = Y << (32 * (kp - k))
        Y = (Ys - M if neg else Ys + M) & ((1 << (32 * (kp + 1))) - 1)
    return Y


def group_sqrt_levels(Xh, n, upto):
    lv = levels(n)
    Z = (2 ** 64 - 1) // math.isqrt((Xh >> (32 * n)) << 32)
    for li in range(1, upto):
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
    return Z


@pytest.fixture(scope="module")
def host_binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("small_levels")
    src, exe = d / "levels.cpp", d / "levels"
    src.write_text(host_source())
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return str(exe)


def test_one_lane_levels_equal_group_levels(host_binary):
    rng = random.Random(3)
    lines, expect = [], []
    for n in list(range(1, 40)) + [64, 100, 127, 128, 129, 255, 256, 512]:
        lv = levels(n)
        last = len(lv) - 1 if n >= 4 else len(lv)
        end = 1
        while end < last and lv[end] <= SMALL:
            end += 1
        for t in range(8):
            B = (1 << (32 * n - 1)) | rng.getrandbits(32 * n - 1)
            if t % 3 == 1:
                B = (1 << (32 * n)) - 1 - rng.getrandbits(16)
            top = [((B >> (32 * (n - SMALL + i))) & M32) if n - SMALL + i >= 0 else 0 for i in range(SMALL)]
            lines.append(f"0 {n} " + " ".join(map(str, top)) + f" {(2 ** 64 - 1) // (B >> (32 * (n - 1)))}")
            expect.append((lv[end - 1], group_div_levels(B, n, end)))
            Xh = B << (32 - rng.getrandbits(1))
            xt = [((Xh >> (32 * (n + 1 - SMALL + i))) & M32) if n + 1 - SMALL + i >= 0 else 0 for i in range(SMALL)]
            z1 = (2 ** 64 - 1) // math.isqrt((Xh >> (32 * n)) << 32)
            lines.append(f"1 {n} " + " ".join(map(str, xt)) + f" {z1}")
            expect.append((lv[end - 1], group_sqrt_levels(Xh, n, end)))
    out = subprocess.run([host_binary], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = out.stdout.strip().split("\n")
    assert len(got) == len(expect)
    for line, (k, value), inp in zip(got, expect, lines):
        f = [int(x) for x in line.split()]
        assert f[0] == k and sum(v << (32 * i) for i, v in enumerate(f[1:])) == value, inp[:60]
