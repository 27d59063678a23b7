"""The one-thread row kernels' arithmetic (row_addsub<N> and row_mul<N> in
cubigfloat_gb300/csrc/fpa_addsub_rows.cuh), compiled for the host from the device source
with host stand-ins for the few GPU intrinsics they use (funnel shift, count leading zeros,
the mad.lo.cc / madc.hi.cc / addc chain), checked bit-exact against the oracle on the
structured add/sub cases and the mul cases of the GPU tests, in every rounding mode, for
N = 8, 16 and 32.  The GPU tests run the same functions in the real kernels."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from test_gpu_addsub import addsub_cases
from test_gpu_rows import mul_cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc")

SHIMS = r"""
#include <cstdint>
#include <cstdio>
#include <vector>
struct uint4 { uint32_t x, y, z, w; };
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }
static inline uint32_t __funnelshift_r(uint32_t lo, uint32_t hi, uint32_t sh) {
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> (sh & 31u));
}
static inline int __clz(int v) { return v == 0 ? 32 : __builtin_clz((unsigned)v); }
static inline uint32_t min(uint32_t a, uint32_t b) { return a < b ? a : b; }
namespace gfpa {
// mad.lo.cc / madc.hi.cc / addc: (lo, hi, tp) += a * b
static inline void mac3(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a, uint32_t b) {
  const uint64_t p = (uint64_t)a * b;
  const uint64_t s0 = (uint64_t)lo + (uint32_t)p;
  lo = (uint32_t)s0;
  const uint64_t s1 = (uint64_t)hi + (p >> 32) + (s0 >> 32);
  hi = (uint32_t)s1;
  tp += (uint32_t)(s1 >> 32);
}
"""

MAIN = r"""
}  // namespace gfpa
using namespace gfpa;
template <int N>
static int run(int op, int mode, int count) {
  constexpr int S = RowSpace<N>::S;
  std::vector<uint32_t> ra(S), rb(S);
  for (int t = 0; t < count; t++) {
    unsigned ae, be;
    if (scanf("%u %u", &ae, &be) != 2) return 1;
    for (int i = 0; i < N; i++) if (scanf("%u", &ra[i]) != 1) return 1;
    for (int i = 0; i < N; i++) if (scanf("%u", &rb[i]) != 1) return 1;
    const uint32_t e = op == 2 ? row_mul<N>(ra.data(), rb.data(), ae, be, mode)
                               : row_addsub<N>(ra.data(), rb.data(), ae, be, mode, op == 1);
    printf("%u", e);
    for (int i = 0; i < N; i++) printf(" %u", e > CLS_SNAN ? ra[i] : 0u);
    printf("\n");
  }
  return 0;
}
int main() {
  int op, n, mode, count;
  while (scanf("%d %d %d %d", &op, &n, &mode, &count) == 4) {
    int rc = n == 8 ? run<8>(op, mode, count) : n == 16 ? run<16>(op, mode, count) : run<32>(op, mode, count);
    if (rc) return rc;
  }
  return 0;
}
"""


def extract(src, start, end):
    a = src.index(start)
    b = src.index(end, a)
    return src[a:b]


def host_source():
    dev = open(os.path.join(CSRC, "fpa_device.cuh")).read()
    ops = open(os.path.join(CSRC, "fpa_ops.cuh")).read()
    rows = open(os.path.join(CSRC, "fpa_addsub_rows.cuh")).read()
    parts = [
        extract(dev, "constexpr uint32_t BIAS", "// Special-value tables"),
        extract(dev, "static __constant__ uint8_t c_action", "static __constant__ uint8_t c_sqrt_action"),
        extract(dev, "__device__ __forceinline__ uint32_t classify", "// ----"),
        extract(dev, "__device__ __forceinline__ uint32_t clz32", "\n", ) + "\n",
        extract(ops, "// exponent word from an unbiased exponent", "// ----"),
        extract(rows, "template <int N>\nstruct RowSpace", "// Copies of one warp's 32 operations"),
    ]
    body = "\n".join(parts)
    body = body.replace("static __constant__", "static const")
    body = re.sub(r"__device__\s+__forceinline__", "static inline", body)
    body = body.replace("#pragma unroll", "")
    return SHIMS + body + MAIN


@pytest.fixture(scope="module")
def host_binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("rows")
    src, exe = d / "rows.cpp", d / "rows"
    src.write_text(host_source())
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return str(exe)


def run_host(exe, op, n, mode, ae, al, be, bl):
    lines = [f"{op} {n} {mode} {len(ae)}"]
    for i in range(len(ae)):
        lines.append(f"{int(ae[i])} {int(be[i])} " + " ".join(map(str, al[i])) + " " + " ".join(map(str, bl[i])))
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout
    rows = np.array([[int(x) for x in line.split()] for line in out.strip().split("\n")], dtype=np.uint64)
    return rows[:, 0].astype(np.uint32), rows[:, 1:].astype(np.uint32)


@pytest.mark.parametrize("n", [8, 16, 32])
def test_row_addsub_and_mul_match_oracle(host_binary, n):
    rng = np.random.default_rng(1200 + n)
    cases = {0: addsub_cases(rng, n), 1: addsub_cases(rng, n), 2: mul_cases(rng, n)}
    for op, (ae, al, be, bl) in cases.items():
        for mode in range(5):
            ge, gl = run_host(host_binary, op, n, mode, ae, al, be, bl)
            ee, el = oracle.run(op, n, mode, ae, al, be, bl)
            assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
            val = ee > 8
            assert np.array_equal(gl[val], el[val]), (op, n, mode)
