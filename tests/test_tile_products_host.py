"""The one-thread product routines of cubigfloat_gb300/csrc/fpa_thread_newton.cuh (tprod:
one output block per pass with the zero half of edge tiles skipped; tprod2: two output blocks
per pass, mul's; tsqr: a square on its symmetric half), compiled for the host from the
device source and checked limb for limb against exact integer products, over a sweep of
operand lengths and output block ranges.  The number of limb products each routine executes
is counted too and compared with the model bench.py reports its executed-product roofline
from.

Operands are read through a checking view that holds each routine to the guard contract the
kernels' layouts provide: zeros from limb len up to 8 limbs past len rounded up to 8 and
in the 8 limbs below limb 0, and 8 more limbs on either side that are readable but hold
anything (here: a marker value, so a result that used one would be wrong).  A read outside
that range is reported as an error."""
import shutil
import subprocess

import numpy as np
import pytest

import bench
from test_thread_newton_host import host_body

MAIN = r"""
}  // namespace gfpa
using namespace gfpa;
static int g_bad = 0;
extern long g_mac3;
// a buffer of len limbs at stride TS with the guard zones of the kernels' layouts
struct Buf {
  std::vector<uint32_t> mem;
  int len, base, top;   // readable limbs: [-16, top)
  Buf(const std::vector<uint32_t> &v) : len((int)v.size()) {
    top = rup8(len) + 16;
    base = 16;
    mem.assign((size_t)TS * (base + top), 0u);
    for (int i = -16; i < top; i++) {
      uint32_t val = 0u;
      if (i < -8 || i >= rup8(len) + 8) val = 0xDEADBEEFu;       // readable, not zero
      else if (i >= 0 && i < len) val = v[i];
      mem[(size_t)TS * (base + i)] = val;
    }
  }
};
struct CV {                      // the unchecked view's reads, checked against the contract
  const Buf *b;
  uint32_t get(int i) const {
    if (i < -16 || i >= b->top) { g_bad = 1; return 0u; }
    return b->mem[(size_t)TS * (b->base + i)];
  }
};
int main() {
  int kind, lx, ly, cb_lo, cb_hi;
  // one case per line: kind lx ly cb_lo cb_hi x[0..lx) y[0..ly)   (kind 2: y ignored, ly = 0)
  while (scanf("%d %d %d %d %d", &kind, &lx, &ly, &cb_lo, &cb_hi) == 5) {
    std::vector<uint32_t> x(lx), y(ly);
    for (auto &v : x) { unsigned t; if (scanf("%u", &t) != 1) return 1; v = t; }
    for (auto &v : y) { unsigned t; if (scanf("%u", &t) != 1) return 1; v = t; }
    Buf bx(x), by(kind == 2 ? x : y);
    std::vector<uint32_t> out;
    int expect_cb = cb_lo;
    auto sink = [&](int cb, const uint32_t (&o)[10]) {
      if (cb != expect_cb) g_bad = 1;
      expect_cb++;
      for (int q = 0; q < 8; q++) out.push_back(o[q]);
    };
    g_bad = 0;
    g_mac3 = 0;
    if (kind == 0) tprod(CV{&bx}, lx, CV{&by}, ly, cb_lo, cb_hi, sink);
    else if (kind == 1) tprod2(CV{&bx}, lx, CV{&by}, ly, cb_lo, cb_hi, sink);
    else tsqr(CV{&bx}, lx, cb_hi, sink);
    printf("%d %ld %d", g_bad, g_mac3, (int)out.size());
    for (uint32_t v : out) printf(" %u", v);
    printf("\n");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("tiles")
    src, out = d / "tiles.cpp", d / "tiles"
    src.write_text(counting(host_body()) + MAIN)
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-o", str(out), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return str(out)


MAC3 = "static inline void mac3(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a, uint32_t b) {"


def counting(body):
    """The host source with every mac3 call counted (g_mac3)."""
    assert body.count(MAC3) == 1
    return body.replace(MAC3, "}\nlong g_mac3 = 0;\nnamespace gfpa {\n" + MAC3 + "\n  g_mac3++;")


def to_int(limbs):
    v = 0
    for w in reversed(limbs):
        v = (v << 32) | int(w)
    return v


def expected(x, y, cb_lo, cb_hi):
    """Limbs 8cb_lo .. of the column sums from column 8cb_lo up (no carry from below), through
    block min(Mx + My, cb_hi) - 1."""
    lx, ly = len(x), len(y)
    mx, my = (lx + 7) // 8, (ly + 7) // 8
    mo = min(mx + my, cb_hi)
    if mo <= cb_lo:
        return []
    c0 = 8 * cb_lo
    X, Y = to_int(x), to_int(y)
    low = 0                                   # the columns below c0
    for i in range(min(lx, c0)):
        low += int(x[i]) * (Y & ((1 << (32 * (c0 - i))) - 1)) << (32 * i)
    v = (X * Y - low) >> (32 * c0)
    nl = 8 * (mo - cb_lo)
    return [(v >> (32 * k)) & 0xFFFFFFFF for k in range(nl)]


def limbs(rng, n, kind):
    if kind == "ones":
        return [0xFFFFFFFF] * n
    if kind == "top":
        v = [0] * n
        v[-1] = 0x80000000
        return v
    return [int(t) for t in rng.integers(0, 1 << 32, n, dtype=np.uint64)]


LENGTHS = [1, 2, 7, 8, 9, 15, 16, 17, 24, 31, 33, 40, 63, 64, 66, 72, 127, 128, 130]


def cases(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        lx, ly = int(rng.choice(LENGTHS)), int(rng.choice(LENGTHS))
        mx, my = (lx + 7) // 8, (ly + 7) // 8
        cb_lo = int(rng.integers(0, mx + my))
        cb_hi = int(rng.choice([cb_lo + 1, cb_lo + 2, cb_lo + 3, int(rng.integers(cb_lo + 1, mx + my + 2)), 1 << 20]))
        pat = str(rng.choice(["rand", "rand", "ones", "top"]))
        out.append((lx, ly, cb_lo, cb_hi, limbs(rng, lx, pat), limbs(rng, ly, pat)))
    return out


def run(exe, lines):
    res = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout
    return [list(map(int, line.split())) for line in res.strip().split("\n")]


@pytest.mark.parametrize("kind", [0, 1])
def test_products_match_integers(exe, kind):
    cs = cases(100 + kind, 1500)
    lines = [f"{kind} {lx} {ly} {lo} {hi} " + " ".join(map(str, x + y)) for lx, ly, lo, hi, x, y in cs]
    for (lx, ly, lo, hi, x, y), row in zip(cs, run(exe, lines)):
        bad, macs, n, got = row[0], row[1], row[2], row[3:]
        assert bad == 0, ("read outside the guard zones or block order", kind, lx, ly, lo, hi)
        assert got == expected(x, y, lo, hi), (kind, lx, ly, lo, hi)
        assert n == len(got)
        # limb products executed = the bench's model (tprod2 adds 2 carry steps per block pair)
        mo = min((lx + 7) // 8 + (ly + 7) // 8, hi)
        if kind == 0:
            assert macs == bench._tprod(lx, ly, lo, hi), (lx, ly, lo, hi)
        else:
            assert macs == bench._tprod2(lx, ly, lo, hi) + 2 * (max(0, mo - lo) // 2), (lx, ly, lo, hi)


def test_square_matches_integers(exe):
    rng = np.random.default_rng(7)
    cs = []
    for lx in LENGTHS:
        mx = (lx + 7) // 8
        for cb_hi in sorted({1, 2, 3, mx, mx + 1, 2 * mx - 1, 2 * mx, 1 << 20}):
            if cb_hi < 1:
                continue
            for pat in ("rand", "ones", "top"):
                cs.append((lx, cb_hi, limbs(rng, lx, pat)))
    lines = [f"2 {lx} 0 0 {hi} " + " ".join(map(str, x)) for lx, hi, x in cs]
    for (lx, hi, x), row in zip(cs, run(exe, lines)):
        bad, macs, got = row[0], row[1], row[3:]
        assert bad == 0, ("read outside the guard zones or block order", lx, hi)
        assert got == expected(x, x, 0, hi), (lx, hi)
        # the bench's model plus 2 carry steps per block
        assert macs == bench._tsqr(lx, hi) + 2 * min(2 * ((lx + 7) // 8), hi), (lx, hi)


def test_two_block_product_equals_one_block(exe):
    """tprod2 and tprod give the same limbs (the kernels use one or the other by operation)."""
    cs = cases(5, 600)
    l0 = [f"0 {lx} {ly} {lo} {hi} " + " ".join(map(str, x + y)) for lx, ly, lo, hi, x, y in cs]
    l1 = [f"1 {lx} {ly} {lo} {hi} " + " ".join(map(str, x + y)) for lx, ly, lo, hi, x, y in cs]
    r0, r1 = run(exe, l0), run(exe, l1)
    assert [[r[0]] + r[2:] for r in r0] == [[r[0]] + r[2:] for r in r1]
