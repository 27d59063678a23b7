"""The register add/sub (op_addsub_regk<G, K> and load_slots in
cubigfloat_gb300/csrc/fpa_addsub_regs.cuh), compiled for the host from the device source and
run on an emulated lane group: G host threads, one per lane, with every warp collective the
code uses (shuffle, shuffle up/down, ballot, broadcast) restated as publish -> group barrier ->
read.  This is faithful because op_addsub_regk reaches each collective with the whole group
(its early returns are group-uniform).  Results are checked bit-exact against the oracle on
the structured add/sub cases of the GPU tests, in every rounding mode, for lane-group shapes
the launcher uses (n = G*K, n just below it, n far below it, and n not a multiple of 4, which
takes the scalar load/store path).  The GPU tests run the same function in the real kernel."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from test_gpu_addsub import addsub_cases
from test_rows_host import extract

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc")

# (G, K) -> sizes n <= G*K
SHAPES = {
    (4, 2): [8, 5, 3],
    (4, 8): [32, 29, 12],
    (8, 4): [32, 30, 17],
    (4, 16): [64, 61, 36],
    (16, 4): [64, 33],
    (32, 8): [128, 9],
    (32, 16): [9],
}

SHIMS = r"""
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>
struct uint2 { uint32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
static inline uint2 make_uint2(uint32_t x, uint32_t y) { return uint2{x, y}; }
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }
template <class T> static inline T __ldcs(const T *p) { return *p; }
template <class T> static inline void __stcs(T *p, T v) { *p = v; }
static inline uint32_t __funnelshift_r(uint32_t lo, uint32_t hi, uint32_t sh) {
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> (sh & 31u));
}
static inline int __clz(int v) { return v == 0 ? 32 : __builtin_clz((unsigned)v); }

// One lane group emulated by G host threads.  A collective stores the caller's value in its
// slot, waits for all G lanes, then reads.  The slots alternate between two banks, so a lane
// that runs ahead to the next collective never overwrites a value another lane still reads.
struct GroupBarrier {                      // generation barrier; waiting lanes yield their core
  std::atomic<uint32_t> arrived{0}, gen{0};
  uint32_t lanes = 0;
  void arrive_and_wait() {
    const uint32_t g = gen.load(std::memory_order_acquire);
    if (arrived.fetch_add(1, std::memory_order_acq_rel) + 1 == lanes) {
      arrived.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_release);
    } else {
      while (gen.load(std::memory_order_acquire) == g) std::this_thread::yield();
    }
  }
};
static GroupBarrier *g_bar;
static uint32_t g_slot[2][32];
static thread_local uint32_t t_lane, t_round;
static inline const uint32_t *publish(uint32_t v) {
  uint32_t *bank = g_slot[t_round++ & 1u];
  bank[t_lane] = v;
  g_bar->arrive_and_wait();
  return bank;
}
static inline uint32_t __shfl_sync(uint32_t, uint32_t v, int src, int width) { return publish(v)[src & (width - 1)]; }
static inline uint32_t __shfl_down_sync(uint32_t, uint32_t v, unsigned d, int width) {
  const uint32_t *b = publish(v);
  return t_lane + d < (unsigned)width ? b[t_lane + d] : v;
}
static inline uint32_t __shfl_up_sync(uint32_t, uint32_t v, unsigned d, int) {
  const uint32_t *b = publish(v);
  return t_lane >= d ? b[t_lane - d] : v;
}
namespace gfpa {
template <int G>
struct Grp {
  uint32_t lane = t_lane, base = 0, mask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u);
  uint32_t ballot(bool p) const {
    const uint32_t *b = publish(p ? 1u : 0u);
    uint32_t m = 0;
    for (int i = 0; i < G; i++) m |= b[i] << i;
    return m;
  }
  uint32_t bcast(uint32_t v, int src) const { return __shfl_sync(mask, v, src, G); }
};
"""

MAIN = r"""
}  // namespace gfpa
using namespace gfpa;
struct Batch {
  int n, mode, is_sub, count; bool vec;
  uint32_t *ae, *be, *re, *a, *b, *r;
};
template <int G, int K>
static void lane_main(uint32_t lane, const Batch *bt) {
  t_lane = lane; t_round = 0;
  Grp<G> g;
  const int n = bt->n;
  for (int i = 0; i < bt->count; i++) {
    uint32_t av[K], bv[K];
    load_slots<G, K>(g, bt->a + (size_t)i * n, n, bt->vec, av);
    load_slots<G, K>(g, bt->b + (size_t)i * n, n, bt->vec, bv);
    op_addsub_regk<G, K>(g, n, bt->mode, bt->is_sub, bt->vec, bt->ae[i], av, bt->be[i], bv, bt->re + i,
                         bt->r + (size_t)i * n);
  }
}
template <int G, int K>
static void run_group(const Batch *bt) {
  GroupBarrier bar;
  bar.lanes = G;
  g_bar = &bar;
  std::vector<std::thread> lanes;
  for (uint32_t l = 0; l < (uint32_t)G; l++) lanes.emplace_back(lane_main<G, K>, l, bt);
  for (auto &t : lanes) t.join();
}
static uint32_t *words(size_t count) {
  const size_t bytes = ((count * 4 + 63) / 64) * 64 + 64;
  return static_cast<uint32_t *>(aligned_alloc(64, bytes));
}
int main() {
  int G, K, n, op, mode, count;
  while (scanf("%d %d %d %d %d %d", &G, &K, &n, &op, &mode, &count) == 6) {
    Batch bt{n, mode, op == 1, count, (n & 3) == 0, words(count), words(count), words(count),
             words((size_t)count * n), words((size_t)count * n), words((size_t)count * n)};
    for (int i = 0; i < count; i++) {
      unsigned x;
      if (scanf("%u", &x) != 1) return 1; bt.ae[i] = x;
      if (scanf("%u", &x) != 1) return 1; bt.be[i] = x;
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; bt.a[(size_t)i * n + j] = x; }
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; bt.b[(size_t)i * n + j] = x; }
    }
    memset(bt.re, 0xA5, (size_t)count * 4);
    memset(bt.r, 0xA5, (size_t)count * n * 4);
    switch (G * 100 + K) {
      case 402: run_group<4, 2>(&bt); break;
      case 408: run_group<4, 8>(&bt); break;
      case 804: run_group<8, 4>(&bt); break;
      case 416: run_group<4, 16>(&bt); break;
      case 1604: run_group<16, 4>(&bt); break;
      case 3208: run_group<32, 8>(&bt); break;
      case 3216: run_group<32, 16>(&bt); break;
      default: return 2;
    }
    for (int i = 0; i < count; i++) {
      printf("%u", bt.re[i]);
      for (int j = 0; j < n; j++) printf(" %u", bt.re[i] > CLS_SNAN ? bt.r[(size_t)i * n + j] : 0u);
      printf("\n");
    }
    free(bt.ae); free(bt.be); free(bt.re); free(bt.a); free(bt.b); free(bt.r);
  }
  return 0;
}
"""


def host_source():
    dev = open(os.path.join(CSRC, "fpa_device.cuh")).read()
    regs = open(os.path.join(CSRC, "fpa_addsub_regs.cuh")).read()
    parts = [
        extract(dev, "constexpr uint32_t BIAS", "// Special-value tables"),
        extract(dev, "static __constant__ uint8_t c_action", "static __constant__ uint8_t c_sqrt_action"),
        extract(dev, "__device__ __forceinline__ uint32_t classify", "// ----"),
        extract(dev, "__device__ __forceinline__ uint32_t clz32", "\n") + "\n",
        extract(dev, "// carry lookahead over the G lanes", "struct Zero"),
        extract(regs, "template <int K>\nstruct Log2", "// add/sub of numbers that fit K limbs per lane"),
    ]
    body = "\n".join(parts)
    body = body.replace("static __constant__", "static const")
    body = body.replace("__device__ __forceinline__", "static inline")
    body = body.replace("#pragma unroll", "")
    return SHIMS + body + MAIN


@pytest.fixture(scope="module")
def host_binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("regk")
    src, exe = d / "regk.cpp", d / "regk"
    src.write_text(host_source())
    r = subprocess.run([cxx, "-O2", "-std=c++20", "-fno-strict-aliasing", "-pthread", "-o", str(exe), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return str(exe)


def run_host(exe, G, K, n, batches):
    """batches: list of (op, mode, (ae, al, be, bl)); returns [(exps, limbs)] in order."""
    lines = []
    for op, mode, (ae, al, be, bl) in batches:
        lines.append(f"{G} {K} {n} {op} {mode} {len(ae)}")
        for i in range(len(ae)):
            lines.append(f"{int(ae[i])} {int(be[i])} " + " ".join(map(str, al[i])) + " " + " ".join(map(str, bl[i])))
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True,
                         timeout=600).stdout.strip().split("\n")
    res, pos = [], 0
    for _, _, (ae, _, _, _) in batches:
        rows = np.array([[int(x) for x in line.split()] for line in out[pos:pos + len(ae)]], dtype=np.uint64)
        pos += len(ae)
        res.append((rows[:, 0].astype(np.uint32), rows[:, 1:].astype(np.uint32)))
    assert pos == len(out)
    return res


@pytest.mark.parametrize("G,K,n", [(G, K, n) for (G, K), ns in SHAPES.items() for n in ns])
def test_register_addsub_matches_oracle(host_binary, G, K, n):
    rng = np.random.default_rng(7000 + 64 * G + K + n)
    cases = addsub_cases(rng, n)
    batches = [(op, mode, cases) for op in (0, 1) for mode in range(5)]
    got = run_host(host_binary, G, K, n, batches)
    for (op, mode, c), (ge, gl) in zip(batches, got):
        ee, el = oracle.run(op, n, mode, *c)
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (op, n, mode)
