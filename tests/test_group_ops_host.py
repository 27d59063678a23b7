"""The lane-group add/sub, mul, div, sqrt and fma (op_addsub, op_mul, op_div, op_sqrt, op_fma
in cubigfloat_gb300/csrc/fpa_ops.cuh, with every building block of fpa_device.cuh under
them) and the elementwise kernels' double-buffered add/sub and mul loops, compiled for the
host from the device source and run on an emulated lane group: G host threads, one per
lane, sharing the group's workspace as the kernel's shared-memory slice.  Each warp
collective becomes publish -> group barrier -> read, and the group sync (__syncwarp)
becomes the barrier alone; the few inline PTX carry chains get host equivalents.  Results
are checked bit-exact against the oracle in every rounding mode on random operands,
near-halfway / near-exact cases, all-ones mantissas and the special classes (fma: the
seeded fma cases with cancellation, and every class combination), for the lane-group
shapes the tuned table uses, at sizes from one limb up to the group's capacity.  A div/sqrt
internal check that fails sets the error word, which must stay 0.  A ThreadSanitizer build
checks that lanes touch shared words only in an order the syncs and collectives fix.  The
GPU tests run the same functions in the kernels."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from cubigfloat_gb300 import workloads as W
from fma_cases import fma_cases, special_cases
from test_gpu_addsub import addsub_cases
from test_gpu_rows import mul_cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc")

# (G, K, R) of the lane-group configurations the tuned table uses for mul, div and sqrt
# (0, 1, 2, 3, 5, 6, 7, 10, 11, 12, 14) and configuration 15 -> sizes n <= G*K*R
SHAPES = {
    (4, 2, 1): [1, 2, 3, 5, 8],
    (8, 2, 1): [13, 16],
    (8, 4, 1): [9, 10, 17, 32],
    (16, 4, 1): [64],
    (8, 4, 2): [33, 64],
    (16, 8, 1): [128],
    (8, 4, 4): [97, 128],
    (16, 4, 2): [100, 128],
    (4, 4, 8): [128],
    (16, 8, 2): [256],
    (32, 8, 1): [256],
    (32, 16, 1): [512],
}
# operand-set sample per op at these sizes and above (first and last cases kept)
SAMPLE_FROM, SAMPLE = 256, 48

SHIMS = r"""
#include <atomic>
#include <chrono>
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
static inline uint32_t __funnelshift_r(uint32_t lo, uint32_t hi, uint32_t sh) {
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> (sh & 31u));
}
static inline uint32_t __funnelshift_l(uint32_t lo, uint32_t hi, uint32_t sh) {
  return (uint32_t)(((((uint64_t)hi << 32) | lo) << (sh & 31u)) >> 32);
}
static inline int __clz(int v) { return v == 0 ? 32 : __builtin_clz((unsigned)v); }
static inline int __clzll(long long v) { return v == 0 ? 64 : __builtin_clzll((unsigned long long)v); }
static inline uint32_t __umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
static inline uint64_t __umul64hi(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }
static inline int __popc(uint32_t v) { return __builtin_popcount(v); }
template <class T> static inline T __ldcs(const T *p) { return *p; }
template <class T> static inline T __ldg(const T *p) { return *p; }
template <class T> static inline void __stcs(T *p, T v) { *p = v; }
static inline uint32_t atomicOr(uint32_t *p, uint32_t v) { return __atomic_fetch_or(p, v, __ATOMIC_RELAXED); }
using std::min;
using std::max;

// One lane group emulated by G host threads.  A collective stores the caller's value in its
// slot, waits for all G lanes, then reads.  The slots alternate between two banks, so a lane
// that runs ahead to the next collective never overwrites a value another lane still reads.
// A wait that outlasts 60 s (a collective some lane never reaches) ends the program.
struct GroupBarrier {
  std::atomic<uint32_t> arrived{0}, gen{0};
  uint32_t lanes = 0;
  void arrive_and_wait() {
    const uint32_t g = gen.load(std::memory_order_acquire);
    if (arrived.fetch_add(1, std::memory_order_acq_rel) + 1 == lanes) {
      arrived.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_release);
      return;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (uint64_t spin = 0; gen.load(std::memory_order_acquire) == g; spin++) {
      std::this_thread::yield();
      if ((spin & 0xFFFF) == 0 && std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60)) {
        fprintf(stderr, "lane group barrier timed out\n");
        std::_Exit(3);
      }
    }
  }
};
struct GroupCtx {                           // one lane group: its barrier and its two slot banks
  GroupBarrier bar;
  uint32_t slot[2][32];
};
static thread_local GroupCtx *t_ctx;
static thread_local uint32_t t_lane, t_round;
static inline const uint32_t *publish(uint32_t v) {
  uint32_t *bank = t_ctx->slot[t_round++ & 1u];
  bank[t_lane] = v;
  t_ctx->bar.arrive_and_wait();
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
static inline uint32_t __shfl_xor_sync(uint32_t, uint32_t v, int m, int width) {
  return publish(v)[(t_lane ^ (uint32_t)m) & (uint32_t)(width - 1)];
}
// (lo, hi, tp) -= (a0, a1, a2) with borrows: the sub.cc / subc.cc / subc chain
static inline void sub3(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a0, uint32_t a1, uint32_t a2) {
  const uint64_t s0 = (uint64_t)lo - a0;
  lo = (uint32_t)s0;
  const uint64_t s1 = (uint64_t)hi - a1 - (uint32_t)(s0 >> 63);
  hi = (uint32_t)s1;
  tp = tp - a2 - (uint32_t)(s1 >> 63);
}
"""

HOST_GRP = r"""template <int G>
struct Grp {
  uint32_t lane = t_lane, base = 0, mask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u);
  void sync() const { t_ctx->bar.arrive_and_wait(); }
  uint32_t ballot(bool p) const {
    const uint32_t *b = publish(p ? 1u : 0u);
    uint32_t m = 0;
    for (int i = 0; i < G; i++) m |= b[i] << i;
    return m;
  }
  uint32_t bcast(uint32_t v, int src) const { return __shfl_sync(mask, v, src, G); }
  uint32_t rmin(uint32_t v) const {
    const uint32_t *b = publish(v);
    uint32_t m = b[0];
    for (int i = 1; i < G; i++) m = b[i] < m ? b[i] : m;
    return m;
  }
  uint32_t rmax(uint32_t v) const {
    const uint32_t *b = publish(v);
    uint32_t m = b[0];
    for (int i = 1; i < G; i++) m = b[i] > m ? b[i] : m;
    return m;
  }
  uint32_t ror(uint32_t v) const {
    const uint32_t *b = publish(v);
    uint32_t m = 0;
    for (int i = 0; i < G; i++) m |= b[i];
    return m;
  }
};
"""

# cp.async lands at the latest point it may: each copy is recorded when issued and made
# when the issuing lane's wait retires its group.
HOST_ASYNC = r"""struct AsyncCopy { uint32_t *dst; const uint32_t *src; int words; };
static thread_local std::vector<AsyncCopy> t_open;
static thread_local std::vector<std::vector<AsyncCopy>> t_groups;
static inline void cp_async4(uint32_t *dst, const uint32_t *src) { t_open.push_back({dst, src, 1}); }
static inline void cp_async16(uint32_t *dst, const uint32_t *src) { t_open.push_back({dst, src, 4}); }
static inline void cp_async_commit() { t_groups.push_back(t_open); t_open.clear(); }
template <int PENDING>
static inline void cp_async_wait() {
  while ((int)t_groups.size() > PENDING) {
    for (const AsyncCopy &c : t_groups.front()) memcpy(c.dst, c.src, 4 * (size_t)c.words);
    t_groups.erase(t_groups.begin());
  }
}
"""

HOST_MAC3 = r"""static inline void mac3(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a, uint32_t b) {
  const uint64_t p = (uint64_t)a * b;
  const uint64_t s0 = (uint64_t)lo + (uint32_t)p;
  lo = (uint32_t)s0;
  const uint64_t s1 = (uint64_t)hi + (p >> 32) + (s0 >> 32);
  hi = (uint32_t)s1;
  tp += (uint32_t)(s1 >> 32);
}
"""

MAIN = r"""
using namespace gfpa;
struct Batch {
  int op, n, mode, count;
  uint32_t *ae, *be, *ce, *re, *a, *b, *c, *r, *ws;
  uint32_t err;
};
template <int G, int K, int R>
static void lane_main(uint32_t lane, Batch *bt, GroupCtx *ctx) {
  t_lane = lane; t_round = 0; t_ctx = ctx;
  Grp<G> g;
  const int n = bt->n;
  for (int i = 0; i < bt->count; i++) {
    const size_t o = (size_t)i * n;
    if (bt->op == OP_ADD || bt->op == OP_SUB)
      op_addsub<G, K, R>(g, bt->ws, n, bt->mode, bt->op == OP_SUB, bt->ae[i], bt->a + o, bt->be[i], bt->b + o,
                         bt->re + i, bt->r + o);
    else if (bt->op == OP_MUL)
      op_mul<G, K, R>(g, bt->ws, n, bt->mode, bt->ae[i], bt->a + o, bt->be[i], bt->b + o, bt->re + i, bt->r + o);
    else if (bt->op == OP_DIV)
      op_div<G, K, R>(g, bt->ws, n, bt->mode, bt->ae[i], bt->a + o, bt->be[i], bt->b + o, bt->re + i, bt->r + o,
                      &bt->err);
    else if (bt->op == OP_SQRT)
      op_sqrt<G, K, R>(g, bt->ws, n, bt->mode, bt->ae[i], bt->a + o, bt->re + i, bt->r + o, &bt->err);
    else
      op_fma<G, K, R>(g, bt->ws, n, bt->mode, bt->ae[i], bt->a + o, bt->be[i], bt->b + o, bt->ce[i], bt->c + o,
                      bt->re + i, bt->r + o);
    g.sync();
  }
}
// the elementwise kernels' pipelined loops, one group taking every operation in turn
// (ops 10 / 11 / 12 / 16: add, sub, mul, mul with the Karatsuba split)
template <int G, int K, int R>
static void lane_pipe(uint32_t lane, Batch *bt, GroupCtx *ctx) {
  t_lane = lane; t_round = 0; t_ctx = ctx;
  Grp<G> g;
  ElementwiseArgs args{};
  args.count = (uint64_t)bt->count; args.n = (uint32_t)bt->n; args.mode = bt->mode;
  args.r_exps = bt->re; args.r_limbs = bt->r; args.a_exps = bt->ae; args.a_limbs = bt->a;
  args.b_exps = bt->be; args.b_limbs = bt->b; args.err = &bt->err;
  if (bt->op == 10) addsub_pipelined<OP_ADD, G, K, R>(g, bt->ws, args, 0, 1);
  else if (bt->op == 11) addsub_pipelined<OP_SUB, G, K, R>(g, bt->ws, args, 0, 1);
  else if (bt->op == 12) mul_pipelined<G, K, R, false>(g, bt->ws, args, 0, 1);
  else mul_pipelined<G, K, R, true>(g, bt->ws, args, 0, 1);
}
template <int G, int K, int R>
static void run_group(Batch *bt) {
  const int words = bt->op >= 10 ? (bt->op <= 11 ? PipeWords<OP_ADD, G, K, R>::aligned()
                                    : bt->op == 12 ? PipeWords<OP_MUL, G, K, R>::aligned()
                                                   : PipeWords<OP_MUL_KARA, G, K, R>::aligned())
                    : bt->op <= OP_SUB ? OpWords<OP_ADD, G, K, R>::aligned()
                    : bt->op == OP_MUL ? OpWords<OP_MUL, G, K, R>::aligned()
                    : bt->op == OP_DIV ? OpWords<OP_DIV, G, K, R>::aligned()
                    : bt->op == OP_SQRT ? OpWords<OP_SQRT, G, K, R>::aligned() : OpWords<OP_FMA, G, K, R>::aligned();
  std::vector<uint32_t> ws((size_t)words + 16, 0x5A5A5A5Au);
  bt->ws = ws.data();
  GroupCtx ctx;
  ctx.bar.lanes = G;
  std::vector<std::thread> lanes;
  for (uint32_t l = 0; l < (uint32_t)G; l++)
    lanes.emplace_back(bt->op >= 10 ? lane_pipe<G, K, R> : lane_main<G, K, R>, l, bt, &ctx);
  for (auto &t : lanes) t.join();
  for (int i = words; i < words + 16; i++)
    if (ws[i] != 0x5A5A5A5Au) { fprintf(stderr, "workspace overrun\n"); std::_Exit(4); }
}
static uint32_t *alloc_words(size_t count) {
  const size_t bytes = ((count * 4 + 63) / 64) * 64 + 64;
  return static_cast<uint32_t *>(aligned_alloc(64, bytes));
}
int main() {
  int G, K, R, op, n, mode, count;
  while (scanf("%d %d %d %d %d %d %d", &G, &K, &R, &op, &n, &mode, &count) == 7) {
    Batch bt{op, n, mode, count, alloc_words(count), alloc_words(count), alloc_words(count), alloc_words(count),
             alloc_words((size_t)count * n), alloc_words((size_t)count * n), alloc_words((size_t)count * n),
             alloc_words((size_t)count * n), nullptr, 0u};
    for (int i = 0; i < count; i++) {
      unsigned x;
      if (scanf("%u", &x) != 1) return 1; bt.ae[i] = x;
      if (scanf("%u", &x) != 1) return 1; bt.be[i] = x;
      if (scanf("%u", &x) != 1) return 1; bt.ce[i] = x;
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; bt.a[(size_t)i * n + j] = x; }
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; bt.b[(size_t)i * n + j] = x; }
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; bt.c[(size_t)i * n + j] = x; }
    }
    memset(bt.re, 0xA5, (size_t)count * 4);
    memset(bt.r, 0xA5, (size_t)count * n * 4);
    switch (G * 10000 + K * 100 + R) {
@CASES@      default: return 2;
    }
    printf("err %u\n", bt.err);
    for (int i = 0; i < count; i++) {
      printf("%u", bt.re[i]);
      for (int j = 0; j < n; j++) printf(" %u", bt.re[i] > CLS_SNAN ? bt.r[(size_t)i * n + j] : 0u);
      printf("\n");
    }
    free(bt.ae); free(bt.be); free(bt.ce); free(bt.re); free(bt.a); free(bt.b); free(bt.c); free(bt.r);
  }
  return 0;
}
"""


def _replace_once(src, start, end, new):
    a = src.index(start)
    b = src.index(end, a) + len(end)
    assert src.find(start, b) < 0, start
    return src[:a] + new + src[b:]


def _host_qualifiers(text):
    for a, b in (("__device__ __forceinline__", "inline"), ("__device__ __noinline__", ""),
                 ("__host__ __device__", ""), ("static __constant__", "static const"), ("__device__", ""),
                 ("__restrict__", "__restrict")):
        text = text.replace(a, b)
    return re.sub(r"#pragma unroll[^\n]*", "", text)


def host_source():
    dev = open(os.path.join(CSRC, "fpa_device.cuh")).read()
    ops = open(os.path.join(CSRC, "fpa_ops.cuh")).read()
    kern = open(os.path.join(CSRC, "fpa_kernels.cu")).read()
    launch = open(os.path.join(CSRC, "fpa_launch.h")).read()
    dev = _replace_once(dev, "template <int G>\nstruct Grp {", "\n};\n", HOST_GRP)
    dev = _replace_once(dev, "__device__ __forceinline__ void cp_async4(",
                        ': "memory"); }\n\n', HOST_ASYNC + "\n")
    dev = _replace_once(dev, "__device__ __forceinline__ void mac3(", '"r"(a), "r"(b));\n}\n', HOST_MAC3)
    dev = _replace_once(dev, 'asm("sub.cc.u32', '"r"(a0), "r"(a1), "r"(a2));',
                        "sub3(lo[c], hi[c], tp[c], a0, a1, a2);")
    at = launch.index("struct ElementwiseArgs {")
    args = launch[at:launch.index("};", at) + 3]
    pipe = kern[kern.index("// add/sub: HBM-bound"):kern.index("// sqrt may run CTAs")]
    body = dev + "\n" + ops + "\nnamespace gfpa {\n" + pipe + "}  // namespace gfpa\n"
    body = args + body
    assert "asm" not in body.replace("asm(", "").replace("asm ", "") or True
    lines = [ln for ln in body.split("\n") if not ln.startswith("#pragma once") and not ln.startswith("#include")]
    body = "\n".join(lines)
    body = _host_qualifiers(body)
    assert "asm(" not in body and "asm volatile" not in body
    cases = "".join(f"      case {G * 10000 + K * 100 + R}: run_group<{G}, {K}, {R}>(&bt); break;\n"
                    for (G, K, R) in SHAPES)
    return SHIMS + body + MAIN.replace("@CASES@", cases)


def device_source(kernel_start, kernel_end, extra_shims=""):
    """SHIMS + fpa_device.cuh + fpa_ops.cuh + the part of fpa_kernels.cu between the two
    markers, transformed for the host (no main)."""
    src = host_source()
    kern = open(os.path.join(CSRC, "fpa_kernels.cu")).read()
    part = kern[kern.index(kernel_start):kern.index(kernel_end)]
    a = src.index("namespace gfpa {\n// add/sub: HBM-bound")
    b = src.index("}  // namespace gfpa\n", a) + len("}  // namespace gfpa\n")
    part = _host_qualifiers(part)
    return extra_shims + src[:a] + "namespace gfpa {\n" + part + "}  // namespace gfpa\n" + src[b:src.index(MAIN[:40])]


@pytest.fixture(scope="module")
def host_binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("group_ops")
    src, exe = d / "group_ops.cpp", d / "group_ops"
    src.write_text(host_source())
    r = subprocess.run([cxx, "-O2", "-std=c++20", "-fno-strict-aliasing", "-pthread", "-w", "-o", str(exe), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return str(exe)


def run_host(exe, shape, n, batches):
    """batches: list of (op, mode, (ae, al, be, bl[, ce, cl])); returns [(err, exps, limbs)] in order."""
    G, K, R = shape
    lines = []
    for op, mode, case in batches:
        ae, al, be, bl = case[:4]
        ce, cl = case[4:] if len(case) == 6 else (np.zeros_like(ae), np.zeros_like(al))
        lines.append(f"{G} {K} {R} {op} {n} {mode} {len(ae)}")
        for i in range(len(ae)):
            lines.append(f"{int(ae[i])} {int(be[i])} {int(ce[i])} " + " ".join(map(str, al[i])) + " "
                         + " ".join(map(str, bl[i])) + " " + " ".join(map(str, cl[i])))
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    out = r.stdout.strip().split("\n")
    res, pos = [], 0
    for _, _, (ae, *_) in batches:
        assert out[pos].startswith("err ")
        err = int(out[pos].split()[1])
        rows = np.array([[int(x) for x in line.split()] for line in out[pos + 1:pos + 1 + len(ae)]], dtype=np.uint64)
        pos += 1 + len(ae)
        res.append((err, rows[:, 0].astype(np.uint32), rows[:, 1:].astype(np.uint32)))
    assert pos == len(out)
    return res


def div_cases(rng, n):
    ae, al = W.uniform(rng, 120, n, -300, 300)
    be, bl = W.uniform(rng, 120, n, -300, 300)
    extra_a, extra_b = [], []
    for _ in range(24):
        A, B = W.div_near_exact(rng, n)
        extra_a.append((W.exp_word(int(rng.integers(-9, 9)), int(rng.integers(0, 2))), W.int_to_limbs(A, n)))
        extra_b.append((W.exp_word(int(rng.integers(-9, 9)), int(rng.integers(0, 2))), W.int_to_limbs(B, n)))
    ones = np.full(n, 0xFFFFFFFF, np.uint32)
    top = W.int_to_limbs(1 << (32 * n - 1), n)
    extra_a += [(W.exp_word(3, 0), ones), (W.exp_word(3, 0), top), (W.exp_word(3, 1), ones)]
    extra_b += [(W.exp_word(1, 0), top), (W.exp_word(1, 0), ones), (W.exp_word(2, 0), ones)]
    for wa, wb in ((6, BIAS_W + 2), (6, BIAS_W - 2), (0x7FFFFFF0, BIAS_W - 20), (0x7FFFFFFF, BIAS_W)):
        for sa, sb in ((0, 0), (1, 0)):
            extra_a.append((np.uint32(2 * wa + sa), W.uniform(rng, 1, n, 0, 0)[1][0]))
            extra_b.append((np.uint32(2 * wb + sb), W.uniform(rng, 1, n, 0, 0)[1][0]))
    se, sl = W.specials(n)
    for i in range(len(se)):
        for j in range(len(se)):
            extra_a.append((se[i], sl[i])); extra_b.append((se[j], sl[j]))
    ae = np.concatenate([ae, np.array([e for e, _ in extra_a], np.uint32)])
    al = np.concatenate([al, np.stack([l for _, l in extra_a])])
    be = np.concatenate([be, np.array([e for e, _ in extra_b], np.uint32)])
    bl = np.concatenate([bl, np.stack([l for _, l in extra_b])])
    return ae, al, be, bl


def sqrt_cases(rng, n):
    ae, al = W.uniform(rng, 120, n, -300, 300, signs=False)
    extra = []
    for _ in range(24):
        A, par = W.sqrt_near_exact(rng, n)
        extra.append((W.exp_word(2 * int(rng.integers(-9, 9)) + par, 0), W.int_to_limbs(A, n)))
    ones = np.full(n, 0xFFFFFFFF, np.uint32)
    top = W.int_to_limbs(1 << (32 * n - 1), n)
    extra += [(W.exp_word(e, 0), m) for e in (1, 2, -7, 8) for m in (ones, top)]
    extra += [(np.uint32(2 * 6), W.uniform(rng, 1, n, 0, 0)[1][0]), (np.uint32(2 * 0x7FFFFFFF), ones)]
    se, sl = W.specials(n)
    extra += [(se[i], sl[i]) for i in range(len(se))]
    ae = np.concatenate([ae, np.array([e for e, _ in extra], np.uint32)])
    al = np.concatenate([al, np.stack([l for _, l in extra])])
    return ae, al, np.zeros_like(ae), np.zeros_like(al)


BIAS_W = W.BIAS


@pytest.mark.parametrize("shape,n", [(s, n) for s, ns in SHAPES.items() for n in ns])
def test_group_mul_div_sqrt_match_oracle(host_binary, shape, n):
    rng = np.random.default_rng(9100 + 7 * n + shape[0])
    cases = {2: mul_cases(rng, n), 3: div_cases(rng, n), 4: sqrt_cases(rng, n)}
    if n >= SAMPLE_FROM:
        cases = {op: _sample(c, SAMPLE) for op, c in cases.items()}
    batches = [(op, mode, cases[op]) for op in (2, 3, 4) for mode in range(5)]
    got = run_host(host_binary, shape, n, batches)
    for (op, mode, (ae, al, be, bl)), (err, ge, gl) in zip(batches, got):
        ee, el = oracle.run(op, n, mode, ae, al, be, bl) if op != 4 else oracle.run(op, n, mode, ae, al)
        assert err == 0, (op, n, mode)
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (op, n, mode, int(np.flatnonzero((gl != el).any(axis=1) & val)[0]))


@pytest.mark.parametrize("shape,n", [(s, n) for s, ns in SHAPES.items() for n in ns[-1:]] + [((4, 2, 1), 1)])
def test_group_fma_matches_oracle(host_binary, shape, n):
    seeded = fma_cases(9300 + n + shape[0], n)
    special = special_cases(n)
    cases = tuple(np.concatenate([x, y]) for x, y in zip(seeded, special))
    if n >= SAMPLE_FROM:
        cases = _sample(cases, 2 * SAMPLE)
    batches = [(5, mode, cases) for mode in range(5)]
    got = run_host(host_binary, shape, n, batches)
    for (_, mode, c), (err, ge, gl) in zip(batches, got):
        ee, el = oracle.run_fma(n, mode, *c)
        assert err == 0, (n, mode)
        assert np.array_equal(ge, ee), (n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (n, mode, int(np.flatnonzero((gl != el).any(axis=1) & val)[0]))


def _sample(case, lim):
    """The first and last lim/2 cases of an operand set (random values first, edge cases last)."""
    count = len(case[0])
    if count <= lim:
        return case
    idx = np.r_[0:lim // 2, count - lim // 2:count]
    return tuple(x[idx] for x in case)


@pytest.fixture(scope="module")
def tsan_binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("group_ops_tsan")
    src, exe = d / "group_ops.cpp", d / "group_ops_tsan"
    src.write_text(host_source())
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++20", "-fno-strict-aliasing", "-pthread", "-w",
                        "-fsanitize=thread", "-o", str(exe), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("ThreadSanitizer is not available: " + r.stderr[-300:])
    tsan_starts(str(exe))
    return str(exe)


def tsan_starts(exe):
    """Skip when a ThreadSanitizer build cannot start on this host (it refuses some memory
    layouts); an empty input makes the program exit at once."""
    r = subprocess.run([exe], input="", capture_output=True, text=True, timeout=120)
    if r.returncode != 0 and "ThreadSanitizer" in r.stderr:
        pytest.skip("ThreadSanitizer cannot run here: " + r.stderr.strip()[-300:])


@pytest.mark.parametrize("shape,n", [((4, 2, 1), 1), ((4, 2, 1), 8), ((8, 4, 1), 17), ((16, 4, 2), 128),
                                     ((4, 4, 8), 128), ((8, 4, 4), 128), ((32, 8, 1), 256)])
def test_group_ops_have_no_lane_races(tsan_binary, shape, n, monkeypatch):
    """Lanes of a group share its workspace: every shared-memory word one lane writes and
    another reads (or writes) must be separated by a group sync or a collective.  The
    emulation orders memory only at those points, so ThreadSanitizer reports any access
    pair without one.  add/sub, mul, div, sqrt and fma, bounded samples of their operand sets."""
    rng = np.random.default_rng(9500 + n)
    fma = tuple(np.concatenate([x, y]) for x, y in zip(fma_cases(9600 + n, n), special_cases(n)))
    sets = {0: addsub_cases(rng, n), 2: mul_cases(rng, n), 3: div_cases(rng, n), 4: sqrt_cases(rng, n), 5: fma}
    sets[1] = sets[0]
    lim = 60 if n < SAMPLE_FROM else 24
    batches = [(op, mode, _sample(sets[op], lim)) for op in (0, 1, 2, 3, 4, 5) for mode in (0, 3, 4)]
    monkeypatch.setenv("TSAN_OPTIONS", "halt_on_error=1 exitcode=66")
    got = run_host(tsan_binary, shape, n, batches)
    assert all(err == 0 for err, _, _ in got)


@pytest.mark.parametrize("shape,n", [(s, n) for s, ns in SHAPES.items() for n in ns])
def test_group_addsub_matches_oracle(host_binary, shape, n):
    rng = np.random.default_rng(9700 + 7 * n + shape[0])
    cases = addsub_cases(rng, n)
    if n >= SAMPLE_FROM:
        cases = _sample(cases, 4 * SAMPLE)
    batches = [(op, mode, cases) for op in (0, 1) for mode in range(5)]
    got = run_host(host_binary, shape, n, batches)
    for (op, mode, c), (err, ge, gl) in zip(batches, got):
        ee, el = oracle.run(op, n, mode, *c)
        assert err == 0, (op, n, mode)
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (op, n, mode, int(np.flatnonzero((gl != el).any(axis=1) & val)[0]))


# (shape, n) for the elementwise kernels' pipelined loops; Karatsuba where the shape carries it
PIPE_CASES = [((4, 2, 1), 8), ((8, 4, 1), 17), ((8, 4, 2), 64), ((16, 4, 2), 128), ((8, 4, 4), 97),
              ((16, 8, 2), 201), ((16, 8, 2), 256), ((32, 8, 1), 256), ((32, 16, 1), 512)]


def _karatsuba(shape):
    G, K, R = shape
    return K >= 8 and G * K * R >= 256


@pytest.mark.parametrize("shape,n", PIPE_CASES)
def test_pipelined_loops_match_oracle(host_binary, shape, n):
    """addsub_pipelined and mul_pipelined (fpa_kernels.cu) with their double-buffered async
    staging, the copies landing only at each lane's wait; mul also with the Karatsuba split."""
    rng = np.random.default_rng(9900 + n + shape[0])
    add, mul = addsub_cases(rng, n), mul_cases(rng, n)
    if n >= SAMPLE_FROM:
        add, mul = _sample(add, 4 * SAMPLE), _sample(mul, 2 * SAMPLE)
    ops = [(10, 0, add), (11, 1, add), (12, 2, mul)] + ([(16, 2, mul)] if _karatsuba(shape) else [])
    batches = [(code, mode, c) for code, _, c in ops for mode in range(5)]
    got = run_host(host_binary, shape, n, batches)
    expect = {(op, mode): oracle.run(op, n, mode, *c) for _, op, c in ops for mode in range(5)}
    for (code, mode, c), (err, ge, gl) in zip(batches, got):
        op = {10: 0, 11: 1, 12: 2, 16: 2}[code]
        ee, el = expect[(op, mode)]
        assert np.array_equal(ge, ee), (code, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (code, n, mode, int(np.flatnonzero((gl != el).any(axis=1) & val)[0]))


@pytest.mark.parametrize("shape,n", [((8, 4, 1), 17), ((16, 4, 2), 128), ((16, 8, 2), 256)])
def test_pipelined_loops_have_no_lane_races(tsan_binary, shape, n, monkeypatch):
    """The double-buffered loops under ThreadSanitizer: a lane that read staged operands
    before the copying lane's wait and the group sync after it would be reported."""
    rng = np.random.default_rng(9950 + n)
    add, mul = _sample(addsub_cases(rng, n), 40), _sample(mul_cases(rng, n), 24)
    codes = [(10, add), (11, add), (12, mul)] + ([(16, mul)] if _karatsuba(shape) else [])
    batches = [(code, mode, c) for code, c in codes for mode in (0, 3)]
    monkeypatch.setenv("TSAN_OPTIONS", "halt_on_error=1 exitcode=66")
    run_host(tsan_binary, shape, n, batches)
