"""The kernels of the path compiled for the host and run as whole CTAs: the elementwise
kernel k_elementwise (cubigfloat_gb300/csrc/fpa_kernels.cu) for all six operations, the
batch kernels' task loop and dispatcher, both chain kernels, the row kernel and the register
add/sub kernel.  Each GPU thread is a host thread; each lane group has its own emulated
collectives (as in test_group_ops_host.py); the CTA's shared memory is one host buffer; and
__syncthreads() is a CTA barrier that also checks where it is called from.

The div/sqrt/fma loop makes every thread of a CTA run the same number of iterations and
meet one CTA barrier per iteration, including the groups whose operation index is past the
end.  On the GPU, bar.sync must be reached by all lanes of a warp at the same instruction;
lanes that diverge onto two different barrier sites hang the CTA.  So the emulated barrier
ends the program when two lanes of one warp arrive from different source lines, and a
thread that skips a barrier makes the others time out.  Grids of 1 to 3 CTAs with 1, 2 or
4 warps per CTA, at operation counts that leave partial last iterations, are checked
bit-exact against the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from cubigfloat_gb300 import workloads as W
from fma_cases import fma_cases
from test_gpu_addsub import addsub_cases
from test_gpu_chain import half, oracle_dot
from test_gpu_rows import mul_cases
from test_group_ops_host import CSRC, _host_qualifiers, device_source, div_cases, sqrt_cases, _sample, tsan_starts

CTA_SHIMS = r"""
#include <cstdint>
struct HostDim3 { uint32_t x = 0, y = 0, z = 0; };
static thread_local HostDim3 threadIdx, blockIdx;
static HostDim3 blockDim, gridDim;
static uint32_t *g_smem;
static inline uint32_t atomicAdd(uint32_t *p, uint32_t v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
"""

CTA_BARRIER = r"""
// CTA barrier: every thread records the source line it calls from; after all arrive, a
// thread whose line differs from its warp's first lane's ends the program.
static GroupBarrier g_cta_bar;
static int g_cta_line[1024];
static inline void cta_sync(int line) {
  const uint32_t t = threadIdx.x;
  g_cta_line[t] = line;
  g_cta_bar.arrive_and_wait();
  if (g_cta_line[t & ~31u] != line) {
    fprintf(stderr, "warp %u: lanes at CTA barriers on lines %d and %d\n", t / 32, g_cta_line[t & ~31u], line);
    std::_Exit(5);
  }
  g_cta_bar.arrive_and_wait();
}
#define __syncthreads() cta_sync(__LINE__)
// __syncwarp(): the warp's barrier (the row kernel runs one operation per thread)
static thread_local GroupBarrier *t_warp_bar;
static inline void __syncwarp() { t_warp_bar->arrive_and_wait(); }
"""

MAIN = r"""
using namespace gfpa;
static ElementwiseArgs g_args;
template <int OP, int G, int K, int R>
static void cta_thread(uint32_t tid, uint32_t block, GroupCtx *groups) {
  threadIdx.x = tid; blockIdx.x = block;
  t_lane = tid % G; t_ctx = &groups[tid / G]; t_round = 0;
  k_elementwise<OP, G, K, R>(g_args);
}
template <int OP, int G, int K, int R>
static void run_grid(int threads, int blocks) {
  blockDim.x = threads; gridDim.x = blocks;
  const int gpc = threads / G;
  const size_t words = (size_t)gpc * PipeWords<OP, G, K, R>::aligned();
  std::vector<uint32_t> smem(words + 64, 0x5A5A5A5Au);
  g_smem = smem.data();
  for (int b = 0; b < blocks; b++) {
    std::vector<GroupCtx> groups(gpc);
    for (auto &c : groups) c.bar.lanes = G;
    g_cta_bar.lanes = threads;
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++) ts.emplace_back(cta_thread<OP, G, K, R>, (uint32_t)t, (uint32_t)b, groups.data());
    for (auto &t : ts) t.join();
  }
  for (size_t i = words; i < words + 64; i++)
    if (smem[i] != 0x5A5A5A5Au) { fprintf(stderr, "shared memory overrun\n"); std::_Exit(4); }
}
static BatchArgs g_bargs;
template <int OP, int G, int K, int R>
static void task_thread(uint32_t tid, GroupCtx *groups, uint32_t count) {
  threadIdx.x = tid; blockIdx.x = 0;
  t_lane = tid % G; t_ctx = &groups[tid / G]; t_round = 0;
  run_task<OP, G, K, R>(g_bargs, 0, count, g_smem);
}
template <int OP, int G, int K, int R>
static void run_batch_task(int threads, uint32_t count) {
  blockDim.x = threads; gridDim.x = 1;
  g_bargs.warp_words = (32 / G) * OpWords<OP, G, K, R>::aligned();
  const size_t words = (size_t)(threads / 32) * g_bargs.warp_words;
  std::vector<uint32_t> smem(words + 64, 0x5A5A5A5Au);
  g_smem = smem.data();
  std::vector<GroupCtx> groups(threads / G);
  for (auto &c : groups) c.bar.lanes = G;
  g_cta_bar.lanes = threads;
  std::vector<std::thread> ts;
  for (int t = 0; t < threads; t++) ts.emplace_back(task_thread<OP, G, K, R>, (uint32_t)t, groups.data(), count);
  for (auto &t : ts) t.join();
  for (size_t i = words; i < words + 64; i++)
    if (smem[i] != 0x5A5A5A5Au) { fprintf(stderr, "shared memory overrun\n"); std::_Exit(4); }
}
static ChainArgs g_cargs;
template <int KIND, int G, int K, int R>
static void chain_thread(uint32_t tid, uint32_t block, GroupCtx *groups) {
  threadIdx.x = tid; blockIdx.x = block;
  t_lane = tid % G; t_ctx = &groups[tid / G]; t_round = 0;
  if (KIND == 0) k_dot<G, K, R>(g_cargs);
  else k_newton_sqrt<G, K, R>(g_cargs);
}
template <int KIND, int G, int K, int R>
static void run_chain(int threads, int blocks) {
  blockDim.x = threads; gridDim.x = blocks;
  const int gpc = threads / G;
  const size_t words = (size_t)gpc * (KIND == 0 ? ChainSpace<G, K, R>::dot() : ChainSpace<G, K, R>::newton());
  std::vector<uint32_t> smem(words + 64, 0x5A5A5A5Au);
  g_smem = smem.data();
  for (int b = 0; b < blocks; b++) {
    std::vector<GroupCtx> groups(gpc);
    for (auto &c : groups) c.bar.lanes = G;
    g_cta_bar.lanes = threads;
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++)
      ts.emplace_back(chain_thread<KIND, G, K, R>, (uint32_t)t, (uint32_t)b, groups.data());
    for (auto &t : ts) t.join();
  }
  for (size_t i = words; i < words + 64; i++)
    if (smem[i] != 0x5A5A5A5Au) { fprintf(stderr, "shared memory overrun\n"); std::_Exit(4); }
}
template <int OP, int G, int K>
static void regk_thread(uint32_t tid, uint32_t block, GroupCtx *groups) {
  threadIdx.x = tid; blockIdx.x = block;
  t_lane = tid % G; t_ctx = &groups[tid / G]; t_round = 0;
  k_addsub_regk<OP, G, K>(g_args);
}
template <int OP, int G, int K>
static void run_regk(int threads, int blocks) {
  blockDim.x = threads; gridDim.x = blocks;
  for (int b = 0; b < blocks; b++) {
    std::vector<GroupCtx> groups(threads / G);
    for (auto &c : groups) c.bar.lanes = G;
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++) ts.emplace_back(regk_thread<OP, G, K>, (uint32_t)t, (uint32_t)b, groups.data());
    for (auto &t : ts) t.join();
  }
}
template <int OP, int N>
static void rows_thread(uint32_t tid, uint32_t block, GroupBarrier *warp_bars) {
  threadIdx.x = tid; blockIdx.x = block; t_warp_bar = &warp_bars[tid / 32];
  k_rows<OP, N>(g_args);
}
template <int OP, int N>
static void run_rows(int threads, int blocks) {
  blockDim.x = threads; gridDim.x = blocks;
  const size_t words = (size_t)(threads / 32) * RowSpace<N>::words;
  std::vector<uint32_t> smem(words + 64, 0x5A5A5A5Au);
  g_smem = smem.data();
  for (int b = 0; b < blocks; b++) {
    std::vector<GroupBarrier> bars(threads / 32);
    for (auto &w : bars) w.lanes = 32;
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++) ts.emplace_back(rows_thread<OP, N>, (uint32_t)t, (uint32_t)b, bars.data());
    for (auto &t : ts) t.join();
  }
  for (size_t i = words; i < words + 64; i++)
    if (smem[i] != 0x5A5A5A5Au) { fprintf(stderr, "shared memory overrun\n"); std::_Exit(4); }
}
template <int OP, int G, int K, int R>
constexpr uint32_t warp_words_of() { return (32 / G) * OpWords<OP, G, K, R>::aligned(); }
// shared-memory words per warp of a class kernel: the largest task body it may run
static uint32_t class_warp_words(int cls) {
  const uint32_t w[2][3] = {
      {std::max(warp_words_of<OP_ADD, 4, 2, 1>(), warp_words_of<OP_MUL, 4, 2, 1>()),
       std::max(warp_words_of<OP_ADD, 8, 4, 1>(), warp_words_of<OP_MUL, 8, 4, 1>()),
       std::max(warp_words_of<OP_ADD, 16, 4, 2>(), warp_words_of<OP_MUL, 16, 4, 2>())},
      {std::max(warp_words_of<OP_DIV, 4, 2, 1>(), warp_words_of<OP_SQRT, 4, 2, 1>()),
       std::max(warp_words_of<OP_DIV, 8, 4, 1>(), warp_words_of<OP_SQRT, 8, 4, 1>()),
       std::max(warp_words_of<OP_DIV, 16, 4, 2>(), warp_words_of<OP_SQRT, 16, 4, 2>())}};
  return std::max(std::max(w[cls][0], w[cls][1]), w[cls][2]);
}
template <int CLS>
static void dispatch_thread(uint32_t tid, uint32_t block, GroupCtx *groups, int G) {
  threadIdx.x = tid; blockIdx.x = block;
  t_lane = tid % G; t_ctx = &groups[tid / G]; t_round = 0;
  k_batch<CLS>(g_bargs);
}
// a mixed batch: operation i is ce[i] (0..4), all on configuration cfg; tasks of at most 7
// operations in descriptor order, class 0 (add/sub/mul) and class 1 (div/sqrt) kernels
static int run_dispatch(int cfg, int G, int n, int mode, int count, int blocks, const uint32_t *ops,
                        std::vector<fpa_batch_desc> &descs) {
  std::vector<uint32_t> order(count);
  std::vector<BatchTask> tasks[2];
  for (int i = 0; i < count; i++) {
    descs[i] = fpa_batch_desc{(uint8_t)ops[i], (uint8_t)mode, (uint16_t)n, 0u, (uint64_t)i * n, (uint64_t)i * n,
                              (uint64_t)i * n};
    order[i] = (uint32_t)i;
  }
  for (int i = 0; i < count;) {
    int j = i;
    while (j < count && j - i < 7 && ops[j] == ops[i]) j++;
    tasks[ops[i] >= 3].push_back(BatchTask{(uint16_t)(cfg * 5 + ops[i]), 0, (uint32_t)i, (uint32_t)(j - i)});
    i = j;
  }
  g_bargs.descs = descs.data(); g_bargs.order = order.data();
  for (int cls = 0; cls < 2; cls++) {
    uint32_t counter = 0;
    g_bargs.tasks = tasks[cls].data(); g_bargs.ntasks = (uint32_t)tasks[cls].size(); g_bargs.counter = &counter;
    g_bargs.warp_words = class_warp_words(cls);
    const int threads = cls == 0 ? ClassShape<0>::threads : ClassShape<1>::threads;
    blockDim.x = threads; gridDim.x = blocks;
    const size_t words = (size_t)(threads / 32) * g_bargs.warp_words;
    std::vector<uint32_t> smem(words + 64, 0x5A5A5A5Au);
    g_smem = smem.data();
    for (int b = 0; b < blocks; b++) {
      std::vector<GroupCtx> groups(threads / G);
      for (auto &c : groups) c.bar.lanes = G;
      g_cta_bar.lanes = threads;
      std::vector<std::thread> ts;
      for (int t = 0; t < threads; t++)
        ts.emplace_back(cls == 0 ? dispatch_thread<0> : dispatch_thread<1>, (uint32_t)t, (uint32_t)b, groups.data(), G);
      for (auto &t : ts) t.join();
    }
    if (counter < g_bargs.ntasks) { fprintf(stderr, "tasks left in the queue\n"); std::_Exit(6); }
    for (size_t i = words; i < words + 64; i++)
      if (smem[i] != 0x5A5A5A5Au) { fprintf(stderr, "shared memory overrun\n"); std::_Exit(4); }
  }
  return 0;
}
static uint32_t *alloc_words(size_t count) {
  return static_cast<uint32_t *>(aligned_alloc(64, ((count * 4 + 63) / 64) * 64 + 64));
}
int main() {
  int G, K, R, op, n, mode, count, warps, blocks, len;
  while (scanf("%d %d %d %d %d %d %d %d %d %d", &G, &K, &R, &op, &n, &mode, &count, &warps, &blocks, &len) == 10) {
    uint32_t *ae = alloc_words(count), *be = alloc_words(count), *ce = alloc_words(count), *re = alloc_words(count);
    uint32_t *a = alloc_words((size_t)count * n), *b = alloc_words((size_t)count * n);
    uint32_t *c = alloc_words((size_t)count * n), *r = alloc_words((size_t)count * n);
    for (int i = 0; i < count; i++) {
      unsigned x;
      if (scanf("%u", &x) != 1) return 1; ae[i] = x;
      if (scanf("%u", &x) != 1) return 1; be[i] = x;
      if (scanf("%u", &x) != 1) return 1; ce[i] = x;
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; a[(size_t)i * n + j] = x; }
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; b[(size_t)i * n + j] = x; }
      for (int j = 0; j < n; j++) { if (scanf("%u", &x) != 1) return 1; c[(size_t)i * n + j] = x; }
    }
    memset(re, 0xA5, (size_t)count * 4);
    memset(r, 0xA5, (size_t)count * n * 4);
    uint32_t err = 0;
    g_args = ElementwiseArgs{};
    g_args.count = (uint64_t)count; g_args.n = (uint32_t)n; g_args.mode = mode;
    g_args.r_exps = re; g_args.r_limbs = r; g_args.a_exps = ae; g_args.a_limbs = a;
    g_args.b_exps = be; g_args.b_limbs = b; g_args.c_exps = ce; g_args.c_limbs = c; g_args.err = &err;
    const int threads = 32 * warps, key = (G * 10000 + K * 100 + R) * 100 + op;
    int results = count;
    if (op == 60) {                              // mixed batch through the class kernels' dispatcher
      std::vector<fpa_batch_desc> descs(count);
      g_bargs = BatchArgs{};
      g_bargs.r_exps = re; g_bargs.r_limbs = r; g_bargs.a_exps = ae; g_bargs.a_limbs = a;
      g_bargs.b_exps = be; g_bargs.b_limbs = b; g_bargs.err = &err;
      const int cfg = G == 4 ? 0 : (G == 8 ? 2 : 12);
      if (run_dispatch(cfg, G, n, mode, count, blocks, ce, descs)) return 2;
    } else if (op >= 50) {                       // register add/sub kernel: op 50 + OP
      switch (key - (op - 50)) {
@REGK_CASES@        default: return 2;
      }
    } else if (op >= 40) {                       // row kernels: op 40 + OP, n = 8, 16 or 32
      switch ((op - 40) * 100 + n) {
        case 8: run_rows<OP_ADD, 8>(threads, blocks); break;
        case 16: run_rows<OP_ADD, 16>(threads, blocks); break;
        case 32: run_rows<OP_ADD, 32>(threads, blocks); break;
        case 108: run_rows<OP_SUB, 8>(threads, blocks); break;
        case 116: run_rows<OP_SUB, 16>(threads, blocks); break;
        case 132: run_rows<OP_SUB, 32>(threads, blocks); break;
        case 208: run_rows<OP_MUL, 8>(threads, blocks); break;
        case 216: run_rows<OP_MUL, 16>(threads, blocks); break;
        case 232: run_rows<OP_MUL, 32>(threads, blocks); break;
        default: return 2;
      }
    } else if (op >= 30) {                       // chains: dot (count / len dots) or Newton sqrt
      g_cargs = ChainArgs{};
      g_cargs.count = (uint64_t)(op == 30 ? count / len : count); g_cargs.n = (uint32_t)n;
      g_cargs.len = (uint32_t)len; g_cargs.mode = mode;
      g_cargs.r_exps = re; g_cargs.r_limbs = r; g_cargs.x_exps = ae; g_cargs.x_limbs = a;
      g_cargs.y_exps = be; g_cargs.y_limbs = b; g_cargs.err = &err;
      results = (int)g_cargs.count;
      switch (key) {
@CHAIN_CASES@        default: return 2;
      }
    } else if (op >= 20) {                              // one batch task of `count` operations
      std::vector<fpa_batch_desc> descs(count);
      std::vector<uint32_t> order(count);
      for (int i = 0; i < count; i++) {
        descs[i] = fpa_batch_desc{(uint8_t)(op - 20), (uint8_t)mode, (uint16_t)n, 0u, (uint64_t)i * n,
                                  (uint64_t)i * n, (uint64_t)i * n};
        order[i] = (uint32_t)i;
      }
      g_bargs = BatchArgs{};
      g_bargs.descs = descs.data(); g_bargs.order = order.data(); g_bargs.ntasks = 1;
      g_bargs.r_exps = re; g_bargs.r_limbs = r; g_bargs.a_exps = ae; g_bargs.a_limbs = a;
      g_bargs.b_exps = be; g_bargs.b_limbs = b; g_bargs.err = &err;
      switch (key) {
@BATCH_CASES@        default: return 2;
      }
    } else
    switch (key) {
@CASES@      default: return 2;
    }
    printf("err %u\n", err);
    for (int i = 0; i < results; i++) {
      printf("%u", re[i]);
      for (int j = 0; j < n; j++) printf(" %u", re[i] > CLS_SNAN ? r[(size_t)i * n + j] : 0u);
      printf("\n");
    }
    free(ae); free(be); free(ce); free(re); free(a); free(b); free(c); free(r);
  }
  return 0;
}
"""

SHAPES = [(4, 2, 1), (8, 4, 1), (16, 4, 2)]
OPS = (0, 1, 2, 3, 4, 5)           # add, sub, mul (double-buffered loops), div, sqrt, fma (lockstep loop)


def cta_source():
    body = device_source("template <int OP, int G, int K, int R>\nusing Words",
                         "template <int OP>\nstatic cudaError_t launch_op", CTA_SHIMS)
    body = body.replace("extern __shared__ __align__(16) uint32_t smem[];", "uint32_t *smem = g_smem;")
    head = "__global__ void __launch_bounds__(CtaBounds<OP, K>::threads, CtaBounds<OP, K>::min_blocks)"
    assert body.count(head) == 1
    body = body.replace(head, "void")
    assert "__global__" not in body and "__shared__" not in body
    # the CTA barrier goes after the group shims (it uses GroupBarrier), before the device code
    mark = "template <int G>\nstruct Grp {"
    body = body.replace(mark, "}  // namespace gfpa\n" + CTA_BARRIER + "namespace gfpa {\n" + mark, 1)
    # the batched form's task body (fpa_batch_kernels.cu) and its argument structs
    bk = open(os.path.join(CSRC, "fpa_batch_kernels.cu")).read()
    task = bk[bk.index("template <int OP, int G, int K, int R>\n__device__ __noinline__ void run_task"):
              bk.index("#define GFPA_TASK_OP")]
    gh = open(os.path.join(CSRC, "..", "..", "include", "fpa_gb300.h")).read()
    desc = gh[gh.index("typedef struct {\n  uint8_t op;"):gh.index("} fpa_batch_desc;") + len("} fpa_batch_desc;")]
    bh = open(os.path.join(CSRC, "fpa_batch.h")).read()
    structs = _host_qualifiers(bh[bh.index("struct BatchTask {"):bh.index("// threads per CTA of each class kernel")])
    body = body.replace("template <int G>\nstruct Grp {", "}  // namespace gfpa\n" + desc + "\n" + structs
                        + "namespace gfpa {\ntemplate <int G>\nstruct Grp {", 1)
    body += "namespace gfpa {\n" + _host_qualifiers(task) + "}  // namespace gfpa\n"
    # the class kernels' task dispatcher, its task list cut down to the configurations here
    disp = bk[bk.index("#define GFPA_TASK_OP"):bk.index("}  // namespace gfpa\n\n#define GFPA_CAT2")]
    tile4 = disp[disp.index("#define GFPA_TASKS_TILE4"):disp.index("template <int CLS>\nstruct ClassShape")]
    subset = "#define GFPA_TASKS_TILE4 GFPA_TASK(0, 4, 2, 1) GFPA_TASK(2, 8, 4, 1) GFPA_TASK(12, 16, 4, 2)\n\n"
    disp = disp.replace(tile4, subset)
    for old in ("GFPA_TASK(5, 32, 8, 1) GFPA_TASK(7, 16, 8, 1) GFPA_TASK(13, 8, 8, 4) GFPA_TASK(14, 16, 8, 2)",
                "GFPA_TASK(6, 32, 16, 1) GFPA_TASK(8, 8, 16, 1) GFPA_TASK(9, 16, 16, 1)"):
        assert disp.count(old) == 1
        disp = disp.replace(old, "")
    head = "__global__ void __launch_bounds__(ClassShape<CLS>::threads, ClassShape<CLS>::min_blocks)"
    assert disp.count(head) == 1 and disp.count("__shared__ uint32_t s_task;") == 1
    disp = disp.replace(head, "void").replace("__shared__ uint32_t s_task;", "static uint32_t s_task;")
    disp = disp.replace("extern __shared__ __align__(16) uint32_t smem[];", "uint32_t *smem = g_smem;")
    body += "namespace gfpa {\n" + _host_qualifiers(disp) + "}  // namespace gfpa\n"
    # the fused chains (fpa_chain.cu)
    ch = open(os.path.join(CSRC, "fpa_chain.cu")).read()
    chain = _host_qualifiers(ch[ch.index("struct ChainArgs {"):
                                ch.index("template <int G, int K, int R>\ncudaError_t launch_chain")])
    assert chain.count("__global__ void __launch_bounds__(128, 4)") == 2
    chain = chain.replace("__global__ void __launch_bounds__(128, 4)", "void")
    chain = chain.replace("extern __shared__ __align__(16) uint32_t smem[];", "uint32_t *smem = g_smem;")
    body += "namespace gfpa {\n" + chain + "}  // namespace gfpa\n"
    # the one-thread row kernels (fpa_addsub_rows.cuh)
    rw = open(os.path.join(CSRC, "fpa_addsub_rows.cuh")).read()
    rows = _host_qualifiers(rw[rw.index("template <int N>\nstruct RowSpace"):
                               rw.index("template <int OP, int N>\nstatic cudaError_t launch_rows")])
    assert rows.count("__global__ void __launch_bounds__(128, 4)") == 1
    rows = rows.replace("__global__ void __launch_bounds__(128, 4)", "void")
    rows = rows.replace("extern __shared__ __align__(16) uint32_t smem[];", "uint32_t *smem = g_smem;")
    body += "namespace gfpa {\n" + rows + "}  // namespace gfpa\n"
    # the register add/sub kernel (fpa_addsub_regs.cuh)
    rg = open(os.path.join(CSRC, "fpa_addsub_regs.cuh")).read()
    regk = _host_qualifiers(rg[rg.index("template <int K>\nstruct Log2"):
                               rg.index("template <int OP, int G, int K>\nstatic cudaError_t launch_addsub_regk")])
    head = "__global__ void __launch_bounds__(128, (K <= 4) ? 8 : (K <= 8 ? 4 : 2))"
    assert regk.count(head) == 1
    body += "namespace gfpa {\n" + regk.replace(head, "void") + "}  // namespace gfpa\n"
    cases = "".join(f"      case {(G * 10000 + K * 100 + R) * 100 + op}: "
                    f"run_grid<{op}, {G}, {K}, {R}>(threads, blocks); break;\n" for (G, K, R) in SHAPES for op in OPS)
    bcases = "".join(f"        case {(G * 10000 + K * 100 + R) * 100 + 20 + op}: run_batch_task<{op}, {G}, {K}, {R}>"
                     f"(threads, (uint32_t)count); break;\n" for (G, K, R) in SHAPES for op in range(5))
    ccases = "".join(f"        case {(G * 10000 + K * 100 + R) * 100 + 30 + kind}: run_chain<{kind}, {G}, {K}, {R}>"
                     f"(threads, blocks); break;\n" for (G, K, R) in SHAPES for kind in (0, 1))
    rcases = "".join(f"        case {(G * 10000 + K * 100 + R) * 100 + 50}: "
                     f"if (op == 50) run_regk<OP_ADD, {G}, {K}>(threads, blocks); "
                     f"else run_regk<OP_SUB, {G}, {K}>(threads, blocks); break;\n" for (G, K, R) in SHAPES)
    main = MAIN.replace("@REGK_CASES@", rcases).replace("@CASES@", cases)
    return body + main.replace("@BATCH_CASES@", bcases).replace("@CHAIN_CASES@", ccases)


def build(src_text, path, flags):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src, exe = path / "cta.cpp", path / "cta"
    src.write_text(src_text)
    r = subprocess.run([cxx] + flags + ["-std=c++20", "-fno-strict-aliasing", "-pthread", "-w", "-o", str(exe),
                                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return str(exe)


@pytest.fixture(scope="module")
def cta_binary(tmp_path_factory):
    return build(cta_source(), tmp_path_factory.mktemp("cta"), ["-O2"])


def run_cta(exe, shape, op, n, mode, case, warps, blocks, length=0):
    G, K, R = shape
    ae, al, be, bl = case[:4]
    ce, cl = case[4:] if len(case) == 6 else (np.zeros_like(ae), np.zeros_like(al))
    lines = [f"{G} {K} {R} {op} {n} {mode} {len(ae)} {warps} {blocks} {length}"]
    for i in range(len(ae)):
        lines.append(f"{int(ae[i])} {int(be[i])} {int(ce[i])} " + " ".join(map(str, al[i])) + " "
                     + " ".join(map(str, bl[i])) + " " + " ".join(map(str, cl[i])))
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    out = r.stdout.strip().split("\n")
    rows = np.array([[int(x) for x in line.split()] for line in out[1:]], dtype=np.uint64)
    return int(out[0].split()[1]), rows[:, 0].astype(np.uint32), rows[:, 1:].astype(np.uint32)


# (shape, n, warps per CTA, CTAs, operations): counts leave the last iteration partial
GRIDS = [((4, 2, 1), 5, 1, 2, 37), ((4, 2, 1), 8, 2, 3, 61), ((8, 4, 1), 17, 4, 1, 29), ((16, 4, 2), 128, 2, 2, 9)]


@pytest.mark.parametrize("shape,n,warps,blocks,count", GRIDS)
@pytest.mark.parametrize("op", OPS)
def test_elementwise_kernel_lockstep_matches_oracle(cta_binary, shape, n, warps, blocks, count, op):
    """k_elementwise on grids of emulated CTAs: add/sub/mul through the grid-stride
    double-buffered loops, div/sqrt/fma through the lockstep loop."""
    rng = np.random.default_rng(10100 + 10 * n + op)
    make = {0: addsub_cases, 1: addsub_cases, 2: mul_cases, 3: div_cases, 4: sqrt_cases}
    case = make[op](rng, n) if op != 5 else fma_cases(10200 + n, n)
    case = _sample(case, count)
    for mode in (0, 3, 4):
        err, ge, gl = run_cta(cta_binary, shape, op, n, mode, case, warps, blocks)
        ee, el = oracle.run_fma(n, mode, *case) if op == 5 else (
            oracle.run(op, n, mode, *case[:4]) if op != 4 else oracle.run(op, n, mode, *case[:2]))
        assert err == 0
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (op, n, mode)


@pytest.mark.parametrize("shape,n,warps,count", [((4, 2, 1), 5, 2, 37), ((8, 4, 1), 17, 4, 29),
                                                 ((16, 4, 2), 128, 2, 9)])
@pytest.mark.parametrize("op", range(5))
def test_batch_task_lockstep_matches_oracle(cta_binary, shape, n, warps, count, op):
    """run_task (fpa_batch_kernels.cu): one task of `count` operations on one CTA of several
    warps.  div and sqrt run the lockstep loop with its single CTA barrier site."""
    rng = np.random.default_rng(10300 + 10 * n + op)
    make = {0: addsub_cases, 1: addsub_cases, 2: mul_cases, 3: div_cases, 4: sqrt_cases}[op]
    case = _sample(make(rng, n), count)
    for mode in (0, 3, 4):
        err, ge, gl = run_cta(cta_binary, shape, 20 + op, n, mode, case, warps, 1)
        ee, el = oracle.run(op, n, mode, *case[:4]) if op != 4 else oracle.run(op, n, mode, *case[:2])
        assert err == 0
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        val = ee > 8
        assert np.array_equal(gl[val], el[val]), (op, n, mode)


@pytest.mark.parametrize("shape,n,warps,blocks,dots,length", [((4, 2, 1), 8, 2, 2, 37, 5), ((8, 4, 1), 17, 4, 1, 19, 4),
                                                              ((16, 4, 2), 64, 2, 2, 9, 3)])
def test_dot_chain_matches_stepwise_oracle(cta_binary, shape, n, warps, blocks, dots, length):
    """k_dot (fpa_chain.cu): acc = RN(acc + RN(x*y)) over each dot's terms, against the
    same steps in the oracle."""
    rng = np.random.default_rng(10400 + n)
    xe, xl = W.uniform(rng, dots * length, n, -30, 30)
    ye, yl = W.uniform(rng, dots * length, n, -30, 30)
    for mode in (1, 3):
        err, ge, gl = run_cta(cta_binary, shape, 30, n, mode, (xe, xl, ye, yl), warps, blocks, length)
        ee, el = oracle_dot(n, mode, xe, xl, ye, yl, dots, length)
        assert err == 0 and np.array_equal(ge, ee) and np.array_equal(gl[ee > 8], el[ee > 8]), (n, mode)


@pytest.mark.parametrize("shape,n,warps,blocks,count,iters", [((4, 2, 1), 5, 2, 2, 37, 4), ((8, 4, 1), 17, 4, 1, 29, 3),
                                                              ((16, 4, 2), 128, 2, 2, 9, 2)])
def test_newton_chain_lockstep_matches_stepwise_oracle(cta_binary, shape, n, warps, blocks, count, iters):
    """k_newton_sqrt (fpa_chain.cu), whose rounds run in lockstep with one CTA barrier per
    Newton step: y = RN(RN(y + RN(x/y)) * 0.5) against the same steps in the oracle."""
    rng = np.random.default_rng(10500 + n)
    xl = rng.integers(0, 1 << 32, size=(count, n), dtype=np.uint64).astype(np.uint32)
    xl[:, -1] |= np.uint32(0x80000000)
    xe = W.exp_word(np.ones(count, dtype=np.int64), 0)
    yl = np.zeros((count, n), np.uint32)
    yl[:, -1] = 0xC0000000
    ye = W.exp_word(np.ones(count, dtype=np.int64), 0)
    mode = 3
    err, ge, gl = run_cta(cta_binary, shape, 31, n, mode, (xe, xl, ye, yl), warps, blocks, iters)
    ee, el = ye.copy(), yl.copy()
    for _ in range(iters):
        te, tl = oracle.run(3, n, mode, xe, xl, ee, el)
        se, sl = oracle.run(0, n, mode, ee, el, te, tl)
        ee, el = half(se), sl
    assert err == 0 and np.array_equal(ge, ee) and np.array_equal(gl, el)


@pytest.fixture(scope="module")
def cta_tsan_binary(tmp_path_factory):
    try:
        exe = build(cta_source(), tmp_path_factory.mktemp("cta_tsan"), ["-O1", "-g", "-fsanitize=thread"])
    except AssertionError as e:
        pytest.skip("ThreadSanitizer build failed: " + str(e)[-300:])
    tsan_starts(exe)
    return exe


@pytest.mark.parametrize("op", [3, 4, 5, 23, 24, 30, 31, 40, 42])
def test_cta_kernels_have_no_lane_races(cta_tsan_binary, op, monkeypatch):
    """Under ThreadSanitizer: the elementwise div/sqrt/fma loop, the batch div/sqrt task
    loop, both chains (4x2x1 groups, 5 limbs) and the row kernel's add and mul (16 limbs),
    on CTAs of two warps (two CTAs where the kernel has a grid).  Every shared word that two
    threads touch must be ordered by a group sync, a collective, a warp sync or the CTA
    barrier."""
    monkeypatch.setenv("TSAN_OPTIONS", "halt_on_error=1 exitcode=66")
    rng = np.random.default_rng(10600 + op)
    n, shape = 5, (4, 2, 1)
    if op >= 40:
        n = 16
        case, length, blocks = _sample((addsub_cases if op == 40 else mul_cases)(rng, n), 70), 0, 2
    elif op in (30, 31):
        count, length = (45, 5) if op == 30 else (21, 3)
        xe, xl = W.uniform(rng, count, n, -30, 30, signs=op == 30)
        ye, yl = W.uniform(rng, count, n, -30, 30, signs=op == 30)
        case, blocks = (xe, xl, ye, yl), 2
    else:
        base = op % 10
        make = {3: div_cases, 4: sqrt_cases}.get(base)
        case = _sample(make(rng, n) if make else fma_cases(10700, n), 40)
        length, blocks = 0, 2 if op < 20 else 1
    err, _, _ = run_cta(cta_tsan_binary, shape, op, n, 3, case, 2, blocks, length)
    assert err == 0


@pytest.mark.parametrize("n", [8, 16, 32])
@pytest.mark.parametrize("op", [0, 1, 2])
def test_row_kernel_matches_oracle(cta_binary, op, n):
    """k_rows (fpa_addsub_rows.cuh) as whole emulated CTAs of four warps: each warp stages 32
    operations' rows cooperatively (async copies landing at each thread's wait), syncs,
    computes one operation per thread and copies the results out cooperatively.  The
    operation counts leave a partial last chunk of 32."""
    rng = np.random.default_rng(10800 + 10 * n + op)
    case = (addsub_cases if op < 2 else mul_cases)(rng, n)
    case = _sample(case, 300)
    for mode in (0, 3):
        err, ge, gl = run_cta(cta_binary, (4, 2, 1), 40 + op, n, mode, case, 4, 2)
        ee, el = oracle.run(op, n, mode, *case[:4])
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        assert np.array_equal(gl[ee > 8], el[ee > 8]), (op, n, mode)


@pytest.mark.parametrize("shape,n", [((4, 2, 1), 8), ((4, 2, 1), 5), ((8, 4, 1), 32), ((8, 4, 1), 19),
                                     ((16, 4, 2), 64)])
@pytest.mark.parametrize("op", [0, 1])
def test_register_addsub_kernel_matches_oracle(cta_binary, shape, n, op):
    """k_addsub_regk (fpa_addsub_regs.cuh) as emulated CTAs of four warps on a grid of two:
    the grid-stride loop that loads the next operation's operands into registers while the
    group computes the current one, at counts that leave groups without a last operation."""
    rng = np.random.default_rng(10900 + n + op)
    case = _sample(addsub_cases(rng, n), 150)
    for mode in (0, 3):
        err, ge, gl = run_cta(cta_binary, shape, 50 + op, n, mode, case, 4, 2)
        ee, el = oracle.run(op, n, mode, *case[:4])
        assert np.array_equal(ge, ee), (op, n, mode, int(np.flatnonzero(ge != ee)[0]))
        assert np.array_equal(gl[ee > 8], el[ee > 8]), (op, n, mode)


@pytest.mark.parametrize("shape,n,blocks", [((4, 2, 1), 5, 2), ((8, 4, 1), 17, 1), ((16, 4, 2), 100, 1)])
def test_batch_dispatcher_matches_oracle(cta_binary, shape, n, blocks):
    """k_batch (fpa_batch_kernels.cu) for register classes 0 and 1: CTAs of the class's size
    take tasks from the queue through a shared word between two CTA barriers until it is
    empty, each task a run of up to 7 same-op operations of a mixed batch (add, sub, mul,
    div, sqrt interleaved in runs).  Every result is checked against the oracle."""
    rng = np.random.default_rng(11000 + n)
    sets = {0: addsub_cases(rng, n), 2: mul_cases(rng, n), 3: div_cases(rng, n), 4: sqrt_cases(rng, n)}
    sets[1] = sets[0]
    per = 12 if n < 64 else 5
    ops = np.array([op for _ in range(3) for op in (0, 3, 2, 4, 1) for _ in range(per // 3 + 1)], np.uint32)
    picks = {op: _sample(sets[op], int((ops == op).sum()) + 1) for op in range(5)}   # _sample keeps an even count
    used = {op: 0 for op in range(5)}
    rows = []
    for op in ops:
        c = picks[op]
        k = used[op]; used[op] += 1
        rows.append((c[0][k], c[1][k], c[2][k] if op != 4 else 0, c[3][k] if op != 4 else np.zeros(n, np.uint32)))
    ae = np.array([r[0] for r in rows], np.uint32); al = np.stack([r[1] for r in rows])
    be = np.array([r[2] for r in rows], np.uint32); bl = np.stack([r[3] for r in rows])
    for mode in (0, 3):
        err, ge, gl = run_cta(cta_binary, shape, 60, n, mode, (ae, al, be, bl, ops, np.zeros_like(al)), 1, blocks)
        assert err == 0
        for op in range(5):
            m = ops == op
            ee, el = (oracle.run(op, n, mode, ae[m], al[m], be[m], bl[m]) if op != 4
                      else oracle.run(op, n, mode, ae[m], al[m]))
            assert np.array_equal(ge[m], ee), (op, n, mode)
            assert np.array_equal(gl[m][ee > 8], el[ee > 8]), (op, n, mode)


def test_batch_dispatcher_has_no_races(cta_tsan_binary, monkeypatch):
    """The dispatcher's shared task word under ThreadSanitizer: thread 0 writes it, every
    thread reads it between the two CTA barriers, and the next write comes after both."""
    monkeypatch.setenv("TSAN_OPTIONS", "halt_on_error=1 exitcode=66")
    n = 5
    rng = np.random.default_rng(11100)
    a = _sample(addsub_cases(rng, n), 24)
    d = _sample(div_cases(rng, n), 24)
    ops = np.array([0] * 10 + [3] * 10 + [1] * 10 + [4] * 10, np.uint32)
    ae = np.concatenate([a[0][:10], d[0][:10], a[0][10:20], d[0][10:20]])
    al = np.concatenate([a[1][:10], d[1][:10], a[1][10:20], d[1][10:20]])
    be = np.concatenate([a[2][:10], d[2][:10], a[2][10:20], d[2][10:20]])
    bl = np.concatenate([a[3][:10], d[3][:10], a[3][10:20], d[3][10:20]])
    err, _, _ = run_cta(cta_tsan_binary, (4, 2, 1), 60, n, 3, (ae, al, be, bl, ops, np.zeros_like(al)), 1, 2)
    assert err == 0
