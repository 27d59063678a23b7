// fpa_batch.cu -- host side of the batched form: one submission runs many operations of
// mixed type and precision.
//
// Plan: every descriptor gets a lane-group configuration (autotuned table, per operation
// and limb count) and therefore a register class; descriptors are sorted by (class,
// configuration, operation, limbs descending) and cut into tasks of about two operations
// per lane group of a CTA, ordered longest-first within each class (longest processing
// time first keeps the persistent CTAs evenly loaded to the end).
// Run: one persistent kernel per non-empty class (fpa_batch_kernels.cu), class 0 on the
// caller's stream and classes 1 and 2 on forked side streams so they share the GPU
// concurrently; a run can be captured once as a CUDA graph and replayed with one launch.
// Batches created by fpa_batch_create also send mul, div and sqrt of 8 to 128 limbs whose
// tuned configuration is a one-thread one to a fourth class (fpa_batch_thread.cu: tasks of
// up to 32 operations of one operation and limb count, one operation per thread, its two
// launches on the caller's stream after class 0).
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>
#include "../../include/fpa_gb300.h"
#include "fpa_ops.cuh"
#include "fpa_launch.h"
#include "fpa_batch.h"

using namespace gfpa;

namespace {

// shared-memory words one warp needs for (configuration, operation)
int warp_words_for(int cfg, int op) {
#define GFPA_W(CFG, GG, KK, RR)                                                               \
  if (cfg == CFG) {                                                                          \
    switch (op) {                                                                            \
      case OP_ADD: case OP_SUB: return (32 / GG) * OpWords<OP_ADD, GG, KK, RR>::aligned();     \
      case OP_MUL: return (32 / GG) * OpWords<OP_MUL, GG, KK, RR>::aligned();                   \
      case OP_DIV: return (32 / GG) * OpWords<OP_DIV, GG, KK, RR>::aligned();                   \
      default: return (32 / GG) * OpWords<OP_SQRT, GG, KK, RR>::aligned();                      \
    }                                                                                        \
  }
  GFPA_W(0, 4, 2, 1) GFPA_W(1, 8, 2, 1) GFPA_W(2, 8, 4, 1) GFPA_W(3, 16, 4, 1) GFPA_W(4, 32, 4, 1)
  GFPA_W(5, 32, 8, 1) GFPA_W(6, 32, 16, 1) GFPA_W(7, 16, 8, 1) GFPA_W(8, 8, 16, 1) GFPA_W(9, 16, 16, 1)
  GFPA_W(10, 8, 4, 2) GFPA_W(11, 8, 4, 4) GFPA_W(12, 16, 4, 2) GFPA_W(13, 8, 8, 4) GFPA_W(14, 16, 8, 2)
  GFPA_W(15, 4, 4, 8)
#undef GFPA_W
  return 0;
}

// relative cost used to order tasks (products plus fixed per-operation work)
double op_weight(int op, int n) {
  const double nn = (double)n * n;
  switch (op) {
    case OP_ADD: case OP_SUB: return 64.0 * n + 2000.0;
    case OP_MUL: return nn + 4000.0;
    case OP_DIV: return 4.0 * nn + 40000.0;
    default: return 6.0 * nn + 60000.0;
  }
}

cudaError_t prepare(int c, size_t smem, int *per_sm) {
  switch (c) {
    case 0: return gfpa_batch_prepare0(smem, per_sm);
    case 1: return gfpa_batch_prepare1(smem, per_sm);
    default: return gfpa_batch_prepare2(smem, per_sm);
  }
}

cudaError_t launch(int c, const BatchArgs *a, int grid, size_t smem, cudaStream_t st) {
  switch (c) {
    case 0: return gfpa_batch_launch0(a, grid, smem, st);
    case 1: return gfpa_batch_launch1(a, grid, smem, st);
    default: return gfpa_batch_launch2(a, grid, smem, st);
  }
}

}  // namespace

int gfpa_batch_warp_words(int cfg, int op) { return warp_words_for(cfg, op); }

int gfpa_batch_cfg_for(int op, uint32_t n) {
  const int cfg = gfpa_cfg_for_op(op, n);
  if (cfg < 0) return cfg;
  // A class kernel's CTAs all carry the largest shared-memory slice among its tasks, so one
  // configuration with a large slice lowers the occupancy of every task in its class.  The
  // elementwise table's choice is kept only while a warp's slice leaves room for three CTAs
  // of its class on an SM; otherwise (and for configurations 16 and 17, which have
  // elementwise kernels only) the default configuration is used.
  const int dflt = gfpa_default_cfg(n < 4 ? 4 : n);
  const size_t budget = (227 * 1024 / 3) / (size_t)(gfpa_class_threads[gfpa_class_of(cfg, op)] / 32);
  if (gfpa_cfg_elementwise_only(cfg) || (size_t)warp_words_for(cfg, op) * 4 > budget) return dflt;
  return cfg;
}
double gfpa_batch_op_weight(int op, int n) { return op_weight(op, n); }
cudaError_t gfpa_batch_prepare_class(int c, size_t smem, int *per_sm) { return prepare(c, smem, per_sm); }
cudaError_t gfpa_batch_launch_class(int c, const BatchArgs *a, int grid, size_t smem, cudaStream_t st) {
  return launch(c, a, grid, smem, st);
}

fpa_result gfpa_batch_plan(const fpa_batch_desc *descs, uint64_t count, int sms, BatchPlan &plan, bool one_thread,
                           int thread_grid_cap) {
  if (count > 0xFFFFFFFFull) return fpa_invalid_counts;
  if (count && !descs) return fpa_math_error;
  std::vector<uint32_t> &order = plan.order;
  order.resize(count);
  std::vector<uint16_t> key(count);
  std::vector<uint8_t> cls(count);
  // (key, class) of each (operation, limb count), worked out once per pair present
  std::vector<int32_t> memo(5 * (GFPA_MAX_LIMBS + 1), -1);
  std::vector<uint32_t> used;                             // memo entries in use
  std::vector<uint32_t> slot(count);                      // each operation's memo entry
  for (uint64_t i = 0; i < count; i++) {
    const fpa_batch_desc &d = descs[i];
    if (d.op > 4 || d.mode > 4) return fpa_math_error;
    if (d.limbs == 0 || d.limbs > GFPA_MAX_LIMBS) return fpa_invalid_precisions;
    const uint32_t me = d.op * (GFPA_MAX_LIMBS + 1) + d.limbs;
    int32_t &m = memo[me];
    if (m < 0) {
      const int tcfg =
          one_thread && d.op >= OP_MUL && d.limbs >= 8 && d.limbs <= 128 ? gfpa_cfg_for_op(d.op, d.limbs) : -1;
      if (tcfg == 18 || tcfg == 19) {                     // one thread per operation
        m = ((18 * 5 + d.op) << 8) | GFPA_THREAD_CLASS;
      } else {
        const int cfg = gfpa_batch_cfg_for(d.op, d.limbs);
        if (cfg < 0) return fpa_invalid_precisions;
        m = ((cfg * 5 + d.op) << 8) | gfpa_class_of(cfg, d.op);
      }
      used.push_back(me);
    }
    key[i] = (uint16_t)(m >> 8);
    cls[i] = (uint8_t)(m & 0xFF);
    slot[i] = me;
  }
  // order by (class, configuration * 5 + operation, limbs descending, index): a counting sort
  // over the (operation, limb count) pairs present, ranked by their (class, key, limbs)
  std::sort(used.begin(), used.end(), [&](uint32_t x, uint32_t y) {
    const int32_t mx = memo[x], my = memo[y];
    if ((mx & 0xFF) != (my & 0xFF)) return (mx & 0xFF) < (my & 0xFF);
    if ((mx >> 8) != (my >> 8)) return (mx >> 8) < (my >> 8);
    return x % (GFPA_MAX_LIMBS + 1) > y % (GFPA_MAX_LIMBS + 1);
  });
  std::vector<uint32_t> rank(memo.size(), 0), start(used.size() + 1, 0);
  for (size_t k = 0; k < used.size(); k++) rank[used[k]] = (uint32_t)k;
  for (uint64_t i = 0; i < count; i++) start[rank[slot[i]] + 1]++;
  for (size_t k = 1; k < start.size(); k++) start[k] += start[k - 1];
  for (uint64_t i = 0; i < count; i++) order[start[rank[slot[i]]]++] = (uint32_t)i;
  std::vector<BatchTask> tasks[4];
  std::vector<double> cost[4];
  uint64_t i = 0;
  plan.thread_ops = 0;
  while (i < count && cls[order[i]] != GFPA_THREAD_CLASS) {
    uint64_t j = i;
    const uint16_t k = key[order[i]];
    while (j < count && key[order[j]] == k) j++;
    const int cfg = k / 5, op = k % 5, c = gfpa_class_of(cfg, op);
    const int groups = (gfpa_class_threads[c] / 32) * (32 / gfpa_cfg_G[cfg]);
    const uint64_t chunk = (uint64_t)groups * 2;
    for (uint64_t s = i; s < j; s += chunk) {
      BatchTask t;
      t.key = k; t.pad = 0; t.first = (uint32_t)s;
      t.count = (uint32_t)std::min<uint64_t>(chunk, j - s);
      double w = 0;
      for (uint64_t q = s; q < s + t.count; q++) w += op_weight(op, descs[order[q]].limbs);
      tasks[c].push_back(t);
      cost[c].push_back(w / groups);
    }
    i = j;
  }
  // one-thread class: runs of one (operation, limb count), 32 operations per task
  while (i < count) {
    uint64_t j = i;
    const fpa_batch_desc &d0 = descs[order[i]];
    while (j < count && descs[order[j]].op == d0.op && descs[order[j]].limbs == d0.limbs) j++;
    for (uint64_t s = i; s < j; s += 32) {
      BatchTask t;
      t.key = (uint16_t)(18 * 5 + d0.op); t.pad = 0; t.first = (uint32_t)s;
      t.count = (uint32_t)std::min<uint64_t>(32, j - s);
      tasks[GFPA_THREAD_CLASS].push_back(t);
      cost[GFPA_THREAD_CLASS].push_back(op_weight(d0.op, d0.limbs));
    }
    plan.thread_ops += j - i;
    i = j;
  }
  plan.tasks.clear();
  for (int c = 0; c < 4; c++) {
    std::vector<size_t> idx(tasks[c].size());
    for (size_t q = 0; q < idx.size(); q++) idx[q] = q;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return cost[c][x] > cost[c][y]; });
    plan.task_base[c] = (uint32_t)plan.tasks.size();
    plan.ntasks[c] = (uint32_t)idx.size();
    for (size_t q : idx) plan.tasks.push_back(tasks[c][q]);
    plan.grid[c] = 0;
    if (c == GFPA_THREAD_CLASS) {
      plan.smem[c] = gfpa_batch_thread_smem();
      if (plan.ntasks[c]) {
        int per = 0;
        if (gfpa_batch_thread_prepare(&per) != cudaSuccess) return fpa_device_error;
        if (per < 1) per = 1;
        plan.grid[c] = (int)std::min<uint64_t>((uint64_t)per * sms, plan.ntasks[c]);
        if (thread_grid_cap > 0) plan.grid[c] = std::min(plan.grid[c], thread_grid_cap);
      }
      continue;
    }
    uint32_t ww = 0;
    for (size_t q : idx) ww = std::max<uint32_t>(ww, (uint32_t)warp_words_for(tasks[c][q].key / 5, tasks[c][q].key % 5));
    plan.warp_words[c] = ww;
    plan.smem[c] = (size_t)(gfpa_class_threads[c] / 32) * ww * 4;
    if (plan.smem[c] > 227 * 1024) return fpa_device_error;
    if (plan.ntasks[c]) {
      int per = 0;
      if (prepare(c, plan.smem[c], &per) != cudaSuccess) return fpa_device_error;
      if (per < 1) per = 1;
      plan.grid[c] = (int)std::min<uint64_t>((uint64_t)per * sms, plan.ntasks[c]);
    }
  }
  return fpa_success;
}

cudaError_t gfpa_batch_enqueue(const BatchPlan &plan, const fpa_batch_desc *d_descs, const uint32_t *d_order,
                               const BatchTask *d_tasks, uint32_t *d_counters, uint32_t *r_exps, uint32_t *r_limbs,
                               const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                               const uint32_t *b_limbs, cudaStream_t st, const cudaStream_t side[2],
                               cudaEvent_t fork, const cudaEvent_t join[2], const ThreadScratch *ts) {
  uint32_t *err;
  int sms;
  if (!gfpa_context(&sms, &err)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counters, 0, 16, st);
  if (e != cudaSuccess) return e;
  BatchArgs A;
  A.descs = d_descs; A.order = d_order; A.err = err;
  A.r_exps = r_exps; A.r_limbs = r_limbs; A.a_exps = a_exps; A.a_limbs = a_limbs;
  A.b_exps = b_exps ? b_exps : a_exps; A.b_limbs = b_limbs ? b_limbs : a_limbs;
  if ((e = cudaEventRecord(fork, st)) != cudaSuccess) return e;
  const cudaStream_t streams[3] = {st, side[0], side[1]};
  for (int c = 1; c < 3; c++)
    if ((e = cudaStreamWaitEvent(streams[c], fork, 0)) != cudaSuccess) return e;
  for (int c = 0; c < 3; c++) {
    if (!plan.ntasks[c]) continue;
    A.tasks = d_tasks + plan.task_base[c];
    A.ntasks = plan.ntasks[c];
    A.counter = d_counters + c;
    A.warp_words = plan.warp_words[c];
    if ((e = launch(c, &A, plan.grid[c], plan.smem[c], streams[c])) != cudaSuccess) return e;
  }
  if (plan.ntasks[GFPA_THREAD_CLASS]) {
    if (!ts || !ts->slabs) return cudaErrorInvalidValue;
    ThreadBatchArgs T;
    T.b = A;
    T.b.tasks = d_tasks + plan.task_base[GFPA_THREAD_CLASS];
    T.b.ntasks = plan.ntasks[GFPA_THREAD_CLASS];
    T.b.counter = d_counters + GFPA_THREAD_CLASS;
    T.b.warp_words = 0;
    T.slabs = ts->slabs; T.hard_count = ts->hard_count; T.hard_idx = ts->hard_idx;
    if ((e = gfpa_batch_thread_launch(&T, plan.grid[GFPA_THREAD_CLASS], st)) != cudaSuccess) return e;
  }
  for (int c = 1; c < 3; c++) {
    if ((e = cudaEventRecord(join[c - 1], streams[c])) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, join[c - 1], 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

struct fpa_batch_s {
  uint64_t count = 0;
  BatchPlan plan;
  fpa_batch_desc *d_descs = nullptr;
  uint32_t *d_order = nullptr;
  BatchTask *d_tasks = nullptr;
  uint32_t *d_counters = nullptr;     // one per class
  ThreadScratch ts;                   // the one-thread class's slabs and deferred list
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" fpa_result fpa_batch_create(fpa_batch_t *out, const fpa_batch_desc *descs, uint64_t count) {
  if (!out) return fpa_math_error;
  *out = nullptr;
  int sms;
  if (!gfpa_context(&sms, nullptr)) return fpa_device_error;
  fpa_batch_s *b = new fpa_batch_s();
  b->count = count;
  fpa_result r = gfpa_batch_plan(descs, count, sms, b->plan, true);
  if (r != fpa_success) { delete b; return r; }
  const std::vector<BatchTask> &all = b->plan.tasks;
  bool ok = true;
  ok = ok && cudaMalloc(&b->d_descs, std::max<size_t>(1, count) * sizeof(fpa_batch_desc)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_order, std::max<size_t>(1, count) * 4) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_tasks, std::max<size_t>(1, all.size()) * sizeof(BatchTask)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_counters, 16) == cudaSuccess;
  if (ok && b->plan.ntasks[GFPA_THREAD_CLASS]) {
    ok = cudaMalloc(&b->ts.slabs, gfpa_batch_thread_slab_bytes(b->plan.grid[GFPA_THREAD_CLASS])) == cudaSuccess &&
         cudaMalloc(&b->ts.hard_count, 256) == cudaSuccess &&
         cudaMalloc(&b->ts.hard_idx, std::max<size_t>(1, b->plan.thread_ops) * 4) == cudaSuccess;
  }
  if (ok && count)
    ok = cudaMemcpy(b->d_descs, descs, count * sizeof(fpa_batch_desc), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_order, b->plan.order.data(), count * 4, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok && !all.empty())
    ok = cudaMemcpy(b->d_tasks, all.data(), all.size() * sizeof(BatchTask), cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&b->side[0], cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&b->side[1], cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->ev_join[0], cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->ev_join[1], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) { fpa_batch_destroy(b); return fpa_device_error; }
  *out = b;
  return fpa_success;
}

static cudaError_t batch_enqueue(fpa_batch_t b, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
                                 const uint32_t *a_limbs, const uint32_t *b_exps, const uint32_t *b_limbs,
                                 cudaStream_t st) {
  return gfpa_batch_enqueue(b->plan, b->d_descs, b->d_order, b->d_tasks, b->d_counters, r_exps, r_limbs, a_exps,
                            a_limbs, b_exps, b_limbs, st, b->side, b->ev_fork, b->ev_join, &b->ts);
}

extern "C" fpa_result fpa_batch_run(fpa_batch_t b, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
                                    const uint32_t *a_limbs, const uint32_t *b_exps, const uint32_t *b_limbs,
                                    void *stream) {
  if (!b) return fpa_math_error;
  if (b->count == 0) return fpa_success;
  return batch_enqueue(b, r_exps, r_limbs, a_exps, a_limbs, b_exps, b_limbs, (cudaStream_t)stream) == cudaSuccess
             ? fpa_success : fpa_device_error;
}

extern "C" fpa_result fpa_batch_capture(fpa_batch_t b, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
                                        const uint32_t *a_limbs, const uint32_t *b_exps, const uint32_t *b_limbs) {
  if (!b) return fpa_math_error;
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  if (b->count == 0) return fpa_success;
  cudaStream_t cs;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return fpa_device_error;
  fpa_result res = fpa_device_error;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    cudaError_t e = batch_enqueue(b, r_exps, r_limbs, a_exps, a_limbs, b_exps, b_limbs, cs);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess && e2 == cudaSuccess && g) {
      b->graph = g;
      if (cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess) res = fpa_success;
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  cudaStreamDestroy(cs);
  return res;
}

extern "C" fpa_result fpa_batch_graph_launch(fpa_batch_t b, void *stream) {
  if (!b) return fpa_math_error;
  if (b->count == 0) return fpa_success;
  if (!b->exec) return fpa_math_error;
  return cudaGraphLaunch(b->exec, (cudaStream_t)stream) == cudaSuccess ? fpa_success : fpa_device_error;
}

extern "C" fpa_result fpa_batch_info(fpa_batch_t b, uint32_t *tasks_per_class, uint32_t *kernels) {
  if (!b) return fpa_math_error;
  uint32_t k = 0;
  for (int c = 0; c < 3; c++) {
    if (tasks_per_class) tasks_per_class[c] = b->plan.ntasks[c];
    k += b->plan.ntasks[c] ? 1 : 0;
  }
  k += b->plan.ntasks[GFPA_THREAD_CLASS] ? 1 : 0;
  if (kernels) *kernels = k;
  return fpa_success;
}

extern "C" fpa_result fpa_batch_destroy(fpa_batch_t b) {
  if (!b) return fpa_success;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  for (int c = 0; c < 2; c++) {
    if (b->ev_join[c]) cudaEventDestroy(b->ev_join[c]);
    if (b->side[c]) cudaStreamDestroy(b->side[c]);
  }
  cudaFree(b->d_descs); cudaFree(b->d_order); cudaFree(b->d_tasks); cudaFree(b->d_counters);
  cudaFree(b->ts.slabs); cudaFree(b->ts.hard_count); cudaFree(b->ts.hard_idx);
  delete b;
  return fpa_success;
}
