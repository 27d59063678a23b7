// fpa_serve.cu -- the served form: a request loop with continuous batching.
//
// Callers submit jobs (one precision, many operations of mixed type) from any thread.  A
// server thread keeps up to `max_inflight` batches on the GPU at once.  Each batch lives in
// a slot: a device arena and a pinned host staging area carved out of the HBM budget at
// creation, plus its own streams.  Whenever a slot is free the loop admits pending jobs in
// arrival order while they fit the slot's arena (the HBM budget), packs their operands,
// plans them with the batched form's planner and enqueues copy-in, the class kernels and
// copy-out on the slot's streams; finished slots hand results back to their jobs.  Jobs
// that arrive while other batches run are therefore admitted as soon as a slot frees and
// their work overlaps on the device with the batches already in flight.
//
// With `batching = 0` the same loop serves each job alone with plain per-operation-type
// elementwise launches, one job at a time: the comparison point for the batched form.
// No CUDA allocation or free happens after creation.
//
// Device-resident results (batching only): a job may keep its result in the server's
// resident store (one device allocation made at creation, handed out first fit) and may take
// either operand from an earlier job's kept result.  Such an operand is copied device to
// device into the batch after the host-to-device copy; when its source is still in flight,
// the copy waits on the source batch's event on the GPU, so a chain of jobs never returns to
// the host between steps.  A job whose source has not been launched yet waits in the queue
// (later jobs may pass it), and fails if a source fails.  A kept result stays until the job
// is released; a source with dependents still pending cannot be released.
//
// Cost account: each batch records CUDA events around its host-to-device copies, its kernels
// and its device-to-host copy, and the server thread times its own packing and planning;
// fpa_server_costs returns the sums.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>
#include <string.h>
#include "../../include/fpa_gb300.h"
#include "fpa_launch.h"
#include "fpa_batch.h"

namespace {

using Clock = std::chrono::steady_clock;

enum JobState { JOB_PENDING = 0, JOB_ADMITTED = 1, JOB_DONE = 2, JOB_FAILED = 3 };

struct Job {
  int64_t id = 0;
  uint32_t n = 0, count = 0;
  std::vector<uint8_t> ops, modes;
  const uint32_t *a_exps = nullptr, *a_limbs = nullptr, *b_exps = nullptr, *b_limbs = nullptr;
  uint32_t *r_exps = nullptr, *r_limbs = nullptr;
  uint64_t bytes = 0;
  uint64_t t_submit = 0, t_admit = 0, t_done = 0;
  int state = JOB_PENDING;
  // device-resident results
  Job *a_src = nullptr, *b_src = nullptr;   // kept results the operands come from
  bool keep = false, copy_out = true;
  uint64_t res_off = 0, res_bytes = 0;      // this job's block of the resident store (keep)
  int slot = -1;                            // slot of the batch that computes it
  int deps = 0;                             // pending jobs that read this job's kept result
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Host work of a batch -- copies of its operands into pinned staging and of its results back
// out (split into pieces of at most 1 MB), and the descriptor fill, job by job -- run by
// worker threads together with the server thread: on one thread this packing bounded the
// served form (the cost account showed 28 ms of packing against 4.5 ms of kernels for a
// 266 MB burst).
struct Copy {
  void *dst;
  const void *src;   // nullptr: fill dst with zeros
  size_t bytes;
};

class CopyPool {
 public:
  explicit CopyPool(int workers) {
    for (int i = 0; i < workers; i++) threads_.emplace_back([this] { work(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread &t : threads_) t.join();
  }
  // Runs every copy; returns when all are done.  Called by one thread at a time.
  void run(const std::vector<Copy> &copies) {
    std::vector<Copy> pieces;
    constexpr size_t kPiece = 1 << 20;
    for (const Copy &c : copies)
      for (size_t o = 0; o < c.bytes; o += kPiece)
        pieces.push_back({(uint8_t *)c.dst + o, c.src ? (const uint8_t *)c.src + o : nullptr,
                          std::min(kPiece, c.bytes - o)});
    for_each(pieces.size(), [&pieces](size_t i) {
      const Copy &c = pieces[i];
      if (c.src) memcpy(c.dst, c.src, c.bytes);
      else memset(c.dst, 0, c.bytes);
    });
  }
  // Runs fn(0 .. n-1) on the workers and the calling thread; returns when all are done.
  // Each call is a round of its own: a worker that wakes late finds that round's items
  // taken and leaves it, whatever later rounds are doing.
  template <class Fn>
  void for_each(size_t n, Fn &&fn) {
    if (n < 2 || threads_.empty()) {
      for (size_t i = 0; i < n; i++) fn(i);
      return;
    }
    auto r = std::make_shared<Round>();
    r->fn = std::forward<Fn>(fn);
    r->n = n;
    {
      std::lock_guard<std::mutex> lk(mu_);
      round_ = r;
      gen_++;
    }
    cv_.notify_all();
    drain(*r);
    while (r->done.load() < n) std::this_thread::yield();
  }

 private:
  struct Round {
    std::function<void(size_t)> fn;
    size_t n = 0;
    std::atomic<size_t> next{0}, done{0};
  };
  static void drain(Round &r) {
    for (;;) {
      const size_t i = r.next.fetch_add(1);
      if (i >= r.n) return;
      r.fn(i);
      r.done.fetch_add(1);
    }
  }
  void work() {
    uint64_t seen = 0;
    for (;;) {
      std::shared_ptr<Round> r;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        r = round_;
      }
      drain(*r);
    }
  }
  std::vector<std::thread> threads_;
  std::shared_ptr<Round> round_;
  std::mutex mu_;
  std::condition_variable cv_;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// device bytes one operation of n limbs needs inside a batch (descriptor, order, task
// share, deferred-list entry, three exponents, three mantissas)
uint64_t op_bytes(uint32_t n) { return 32 + 4 + 16 + 4 + 12 + 12ull * n; }

// The resident store's free blocks (offset -> bytes): first fit, and a released block merges
// with free neighbours on both sides, so the free list never holds two adjacent blocks.
struct ResidentStore {
  std::map<uint64_t, uint64_t> free_blocks;
  void reset(uint64_t cap) {
    free_blocks.clear();
    if (cap) free_blocks.emplace(0, cap);
  }
  // offset of a block of `bytes`, or UINT64_MAX when no free block is large enough
  uint64_t alloc(uint64_t bytes) {
    for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
      if (it->second < bytes) continue;
      const uint64_t off = it->first, rest = it->second - bytes;
      free_blocks.erase(it);
      if (rest) free_blocks.emplace(off + bytes, rest);
      return off;
    }
    return UINT64_MAX;
  }
  void release(uint64_t off, uint64_t bytes) {
    auto it = free_blocks.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_blocks.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_blocks.erase(nx);
    }
    if (it != free_blocks.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_blocks.erase(it);
      }
    }
  }
};

struct Slot {
  cudaStream_t st = nullptr, side[2] = {nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr}, done = nullptr;
  cudaEvent_t kept = nullptr;                        // the batch's kept results are in the store
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};   // timing: in, inputs copied, computed, out
  uint64_t pack_ns = 0;
  uint8_t *d_arena = nullptr, *h_stage = nullptr;
  size_t cap = 0, used = 0;             // arena capacity, bytes of the batch in flight
  uint32_t *thread_slabs = nullptr;     // the one-thread class's slabs, at the end of the arena
  bool busy = false;
  std::vector<Job *> jobs;
  std::vector<uint64_t> job_first;      // first op index of each job in the batch
  std::vector<uint64_t> job_limb0;      // first limb offset of each job in the pools
  size_t o_re = 0, o_rl = 0;            // result sections
  uint64_t nops = 0, nlimbs = 0;
  BatchPlan plan;
  std::vector<uint32_t> perm;           // plain mode: staged position -> job-local op index
};

}  // namespace

struct fpa_server_s {
  fpa_server_config cfg;
  int sms = 0, device = 0;
  int thread_grid = 0;                  // CTAs of the one-thread class per batch (0: class off)
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> pending;
  std::unordered_map<int64_t, std::unique_ptr<Job>> jobs;
  int64_t next_id = 1;
  bool stop = false;
  std::thread thread;
  std::unique_ptr<CopyPool> pool;        // host copies, used by the server thread only
  Clock::time_point t0;
  // statistics
  std::atomic<uint64_t> jobs_done{0}, ops_done{0}, batches{0}, peak_bytes{0}, resident{0}, failures{0};
  std::atomic<uint64_t> cost_ns[4] = {{0}, {0}, {0}, {0}};   // pack, h2d, device, d2h
  // resident store, its free blocks guarded by mu
  uint8_t *d_res = nullptr;
  uint64_t res_cap = 0;
  ResidentStore res_store;

  uint64_t now() const {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
  }
  bool launch(Slot &s, std::vector<Job *> &batch);
  void retire(Slot &s, bool ok);
  void loop();
};

// Pack `batch` into slot `s` and enqueue its copy-in, kernels and copy-out.
bool fpa_server_s::launch(Slot &s, std::vector<Job *> &batch) {
  const uint64_t t_pack0 = now();
  s.jobs = batch;
  s.job_first.clear(); s.job_limb0.clear();
  uint64_t nops = 0, nlimbs = 0;
  for (Job *j : batch) {
    s.job_first.push_back(nops); s.job_limb0.push_back(nlimbs);
    nops += j->count; nlimbs += (uint64_t)j->count * j->n;
  }
  s.nops = nops; s.nlimbs = nlimbs;
  const bool batching = cfg.batching != 0;
  // section layout (same offsets in the device arena and the pinned staging area)
  size_t off = 0;
  const size_t o_descs = off; off = align256(off + nops * sizeof(fpa_batch_desc));
  const size_t o_order = off; off = align256(off + nops * 4);
  const size_t o_tasks = off; off = align256(off + (nops + 3) * sizeof(BatchTask));
  const size_t o_cnt = off; off = align256(off + 16);
  const size_t o_hard = off; off = align256(off + 16 + nops * 4);    // one-thread class: deferred list
  const size_t o_ae = off; off = align256(off + nops * 4);
  const size_t o_be = off; off = align256(off + nops * 4);
  const size_t o_al = off; off = align256(off + nlimbs * 4);
  const size_t o_bl = off; off = align256(off + nlimbs * 4);
  const size_t in_end = off;
  s.o_re = off; off = align256(off + nops * 4);
  s.o_rl = off; off = align256(off + nlimbs * 4);
  if (off > s.cap) return false;
  uint8_t *H = s.h_stage, *D = s.d_arena;
  fpa_batch_desc *descs = (fpa_batch_desc *)(H + o_descs);
  uint32_t *ae = (uint32_t *)(H + o_ae), *be = (uint32_t *)(H + o_be);
  uint32_t *al = (uint32_t *)(H + o_al), *bl = (uint32_t *)(H + o_bl);
  s.perm.clear();
  if (batching) {
    std::vector<Copy> copies;
    for (size_t q = 0; q < batch.size(); q++) {
      Job *j = batch[q];
      const uint64_t f = s.job_first[q], l0 = s.job_limb0[q], jl = (uint64_t)j->count * j->n;
      if (!j->a_src) {                          // (a kept operand is copied on the device below)
        copies.push_back({ae + f, j->a_exps, (size_t)j->count * 4});
        copies.push_back({al + l0, j->a_limbs, (size_t)jl * 4});
      }
      if (!j->b_src) {
        copies.push_back({be + f, j->b_exps, (size_t)j->count * 4});
        copies.push_back({bl + l0, j->b_limbs, (size_t)jl * 4});
      }
    }
    pool->run(copies);
    pool->for_each(batch.size(), [&](size_t q) {
      Job *j = batch[q];
      const uint64_t f = s.job_first[q], l0 = s.job_limb0[q];
      for (uint32_t i = 0; i < j->count; i++) {
        fpa_batch_desc &d = descs[f + i];
        d.op = j->ops[i]; d.mode = j->modes[i]; d.limbs = (uint16_t)j->n; d.reserved = 0;
        d.r_off = d.a_off = d.b_off = l0 + (uint64_t)i * j->n;
      }
    });
    if (gfpa_batch_plan(descs, nops, sms, s.plan, s.thread_slabs != nullptr, thread_grid) != fpa_success) return false;
    if (s.plan.tasks.size() > nops + 3) return false;
    memcpy(H + o_order, s.plan.order.data(), nops * 4);
    memcpy(H + o_tasks, s.plan.tasks.data(), s.plan.tasks.size() * sizeof(BatchTask));
  } else {
    // plain: one job, operations grouped by type so each type is one elementwise launch
    Job *j = batch[0];
    const uint32_t n = j->n;
    s.perm.resize(j->count);
    for (uint32_t i = 0; i < j->count; i++) s.perm[i] = i;
    std::stable_sort(s.perm.begin(), s.perm.end(), [&](uint32_t x, uint32_t y) {
      return j->ops[x] != j->ops[y] ? j->ops[x] < j->ops[y] : j->modes[x] < j->modes[y];
    });
    for (uint32_t p = 0; p < j->count; p++) {
      const uint32_t i = s.perm[p];
      ae[p] = j->a_exps[i];
      be[p] = j->b_exps ? j->b_exps[i] : 0u;
      memcpy(al + (uint64_t)p * n, j->a_limbs + (uint64_t)i * n, n * 4);
      if (j->b_limbs) memcpy(bl + (uint64_t)p * n, j->b_limbs + (uint64_t)i * n, n * 4);
      else memset(bl + (uint64_t)p * n, 0, n * 4);
    }
  }
  const uint64_t t = now();
  s.pack_ns = t - t_pack0;
  const int slot_index = (int)(&s - slots.data());
  for (Job *j : batch) { j->t_admit = t; j->state = JOB_ADMITTED; j->slot = slot_index; }
  cudaError_t e = cudaEventRecord(s.ev[0], s.st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(D, H, in_end, cudaMemcpyHostToDevice, s.st);
  // operands taken from kept results: device-to-device into the batch's input sections
  for (size_t q = 0; q < batch.size() && e == cudaSuccess && batching; q++) {
    Job *j = batch[q];
    const uint64_t f = s.job_first[q], l0 = s.job_limb0[q], jl = (uint64_t)j->count * j->n;
    for (int which = 0; which < 2 && e == cudaSuccess; which++) {
      Job *src = which == 0 ? j->a_src : j->b_src;
      if (!src) continue;
      if (src->state != JOB_DONE) e = cudaStreamWaitEvent(s.st, slots[src->slot].kept, 0);
      const uint8_t *R = d_res + src->res_off;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(D + (which == 0 ? o_ae : o_be) + f * 4, R, (size_t)j->count * 4, cudaMemcpyDeviceToDevice, s.st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(D + (which == 0 ? o_al : o_bl) + l0 * 4, R + align256((size_t)j->count * 4), jl * 4,
                            cudaMemcpyDeviceToDevice, s.st);
    }
  }
  if (e == cudaSuccess) e = cudaEventRecord(s.ev[1], s.st);
  uint32_t *d_re = (uint32_t *)(D + s.o_re), *d_rl = (uint32_t *)(D + s.o_rl);
  if (e == cudaSuccess) {
    if (batching) {
      ThreadScratch ts;
      ts.slabs = s.thread_slabs;
      ts.hard_count = (uint32_t *)(D + o_hard);
      ts.hard_idx = ts.hard_count + 4;
      e = gfpa_batch_enqueue(s.plan, (const fpa_batch_desc *)(D + o_descs), (const uint32_t *)(D + o_order),
                             (const BatchTask *)(D + o_tasks), (uint32_t *)(D + o_cnt), d_re, d_rl,
                             (const uint32_t *)(D + o_ae), (const uint32_t *)(D + o_al),
                             (const uint32_t *)(D + o_be), (const uint32_t *)(D + o_bl), s.st, s.side, s.fork,
                             s.join, &ts);
    } else {
      Job *j = batch[0];
      uint32_t *err;
      int smsx;
      gfpa_context(&smsx, &err);
      uint32_t p = 0;
      while (p < j->count && e == cudaSuccess) {
        const uint32_t i0 = s.perm[p];
        uint32_t q = p;
        while (q < j->count && j->ops[s.perm[q]] == j->ops[i0] && j->modes[s.perm[q]] == j->modes[i0]) q++;
        ElementwiseArgs a;
        a.count = q - p; a.n = j->n; a.mode = j->modes[i0];
        a.r_exps = d_re + p; a.r_limbs = d_rl + (uint64_t)p * j->n;
        a.a_exps = (const uint32_t *)(D + o_ae) + p; a.a_limbs = (const uint32_t *)(D + o_al) + (uint64_t)p * j->n;
        a.b_exps = (const uint32_t *)(D + o_be) + p; a.b_limbs = (const uint32_t *)(D + o_bl) + (uint64_t)p * j->n;
        a.err = err;
        const int cfgi = gfpa_cfg_for_op(j->ops[i0], j->n);
        e = cfgi < 0 ? cudaErrorInvalidValue : gfpa_launch(cfgi, j->ops[i0], &a, s.st, sms);
        p = q;
      }
    }
  }
  // kept results: device-to-device into the resident store
  for (size_t q = 0; q < batch.size() && e == cudaSuccess && batching; q++) {
    Job *j = batch[q];
    if (!j->keep) continue;
    const uint64_t f = s.job_first[q], l0 = s.job_limb0[q], jl = (uint64_t)j->count * j->n;
    uint8_t *R = d_res + j->res_off;
    e = cudaMemcpyAsync(R, d_re + f, (size_t)j->count * 4, cudaMemcpyDeviceToDevice, s.st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R + align256((size_t)j->count * 4), d_rl + l0, jl * 4, cudaMemcpyDeviceToDevice, s.st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(s.kept, s.st);
  if (e == cudaSuccess) e = cudaEventRecord(s.ev[2], s.st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H + s.o_re, D + s.o_re, off - s.o_re, cudaMemcpyDeviceToHost, s.st);
  if (e == cudaSuccess) e = cudaEventRecord(s.ev[3], s.st);
  if (e == cudaSuccess) e = cudaEventRecord(s.done, s.st);
  s.busy = true;
  s.used = off;
  const uint64_t r = resident.fetch_add(off) + off;
  uint64_t pk = peak_bytes.load();
  while (r > pk && !peak_bytes.compare_exchange_weak(pk, r)) {}
  batches++;
  if (e != cudaSuccess) { cudaStreamSynchronize(s.st); retire(s, false); return false; }
  return true;
}

// Hand results back to the slot's jobs.
void fpa_server_s::retire(Slot &s, bool ok) {
  const uint32_t *re = (const uint32_t *)(s.h_stage + s.o_re), *rl = (const uint32_t *)(s.h_stage + s.o_rl);
  if (ok) {
    cost_ns[0] += s.pack_ns;
    for (int k = 0; k < 3; k++) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, s.ev[k], s.ev[k + 1]) == cudaSuccess) cost_ns[k + 1] += (uint64_t)(ms * 1e6);
    }
  }
  if (ok && cfg.batching) {
    std::vector<Copy> copies;
    for (size_t q = 0; q < s.jobs.size(); q++) {
      Job *j = s.jobs[q];
      if (!j->copy_out) continue;
      const uint64_t f = s.job_first[q], l0 = s.job_limb0[q];
      copies.push_back({j->r_exps, re + f, (size_t)j->count * 4});
      copies.push_back({j->r_limbs, rl + l0, (size_t)j->count * j->n * 4});
    }
    pool->run(copies);
  }
  const uint64_t t = now();
  for (size_t q = 0; q < s.jobs.size(); q++) {
    Job *j = s.jobs[q];
    if (ok && j->copy_out && !cfg.batching) {    // plain: undo the grouping by operation type
      for (uint32_t p = 0; p < j->count; p++) {
        const uint32_t i = s.perm[p];
        j->r_exps[i] = re[p];
        memcpy(j->r_limbs + (uint64_t)i * j->n, rl + (uint64_t)p * j->n, j->n * 4);
      }
    }
    ops_done += j->count;
    jobs_done++;
    if (!ok) failures++;
    {
      std::lock_guard<std::mutex> lk(mu);
      j->t_done = t;
      j->state = ok ? JOB_DONE : JOB_FAILED;
      if (j->a_src) j->a_src->deps--;
      if (j->b_src) j->b_src->deps--;
    }
  }
  resident -= s.used;
  s.used = 0;
  s.jobs.clear();
  s.busy = false;
  cv_done.notify_all();
}

void fpa_server_s::loop() {
  cudaSetDevice(device);
  for (;;) {
    bool progressed = false;
    for (Slot &s : slots) {
      if (s.busy) {
        cudaError_t q = cudaEventQuery(s.done);
        if (q == cudaSuccess) { retire(s, true); progressed = true; }
        else if (q != cudaErrorNotReady) { retire(s, false); progressed = true; }
      }
    }
    for (Slot &s : slots) {
      if (s.busy) continue;
      std::vector<Job *> batch;
      {
        std::lock_guard<std::mutex> lk(mu);
        uint64_t bytes = 0, ops = 0;
        for (auto it = pending.begin(); it != pending.end();) {
          Job *j = *it;
          // a kept-result operand needs its source launched in an earlier batch (or failed:
          // the job then fails with it)
          auto unready = [](const Job *src) { return src && src->state == JOB_PENDING; };
          auto failed = [](const Job *src) { return src && src->state == JOB_FAILED; };
          if (failed(j->a_src) || failed(j->b_src)) {
            j->state = JOB_FAILED; j->t_done = now(); failures++;
            if (j->a_src) j->a_src->deps--;
            if (j->b_src) j->b_src->deps--;
            it = pending.erase(it);
            cv_done.notify_all();
            continue;
          }
          if (unready(j->a_src) || unready(j->b_src)) { ++it; continue; }
          const uint64_t jb = j->bytes + 4096;
          if (!batch.empty() && (bytes + jb > s.cap || ops + j->count > cfg.max_batch_ops || !cfg.batching)) break;
          batch.push_back(j);
          bytes += jb; ops += j->count;
          it = pending.erase(it);
        }
      }
      if (batch.empty()) break;
      if (!launch(s, batch)) {
        for (Job *j : batch) {
          std::lock_guard<std::mutex> lk(mu);
          if (j->state != JOB_DONE && j->state != JOB_FAILED) { j->state = JOB_FAILED; j->t_done = now(); }
        }
        cv_done.notify_all();
      }
      progressed = true;
      if (!cfg.batching) {                       // plain: one job at a time, to completion
        cudaEventSynchronize(s.done);
        retire(s, cudaEventQuery(s.done) == cudaSuccess);
      }
    }
    if (!progressed) {
      std::unique_lock<std::mutex> lk(mu);
      bool any_busy = false;
      for (Slot &s : slots) any_busy = any_busy || s.busy;
      if (stop && pending.empty() && !any_busy) break;
      if (pending.empty() && !any_busy) cv_work.wait_for(lk, std::chrono::milliseconds(2));
      else {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
  }
}

extern "C" fpa_result fpa_server_create(fpa_server_t *out, const fpa_server_config *cfg) {
  return fpa_server_create_resident(out, cfg, 0);
}

extern "C" fpa_result fpa_server_create_resident(fpa_server_t *out, const fpa_server_config *cfg,
                                                 uint64_t resident_bytes) {
  if (!out || !cfg) return fpa_math_error;
  *out = nullptr;
  int sms;
  if (!gfpa_context(&sms, nullptr)) return fpa_device_error;
  fpa_server_s *srv = new fpa_server_s();
  srv->cfg = *cfg;
  if (srv->cfg.max_inflight < 1) srv->cfg.max_inflight = 1;
  if (!srv->cfg.batching) srv->cfg.max_inflight = 1;
  if (srv->cfg.max_batch_ops == 0) srv->cfg.max_batch_ops = 1u << 20;
  srv->sms = sms;
  if (cudaGetDevice(&srv->device) != cudaSuccess) { delete srv; return fpa_device_error; }
  srv->t0 = Clock::now();
  const size_t cap = align256((size_t)(srv->cfg.hbm_budget_bytes / srv->cfg.max_inflight));
  srv->slots.resize(srv->cfg.max_inflight);
  bool ok = cap >= 65536;
  for (Slot &s : srv->slots) {
    if (!ok) break;
    s.cap = cap;
    ok = cudaMalloc(&s.d_arena, cap) == cudaSuccess && cudaMallocHost(&s.h_stage, cap) == cudaSuccess &&
         cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&s.side[0], cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&s.side[1], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&s.join[0], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&s.join[1], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&s.kept, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < 4 && ok; k++) ok = cudaEventCreate(&s.ev[k]) == cudaSuccess;
  }
  // the one-thread class's slabs come out of each slot's arena: 4 one-warp CTAs per SM, when
  // that leaves at least three quarters of the arena for operands
  int per = 0;
  if (ok && srv->cfg.batching && gfpa_batch_thread_prepare(&per) == cudaSuccess && per > 0) {
    const int grid = std::min(per, 4) * sms;
    const size_t slab = align256(gfpa_batch_thread_slab_bytes(grid));
    if (slab * 4 <= cap) {
      srv->thread_grid = grid;
      for (Slot &s : srv->slots) {
        s.cap = cap - slab;
        s.thread_slabs = (uint32_t *)(s.d_arena + s.cap);
      }
    }
  }
  if (ok && resident_bytes) {
    srv->res_cap = align256(resident_bytes);
    ok = cudaMalloc(&srv->d_res, srv->res_cap) == cudaSuccess;
    if (ok) srv->res_store.reset(srv->res_cap);
  }
  if (!ok) { fpa_server_destroy(srv); return fpa_device_error; }
  const unsigned hw = std::thread::hardware_concurrency();
  srv->pool.reset(new CopyPool((int)std::min(15u, hw > 2 ? hw - 1 : 1u)));
  srv->thread = std::thread([srv] { srv->loop(); });
  *out = srv;
  return fpa_success;
}

extern "C" int64_t fpa_server_submit(fpa_server_t srv, uint32_t precision, uint32_t count, const uint8_t *ops,
                                     const uint8_t *modes, const uint32_t *a_exps, const uint32_t *a_limbs,
                                     const uint32_t *b_exps, const uint32_t *b_limbs, uint32_t *r_exps,
                                     uint32_t *r_limbs) {
  return fpa_server_submit_ex(srv, precision, count, ops, modes, a_exps, a_limbs, b_exps, b_limbs, r_exps, r_limbs,
                              nullptr);
}

extern "C" int64_t fpa_server_submit_ex(fpa_server_t srv, uint32_t precision, uint32_t count, const uint8_t *ops,
                                        const uint8_t *modes, const uint32_t *a_exps, const uint32_t *a_limbs,
                                        const uint32_t *b_exps, const uint32_t *b_limbs, uint32_t *r_exps,
                                        uint32_t *r_limbs, const fpa_server_job_opts *opts) {
  fpa_server_job_opts o = {0, 0, 0, 1};
  if (opts) o = *opts;
  const bool a_dev = o.a_from > 0, b_dev = o.b_from > 0;
  if (!srv || !ops || (!a_dev && (!a_exps || !a_limbs)) || (o.copy_out && (!r_exps || !r_limbs)))
    return -(int64_t)fpa_math_error;
  if ((a_dev || b_dev || o.keep) && !srv->cfg.batching) return -(int64_t)fpa_math_error;
  if (precision < 32 || precision > 32u * GFPA_MAX_LIMBS || precision % 32) return -(int64_t)fpa_invalid_precisions;
  if (count == 0) return -(int64_t)fpa_invalid_counts;
  auto j = std::make_unique<Job>();
  j->n = precision / 32;
  j->count = count;
  j->ops.assign(ops, ops + count);
  j->modes.assign(count, (uint8_t)fpa_round_ties_to_even);
  if (modes) j->modes.assign(modes, modes + count);
  for (uint32_t i = 0; i < count; i++) {
    if (j->ops[i] > 4 || j->modes[i] > 4) return -(int64_t)fpa_math_error;
    if (j->ops[i] != 4 && !b_dev && (!b_exps || !b_limbs)) return -(int64_t)fpa_math_error;
  }
  j->a_exps = a_exps; j->a_limbs = a_limbs; j->b_exps = b_exps; j->b_limbs = b_limbs;
  j->r_exps = r_exps; j->r_limbs = r_limbs;
  j->keep = o.keep != 0; j->copy_out = o.copy_out != 0;
  j->bytes = (uint64_t)count * op_bytes(j->n) + 10 * 256;
  if (j->bytes + 4096 > srv->slots[0].cap) return -(int64_t)fpa_invalid_counts;   // larger than a slot's budget
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->stop) return -(int64_t)fpa_device_error;
  // kept-result operands: the source must be a kept job of the same shape
  for (int which = 0; which < 2; which++) {
    const int64_t from = which == 0 ? o.a_from : o.b_from;
    if (from <= 0) continue;
    auto it = srv->jobs.find(from);
    if (it == srv->jobs.end()) return -(int64_t)fpa_math_error;
    Job *src = it->second.get();
    if (!src->keep || src->n != j->n || src->count != count || src->state == JOB_FAILED) return -(int64_t)fpa_math_error;
    (which == 0 ? j->a_src : j->b_src) = src;
  }
  if (j->keep) {                                  // a block of the resident store: exponents, then limbs
    j->res_bytes = align256((size_t)count * 4) + align256((size_t)count * j->n * 4);
    j->res_off = srv->res_cap ? srv->res_store.alloc(j->res_bytes) : UINT64_MAX;
    if (j->res_off == UINT64_MAX) return -(int64_t)fpa_invalid_counts;       // the resident store is full
  }
  if (j->a_src) j->a_src->deps++;
  if (j->b_src) j->b_src->deps++;
  j->id = srv->next_id++;
  j->t_submit = srv->now();
  const int64_t id = j->id;
  srv->pending.push_back(j.get());
  srv->jobs.emplace(id, std::move(j));
  srv->cv_work.notify_one();
  return id;
}

extern "C" fpa_result fpa_server_wait(fpa_server_t srv, int64_t job, int64_t timeout_ms) {
  if (!srv) return fpa_math_error;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(job);
  if (it == srv->jobs.end()) return fpa_math_error;
  Job *j = it->second.get();
  auto pred = [j] { return j->state == JOB_DONE || j->state == JOB_FAILED; };
  if (timeout_ms < 0) srv->cv_done.wait(lk, pred);
  else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return fpa_math_error;
  return j->state == JOB_DONE ? fpa_success : fpa_device_error;
}

extern "C" fpa_result fpa_server_job_times(fpa_server_t srv, int64_t job, uint64_t *t_submit, uint64_t *t_admit,
                                           uint64_t *t_done) {
  if (!srv) return fpa_math_error;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(job);
  if (it == srv->jobs.end()) return fpa_math_error;
  if (t_submit) *t_submit = it->second->t_submit;
  if (t_admit) *t_admit = it->second->t_admit;
  if (t_done) *t_done = it->second->t_done;
  return fpa_success;
}

extern "C" fpa_result fpa_server_release(fpa_server_t srv, int64_t job) {
  if (!srv) return fpa_math_error;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(job);
  if (it == srv->jobs.end()) return fpa_math_error;
  Job *j = it->second.get();
  if (j->state != JOB_DONE && j->state != JOB_FAILED) return fpa_math_error;
  if (j->deps > 0) return fpa_math_error;         // pending jobs still read its kept result
  if (j->keep) srv->res_store.release(j->res_off, j->res_bytes);
  srv->jobs.erase(it);
  return fpa_success;
}

extern "C" fpa_result fpa_server_read(fpa_server_t srv, int64_t job, uint32_t *r_exps, uint32_t *r_limbs) {
  if (!srv || !r_exps || !r_limbs) return fpa_math_error;
  fpa_result r = fpa_server_wait(srv, job, -1);
  if (r != fpa_success) return r;
  uint64_t off = 0, count = 0, n = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job);
    if (it == srv->jobs.end() || !it->second->keep) return fpa_math_error;
    off = it->second->res_off; count = it->second->count; n = it->second->n;
  }
  if (cudaSetDevice(srv->device) != cudaSuccess) return fpa_device_error;
  const uint8_t *R = srv->d_res + off;
  if (cudaMemcpy(r_exps, R, count * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(r_limbs, R + align256(count * 4), count * n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fpa_device_error;
  return fpa_success;
}

extern "C" fpa_result fpa_server_costs(fpa_server_t srv, uint64_t *ns) {
  if (!srv || !ns) return fpa_math_error;
  for (int k = 0; k < 4; k++) ns[k] = srv->cost_ns[k];
  return fpa_success;
}

extern "C" fpa_result fpa_server_stats(fpa_server_t srv, uint64_t *stats) {
  if (!srv || !stats) return fpa_math_error;
  stats[0] = srv->jobs_done; stats[1] = srv->ops_done; stats[2] = srv->batches;
  stats[3] = srv->peak_bytes; stats[4] = srv->failures;
  stats[5] = (uint64_t)srv->slots.size() * (srv->slots.empty() ? 0 : srv->slots[0].cap);
  return fpa_success;
}

extern "C" fpa_result fpa_server_destroy(fpa_server_t srv) {
  if (!srv) return fpa_success;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  if (srv->thread.joinable()) srv->thread.join();
  for (Slot &s : srv->slots) {
    if (s.st) cudaStreamSynchronize(s.st);
    if (s.d_arena) cudaFree(s.d_arena);
    if (s.h_stage) cudaFreeHost(s.h_stage);
    for (int c = 0; c < 2; c++) {
      if (s.side[c]) cudaStreamDestroy(s.side[c]);
      if (s.join[c]) cudaEventDestroy(s.join[c]);
    }
    if (s.st) cudaStreamDestroy(s.st);
    if (s.fork) cudaEventDestroy(s.fork);
    if (s.done) cudaEventDestroy(s.done);
    if (s.kept) cudaEventDestroy(s.kept);
    for (int k = 0; k < 4; k++)
      if (s.ev[k]) cudaEventDestroy(s.ev[k]);
  }
  if (srv->d_res) cudaFree(srv->d_res);
  delete srv;
  return fpa_success;
}
