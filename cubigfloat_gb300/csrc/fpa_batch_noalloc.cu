// fpa_batch_noalloc.cu -- a batched run that allocates no memory.
//
// fpa_batch_run_noalloc is for callers that must not allocate GPU memory at the point where
// they compute: a serving loop whose latency budget cannot absorb cudaMalloc / cudaFree
// (which may synchronize the device and wait on unrelated work), and host applications
// that give all device memory to their own allocator up front and treat any later
// allocation by a library as a failure.  They pass inputs and outputs in memory they
// already own; the batch's own working memory (descriptors, schedule, task counters and the
// error word) lives in one fixed array in device memory, sized for FPA_NOALLOC_MAX_OPS
// operations.  Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
//
// The array is a file-scope __device__ variable, so every GPU that loads the library keeps
// it (about 200 KB) until the process exits.  Host code cannot use the variable's name as a
// device address; the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current, and later calls reuse it, so that
// first call should come before any stream capture, and a device reset (which would give the
// variable a new address) is not supported.  Every call shares the array and it keeps the
// last call's contents; the task counters and the error word are cleared by each call
// before its kernels run, and two calls whose work overlaps on the GPU race on the array,
// so calls must be ordered (one stream, or an event between streams).  Planning uses fixed
// host arrays under a lock and the class kernels run one after the other on the caller's
// stream.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include <string.h>
#include "../../include/fpa_gb300.h"
#include "fpa_launch.h"
#include "fpa_batch.h"

namespace {

constexpr uint32_t kMaxOps = FPA_NOALLOC_MAX_OPS;
constexpr uint32_t kMaxTasks = kMaxOps;            // every task holds at least one operation
constexpr size_t kOffDescs = 0;
constexpr size_t kOffOrder = kOffDescs + (size_t)kMaxOps * sizeof(fpa_batch_desc);
constexpr size_t kOffTasks = kOffOrder + (size_t)kMaxOps * 4;
constexpr size_t kOffCounters = (kOffTasks + (size_t)kMaxTasks * sizeof(BatchTask) + 255) & ~(size_t)255;
constexpr size_t kOffErr = kOffCounters + 16;
constexpr size_t kScratchBytes = (kOffErr + 16 + 255) & ~(size_t)255;

// Host planning state (guarded by g_mu).
std::mutex g_mu;
uint32_t h_order[kMaxOps];
uint16_t h_key[kMaxOps];
uint8_t h_cls[kMaxOps];
BatchTask h_tasks[kMaxTasks], h_sorted[kMaxTasks];
double h_cost[kMaxTasks];
uint32_t h_tidx[kMaxTasks];
void *g_addr[64];                                   // scratch address per device

}  // namespace

// The working memory itself.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

extern "C" fpa_result fpa_batch_run_noalloc(const fpa_batch_desc *descs, uint32_t count, uint32_t *r_exps,
                                            uint32_t *r_limbs, const uint32_t *a_exps, const uint32_t *a_limbs,
                                            const uint32_t *b_exps, const uint32_t *b_limbs, void *stream) {
  if (count > kMaxOps) return fpa_invalid_counts;   // larger than the fixed working memory
  if (count == 0) return fpa_success;
  if (!descs) return fpa_math_error;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fpa_device_error;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fpa_device_error;
  if (!g_addr[dev]) {                               // once per device, with that device current
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return fpa_device_error;
    g_addr[dev] = p;
  }
  unsigned char *scratch = (unsigned char *)g_addr[dev];
  // ---- plan: sort by (class, configuration, operation, limbs descending, index)
  for (uint32_t i = 0; i < count; i++) {
    const fpa_batch_desc &d = descs[i];
    if (d.op > 4 || d.mode > 4) return fpa_math_error;
    if (d.limbs == 0 || d.limbs > GFPA_MAX_LIMBS) return fpa_invalid_precisions;
    const int cfg = gfpa_batch_cfg_for(d.op, d.limbs);
    if (cfg < 0) return fpa_invalid_precisions;
    h_key[i] = (uint16_t)(cfg * 5 + d.op);
    h_cls[i] = (uint8_t)gfpa_class_of(cfg, d.op);
    h_order[i] = i;
  }
  std::sort(h_order, h_order + count, [&](uint32_t x, uint32_t y) {
    if (h_cls[x] != h_cls[y]) return h_cls[x] < h_cls[y];
    if (h_key[x] != h_key[y]) return h_key[x] < h_key[y];
    if (descs[x].limbs != descs[y].limbs) return descs[x].limbs > descs[y].limbs;
    return x < y;
  });
  uint32_t nt = 0, ntasks[3] = {0, 0, 0}, base[3] = {0, 0, 0}, ww[3] = {0, 0, 0};
  for (int c = 0; c < 3; c++) {
    base[c] = nt;
    uint32_t i = 0;
    while (i < count && h_cls[h_order[i]] != c) i++;
    while (i < count && h_cls[h_order[i]] == c) {
      uint32_t j = i;
      const uint16_t k = h_key[h_order[i]];
      while (j < count && h_key[h_order[j]] == k) j++;
      const int cfg = k / 5, op = k % 5;
      const int groups = (gfpa_class_threads[c] / 32) * (32 / gfpa_cfg_G[cfg]);
      const uint32_t chunk = (uint32_t)groups * 2;
      ww[c] = std::max<uint32_t>(ww[c], (uint32_t)gfpa_batch_warp_words(cfg, op));
      for (uint32_t s = i; s < j; s += chunk) {
        if (nt >= kMaxTasks) return fpa_invalid_counts;
        BatchTask &t = h_tasks[nt];
        t.key = k; t.pad = 0; t.first = s; t.count = std::min(chunk, j - s);
        double w = 0;
        for (uint32_t q = s; q < s + t.count; q++) w += gfpa_batch_op_weight(op, descs[h_order[q]].limbs);
        h_cost[nt] = w / groups;
        h_tidx[nt] = nt;
        nt++;
      }
      i = j;
    }
    ntasks[c] = nt - base[c];
    std::sort(h_tidx + base[c], h_tidx + nt, [&](uint32_t x, uint32_t y) {
      return h_cost[x] != h_cost[y] ? h_cost[x] > h_cost[y] : x < y;
    });
  }
  for (uint32_t q = 0; q < nt; q++) h_sorted[q] = h_tasks[h_tidx[q]];
  // ---- copy the plan into the fixed array and clear what must start at zero
  cudaError_t e = cudaMemcpyAsync(scratch + kOffDescs, descs, (size_t)count * sizeof(fpa_batch_desc),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(scratch + kOffOrder, h_order, (size_t)count * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kOffTasks, h_sorted, (size_t)nt * sizeof(BatchTask), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kOffCounters, 0, 32, st);   // counters + error word
  if (e != cudaSuccess) return fpa_device_error;
  // ---- class kernels, one after the other on the caller's stream
  BatchArgs A;
  A.descs = (const fpa_batch_desc *)(scratch + kOffDescs);
  A.order = (const uint32_t *)(scratch + kOffOrder);
  A.err = (uint32_t *)(scratch + kOffErr);
  A.r_exps = r_exps; A.r_limbs = r_limbs; A.a_exps = a_exps; A.a_limbs = a_limbs;
  A.b_exps = b_exps ? b_exps : a_exps; A.b_limbs = b_limbs ? b_limbs : a_limbs;
  for (int c = 0; c < 3; c++) {
    if (!ntasks[c]) continue;
    const size_t smem = (size_t)(gfpa_class_threads[c] / 32) * ww[c] * 4;
    if (smem > 227 * 1024) return fpa_device_error;
    int per = 0;
    if (gfpa_batch_prepare_class(c, smem, &per) != cudaSuccess) return fpa_device_error;
    if (per < 1) per = 1;
    const int grid = (int)std::min<uint64_t>((uint64_t)per * sms, ntasks[c]);
    A.tasks = (const BatchTask *)(scratch + kOffTasks) + base[c];
    A.ntasks = ntasks[c];
    A.counter = (uint32_t *)(scratch + kOffCounters) + c;
    A.warp_words = ww[c];
    if (gfpa_batch_launch_class(c, &A, grid, smem, st) != cudaSuccess) return fpa_device_error;
  }
  return fpa_success;
}

extern "C" uint32_t fpa_batch_noalloc_errors(void *stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || !g_addr[dev]) return 0;
  uint32_t v = 0;
  if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return 0xFFFFFFFFu;
  if (cudaMemcpy(&v, (unsigned char *)g_addr[dev] + kOffErr, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return 0xFFFFFFFFu;
  return v;
}
