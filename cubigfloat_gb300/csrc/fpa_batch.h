// fpa_batch.h -- internal interface of the batched and served forms.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "../../include/fpa_gb300.h"

// Per-process device context (SM count, device error word); false on CUDA failure.
bool gfpa_context(int *sms, uint32_t **err);
// Lane-group configuration for operation `op` on numbers of `n` limbs (autotuned table,
// else the smallest default configuration that holds n).
int gfpa_cfg_for_op(int op, uint32_t n);

// One task = `count` operations of one (configuration, operation) pair, taken from the
// sorted order array starting at `first`.
struct BatchTask {
  uint16_t key;      // cfg * 5 + op
  uint16_t pad;
  uint32_t first;
  uint32_t count;
};

struct BatchArgs {
  const fpa_batch_desc *descs;
  const uint32_t *order;
  const BatchTask *tasks;
  uint32_t ntasks;
  uint32_t *counter;          // next task of this class (device)
  uint32_t warp_words;        // shared-memory words per warp
  uint32_t *r_exps, *r_limbs;
  const uint32_t *a_exps, *a_limbs, *b_exps, *b_limbs;
  uint32_t *err;
};

// Tile width K of configuration cfg (the table in fpa_launch.h, usable in device code).
__host__ __device__ constexpr int gfpa_cfg_tile(int cfg) {
  return (cfg == 6 || cfg == 8 || cfg == 9) ? 16 : ((cfg == 5 || cfg == 7 || cfg == 13 || cfg == 14) ? 8 : (cfg <= 1 ? 2 : 4));
}

// Register class of (configuration, operation): 0 = tiles <= 4 limbs for add/sub/mul,
// 1 = 8-limb tiles and div/sqrt with tiles <= 8 limbs, 2 = 16-limb tiles.
__host__ __device__ constexpr int gfpa_class_of(int cfg, int op) {
  return gfpa_cfg_tile(cfg) >= 16 ? 2 : ((gfpa_cfg_tile(cfg) == 8 || op == 3 || op == 4) ? 1 : 0);
}

// threads per CTA of each class kernel
static const int gfpa_class_threads[3] = {256, 128, 128};

// The one-thread class (fpa_batch_thread.cu): the batch fields above (tasks of up to 32
// operations of one operation and limb count, `counter` its task counter) plus this batch's
// per-CTA slabs and the list of operations its first pass defers to the exact pass.
struct ThreadBatchArgs {
  BatchArgs b;
  uint32_t *slabs;
  uint32_t *hard_count, *hard_idx;
};
// Device scratch of the one-thread class, owned by the batch.
struct ThreadScratch {
  uint32_t *slabs = nullptr, *hard_count = nullptr, *hard_idx = nullptr;
};
size_t gfpa_batch_thread_smem();
size_t gfpa_batch_thread_slab_bytes(int grid);
cudaError_t gfpa_batch_thread_prepare(int *blocks_per_sm);
cudaError_t gfpa_batch_thread_launch(const ThreadBatchArgs *a, int grid, cudaStream_t st);
// the class index of the one-thread class
constexpr int GFPA_THREAD_CLASS = 3;

// Host-side plan of a batch: descriptor order, tasks (concatenated class by class) and the
// launch shape of each class kernel (classes 0-2: lane groups; 3: one thread per operation).
#include <vector>
struct BatchPlan {
  std::vector<uint32_t> order;
  std::vector<BatchTask> tasks;
  uint32_t ntasks[4] = {0, 0, 0, 0}, task_base[4] = {0, 0, 0, 0}, warp_words[4] = {0, 0, 0, 0};
  size_t smem[4] = {0, 0, 0, 0};
  int grid[4] = {0, 0, 0, 0};
  uint64_t thread_ops = 0;    // operations of the one-thread class
};
// Plan `count` descriptors; fpa_success or the validation error.  With `one_thread`, mul,
// div and sqrt of 8 to 128 limbs whose tuned configuration is a one-thread one (18, 19) go to
// the one-thread class, which needs a ThreadScratch at enqueue with slabs for its grid (at
// most `thread_grid_cap` CTAs when that is nonzero).
fpa_result gfpa_batch_plan(const fpa_batch_desc *descs, uint64_t count, int sms, BatchPlan &plan,
                           bool one_thread = false, int thread_grid_cap = 0);
// Enqueue one run of a plan whose descriptors, order and tasks are already in device memory.
// Classes 0 and 3 run on `st`, classes 1 and 2 on `side[0]`, `side[1]` (forked from and
// joined back into `st` with the given events).  `ts`: the one-thread class's scratch (only
// read when the plan has that class).
cudaError_t gfpa_batch_enqueue(const BatchPlan &plan, const fpa_batch_desc *d_descs, const uint32_t *d_order,
                               const BatchTask *d_tasks, uint32_t *d_counters, uint32_t *r_exps, uint32_t *r_limbs,
                               const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                               const uint32_t *b_limbs, cudaStream_t st, const cudaStream_t side[2],
                               cudaEvent_t fork, const cudaEvent_t join[2], const ThreadScratch *ts = nullptr);

// Planner helpers shared with other entry points of the batched form.
int gfpa_batch_warp_words(int cfg, int op);          // shared-memory words per warp
int gfpa_batch_cfg_for(int op, uint32_t n);           // configuration a batch task runs with
double gfpa_batch_op_weight(int op, int n);           // relative cost of one operation
cudaError_t gfpa_batch_prepare_class(int c, size_t smem, int *blocks_per_sm);
cudaError_t gfpa_batch_launch_class(int c, const BatchArgs *a, int grid, size_t smem, cudaStream_t st);

// Class kernels (fpa_batch_kernels.cu, one object per class).
extern "C" {
cudaError_t gfpa_batch_prepare0(size_t smem, int *blocks_per_sm);
cudaError_t gfpa_batch_prepare1(size_t smem, int *blocks_per_sm);
cudaError_t gfpa_batch_prepare2(size_t smem, int *blocks_per_sm);
cudaError_t gfpa_batch_launch0(const BatchArgs *a, int grid, size_t smem, cudaStream_t st);
cudaError_t gfpa_batch_launch1(const BatchArgs *a, int grid, size_t smem, cudaStream_t st);
cudaError_t gfpa_batch_launch2(const BatchArgs *a, int grid, size_t smem, cudaStream_t st);
}
