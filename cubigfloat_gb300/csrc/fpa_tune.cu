// fpa_tune.cu -- the configuration autotuner and the tuning table file.
//
// For one (operation, limb count) the tuner fills a device batch with seeded random
// operands, times every lane-group configuration that can hold the limb count (and is
// not more than four times too large) with CUDA events, and returns the fastest.  The
// table maps (operation, limbs) to a configuration; it is stored as text lines
// "op limbs cfg" and loaded at library start-up from tuned_configs.txt beside the package
// (or from the file named by FPA_GB300_TUNING), and by fpa_gb300_load_tuning.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include "../../include/fpa_gb300.h"
#include "fpa_launch.h"
#include "fpa_batch.h"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// random normalized operands: exponents in [-64, 64], positive when `positive`
__global__ void k_fill(uint32_t *exps, uint32_t *limbs, uint32_t n, uint64_t count, uint64_t seed, int positive) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count * n; i += stride) {
    uint32_t v = (uint32_t)mix64(seed ^ (i * 0xD6E8FEB86659FD93ull));
    if (i % n == n - 1) v |= 0x80000000u;
    limbs[i] = v;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t h = mix64(seed * 31 + i);
    const int e = (int)(h % 129) - 64;
    exps[i] = (uint32_t)(2 * ((int64_t)0x3FFFFFF3 + e)) + (positive ? 0u : (uint32_t)((h >> 40) & 1));
  }
}

}  // namespace

extern "C" fpa_result fpa_gb300_autotune(fpa_op op, uint32_t limbs, uint32_t sample, int *best_cfg,
                                         double *ops_per_s) {
  if ((int)op < 0 || (int)op > 4 || limbs == 0 || limbs > GFPA_MAX_LIMBS) return fpa_math_error;
  if (sample == 0) sample = 1u << 16;
  int sms;
  uint32_t *err;
  if (!gfpa_context(&sms, &err)) return fpa_device_error;
  const size_t nl = (size_t)sample * limbs;
  uint32_t *buf = nullptr;
  if (cudaMalloc(&buf, (nl * 3 + (size_t)sample * 3) * 4) != cudaSuccess) return fpa_device_error;
  uint32_t *al = buf, *bl = al + nl, *rl = bl + nl, *ae = rl + nl, *be = ae + sample, *re = be + sample;
  k_fill<<<sms * 4, 256>>>(ae, al, limbs, sample, 1234567u + limbs, op == fpa_op_sqrt);
  k_fill<<<sms * 4, 256>>>(be, bl, limbs, sample, 7654321u + limbs, 0);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  int best = -1;
  double best_rate = 0.0;
  const uint32_t need = limbs < 4 ? 4 : limbs;
  for (int c = 0; c < GFPA_NUM_CFGS; c++) {
    const uint32_t cap = (uint32_t)gfpa_cfg_capacity(c);
    if (cap < need || cap > 4 * (need < 8 ? 8 : need) || !gfpa_cfg_supports(c, (int)op)) continue;
    ElementwiseArgs a;
    a.count = sample; a.n = limbs; a.mode = fpa_round_ties_to_even;
    a.r_exps = re; a.r_limbs = rl; a.a_exps = ae; a.a_limbs = al; a.b_exps = be; a.b_limbs = bl; a.err = err;
    if (gfpa_launch(c, (int)op, &a, 0, sms) != cudaSuccess) continue;     // warm-up (and attribute set-up)
    cudaEventRecord(e0);
    for (int rep = 0; rep < 4; rep++) gfpa_launch(c, (int)op, &a, 0, sms);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double rate = ms > 0.f ? 4.0 * sample / (ms * 1e-3) : 0.0;
    if (rate > best_rate) { best_rate = rate; best = c; }
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  if (e != cudaSuccess || best < 0) return fpa_device_error;
  if (best_cfg) *best_cfg = best;
  if (ops_per_s) *ops_per_s = best_rate;
  return fpa_success;
}

extern "C" fpa_result fpa_gb300_load_tuning(const char *path) {
  if (!path) return fpa_math_error;
  FILE *f = fopen(path, "r");
  if (!f) return fpa_math_error;
  char line[256];
  fpa_result res = fpa_success;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    int op, cfg;
    unsigned lo, hi;
    const int got = sscanf(line, "%d %u %u %d", &op, &lo, &hi, &cfg);
    if (got != 4) { res = fpa_math_error; continue; }
    for (unsigned n = lo; n <= hi && n <= GFPA_MAX_LIMBS; n++)
      if (fpa_gb300_set_op_config((fpa_op)op, n, cfg) != fpa_success) res = fpa_math_error;
  }
  fclose(f);
  return res;
}

// Load the committed table when the library is loaded: FPA_GB300_TUNING, else
// <directory of this library>/../tuned_configs.txt.
namespace {
struct AutoLoad {
  AutoLoad() {
    const char *env = getenv("FPA_GB300_TUNING");
    if (env && *env) { fpa_gb300_load_tuning(env); return; }
    Dl_info info;
    if (dladdr((void *)&fpa_gb300_load_tuning, &info) && info.dli_fname) {
      std::string p(info.dli_fname);
      const size_t slash = p.rfind('/');
      if (slash != std::string::npos) {
        p = p.substr(0, slash) + "/../tuned_configs.txt";
        FILE *f = fopen(p.c_str(), "r");
        if (f) { fclose(f); fpa_gb300_load_tuning(p.c_str()); }
      }
    }
  }
};
AutoLoad g_autoload;
}  // namespace
