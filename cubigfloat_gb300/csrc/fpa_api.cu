// fpa_api.cu -- the C-ABI layer: fpa.h (drop-in) and fpa_gb300.h (additions).
//
// Host side of each entry point mirrors the reference's fpa_management.h / fpa_dispatch.h:
// same argument checks in the same order, same result codes, operations asynchronous on
// the legacy default stream.  Differences: device numbers are stored in natural limb
// order (instance-major, little-endian limbs), so copies are plain cudaMemcpy calls with
// no host-side transpose; CUDA errors are returned as fpa_device_error.
#include <cuda_runtime.h>
#include <atomic>
#include <mutex>
#include <string.h>
#include "../../include/fpa.h"
#include "../../include/fpa_gb300.h"
#include "fpa_launch.h"
#include "fpa_misc.h"
#include "fpa_batch.h"
#include "fpa_devctx.h"

namespace {

struct State {
  std::mutex mu;
  // per operation and limb count: configuration + 1, 0 = default.  Zero-initialised (no
  // constructor), so the table is ready before any static initialiser of another file runs.
  int8_t cfg_override[5][GFPA_MAX_LIMBS + 1];
};
State g_state;

// Per-device context: the SM count that sizes the grids and the device word the kernels
// OR their error bits into, made on the first call that finds the device current.
struct DevCtx {
  int sms;
  uint32_t *err;
  cudaMemPool_t pool;      // stream-ordered scratch of the one-thread div/sqrt kernels
};
PerDevice<DevCtx> g_dev;

bool devctx(DevCtx &c);
bool ctx(int &sms, uint32_t *&err);

}  // namespace

bool gfpa_scratch_pool(cudaMemPool_t *pool) {
  DevCtx c{};
  if (!devctx(c)) return false;
  *pool = c.pool;
  return true;
}

bool gfpa_context(int *sms, uint32_t **err) {
  int s; uint32_t *e;
  if (!ctx(s, e)) return false;
  if (sms) *sms = s;
  if (err) *err = e;
  return true;
}

static bool cfg_fits(int c, uint32_t n) {
  const uint32_t cap = (uint32_t)gfpa_cfg_capacity(c);
  return cap >= n && cap >= 4;
}

int gfpa_cfg_for_op(int op, uint32_t n) {
  if (op < 0 || op > 4 || n == 0 || n > GFPA_MAX_LIMBS) return -1;
  const int c = g_state.cfg_override[op][n] - 1;
  if (c >= 0 && cfg_fits(c, n) && gfpa_cfg_supports(c, op)) return c;
  return gfpa_default_cfg(n < 4 ? 4 : n);
}

namespace {

// the current device's context (made with that device current on first use)
bool devctx(DevCtx &c) {
  return g_dev.get([](int &dev) { return cudaGetDevice(&dev) == cudaSuccess; },
                   [](int dev, DevCtx &v) {
                     int n;
                     if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
                     uint32_t *e;
                     if (cudaMalloc(&e, sizeof(uint32_t)) != cudaSuccess) return false;
                     if (cudaMemset(e, 0, sizeof(uint32_t)) != cudaSuccess) { cudaFree(e); return false; }
                     // the library's own pool, which keeps what it reserved (no release back
                     // to the driver at synchronizations)
                     cudaMemPoolProps props = {};
                     props.allocType = cudaMemAllocationTypePinned;
                     props.location.type = cudaMemLocationTypeDevice;
                     props.location.id = dev;
                     cudaMemPool_t pool;
                     if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) { cudaFree(e); return false; }
                     uint64_t keep = ~0ull;
                     cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
                     v.sms = n; v.err = e; v.pool = pool;
                     return true;
                   },
                   c);
}

bool ctx(int &sms, uint32_t *&err) {
  DevCtx c{};
  if (!devctx(c)) return false;
  sms = c.sms; err = c.err;
  return true;
}

bool valid_precision(uint32_t precision) {
  return precision >= 32 && precision <= 32u * GFPA_MAX_LIMBS && precision % 32 == 0;
}


// mul: Karatsuba split from this many limbs (0xFFFFFFFF = never)
static std::atomic<uint32_t> g_kara_min{GFPA_KARATSUBA_DEFAULT};

fpa_result launch_elementwise(int op, uint32_t precision, uint64_t count, int mode, uint32_t *r_exps, uint32_t *r_limbs,
                              const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                              const uint32_t *b_limbs, cudaStream_t stream) {
  if (!valid_precision(precision)) return fpa_invalid_precisions;
  if (mode < 0 || mode > 4 || op < 0 || op > 4) return fpa_math_error;
  if (count == 0) return fpa_success;
  int sms; uint32_t *err;
  if (!ctx(sms, err)) return fpa_device_error;
  ElementwiseArgs args;
  args.count = count; args.n = precision / 32; args.mode = mode;
  args.r_exps = r_exps; args.r_limbs = r_limbs;
  args.a_exps = a_exps; args.a_limbs = a_limbs;
  args.b_exps = (op == 4) ? a_exps : b_exps; args.b_limbs = (op == 4) ? a_limbs : b_limbs;
  args.err = err;
  if (op == 2) args.kara_min = g_kara_min.load(std::memory_order_relaxed);
  int cfg = gfpa_cfg_for_op(op, args.n);
  if (cfg < 0) return fpa_invalid_precisions;
  return gfpa_launch(cfg, op, &args, stream, sms) == cudaSuccess ? fpa_success : fpa_device_error;
}

// fpa_dispatch.h:175-183: counts first, then precisions
fpa_result binary_op(int op, fpa_ptr r, fpa_ptr a, fpa_ptr b, fpa_rounding_mode mode, cudaStream_t stream) {
  uint32_t count = r->count, precision = r->precision;
  if (count != a->count || count != b->count) return fpa_invalid_counts;
  if (precision != a->precision || precision != b->precision) return fpa_invalid_precisions;
  return launch_elementwise(op, precision, count, (int)mode, r->gpu_exps, r->gpu_limbs, a->gpu_exps, a->gpu_limbs,
                            b->gpu_exps, b->gpu_limbs, stream);
}

// fpa_dispatch.h:375-383
fpa_result unary_op(int op, fpa_ptr r, fpa_ptr x, fpa_rounding_mode mode, cudaStream_t stream) {
  uint32_t count = r->count, precision = r->precision;
  if (count != x->count) return fpa_invalid_counts;
  if (precision != x->precision) return fpa_invalid_precisions;
  return launch_elementwise(op, precision, count, (int)mode, r->gpu_exps, r->gpu_limbs, x->gpu_exps, x->gpu_limbs,
                            nullptr, nullptr, stream);
}

fpa_result dev(cudaError_t e) { return e == cudaSuccess ? fpa_success : fpa_device_error; }

// host values -> temporary device buffer (fpa_dispatch.h:8-26 pattern)
template <class F>
fpa_result with_device_values(const void *host, size_t bytes, F body) {
  void *d = nullptr;
  if (bytes == 0) return body(nullptr);
  if (cudaMalloc(&d, bytes) != cudaSuccess) return fpa_device_error;
  fpa_result res = fpa_device_error;
  if (cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice) == cudaSuccess) res = body(d);
  if (cudaDeviceSynchronize() != cudaSuccess) res = fpa_device_error;   // kernel reads d before it is freed
  cudaFree(d);
  return res;
}

}  // namespace

extern "C" {

// fpa_management.h:1-9
fpa_result fpa_init(fpa_t fpa, uint32_t count, uint32_t precision) {
  if (!valid_precision(precision)) return fpa_invalid_precisions;
  fpa->count = count;
  fpa->precision = precision;
  fpa->gpu_exps = nullptr;
  fpa->gpu_limbs = nullptr;
  size_t ne = (size_t)(count ? count : 1) * 4, nl = (size_t)(count ? count : 1) * (precision / 8);
  if (cudaMalloc(&fpa->gpu_exps, ne) != cudaSuccess) return fpa_device_error;
  if (cudaMalloc(&fpa->gpu_limbs, nl) != cudaSuccess) {
    cudaFree(fpa->gpu_exps); fpa->gpu_exps = nullptr;
    return fpa_device_error;
  }
  return fpa_success;
}

// fpa_management.h:11-15
fpa_result fpa_clear(fpa_t fpa) {
  cudaError_t e1 = cudaFree(fpa->gpu_exps), e2 = cudaFree(fpa->gpu_limbs);
  fpa->gpu_exps = nullptr; fpa->gpu_limbs = nullptr;
  return (e1 == cudaSuccess && e2 == cudaSuccess) ? fpa_success : fpa_device_error;
}

// fpa_management.h:17-31 (no transpose: the device layout equals the host layout)
fpa_result fpa_copy_array_to_device(fpa_t fpa, uint32_t *exps, uint32_t *limbs) {
  size_t count = fpa->count;
  if (count == 0) return fpa_success;
  if (cudaMemcpy(fpa->gpu_exps, exps, count * 4, cudaMemcpyHostToDevice) != cudaSuccess) return fpa_device_error;
  return dev(cudaMemcpy(fpa->gpu_limbs, limbs, count * (fpa->precision / 8), cudaMemcpyHostToDevice));
}

// fpa_management.h:33-47
fpa_result fpa_copy_array_to_host(fpa_t fpa, uint32_t *exps, uint32_t *limbs) {
  size_t count = fpa->count;
  if (count == 0) return fpa_success;
  if (cudaMemcpy(exps, fpa->gpu_exps, count * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return fpa_device_error;
  return dev(cudaMemcpy(limbs, fpa->gpu_limbs, count * (fpa->precision / 8), cudaMemcpyDeviceToHost));
}

// fpa_dispatch.h:8-26
fpa_result fpa_set_ui(fpa_t r, uint64_t *ui) {
  return with_device_values(ui, (size_t)r->count * 8, [&](void *d) {
    return dev(gfpa_misc_set_int(r->gpu_exps, r->gpu_limbs, r->precision / 32, r->count, d, 0, 0));
  });
}
// fpa_dispatch.h:28-46
fpa_result fpa_set_si(fpa_t r, int64_t *si) {
  return with_device_values(si, (size_t)r->count * 8, [&](void *d) {
    return dev(gfpa_misc_set_int(r->gpu_exps, r->gpu_limbs, r->precision / 32, r->count, d, 1, 0));
  });
}
// fpa_dispatch.h:48-66
fpa_result fpa_set_float(fpa_t r, float *floats) {
  return with_device_values(floats, (size_t)r->count * 4, [&](void *d) {
    return dev(gfpa_misc_set_fp(r->gpu_exps, r->gpu_limbs, r->precision / 32, r->count, d, 0, 0));
  });
}
// fpa_dispatch.h:68-86
fpa_result fpa_set_double(fpa_t r, double *doubles) {
  return with_device_values(doubles, (size_t)r->count * 8, [&](void *d) {
    return dev(gfpa_misc_set_fp(r->gpu_exps, r->gpu_limbs, r->precision / 32, r->count, d, 1, 0));
  });
}
// fpa_dispatch.h:88-107
fpa_result fpa_set(fpa_t r, fpa_t x, fpa_rounding_mode mode) {
  if (r->count != x->count) return fpa_invalid_counts;
  if ((int)mode < 0 || (int)mode > 4) return fpa_math_error;
  return dev(gfpa_misc_set_prec(r->gpu_exps, r->gpu_limbs, r->precision / 32, x->gpu_exps, x->gpu_limbs,
                                x->precision / 32, r->count, (int)mode, 0));
}
// fpa_dispatch.h:109-126
fpa_result fpa_sgn(int32_t *r, fpa_t x) { return dev(gfpa_misc_sgn(r, x->gpu_exps, x->count, 0)); }
// fpa_dispatch.h:128-151
fpa_result fpa_cmp(int32_t *r, fpa_t a, fpa_t b) {
  if (a->count != b->count) return fpa_invalid_counts;
  if (a->precision != b->precision) return fpa_invalid_precisions;
  return dev(gfpa_misc_cmp(r, a->gpu_exps, a->gpu_limbs, b->gpu_exps, b->gpu_limbs, a->precision / 32, a->count, 0));
}
// fpa_dispatch.h:153-173
fpa_result fpa_neg(fpa_t r, fpa_t a) {
  if (r->count != a->count) return fpa_invalid_counts;
  if (r->precision != a->precision) return fpa_invalid_precisions;
  return dev(gfpa_misc_neg(r->gpu_exps, r->gpu_limbs, a->gpu_exps, a->gpu_limbs, r->precision / 32, r->count, 0));
}

// fpa_dispatch.h:175-223, 225-273, 275-323, 325-373, 375-421
fpa_result fpa_add(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode) { return binary_op(0, r, a, b, mode, 0); }
fpa_result fpa_sub(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode) { return binary_op(1, r, a, b, mode, 0); }
fpa_result fpa_mul(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode) { return binary_op(2, r, a, b, mode, 0); }
fpa_result fpa_div(fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode) { return binary_op(3, r, a, b, mode, 0); }
fpa_result fpa_sqrt(fpa_t r, fpa_t x, fpa_rounding_mode mode) { return unary_op(4, r, x, mode, 0); }

// ---- additions (fpa_gb300.h) ------------------------------------------------------------

fpa_result fpa_gb300_elementwise(fpa_op op, uint32_t precision, uint64_t count, fpa_rounding_mode mode,
                                 uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps, const uint32_t *a_limbs,
                                 const uint32_t *b_exps, const uint32_t *b_limbs, void *stream) {
  if ((int)op != 4 && (b_exps == nullptr || b_limbs == nullptr)) return fpa_math_error;
  return launch_elementwise((int)op, precision, count, (int)mode, r_exps, r_limbs, a_exps, a_limbs, b_exps, b_limbs,
                            (cudaStream_t)stream);
}

// r = RND(a*b + c), one rounding (no counterpart in the reference); argument checks as
// fpa_dispatch.h:175-183 (counts first, then precisions)
fpa_result fpa_gb300_fma(fpa_t r, fpa_t a, fpa_t b, fpa_t c, fpa_rounding_mode mode) {
  const uint32_t count = r->count, precision = r->precision;
  if (count != a->count || count != b->count || count != c->count) return fpa_invalid_counts;
  if (precision != a->precision || precision != b->precision || precision != c->precision)
    return fpa_invalid_precisions;
  if (!valid_precision(precision)) return fpa_invalid_precisions;
  if ((int)mode < 0 || (int)mode > 4) return fpa_math_error;
  if (count == 0) return fpa_success;
  int sms; uint32_t *err;
  if (!ctx(sms, err)) return fpa_device_error;
  ElementwiseArgs args;
  args.count = count; args.n = precision / 32; args.mode = (int)mode;
  args.r_exps = r->gpu_exps; args.r_limbs = r->gpu_limbs;
  args.a_exps = a->gpu_exps; args.a_limbs = a->gpu_limbs;
  args.b_exps = b->gpu_exps; args.b_limbs = b->gpu_limbs;
  args.c_exps = c->gpu_exps; args.c_limbs = c->gpu_limbs;
  args.err = err;
  const int cfg = gfpa_default_cfg(args.n < 4 ? 4 : args.n);
  if (cfg < 0) return fpa_invalid_precisions;
  return gfpa_launch(cfg, GFPA_OP_FMA, &args, 0, sms) == cudaSuccess ? fpa_success : fpa_device_error;
}

fpa_result fpa_op_async(fpa_op op, fpa_t r, fpa_t a, fpa_t b, fpa_rounding_mode mode, void *stream) {
  if ((int)op == 4) return unary_op(4, r, a, mode, (cudaStream_t)stream);
  if ((int)op < 0 || (int)op > 4) return fpa_math_error;
  return binary_op((int)op, r, a, b, mode, (cudaStream_t)stream);
}

fpa_result fpa_copy_array_to_device_async(fpa_t fpa, const uint32_t *exps, const uint32_t *limbs, void *stream) {
  size_t count = fpa->count;
  if (count == 0) return fpa_success;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(fpa->gpu_exps, exps, count * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return fpa_device_error;
  return dev(cudaMemcpyAsync(fpa->gpu_limbs, limbs, count * (fpa->precision / 8), cudaMemcpyHostToDevice, s));
}

fpa_result fpa_copy_array_to_host_async(fpa_t fpa, uint32_t *exps, uint32_t *limbs, void *stream) {
  size_t count = fpa->count;
  if (count == 0) return fpa_success;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(exps, fpa->gpu_exps, count * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return fpa_device_error;
  return dev(cudaMemcpyAsync(limbs, fpa->gpu_limbs, count * (fpa->precision / 8), cudaMemcpyDeviceToHost, s));
}

uint32_t fpa_gb300_device_errors(void) {
  int sms; uint32_t *err;
  if (!ctx(sms, err)) return 0xFFFFFFFFu;
  uint32_t v = 0;
  if (cudaDeviceSynchronize() != cudaSuccess) return 0xFFFFFFFFu;
  if (cudaMemcpy(&v, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 0xFFFFFFFFu;
  cudaMemset(err, 0, 4);
  return v;
}

int fpa_gb300_num_configs(void) { return GFPA_NUM_CFGS; }

fpa_result fpa_gb300_config_shape(int cfg, uint32_t *lanes, uint32_t *tile_limbs, uint32_t *pairs) {
  if (cfg < 0 || cfg >= GFPA_NUM_CFGS) return fpa_math_error;
  if (lanes) *lanes = (uint32_t)gfpa_cfg_G[cfg];
  if (tile_limbs) *tile_limbs = (uint32_t)gfpa_cfg_K[cfg];
  if (pairs) *pairs = (uint32_t)gfpa_cfg_R[cfg];
  return fpa_success;
}

fpa_result fpa_gb300_set_op_config(fpa_op op, uint32_t limbs, int cfg) {
  if ((int)op < 0 || (int)op > 4) return fpa_math_error;
  if (limbs == 0 || limbs > GFPA_MAX_LIMBS) return fpa_invalid_precisions;
  if (cfg < -1 || cfg >= GFPA_NUM_CFGS) return fpa_math_error;
  if (cfg >= 0 && !cfg_fits(cfg, limbs)) return fpa_invalid_precisions;
  if (cfg >= 0 && !gfpa_cfg_supports(cfg, (int)op)) return fpa_math_error;
  std::lock_guard<std::mutex> lk(g_state.mu);
  g_state.cfg_override[(int)op][limbs] = (int8_t)(cfg + 1);
  return fpa_success;
}

int fpa_gb300_get_op_config(fpa_op op, uint32_t limbs) { return gfpa_cfg_for_op((int)op, limbs); }

fpa_result fpa_gb300_set_config(uint32_t limbs, int cfg) {
  for (int op = 0; op < 5; op++) {
    if (cfg >= 0 && !gfpa_cfg_supports(cfg, op)) continue;      // add/sub-only configuration
    fpa_result r = fpa_gb300_set_op_config((fpa_op)op, limbs, cfg);
    if (r != fpa_success) return r;
  }
  return fpa_success;
}

int fpa_gb300_get_config(uint32_t limbs) { return gfpa_cfg_for_op(2, limbs); }

fpa_result fpa_gb300_set_karatsuba_limbs(uint32_t limbs) {
  g_kara_min.store(limbs == 0 ? 0xFFFFFFFFu : limbs, std::memory_order_relaxed);
  return fpa_success;
}

uint32_t fpa_gb300_get_karatsuba_limbs(void) {
  const uint32_t v = g_kara_min.load(std::memory_order_relaxed);
  return v == 0xFFFFFFFFu ? 0u : v;
}

const char *fpa_gb300_version(void) { return "fpa_gb300 0.1 (sm_103a)"; }

}  // extern "C"
