/*
 * ref_runner.c -- runs the reference's own GPU kernels (TEST INFRASTRUCTURE).
 *
 * Loads oracle/_ref/ref_fpa.cubin (the reference's fpa.cu compiled for sm_103a by
 * oracle.build_ref()) through the CUDA driver API and launches its kernels exactly as its
 * host dispatcher does: one warp per number, <<<ceil(count*32/128), 128>>>, with the
 * fpa_arguments block passed by value (fpa_internal.h:34-46, fpa_dispatch.h:175-222) and
 * operands in its lane-interleaved device layout (fpa_management.h:17-47).  Used by the
 * tests to compare against the reference's GPU output and by bench.py to time it.
 *
 * libcuda is opened with dlopen so that no CUDA driver library is needed at link time.
 */
#include <dlfcn.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int CUresult;
typedef int CUdevice;
typedef void *CUcontext;
typedef void *CUmodule;
typedef void *CUfunction;
typedef void *CUstream;
typedef void *CUevent;
typedef unsigned long long CUdeviceptr;

static struct {
  void *h;
  CUresult (*Init)(unsigned);
  CUresult (*DeviceGet)(CUdevice *, int);
  CUresult (*PrimaryRetain)(CUcontext *, CUdevice);
  CUresult (*CtxSetCurrent)(CUcontext);
  CUresult (*ModuleLoad)(CUmodule *, const char *);
  CUresult (*ModuleGetFunction)(CUfunction *, CUmodule, const char *);
  CUresult (*MemAlloc)(CUdeviceptr *, size_t);
  CUresult (*MemFree)(CUdeviceptr);
  CUresult (*MemcpyHtoD)(CUdeviceptr, const void *, size_t);
  CUresult (*MemcpyDtoH)(void *, CUdeviceptr, size_t);
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           CUstream, void **, void **);
  CUresult (*CtxSynchronize)(void);
  CUresult (*EventCreate)(CUevent *, unsigned);
  CUresult (*EventRecord)(CUevent, CUstream);
  CUresult (*EventSynchronize)(CUevent);
  CUresult (*EventElapsedTime)(float *, CUevent, CUevent);
  CUresult (*EventDestroy)(CUevent);
  CUmodule mod;
  int ready;
} D;

/* fpa_internal.h:34-46 */
typedef struct {
  uint32_t count, precision, set_source_precision;
  int mode;
  CUdeviceptr r_exps, r_limbs, a_exps, a_limbs, b_exps, b_limbs;
  CUdeviceptr values;
} ref_arguments;

#define SYM(field, name) if (!(*(void **)&D.field = dlsym(D.h, name))) return -2;

int ref_load(const char *cubin) {
  if (D.ready) return 0;
  D.h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_GLOBAL);
  if (!D.h) return -1;
  SYM(Init, "cuInit"); SYM(DeviceGet, "cuDeviceGet"); SYM(PrimaryRetain, "cuDevicePrimaryCtxRetain");
  SYM(CtxSetCurrent, "cuCtxSetCurrent"); SYM(ModuleLoad, "cuModuleLoad");
  SYM(ModuleGetFunction, "cuModuleGetFunction"); SYM(MemAlloc, "cuMemAlloc_v2"); SYM(MemFree, "cuMemFree_v2");
  SYM(MemcpyHtoD, "cuMemcpyHtoD_v2"); SYM(MemcpyDtoH, "cuMemcpyDtoH_v2"); SYM(LaunchKernel, "cuLaunchKernel");
  SYM(CtxSynchronize, "cuCtxSynchronize"); SYM(EventCreate, "cuEventCreate"); SYM(EventRecord, "cuEventRecord");
  SYM(EventSynchronize, "cuEventSynchronize"); SYM(EventElapsedTime, "cuEventElapsedTime_v2");
  SYM(EventDestroy, "cuEventDestroy_v2");
  CUdevice dev; CUcontext ctx;
  if (D.Init(0) || D.DeviceGet(&dev, 0) || D.PrimaryRetain(&ctx, dev) || D.CtxSetCurrent(ctx)) return -3;
  if (D.ModuleLoad(&D.mod, cubin)) return -4;
  D.ready = 1;
  return 0;
}

/* reference device layout: device[i*n + word*32 + lane] = host[i*n + lane*size + word] */
static void to_ref_layout(uint32_t *dst, const uint32_t *src, uint32_t count, uint32_t n) {
  uint32_t size = n / 32;
  for (uint64_t i = 0; i < count; i++)
    for (uint32_t w = 0; w < size; w++)
      for (uint32_t t = 0; t < 32; t++) dst[i * n + w * 32 + t] = src[i * n + t * size + w];
}
static void from_ref_layout(uint32_t *dst, const uint32_t *src, uint32_t count, uint32_t n) {
  uint32_t size = n / 32;
  for (uint64_t i = 0; i < count; i++)
    for (uint32_t w = 0; w < size; w++)
      for (uint32_t t = 0; t < 32; t++) dst[i * n + t * size + w] = src[i * n + w * 32 + t];
}

/* op: "add", "sub", "mul", "div", "sqrt".  precision in 1024..8192 (step 1024).  Runs the
 * kernel `repeat` times (timed with driver events; *ms = mean per launch) and returns the
 * result of the last launch in host layout.  r_limbs of class results are left as the
 * kernel left them (it does not write them). */
int ref_run(const char *op, uint32_t precision, uint32_t count, int mode, uint32_t *r_exps, uint32_t *r_limbs,
            const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps, const uint32_t *b_limbs,
            int repeat, float *ms) {
  if (!D.ready) return -10;
  if (precision < 1024 || precision > 8192 || precision % 1024) return -11;
  uint32_t n = precision / 32, size = precision / 1024;
  char name[96];
  snprintf(name, sizeof name, "fpa_kernel_warp_%s_%u", op, size);
  char mangled[128];
  snprintf(mangled, sizeof mangled, "_Z%zu%s13fpa_arguments", strlen(name), name);
  CUfunction f;
  if (D.ModuleGetFunction(&f, D.mod, mangled)) return -12;
  size_t lb = (size_t)count * n * 4, eb = (size_t)count * 4;
  uint32_t *tmp = (uint32_t *)malloc(lb ? lb : 4);
  CUdeviceptr d[6] = {0};
  int rc = 0;
  for (int k = 0; k < 6; k++)
    if (D.MemAlloc(&d[k], (k % 2) ? (lb ? lb : 4) : (eb ? eb : 4))) { rc = -13; goto out; }
  to_ref_layout(tmp, a_limbs, count, n);
  if (D.MemcpyHtoD(d[2], a_exps, eb) || D.MemcpyHtoD(d[3], tmp, lb)) { rc = -14; goto out; }
  if (b_exps) {
    to_ref_layout(tmp, b_limbs, count, n);
    if (D.MemcpyHtoD(d[4], b_exps, eb) || D.MemcpyHtoD(d[5], tmp, lb)) { rc = -14; goto out; }
  }
  ref_arguments args;
  memset(&args, 0, sizeof args);
  args.count = count; args.precision = precision; args.mode = mode;
  args.r_exps = d[0]; args.r_limbs = d[1]; args.a_exps = d[2]; args.a_limbs = d[3];
  args.b_exps = d[4]; args.b_limbs = d[5];
  void *params[1] = {&args};
  unsigned grid = (unsigned)(((uint64_t)count * 32 + 127) / 128);
  CUevent e0, e1;
  D.EventCreate(&e0, 0); D.EventCreate(&e1, 0);
  if (D.LaunchKernel(f, grid, 1, 1, 128, 1, 1, 0, NULL, params, NULL)) { rc = -15; goto ev; }   /* warm-up */
  D.EventRecord(e0, NULL);
  for (int r = 0; r < repeat; r++)
    if (D.LaunchKernel(f, grid, 1, 1, 128, 1, 1, 0, NULL, params, NULL)) { rc = -15; goto ev; }
  D.EventRecord(e1, NULL);
  if (D.EventSynchronize(e1) || D.CtxSynchronize()) { rc = -16; goto ev; }
  float t = 0; D.EventElapsedTime(&t, e0, e1);
  if (ms) *ms = repeat > 0 ? t / repeat : 0.f;
  if (D.MemcpyDtoH(r_exps, d[0], eb) || D.MemcpyDtoH(tmp, d[1], lb)) { rc = -17; goto ev; }
  from_ref_layout(r_limbs, tmp, count, n);
ev:
  D.EventDestroy(e0); D.EventDestroy(e1);
out:
  for (int k = 0; k < 6; k++) if (d[k]) D.MemFree(d[k]);
  free(tmp);
  return rc;
}
