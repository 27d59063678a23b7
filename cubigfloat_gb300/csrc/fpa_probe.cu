// fpa_probe.cu -- measures this GPU's integer-multiply throughput, the roofline
// denominator for the multiply-bound kernels (mul, div, sqrt).
//
// Two probes over enough blocks to fill every SM:
//   - isolated mad.lo.u32 / mad.hi.u32: 8 independent chains per thread, the rate of each
//     instruction alone;
//   - limb products: the instruction triple the product kernels issue for one 32x32-bit
//     limb product accumulated into a 96-bit column (mad.lo.cc, madc.hi.cc, addc; the same
//     mac3 as fpa_device.cuh), on an 8-column tile fed from registers as in the product
//     loops.  Its rate, limb products per second, is the roofline denominator.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/fpa_gb300.h"

namespace {

template <bool HI>
__global__ void k_imad_rate(uint32_t *out, uint32_t x, uint32_t y, int iters) {
  uint32_t acc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) acc[k] = threadIdx.x + k;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      uint32_t r;
      if (HI) asm volatile("mad.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(acc[k]), "r"(x), "r"(y + k));
      else asm volatile("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(acc[k]), "r"(x), "r"(y + k));
      acc[k] = r;
    }
  }
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s ^= acc[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// one limb product into a 96-bit column, as the product kernels issue it
__device__ __forceinline__ void mac3p(uint32_t &lo, uint32_t &hi, uint32_t &tp, uint32_t a, uint32_t b) {
  asm volatile("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
               "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
               "addc.u32 %2, %2, 0;"
               : "+r"(lo), "+r"(hi), "+r"(tp) : "r"(a), "r"(b));
}

// 8 columns x 8 operand limbs per step: 64 limb products per thread per iteration
__global__ void k_product_rate(uint32_t *out, uint32_t seed, int iters) {
  uint32_t lo[8], hi[8], tp[8], a[8], w[16];
#pragma unroll
  for (int c = 0; c < 8; c++) { lo[c] = 0; hi[c] = 0; tp[c] = 0; a[c] = seed * (threadIdx.x + c) + 1u; }
#pragma unroll
  for (int c = 0; c < 16; c++) w[c] = seed ^ (blockIdx.x * 16u + c);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int c = 0; c < 8; c++) mac3p(lo[c], hi[c], tp[c], a[i], w[8 + c - i]);
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] += lo[c];      // keep the operands live across iterations
  }
  uint32_t s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s ^= lo[c] ^ hi[c] ^ tp[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class Launch>
float best_ms(Launch launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  launch();                                         // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  return best;
}

template <bool HI>
double rate(uint32_t *buf, int blocks, int threads, int iters) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  k_imad_rate<HI><<<blocks, threads>>>(buf, 3u, 5u, iters);   // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    k_imad_rate<HI><<<blocks, threads>>>(buf, 3u, 5u, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  return (double)blocks * threads * iters * 8 / (best * 1e-3);
}

}  // namespace

extern "C" fpa_result fpa_gb300_measure_product_peak(double *products_per_s) {
  int dev, sms;
  if (cudaGetDevice(&dev) != cudaSuccess) return fpa_device_error;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fpa_device_error;
  const int threads = 256, blocks = sms * 8, iters = 2048;
  uint32_t *buf;
  if (cudaMalloc(&buf, (size_t)blocks * threads * 4) != cudaSuccess) return fpa_device_error;
  const float ms = best_ms([&] { k_product_rate<<<blocks, threads>>>(buf, 0x9E3779B9u, iters); });
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  if (e != cudaSuccess) return fpa_device_error;
  if (products_per_s) *products_per_s = (double)blocks * threads * iters * 64 / (ms * 1e-3);
  return fpa_success;
}

extern "C" fpa_result fpa_gb300_measure_imad_peak(double *mad_lo_per_s, double *mad_hi_per_s) {
  int dev, sms;
  if (cudaGetDevice(&dev) != cudaSuccess) return fpa_device_error;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fpa_device_error;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  uint32_t *buf;
  if (cudaMalloc(&buf, (size_t)blocks * threads * 4) != cudaSuccess) return fpa_device_error;
  double lo = rate<false>(buf, blocks, threads, iters);
  double hi = rate<true>(buf, blocks, threads, iters);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  if (e != cudaSuccess) return fpa_device_error;
  if (mad_lo_per_s) *mad_lo_per_s = lo;
  if (mad_hi_per_s) *mad_hi_per_s = hi;
  return fpa_success;
}
