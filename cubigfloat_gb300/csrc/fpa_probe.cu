// fpa_probe.cu -- measures this GPU's integer-multiply throughput, the roofline
// denominator for the multiply-bound kernels (mul, div, sqrt).
//
// Each thread runs 8 independent chains of mad.lo.u32 (or mad.hi.u32) over enough blocks
// to fill every SM; the rate is multiply-adds per second over the whole device.
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
