// FP64 pipe throughput probe, used as the roofline denominator of the FP64
// decimation (the measured peaks cover HBM copy and bf16 GEMM only).
// Eight independent DFMA chains per thread, 8 CTAs of 256 threads per SM,
// best of three timed launches.
#include "../../include/wtgpu.h"
#include "wtg_common.cuh"

namespace {

__global__ void k_dfma_chain(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int wtg_probe_fp64_peak(double* tflops) {
  if (!tflops) return WTG_EINVAL;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WTG_ENODEV;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return WTG_ECUDA;
  const int blocks = nsm * 8, threads = 256, iters = 2000;
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return WTG_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  k_dfma_chain<<<blocks, threads>>>(buf, iters, 0.999, 1e-3);
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dfma_chain<<<blocks, threads>>>(buf, iters, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess) return WTG_ECUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return WTG_OK;
}
