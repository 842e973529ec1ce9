// FP64 throughput probes, the roofline denominators of the FP64 decimation
// (the measured peaks cover HBM copy and bf16 GEMM only):
//   wtg_probe_fp64_peak   the DFMA pipe: eight independent DFMA chains per
//                         thread, 8 CTAs of 256 threads per SM;
//   wtg_probe_dmma_peak   the FP64 tensor path (mma.sync m8n8k4 .f64, the
//                         instruction a zgemm on tensor cores would use):
//                         eight independent accumulator tiles per warp, same
//                         grid.
// Best of three timed launches each.  The FP64 form issues DFMA because the
// DMMA path measures slower on GB300.
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

// D = A B + D for eight independent 8x8x4 FP64 tiles per warp, iters times
__global__ void k_dmma_chain(double* out, int iters, double a, double b) {
  const double av = a + 1e-3 * (threadIdx.x & 31), bv = b;
  double d[8][2];
#pragma unroll
  for (int t = 0; t < 8; ++t) d[t][0] = d[t][1] = (double)t;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int t = 0; t < 8; ++t)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(d[t][0]), "+d"(d[t][1])
                   : "d"(av), "d"(bv));
  }
  double acc = 0.0;
#pragma unroll
  for (int t = 0; t < 8; ++t) acc += d[t][0] + d[t][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// best-of-three time (ms) of one launch of kernel k on blocks x threads
template <class K>
int time_probe(K k, int blocks, int threads, int iters, float* best_ms) {
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return WTG_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  k<<<blocks, threads>>>(buf, iters, 0.999, 1e-3);
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k<<<blocks, threads>>>(buf, iters, 0.999, 1e-3);
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
  *best_ms = best;
  return WTG_OK;
}

}  // namespace

extern "C" int wtg_probe_dmma_peak(double* tflops) {
  if (!tflops) return WTG_EINVAL;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WTG_ENODEV;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return WTG_ECUDA;
  const int blocks = nsm * 8, threads = 256, iters = 1000;
  float ms = 0.f;
  const int rc = time_probe(k_dmma_chain, blocks, threads, iters, &ms);
  if (rc != WTG_OK) return rc;
  // per warp and iteration: 8 tiles x 8 x 8 x 4 multiply-adds = 2048 FMA = 4096 flops
  *tflops = 4096.0 * iters * (double)blocks * (threads / 32) / (ms * 1e-3) / 1e12;
  return WTG_OK;
}

extern "C" int wtg_probe_fp64_peak(double* tflops) {
  if (!tflops) return WTG_EINVAL;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WTG_ENODEV;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return WTG_ECUDA;
  const int blocks = nsm * 8, threads = 256, iters = 2000;
  float best = 0.f;
  const int rc = time_probe(k_dfma_chain, blocks, threads, iters, &best);
  if (rc != WTG_OK) return rc;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return WTG_OK;
}
