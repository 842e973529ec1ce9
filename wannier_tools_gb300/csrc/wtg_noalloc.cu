// Allocation-free batched decimation.
//
// Some callers cannot let this library call cudaMalloc: a host program whose
// device memory is owned by another allocator (a framework's caching pool that
// has already reserved the free HBM, where a fresh cudaMalloc fails or
// fragments the pool), and latency-critical loops in which cudaMalloc /
// cudaFree would synchronise the whole device and stall work on other
// streams.  For them, wtg_surfgreen_batch_noalloc runs the FP64 decimation
// kernel with its scratch (the per-CTA workspace of eight Ndim x Ndim complex
// matrices and the work counter) taken from the fixed array below instead of
// from device allocations.  The caller passes every input and output as device
// memory it already owns.
//
// Properties of the fixed scratch:
//   * WTG_NOALLOC_SCRATCH_BYTES (64 MiB) on every GPU that loads the library,
//     held until the process exits;
//   * its device address is looked up once per device, on the first call made
//     with that device current (cudaGetSymbolAddress); make that first call
//     before any stream capture;
//   * every call shares it and it keeps the previous call's contents: the work
//     counter is cleared at the start of each call (the workspace is fully
//     rewritten per instance by the kernel), and calls whose kernels overlap on
//     the GPU (different streams, or different host threads) race on it — the
//     caller must order them.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/wtgpu.h"
#include "wtg_common.cuh"

#define WTG_NOALLOC_SCRATCH_BYTES (64u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[WTG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int nerr(int code, const std::string& msg) {
  wtg::set_last_error(msg.c_str());          // read back with wtg_last_error
  return code;
}

// Device address of the fixed scratch on the current device (set-up, once per device).
cudaError_t scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int wtg_surfgreen_batch_noalloc(int ndim, int nw, int nk, const double* d_h, int nomega,
                                           const double* d_omega, double eta, double tol,
                                           int itermax, int ntop, const int* top, int nbot,
                                           const int* bot, int divide_by_pi, double* d_dos_l,
                                           double* d_dos_r, double* d_dos_bulk, int32_t* d_iters,
                                           uint8_t* d_status, void* stream) {
  if (ndim < 1 || nw < 1 || ndim % nw != 0 || nk < 0 || nomega < 0 || itermax < 0)
    return nerr(WTG_EINVAL, "bad sizes (ndim, nw, nk, nomega, itermax)");
  if (nk == 0 || nomega == 0) return WTG_OK;
  if (!d_h || !d_omega || !d_dos_l || !d_dos_r || !d_dos_bulk)
    return nerr(WTG_EINVAL, "null device array");
  if (ntop < 0 || nbot < 0 || ntop > wtg::MAX_ORB || nbot > wtg::MAX_ORB || (ntop && !top) ||
      (nbot && !bot))
    return nerr(WTG_EINVAL, "orbital list length out of range [0, 1024] or null");
  for (int q = 0; q < ntop; ++q)
    if (top[q] < 1 || top[q] > nw) return nerr(WTG_EINVAL, "top orbital index outside 1..nw");
  for (int q = 0; q < nbot; ++q)
    if (bot[q] < 1 || bot[q] > nw) return nerr(WTG_EINVAL, "bottom orbital index outside 1..nw");
  if (ndim > wtg::decim_fp64_max_n())
    return nerr(WTG_EUNSUPPORTED, "ndim " + std::to_string(ndim) + " exceeds the kernel limit " +
                                      std::to_string(wtg::decim_fp64_max_n()));
  const size_t per_cta = sizeof(double2) * 8 * (size_t)ndim * ndim;
  const size_t counter_bytes = 256;
  if (per_cta + counter_bytes > WTG_NOALLOC_SCRATCH_BYTES)
    return nerr(WTG_EUNSUPPORTED, "one CTA's workspace (" + std::to_string(per_cta) +
                                      " bytes) exceeds the fixed scratch of " +
                                      std::to_string(WTG_NOALLOC_SCRATCH_BYTES) + " bytes");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return nerr(WTG_ENODEV, "no usable CUDA device");
  void* base = nullptr;
  e = scratch_address(dev, &base);
  if (e != cudaSuccess)
    return nerr(WTG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

  wtg::DecimConfig cfg;
  e = wtg::decim_fp64_config(ndim, 0, &cfg);
  if (e != cudaSuccess) return nerr(WTG_ECUDA, std::string("config: ") + cudaGetErrorString(e));
  if (cfg.ctas_per_sm < 1) return nerr(WTG_EUNSUPPORTED, "decimation kernel does not fit an SM");
  int nsm = 0;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return nerr(WTG_ECUDA, cudaGetErrorString(e));
  const long long n_inst = (long long)nk * nomega;
  const size_t fit = (WTG_NOALLOC_SCRATCH_BYTES - counter_bytes) / per_cta;
  long long grid = (long long)cfg.ctas_per_sm * nsm;
  if ((long long)fit < grid) grid = (long long)fit;
  // every CTA takes one more ticket from the counter after the last instance, so the
  // counter runs to n_inst + grid: that must stay a valid int
  if (n_inst > 0x7fffffffLL - grid)
    return nerr(WTG_EINVAL, "nk * nomega exceeds 2^31 - 1 - " + std::to_string(grid));
  if (n_inst < grid) grid = n_inst;

  cudaStream_t s = (cudaStream_t)stream;
  int* counter = (int*)base;                                      // first 256 bytes
  double2* ws = (double2*)((unsigned char*)base + counter_bytes);  // then the workspace
  e = cudaMemsetAsync(counter, 0, sizeof(int), s);                  // clear the shared counter
  if (e != cudaSuccess) return nerr(WTG_ECUDA, std::string("memset: ") + cudaGetErrorString(e));

  wtg::DecimArgs a;
  memset(&a, 0, sizeof(a));
  a.N = ndim;
  a.nw = nw;
  a.nomega = nomega;
  a.n_inst = (int)n_inst;
  a.h = (const double2*)d_h;
  a.omega = d_omega;
  a.eta = eta;
  a.tol = tol;
  a.itermax = itermax;
  a.divide_by_pi = divide_by_pi;
  a.nk_total = nk;
  a.k_offset = 0;
  a.dos_l = d_dos_l;
  a.dos_r = d_dos_r;
  a.dos_bulk = d_dos_bulk;
  a.iters = d_iters;
  a.status = d_status;
  a.ws = ws;
  a.counter = counter;
  a.KC = cfg.KC;
  a.ntop = ntop;
  a.nbot = nbot;
  for (int q = 0; q < ntop; ++q) a.top[q] = top[q];
  for (int q = 0; q < nbot; ++q) a.bot[q] = bot[q];
  e = wtg::launch_decimate_fp64(a, cfg, (int)grid, s);
  if (e != cudaSuccess) return nerr(WTG_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
  return WTG_OK;
}
