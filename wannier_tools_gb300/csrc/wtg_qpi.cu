// Joint density of states (quasi-particle interference) from computed surface
// spectra.  Both are autocorrelations of the dos arrays, evaluated here in
// FP64 with the reference's summation order (one thread per output, the sum
// in the reference's loop order, multiplies and adds kept unfused), so the
// results equal a sequential evaluation bit for bit.
//
//  * k-path form, src/surfstat.f90:889-905: for each omega j and shift
//    s = iq - Nh (Nh = (nk-1)/2, 1-based iq), the sum over ik1 in
//    [max(-Nh-s, -Nh)+Nh+1, min(Nh-s, Nh)+Nh+1] of dos(ik1, j) * dos(ik1+s, j).
//  * k-plane form (QPI), src/fermiarc.f90:497-545: for each grid point
//    q = (iq1, iq2) in ikp order (second index fastest), the sum over
//    ik2 = 1..nky (outer), ik1 = 1..nkx (inner) of
//    sum_c in_c(ik1, ik2) * in_c(mod(ik1+iq1-2, p1)+1, mod(ik2+iq2-2, p2)+1),
//    with the channel products added left to right ((c0 + c1) + c2) + c3 as in
//    the reference's jsdos statement; p1, p2 are the periods the reference uses
//    (nkx-1, nky-1 for jdos; Nk1-1, Nk2-1 for the spin-resolved jsdos).
#include <string>

#include "../../include/wtgpu.h"
#include "wtg_common.cuh"

namespace wtg {
namespace {

__global__ void k_jdos_kpath(int nk, int nomega, const double* __restrict__ dos,
                             double* __restrict__ jdos) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nk * nomega) return;
  const int iq = (int)(t % nk), j = (int)(t / nk);          // 0-based
  const int nh = (nk - 1) / 2;
  const int s = iq + 1 - nh;                                 // iq1 of the reference
  const int imin = max(-nh - s, -nh) + nh + 1, imax = min(nh - s, nh) + nh + 1;   // 1-based
  const double* d = dos + (size_t)j * nk;
  double acc = 0.0;
  for (int ik1 = imin; ik1 <= imax; ++ik1)
    acc = __dadd_rn(acc, __dmul_rn(d[ik1 - 1], d[ik1 - 1 + s]));
  jdos[t] = acc;
}

__global__ void k_jdos_kplane(int nkx, int nky, int p1, int p2, int nchan,
                              const double* __restrict__ in, double scale,
                              double* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = nkx * nky;
  if (q >= nn) return;
  const int b1 = q / nky, b2 = q % nky;                      // iq1-1, iq2-1
  double acc = 0.0;
  for (int a2 = 0; a2 < nky; ++a2) {
    const int c2 = (a2 + b2) % p2;
    for (int a1 = 0; a1 < nkx; ++a1) {
      const int c1 = (a1 + b1) % p1;
      const int e0 = a1 + a2 * nkx, e1 = c1 + c2 * nkx;
      double term = __dmul_rn(in[e0], in[e1]);
      for (int c = 1; c < nchan; ++c)
        term = __dadd_rn(term, __dmul_rn(in[(size_t)c * nn + e0], in[(size_t)c * nn + e1]));
      acc = __dadd_rn(acc, term);
    }
  }
  out[q] = scale == 1.0 ? acc : acc * scale;
}

int qfail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

int qcuda(cudaError_t e, const char* where) {
  set_last_error((std::string(where) + ": " + cudaGetErrorString(e)).c_str());
  return WTG_ECUDA;
}

}  // namespace
}  // namespace wtg

extern "C" {

int wtg_jdos_kpath(int nk, int nomega, const double* dos, double* jdos) {
  using namespace wtg;
  if (nk < 0 || nomega < 0) return qfail(WTG_EINVAL, "nk, nomega must be >= 0");
  if ((size_t)nk * nomega == 0) return WTG_OK;
  if (!dos || !jdos) return qfail(WTG_EINVAL, "null array");
  const size_t n = (size_t)nk * nomega;
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * n);
  if (e != cudaSuccess) return qcuda(e, "wtg_jdos_kpath");
  e = cudaMemcpy(d, dos, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_jdos_kpath<<<(unsigned)((n + 255) / 256), 256>>>(nk, nomega, d, d + n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(jdos, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? WTG_OK : qcuda(e, "wtg_jdos_kpath");
}

int wtg_jdos_kplane(int nkx, int nky, int p1, int p2, int nchan, const double* chans, double scale,
                    double* jdos) {
  using namespace wtg;
  if (nkx < 1 || nky < 1 || nchan < 1) return qfail(WTG_EINVAL, "nkx, nky, nchan must be >= 1");
  if (p1 < 1 || p2 < 1) return qfail(WTG_EINVAL, "periods p1, p2 must be >= 1");
  if (p1 > nkx || p2 > nky) return qfail(WTG_EINVAL, "periods exceed the grid");
  if (!chans || !jdos) return qfail(WTG_EINVAL, "null array");
  const size_t nn = (size_t)nkx * nky;
  if (nn > (size_t)1 << 30) return qfail(WTG_EUNSUPPORTED, "grid too large");
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * (nchan + 1) * nn);
  if (e != cudaSuccess) return qcuda(e, "wtg_jdos_kplane");
  e = cudaMemcpy(d, chans, sizeof(double) * nchan * nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_jdos_kplane<<<(unsigned)((nn + 127) / 128), 128>>>(nkx, nky, p1, p2, nchan, d, scale,
                                                          d + (size_t)nchan * nn);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(jdos, d + (size_t)nchan * nn, sizeof(double) * nn, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? WTG_OK : qcuda(e, "wtg_jdos_kplane");
}

}  // extern "C"
