// Principal-layer Fourier sum: H00/H01 for a chunk of in-plane k points.
//
// Restates src/ham_qlayer2qlayer.f90:45-87 for a batch of k:
//   Hij(:,:,ic) = sum_{R : R3 = ic} HmnR(:,:,R) * exp(2 pi i (k1 R1 + k2 R2)) / ndegen(R)
//   H00 block (i,j) = Hij(j-i),  H01 block (i, j-Np) = Hij(j-i),  j in Np+1..2Np.
// Layout in HBM: HmnR blocks sorted by R3 (stable in the reference's iR
// order, so each Hij element is summed in the reference's order), one
// Nw*Nw column-major block per R.  Phases e^{2 pi i k.R} are computed once per
// (k, R) in FP64 into a [k][R] table; each thread then owns one matrix element
// for FK k points and streams the R blocks with coalesced 16-byte loads.
#include "wtg_common.cuh"

namespace wtg {

constexpr int FK = 8;          // k points per thread
constexpr int FT = 128;        // threads per CTA

__global__ void k_phases(const double* __restrict__ k, int nk_total, int k0, int kc,
                         const double2* __restrict__ rab, int nRu, double2* __restrict__ phase) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)kc * nRu) return;
  const int ikl = (int)(t / nRu), r = (int)(t % nRu);
  const double k1 = k[k0 + ikl], k2 = k[k0 + ikl + nk_total];
  const double kdotr = k1 * rab[r].x + k2 * rab[r].y;      // src/ham_qlayer2qlayer.f90:55
  double s, c;
  sincos(2.0 * PI_REF * kdotr, &s, &c);                     // :56
  phase[t] = make_double2(c, s);
}

__global__ void __launch_bounds__(FT) k_fourier(const FourierArgs a) {
  const int nw2 = a.nw * a.nw;
  const int e = blockIdx.x * FT + threadIdx.x;
  const int g = blockIdx.y;                 // R3 group
  const int kb = blockIdx.z * FK;
  if (e >= nw2) return;
  const int ic = a.ic_lo + g;
  double2 acc[FK];
#pragma unroll
  for (int f = 0; f < FK; ++f) acc[f] = make_double2(0.0, 0.0);
  const int r1 = a.icoff[g + 1];
  for (int r = a.icoff[g]; r < r1; ++r) {
    const double2 hv = __ldg(a.hr + (size_t)r * nw2 + e);
#pragma unroll
    for (int f = 0; f < FK; ++f) {
      if (kb + f < a.kc) cfma(acc[f], hv, __ldg(a.phase + (size_t)(kb + f) * a.nRu + r));
    }
  }
  const int N = a.nw * a.np;
  const int ie = e % a.nw, je = e / a.nw;
  for (int f = 0; f < FK; ++f) {
    if (kb + f >= a.kc) break;
    double2* H00 = a.h + (size_t)(kb + f) * 2 * N * N;
    double2* H01 = H00 + (size_t)N * N;
    for (int bi = 0; bi < a.np; ++bi) {
      const int bj = bi + ic;                 // H00 block (bi, bj), ic = bj - bi
      if (bj >= 0 && bj < a.np) H00[(bi * a.nw + ie) + (size_t)(bj * a.nw + je) * N] = acc[f];
      const int bj1 = bi + ic - a.np;         // H01 block (bi, bj1), ic = bj1 + Np - bi
      if (bj1 >= 0 && bj1 < a.np) H01[(bi * a.nw + ie) + (size_t)(bj1 * a.nw + je) * N] = acc[f];
    }
  }
}

void launch_fourier(const FourierArgs& a, cudaStream_t s) {
  const long nph = (long)a.kc * a.nRu;
  if (nph > 0) {
    k_phases<<<(unsigned)((nph + 255) / 256), 256, 0, s>>>(a.k, a.nk_total, a.k0, a.kc, a.rab,
                                                          a.nRu, a.phase);
  }
  const int N = a.nw * a.np;
  cudaMemsetAsync(a.h, 0, sizeof(double2) * (size_t)a.kc * 2 * N * N, s);
  if (a.nic > 0) {
    dim3 grid((a.nw * a.nw + FT - 1) / FT, a.nic, (a.kc + FK - 1) / FK);
    k_fourier<<<grid, FT, 0, s>>>(a);
  }
}

}  // namespace wtg
