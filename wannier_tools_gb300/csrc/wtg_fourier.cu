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

// the LO-TO form evaluates everything at k shifted off Gamma:
// |k|^2 <= 1e-4 -> k = (1e-4, 1e-4) (src/ham_qlayer2qlayer.f90:366-370)
__device__ __forceinline__ void loto_k(double& k1, double& k2) {
  if (fabs(k1 * k1 + k2 * k2) <= 0.0001) {
    k1 = 0.0001;
    k2 = 0.0001;
  }
}

__global__ void k_phases(const double* __restrict__ k, int nk_total, int k0, int kc,
                         const double2* __restrict__ rab, int nRu, double2* __restrict__ phase,
                         int loto) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)kc * nRu) return;
  const int ikl = (int)(t / nRu), r = (int)(t % nRu);
  double k1 = k[k0 + ikl], k2 = k[k0 + ikl + nk_total];
  if (loto) loto_k(k1, k2);
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
  if (a.loto) {
    // src/ham_qlayer2qlayer.f90:372-413: the k-dependent non-analytic term
    // nac(i, j) = kZ(j) kZ(i) c / sqrt(M(ii) M(jj)) is added to every H(R) of
    // the group, i.e. nac times the group's sum of phase / ndegen
    const int ie = e % a.nw, je = e / a.nw;
    const int ii = ie / 3, pp = ie % 3, jj = je / 3, qq = je % 3;
    for (int f = 0; f < FK; ++f) {
      if (kb + f >= a.kc) break;
      double k1 = a.k[a.k0 + kb + f], k2 = a.k[a.k0 + kb + f + a.nk_total];
      loto_k(k1, k2);
      const double t1 = k1 * a.ld[0] + k2 * a.ld[1], t2 = k1 * a.ld[2] + k2 * a.ld[3];
      const double temp2 = k1 * t1 + k2 * t2;
      const double c = 4.0 * 3.1415926 / (temp2 * a.lvol) * 29.54263748 / 0.529177;
      const double kzi = k1 * a.lz[(ii * 2 + 0) * 3 + pp] + k2 * a.lz[(ii * 2 + 1) * 3 + pp];
      const double kzj = k1 * a.lz[(jj * 2 + 0) * 3 + qq] + k2 * a.lz[(jj * 2 + 1) * 3 + qq];
      const double nac = kzj * kzi * c / sqrt(a.lmass[ii] * a.lmass[jj]);
      double2 ps = make_double2(0.0, 0.0);
      for (int r = a.icoff[g]; r < r1; ++r) {
        const double2 ph = __ldg(a.phase + (size_t)(kb + f) * a.nRu + r);
        const double w = __ldg(a.wr + r);
        ps.x = fma(ph.x, w, ps.x);
        ps.y = fma(ph.y, w, ps.y);
      }
      acc[f].x = fma(nac, ps.x, acc[f].x);
      acc[f].y = fma(nac, ps.y, acc[f].y);
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
                                                          a.nRu, a.phase, a.loto);
  }
  const int N = a.nw * a.np;
  cudaMemsetAsync(a.h, 0, sizeof(double2) * (size_t)a.kc * 2 * N * N, s);
  if (a.nic > 0) {
    dim3 grid((a.nw * a.nw + FT - 1) / FT, a.nic, (a.kc + FK - 1) / FK);
    k_fourier<<<grid, FT, 0, s>>>(a);
  }
}

}  // namespace wtg
