// All-FP64 Lopez-Sancho decimation (surfgreen_1985) for a batch of (k, omega)
// instances, one CTA per instance, persistent over an atomic work counter.
//
// Restates src/surfgreen.f90:74-134 per instance:
//   eps = eps_s = eps_t = H00, alpha = H01, beta = H01^dagger, w = omega + i eta
//   repeat (<= itermax):
//     g = (w - eps)^-1                           (Gauss-Jordan, shared memory)
//     m1 = alpha g ; m2 = beta g
//     t = m1 beta ; eps += t ; eps_s += t
//     t = m2 alpha; eps += t ; eps_t += t
//     alpha = m1 alpha ; beta = m2 beta
//     stop when sum_ij |alpha_ij| <= tol
//   GLL = (w - eps_s)^-1, GRR = (w - eps_t)^-1, GB = (w - eps)^-1
// followed by the spectral sums of src/surfstat.f90:149-160 /
// src/fermiarc.f90:237-248.
//
// GB300 notes.  FP64 runs at 2 DFMA/clk/SM on this part (1.2 TFLOP/s measured,
// with FP64 mma.sync slower still), so the kernel is bound by the FP64 pipe,
// not by memory: the eight N x N matrices of an instance live in a per-CTA
// global workspace (L2-resident), GEMM operands are staged through shared
// memory in k-chunks, and the inverse runs in shared memory.  What matters is
// the count of FP64 instructions (exactly 4 DFMA per complex multiply-add)
// and keeping the pipe fed; pivot searches compare magnitudes as integers.
#include "wtg_common.cuh"

namespace wtg {

namespace {

constexpr int EPI_STORE = 0;       // out0 = acc
constexpr int EPI_ADD2 = 1;        // out0 += acc ; out1 += acc
constexpr int EPI_STORE_NORM = 2;  // out0 = acc ; return sum |acc|

// C = X*Y for N x N column-major X, Y (global), written through an epilogue.
// Thread t owns the flattened column-major indices t + r*T; each pass keeps RP
// of them in registers while X[:, k0:k0+kc] and Y[k0:k0+kc, :] stream
// through shared memory.
template <int RP, int EPI>
__device__ double cta_gemm(const double2* __restrict__ X, const double2* __restrict__ Y, int N,
                           int KC, double2* sX, double2* sY, double2* out0, double2* out1) {
  const int T = blockDim.x, tid = threadIdx.x, NN = N * N;
  const int rounds = (NN + T - 1) / T;
  double nrm = 0.0;
  for (int r0 = 0; r0 < rounds; r0 += RP) {
    const int nr = min(RP, rounds - r0);
    int oa[RP], ob[RP];
    double2 acc[RP];
#pragma unroll
    for (int r = 0; r < RP; ++r) {
      const int idx = tid + (r0 + r) * T;
      int i = 0, j = 0;
      if (idx < NN) {
        i = idx % N;
        j = idx / N;
      }
      oa[r] = i;
      ob[r] = j * KC;
      acc[r] = make_double2(0.0, 0.0);
    }
    for (int k0 = 0; k0 < N; k0 += KC) {
      const int kc = min(KC, N - k0);
      const double2* Xc = X + (size_t)k0 * N;        // columns k0.. are contiguous
      for (int e = tid; e < N * kc; e += T) sX[e] = Xc[e];
      for (int e = tid; e < N * kc; e += T) {
        const int kk = e % kc, j = e / kc;
        sY[kk + j * KC] = Y[(k0 + kk) + (size_t)j * N];
      }
      __syncthreads();
      for (int kk = 0; kk < kc; ++kk) {
        const double2* xr = sX + kk * N;
        const double2* yr = sY + kk;
#pragma unroll
        for (int r = 0; r < RP; ++r) {
          if (r < nr) cfma(acc[r], xr[oa[r]], yr[ob[r]]);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < RP; ++r) {
      const int idx = tid + (r0 + r) * T;
      if (r < nr && idx < NN) {
        if (EPI == EPI_STORE) {
          out0[idx] = acc[r];
        } else if (EPI == EPI_ADD2) {
          double2 v = out0[idx];
          v.x += acc[r].x;
          v.y += acc[r].y;
          out0[idx] = v;
          double2 w = out1[idx];
          w.x += acc[r].x;
          w.y += acc[r].y;
          out1[idx] = w;
        } else {
          out0[idx] = acc[r];
          nrm += sqrt(acc[r].x * acc[r].x + acc[r].y * acc[r].y);
        }
      }
    }
  }
  return nrm;
}

struct Shared {
  double2* big;      // N*N inverse work, or the GEMM stages
  double2* sX;
  double2* sY;
  double2* colbuf;   // [N]
  double2* rowbuf;   // [N]
  double2* recip;    // [2]
  double* red;       // [32]
  int* perm;         // [N]
  int* cols;         // [N]
  int* misc;         // [4]: 0 instance, 1 singular flag
};

// |re| + |im| (LAPACK's dcabs1, the izamax criterion) as an order-preserving
// integer key: non-negative doubles compare like their bit patterns.
__device__ __forceinline__ long long cabs1_key(double2 v) {
  return __double_as_longlong(fabs(v.x) + fabs(v.y));
}

// sM := (w I - X)^-1 by in-place Gauss-Jordan with partial pivoting (first
// maximal |re|+|im| in the column, as izamax).  The inverse is left with its
// columns permuted: inverse(i, j) = sM[i + cols[j]*N].  An exact zero pivot
// leaves the identity (zgesv + inv do the same, src/inverse.f90:51-55) and
// returns 1.
__device__ int gj_invert(const double2* __restrict__ X, double2 w, int N, const Shared& s) {
  const int T = blockDim.x, tid = threadIdx.x, NN = N * N;
  const int warp = tid >> 5, lane = tid & 31;
  double2* sM = s.big;
  for (int e = tid; e < NN; e += T) {
    const double2 x = X[e];
    double2 v = make_double2(-x.x, -x.y);                 // 0 - eps off the diagonal
    if (e % (N + 1) == 0) v = make_double2(w.x - x.x, w.y - x.y);
    sM[e] = v;
  }
  if (tid == 0) s.misc[1] = 0;
  __syncthreads();
  for (int k = 0; k < N; ++k) {
    if (warp == 0) {
      long long best = -1;
      int bi = N;
      for (int i = k + lane; i < N; i += 32) {
        const long long v = cabs1_key(sM[i + k * N]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const long long ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      const int p = bi;
      // column k after the row swap k <-> p (entry k itself is not used)
      for (int i = lane; i < N; i += 32) s.colbuf[i] = sM[(i == p ? k : i) + k * N];
      if (lane == 0) {
        s.perm[k] = p;
        if (best == 0) {
          s.misc[1] = 1;
        } else {
          const double2 pv = sM[p + k * N];
          const double inv_d = 1.0 / (pv.x * pv.x + pv.y * pv.y);
          s.recip[0] = make_double2(pv.x * inv_d, -pv.y * inv_d);
        }
      }
    }
    __syncthreads();
    if (s.misc[1]) break;
    const int p = s.perm[k];
    const double2 r = s.recip[0];
    for (int j = tid; j < N; j += T) {
      const double2 akj = sM[k + j * N];
      const double2 apj = sM[p + j * N];
      if (p != k) sM[p + j * N] = akj;
      const double2 nk = (j == k) ? r : cmul(apj, r);
      sM[k + j * N] = nk;
      s.rowbuf[j] = nk;
    }
    __syncthreads();
    for (int e = tid; e < NN; e += T) {
      const int i = e % N, j = e / N;
      if (i != k) {
        double2 v = (j == k) ? make_double2(0.0, 0.0) : sM[e];
        const double2 f = s.colbuf[i];
        const double2 rk = s.rowbuf[j];
        v.x = fma(-f.x, rk.x, v.x);
        v.x = fma(f.y, rk.y, v.x);
        v.y = fma(-f.x, rk.y, v.y);
        v.y = fma(-f.y, rk.x, v.y);
        sM[e] = v;
      }
    }
    __syncthreads();
  }
  const int singular = s.misc[1];
  if (singular) {
    for (int e = tid; e < NN; e += T) sM[e] = make_double2(e % (N + 1) == 0 ? 1.0 : 0.0, 0.0);
    for (int j = tid; j < N; j += T) s.cols[j] = j;
  } else if (tid == 0) {
    for (int j = 0; j < N; ++j) s.cols[j] = j;
    for (int k = N - 1; k >= 0; --k) {      // undo the row swaps as column swaps
      const int p = s.perm[k];
      const int t = s.cols[k];
      s.cols[k] = s.cols[p];
      s.cols[p] = t;
    }
  }
  __syncthreads();
  return singular;
}

// write the un-permuted inverse from shared memory to global
__device__ void gj_store(int N, const Shared& s, double2* out) {
  const int T = blockDim.x, NN = N * N;
  for (int e = threadIdx.x; e < NN; e += T) {
    const int i = e % N, j = e / N;
    out[e] = s.big[i + s.cols[j] * N];
  }
}

__device__ __forceinline__ double2 gj_diag(int N, const Shared& s, int i) {
  return s.big[i + s.cols[i] * N];
}

__device__ double block_sum(double v, const Shared& s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) s.red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t += s.red[w];
    s.red[0] = t;
  }
  __syncthreads();
  t = s.red[0];
  __syncthreads();
  return t;
}

template <int RP>
__global__ void __launch_bounds__(512, 1) k_decimate_fp64(const DecimArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = a.N, NN = N * N, T = blockDim.x, tid = threadIdx.x;
  const size_t big = (size_t)max(NN, 2 * N * a.KC);
  Shared s;
  s.big = reinterpret_cast<double2*>(smraw);
  s.sX = s.big;
  s.sY = s.big + (size_t)N * a.KC;
  s.colbuf = s.big + big;
  s.rowbuf = s.colbuf + N;
  s.recip = s.rowbuf + N;
  s.red = reinterpret_cast<double*>(s.recip + 2);
  s.perm = reinterpret_cast<int*>(s.red + 32);
  s.cols = s.perm + N;
  s.misc = s.cols + N;

  double2* W = a.ws + (size_t)blockIdx.x * 8 * NN;
  double2* E = W;
  double2* ES = W + (size_t)NN;
  double2* ET = W + (size_t)2 * NN;
  double2* bufs[5] = {W + (size_t)3 * NN, W + (size_t)4 * NN, W + (size_t)5 * NN,
                      W + (size_t)6 * NN, W + (size_t)7 * NN};

  for (;;) {
    if (tid == 0) s.misc[0] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int inst = s.misc[0];
    __syncthreads();
    if (inst >= a.n_inst) break;
    const int ik = inst / a.nomega, iw = inst % a.nomega;
    const double2* H00 = a.h + (size_t)ik * 2 * NN;
    const double2* H01 = H00 + NN;
    const double2 w = make_double2(a.omega[iw], a.eta);     // src/surfgreen.f90:82

    double2* Al = bufs[0];
    double2* Be = bufs[1];
    double2* G = bufs[2];
    double2* M1 = bufs[3];
    double2* M2 = bufs[4];
    for (int e = tid; e < NN; e += T) {                       // src/surfgreen.f90:74-78
      const double2 h = H00[e];
      E[e] = h;
      ES[e] = h;
      ET[e] = h;
      Al[e] = H01[e];
      const int i = e % N, j = e / N;
      const double2 t = H01[j + (size_t)i * N];
      Be[e] = make_double2(t.x, -t.y);
    }
    __syncthreads();

    int st = 0, it = 0;
    bool conv = false;
    for (int itc = 1; itc <= a.itermax; ++itc) {              // src/surfgreen.f90:86
      it = itc;
      if (gj_invert(E, w, N, s)) st |= PT_SINGULAR;           // :88-89
      gj_store(N, s, G);
      __syncthreads();
      cta_gemm<RP, EPI_STORE>(Al, G, N, a.KC, s.sX, s.sY, M1, nullptr);    // :92
      cta_gemm<RP, EPI_STORE>(Be, G, N, a.KC, s.sX, s.sY, M2, nullptr);    // :95
      cta_gemm<RP, EPI_ADD2>(M1, Be, N, a.KC, s.sX, s.sY, E, ES);          // :98-102
      cta_gemm<RP, EPI_ADD2>(M2, Al, N, a.KC, s.sX, s.sY, E, ET);          // :107-110
      double part = cta_gemm<RP, EPI_STORE_NORM>(M1, Al, N, a.KC, s.sX, s.sY, G, nullptr);  // :113
      cta_gemm<RP, EPI_STORE>(M2, Be, N, a.KC, s.sX, s.sY, M1, nullptr);   // :116
      // rotate buffers: alpha <- G, beta <- M1
      double2* t0 = Al;
      Al = G;
      G = t0;
      double2* t1 = Be;
      Be = M1;
      M1 = t1;
      const double nrm = block_sum(part, s);                  // :120
      if (nrm <= a.tol) {                                     // :121
        conv = true;
        break;
      }
    }
    if (!conv) st |= PT_NOT_CONVERGED;

    const size_t oidx = (size_t)(a.k_offset + ik) + (size_t)iw * a.nk_total;
    double dl = 0.0, dr = 0.0, db = 0.0;
    // GLL = (w - eps_s)^-1                                   // :127-128
    if (gj_invert(ES, w, N, s)) st |= PT_SINGULAR;
    if (a.gll) gj_store(N, s, a.gll + (size_t)inst * NN);
    if (tid == 0) {
      for (int q = 0; q < a.ntop; ++q) {
        const int io = a.top[q] - 1;
        const double v = gj_diag(N, s, io).y;
        dl = a.divide_by_pi ? dl - v / PI_REF : dl - v;
      }
    }
    __syncthreads();
    // GRR = (w - eps_t)^-1                                   // :130-131
    if (gj_invert(ET, w, N, s)) st |= PT_SINGULAR;
    if (a.grr) gj_store(N, s, a.grr + (size_t)inst * NN);
    if (tid == 0) {
      for (int q = 0; q < a.nbot; ++q) {
        const int io = N - a.nw + a.bot[q] - 1;
        const double v = gj_diag(N, s, io).y;
        dr = a.divide_by_pi ? dr - v / PI_REF : dr - v;
      }
    }
    __syncthreads();
    // GB = (w - eps)^-1                                      // :133-134
    if (gj_invert(E, w, N, s)) st |= PT_SINGULAR;
    if (a.gb) gj_store(N, s, a.gb + (size_t)inst * NN);
    if (tid == 0) {
      for (int i = 0; i < N; ++i) {
        const double v = gj_diag(N, s, i).y;
        db = a.divide_by_pi ? db - v / PI_REF : db - v;
      }
      if (!isfinite(dl) || !isfinite(dr) || !isfinite(db)) st |= PT_NONFINITE;
      a.dos_l[oidx] = dl;
      a.dos_r[oidx] = dr;
      a.dos_bulk[oidx] = db;
      if (a.iters) a.iters[oidx] = it;
      if (a.status) a.status[oidx] = (uint8_t)st;
    }
    __syncthreads();
  }
}

size_t smem_bytes(int N, int KC) {
  const size_t big = (size_t)(N * N > 2 * N * KC ? N * N : 2 * N * KC);
  return big * 16 + (size_t)N * 32 + 32 + 32 * 8 + (size_t)N * 8 + 16;
}

}  // namespace

int decim_fp64_max_n() {
  int n = 8;
  while (smem_bytes(n + 1, (n + 1) / 2) <= 227 * 1024) ++n;
  return n;
}

cudaError_t decim_fp64_config(int N, int threads_override, DecimConfig* cfg) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int smem_optin = 0;
  e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  int T = threads_override > 0 ? threads_override : (N <= 48 ? 128 : (N <= 80 ? 256 : 512));
  int KC = N;
  if (smem_bytes(N, KC) > (size_t)smem_optin) KC = (N + 1) / 2;
  while (KC > 1 && smem_bytes(N, KC) > (size_t)smem_optin) --KC;
  const int rounds = (N * N + T - 1) / T;
  int RP = 13;
  if (rounds <= 4) RP = 4;
  else if (rounds <= 8) RP = 8;
  cfg->threads = T;
  cfg->KC = KC;
  cfg->RP = RP;
  cfg->smem = smem_bytes(N, KC);
  int occ = 0;
  const void* fn = RP == 4 ? (const void*)k_decimate_fp64<4>
                           : (RP == 8 ? (const void*)k_decimate_fp64<8> : (const void*)k_decimate_fp64<13>);
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg->smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, T, cfg->smem);
  if (e != cudaSuccess) return e;
  cfg->ctas_per_sm = occ;
  return cudaSuccess;
}

cudaError_t launch_decimate_fp64(const DecimArgs& a, const DecimConfig& cfg, int grid,
                                 cudaStream_t s) {
  switch (cfg.RP) {
    case 4: k_decimate_fp64<4><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
    case 8: k_decimate_fp64<8><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
    default: k_decimate_fp64<13><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
  }
  return cudaGetLastError();
}

}  // namespace wtg
