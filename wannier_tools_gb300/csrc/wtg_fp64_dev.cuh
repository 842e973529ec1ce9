// FP64 device building blocks of the decimation: the shared-memory staged
// complex product (zgemm, src/mat_mul.f90:23) and the in-place Gauss-Jordan
// inverse (zgesv with an identity right-hand side, src/inverse.f90:43-55).
// Included inside an anonymous namespace by each translation unit that uses it.
#pragma once

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

