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

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(NPEND) : "memory");
}

// cta_gemm for operands that live in DRAM (the large-Ndim workspaces exceed the
// L2): the same shared area (2 N KC double2) holds two stages of KS = KC / 2
// columns, filled with cp.async, so that the next K chunk loads while the
// current one is computed instead of between two barriers.  Every output sums
// the same products in the same (ascending k) order as cta_gemm: the results
// are bit-identical.
template <int RP, int EPI>
__device__ double cta_gemm_db(const double2* __restrict__ X, const double2* __restrict__ Y, int N,
                              int KC, double2* stages, double2* out0, double2* out1) {
  const int T = blockDim.x, tid = threadIdx.x, NN = N * N;
  const int KS = KC / 2;
  const int nch = (N + KS - 1) / KS;
  const int rounds = (NN + T - 1) / T;
  double nrm = 0.0;
  auto stage = [&](int c) {
    const int k0 = c * KS, kc = min(KS, N - k0);
    double2* sx = stages + (size_t)(c & 1) * 2 * N * KS;
    double2* sy = sx + (size_t)N * KS;
    const double2* Xc = X + (size_t)k0 * N;          // columns k0.. are contiguous
    for (int e = tid; e < N * kc; e += T) cp_async16(sx + e, Xc + e);
    for (int e = tid; e < N * kc; e += T) {
      const int kk = e % kc, j = e / kc;
      cp_async16(sy + kk + j * KS, Y + (k0 + kk) + (size_t)j * N);
    }
    cp_async_commit();
  };
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
      ob[r] = j * KS;
      acc[r] = make_double2(0.0, 0.0);
    }
    stage(0);
    for (int c = 0; c < nch; ++c) {
      if (c + 1 < nch) {
        stage(c + 1);                 // its buffer was last read before the previous barrier
        cp_async_wait<1>();           // this thread's copies of chunk c have landed
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();                // everyone's copies of chunk c are visible
      const int kc = min(KS, N - c * KS);
      const double2* sx = stages + (size_t)(c & 1) * 2 * N * KS;
      const double2* sy = sx + (size_t)N * KS;
      for (int kk = 0; kk < kc; ++kk) {
        const double2* xr = sx + kk * N;
        const double2* yr = sy + kk;
#pragma unroll
        for (int r = 0; r < RP; ++r) {
          if (r < nr) cfma(acc[r], xr[oa[r]], yr[ob[r]]);
        }
      }
      __syncthreads();                // chunk c's buffer may be refilled
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

constexpr int GJ_PANEL = 8;   // pivot steps per pass of the global-memory Gauss-Jordan

struct Shared {
  double2* big;      // N*N inverse work, or the GEMM stages
  double2* sX;
  double2* sY;
  double2* pan;      // [N][GJ_PANEL] panel columns (global-memory inverse; aliases the stages)
  double2* mult;     // [N][GJ_PANEL] elimination multipliers of the panel's steps (same)
  double2* colbuf;   // [N]
  double2* rowbuf;   // [N]
  double2* recip;    // [GJ_PANEL] pivot reciprocals
  double* red;       // [32]
  int* perm;         // [N]
  int* cols;         // [N]
  int* misc;         // [4]: 0 instance, 1 singular flag
};

// Shared-memory layout: the first region holds either the N x N inverse (when
// it runs in shared memory) or the two GEMM stages of N x KC; the small arrays
// follow.  fp64_smem_bytes on the host gives the same size.
__device__ __forceinline__ Shared fp64_layout(unsigned char* smraw, int N, int KC, bool inv_in_smem) {
  const size_t big = inv_in_smem ? (size_t)max(N * N, 2 * N * KC) : (size_t)2 * N * KC;
  Shared s;
  s.big = reinterpret_cast<double2*>(smraw);
  s.sX = s.big;
  s.sY = s.big + (size_t)N * KC;
  s.pan = s.big;
  s.mult = s.big + (size_t)N * GJ_PANEL;
  s.colbuf = s.big + big;
  s.rowbuf = s.colbuf + N;
  s.recip = s.rowbuf + N;
  s.red = reinterpret_cast<double*>(s.recip + GJ_PANEL);
  s.perm = reinterpret_cast<int*>(s.red + 32);
  s.cols = s.perm + N;
  s.misc = s.cols + N;
  return s;
}

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
// Gauss-Jordan of the n x n matrix at sM (leading dimension ld) in place, with
// partial pivoting (first maximal |re|+|im| in the column, as izamax).  The
// inverse is left with its columns permuted: inverse(i, j) = sM[i + cols[j]*ld].
// An exact zero pivot leaves the identity (zgesv + inv do the same,
// src/inverse.f90:51-55) and returns 1.
__device__ int gj_core(double2* __restrict__ sM, int n, int ld, const Shared& s) {
  const int T = blockDim.x, tid = threadIdx.x, nn = n * n;
  const int warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s.misc[1] = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (warp == 0) {
      long long best = -1;
      int bi = n;
      for (int i = k + lane; i < n; i += 32) {
        const long long v = cabs1_key(sM[i + k * ld]);
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
      for (int i = lane; i < n; i += 32) s.colbuf[i] = sM[(i == p ? k : i) + k * ld];
      if (lane == 0) {
        s.perm[k] = p;
        if (best == 0) {
          s.misc[1] = 1;
        } else {
          const double2 pv = sM[p + k * ld];
          const double inv_d = 1.0 / (pv.x * pv.x + pv.y * pv.y);
          s.recip[0] = make_double2(pv.x * inv_d, -pv.y * inv_d);
        }
      }
    }
    __syncthreads();
    if (s.misc[1]) break;
    const int p = s.perm[k];
    const double2 r = s.recip[0];
    for (int j = tid; j < n; j += T) {
      const double2 akj = sM[k + j * ld];
      const double2 apj = sM[p + j * ld];
      if (p != k) sM[p + j * ld] = akj;
      const double2 nk = (j == k) ? r : cmul(apj, r);
      sM[k + j * ld] = nk;
      s.rowbuf[j] = nk;
    }
    __syncthreads();
    for (int e = tid; e < nn; e += T) {
      const int i = e % n, j = e / n;
      if (i != k) {
        double2* a = sM + i + j * ld;
        double2 v = (j == k) ? make_double2(0.0, 0.0) : *a;
        const double2 f = s.colbuf[i];
        const double2 rk = s.rowbuf[j];
        v.x = fma(-f.x, rk.x, v.x);
        v.x = fma(f.y, rk.y, v.x);
        v.y = fma(-f.x, rk.y, v.y);
        v.y = fma(-f.y, rk.x, v.y);
        *a = v;
      }
    }
    __syncthreads();
  }
  const int singular = s.misc[1];
  if (singular) {
    for (int e = tid; e < nn; e += T)
      sM[e % n + (e / n) * ld] = make_double2(e % (n + 1) == 0 ? 1.0 : 0.0, 0.0);
    for (int j = tid; j < n; j += T) s.cols[j] = j;
  } else if (tid == 0) {
    for (int j = 0; j < n; ++j) s.cols[j] = j;
    for (int k = n - 1; k >= 0; --k) {      // undo the row swaps as column swaps
      const int p = s.perm[k];
      const int t = s.cols[k];
      s.cols[k] = s.cols[p];
      s.cols[p] = t;
    }
  }
  __syncthreads();
  return singular;
}

// (w I - X) into the shared N x N area; rev reads X's indices in reverse order
__device__ void gj_load(const double2* __restrict__ X, double2 w, int N, bool rev, const Shared& s) {
  const int T = blockDim.x, NN = N * N;
  for (int e = threadIdx.x; e < NN; e += T) {
    const int src = rev ? NN - 1 - e : e;      // (N-1-i) + (N-1-j) N
    const double2 x = X[src];
    double2 v = make_double2(-x.x, -x.y);                 // 0 - eps off the diagonal
    if (e % (N + 1) == 0) v = make_double2(w.x - x.x, w.y - x.y);
    s.big[e] = v;
  }
}

// sM := (w I - X)^-1 by in-place Gauss-Jordan in shared memory (gj_core); the
// inverse is left with its columns permuted: inverse(i, j) = sM[i + cols[j]*N].
__device__ int gj_invert(const double2* __restrict__ X, double2 w, int N, const Shared& s) {
  gj_load(X, w, N, false, s);
  return gj_core(s.big, N, N, s);
}

// The trailing nb x nb block of (w I - X)^-1, or with rev the leading block
// (X's indices read in reverse order), in shared memory: Gaussian elimination
// of the other m = N - nb columns, pivoting among their own rows, leaves the
// Schur complement of that part in the trailing block, and gj_core inverts it:
// (N^3 - nb^3) / 3 + nb^3 complex multiply-adds instead of N^3.  The block
// inverse stays at s.big + m + m N: block(i, j) = s.big[m + i + (m + cols[j]) N].
// The spectral sums of src/surfstat.f90:149-160 and src/fermiarc.f90:237-248
// read one principal layer's block of GLL or GRR only.  Returns 1 on an exact
// zero pivot (the caller then takes the full inverse).
__device__ int schur_block_invert(const double2* __restrict__ X, double2 w, int N, int nb,
                                  bool rev, const Shared& s) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarp = blockDim.x >> 5;
  const int m = N - nb;
  double2* sM = s.big;
  gj_load(X, w, N, rev, s);
  if (tid == 0) s.misc[1] = 0;
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    if (warp == 0) {
      long long best = -1;
      int bi = m;
      for (int i = k + lane; i < m; i += 32) {
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
      if (best == 0) {
        if (lane == 0) s.misc[1] = 1;
      } else {
        const double2 pv = sM[p + k * N];
        const double inv_d = 1.0 / (pv.x * pv.x + pv.y * pv.y);
        const double2 r = make_double2(pv.x * inv_d, -pv.y * inv_d);
        // multipliers of the rows below k after the swap k <-> p, and the pivot row
        for (int i = k + 1 + lane; i < N; i += 32)
          s.colbuf[i] = cmul(sM[(i == p ? k : i) + k * N], r);
        for (int j = k + 1 + lane; j < N; j += 32) s.rowbuf[j] = sM[p + j * N];
        if (lane == 0) s.misc[2] = p;
      }
    }
    __syncthreads();
    if (s.misc[1]) break;
    const int p = s.misc[2];
    // trailing update; row p receives what row k held (row k itself is done)
    for (int j = k + 1 + warp; j < N; j += nwarp) {
      const double2 rk = s.rowbuf[j];
      for (int i = k + 1 + lane; i < N; i += 32) {
        double2 v = sM[(i == p ? k : i) + j * N];
        const double2 f = s.colbuf[i];
        v.x = fma(-f.x, rk.x, v.x);
        v.x = fma(f.y, rk.y, v.x);
        v.y = fma(-f.x, rk.y, v.y);
        v.y = fma(-f.y, rk.x, v.y);
        sM[i + j * N] = v;
      }
    }
    __syncthreads();
  }
  if (s.misc[1]) {
    __syncthreads();
    return 1;
  }
  return gj_core(sM + m + (size_t)m * N, nb, N, s);
}

// dynamic shared memory of an FP64 decimation launch whose inverse runs in
// global memory (two GEMM stages of N x 16, then the small arrays): the same for
// the per-model and the batch kernels at this Ndim
__host__ __device__ constexpr int fp64_gi_smem_bytes(int N) {
  return 2 * N * 16 * 16 + N * 32 + 16 * GJ_PANEL + 32 * 8 + N * 8 + 16;
}

// Layout of schur_block_invert_global: the nb x nb Schur complement, then the
// small arrays sized for the full N (the elimination's multipliers and pivot row).
__host__ __device__ constexpr int schur_area_bytes(int N, int nb) {
  return nb * nb * 16 + N * 32 + 16 * GJ_PANEL + 32 * 8 + N * 8 + 16;
}
__device__ __forceinline__ Shared schur_layout(unsigned char* smraw, int N, int nb) {
  Shared s;
  s.big = reinterpret_cast<double2*>(smraw);
  s.sX = s.sY = s.pan = s.mult = nullptr;
  s.colbuf = s.big + (size_t)nb * nb;
  s.rowbuf = s.colbuf + N;
  s.recip = s.rowbuf + N;
  s.red = reinterpret_cast<double*>(s.recip + GJ_PANEL);
  s.perm = reinterpret_cast<int*>(s.red + 32);
  s.cols = s.perm + N;
  s.misc = s.cols + N;
  return s;
}

// schur_block_invert for an N x N matrix too large for shared memory: the
// elimination runs on Mg in global memory (a warp per column, its lanes on
// consecutive rows), then the nb x nb Schur complement is copied into shared
// memory (schur_layout) and inverted there by gj_core: block(i, j) =
// s.big[i + cols[j] nb].  Returns 1 on an exact zero pivot.
__device__ int schur_block_invert_global(const double2* __restrict__ X, double2 w, int N, int nb,
                                         bool rev, double2* __restrict__ Mg, const Shared& s) {
  const int T = blockDim.x, tid = threadIdx.x, NN = N * N;
  const int warp = tid >> 5, lane = tid & 31, nwarp = T >> 5;
  const int m = N - nb;
  for (int e = tid; e < NN; e += T) {
    const double2 x = X[rev ? NN - 1 - e : e];
    double2 v = make_double2(-x.x, -x.y);
    if (e % (N + 1) == 0) v = make_double2(w.x - x.x, w.y - x.y);
    Mg[e] = v;
  }
  if (tid == 0) s.misc[1] = 0;
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    if (warp == 0) {
      long long best = -1;
      int bi = m;
      for (int i = k + lane; i < m; i += 32) {
        const long long v = cabs1_key(Mg[i + (size_t)k * N]);
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
      if (best == 0) {
        if (lane == 0) s.misc[1] = 1;
      } else {
        const double2 pv = Mg[p + (size_t)k * N];
        const double inv_d = 1.0 / (pv.x * pv.x + pv.y * pv.y);
        const double2 r = make_double2(pv.x * inv_d, -pv.y * inv_d);
        for (int i = k + 1 + lane; i < N; i += 32)
          s.colbuf[i] = cmul(Mg[(i == p ? k : i) + (size_t)k * N], r);
        for (int j = k + 1 + lane; j < N; j += 32) s.rowbuf[j] = Mg[p + (size_t)j * N];
        if (lane == 0) s.misc[2] = p;
      }
    }
    __syncthreads();
    if (s.misc[1]) break;
    const int p = s.misc[2];
    for (int j = k + 1 + warp; j < N; j += nwarp) {
      const double2 rk = s.rowbuf[j];
      double2* col = Mg + (size_t)j * N;
      for (int i = k + 1 + lane; i < N; i += 32) {
        double2 v = col[i == p ? k : i];
        const double2 f = s.colbuf[i];
        v.x = fma(-f.x, rk.x, v.x);
        v.x = fma(f.y, rk.y, v.x);
        v.y = fma(-f.x, rk.y, v.y);
        v.y = fma(-f.y, rk.x, v.y);
        col[i] = v;
      }
    }
    __syncthreads();
  }
  if (s.misc[1]) {
    __syncthreads();
    return 1;
  }
  for (int e = tid; e < nb * nb; e += T)
    s.big[e] = Mg[m + e % nb + (size_t)(m + e / nb) * N];
  __syncthreads();
  return gj_core(s.big, nb, nb, s);
}

constexpr int GJ_ROWS = 10;    // rows per lane of the global-memory inverse: Ndim <= 320

// one complex entry of a lane's register column (row = lane + 32 m) by a
// warp-uniform slot index, without local memory
__device__ __forceinline__ double2 gj_pick(const double2 (&x)[GJ_ROWS], int m) {
  double2 v = x[0];
#pragma unroll
  for (int q = 1; q < GJ_ROWS; ++q)
    if (q == m) v = x[q];
  return v;
}

__device__ __forceinline__ double2 shfl_c(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Mg := (w I - X)^-1 by the Gauss-Jordan steps of gj_invert, with the matrix
// in global memory (Ndim too large for shared memory).  The steps run in
// panels of GJ_PANEL columns: a panel is reduced in shared memory, recording
// each step's pivot row, reciprocal and multiplier column; then every other
// column is read once into registers (one warp per column, lane l holding
// rows l, l+32, ...), put through the panel's steps in order and written
// back.  Every entry sees the same operations in the same order as in
// gj_invert, so the two agree bit for bit; global traffic is two N x N sweeps
// per panel instead of per step.  The inverse is left with permuted columns
// (inverse(i, j) = Mg[i + cols[j]*N]); an exact zero pivot leaves the
// identity and returns 1.
__device__ int gj_invert_global(const double2* __restrict__ X, double2 w, int N,
                                double2* __restrict__ Mg, const Shared& s) {
  const int T = blockDim.x, tid = threadIdx.x, NN = N * N;
  const int warp = tid >> 5, lane = tid & 31, nwarp = T >> 5;
  double2* __restrict__ P = s.pan;
  double2* __restrict__ Cm = s.mult;
  for (int e = tid; e < NN; e += T) {
    const double2 x = X[e];
    double2 v = make_double2(-x.x, -x.y);
    if (e % (N + 1) == 0) v = make_double2(w.x - x.x, w.y - x.y);
    Mg[e] = v;
  }
  if (tid == 0) s.misc[1] = 0;
  __syncthreads();
  for (int k0 = 0; k0 < N; k0 += GJ_PANEL) {
    const int pb = min(GJ_PANEL, N - k0);
    for (int e = tid; e < N * pb; e += T) P[e] = Mg[(size_t)k0 * N + e];   // panel columns
    __syncthreads();
    for (int t = 0; t < pb; ++t) {
      const int k = k0 + t;
      if (warp == 0) {
        long long best = -1;
        int bi = N;
        for (int i = k + lane; i < N; i += 32) {
          const long long v = cabs1_key(P[i + t * N]);
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
        for (int i = lane; i < N; i += 32) Cm[i + t * N] = P[(i == p ? k : i) + t * N];
        if (lane == 0) {
          s.perm[k] = p;
          if (best == 0) {
            s.misc[1] = 1;
          } else {
            const double2 pv = P[p + t * N];
            const double inv_d = 1.0 / (pv.x * pv.x + pv.y * pv.y);
            s.recip[t] = make_double2(pv.x * inv_d, -pv.y * inv_d);
          }
        }
      }
      __syncthreads();
      if (s.misc[1]) break;
      const int p = s.perm[k];
      const double2 r = s.recip[t];
      if (tid < pb) {                       // pivot row of the panel
        const int j = tid;
        const double2 akj = P[k + j * N];
        const double2 apj = P[p + j * N];
        if (p != k) P[p + j * N] = akj;
        const double2 nk = (j == t) ? r : cmul(apj, r);
        P[k + j * N] = nk;
        s.rowbuf[j] = nk;
      }
      __syncthreads();
      for (int e = tid; e < N * pb; e += T) {
        const int i = e % N, j = e / N;
        if (i != k) {
          double2 v = (j == t) ? make_double2(0.0, 0.0) : P[e];
          const double2 f = Cm[i + t * N];
          const double2 rk = s.rowbuf[j];
          v.x = fma(-f.x, rk.x, v.x);
          v.x = fma(f.y, rk.y, v.x);
          v.y = fma(-f.x, rk.y, v.y);
          v.y = fma(-f.y, rk.x, v.y);
          P[e] = v;
        }
      }
      __syncthreads();
    }
    if (s.misc[1]) break;
    // every column outside the panel through the panel's steps, in registers
    for (int j = warp; j < N; j += nwarp) {
      if (j >= k0 && j < k0 + pb) continue;
      double2* col = Mg + (size_t)j * N;
      double2 x[GJ_ROWS];
#pragma unroll
      for (int q = 0; q < GJ_ROWS; ++q) {
        const int i = lane + 32 * q;
        x[q] = i < N ? col[i] : make_double2(0.0, 0.0);
      }
      for (int t = 0; t < pb; ++t) {
        const int k = k0 + t, p = s.perm[k];
        const double2 r = s.recip[t];
        const double2 akj = shfl_c(gj_pick(x, k >> 5), k & 31);
        const double2 apj = shfl_c(gj_pick(x, p >> 5), p & 31);
        const double2 nk = cmul(apj, r);
        const double2* cm = Cm + t * N;
#pragma unroll
        for (int q = 0; q < GJ_ROWS; ++q) {
          const int i = lane + 32 * q;
          if (i < N && i != k) {
            double2 v = (i == p) ? akj : x[q];
            const double2 f = cm[i];
            v.x = fma(-f.x, nk.x, v.x);
            v.x = fma(f.y, nk.y, v.x);
            v.y = fma(-f.x, nk.y, v.y);
            v.y = fma(-f.y, nk.x, v.y);
            x[q] = v;
          } else if (i == k) {
            x[q] = nk;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < GJ_ROWS; ++q) {
        const int i = lane + 32 * q;
        if (i < N) col[i] = x[q];
      }
    }
    for (int e = tid; e < N * pb; e += T) Mg[(size_t)k0 * N + e] = P[e];
    __syncthreads();
  }
  const int singular = s.misc[1];
  if (singular) {
    for (int e = tid; e < NN; e += T) Mg[e] = make_double2(e % (N + 1) == 0 ? 1.0 : 0.0, 0.0);
    for (int j = tid; j < N; j += T) s.cols[j] = j;
  } else if (tid == 0) {
    for (int j = 0; j < N; ++j) s.cols[j] = j;
    for (int k = N - 1; k >= 0; --k) {
      const int p = s.perm[k];
      const int t = s.cols[k];
      s.cols[k] = s.cols[p];
      s.cols[p] = t;
    }
  }
  __syncthreads();
  return singular;
}

// out = the un-permuted inverse left in Mg by gj_invert_global
__device__ void gj_store_global(int N, const double2* __restrict__ Mg, const Shared& s,
                                double2* __restrict__ out) {
  const int T = blockDim.x, NN = N * N;
  for (int e = threadIdx.x; e < NN; e += T) {
    const int i = e % N, j = e / N;
    out[e] = Mg[i + (size_t)s.cols[j] * N];
  }
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

// H00 / H01 of one in-plane k point straight into workspace matrices 0..4
// (eps, eps_s, eps_t = H00; alpha = H01; beta = H01^dagger).  Each entry is
// the same sum, in the same R order with the same phases, as k_fourier's
// (src/ham_qlayer2qlayer.f90:45-87); ph is a shared-memory table of nRu phases.
__device__ void fourier_fill(const BatchModel& m, double k1, double k2, double2* W,
                             double2* __restrict__ ph) {
  const int N = m.N, NN = N * N, nw = m.nw, nw2 = nw * nw, T = blockDim.x, tid = threadIdx.x;
  for (int r = tid; r < m.nRu; r += T) {
    const double kdotr = k1 * m.rab[r].x + k2 * m.rab[r].y;  // :55
    double sn, cs;
    sincos(2.0 * PI_REF * kdotr, &sn, &cs);                   // :56
    ph[r] = make_double2(cs, sn);
  }
  __syncthreads();
  for (int e = tid; e < NN; e += T) {
    const int i = e % N, j = e / N;
    const int bi = i / nw, ie = i % nw, bj = j / nw, je = j % nw;
    const int el = ie + je * nw;
    double2 v0 = make_double2(0.0, 0.0), v1 = v0;
    const int g0 = bj - bi - m.ic_lo;                         // H00 block (bi, bj): ic = bj - bi
    if (g0 >= 0 && g0 < m.nic)
      for (int r = m.icoff[g0]; r < m.icoff[g0 + 1]; ++r) cfma(v0, m.hr[(size_t)r * nw2 + el], ph[r]);
    const int g1 = bj + m.np - bi - m.ic_lo;                  // H01 block (bi, bj): ic = bj + Np - bi
    if (g1 >= 0 && g1 < m.nic)
      for (int r = m.icoff[g1]; r < m.icoff[g1 + 1]; ++r) cfma(v1, m.hr[(size_t)r * nw2 + el], ph[r]);
    W[e] = v0;
    W[NN + e] = v0;
    W[2 * NN + e] = v0;
    W[3 * NN + e] = v1;
    W[4 * NN + j + (size_t)i * N] = make_double2(v1.x, -v1.y);
  }
  __syncthreads();
}
