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
#include <algorithm>

#include <mutex>

#include "wtg_common.cuh"

namespace wtg {

namespace {

#include "wtg_fp64_dev.cuh"

// Options of one solve for the batch kernel, with the member names of
// DecimArgs (whose kernel parameter the plain kernel passes directly, so its
// lists are read from parameter space).  Orbital lists are 1-based.
struct SolveOpts {
  int nw;
  double tol;
  int itermax;
  int divide_by_pi;
  int ntop, nbot;
  const int* top;
  const int* bot;
  double* spin[6];             // null: no spin-resolved sums
  int spin_right_bottom;
};

// The products of one decimation step.  At the large Ndim of the global-memory
// inverse the eight workspaces of all resident CTAs no longer fit the L2, so
// operands come from DRAM and their staging is double-buffered.
template <int RP, int EPI, bool GI>
__device__ __forceinline__ double gemm(const double2* X, const double2* Y, int N, int KC,
                                       const Shared& s, double2* out0, double2* out1) {
  if (GI) return cta_gemm_db<RP, EPI>(X, Y, N, KC, s.sX, out0, out1);
  return cta_gemm<RP, EPI>(X, Y, N, KC, s.sX, s.sY, out0, out1);
}

// Decimation of one instance whose eps, eps_s, eps_t (= H00), alpha (= H01)
// and beta (= H01^dagger) already sit in workspace matrices 0..4 of W; the
// spectral sums of the three final inverses are handed to emit(dl, dr, db,
// spin[6], iterations, status) in thread 0, the inverses themselves go to
// gll / grr / gb when those are not null.
// GI = false: the inverse runs in shared memory (Ndim <= decim_fp64_max_n());
// GI = true: it runs in workspace matrix 8 in global memory, in panels
// (gj_invert_global; Ndim <= 320).
template <int RP, bool GI, class O, class Emit>
__device__ void fp64_solve(int N, int KC, double2 w, const O& o, double2* gll, double2* grr,
                           double2* gb, double2* W, const Shared& s, Emit emit) {
  const int NN = N * N, tid = threadIdx.x;
  double2* Mg = GI ? W + (size_t)8 * NN : nullptr;   // global-memory inverse work
  double2* E = W;
  double2* ES = W + (size_t)NN;
  double2* ET = W + (size_t)2 * NN;
  double2* Al = W + (size_t)3 * NN;
  double2* Be = W + (size_t)4 * NN;
  double2* G = W + (size_t)5 * NN;
  double2* M1 = W + (size_t)6 * NN;
  double2* M2 = W + (size_t)7 * NN;
  // (w - X)^-1, optionally stored un-permuted to dst; ginv reads the result
  // blk 1 / 2: only the leading / trailing Num_wann block of the inverse (one
  // principal layer), from the Schur complement of the rest, where the spectral
  // sums read nothing else (schur_block_invert); a zero pivot there takes the
  // full inverse.  With GI the block's inverse needs its Num_wann^2 area within
  // the stage area every launch of this Ndim has (KC = 16).
  const int m = N - o.nw;
  const bool gblk = !GI || schur_area_bytes(N, o.nw) <= fp64_gi_smem_bytes(N);
  const Shared fb = schur_layout(reinterpret_cast<unsigned char*>(s.big), N, o.nw);
  int blk = 0;
  auto invert = [&](const double2* X, double2* dst, int want_blk) -> int {
    blk = (gblk && !dst && m > 0) ? want_blk : 0;
    if (blk && !(GI ? schur_block_invert_global(X, w, N, o.nw, blk == 1, Mg, fb)
                    : schur_block_invert(X, w, N, o.nw, blk == 1, s)))
      return 0;
    blk = 0;
    int sing;
    if (GI) {
      sing = gj_invert_global(X, w, N, Mg, s);
      if (dst) gj_store_global(N, Mg, s, dst);
    } else {
      sing = gj_invert(X, w, N, s);
      if (dst) gj_store(N, s, dst);
    }
    return sing;
  };
  auto ginv = [&](int i, int j) {
    if (blk) {                        // block entry (i, j): local indices in the block
      const int li = blk == 1 ? o.nw - 1 - i : i - m;
      const int lj = blk == 1 ? o.nw - 1 - j : j - m;
      return GI ? fb.big[li + (size_t)fb.cols[lj] * o.nw]
                : s.big[m + li + (size_t)(m + s.cols[lj]) * N];
    }
    return GI ? Mg[i + (size_t)s.cols[j] * N] : s.big[i + s.cols[j] * N];
  };

  int st = 0, it = 0;
  bool conv = false;
  for (int itc = 1; itc <= o.itermax; ++itc) {                // src/surfgreen.f90:86
    it = itc;
    if (invert(E, G, 0)) st |= PT_SINGULAR;                   // :88-89
    __syncthreads();
    gemm<RP, EPI_STORE, GI>(Al, G, N, KC, s, M1, nullptr);              // :92
    gemm<RP, EPI_STORE, GI>(Be, G, N, KC, s, M2, nullptr);              // :95
    gemm<RP, EPI_ADD2, GI>(M1, Be, N, KC, s, E, ES);                    // :98-102
    gemm<RP, EPI_ADD2, GI>(M2, Al, N, KC, s, E, ET);                    // :107-110
    double part = gemm<RP, EPI_STORE_NORM, GI>(M1, Al, N, KC, s, G, nullptr);  // :113
    gemm<RP, EPI_STORE, GI>(M2, Be, N, KC, s, M1, nullptr);             // :116
    // rotate buffers: alpha <- G, beta <- M1
    double2* t0 = Al;
    Al = G;
    G = t0;
    double2* t1 = Be;
    Be = M1;
    M1 = t1;
    const double nrm = block_sum(part, s);                    // :120
    if (nrm <= o.tol) {                                       // :121
      conv = true;
      break;
    }
  }
  if (!conv) st |= PT_NOT_CONVERGED;

  double dl = 0.0, dr = 0.0, db = 0.0;
  double spin[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  // GLL = (w - eps_s)^-1                                     // :127-128
  if (invert(ES, gll, 1)) st |= PT_SINGULAR;
  if (tid == 0) {
    for (int q = 0; q < o.ntop; ++q) {
      const int io = o.top[q] - 1;
      const double v = ginv(io, io).y;
      dl = o.divide_by_pi ? dl - v / PI_REF : dl - v;
    }
    if (o.spin[0])                                            // src/surfstat.f90:162-177
      spin_sums(ginv, o.nw, o.ntop, o.top, 0, o.divide_by_pi, spin[0], spin[1], spin[2]);
  }
  __syncthreads();
  // GRR = (w - eps_t)^-1                                     // :130-131
  // surfstat's spin sums read GRR's leading block as well (src/surfstat.f90:178-192)
  if (invert(ET, grr, (o.spin[0] && !o.spin_right_bottom) ? 0 : 2)) st |= PT_SINGULAR;
  if (tid == 0) {
    for (int q = 0; q < o.nbot; ++q) {
      const int io = N - o.nw + o.bot[q] - 1;
      const double v = ginv(io, io).y;
      dr = o.divide_by_pi ? dr - v / PI_REF : dr - v;
    }
    if (o.spin[0]) {                                          // src/surfstat.f90:178-192
      if (o.spin_right_bottom)                                // src/fermiarc.f90:300-327
        spin_sums(ginv, o.nw, o.nbot, o.bot, N - o.nw, o.divide_by_pi, spin[3], spin[4], spin[5]);
      else
        spin_sums(ginv, o.nw, o.ntop, o.top, 0, o.divide_by_pi, spin[3], spin[4], spin[5]);
    }
  }
  __syncthreads();
  // GB = (w - eps)^-1                                        // :133-134
  if (invert(E, gb, 0)) st |= PT_SINGULAR;
  if (tid == 0) {
    for (int i = 0; i < N; ++i) {
      const double v = ginv(i, i).y;
      db = o.divide_by_pi ? db - v / PI_REF : db - v;
    }
    if (!isfinite(dl) || !isfinite(dr) || !isfinite(db)) st |= PT_NONFINITE;
    emit(dl, dr, db, spin, it, st);
  }
  __syncthreads();
}

template <int RP, bool GI>
__global__ void __launch_bounds__(GI ? 256 : 512, 1) k_decimate_fp64(const __grid_constant__ DecimArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = a.N, NN = N * N, T = blockDim.x, tid = threadIdx.x;
  const Shared s = fp64_layout(smraw, N, a.KC, !GI);
  double2* W = a.ws + (size_t)blockIdx.x * (GI ? 9 : 8) * NN;

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
    for (int e = tid; e < NN; e += T) {                       // src/surfgreen.f90:74-78
      const double2 h = H00[e];
      W[e] = h;
      W[NN + e] = h;
      W[2 * NN + e] = h;
      W[3 * NN + e] = H01[e];
      const int i = e % N, j = e / N;
      const double2 t = H01[j + (size_t)i * N];
      W[4 * NN + e] = make_double2(t.x, -t.y);
    }
    __syncthreads();
    const size_t oidx = (size_t)(a.k_offset + ik) + (size_t)iw * a.nk_total;
    fp64_solve<RP, GI>(N, a.KC, w, a, a.gll ? a.gll + (size_t)inst * NN : nullptr,
                       a.grr ? a.grr + (size_t)inst * NN : nullptr,
                       a.gb ? a.gb + (size_t)inst * NN : nullptr, W, s,
                       [&](double dl, double dr, double db, const double* spin, int it, int st) {
                         a.dos_l[oidx] = dl;
                         a.dos_r[oidx] = dr;
                         a.dos_bulk[oidx] = db;
                         if (a.spin[0])
                           for (int c = 0; c < 6; ++c) a.spin[c][oidx] = spin[c];
                         if (a.iters) a.iters[oidx] = it;
                         if (a.status) a.status[oidx] = (uint8_t)st;
                       });
  }
}

// Uneven batch: points of several models (different Ndim, eta per point) in
// one persistent launch.  CTAs take points in the host's cost order (largest
// first); each point runs its own Fourier sum, then the shared-memory or the
// global-memory inverse variant by its Ndim, and stops at its own convergence.
__global__ void __launch_bounds__(256, 1) k_batch_fp64(const __grid_constant__ BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int tid = threadIdx.x;
  double2* W = a.ws + (size_t)blockIdx.x * a.ws_stride;
  __shared__ int sinst;
  const int npts = a.run ? a.run->npts : a.npts;
  const double tol = a.run ? a.run->tol : a.tol;
  const int itermax = a.run ? a.run->itermax : a.itermax;
  const int divide_by_pi = a.run ? a.run->divide_by_pi : a.divide_by_pi;
  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.counter, 1);
      sinst = q < npts ? a.order[q] : -1;
    }
    __syncthreads();
    const int p = sinst;
    __syncthreads();
    if (p < 0) break;
    const BatchModel& m = a.models[a.pmodel[p]];
    const int N = m.N;
    const bool gi = N > a.smem_gj_max;
    const Shared s = fp64_layout(smraw, N, a.KC, !gi);
    fourier_fill(m, a.k[p], a.k[p + a.npts], W, reinterpret_cast<double2*>(smraw + a.ph_off));
    SolveOpts o;
    o.nw = m.nw;
    o.tol = tol;
    o.itermax = itermax;
    o.divide_by_pi = divide_by_pi;
    o.ntop = m.ntop;
    o.nbot = m.nbot;
    o.top = m.top;
    o.bot = m.bot;
    for (int c = 0; c < 6; ++c) o.spin[c] = nullptr;
    o.spin_right_bottom = 0;
    const double2 w = make_double2(a.omega[p], a.eta[p]);
    auto emit = [&](double dl, double dr, double db, const double*, int it, int st) {
      a.dos_l[p] = dl;
      a.dos_r[p] = dr;
      a.dos_bulk[p] = db;
      if (a.iters) a.iters[p] = it;
      if (a.status) a.status[p] = (uint8_t)st;
    };
    if (gi) fp64_solve<13, true>(N, a.KC, w, o, nullptr, nullptr, nullptr, W, s, emit);
    else fp64_solve<13, false>(N, a.KC, w, o, nullptr, nullptr, nullptr, W, s, emit);
  }
}

// one product C = X*Y (op 0) or inverse C = X^-1 (op 1) in FP64 by one CTA;
// gi: the inverse in global memory (work: negX then Mg, N x N each)
template <bool GI>
__global__ void __launch_bounds__(GI ? 256 : 512, 1) k_fp64_unit(int op, int N, int KC,
                                                     const double2* X, const double2* Y,
                                                     double2* C, double2* negX, double2* Mg,
                                                     int* status) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int NN = N * N;
  const Shared s = fp64_layout(smraw, N, KC, !GI);
  if (op == 0) {
    cta_gemm<13, EPI_STORE>(X, Y, N, KC, s.sX, s.sY, C, nullptr);
    if (threadIdx.x == 0) *status = 0;
  } else {
    for (int e = threadIdx.x; e < NN; e += blockDim.x) negX[e] = make_double2(-X[e].x, -X[e].y);
    __syncthreads();
    int sing;
    if (GI) {                                                   // (0 I - (-X))^-1
      sing = gj_invert_global(negX, make_double2(0.0, 0.0), N, Mg, s);
      gj_store_global(N, Mg, s, C);
    } else {
      sing = gj_invert(negX, make_double2(0.0, 0.0), N, s);
      gj_store(N, s, C);
    }
    if (threadIdx.x == 0) *status = sing ? PT_SINGULAR : 0;
  }
}

size_t smem_bytes(int N, int KC, bool inv_in_smem) {
  const size_t big = inv_in_smem ? (size_t)(N * N > 2 * N * KC ? N * N : 2 * N * KC)
                                 : (size_t)2 * N * KC;
  return big * 16 + (size_t)N * 32 + 16 * GJ_PANEL + 32 * 8 + (size_t)N * 8 + 16;
}

template <int RP>
const void* fp64_kernel(bool gi) {
  return gi ? (const void*)k_decimate_fp64<13, true> : (const void*)k_decimate_fp64<RP, false>;
}

}  // namespace

int decim_fp64_max_n() {
  int n = 8;
  while (smem_bytes(n + 1, (n + 1) / 2, true) <= 227 * 1024) ++n;
  return n;
}

int decim_fp64_large_max_n() { return 32 * GJ_ROWS; }

int fp64_threads_default(int N) { return N <= 48 ? 128 : (N <= 80 ? 256 : 512); }

size_t decim_fp64_ws_matrices(const DecimConfig& cfg) { return cfg.inv_global ? 9 : 8; }

cudaError_t decim_fp64_config(int N, int threads_override, DecimConfig* cfg, bool force_global) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int smem_optin = 0;
  e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const bool gi = force_global || N > decim_fp64_max_n();
  if (gi && N > decim_fp64_large_max_n()) return cudaErrorInvalidValue;
  if (threads_override <= 0) threads_override = tile_value(0, N);
  int T = threads_override > 0 ? threads_override : fp64_threads_default(N);
  int KC = N;
  if (gi) {
    T = 256;                       // 255 registers: a lane keeps 10 rows of a column
    KC = 16;
  } else if (smem_bytes(N, KC, true) > (size_t)smem_optin) {
    KC = (N + 1) / 2;
  }
  while (KC > GJ_PANEL && smem_bytes(N, KC, !gi) > (size_t)smem_optin) --KC;
  if (smem_bytes(N, KC, !gi) > (size_t)smem_optin) return cudaErrorInvalidValue;
  const int rounds = (N * N + T - 1) / T;
  int RP = 13;
  if (!gi && rounds <= 4) RP = 4;
  else if (!gi && rounds <= 8) RP = 8;
  cfg->threads = T;
  cfg->KC = KC;
  cfg->RP = RP;
  cfg->inv_global = gi ? 1 : 0;
  cfg->smem = smem_bytes(N, KC, !gi);
  int occ = 0;
  const void* fn = RP == 4 ? fp64_kernel<4>(gi) : (RP == 8 ? fp64_kernel<8>(gi) : fp64_kernel<13>(gi));
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg->smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, T, cfg->smem);
  if (e != cudaSuccess) return e;
  cfg->ctas_per_sm = occ;
  return cudaSuccess;
}

cudaError_t launch_decimate_fp64(const DecimArgs& a, const DecimConfig& cfg, int grid,
                                 cudaStream_t s) {
  if (cfg.inv_global) {
    k_decimate_fp64<13, true><<<grid, cfg.threads, cfg.smem, s>>>(a);
    return cudaGetLastError();
  }
  switch (cfg.RP) {
    case 4: k_decimate_fp64<4, false><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
    case 8: k_decimate_fp64<8, false><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
    default: k_decimate_fp64<13, false><<<grid, cfg.threads, cfg.smem, s>>>(a); break;
  }
  return cudaGetLastError();
}

size_t batch_ws_matrices(int precision_mixed) { return precision_mixed ? 11 : 9; }

static size_t batch_fp64_smem(int max_n, int max_smem_gj_n, int KC) {
  size_t b = smem_bytes(max_n, KC, false);
  if (max_smem_gj_n > 0) {
    const size_t t = smem_bytes(max_smem_gj_n, KC, true);
    if (t > b) b = t;
  }
  return b;
}

cudaError_t batch_fp64_config(int max_n, size_t extra_smem, int* smem_gj_max, DecimConfig* cfg) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int smem_optin = 0;
  e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (max_n > decim_fp64_large_max_n()) return cudaErrorInvalidValue;
  const int KC = 16;
  // the shared-memory inverse up to the largest Ndim that fits beside the stages
  int g = 0;
  while (g + 1 <= decim_fp64_max_n() && smem_bytes(g + 1, KC, true) + extra_smem + 16 <= (size_t)smem_optin)
    ++g;
  *smem_gj_max = g;
  cfg->threads = 256;
  cfg->KC = KC;
  cfg->RP = 13;
  cfg->inv_global = 1;
  cfg->smem = batch_fp64_smem(max_n, std::min(g, max_n), KC);
  if (cfg->smem + extra_smem + 16 > (size_t)smem_optin) return cudaErrorInvalidValue;
  cfg->ctas_per_sm = 1;
  return cudaSuccess;
}

// the batch kernel's dynamic shared-memory limit raised once per device to the
// opt-in maximum (engines of any size launch it, also from captured graphs)
cudaError_t batch_fp64_prepare() {
  static std::mutex mu;
  static bool done[64];
  int dev = 0, optin = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && done[dev]) return cudaSuccess;
  cudaFuncAttributes fa;
  err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, k_batch_fp64);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_batch_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               optin - (int)fa.sharedSizeBytes);
  if (err == cudaSuccess && dev < 64) done[dev] = true;
  return err;
}

cudaError_t launch_batch_fp64(const BatchArgs& a, const DecimConfig& cfg, int grid, cudaStream_t s) {
  k_batch_fp64<<<grid, cfg.threads, cfg.smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fp64_unit(int op, int N, const double2* X, const double2* Y, double2* C,
                             double2* work, int* status, cudaStream_t st) {
  DecimConfig cfg;
  cudaError_t e = decim_fp64_config(N, 512, &cfg);
  if (e != cudaSuccess) return e;
  const void* fn = cfg.inv_global ? (const void*)k_fp64_unit<true> : (const void*)k_fp64_unit<false>;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
  if (e != cudaSuccess) return e;
  double2* mg = work + (size_t)N * N;
  if (cfg.inv_global)
    k_fp64_unit<true><<<1, cfg.threads, cfg.smem, st>>>(op, N, cfg.KC, X, Y, C, work, mg, status);
  else
    k_fp64_unit<false><<<1, 512, cfg.smem, st>>>(op, N, cfg.KC, X, Y, C, work, mg, status);
  return cudaGetLastError();
}

}  // namespace wtg
