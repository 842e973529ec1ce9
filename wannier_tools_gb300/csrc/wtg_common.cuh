// Shared declarations of the GB300 (sm_103a) surface Green's-function kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wtg {

// The reference's truncated pi literal (src/module.f90:719); the Fourier
// phases use it exactly as ham_qlayer2qlayer does (src/ham_qlayer2qlayer.f90:56).
constexpr double PI_REF = 3.14159265358979;

constexpr int MAX_ORB = 1024;     // longest top / bottom orbital list per launch

// per-point status bits (mirrors WTG_PT_* of include/wtgpu.h)
constexpr int PT_NOT_CONVERGED = 1;
constexpr int PT_SINGULAR = 2;
constexpr int PT_NONFINITE = 4;
constexpr int PT_TIMEOUT_BIT = 8;

// Spin-resolved sums -Im (G sigma_a)(io, io) over an orbital list, with the
// Pauli matrices of src/surfstat.f90:103-114 (|up..up down..down> basis per
// Num_wann block): (G sx)(io,io) = G(io,p), (G sy)(io,io) = +-i G(io,p),
// (G sz)(io,io) = +-G(io,io), p the spin partner of io.  `g(i, j)` returns G.
template <class GetG>
__device__ void spin_sums(GetG g, int nw, int n_list, const int* list, int offset,
                          int divide_by_pi, double& sx, double& sy, double& sz) {
  const int nwh = nw / 2;
  for (int q = 0; q < n_list; ++q) {
    const int io = offset + list[q] - 1;
    const int jl = io % nw;
    int partner = -1;
    double sgn = 0.0;
    if (jl < nwh) {
      partner = io + nwh;
      sgn = 1.0;
    } else if (jl < 2 * nwh) {
      partner = io - nwh;
      sgn = -1.0;
    }
    double vx = 0.0, vy = 0.0, vz = 0.0;
    if (partner >= 0) {
      const double2 gp = g(io, partner);
      const double2 gd = g(io, io);
      vx = gp.y;
      vy = sgn * gp.x;
      vz = sgn * gd.y;
    }
    if (divide_by_pi) {
      sx = sx - vx / PI_REF;
      sy = sy - vy / PI_REF;
      sz = sz - vz / PI_REF;
    } else {
      sx = sx - vx;
      sy = sy - vy;
      sz = sz - vz;
    }
  }
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// acc += a*b with four fused multiply-adds (one complex multiply-accumulate)
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

// ---------------------------------------------------------------------------
// Principal-layer Fourier sum (ham_qlayer2qlayer)
// ---------------------------------------------------------------------------
struct FourierArgs {
  const double* k;        // (nk_total, 2) column-major, device
  int nk_total;           // leading dimension of k
  int k0, kc;             // k chunk [k0, k0+kc)
  const double2* rab;     // [nRu] (ia, ib) of the used R vectors, device
  const double2* hr;      // [nRu][nw*nw] column-major blocks, sorted by R3, device
  const int* icoff;       // [nic+1] offsets of each R3 group in hr, device
  int ic_lo, nic;         // R3 = ic_lo + group index
  int nRu, nw, np, ijmax;
  double2* phase;         // [kc][nRu] scratch
  double2* h;             // [kc][2][N*N] output: H00 then H01, column-major
  // phonon LO-TO correction (ham_qlayer2qlayer_LOTO); loto = 0: plain sum
  int loto;
  const double* wr;       // [nRu] 1 / ndegen of the used R vectors
  const double* lz;       // [natoms][2][3] Born charges Z(atom, k direction, cartesian)
  const double* lmass;    // [natoms] atomic masses
  double ld[4];           // in-plane dielectric tensor D(1,1), D(1,2), D(2,1), D(2,2)
  double lvol;            // cell volume
};
void launch_fourier(const FourierArgs& a, cudaStream_t s);

// ---------------------------------------------------------------------------
// Lopez-Sancho decimation, all FP64 (surfgreen_1985)
// ---------------------------------------------------------------------------
struct DecimArgs {
  int N, nw;                  // Ndim, Num_wann
  int nomega;                 // omega points per k
  int n_inst;                 // instances in this launch: (k chunk) x nomega, omega fastest
  const double2* h;           // [kc][2][N*N] H00/H01 of the chunk
  const double* omega;        // [nomega]
  double eta, tol;
  int itermax;
  int divide_by_pi;
  int nk_total, k_offset;     // output index = (k_offset + ik) + iw * nk_total
  double* dos_l;
  double* dos_r;
  double* dos_bulk;
  int32_t* iters;             // may be null
  uint8_t* status;            // may be null
  double* spin[6];            // optional sx_l, sy_l, sz_l, sx_r, sy_r, sz_r (null = skip)
  int spin_right_bottom;      // 0: right spin over the top list (surfstat), 1: over Ndim-nw+bottom
  double2* gll;               // optional full outputs [n_inst][N*N] (null = skip)
  double2* grr;
  double2* gb;
  double2* ws;                // [grid][8 or 9][N*N] workspace (decim_fp64_ws_matrices)
  int* counter;               // work counter, zero at launch
  int KC;                     // GEMM k-chunk staged in shared memory
  int w0;                     // mixed: output-column pass width (tile table; 0 = built-in)
  int ntop, nbot;
  int top[MAX_ORB];           // 1-based orbital lists (TopOrbitals / BottomOrbitals)
  int bot[MAX_ORB];
};

// Uneven batch (several models, one launch): per-model tables, device-resident
struct BatchModel {
  int N, nw, np;
  int nRu, nic, ic_lo;        // Fourier tables as FourierArgs
  const double2* hr;
  const double2* rab;
  const int* icoff;
  int ntop, nbot;
  const int* top;             // 1-based orbital lists, device
  const int* bot;
  int w0;                     // mixed: output-column pass width (tile table; 0 = built-in)
};

// a run's scalars, staged with its points: a captured run reads them from device memory
struct BatchRunHeader {
  int npts, itermax, divide_by_pi, pad;
  double tol, pad2;
};

struct BatchArgs {
  int npts;                   // points, and the column stride of k (a staging capacity in graphs)
  const BatchRunHeader* run;  // if set, npts / tol / itermax / divide_by_pi are read here
  const BatchModel* models;   // device
  const int* pmodel;          // [npts] model of each point
  const int* order;           // [npts] points in launch order (largest estimated cost first)
  const double* k;            // (npts, 2) column-major
  const double* omega;        // [npts]
  const double* eta;          // [npts]
  double tol;
  int itermax;
  int divide_by_pi;
  double* dos_l;              // [npts]
  double* dos_r;
  double* dos_bulk;
  int32_t* iters;             // may be null
  uint8_t* status;            // may be null
  double2* ws;                // [grid][ws_stride]
  size_t ws_stride;           // double2 per CTA
  int* counter;               // zero at launch
  int KC;                     // FP64 GEMM k-chunk
  int smem_gj_max;            // FP64: largest Ndim whose inverse runs in shared memory
  int wb;                     // mixed: B-plane width of the shared-memory layout
  size_t ph_off;              // byte offset of the phase table (max nRu double2) in shared memory
};

struct DecimConfig {
  int threads;
  int KC;
  int RP;                     // register rows per pass in the GEMM (template)
  size_t smem;                // dynamic shared memory per CTA
  int ctas_per_sm;
  int inv_global = 0;         // FP64: 1 = the inverse runs in global memory (large Ndim)
  int w0 = 0;                 // mixed: output-column pass width
};

// Built-in choices and limits of the tunable shapes, and the mixed form's pass
// width for Ndim N after the tile table.
int fp64_threads_default(int N);
int mixed_w0_default(int N);
int mixed_w0_max(int N);
int batch_mixed_w0(int N);
// Raise the batch kernels' dynamic shared-memory limit to the device maximum (once).
cudaError_t batch_fp64_prepare();
cudaError_t batch_mixed_prepare();

// Tile table: per-Ndim launch shapes chosen by the autotuner (wtg_tile_set).
// precision 0 (FP64): threads per CTA of the per-model kernel (128, 256 or 512);
// precision 1 (mixed): output-column pass width (a multiple of 8).  0 = built-in choice.
constexpr int TILE_MAX_N = 4096;
int tile_value(int precision, int N);
void tile_store(int precision, int N, int value);

// Largest Ndim the shared-memory Gauss-Jordan kernel takes.
int decim_fp64_max_n();
// Largest Ndim of the FP64 kernel whose inverse runs in global memory (above decim_fp64_max_n).
int decim_fp64_large_max_n();
// N x N complex workspace matrices per CTA of the FP64 kernel in this configuration (8, or 9
// when the inverse runs in global memory).
size_t decim_fp64_ws_matrices(const DecimConfig& cfg);
// Launch shape for a given N on the current device (threads override: 0 = auto).  The inverse
// runs in global memory above decim_fp64_max_n(), or at any N with force_global (the two
// variants agree bit for bit).
cudaError_t decim_fp64_config(int N, int threads_override, DecimConfig* cfg,
                              bool force_global = false);
cudaError_t launch_decimate_fp64(const DecimArgs& a, const DecimConfig& cfg, int grid,
                                 cudaStream_t s);

// Mixed-precision (split BF16 on tcgen05) decimation; same arguments, workspace of
// decim_mixed_ws_matrices() N x N complex matrices per CTA.
int decim_mixed_max_n();
size_t decim_mixed_ws_matrices();
cudaError_t decim_mixed_config(int N, DecimConfig* cfg);
cudaError_t launch_decimate_mixed(const DecimArgs& a, const DecimConfig& cfg, int grid,
                                  cudaStream_t s);

// Uneven batch launch shapes and launches.  The configs' shared memory excludes the
// phase table, which the caller appends at BatchArgs::ph_off and adds to cfg.smem before
// launching; extra_smem reserves room for it.
cudaError_t batch_fp64_config(int max_n, size_t extra_smem, int* smem_gj_max, DecimConfig* cfg);
cudaError_t launch_batch_fp64(const BatchArgs& a, const DecimConfig& cfg, int grid, cudaStream_t s);
cudaError_t batch_mixed_config(int max_n, int* wb, DecimConfig* cfg);
cudaError_t launch_batch_mixed(const BatchArgs& a, const DecimConfig& cfg, int grid, cudaStream_t s);
// Workspace matrices per CTA of the batch kernels.
size_t batch_ws_matrices(int precision_mixed);

// One product (op 0: C = X*Y) or inverse (op 1: C = X^-1) by a single CTA.
// Mixed: ws holds 5 N x N complex matrices; FP64: work holds two.
cudaError_t launch_mixed_unit(int op, int N, const double2* X, const double2* Y, double2* C,
                              double2* ws, int ns, int* status, cudaStream_t s);
cudaError_t launch_fp64_unit(int op, int N, const double2* X, const double2* Y, double2* C,
                             double2* work, int* status, cudaStream_t s);

// Sets the calling thread's message returned by wtg_last_error.
void set_last_error(const char* msg);

// Process-wide test switches (wtg_test_option; WTG_TEST_* of include/wtgpu.h); 0 = off.
int test_option(int option);
void set_test_option(int option, int value);

}  // namespace wtg
