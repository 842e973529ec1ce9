/*
 * wtgpu.h — C ABI of the GB300-native surface Green's-function path for
 * WannierTools (quanshengwu/wannier_tools 2.7.1).
 *
 * The library replaces, behind plain C entry points, the per-(k, omega) hot
 * path of the reference's surface-state drivers:
 *
 *   ham_qlayer2qlayer(k, H00, H01)                src/ham_qlayer2qlayer.f90:1-102
 *   surfgreen_1985(omega, GLL, GRR, GB, H00, H01, ones, eta)
 *                                                  src/surfgreen.f90:7-137
 *   inv / mat_mul (zgesv / zgemm)                  src/inverse.f90:1-58, src/mat_mul.f90:3-27
 *   the k x omega loop bodies of surfstat          src/surfstat.f90:123-197
 *   and of SurfaceDOSkk                            src/fermiarc.f90:206-248
 *
 * Conventions (those of the reference, so a Fortran iso_c_binding interface
 * can pass its arrays unchanged):
 *   - complex arrays are interleaved (re, im) double pairs, i.e. the memory
 *     layout of Fortran complex(dp) / C99 double _Complex;
 *   - matrices are column-major, leading dimension = their row count;
 *   - orbital index lists (top / bottom) are 1-based, as TopOrbitals /
 *     BottomOrbitals in src/module.f90;
 *   - energies are in Hartree (src/readinput.f90:721-724);
 *   - the caller owns every buffer it passes; the library copies in and out.
 *
 * Return codes: WTG_OK (0) on success; > 0 when at least one (k, omega)
 * point carries a warning bit in its status entry (count of such points,
 * saturated at INT32_MAX); < 0 on hard errors.  The library never calls
 * exit/abort.  A textual reason for the last error of the calling thread is
 * available from wtg_last_error.
 *
 * Threading: distinct model handles are independent.  Calls on one handle
 * are serialised by the library (host side) and ordered on the GPU.
 */
#ifndef WTGPU_H
#define WTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* hard error codes */
#define WTG_OK              0
#define WTG_EINVAL         -1   /* bad argument */
#define WTG_ENOMEM         -2   /* device or host allocation failed */
#define WTG_ECUDA          -3   /* CUDA runtime error */
#define WTG_ENODEV         -4   /* no usable CUDA device */
#define WTG_EUNSUPPORTED   -6   /* size / mode not supported by this build */

/* per-point status bits (status[] outputs) */
#define WTG_PT_NOT_CONVERGED 1  /* itermax reached, sum|alpha| > tol (src/surfgreen.f90:86-123) */
#define WTG_PT_SINGULAR      2  /* exact zero pivot; the inverse is replaced by the
                                   identity, as zgesv+inv do (src/inverse.f90:51-55) */
#define WTG_PT_NONFINITE     4  /* a spectral sum is NaN or Inf */
#define WTG_PT_TIMEOUT       8  /* a bounded wait on the tensor cores gave up (mixed form);
                                   the point's outputs are not valid */

/* precision modes */
#define WTG_PREC_FP64  0        /* all-FP64 decimation (FP64 DFMA pipe); Ndim <= 320 (above
                                   119 the inverse runs in global memory) */
#define WTG_PREC_MIXED 1        /* products as BF16 digit splits on the tcgen05 tensor cores
                                   (49-bit rounded operands in balanced 7-bit digits, FP32
                                   accumulation exact per slice order up to 6, int64
                                   recombination); in-loop inverses FP32 Gauss-Jordan +
                                   Newton-Schulz refinement on those products; the final
                                   GLL / GRR / GB inverses and the convergence norm in FP64;
                                   Ndim <= 320 */

typedef struct wtg_model* wtg_model_t;

/*
 * Upload a principal-layer tight-binding model and keep it resident on the
 * device.  Replaces the module-global state read by ham_qlayer2qlayer
 * (HmnR_surfacecell / irvec_surfacecell / ndegen_surfacecell produced by
 * get_hmnr_cell, src/readHmnR.f90:578-766; Np and ijmax, src/module.f90:503-507).
 *
 *   nw      Num_wann
 *   nrpts   nrpts_surfacecell
 *   irvec   int[3*nrpts], column-major (3, nrpts) like irvec_surfacecell
 *   hmnr    complex[nw*nw*nrpts], column-major (nw, nw, nrpts), Hartree
 *   ndegen  int[nrpts] (NULL = all ones); each term is divided by it as at
 *           src/ham_qlayer2qlayer.f90:60
 *   np      number of principal layers Np (Ndim = nw*np)
 *   ijmax   layer cut-off (reference default 10, src/module.f90:505)
 */
int wtg_model_create(int nw, int nrpts, const int* irvec, const double* hmnr,
                     const int* ndegen, int np, int ijmax, wtg_model_t* out);

/* Release a model and all device memory it holds. */
int wtg_model_destroy(wtg_model_t model);

/*
 * Phonon models: switch the model's Fourier sum to ham_qlayer2qlayer_LOTO
 * (src/ham_qlayer2qlayer.f90:312-476, used by SurfaceDOSkk when
 * LOTO_correction is set, src/fermiarc.f90:215-216): the non-analytic term
 *   nac(i,j) = kZ(jj,qq) kZ(ii,pp) * 4*3.1415926/(k.D.k * V) * VASPToTHZ/0.529177
 *              / sqrt(M(ii) M(jj)),   kZ(ii,pp) = k1 Z(ii,1,pp) + k2 Z(ii,2,pp),
 * is added to every H(R) before the sum, and k is moved to (1e-4, 1e-4) when
 * |k|^2 <= 1e-4 (all with the reference's constants).  Applies to
 * wtg_ham_qlayer2qlayer and the spectrum entry points of this model.
 *   born[natoms*3*3]  Born_Charge(natoms, 3, 3), column-major
 *   diele[9]          Diele_Tensor(3, 3), column-major
 *   masses[natoms]    Atom_Mass;  cell_volume  Origin_cell%CellVolume
 * Num_wann must be 3*natoms.  natoms = 0 switches the correction off.
 * (The overlap variant s_qlayer2qlayer, src/ham_qlayer2qlayer.f90:104-205, is
 * wtg_ham_qlayer2qlayer of a model created from SmnR instead of HmnR.)
 */
int wtg_model_set_loto(wtg_model_t model, int natoms, const double* born, const double* diele,
                       const double* masses, double cell_volume);

/* Ndim = nw*np of a model (or < 0 on a bad handle). */
int wtg_model_ndim(wtg_model_t model);

/*
 * H00/H01 for one in-plane k (fractional surface-BZ coordinates, k[2]).
 * Replaces ham_qlayer2qlayer(k, H00, H01), src/ham_qlayer2qlayer.f90:1-102.
 * h00, h01: complex[Ndim*Ndim] column-major (host buffers).
 */
int wtg_ham_qlayer2qlayer(wtg_model_t model, const double* k, double* h00, double* h01);

/*
 * One Lopez-Sancho decimation on the GPU with full outputs.
 * Replaces surfgreen_1985(omega, GLL, GRR, GB, H00, H01, ones, eta),
 * src/surfgreen.f90:7-137 (the identity "ones" argument is implicit).
 *   tol      convergence threshold on sum_ij |alpha_ij| (reference: 1e-16
 *            single-precision literal, src/surfgreen.f90:42)
 *   itermax  iteration cap (reference: 100, src/surfgreen.f90:39)
 * h00/h01 in, gll/grr/gb out: complex[ndim*ndim] column-major host buffers.
 * iters / status (may be NULL): iterations executed and WTG_PT_* bits.
 */
int wtg_surfgreen_1985(int ndim, double omega, double eta, const double* h00,
                       const double* h01, double tol, int itermax,
                       double* gll, double* grr, double* gb,
                       int* iters, int* status);

/*
 * One complex product C = A*B, replacing mat_mul (ZGEMM, src/mat_mul.f90:3-27),
 * and one inverse A := A^-1 in place, replacing inv (zgesv with an identity
 * right-hand side, src/inverse.f90:1-58), on the GPU with the decimation's own
 * device code in either precision.  n x n column-major complex host buffers.
 * wtg_inv returns 1 (and status PT_SINGULAR) on an exact zero pivot, leaving
 * the identity as the reference's inv does.
 */
int wtg_mat_mul(int n, const double* a, const double* b, double* c, int precision);
int wtg_inv(int n, double* a, int precision, int* status);

/*
 * Batched surface spectrum over an explicit k list x omega list: for every
 * (k, omega) the Fourier sum of ham_qlayer2qlayer, one surfgreen_1985
 * decimation, and the spectral sums
 *   dos_l(ik,j)    = - sum_{io in top}  Im GLL(io,io)            * scale
 *   dos_r(ik,j)    = - sum_{io in bot}  Im GRR(Ndim-nw+io, same) * scale
 *   dos_bulk(ik,j) = - sum_{i=1..Ndim}  Im GB(i,i)               * scale
 * i.e. the loop bodies of surfstat (scale = 1, src/surfstat.f90:123-160)
 * and SurfaceDOSkk (scale = 1/pi applied per term, src/fermiarc.f90:206-248).
 *
 *   k        double[nk*2], column-major (nk, 2) like k2_path (src/module.f90)
 *   omega    double[nomega], Hartree
 *   eta      broadening, Hartree (surfstat: 3*(wmax-wmin)/nomega,
 *            src/surfstat.f90:84; SurfaceDOSkk: Fermi_broadening,
 *            src/fermiarc.f90:194)
 *   top/bot  1-based orbital lists (TopOrbitals / BottomOrbitals)
 *   divide_by_pi  0 for surfstat, 1 for SurfaceDOSkk
 *   precision     WTG_PREC_FP64 or WTG_PREC_MIXED
 *   dos_l, dos_r, dos_bulk  double[nk*nomega], column-major (nk, nomega)
 *   iters (int32) / status (uint8) [nk*nomega], optional (NULL)
 * All pointers are host pointers.
 */
int wtg_surface_spectrum(wtg_model_t model, int nk, const double* k,
                         int nomega, const double* omega, double eta,
                         double tol, int itermax,
                         int ntop, const int* top, int nbot, const int* bot,
                         int divide_by_pi, int precision,
                         double* dos_l, double* dos_r, double* dos_bulk,
                         int32_t* iters, uint8_t* status);

/*
 * wtg_surface_spectrum plus the spin-resolved surface spectra
 * sx/sy/sz_l = -sum Im (GLL sigma_{x,y,z})(io,io) and sx/sy/sz_r from GRR, with
 * the Pauli matrices of src/surfstat.f90:103-114 (|up..up down..down> basis
 * per Num_wann block).  Only the entries of G that sigma*G needs are read,
 * replacing the six full products of the reference.
 *   arc_mode 0: surfstat (src/surfstat.f90:162-192): no 1/pi, and the right
 *               spin sums run over the TOP orbital list (as the reference does);
 *   arc_mode 1: SurfaceDOSkk spin texture (src/fermiarc.f90:250-330): every
 *               term divided by pi, right sums over Ndim - nw + bottom orbitals.
 *   spin_out   double[6 * nk * nomega]: sx_l, sy_l, sz_l, sx_r, sy_r, sz_r, each
 *              (nk, nomega) column-major, host buffer.
 */
int wtg_surface_spectrum_spin(wtg_model_t model, int nk, const double* k, int nomega,
                              const double* omega, double eta, double tol, int itermax,
                              int ntop, const int* top, int nbot, const int* bot, int arc_mode,
                              int precision, double* dos_l, double* dos_r, double* dos_bulk,
                              double* spin_out, int32_t* iters, uint8_t* status);

/*
 * Same computation with every array already on the device, enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) without a host
 * synchronisation.  top/bot are host arrays (they are small and copied
 * into the launch).  Returns after enqueueing; per-point status is in
 * `status` once the stream reaches that point.
 */
int wtg_surface_spectrum_device(wtg_model_t model, int nk, const double* d_k,
                                int nomega, const double* d_omega, double eta,
                                double tol, int itermax,
                                int ntop, const int* top, int nbot, const int* bot,
                                int divide_by_pi, int precision,
                                double* d_dos_l, double* d_dos_r, double* d_dos_bulk,
                                int32_t* d_iters, uint8_t* d_status, void* stream);

/*
 * Tracing (no reference counterpart beyond its wall-clock timers,
 * src/wt_aux.f90:6-37 and the time_q / time_ss split of
 * src/fermiarc.f90:214-232).  wtg_model_profile(m, 1) resets the counters
 * and records CUDA events around every Fourier-sum and decimation launch of
 * the handle; wtg_model_profile_read synchronises them and returns the
 * summed device milliseconds of each phase, the number of this library's
 * kernels the handle has launched since the reset, and the number of
 * decimation launches.
 */
int wtg_model_profile(wtg_model_t model, int enable);
int wtg_model_profile_read(wtg_model_t model, double* fourier_ms, double* decim_ms,
                           long long* launches, int* decim_launches);

/* FP64 (DFMA) throughput of the current device in TFLOP/s: the roofline
   denominator of the FP64 path, measured with a short throughput kernel.
   No counterpart in the reference. */
int wtg_probe_fp64_peak(double* tflops);
/* FP64 tensor-core (mma.sync m8n8k4 .f64, DMMA) throughput of the current
   device in TFLOP/s, measured the same way: the rate a zgemm on the FP64
   tensor path (src/mat_mul.f90:23 through a tensor-core BLAS) could reach. */
int wtg_probe_dmma_peak(double* tflops);

/*
 * Allocation-free batched decimation.  No counterpart in the reference: it
 * exists for callers that cannot let the library call cudaMalloc -- a host
 * whose device memory is owned by another allocator (a caching pool that has
 * reserved the free HBM), or a latency-critical loop where cudaMalloc/cudaFree
 * would synchronise the device.  Runs the FP64 decimation + spectral sums of
 * wtg_surface_spectrum_device on H00/H01 the caller already holds on the
 * device, with all scratch in a fixed 64 MiB device array inside the library
 * (held on every GPU that loads it, until exit).  Nothing is allocated.
 *
 *   ndim, nw   Ndim and Num_wann (ndim a multiple of nw; ndim <= 119, the kernel limit)
 *   d_h        device complex[nk][2][ndim*ndim]: per k, H00 then H01, column-major
 *   d_omega    device double[nomega]; outputs device arrays (nk, nomega) column-major
 *   top/bot    host 1-based orbital lists; stream a cudaStream_t (NULL = default)
 * Sizes beyond the kernel limit or the fixed scratch return WTG_EUNSUPPORTED.
 * The first call on a device looks up the scratch address (make it before
 * any stream capture).  Calls share the scratch: calls that overlap on the
 * GPU race; the caller orders them (e.g. one stream).
 */
int wtg_surfgreen_batch_noalloc(int ndim, int nw, int nk, const double* d_h, int nomega,
                                const double* d_omega, double eta, double tol, int itermax,
                                int ntop, const int* top, int nbot, const int* bot,
                                int divide_by_pi, double* d_dos_l, double* d_dos_r,
                                double* d_dos_bulk, int32_t* d_iters, uint8_t* d_status,
                                void* stream);

/* Copy the calling thread's last error message into buf (NUL-terminated). */
int wtg_last_error(char* buf, int len);

/* Describe the device the library runs on ("name, SMs, cc") into buf. */
int wtg_device_info(char* buf, int len);

/*
 * Joint density of states along a k path, per omega: the loop of
 * src/surfstat.f90:889-905 (surfstat's JDOS).  dos(nk, nomega) column-major in
 * (dos_l, dos_r or their *_only forms), jdos(nk, nomega) out:
 *   jdos(iq, j) = sum_{ik1} dos(ik1, j) * dos(ik1 + iq - Nh, j),  Nh = (nk-1)/2,
 * over the reference's ik1 range.  Sums in the reference's order, unfused.
 */
int wtg_jdos_kpath(int nk, int nomega, const double* dos, double* jdos);

/*
 * Quasi-particle interference on a k plane: the JDOS loops of
 * src/fermiarc.f90:497-545 (SlabQPI_kplane_calc).  chans holds nchan arrays
 * (nkx, nky) column-major back to back: 1 channel (dos_l_only or dos_r_only)
 * gives jdos, 4 channels (dos_only, sx, sy, sz) give the spin form jsdos.
 *   out(q) = scale * sum_{ik2, ik1} sum_c in_c(ik1, ik2) * in_c(k1q, k2q),
 *   k1q = mod(ik1 + iq1 - 2, p1) + 1, k2q = mod(ik2 + iq2 - 2, p2) + 1,
 * q = (iq1, iq2) in the reference's ikp order (second index fastest).  The
 * reference's periods are p1 = nkx-1, p2 = nky-1 for jdos and Nk1-1, Nk2-1 for
 * jsdos; its jdos is then divided by nkx*nky (scale = 1/(nkx*nky)), jsdos not.
 */
int wtg_jdos_kplane(int nkx, int nky, int p1, int p2, int nchan, const double* chans,
                    double scale, double* jdos);

/*
 * Uneven batches: (k, omega, eta) points of several resident models, of
 * different Ndim, solved in ONE persistent kernel launch.  The CTAs take the
 * points in order of estimated cost (Ndim^3 x an iteration estimate growing as
 * eta shrinks, largest first); each point runs its own Fourier sum (as
 * wtg_ham_qlayer2qlayer) and decimation (as wtg_surface_spectrum) and stops at
 * its own convergence, so one result never depends on the other points of the
 * batch.  No counterpart in the reference, which solves one (k, omega) at a
 * time (src/surfstat.f90:123-160, src/fermiarc.f90:206-248); the per-point
 * arithmetic is the same as wtg_surface_spectrum's.
 *
 * An engine holds the device tables of a fixed model set, a workspace sized for
 * the largest Ndim, pinned staging and its own stream; it runs one batch at a
 * time and several engines run concurrently (a serving loop keeps one per
 * in-flight batch).
 *   models[nmodels]      handles of one device (they must outlive the engine)
 *   precision            WTG_PREC_FP64 or WTG_PREC_MIXED
 *   max_points           largest npts of one run
 *   ntop[nmodels], top   per-model TopOrbitals lists, concatenated (1-based)
 *   nbot[nmodels], bot   per-model BottomOrbitals lists, concatenated
 */
typedef struct wtg_engine* wtg_engine_t;

int wtg_engine_create(int nmodels, const wtg_model_t* models, int precision, int max_points,
                      const int* ntop, const int* top, const int* nbot, const int* bot,
                      wtg_engine_t* engine);
int wtg_engine_destroy(wtg_engine_t engine);
/* Device bytes the engine holds, its max_points and the kernels it launched (any may be NULL). */
int wtg_engine_info(wtg_engine_t engine, long long* device_bytes, int* max_points,
                    long long* launches);
/*
 * One batch (host buffers, synchronous):
 *   point_model[npts]          index into the engine's models
 *   k[npts*2]                  column-major (npts, 2) fractional in-plane k
 *   omega[npts], eta[npts]     Hartree
 *   tol, itermax, divide_by_pi as wtg_surface_spectrum
 *   dos_l/dos_r/dos_bulk[npts] out; iters[npts], status[npts] out (may be NULL)
 * Returns the number of flagged points (>= 0) or a negative error code.
 */
int wtg_engine_run(wtg_engine_t engine, int npts, const int* point_model, const double* k,
                   const double* omega, const double* eta, double tol, int itermax,
                   int divide_by_pi, double* dos_l, double* dos_r, double* dos_bulk, int* iters,
                   unsigned char* status);
/*
 * CUDA graphs (on by default; wtg_engine_set_graphs(engine, 0) turns them off
 * for that engine): a run's copy-in, counter reset, batch kernel and
 * copy-out are captured once per staging capacity (the powers of two from 64 up
 * to max_points) and replayed with one cudaGraphLaunch; the point count and the
 * run's scalars travel in the staged header.  Results are bit-identical with
 * graphs on and off.  graphs = captured capacities, graph_launches = replays.
 */
int wtg_engine_set_graphs(wtg_engine_t engine, int on);
int wtg_engine_graph_info(wtg_engine_t engine, int* graphs, long long* graph_launches);

/*
 * Tile table (the autotuner's output, wannier_tools_gb300/autotune.py): the
 * launch shape the kernels use at a given Ndim.
 *   WTG_PREC_FP64   value = threads per CTA of the per-model FP64 kernel, 128, 256
 *                   or 512 (Ndim above the shared-memory inverse always uses 256)
 *   WTG_PREC_MIXED  value = output-column pass width of the split-BF16 products, a
 *                   multiple of 8 up to 40
 * value 0 restores the built-in choice.  Results do not depend on the tile beyond
 * the order of the convergence norm's block sum (every output element is summed in
 * the same order; spectra agree to 1e-12).  Set tiles before creating engines
 * (an engine keeps the widths it was created with); wtg_tile_get returns the
 * value in use and the built-in one.  No counterpart in the reference.
 */
int wtg_tile_set(int precision, int ndim, int value);
int wtg_tile_get(int precision, int ndim, int* value, int* builtin);

/* One-shot: create an engine for these models and points, run, destroy. */
int wtg_batch_spectrum(int nmodels, const wtg_model_t* models, int npts, const int* point_model,
                       const double* k, const double* omega, const double* eta, double tol,
                       int itermax, const int* ntop, const int* top, const int* nbot,
                       const int* bot, int divide_by_pi, int precision, double* dos_l,
                       double* dos_r, double* dos_bulk, int* iters, unsigned char* status);

/*
 * Test-only switches, process-wide (no counterpart in the reference).  They
 * exist so that a test can reach code paths that normal inputs do not; a
 * production caller never sets them.  value 0 restores normal operation.
 *   WTG_TEST_FP64_GLOBAL_INVERSE  non-zero: the per-model FP64 kernel inverts in
 *                                 global memory at every Ndim (the variant that
 *                                 normally runs above Ndim 119; both agree bit
 *                                 for bit)
 *   WTG_TEST_MIXED_SPIN_LIMIT     > 0: the mixed kernels' pipeline waits on the
 *                                 tensor cores give up after this many
 *                                 non-blocking polls instead of the built-in
 *                                 bound, so that a test can make them run out:
 *                                 the points get WTG_PT_TIMEOUT and the call
 *                                 returns normally.  Read when a launch is
 *                                 made (an engine's captured graphs keep the
 *                                 value they were captured with).
 * Returns WTG_OK, or WTG_EINVAL for an unknown option or a negative value.
 */
#define WTG_TEST_FP64_GLOBAL_INVERSE 1
#define WTG_TEST_MIXED_SPIN_LIMIT    2
#define WTG_TEST_OPTIONS             3
int wtg_test_option(int option, int value);

#ifdef __cplusplus
}
#endif

#endif /* WTGPU_H */
