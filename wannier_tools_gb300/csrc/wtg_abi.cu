// C ABI of the surface Green's-function path (declarations: include/wtgpu.h).
//
// Host side: validation, model upload (HmnR resident in HBM, grouped by R3),
// device buffers, k chunking, launch configuration, host<->device staging for
// the host-pointer entry points.  No CPU computation of the path happens here:
// every H00/H01, inverse, product and spectral sum is computed by the kernels
// in wtg_fourier.cu / wtg_decimate.cu.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wtgpu.h"
#include "wtg_common.cuh"
#include "wtg_plan.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return WTG_ECUDA;
}

#define WTG_CK(call)                                  \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// grow-only device buffer
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Upper bound on the H00/H01 buffer of one k chunk.
constexpr size_t H_CHUNK_BYTES = (size_t)8 << 30;

}  // namespace

namespace wtg {
void set_last_error(const char* msg) { g_err = msg ? msg : ""; }

namespace {
std::atomic<int> g_test_opts[WTG_TEST_OPTIONS];
}  // namespace

int test_option(int option) {
  return option >= 0 && option < WTG_TEST_OPTIONS ? g_test_opts[option].load() : 0;
}

void set_test_option(int option, int value) {
  if (option >= 0 && option < WTG_TEST_OPTIONS) g_test_opts[option].store(value);
}
}  // namespace wtg

struct wtg_model {
  int device = 0;
  int nw = 0, nR = 0, np = 0, ijmax = 0, N = 0;
  int ic_lo = 0, nic = 0, nRu = 0;
  double2* d_hr = nullptr;
  double2* d_rab = nullptr;
  int* d_icoff = nullptr;
  double* d_wr = nullptr;              // 1 / ndegen of the used R vectors
  // phonon LO-TO correction (wtg_model_set_loto)
  int loto = 0;
  DevBuf d_lz, d_lm;
  double ld[4] = {0, 0, 0, 0};
  double lvol = 0.0;
  DevBuf phase, h, ws, counter;
  // staging for the host-pointer entry points
  DevBuf k_in, w_in, out_dos, out_it, out_st;
  cudaStream_t stream = nullptr;       // stream of the host-pointer entry points
  cudaEvent_t done = nullptr;          // orders calls on this handle on the GPU
  std::mutex mu;
  // tracing: CUDA events around each Fourier / decimation launch
  bool profile = false;
  long long launches = 0;              // kernels of this library launched by the handle
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<size_t, size_t>> fourier_ev, decim_ev;
  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e = nullptr;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
};

namespace {

void set_loto_args(const wtg_model* m, wtg::FourierArgs& f) {
  f.loto = m->loto;
  f.wr = m->d_wr;
  f.lz = (const double*)m->d_lz.p;
  f.lmass = (const double*)m->d_lm.p;
  for (int i = 0; i < 4; ++i) f.ld[i] = m->ld[i];
  f.lvol = m->lvol;
}

int run_spectrum(wtg_model* m, int nk, const double* d_k, int nomega, const double* d_omega,
                 double eta, double tol, int itermax, int ntop, const int* top, int nbot,
                 const int* bot, int divide_by_pi, int precision, double* d_dl, double* d_dr,
                 double* d_db, int32_t* d_it, uint8_t* d_st, cudaStream_t s,
                 double* const* d_spin = nullptr, int spin_right_bottom = 0) {
  const int N = m->N;
  const bool mixed = precision == WTG_PREC_MIXED;
  const int nmax = mixed ? wtg::decim_mixed_max_n() : wtg::decim_fp64_large_max_n();
  if (N > nmax)
    return fail(WTG_EUNSUPPORTED, "Ndim " + std::to_string(N) + " exceeds the " +
                                      (mixed ? "mixed" : "FP64") + " kernel limit " +
                                      std::to_string(nmax));
  wtg::DecimConfig cfg;
  if (mixed) {
    WTG_CK(wtg::decim_mixed_config(N, &cfg));
  } else {
    // the large-Ndim (global-memory inverse) variant at any Ndim when a test asks for it
    WTG_CK(wtg::decim_fp64_config(N, 0, &cfg,
                                  wtg::test_option(WTG_TEST_FP64_GLOBAL_INVERSE) != 0));
  }
  const size_t ws_mats = mixed ? wtg::decim_mixed_ws_matrices() : wtg::decim_fp64_ws_matrices(cfg);
  if (cfg.ctas_per_sm < 1) return fail(WTG_EUNSUPPORTED, "decimation kernel does not fit an SM");
  int nsm = 0;
  WTG_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, m->device));

  const size_t hk = sizeof(double2) * 2 * (size_t)N * N;   // H00+H01 per k
  const int grid_max = cfg.ctas_per_sm * nsm;
  const int kchunk = wtg::spectrum_kchunk(nk, nomega, N, grid_max, H_CHUNK_BYTES);
  if (kchunk < 1)
    return fail(WTG_EINVAL, "nomega " + std::to_string(nomega) + " exceeds " +
                                std::to_string(INT_MAX - grid_max) + " (instances are 32-bit)");
  const long long max_inst = (long long)kchunk * nomega;
  const int grid = (int)std::min<long long>(grid_max, max_inst);

  WTG_CK(m->phase.ensure(sizeof(double2) * (size_t)kchunk * std::max(1, m->nRu)));
  WTG_CK(m->h.ensure(hk * kchunk));
  WTG_CK(m->ws.ensure(sizeof(double2) * ws_mats * (size_t)N * N * grid));
  WTG_CK(m->counter.ensure(sizeof(int) * 64));

  WTG_CK(cudaStreamWaitEvent(s, m->done, 0));
  wtg::DecimArgs a;
  memset(&a, 0, sizeof(a));
  a.N = N;
  a.nw = m->nw;
  a.nomega = nomega;
  a.omega = d_omega;
  a.eta = eta;
  a.tol = tol;
  a.itermax = itermax;
  a.divide_by_pi = divide_by_pi;
  a.nk_total = nk;
  a.dos_l = d_dl;
  a.dos_r = d_dr;
  a.dos_bulk = d_db;
  a.iters = d_it;
  a.status = d_st;
  a.ws = (double2*)m->ws.p;
  a.KC = cfg.KC;
  a.w0 = cfg.w0;
  a.ntop = ntop;
  a.nbot = nbot;
  for (int q = 0; q < ntop; ++q) a.top[q] = top[q];
  for (int q = 0; q < nbot; ++q) a.bot[q] = bot[q];
  if (d_spin)
    for (int c = 0; c < 6; ++c) a.spin[c] = d_spin[c];
  a.spin_right_bottom = spin_right_bottom;
  int chunk_id = 0;
  for (int k0 = 0; k0 < nk; k0 += kchunk, ++chunk_id) {
    const int kc = std::min(kchunk, nk - k0);
    wtg::FourierArgs f;
    f.k = d_k;
    f.nk_total = nk;
    f.k0 = k0;
    f.kc = kc;
    f.rab = m->d_rab;
    set_loto_args(m, f);
    f.hr = m->d_hr;
    f.icoff = m->d_icoff;
    f.ic_lo = m->ic_lo;
    f.nic = m->nic;
    f.nRu = m->nRu;
    f.nw = m->nw;
    f.np = m->np;
    f.ijmax = m->ijmax;
    f.phase = (double2*)m->phase.p;
    f.h = (double2*)m->h.p;
    const size_t fe0 = m->ev_used;
    if (m->profile) WTG_CK(cudaEventRecord(m->next_event(), s));
    wtg::launch_fourier(f, s);
    WTG_CK(cudaGetLastError());
    m->launches += (kc > 0 && m->nRu > 0 ? 1 : 0) + (m->nic > 0 ? 1 : 0);
    if (m->profile) {
      WTG_CK(cudaEventRecord(m->next_event(), s));
      m->fourier_ev.push_back({fe0, fe0 + 1});
    }
    int* ctr = (int*)m->counter.p + (chunk_id & 63);
    WTG_CK(cudaMemsetAsync(ctr, 0, sizeof(int), s));
    a.h = (const double2*)m->h.p;
    a.n_inst = kc * nomega;
    a.k_offset = k0;
    a.counter = ctr;
    const int g = (int)std::min<long long>(grid, a.n_inst);
    const size_t de0 = m->ev_used;
    if (m->profile) WTG_CK(cudaEventRecord(m->next_event(), s));
    if (mixed) {
      WTG_CK(wtg::launch_decimate_mixed(a, cfg, g, s));
    } else {
      WTG_CK(wtg::launch_decimate_fp64(a, cfg, g, s));
    }
    m->launches += 1;
    if (m->profile) {
      WTG_CK(cudaEventRecord(m->next_event(), s));
      m->decim_ev.push_back({de0, de0 + 1});
    }
  }
  WTG_CK(cudaEventRecord(m->done, s));
  return WTG_OK;
}

int check_lists(int nw, int ntop, const int* top, int nbot, const int* bot) {
  if (ntop < 0 || nbot < 0 || ntop > wtg::MAX_ORB || nbot > wtg::MAX_ORB)
    return fail(WTG_EINVAL, "orbital list length out of range [0, 1024]");
  if ((ntop > 0 && !top) || (nbot > 0 && !bot)) return fail(WTG_EINVAL, "null orbital list");
  for (int q = 0; q < ntop; ++q)
    if (top[q] < 1 || top[q] > nw) return fail(WTG_EINVAL, "top orbital index outside 1..nw");
  for (int q = 0; q < nbot; ++q)
    if (bot[q] < 1 || bot[q] > nw) return fail(WTG_EINVAL, "bottom orbital index outside 1..nw");
  return WTG_OK;
}

int count_flagged(const uint8_t* st, size_t n) {
  long long c = 0;
  for (size_t i = 0; i < n; ++i) c += st[i] != 0;
  return (int)std::min<long long>(c, INT_MAX);
}

}  // namespace

// A batch engine: the device tables of a fixed set of models, one workspace
// sized for their largest Ndim, its own stream and staging.  One engine runs
// one batch at a time (calls are serialised by its mutex); several engines
// run concurrently on one device.
namespace wtg {
namespace {
std::atomic<int> g_tiles[2][TILE_MAX_N + 1];
}  // namespace

int tile_value(int precision, int N) {
  if (precision < 0 || precision > 1 || N < 1 || N > TILE_MAX_N) return 0;
  return g_tiles[precision][N].load(std::memory_order_relaxed);
}

void tile_store(int precision, int N, int value) {
  g_tiles[precision][N].store(value, std::memory_order_relaxed);
}
}  // namespace wtg

struct wtg_engine {
  int device = 0;
  int precision = 0;
  int nmodels = 0;
  int max_points = 0;
  int max_n = 0;
  std::vector<int> model_n;
  wtg::DecimConfig cfg;
  int smem_gj_max = 0, wb = 0;
  size_t ph_off = 0;
  int grid = 0;
  size_t ws_stride = 0;
  DevBuf models_d, lists_d, ws, io_d, counter;
  unsigned char* pinned = nullptr;
  size_t in_bytes = 0, out_bytes = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  long long launches = 0;
  size_t device_bytes = 0;
  // captured runs, one per staging capacity (powers of two up to max_points)
  bool use_graphs = true;
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;
  long long graph_launches = 0;
  ~wtg_engine() {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    models_d.release();
    lists_d.release();
    ws.release();
    io_d.release();
    counter.release();
    if (pinned) cudaFreeHost(pinned);
    if (stream) cudaStreamDestroy(stream);
    cudaSetDevice(cur);
  }
};

namespace {

// per-point input block (device and pinned host): pmodel, order, k (npts x 2), omega, eta;
// output block: dos_l, dos_r, dos_bulk, iters, status
// input staging of capacity n: the run header (BatchRunHeader, 32 bytes) | pmodel |
// order | k (n x 2) | omega | eta; output: dos_l | dos_r | dos_bulk | iters | status
constexpr size_t RUN_HDR = sizeof(wtg::BatchRunHeader);
size_t engine_in_bytes(int n) { return RUN_HDR + (size_t)n * (4 + 4 + 16 + 8 + 8); }
size_t engine_out_bytes(int n) { return (size_t)n * (8 * 3 + 4 + 1); }

int engine_create(int nmodels, const wtg_model_t* models, int precision, int max_points,
                  const int* ntop, const int* top, const int* nbot, const int* bot,
                  wtg_engine_t* out) {
  if (!out) return fail(WTG_EINVAL, "out is null");
  *out = nullptr;
  if (nmodels < 1 || !models || max_points < 1 || !ntop || !nbot)
    return fail(WTG_EINVAL, "bad argument");
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  const bool mixed = precision == WTG_PREC_MIXED;
  int max_n = 0, max_nru = 1, dev = -1;
  for (int i = 0; i < nmodels; ++i) {
    if (!models[i]) return fail(WTG_EINVAL, "null model");
    if (models[i]->loto)
      return fail(WTG_EUNSUPPORTED, "batch engines take models without the LO-TO correction");
    if (dev >= 0 && models[i]->device != dev) return fail(WTG_EINVAL, "models on different devices");
    dev = models[i]->device;
    max_n = std::max(max_n, models[i]->N);
    max_nru = std::max(max_nru, models[i]->nRu);
  }
  const int nmax = mixed ? wtg::decim_mixed_max_n() : wtg::decim_fp64_large_max_n();
  if (max_n > nmax)
    return fail(WTG_EUNSUPPORTED, "Ndim " + std::to_string(max_n) + " exceeds the kernel limit " +
                                      std::to_string(nmax));
  // orbital lists: check each model's slice
  {
    size_t ot = 0, ob = 0;
    for (int i = 0; i < nmodels; ++i) {
      const int rc = check_lists(models[i]->nw, ntop[i], top ? top + ot : nullptr, nbot[i],
                                 bot ? bot + ob : nullptr);
      if (rc != WTG_OK) return rc;
      ot += (size_t)ntop[i];
      ob += (size_t)nbot[i];
    }
  }
  WTG_CK(cudaSetDevice(dev));
  auto* e = new wtg_engine();
  e->device = dev;
  e->precision = precision;
  e->nmodels = nmodels;
  e->max_points = max_points;
  e->max_n = max_n;
  const size_t ph_bytes = (size_t)max_nru * sizeof(double2);
  cudaError_t ce;
  if (mixed) {
    ce = wtg::batch_mixed_prepare();
    if (ce == cudaSuccess) ce = wtg::batch_mixed_config(max_n, &e->wb, &e->cfg);
  } else {
    ce = wtg::batch_fp64_prepare();
    if (ce == cudaSuccess) ce = wtg::batch_fp64_config(max_n, ph_bytes, &e->smem_gj_max, &e->cfg);
  }
  if (ce != cudaSuccess) {
    delete e;
    return cuda_fail(ce, "batch config");
  }
  e->ph_off = (e->cfg.smem + 15) & ~(size_t)15;
  e->cfg.smem = e->ph_off + ph_bytes;
  int optin = 0, nsm = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e->cfg.smem > (size_t)optin) {
    delete e;
    return fail(WTG_EUNSUPPORTED, "batch kernel shared memory exceeds the device limit");
  }
  e->grid = nsm * std::max(1, e->cfg.ctas_per_sm);
  e->ws_stride = wtg::batch_ws_matrices(mixed ? 1 : 0) * (size_t)max_n * max_n;
  // device tables
  std::vector<int> lists;
  size_t ot = 0, ob = 0;
  std::vector<size_t> toff(nmodels), boff(nmodels);
  for (int i = 0; i < nmodels; ++i) {
    toff[i] = lists.size();
    for (int q = 0; q < ntop[i]; ++q) lists.push_back(top[ot + q]);
    ot += (size_t)ntop[i];
    boff[i] = lists.size();
    for (int q = 0; q < nbot[i]; ++q) lists.push_back(bot[ob + q]);
    ob += (size_t)nbot[i];
  }
  if (lists.empty()) lists.push_back(0);
  ce = e->lists_d.ensure(sizeof(int) * lists.size());
  if (ce == cudaSuccess)
    ce = cudaMemcpy(e->lists_d.p, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice);
  std::vector<wtg::BatchModel> bm(nmodels);
  for (int i = 0; i < nmodels && ce == cudaSuccess; ++i) {
    const wtg_model* m = models[i];
    wtg::BatchModel& b = bm[i];
    b.N = m->N;
    b.nw = m->nw;
    b.np = m->np;
    b.nRu = m->nRu;
    b.nic = m->nic;
    b.ic_lo = m->ic_lo;
    b.hr = m->d_hr;
    b.rab = m->d_rab;
    b.icoff = m->d_icoff;
    b.ntop = ntop[i];
    b.nbot = nbot[i];
    b.top = (const int*)e->lists_d.p + toff[i];
    b.bot = (const int*)e->lists_d.p + boff[i];
    b.w0 = mixed ? wtg::batch_mixed_w0(m->N) : 0;
    e->model_n.push_back(m->N);
  }
  if (ce == cudaSuccess) ce = e->models_d.ensure(sizeof(wtg::BatchModel) * nmodels);
  if (ce == cudaSuccess)
    ce = cudaMemcpy(e->models_d.p, bm.data(), sizeof(wtg::BatchModel) * nmodels, cudaMemcpyHostToDevice);
  e->in_bytes = engine_in_bytes(max_points);
  e->out_bytes = engine_out_bytes(max_points);
  const size_t ws_bytes = sizeof(double2) * e->ws_stride * e->grid;
  if (ce == cudaSuccess) ce = e->ws.ensure(ws_bytes);
  if (ce == cudaSuccess) ce = e->io_d.ensure(e->in_bytes + e->out_bytes);
  if (ce == cudaSuccess) ce = e->counter.ensure(64);
  if (ce == cudaSuccess) ce = cudaMallocHost((void**)&e->pinned, e->in_bytes + e->out_bytes);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    delete e;
    return cuda_fail(ce, "wtg_engine_create");
  }
  e->device_bytes = ws_bytes + e->in_bytes + e->out_bytes + sizeof(int) * lists.size() +
                    sizeof(wtg::BatchModel) * nmodels + 64;
  *out = e;
  return WTG_OK;
}

// one run's stream work for staging capacity C: inputs in, counter reset, the
// batch kernel, outputs back.  With from_device the kernel reads the point count
// and the run's scalars from the staged header (a captured graph replays any run
// of up to C points); otherwise they are kernel arguments (C = the point count).
cudaError_t engine_enqueue(wtg_engine* e, int C, bool from_device) {
  const size_t c = (size_t)C;
  unsigned char* d = (unsigned char*)e->io_d.p;
  unsigned char* din = d + RUN_HDR;
  unsigned char* dout = d + e->in_bytes;
  cudaStream_t s = e->stream;
  const wtg::BatchRunHeader* hdr = (const wtg::BatchRunHeader*)e->pinned;
  cudaError_t ce = cudaMemcpyAsync(d, e->pinned, RUN_HDR + 40 * c, cudaMemcpyHostToDevice, s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e->counter.p, 0, sizeof(int), s);
  if (ce != cudaSuccess) return ce;
  wtg::BatchArgs a;
  memset(&a, 0, sizeof(a));
  a.npts = C;
  a.run = from_device ? (const wtg::BatchRunHeader*)d : nullptr;
  a.models = (const wtg::BatchModel*)e->models_d.p;
  a.pmodel = (const int*)din;
  a.order = (const int*)(din + 4 * c);
  a.k = (const double*)(din + 8 * c);
  a.omega = (const double*)(din + 24 * c);
  a.eta = (const double*)(din + 32 * c);
  a.tol = hdr->tol;                      // the direct path: the run's scalars as arguments
  a.itermax = hdr->itermax;
  a.divide_by_pi = hdr->divide_by_pi;
  a.dos_l = (double*)dout;
  a.dos_r = (double*)(dout + 8 * c);
  a.dos_bulk = (double*)(dout + 16 * c);
  a.iters = (int32_t*)(dout + 24 * c);
  a.status = (uint8_t*)(dout + 28 * c);
  a.ws = (double2*)e->ws.p;
  a.ws_stride = e->ws_stride;
  a.counter = (int*)e->counter.p;
  a.KC = e->cfg.KC;
  a.smem_gj_max = e->smem_gj_max;
  a.wb = e->wb;
  a.ph_off = e->ph_off;
  const int grid = std::min(e->grid, C);
  ce = e->precision == WTG_PREC_MIXED ? wtg::launch_batch_mixed(a, e->cfg, grid, s)
                                      : wtg::launch_batch_fp64(a, e->cfg, grid, s);
  if (ce != cudaSuccess) return ce;
  return cudaMemcpyAsync(e->pinned + e->in_bytes, dout, 29 * c, cudaMemcpyDeviceToHost, s);
}

int engine_run(wtg_engine* e, int npts, const int* point_model, const double* k,
               const double* omega, const double* eta, double tol, int itermax, int divide_by_pi,
               double* dos_l, double* dos_r, double* dos_bulk, int* iters, unsigned char* status) {
  if (!e) return fail(WTG_EINVAL, "null engine");
  if (npts < 0 || npts > e->max_points) return fail(WTG_EINVAL, "npts outside 0..max_points");
  if (itermax < 0) return fail(WTG_EINVAL, "itermax < 0");
  if (npts == 0) return WTG_OK;
  if (!point_model || !k || !omega || !eta || !dos_l || !dos_r || !dos_bulk)
    return fail(WTG_EINVAL, "null array");
  for (int p = 0; p < npts; ++p)
    if (point_model[p] < 0 || point_model[p] >= e->nmodels)
      return fail(WTG_EINVAL, "point_model outside 0..nmodels-1");
  std::lock_guard<std::mutex> lk(e->mu);
  WTG_CK(cudaSetDevice(e->device));
  // launch order: largest estimated cost first (Ndim^3 x an iteration estimate that
  // grows as eta shrinks), so the persistent CTAs finish together
  std::vector<int> order(npts);
  std::vector<double> cost(npts);
  for (int p = 0; p < npts; ++p) {
    const double n = (double)e->model_n[point_model[p]];
    const double ev = std::max(1e-12, std::fabs(eta[p]) * 27.211385);
    cost[p] = n * n * n * (1.0 + std::max(0.0, -std::log10(ev)));
    order[p] = p;
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  // stage inputs in the layout of capacity C: the smallest power of two >= npts
  // (at least 64, at most max_points) when the run replays a captured graph, npts
  // otherwise
  const bool graphed = e->use_graphs;
  size_t C = (size_t)npts;
  if (graphed) {
    C = 64;
    while (C < (size_t)npts) C <<= 1;
    C = std::min(C, (size_t)e->max_points);
  }
  unsigned char* h = e->pinned;
  const size_t n = (size_t)npts;
  wtg::BatchRunHeader hdr;
  memset(&hdr, 0, sizeof(hdr));
  hdr.npts = npts;
  hdr.itermax = itermax;
  hdr.divide_by_pi = divide_by_pi ? 1 : 0;
  hdr.tol = tol;
  memcpy(h, &hdr, RUN_HDR);
  unsigned char* hin = h + RUN_HDR;
  memcpy(hin, point_model, 4 * n);
  memcpy(hin + 4 * C, order.data(), 4 * n);
  memcpy(hin + 8 * C, k, 8 * n);                 // k(:, 1)
  memcpy(hin + 8 * C + 8 * C, k + n, 8 * n);     // k(:, 2) at column stride C
  memcpy(hin + 24 * C, omega, 8 * n);
  memcpy(hin + 32 * C, eta, 8 * n);
  unsigned char* hout = h + e->in_bytes;
  cudaStream_t s = e->stream;
  if (graphed) {
    cudaGraphExec_t ge = nullptr;
    for (auto& g : e->graphs)
      if (g.first == (int)C) ge = g.second;
    if (!ge) {
      cudaGraph_t graph = nullptr;
      WTG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = engine_enqueue(e, (int)C, true);
      const cudaError_t ce2 = cudaStreamEndCapture(s, &graph);
      if (ce == cudaSuccess) ce = ce2;
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ge, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return cuda_fail(ce, "engine graph capture");
      e->graphs.emplace_back((int)C, ge);
    }
    WTG_CK(cudaGraphLaunch(ge, s));
    e->graph_launches += 1;
  } else {
    WTG_CK(engine_enqueue(e, (int)C, false));
  }
  e->launches += 1;
  WTG_CK(cudaStreamSynchronize(s));
  memcpy(dos_l, hout, 8 * n);
  memcpy(dos_r, hout + 8 * C, 8 * n);
  memcpy(dos_bulk, hout + 16 * C, 8 * n);
  if (iters) memcpy(iters, hout + 24 * C, 4 * n);
  if (status) memcpy(status, hout + 28 * C, n);
  return count_flagged(hout + 28 * C, n);
}

}  // namespace

extern "C" {

int wtg_model_create(int nw, int nrpts, const int* irvec, const double* hmnr, const int* ndegen,
                     int np, int ijmax, wtg_model_t* out) {
  if (!out) return fail(WTG_EINVAL, "out is null");
  *out = nullptr;
  if (nw < 1 || nrpts < 0 || np < 1 || ijmax < 0)
    return fail(WTG_EINVAL, "nw, np must be >= 1; nrpts, ijmax >= 0");
  if (nrpts > 0 && (!irvec || !hmnr)) return fail(WTG_EINVAL, "irvec/hmnr null");
  if ((long long)nw * np > 4096) return fail(WTG_EINVAL, "Ndim too large");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(WTG_ENODEV, "no CUDA device available");
  wtg_model* m = new wtg_model();
  cudaGetDevice(&m->device);
  m->nw = nw;
  m->nR = nrpts;
  m->np = np;
  m->ijmax = ijmax;
  m->N = nw * np;
  // R3 values that reach H00 (|j-i| <= Np-1) or H01 (1 <= j-i <= 2Np-1),
  // cut at |R3| <= ijmax (src/ham_qlayer2qlayer.f90:54,72,83).
  const int lo = std::max(-(np - 1), -ijmax), hi = std::min(2 * np - 1, ijmax);
  m->ic_lo = lo;
  m->nic = hi >= lo ? hi - lo + 1 : 0;
  std::vector<int> order;
  for (int r = 0; r < nrpts; ++r) {
    const int ic = irvec[3 * r + 2];
    if (ic >= lo && ic <= hi) order.push_back(r);
  }
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return irvec[3 * x + 2] < irvec[3 * y + 2]; });
  m->nRu = (int)order.size();
  std::vector<int> icoff(m->nic + 1, 0);
  for (int r : order) icoff[irvec[3 * r + 2] - lo + 1]++;
  for (int g = 0; g < m->nic; ++g) icoff[g + 1] += icoff[g];
  const size_t nw2 = (size_t)nw * nw;
  std::vector<double2> hr(std::max<size_t>(1, nw2 * m->nRu));
  std::vector<double2> rab(std::max(1, m->nRu));
  std::vector<double> wr(std::max(1, m->nRu));
  for (int u = 0; u < m->nRu; ++u) {
    const int r = order[u];
    const double nd = ndegen ? (double)ndegen[r] : 1.0;
    wr[u] = 1.0 / nd;
    if (nd == 0.0) {
      delete m;
      return fail(WTG_EINVAL, "ndegen entry is zero");
    }
    for (size_t e = 0; e < nw2; ++e) {
      const double re = hmnr[2 * (nw2 * r + e)], im = hmnr[2 * (nw2 * r + e) + 1];
      hr[nw2 * u + e] = make_double2(nd == 1.0 ? re : re / nd, nd == 1.0 ? im : im / nd);
    }
    rab[u] = make_double2((double)irvec[3 * r], (double)irvec[3 * r + 1]);
  }
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&m->d_hr, sizeof(double2) * hr.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_rab, sizeof(double2) * rab.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_icoff, sizeof(int) * icoff.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_wr, sizeof(double) * wr.size());
  if (e == cudaSuccess) e = cudaMemcpy(m->d_wr, wr.data(), sizeof(double) * wr.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_hr, hr.data(), sizeof(double2) * hr.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_rab, rab.data(), sizeof(double2) * rab.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_icoff, icoff.data(), sizeof(int) * icoff.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(m->done, m->stream);
  if (e != cudaSuccess) {
    wtg_model_destroy(m);
    return cuda_fail(e, "wtg_model_create");
  }
  *out = m;
  return WTG_OK;
}

int wtg_model_set_loto(wtg_model_t m, int natoms, const double* born, const double* diele,
                       const double* masses, double cell_volume) {
  if (!m) return fail(WTG_EINVAL, "null model");
  std::lock_guard<std::mutex> lk(m->mu);
  if (natoms == 0) {
    m->loto = 0;
    return WTG_OK;
  }
  if (natoms < 0 || !born || !diele || !masses) return fail(WTG_EINVAL, "bad argument");
  if (3 * natoms != m->nw) return fail(WTG_EINVAL, "Num_wann must be 3 x natoms for phonons");
  for (int i = 0; i < natoms; ++i)
    if (!(masses[i] > 0.0)) return fail(WTG_EINVAL, "masses must be > 0");
  WTG_CK(cudaSetDevice(m->device));
  // Born_Charge(atom, k direction 1..2, cartesian 1..3) from the Fortran (natoms, 3, 3) array
  std::vector<double> lz((size_t)natoms * 6);
  for (int i = 0; i < natoms; ++i)
    for (int a = 0; a < 2; ++a)
      for (int p = 0; p < 3; ++p) lz[(i * 2 + a) * 3 + p] = born[i + natoms * (a + 3 * p)];
  WTG_CK(cudaEventSynchronize(m->done));
  WTG_CK(m->d_lz.ensure(sizeof(double) * lz.size()));
  WTG_CK(m->d_lm.ensure(sizeof(double) * natoms));
  WTG_CK(cudaMemcpy(m->d_lz.p, lz.data(), sizeof(double) * lz.size(), cudaMemcpyHostToDevice));
  WTG_CK(cudaMemcpy(m->d_lm.p, masses, sizeof(double) * natoms, cudaMemcpyHostToDevice));
  // Diele_Tensor(qq, 1..2) for qq = 1, 2 from the Fortran (3, 3) array
  m->ld[0] = diele[0];
  m->ld[1] = diele[3];
  m->ld[2] = diele[1];
  m->ld[3] = diele[4];
  m->lvol = cell_volume;
  m->loto = 1;
  return WTG_OK;
}

int wtg_model_destroy(wtg_model_t m) {
  if (!m) return fail(WTG_EINVAL, "null model");
  {
    std::lock_guard<std::mutex> lk(m->mu);
    cudaSetDevice(m->device);
    if (m->done) cudaEventSynchronize(m->done);
    cudaFree(m->d_hr);
    cudaFree(m->d_rab);
    cudaFree(m->d_icoff);
    cudaFree(m->d_wr);
    m->d_lz.release();
    m->d_lm.release();
    m->phase.release();
    m->h.release();
    m->ws.release();
    m->counter.release();
    m->k_in.release();
    m->w_in.release();
    m->out_dos.release();
    m->out_it.release();
    m->out_st.release();
    if (m->done) cudaEventDestroy(m->done);
    for (cudaEvent_t e : m->ev_pool) cudaEventDestroy(e);
    if (m->stream) cudaStreamDestroy(m->stream);
  }
  delete m;
  return WTG_OK;
}

int wtg_model_ndim(wtg_model_t m) {
  if (!m) return fail(WTG_EINVAL, "null model");
  return m->N;
}

int wtg_ham_qlayer2qlayer(wtg_model_t m, const double* k, double* h00, double* h01) {
  if (!m || !k || !h00 || !h01) return fail(WTG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(m->mu);
  WTG_CK(cudaSetDevice(m->device));
  cudaStream_t s = m->stream;
  WTG_CK(cudaStreamWaitEvent(s, m->done, 0));
  WTG_CK(m->k_in.ensure(sizeof(double) * 2));
  WTG_CK(m->phase.ensure(sizeof(double2) * std::max(1, m->nRu)));
  const size_t nn = (size_t)m->N * m->N;
  WTG_CK(m->h.ensure(sizeof(double2) * 2 * nn));
  WTG_CK(cudaMemcpyAsync(m->k_in.p, k, sizeof(double) * 2, cudaMemcpyHostToDevice, s));
  wtg::FourierArgs f;
  f.k = (const double*)m->k_in.p;
  f.nk_total = 1;
  f.k0 = 0;
  f.kc = 1;
  f.rab = m->d_rab;
  set_loto_args(m, f);
  f.hr = m->d_hr;
  f.icoff = m->d_icoff;
  f.ic_lo = m->ic_lo;
  f.nic = m->nic;
  f.nRu = m->nRu;
  f.nw = m->nw;
  f.np = m->np;
  f.ijmax = m->ijmax;
  f.phase = (double2*)m->phase.p;
  f.h = (double2*)m->h.p;
  wtg::launch_fourier(f, s);
  WTG_CK(cudaGetLastError());
  WTG_CK(cudaMemcpyAsync(h00, f.h, sizeof(double2) * nn, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(h01, f.h + nn, sizeof(double2) * nn, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaEventRecord(m->done, s));
  WTG_CK(cudaStreamSynchronize(s));
  return WTG_OK;
}

int wtg_surfgreen_1985(int ndim, double omega, double eta, const double* h00, const double* h01,
                       double tol, int itermax, double* gll, double* grr, double* gb, int* iters,
                       int* status) {
  if (ndim < 1 || !h00 || !h01 || !gll || !grr || !gb) return fail(WTG_EINVAL, "bad argument");
  if (itermax < 0) return fail(WTG_EINVAL, "itermax < 0");
  if (ndim > wtg::decim_fp64_large_max_n())
    return fail(WTG_EUNSUPPORTED, "Ndim exceeds the FP64 kernel limit");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(WTG_ENODEV, "no CUDA device available");
  const size_t nn = (size_t)ndim * ndim;
  wtg::DecimConfig cfg;
  WTG_CK(wtg::decim_fp64_config(ndim, 0, &cfg));
  // one allocation: h[2nn] | gll grr gb [3nn] | ws [8 or 9 nn] | omega | outputs
  const size_t wsm = wtg::decim_fp64_ws_matrices(cfg);
  const size_t bytes = sizeof(double2) * ((5 + wsm) * nn) + 64 + 64;
  char* base = nullptr;
  WTG_CK(cudaMalloc(&base, bytes));
  double2* dh = (double2*)base;
  double2* dgll = dh + 2 * nn;
  double2* dgrr = dgll + nn;
  double2* dgb = dgrr + nn;
  double2* dws = dgb + nn;
  char* tail = (char*)(dws + wsm * nn);
  double* dw = (double*)tail;          // omega
  double* ddos = dw + 1;               // 3 doubles
  int* dctr = (int*)(ddos + 3);
  int32_t* dit = dctr + 1;
  uint8_t* dst = (uint8_t*)(dit + 1);
  int rc = WTG_OK;
  cudaError_t e = cudaMemcpy(dh, h00, sizeof(double2) * nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dh + nn, h01, sizeof(double2) * nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dw, &omega, sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dctr, 0, sizeof(int));
  if (e == cudaSuccess) {
    wtg::DecimArgs a;
    memset(&a, 0, sizeof(a));
    a.N = ndim;
    a.nw = ndim;
    a.nomega = 1;
    a.n_inst = 1;
    a.h = dh;
    a.omega = dw;
    a.eta = eta;
    a.tol = tol;
    a.itermax = itermax;
    a.nk_total = 1;
    a.dos_l = ddos;
    a.dos_r = ddos + 1;
    a.dos_bulk = ddos + 2;
    a.iters = dit;
    a.status = dst;
    a.gll = dgll;
    a.grr = dgrr;
    a.gb = dgb;
    a.ws = dws;
    a.counter = dctr;
    a.KC = cfg.KC;
    e = wtg::launch_decimate_fp64(a, cfg, 1, 0);
  }
  if (e == cudaSuccess) e = cudaMemcpy(gll, dgll, sizeof(double2) * nn, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(grr, dgrr, sizeof(double2) * nn, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(gb, dgb, sizeof(double2) * nn, cudaMemcpyDeviceToHost);
  int32_t it = 0;
  uint8_t st = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&it, dit, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(uint8_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = cuda_fail(e, "wtg_surfgreen_1985");
  cudaFree(base);
  if (rc != WTG_OK) return rc;
  if (iters) *iters = it;
  if (status) *status = st;
  return st ? 1 : WTG_OK;
}

int wtg_surface_spectrum_device(wtg_model_t m, int nk, const double* d_k, int nomega,
                                const double* d_omega, double eta, double tol, int itermax,
                                int ntop, const int* top, int nbot, const int* bot,
                                int divide_by_pi, int precision, double* d_dos_l, double* d_dos_r,
                                double* d_dos_bulk, int32_t* d_iters, uint8_t* d_status,
                                void* stream) {
  if (!m) return fail(WTG_EINVAL, "null model");
  if (nk < 0 || nomega < 0 || itermax < 0) return fail(WTG_EINVAL, "negative size");
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  if (nk == 0 || nomega == 0) return WTG_OK;
  if (!d_k || !d_omega || !d_dos_l || !d_dos_r || !d_dos_bulk) return fail(WTG_EINVAL, "null array");
  int rc = check_lists(m->nw, ntop, top, nbot, bot);
  if (rc != WTG_OK) return rc;
  std::lock_guard<std::mutex> lk(m->mu);
  WTG_CK(cudaSetDevice(m->device));
  return run_spectrum(m, nk, d_k, nomega, d_omega, eta, tol, itermax, ntop, top, nbot, bot,
                      divide_by_pi, precision, d_dos_l, d_dos_r, d_dos_bulk, d_iters, d_status,
                      (cudaStream_t)stream);
}

int wtg_surface_spectrum(wtg_model_t m, int nk, const double* k, int nomega, const double* omega,
                         double eta, double tol, int itermax, int ntop, const int* top, int nbot,
                         const int* bot, int divide_by_pi, int precision, double* dos_l,
                         double* dos_r, double* dos_bulk, int32_t* iters, uint8_t* status) {
  if (!m) return fail(WTG_EINVAL, "null model");
  if (nk < 0 || nomega < 0 || itermax < 0) return fail(WTG_EINVAL, "negative size");
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  if (nk == 0 || nomega == 0) return WTG_OK;
  if (!k || !omega || !dos_l || !dos_r || !dos_bulk) return fail(WTG_EINVAL, "null array");
  int rc = check_lists(m->nw, ntop, top, nbot, bot);
  if (rc != WTG_OK) return rc;
  std::lock_guard<std::mutex> lk(m->mu);
  WTG_CK(cudaSetDevice(m->device));
  const size_t npts = (size_t)nk * nomega;
  cudaStream_t s = m->stream;
  WTG_CK(cudaStreamWaitEvent(s, m->done, 0));
  WTG_CK(m->k_in.ensure(sizeof(double) * 2 * (size_t)nk));
  WTG_CK(m->w_in.ensure(sizeof(double) * (size_t)nomega));
  WTG_CK(m->out_dos.ensure(sizeof(double) * 3 * npts));
  WTG_CK(m->out_it.ensure(sizeof(int32_t) * npts));
  WTG_CK(m->out_st.ensure(sizeof(uint8_t) * npts));
  WTG_CK(cudaMemcpyAsync(m->k_in.p, k, sizeof(double) * 2 * nk, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(m->w_in.p, omega, sizeof(double) * nomega, cudaMemcpyHostToDevice, s));
  double* dd = (double*)m->out_dos.p;
  rc = run_spectrum(m, nk, (const double*)m->k_in.p, nomega, (const double*)m->w_in.p, eta, tol,
                    itermax, ntop, top, nbot, bot, divide_by_pi, precision, dd, dd + npts,
                    dd + 2 * npts,
                    (int32_t*)m->out_it.p, (uint8_t*)m->out_st.p, s);
  if (rc != WTG_OK) return rc;
  WTG_CK(cudaMemcpyAsync(dos_l, dd, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(dos_r, dd + npts, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(dos_bulk, dd + 2 * npts, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  std::vector<uint8_t> st_local;
  uint8_t* st_host = status;
  if (!st_host) {
    st_local.resize(npts);
    st_host = st_local.data();
  }
  WTG_CK(cudaMemcpyAsync(st_host, m->out_st.p, npts, cudaMemcpyDeviceToHost, s));
  if (iters)
    WTG_CK(cudaMemcpyAsync(iters, m->out_it.p, sizeof(int32_t) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  return count_flagged(st_host, npts);
}

static int unit_op(int op, int n, const double* a, const double* b, double* c, int precision,
                   int* status) {
  if (n < 1 || !a || !c || (op == 0 && !b)) return fail(WTG_EINVAL, "bad argument");
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  const bool mixed = precision == WTG_PREC_MIXED;
  const int nmax = mixed ? wtg::decim_mixed_max_n() : wtg::decim_fp64_large_max_n();
  if (n > nmax) return fail(WTG_EUNSUPPORTED, "n exceeds the kernel limit " + std::to_string(nmax));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(WTG_ENODEV, "no CUDA device available");
  const size_t nn = (size_t)n * n;
  char* base = nullptr;
  WTG_CK(cudaMalloc(&base, sizeof(double2) * 8 * nn + 64));
  double2* dx = (double2*)base;
  double2* dy = dx + nn;
  double2* dc = dy + nn;
  double2* dws = dc + nn;            // 5 nn
  int* dst = (int*)(dws + 5 * nn);
  cudaError_t e = cudaMemcpy(dx, a, sizeof(double2) * nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && op == 0) e = cudaMemcpy(dy, b, sizeof(double2) * nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = mixed ? wtg::launch_mixed_unit(op, n, dx, dy, dc, dws, 8, dst, 0)
              : wtg::launch_fp64_unit(op, n, dx, dy, dc, dws, dst, 0);
  if (e == cudaSuccess) e = cudaMemcpy(c, dc, sizeof(double2) * nn, cudaMemcpyDeviceToHost);
  int st = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(base);
  if (e != cudaSuccess) return cuda_fail(e, op == 0 ? "wtg_mat_mul" : "wtg_inv");
  if (status) *status = st;
  return st ? 1 : WTG_OK;
}

int wtg_mat_mul(int n, const double* a, const double* b, double* c, int precision) {
  return unit_op(0, n, a, b, c, precision, nullptr);
}

int wtg_inv(int n, double* a, int precision, int* status) {
  return unit_op(1, n, a, nullptr, a, precision, status);
}

int wtg_model_profile(wtg_model_t m, int enable) {
  if (!m) return fail(WTG_EINVAL, "null model");
  std::lock_guard<std::mutex> lk(m->mu);
  if (m->done) cudaEventSynchronize(m->done);
  m->profile = enable != 0;
  m->ev_used = 0;
  m->fourier_ev.clear();
  m->decim_ev.clear();
  m->launches = 0;
  return WTG_OK;
}

int wtg_model_profile_read(wtg_model_t m, double* fourier_ms, double* decim_ms,
                           long long* launches, int* decim_launches) {
  if (!m) return fail(WTG_EINVAL, "null model");
  std::lock_guard<std::mutex> lk(m->mu);
  WTG_CK(cudaSetDevice(m->device));
  WTG_CK(cudaEventSynchronize(m->done));
  double tf = 0.0, td = 0.0;
  for (auto& pr : m->fourier_ev) {
    float ms = 0.f;
    WTG_CK(cudaEventElapsedTime(&ms, m->ev_pool[pr.first], m->ev_pool[pr.second]));
    tf += ms;
  }
  for (auto& pr : m->decim_ev) {
    float ms = 0.f;
    WTG_CK(cudaEventElapsedTime(&ms, m->ev_pool[pr.first], m->ev_pool[pr.second]));
    td += ms;
  }
  if (fourier_ms) *fourier_ms = tf;
  if (decim_ms) *decim_ms = td;
  if (launches) *launches = m->launches;
  if (decim_launches) *decim_launches = (int)m->decim_ev.size();
  return WTG_OK;
}

int wtg_surface_spectrum_spin(wtg_model_t m, int nk, const double* k, int nomega,
                              const double* omega, double eta, double tol, int itermax, int ntop,
                              const int* top, int nbot, const int* bot, int arc_mode,
                              int precision, double* dos_l, double* dos_r, double* dos_bulk,
                              double* spin_out, int32_t* iters, uint8_t* status) {
  if (!m) return fail(WTG_EINVAL, "null model");
  if (nk < 0 || nomega < 0 || itermax < 0) return fail(WTG_EINVAL, "negative size");
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  if (nk == 0 || nomega == 0) return WTG_OK;
  if (!k || !omega || !dos_l || !dos_r || !dos_bulk || !spin_out)
    return fail(WTG_EINVAL, "null array");
  int rc = check_lists(m->nw, ntop, top, nbot, bot);
  if (rc != WTG_OK) return rc;
  std::lock_guard<std::mutex> lk(m->mu);
  WTG_CK(cudaSetDevice(m->device));
  const size_t npts = (size_t)nk * nomega;
  cudaStream_t s = m->stream;
  WTG_CK(cudaStreamWaitEvent(s, m->done, 0));
  WTG_CK(m->k_in.ensure(sizeof(double) * 2 * (size_t)nk));
  WTG_CK(m->w_in.ensure(sizeof(double) * (size_t)nomega));
  WTG_CK(m->out_dos.ensure(sizeof(double) * 9 * npts));
  WTG_CK(m->out_it.ensure(sizeof(int32_t) * npts));
  WTG_CK(m->out_st.ensure(sizeof(uint8_t) * npts));
  WTG_CK(cudaMemcpyAsync(m->k_in.p, k, sizeof(double) * 2 * nk, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(m->w_in.p, omega, sizeof(double) * nomega, cudaMemcpyHostToDevice, s));
  double* dd = (double*)m->out_dos.p;
  double* dspin[6];
  for (int c = 0; c < 6; ++c) dspin[c] = dd + (3 + c) * npts;
  rc = run_spectrum(m, nk, (const double*)m->k_in.p, nomega, (const double*)m->w_in.p, eta, tol,
                    itermax, ntop, top, nbot, bot, arc_mode ? 1 : 0, precision, dd, dd + npts,
                    dd + 2 * npts, (int32_t*)m->out_it.p, (uint8_t*)m->out_st.p, s, dspin,
                    arc_mode ? 1 : 0);
  if (rc != WTG_OK) return rc;
  WTG_CK(cudaMemcpyAsync(dos_l, dd, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(dos_r, dd + npts, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(dos_bulk, dd + 2 * npts, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(spin_out, dd + 3 * npts, sizeof(double) * 6 * npts, cudaMemcpyDeviceToHost, s));
  std::vector<uint8_t> st_local;
  uint8_t* st_host = status;
  if (!st_host) {
    st_local.resize(npts);
    st_host = st_local.data();
  }
  WTG_CK(cudaMemcpyAsync(st_host, m->out_st.p, npts, cudaMemcpyDeviceToHost, s));
  if (iters)
    WTG_CK(cudaMemcpyAsync(iters, m->out_it.p, sizeof(int32_t) * npts, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  return count_flagged(st_host, npts);
}

int wtg_test_option(int option, int value) {
  if (option < 1 || option >= WTG_TEST_OPTIONS) return fail(WTG_EINVAL, "unknown test option");
  if (value < 0) return fail(WTG_EINVAL, "test option value < 0");
  wtg::set_test_option(option, value);
  return WTG_OK;
}

int wtg_last_error(char* buf, int len) {
  if (!buf || len <= 0) return WTG_EINVAL;
  snprintf(buf, (size_t)len, "%s", g_err.c_str());
  return WTG_OK;
}

int wtg_device_info(char* buf, int len) {
  if (!buf || len <= 0) return WTG_EINVAL;
  int dev = 0;
  cudaDeviceProp p;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess)
    return fail(WTG_ENODEV, "no CUDA device available");
  snprintf(buf, (size_t)len, "%s, %d SMs, cc %d.%d, %.1f GiB", p.name, p.multiProcessorCount,
           p.major, p.minor, p.totalGlobalMem / 1073741824.0);
  return WTG_OK;
}

int wtg_engine_create(int nmodels, const wtg_model_t* models, int precision, int max_points,
                      const int* ntop, const int* top, const int* nbot, const int* bot,
                      wtg_engine_t* out) {
  return engine_create(nmodels, models, precision, max_points, ntop, top, nbot, bot, out);
}

int wtg_engine_destroy(wtg_engine_t e) {
  if (!e) return fail(WTG_EINVAL, "null engine");
  delete e;
  return WTG_OK;
}

int wtg_engine_set_graphs(wtg_engine_t e, int on) {
  if (!e) return fail(WTG_EINVAL, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  e->use_graphs = on != 0;
  return WTG_OK;
}

int wtg_engine_graph_info(wtg_engine_t e, int* graphs, long long* graph_launches) {
  if (!e) return fail(WTG_EINVAL, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  if (graphs) *graphs = (int)e->graphs.size();
  if (graph_launches) *graph_launches = e->graph_launches;
  return WTG_OK;
}

int wtg_tile_set(int precision, int ndim, int value) {
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  if (ndim < 1 || ndim > wtg::TILE_MAX_N) return fail(WTG_EINVAL, "ndim outside 1..4096");
  if (value != 0) {
    if (precision == WTG_PREC_FP64 && value != 128 && value != 256 && value != 512)
      return fail(WTG_EINVAL, "FP64 tile: threads per CTA must be 128, 256 or 512");
    if (precision == WTG_PREC_MIXED &&
        (value < 8 || (value & 7) != 0 || ndim > wtg::decim_mixed_max_n() ||
         value > wtg::mixed_w0_max(ndim)))
      return fail(WTG_EINVAL, "mixed tile: pass width must be a multiple of 8 in 8.." +
                                  std::to_string(ndim <= wtg::decim_mixed_max_n()
                                                     ? wtg::mixed_w0_max(ndim) : 0));
  }
  wtg::tile_store(precision, ndim, value);
  return WTG_OK;
}

int wtg_tile_get(int precision, int ndim, int* value, int* builtin) {
  if (precision != WTG_PREC_FP64 && precision != WTG_PREC_MIXED)
    return fail(WTG_EINVAL, "unknown precision mode");
  if (ndim < 1 || ndim > wtg::TILE_MAX_N) return fail(WTG_EINVAL, "ndim outside 1..4096");
  int b = 0;
  if (precision == WTG_PREC_FP64) {
    b = ndim > wtg::decim_fp64_max_n() ? 256 : wtg::fp64_threads_default(ndim);
  } else {
    b = ndim <= wtg::decim_mixed_max_n() ? wtg::mixed_w0_default(ndim) : 0;
  }
  const int t = wtg::tile_value(precision, ndim);
  if (builtin) *builtin = b;
  if (value) *value = t != 0 ? t : b;
  return WTG_OK;
}

int wtg_engine_info(wtg_engine_t e, long long* device_bytes, int* max_points, long long* launches) {
  if (!e) return fail(WTG_EINVAL, "null engine");
  if (device_bytes) *device_bytes = (long long)e->device_bytes;
  if (max_points) *max_points = e->max_points;
  if (launches) *launches = e->launches;
  return WTG_OK;
}

int wtg_engine_run(wtg_engine_t e, int npts, const int* point_model, const double* k,
                   const double* omega, const double* eta, double tol, int itermax,
                   int divide_by_pi, double* dos_l, double* dos_r, double* dos_bulk, int* iters,
                   unsigned char* status) {
  return engine_run(e, npts, point_model, k, omega, eta, tol, itermax, divide_by_pi, dos_l, dos_r,
                    dos_bulk, iters, status);
}

int wtg_batch_spectrum(int nmodels, const wtg_model_t* models, int npts, const int* point_model,
                       const double* k, const double* omega, const double* eta, double tol,
                       int itermax, const int* ntop, const int* top, const int* nbot,
                       const int* bot, int divide_by_pi, int precision, double* dos_l,
                       double* dos_r, double* dos_bulk, int* iters, unsigned char* status) {
  if (npts == 0) return WTG_OK;
  wtg_engine_t e = nullptr;
  int rc = engine_create(nmodels, models, precision, std::max(1, npts), ntop, top, nbot, bot, &e);
  if (rc != WTG_OK) return rc;
  rc = engine_run(e, npts, point_model, k, omega, eta, tol, itermax, divide_by_pi, dos_l, dos_r,
                  dos_bulk, iters, status);
  delete e;
  return rc;
}

}  // extern "C"
