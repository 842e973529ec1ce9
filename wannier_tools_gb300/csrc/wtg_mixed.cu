// Mixed-precision Lopez-Sancho decimation on the 5th-generation tensor cores.
//
// Every complex product of surfgreen_1985 (src/surfgreen.f90:92-116, zgemm at
// src/mat_mul.f90:23) runs as an exactly-split BF16 product on tcgen05:
//   * each FP64 operand is written as 49-bit fixed point (rounded to nearest)
//     against a shared exponent per row (left factor) or per column (right
//     factor) and cut into seven balanced base-128 digits (the leading one in
//     [0, 128], the others in [-64, 63], so that rounding and truncation errors
//     have no sign bias); a digit is an exact BF16 value (with a power-of-two
//     scale folded in), made by one FFMA from the digit's integer bits;
//   * slice products A^p B^q with p + q <= 8 are issued as BF16 MMAs with FP32
//     accumulators in tensor memory, one accumulator per slice order
//     t = p + q for t = 2 .. 6 (integer terms in the order's unit, exact while
//     the partial sums stay below 2^24, MxPlan) and one for t = 7, 8 (its
//     accumulation truncates; at 2^-35 of the result that costs ~2^-51);  49
//     bits are needed because the Newton-Schulz refinement below can only be
//     as accurate as its residual product;
//   * the accumulators are read back (tcgen05.ld), converted to integers and
//     summed in int64, and the FP64 result is assembled with integer
//     operations (no FP64 arithmetic for the product itself).
// The complex product runs in passes over row blocks of 128 (the MMA's M) and
// column blocks of w <= 40: the B digit planes are stored in two runs, Yr, Yi
// and -Yi, Yr per digit, so that per slice pair two MMAs of N = 2w, Xr [Yr; Yi]
// and Xi [-Yi; Yr], accumulate [Cr | Ci] = [Xr Yr - Xi Yi | Xr Yi + Xi Yr]; both
// components share one generation of the A planes, and the pairs of one A digit
// with up to 128 / w consecutive B digits whose orders have consecutive
// accumulators are one MMA of N = 2wg (oz_issue).
// Inverses in the loop (zgesv with identity, src/inverse.f90:43-55) are an
// FP32 Gauss-Jordan (shared memory up to Ndim 112, global memory in panels
// above) followed by Newton-Schulz refinement X <- X + X (I - M X): the
// residual I - M X is a 7-digit split product, the correction X R a 4-digit
// one (R is small).  The three final inverses (src/surfgreen.f90:127-134) are
// FP64 Gauss-Jordan (the FP64 form's own code), and the convergence test
// sum |alpha_ij| (src/surfgreen.f90:120) takes each |alpha_ij| and the sum in
// FP64.
//
// Operands are staged per K chunk of 16 (one MMA k-step) into a double-buffered
// shared-memory area in the canonical K-major, no-swizzle layout (8 x 16-byte
// core matrices; K-adjacent core matrices 128 B apart, 8-row groups 256 B
// apart).  Warps 1..15 generate a chunk's digit planes while warp 0 issues the
// previous chunk's MMAs (one thread) and commits them to the buffer's mbarrier.
// Every mbarrier wait is bounded; on a timeout the CTA stops issuing work,
// marks the instance, waits (bounded) for its MMAs and frees tensor memory.
#include <cuda_bf16.h>

#include <mutex>

#include "../../include/wtgpu.h"
#include "wtg_common.cuh"

namespace wtg {

namespace {

#include "wtg_fp64_dev.cuh"

constexpr int MX_T = 512;            // threads per CTA (16 warps)
constexpr int NSL = 7;               // digits per operand (49-bit fixed point)
constexpr int KCH = 16;              // K per staged chunk
constexpr int APLANE = 128 * KCH * 2;  // bytes of one A plane (128 rows x 16 bf16)
constexpr unsigned SPIN_LIMIT = 1u << 22;
constexpr int PT_TIMEOUT = 8;

constexpr int OZ_STORE = 0, OZ_ADD2 = 1, OZ_STORE_NORM = 2, OZ_IMINUS = 3, OZ_ADDTO = 4;
constexpr int MX_MAXN = 320;         // largest Ndim
constexpr int MX_SMEM_GJ_N = 112;    // up to here the FP32 Gauss-Jordan runs in shared memory
constexpr int MX_PANEL = 16;         // pivot steps per panel of the global-memory Gauss-Jordan
constexpr int MX_ROWS = MX_MAXN / 32;  // rows per lane of a register-resident column

// How one product is cut into tensor-memory passes.  Rows go in blocks of
// M = 128.  Each pass holds nacc FP32 accumulators of 2w columns (both
// components side by side), so 512 tensor-memory columns bound 2 nacc w;
// output columns [0, NP) go in ncb blocks of w0 (a multiple of 8; the last
// block narrower).  A 7-digit product keeps one accumulator for each slice
// order t = 2..6, whose terms are integers in the order's own unit, and one
// for the orders 7 and 8 (nacc = 6).  An accumulator of integer terms adds
// exactly while its partial sums stay below 2^24.  With the leading digit in
// [0, 128] and the others in [-64, 63] (balanced digits), order t gathers
// 2 (t - 1) K digit products (two MMAs a slice pair, one per input component)
// of at most 2^14 (1, 1), 2^13 (1, q) or 2^12: at most 57344 K for order 6,
// 49152 K for order 5, so every exact order stays below 2^24 for K <= 292 even
// with every product at its bound and of one sign (orders <= 5 up to K = 341),
// and expected partial sums of random digits are a few 10^4.  Terms of
// different orders in one accumulator are not integers in a common unit and
// the tensor core's FP32 accumulation truncates them: the orders 7 and 8 share
// the last accumulator, whose truncation costs about 2^-51 of the result
// (sharing it with order 6 as well costs about 2^-44).
struct MxPlan {
  int N, NP, nrb, nacc, ncb, w0;
  int wb;                    // B-plane width of the shared-memory layout
  int lumped;                // the last accumulator sums the orders 7 and 8 (7-digit products)
};

// accumulators of a 7-digit product: orders 2 .. MX_NACC exact, the rest lumped
constexpr int MX_NACC = 6;

// widest pass: both components side by side, 2 x MX_NACC accumulators of w
// columns in the 512 tensor-memory columns
__host__ __device__ inline int mx_wmax(int) { return (512 / (2 * MX_NACC)) & ~7; }

// The plan of a 4-digit product (28-bit operands, slice pairs p + q <= 5, every
// order exact: accumulators for orders 2..5, nothing lumped), used where the
// product only corrects a value whose size it is small against (the
// Newton-Schulz update G + G R, |R| << 1).  Its passes are as wide as the
// tensor memory and the layout's B area (4 NSL planes of wb rows per buffer)
// allow.
__host__ __device__ inline MxPlan mx_plan4(const MxPlan& p7) {
  MxPlan p = p7;
  p.nacc = 4;
  p.lumped = 0;
  int wmax = (512 / (2 * p.nacc)) & ~7;
  const int bcap = ((4 * NSL * p7.wb) / (4 * 4)) & ~7;
  if (bcap < wmax) wmax = bcap;
  p.ncb = (p.NP + wmax - 1) / wmax;
  p.w0 = ((p.NP + p.ncb - 1) / p.ncb + 7) & ~7;
  while (p.ncb > 1 && (p.ncb - 1) * p.w0 >= p.NP) --p.ncb;
  return p;
}

// w0_req: a pass width from the tile table (a multiple of 8 in [8, mx_wmax]); any
// other value takes the built-in choice (the fewest passes, evenly split)
__host__ __device__ inline MxPlan mx_plan(int N, int w0_req = 0) {
  MxPlan p;
  p.N = N;
  p.NP = (N + 7) & ~7;          // an MMA's N (2w, both components) needs w a multiple of 8 only
  p.nrb = (N + 127) / 128;
  p.nacc = MX_NACC;
  p.lumped = 1;
  const int wmax = mx_wmax(N);
  if (w0_req >= 8 && w0_req <= wmax && (w0_req & 7) == 0) {
    p.w0 = w0_req;
    p.ncb = (p.NP + w0_req - 1) / w0_req;
  } else {
    p.ncb = (p.NP + wmax - 1) / wmax;
    p.w0 = ((p.NP + p.ncb - 1) / p.ncb + 7) & ~7;
    while (p.ncb > 1 && (p.ncb - 1) * p.w0 >= p.NP) --p.ncb;
  }
  p.wb = p.w0;
  return p;
}

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle, LBO 128 B (K), SBO 256 B (rows)
__device__ __forceinline__ uint64_t sdesc(uint32_t a) {
  return (uint64_t)((a >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(256 >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: kind::f16, BF16 x BF16 -> FP32, K-major A and B, M = 128
__device__ __forceinline__ uint32_t idesc(int n, int negb) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)negb << 14) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t id,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* mb) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   saddr(mb))
               : "memory");
}

// Bounded wait for an mbarrier phase.  limit 0: up to SPIN_LIMIT blocking
// try_wait polls (the normal bound); limit > 0 (a test's bound): that many
// non-blocking test_wait polls, so that a short limit reliably runs out while
// the tensor cores are still busy.
__device__ __forceinline__ bool mbar_wait(uint64_t* mb, uint32_t parity, unsigned limit = 0) {
  const uint32_t a = saddr(mb);
  if (limit == 0) {
    for (unsigned spin = 0; spin < SPIN_LIMIT; ++spin) {
      uint32_t ok;
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          " selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(ok)
          : "r"(a), "r"(parity)
          : "memory");
      if (ok) return true;
    }
    return false;
  }
  for (unsigned spin = 0; spin < limit; ++spin) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- integer-only conversions ---------------------------------------------

__device__ __forceinline__ int bexp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// |x| as 49-bit fixed point against biased exponent E (|x| < 2^(E-1022)),
// rounded to nearest (ties up): at most 2^49
__device__ __forceinline__ unsigned long long fixed49(double x, int E, unsigned& neg) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  neg = (unsigned)(u >> 63);
  int ex = (int)((u >> 52) & 0x7FF);
  unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  if (ex) m |= 1ull << 52;
  else ex = 1;
  const int sh = E - ex + 4;          // >= 4: E is the maximum exponent of the row or column
  return sh < 64 ? ((m + (1ull << (sh - 1))) >> sh) : 0ull;
}

// 64 in every 7-bit digit position: f + DIGIT_BIAS has digits g_p in [0, 127]
// below the leading one, and f = sum (g_p - 64) 128^(7-p) (balanced digits)
constexpr unsigned long long DIGIT_BIAS = 0x1020408102040ull;

// integer value of an integer-valued float, divided by 2^7 (truncating)
__device__ __forceinline__ long long f2ll_bits(uint32_t w) {
  const int e = (int)((w >> 23) & 0xFF);
  if (e < 134) return 0;
  const long long m = (long long)((w & 0x7FFFFFu) | 0x800000u);
  const int sh = e - 157;
  const long long v = sh >= 0 ? (m << sh) : (m >> (-sh));
  return (w >> 31) ? -v : v;
}

// double with value S * 2^(be0 - 1023) assembled from bits (truncating)
__device__ __forceinline__ double assemble(long long S, int be0) {
  if (S == 0) return 0.0;
  const unsigned long long neg = S < 0 ? 1ull : 0ull;
  const unsigned long long a = neg ? (unsigned long long)(-S) : (unsigned long long)S;
  const int L = 63 - __clzll((long long)a);
  const unsigned long long mant = L >= 52 ? (a >> (L - 52)) : (a << (52 - L));
  const int be = L + be0;
  if (be <= 0) return 0.0;
  if (be >= 2047) return __longlong_as_double((long long)((neg << 63) | (0x7FFull << 52)));
  return __longlong_as_double(
      (long long)((neg << 63) | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

__device__ __forceinline__ float d2f_bits(double x) {    // truncating FP64 -> FP32
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(u >> 63) << 31;
  const int ex = (int)((u >> 52) & 0x7FF);
  const int e32 = ex - 1023 + 127;
  if (ex == 0 || e32 <= 0) return __uint_as_float(sign);
  if (e32 >= 255) return __uint_as_float(sign | 0x7F800000u);
  return __uint_as_float(sign | ((uint32_t)e32 << 23) | (uint32_t)((u >> 29) & 0x7FFFFFu));
}

__device__ __forceinline__ double f2d_bits(float f) {     // exact FP32 -> FP64
  const uint32_t w = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(w >> 31) << 63;
  const int e = (int)((w >> 23) & 0xFF);
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 255) return __longlong_as_double((long long)(sign | (0x7FFull << 52)));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) |
                  ((unsigned long long)(w & 0x7FFFFFu) << 29)));
}

// ---- shared state ------------------------------------------------------------

struct MxShared {
  unsigned char* buf[2];   // per buffer: 2*NSL A planes then 2*NSL B planes
  float2* gj;              // FP32 Gauss-Jordan matrix (aliases the buffers)
  float2* mult;            // [MX_MAXN][MX_PANEL] multiplier columns of the global-memory
                           // Gauss-Jordan's panel (aliases the buffers)
  float2* colbuf;
  float2* rowbuf;
  float2* recip;
  int* perm;
  int* cols;
  int* expA;               // [2 MX_MAXN] row exponents (rows of a row-stacked product)
  int* expB;               // [MX_MAXN] column exponents
  float* red;              // [32]
  uint64_t* mbar;          // [2]
  uint32_t* tslot;
  int* misc;               // 0 instance, 1 singular, 2-3 pivot rows (shared-memory Gauss-Jordan)
};

__host__ __device__ __forceinline__ int bufbytes_of(int WB) {
  return 2 * NSL * APLANE + 4 * NSL * WB * KCH * 2;
}

// Bytes of the FP64 Gauss-Jordan working area of the final inverses
// (fp64_layout with KC = GJ_PANEL): the N x N matrix and its small arrays when
// the inverse runs in shared memory, the panel arrays when it runs in global
// memory.
__host__ __device__ constexpr int fp64_area_bytes(int N, bool in_smem) {
  return (in_smem ? (N * N > 2 * N * GJ_PANEL ? N * N : 2 * N * GJ_PANEL) : 2 * N * GJ_PANEL) * 16 +
         N * 32 + 16 * GJ_PANEL + 32 * 8 + N * 8 + 16;
}
// the largest over Ndim 1..MX_MAXN (shared-memory inverse up to MX_SMEM_GJ_N)
constexpr int MX_FP64_AREA =
    fp64_area_bytes(MX_SMEM_GJ_N, true) > fp64_area_bytes(MX_MAXN, false)
        ? fp64_area_bytes(MX_SMEM_GJ_N, true) : fp64_area_bytes(MX_MAXN, false);

// bytes before the small arrays: the two operand buffers, which the FP32
// Gauss-Jordan matrix (or its panel multipliers) and the FP64 final-inverse
// area alias
__host__ __device__ __forceinline__ int planes_bytes_of(int WB) {
  const int two = 2 * bufbytes_of(WB);
  return ((two > MX_FP64_AREA ? two : MX_FP64_AREA) + 1023) & ~1023;
}

// shared-memory layout: two operand buffers (the Gauss-Jordan areas alias
// them), then the small arrays
__device__ __forceinline__ MxShared mx_layout(unsigned char* smraw, int WB) {
  MxShared s;
  const int bb = bufbytes_of(WB);
  s.buf[0] = smraw;
  s.buf[1] = smraw + bb;
  s.gj = reinterpret_cast<float2*>(smraw);
  s.mult = reinterpret_cast<float2*>(smraw);
  unsigned char* tail = smraw + planes_bytes_of(WB);
  s.colbuf = reinterpret_cast<float2*>(tail);
  s.rowbuf = s.colbuf + MX_MAXN;
  s.recip = s.rowbuf + MX_MAXN;
  s.perm = reinterpret_cast<int*>(s.recip + MX_PANEL);
  s.cols = s.perm + MX_MAXN;
  s.expA = s.cols + MX_MAXN;              // 2 MX_MAXN: the rows of a row-stacked product
  s.expB = s.expA + 2 * MX_MAXN;
  s.red = reinterpret_cast<float*>(s.expB + MX_MAXN);
  s.mbar = reinterpret_cast<uint64_t*>(s.red + 32);
  s.tslot = reinterpret_cast<uint32_t*>(s.mbar + 2);
  s.misc = reinterpret_cast<int*>(s.tslot + 2);
  return s;
}

// a pointer into the dynamic shared memory, re-derived from the shared array
// itself so that accesses through it compile to shared-memory instructions
// (pointers read back from MxShared are generic)
template <class T>
__device__ __forceinline__ T* shm(const MxShared& s, T* p) {
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  return reinterpret_cast<T*>(smem_dyn + (reinterpret_cast<const unsigned char*>(p) - s.buf[0]));
}

struct MxState {           // per-thread copies of the (uniform) pipeline counters
  uint32_t tmem;
  uint32_t ncommit[2];
  uint32_t nwaited[2];
  int abort;
  unsigned spin;           // pipeline waits' bound (0 = built-in; see mbar_wait)
};

__device__ __forceinline__ void buffer_ready(MxShared& s, MxState& st, int b) {
  if (st.ncommit[b] > st.nwaited[b]) {
    if (!mbar_wait(&s.mbar[b], (st.ncommit[b] - 1) & 1, st.spin)) {
      st.abort = 1;        // the buffer's MMAs stay pending: only the teardown waits for them
      return;
    }
    st.nwaited[b] = st.ncommit[b];
  }
}


// row exponents of X (over re and im) into expA, column exponents of Y into
// expB: biased-exponent maxima by integer max.  Warp w walks columns w, w+8,
// ... with its lanes on consecutive rows (coalesced); no integer division.
// A part whose flag is off keeps what the previous product left (the same
// operand on the same side).
__device__ void oz_exponents(const double2* __restrict__ X, const double2* __restrict__ Y, int N,
                             MxShared& s, bool rows, bool cols, const double2* __restrict__ Xlo = nullptr) {
  const int M = Xlo ? 2 * N : N;         // rows N.. of a row-stacked product come from Xlo
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  if (rows) {
  for (int r = threadIdx.x; r < M; r += blockDim.x) s.expA[r] = 0;
  __syncthreads();
  // rows in slabs of 32 MX_ROWS (a stacked product has up to 2 MX_MAXN)
  for (int r0 = 0; r0 < M; r0 += 32 * MX_ROWS) {
    int rmax[MX_ROWS];
#pragma unroll
    for (int m = 0; m < MX_ROWS; ++m) rmax[m] = 0;
    // two columns of X per step so that twice the loads are in flight
    for (int k = warp; k < N; k += 2 * nwarp) {
      const size_t c0 = (size_t)k * N, c1 = (size_t)min(k + nwarp, N - 1) * N;
      const bool two = k + nwarp < N;
#pragma unroll
      for (int m = 0; m < MX_ROWS; ++m) {
        const int i = r0 + lane + 32 * m;
        if (i < M) {
          const double2* xr = i < N ? X + i : Xlo + (i - N);
          const double2 v0 = xr[c0];
          const double2 v1 = two ? xr[c1] : v0;
          rmax[m] = max(rmax[m], max(max(bexp(v0.x), bexp(v0.y)), max(bexp(v1.x), bexp(v1.y))));
        }
      }
    }
#pragma unroll
    for (int m = 0; m < MX_ROWS; ++m)
      if (r0 + lane + 32 * m < M) atomicMax(&s.expA[r0 + lane + 32 * m], rmax[m]);
  }
  }
  if (cols)
  for (int j = warp; j < N; j += 2 * nwarp) {
    const int j1 = j + nwarp;
    const double2* yc0 = Y + (size_t)j * N;
    const double2* yc1 = Y + (size_t)min(j1, N - 1) * N;
    int c0 = 0, c1 = 0;
    for (int k = lane; k < N; k += 32) {
      const double2 v0 = yc0[k];
      const double2 v1 = yc1[k];
      c0 = max(c0, max(bexp(v0.x), bexp(v0.y)));
      c1 = max(c1, max(bexp(v1.x), bexp(v1.y)));
    }
    c0 = __reduce_max_sync(0xffffffffu, c0);
    c1 = __reduce_max_sync(0xffffffffu, c1);
    if (lane == 0) {
      s.expB[j] = c0;
      if (j1 < N) s.expB[j1] = c1;
    }
  }
  __syncthreads();
}

// BF16x2 bits of ((g0 - 64) * 2^s, (g1 - 64) * 2^s) for biased digits g in
// [0, 192], element signs in sgn (bits 15 and 31).  (2^23 + g) * 2^s -
// (2^23 + 64) * 2^s by one FFMA is (g - 64) * 2^s exactly, an integer of at
// most 8 significant bits times a power of two, so the BF16 value is the
// float's upper half; the element's sign flips the digit's own.
__device__ __forceinline__ uint32_t dig2f(uint32_t g0, uint32_t g1, float sc, float off,
                                          uint32_t sgn) {
  const float f0 = __fmaf_rn(__uint_as_float(0x4B000000u | g0), sc, off);
  const float f1 = __fmaf_rn(__uint_as_float(0x4B000000u | g1), sc, off);
  return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632) ^ sgn;
}

// biased digit p (1 = most significant) of g = f + DIGIT_BIAS split as hi =
// bits 21.., lo = bits 0..20; the leading digit keeps every bit above 42 (g < 2^50)
template <int P>
__device__ __forceinline__ uint32_t digit7(uint32_t hi, uint32_t lo) {
  return P == 1 ? hi >> 21 : P <= 4 ? (hi >> (7 * (4 - P))) & 127u : (lo >> (7 * (7 - P))) & 127u;
}

// 2^e as a float constant
__host__ __device__ constexpr float pow2f(int e) {
  return e >= 0 ? (float)(1ull << (e < 63 ? e : 62)) : 1.0f / (float)(1ull << (-e));
}

// the D (7 or 4) leading digit planes (real and imaginary) of one element
// pair, stored at dst + plane * pstride (words); scale 2^(7 (e0 - p)) for plane
// p.  The digits are balanced (the leading one in [0, 128], the others in
// [-64, 63]); D = 4 keeps the four leading ones, the operand rounded to 28 bits.
template <int E0, int D>
__device__ __forceinline__ void put_digits(uint32_t* dst, int pstride, unsigned long long fr0,
                                           unsigned long long fr1, unsigned long long fi0,
                                           unsigned long long fi1, uint32_t sr, uint32_t si) {
  fr0 += DIGIT_BIAS;
  fr1 += DIGIT_BIAS;
  fi0 += DIGIT_BIAS;
  fi1 += DIGIT_BIAS;
  const uint32_t hr0 = (uint32_t)(fr0 >> 21), lr0 = (uint32_t)fr0 & 0x1FFFFFu;
  const uint32_t hr1 = (uint32_t)(fr1 >> 21), lr1 = (uint32_t)fr1 & 0x1FFFFFu;
  const uint32_t hi0 = (uint32_t)(fi0 >> 21), li0 = (uint32_t)fi0 & 0x1FFFFFu;
  const uint32_t hi1 = (uint32_t)(fi1 >> 21), li1 = (uint32_t)fi1 & 0x1FFFFFu;
#define WTG_PUT(P)                                                                          \
  {                                                                                          \
    constexpr float sc = pow2f(7 * (E0 - P)), off = -(8388608.0f + 64.0f) * sc;             \
    dst[(2 * (P - 1)) * pstride] =                                                           \
        dig2f(digit7<P>(hr0, lr0), digit7<P>(hr1, lr1), sc, off, sr);                        \
    dst[(2 * (P - 1) + 1) * pstride] =                                                       \
        dig2f(digit7<P>(hi0, li0), digit7<P>(hi1, li1), sc, off, si);                        \
  }
  WTG_PUT(1) WTG_PUT(2) WTG_PUT(3) WTG_PUT(4)
  if constexpr (D > 4) {
    WTG_PUT(5) WTG_PUT(6) WTG_PUT(7)
  }
#undef WTG_PUT
}

// the B digit planes of one element pair, in two runs: Yr, Yi of digit q at
// planes 2(q-1), +1 and -Yi, Yr at 2D + 2(q-1), +1, so that [Yr; Yi] and
// [-Yi; Yr] of g consecutive digits are each one operand of 2wg rows (oz_issue);
// -Yi is Yi with both BF16 sign bits flipped.  D leading balanced digits (7 or
// 4), as put_digits.
template <int D>
__device__ __forceinline__ void put_digits_b(uint32_t* dst, int pstride, unsigned long long fr0,
                                             unsigned long long fr1, unsigned long long fi0,
                                             unsigned long long fi1, uint32_t sr, uint32_t si) {
  fr0 += DIGIT_BIAS;
  fr1 += DIGIT_BIAS;
  fi0 += DIGIT_BIAS;
  fi1 += DIGIT_BIAS;
  const uint32_t hr0 = (uint32_t)(fr0 >> 21), lr0 = (uint32_t)fr0 & 0x1FFFFFu;
  const uint32_t hr1 = (uint32_t)(fr1 >> 21), lr1 = (uint32_t)fr1 & 0x1FFFFFu;
  const uint32_t hi0 = (uint32_t)(fi0 >> 21), li0 = (uint32_t)fi0 & 0x1FFFFFu;
  const uint32_t hi1 = (uint32_t)(fi1 >> 21), li1 = (uint32_t)fi1 & 0x1FFFFFu;
#define WTG_PUTB(P)                                                                         \
  {                                                                                          \
    constexpr float sc = pow2f(7 * (5 - P)), off = -(8388608.0f + 64.0f) * sc;              \
    const uint32_t br = dig2f(digit7<P>(hr0, lr0), digit7<P>(hr1, lr1), sc, off, sr);       \
    const uint32_t bi = dig2f(digit7<P>(hi0, li0), digit7<P>(hi1, li1), sc, off, si);       \
    dst[(2 * (P - 1)) * pstride] = br;                                                       \
    dst[(2 * (P - 1) + 1) * pstride] = bi;                                                   \
    dst[(2 * D + 2 * (P - 1)) * pstride] = bi ^ 0x80008000u;                                 \
    dst[(2 * D + 2 * (P - 1) + 1) * pstride] = br;                                           \
  }
  WTG_PUTB(1) WTG_PUTB(2) WTG_PUTB(3) WTG_PUTB(4)
  if constexpr (D > 4) {
    WTG_PUTB(5) WTG_PUTB(6) WTG_PUTB(7)
  }
#undef WTG_PUTB
}

// digit planes of chunk [k0, k0+16) into buffer b: A = rows [rb0, rb0+128) of
// X, B = columns [jb, jb+width) of Y (as rows of the K-major B^T layout).
// Work item `it` covers rows (or columns) 8 (it >> 6) + (lane >> 2) and K pair
// 8 ((it >> 5) & 1) + 2 (lane & 3); in the canonical layout its word sits at
// byte 4 it of a plane, so each warp store fills one 128-byte core matrix
// (no bank conflicts).  Generated by threads gtid = 0 .. gthreads-1.  D digits.
template <int D>
__device__ void oz_generate(const double2* __restrict__ X, const double2* __restrict__ Y, int N,
                            int WB, int k0, int rb0, int jb, int width, const MxShared& s, int b,
                            int gtid, int gthreads, const double2* __restrict__ Xlo) {
  const int M = Xlo ? 2 * N : N;         // rows N.. of a row-stacked product come from Xlo
  unsigned char* __restrict__ A = shm(s, s.buf[b]);
  unsigned char* __restrict__ B = A + 2 * NSL * APLANE;
  const int* __restrict__ expA = shm(s, s.expA);
  const int* __restrict__ expB = shm(s, s.expB);
  const int bstride = width * KCH * 2 / 4;        // B plane stride in words (= pass width)
  for (int it = gtid; it < 128 * (KCH / 2); it += gthreads) {
    const int cm = it >> 5, ln = it & 31;
    const int il = (cm >> 1) * 8 + (ln >> 2), kk = (cm & 1) * 8 + (ln & 3) * 2, i = rb0 + il;
    uint32_t* dst = reinterpret_cast<uint32_t*>(A) + it;
    if (i >= M) {                                  // padding rows of the M = 128 tile
#pragma unroll
      for (int pl = 0; pl < 2 * D; ++pl) dst[pl * (APLANE / 4)] = 0u;
      continue;
    }
    const int E = expA[i];
    const double2* xr = i < N ? X + i : Xlo + (i - N);
    double2 x0 = make_double2(0.0, 0.0), x1 = x0;
    if (k0 + kk < N) x0 = xr[(size_t)(k0 + kk) * N];
    if (k0 + kk + 1 < N) x1 = xr[(size_t)(k0 + kk + 1) * N];
    unsigned n0r, n0i, n1r, n1i;
    const unsigned long long f0r = fixed49(x0.x, E, n0r), f0i = fixed49(x0.y, E, n0i);
    const unsigned long long f1r = fixed49(x1.x, E, n1r), f1i = fixed49(x1.y, E, n1i);
    put_digits<3, D>(dst, APLANE / 4, f0r, f1r, f0i, f1i, (n0r << 15) | (n1r << 31),
                     (n0i << 15) | (n1i << 31));
  }
  for (int it = gtid; it < width * (KCH / 2); it += gthreads) {
    const int cm = it >> 5, ln = it & 31;
    const int jl = (cm >> 1) * 8 + (ln >> 2), kk = (cm & 1) * 8 + (ln & 3) * 2, j = jb + jl;
    uint32_t* dst = reinterpret_cast<uint32_t*>(B) + it;
    if (j >= N) {                                  // padding columns
#pragma unroll
      for (int pl = 0; pl < 4 * D; ++pl) dst[pl * bstride] = 0u;
      continue;
    }
    const int F = expB[j];
    double2 y0 = make_double2(0.0, 0.0), y1 = y0;
    if (k0 + kk < N) y0 = Y[(k0 + kk) + (size_t)j * N];
    if (k0 + kk + 1 < N) y1 = Y[(k0 + kk + 1) + (size_t)j * N];
    unsigned n0r, n0i, n1r, n1i;
    const unsigned long long f0r = fixed49(y0.x, F, n0r), f0i = fixed49(y0.y, F, n0i);
    const unsigned long long f1r = fixed49(y1.x, F, n1r), f1i = fixed49(y1.y, F, n1i);
    put_digits_b<D>(dst, bstride, f0r, f1r, f0i, f1i, (n0r << 15) | (n1r << 31),
                    (n0i << 15) | (n1i << 31));
  }
}

// all slice-pair MMAs of one chunk (thread 0 only).  The descriptors' start
// address field holds (address >> 4) in its low 14 bits, so a plane offset is
// added to a base descriptor directly.  Both components in two MMAs per group
// of slice pairs: Xr [Yr; Yi] and Xi [-Yi; Yr] accumulate [Cr | Ci].  Slice
// order t = p + q goes to accumulator t - 2 while that is one of the nexact
// exact ones and to the last (lumped) accumulator above; accumulator a sits at
// tensor-memory column 2 w a.  For one digit p of X, the pairs of g
// consecutive digits q whose orders go to g consecutive accumulators are one
// MMA of N = 2 w g <= 256 over the B planes of those digits (stored side by
// side, put_digits_b): the A planes are read once for the group.  amask holds
// the accumulators already written in this pass: the first MMA into one
// overwrites, so a group takes accumulators that are all new or all written
// (digit p = 1 reaches every accumulator first).  D digits: slice pairs
// p + q <= D + 1.
template <int D>
__device__ void oz_issue(const MxShared& s, uint32_t tmem, int b, int width, int nacc, int nexact,
                         uint32_t& amask) {
  const uint32_t A = saddr(s.buf[b]);
  const uint32_t B = A + 2 * NSL * APLANE;
  const uint64_t bplane16 = (uint64_t)width * KCH * 2 >> 4;
  const uint64_t adesc0 = sdesc(A), bdesc0 = sdesc(B);
  const int gmax = 128 / width;                  // 2 w g <= 256 columns
#pragma unroll 1
  for (int p = 1; p <= D; ++p) {
    const uint64_t aR = adesc0 + (uint64_t)(2 * (p - 1)) * (APLANE >> 4);
    const uint64_t aI = aR + (APLANE >> 4);
    int q = 1;
#pragma unroll 1
    while (q + p <= D + 1) {
      const int t0 = p + q;
      const int a0 = t0 - 2 < nexact ? t0 - 2 : nacc - 1;
      const uint32_t touched = (amask >> a0) & 1u;
      int g = 1;
      while (g < gmax && q + g + p <= D + 1) {
        const int t = t0 + g;
        const int a = t - 2 < nexact ? t - 2 : nacc - 1;
        if (a != a0 + g || ((amask >> a) & 1u) != touched) break;
        ++g;
      }
      const uint32_t d = tmem + (uint32_t)(a0 * 2 * width);
      const uint64_t bRI = bdesc0 + (uint64_t)(2 * (q - 1)) * bplane16;           // [Yr; Yi] ...
      const uint64_t bNR = bdesc0 + (uint64_t)(2 * D + 2 * (q - 1)) * bplane16;   // [-Yi; Yr] ...
      const uint32_t id = idesc(2 * width * g, 0);
      amask |= ((1u << g) - 1u) << a0;
      mma_bf16(d, aR, bRI, id, touched);
      mma_bf16(d, aI, bNR, id, 1u);
      q += g;
    }
  }
}

// |re + i im| in FP64 (Fortran's abs of a complex(dp)); hypot's scaling only
// outside the range where the squares neither overflow nor underflow
__device__ __forceinline__ double cabs64(double re, double im) {
  const double a = fabs(re), b = fabs(im), h = fmax(a, b);
  if (h < 0x1p500 && h > 0x1p-500) return sqrt(fma(a, a, b * b));
  return h == 0.0 ? 0.0 : hypot(a, b);
}

// C = X * Y through the epilogue; returns this thread's partial of sum |C|:
// OZ_STORE_NORM (the decimation's convergence norm) sums each |C_ij|, both in
// FP64; OZ_IMINUS (the refinement residual) sums |re| + |im| in FP32.
// out0/out1/src: FP64 N x N column-major.
// REUSE bit 0: X is the previous product's X (its row exponents are in expA);
// bit 1: Y is the previous product's Y (column exponents in expB).
constexpr int REUSE_X = 1, REUSE_Y = 2;

// Rows N .. 2N-1 of a row-stacked product: X' Y with its own left factor,
// epilogue (EPI2 of oz_gemm) and outputs, in the 128-row tiles that follow the
// first product's rows (the first product's last, partly filled tile takes the
// first rows of X').  Each output element sees the same digits and the same
// MMA sums as in a product of its own.
struct OzLower {
  const double2* X;
  double2* out0;
  double2* out1;
  const double2* src;
};

template <int EPI, int EPI2 = -1, int D = NSL>
__device__ double oz_gemm(const double2* __restrict__ X, const double2* __restrict__ Y,
                          const MxPlan& pl, double2* out0, double2* out1, const double2* src,
                          MxShared& s, MxState& st, int reuse = 0, OzLower lo = OzLower{}) {
  const int N = pl.N, tid = threadIdx.x;
  const bool stacked = EPI2 >= 0;
  const int M = stacked ? 2 * N : N;       // rows of the tile that hold outputs
  const int nch = (N + KCH - 1) / KCH;
  const int nacc = pl.nacc, WB = pl.wb;
  const int npass = pl.ncb;
  float nrm = 0.f;
  double nrm_d = 0.0;
  oz_exponents(X, Y, N, s, !(reuse & REUSE_X), !(reuse & REUSE_Y), stacked ? lo.X : nullptr);
  __syncthreads();
  const int nrb = stacked ? (M + 127) / 128 : pl.nrb;
  for (int rb = 0; rb < nrb && !st.abort; ++rb) {
    const int rb0 = rb * 128;
    for (int pass = 0; pass < npass && !st.abort; ++pass) {
      const int cbi = pass;
      const int jb = cbi * pl.w0;
      const int width = min(pl.w0, pl.NP - jb);
      uint32_t amask = 0u;
      for (int c = 0; c < nch; ++c) {
        const int b = c & 1;
        if (tid >= 32) {     // warps 1.. generate while warp 0 issues the previous chunk
          buffer_ready(s, st, b);
          if (!st.abort)
            oz_generate<D>(X, Y, N, WB, c * KCH, rb0, jb, width, s, b, tid - 32, blockDim.x - 32,
                           stacked ? lo.X : nullptr);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        st.abort = __syncthreads_or(st.abort);
        tc_fence_after();
        if (st.abort) break;
        if (tid == 0) {
          oz_issue<D>(s, st.tmem, b, width, nacc, nacc - pl.lumped, amask);
          mma_commit(&s.mbar[b]);
        }
        st.ncommit[b] += 1;
      }
      // all MMAs of this pass: the last commit covers every earlier one
      const int bl = (nch - 1) & 1;
      if (!st.abort && !mbar_wait(&s.mbar[bl], (st.ncommit[bl] - 1) & 1, st.spin)) st.abort = 1;
      if (!st.abort) {
        st.nwaited[0] = st.ncommit[0];
        st.nwaited[1] = st.ncommit[1];
      }
      st.abort = __syncthreads_or(st.abort);
      tc_fence_after();
      const int* __restrict__ expB = shm(s, s.expB);
      const int* __restrict__ expA = shm(s, s.expA);
      for (int comp = 0; comp < 2 && !st.abort; ++comp) {
        const int warp = tid >> 5, lane = tid & 31;
        const int quad = warp & 3, hw = warp >> 2;
        const int row = rb0 + quad * 32 + lane;
        // a warp whose 32 tensor-memory lanes are all padding rows has nothing to drain
        const int nhw = blockDim.x >> 7;
        const int cb = hw * 4, ce = rb0 + quad * 32 < M ? width : 0;
        const int er = row < M ? expA[row] : 0;
        // the lower rows of a stacked product: their own epilogue and outputs
        const bool upper = !stacked || row < N;
        const int epi = upper ? EPI : EPI2;
        const int rowL = upper ? row : row - N;
        double2* const o0b = upper ? out0 : lo.out0;
        double2* const o1b = upper ? out1 : lo.out1;
        const double2* const srcb = upper ? src : lo.src;
        const uint32_t bank = (uint32_t)(comp * width);
        for (int c0 = cb; c0 < ce; c0 += 4 * nhw) {
          uint32_t v[6][4];
          const uint32_t ta = st.tmem + bank + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
#pragma unroll
          for (int a = 0; a < 6; ++a)
            if (a < nacc) tmem_ld4(ta + (uint32_t)(a * 2 * width), v[a]);
          tmem_wait_ld();
          if (row < M) {
            double old0[4], old1[4];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {            // the epilogue's loads first
              const int j = jb + c0 + jj;
              const size_t idx = (size_t)rowL + (size_t)j * N;
              old0[jj] = 0.0;
              old1[jj] = 0.0;
              if (j < N) {
                if (epi == OZ_ADD2) {
                  old0[jj] = reinterpret_cast<const double*>(o0b + idx)[comp];
                  old1[jj] = reinterpret_cast<const double*>(o1b + idx)[comp];
                } else if (epi == OZ_ADDTO) {
                  old0[jj] = reinterpret_cast<const double*>(srcb + idx)[comp];
                } else if ((epi == OZ_STORE_NORM || epi == OZ_IMINUS) && comp == 1) {
                  old0[jj] = o0b[idx].x;
                }
              }
            }
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              const int j = jb + c0 + jj;
              if (j < N) {
                long long S = 0;
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                  if (a >= nacc) continue;
                  if (pl.lumped && a == nacc - 1) {
                    S += f2ll_bits(v[a][jj]);               // lumped orders >= 7
                  } else {
                    // exact order t: the value is m 2^(56-7t) with |m| < 2^24
                    const int t = a + 2;
                    const float sc = __int_as_float((127 + 7 * t - 56) << 23);
                    S += (long long)__float2int_rz(__uint_as_float(v[a][jj]) * sc) << (49 - 7 * t);
                  }
                }
                const double val = assemble(S, er + expB[j] - 1070);
                const size_t idx = (size_t)rowL + (size_t)j * N;
                double* o0 = reinterpret_cast<double*>(o0b + idx) + comp;
                if (epi == OZ_STORE) {
                  *o0 = val;
                } else if (epi == OZ_ADD2) {
                  *o0 = old0[jj] + val;
                  *(reinterpret_cast<double*>(o1b + idx) + comp) = old1[jj] + val;
                } else if (epi == OZ_STORE_NORM) {
                  *o0 = val;
                  if (comp == 1) nrm_d += cabs64(old0[jj], val);   // |alpha_ij| in FP64
                } else if (epi == OZ_IMINUS) {
                  double w = -val;
                  if (comp == 0 && rowL == j) w += 1.0;
                  *o0 = w;
                  if (comp == 1) nrm += fabsf(d2f_bits(old0[jj])) + fabsf(d2f_bits(w));
                } else {   // OZ_ADDTO
                  *o0 = old0[jj] + val;
                }
              }
            }
          }
        }
      }
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    }
  }
  return (EPI == OZ_STORE_NORM || EPI2 == OZ_STORE_NORM) ? nrm_d : (double)nrm;
}

__device__ float block_sum_f(float v, MxShared& s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) s.red[warp] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t += s.red[w];
    s.red[0] = t;
  }
  __syncthreads();
  t = s.red[0];
  __syncthreads();
  return t;
}

// block sum in FP64 (16 warps: the 32-float reduction area holds 16 doubles)
static_assert(MX_T / 32 <= 16, "block_sum_d keeps one double per warp in s.red");
__device__ double block_sum_d(double v, MxShared& s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* red = reinterpret_cast<double*>(s.red);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t += red[w];
    red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// entry m (warp-uniform) of a 4-entry register column, without local memory
__device__ __forceinline__ float2 pick4(const float2 (&x)[4], int m) {
  float2 v = x[0];
  v = m == 1 ? x[1] : v;
  v = m == 2 ? x[2] : v;
  v = m == 3 ? x[3] : v;
  return v;
}

__device__ __forceinline__ float2 shfl_f2c(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Gauss-Jordan without physical row swaps: row i of the working matrix stays
// in place and pos_of[i] / row_at[q] record the position it would hold in the
// swapped form.  Step t's pivot is the first maximal |re| + |im| of column t
// over the rows at positions >= t (izamax's rule in position order), so the
// pivots, and every FMA of every entry, are those of the swapped form; only
// the storage order differs.  Publishes the multiplier column (column t as it
// stands), the pivot's position (perm[t]) and physical row (misc[2 + (t & 1)])
// and its reciprocal, and moves the pivot to position t.
__device__ __forceinline__ void gj_pivot_publish_u(const float2 (&x)[4], int t, int N, float2* cb,
                                                float2* recip, int* perm, int* misc, int* pos_of,
                                                int* row_at) {
  const int lane = threadIdx.x & 31;
  int bkey = -1, bpos = 0x7fffffff, brow = N;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int i = lane + 32 * m;
    if (i < N) {
      const int ps = pos_of[i];
      const int key = __float_as_int(fabsf(x[m].x) + fabsf(x[m].y));
      if (ps >= t && (key > bkey || (key == bkey && ps < bpos))) {
        bkey = key;
        bpos = ps;
        brow = i;
      }
    }
  }
  {  // warp maximum of the key, then the smallest position among the lanes that hold it
    const unsigned kmax = __reduce_max_sync(0xffffffffu, (unsigned)(bkey + 1));
    const bool cand = (unsigned)(bkey + 1) == kmax;
    const int pmin = (int)__reduce_min_sync(0xffffffffu, cand ? (unsigned)bpos : 0xffffffffu);
    const int src = __ffs(__ballot_sync(0xffffffffu, cand && bpos == pmin)) - 1;
    brow = __shfl_sync(0xffffffffu, brow, src);
    bkey = (int)kmax - 1;
    bpos = pmin;
  }
  const float2 xp = shfl_f2c(pick4(x, brow >> 5), brow & 31);
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int i = lane + 32 * m;
    if (i < N) cb[i] = x[m];
  }
  if (lane == 0) {
    perm[t] = bpos;
    misc[2 + (t & 1)] = brow;
    const int rk = row_at[t];            // the row at position t moves to the pivot's position
    row_at[bpos] = rk;
    pos_of[rk] = bpos;
    row_at[t] = brow;
    pos_of[brow] = t;
    if (bkey == 0) {
      misc[1] = 1;
    } else {
      const float inv_d = 1.0f / (xp.x * xp.x + xp.y * xp.y);
      recip[t & 1] = make_float2(xp.x * inv_d, -xp.y * inv_d);
    }
  }
}

// M = w I - X (FP64, kept in Mi for the refinement), then FP32 Gauss-Jordan
// into G (FP64).  Returns 1 on an exact zero pivot (G = identity then).
// Ndim <= 112.  Each pivot step is one pass in which every warp takes whole
// columns into registers (lane l holds rows l, l+32, ...): the pivot-row
// scaling and the elimination of a column happen in registers with one
// shuffle pair.  Rows stay in place (gj_pivot_publish_u), so an entry needs
// one select besides its four FMAs; the output reads the rows back in pivot
// order.  The warp that owns column k+1 also finds step k+1's pivot
// (look-ahead) and publishes its multiplier column into the other of two
// buffers, so a step needs one barrier.  Same operations per entry as the
// step-by-step form with row swaps.
__device__ __noinline__ int gj32_start(const double2* __restrict__ X, double2 w, int N, double2* Mi,
                          double2* G, MxShared& s_) {
  const int T = blockDim.x, tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = T >> 5;
  // pointers re-derived from the dynamic shared-memory array, so that the
  // compiler emits shared-memory (not generic) loads and stores
  float2* __restrict__ sM = shm(s_, s_.gj);
  float2* const cb0 = shm(s_, s_.colbuf);   // multiplier columns of even / odd steps
  float2* const cb1 = shm(s_, s_.rowbuf);
  float2* __restrict__ recip = shm(s_, s_.recip);
  int* __restrict__ perm = shm(s_, s_.perm);
  int* __restrict__ cols = shm(s_, s_.cols);
  int* __restrict__ misc = shm(s_, s_.misc);
  int* __restrict__ pos_of = shm(s_, s_.expA);   // the exponent arrays are free here
  int* __restrict__ row_at = shm(s_, s_.expB);
  for (int j = warp; j < N; j += nwarp) {
    for (int i = lane; i < N; i += 32) {
      const size_t e = (size_t)i + (size_t)j * N;
      const double2 x = X[e];
      double2 m = make_double2(-x.x, -x.y);
      if (i == j) m = make_double2(w.x - x.x, w.y - x.y);
      Mi[e] = m;
      sM[e] = make_float2(d2f_bits(m.x), d2f_bits(m.y));
    }
  }
  for (int i = tid; i < N; i += T) {
    pos_of[i] = i;
    row_at[i] = i;
  }
  if (tid == 0) misc[1] = 0;
  __syncthreads();
  if (warp == 0) {                        // step 0's pivot
    float2 x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = lane + 32 * m;
      x[m] = i < N ? sM[i] : make_float2(0.f, 0.f);
    }
    gj_pivot_publish_u(x, 0, N, cb0, recip, perm, misc, pos_of, row_at);
  }
  __syncthreads();
  for (int k = 0; k < N; ++k) {
    if (misc[1]) break;
    const int p = misc[2 + (k & 1)];        // the pivot's row
    const float2 r = recip[k & 1];
    const float2* cb = (k & 1) ? cb1 : cb0;
    float2* cbn = (k & 1) ? cb0 : cb1;
    float2 f[4];                          // this lane's multipliers
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = lane + 32 * m;
      f[m] = i < N ? cb[i] : make_float2(0.f, 0.f);
    }
    for (int j = warp; j < N; j += nwarp) {
      float2* col = sM + (size_t)j * N;
      float2 x[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int i = lane + 32 * m;
        x[m] = i < N ? col[i] : make_float2(0.f, 0.f);
      }
      float2 nk = r;
      if (j == k) {                       // the pivot column becomes a column of the inverse
#pragma unroll
        for (int m = 0; m < 4; ++m) x[m] = make_float2(0.f, 0.f);
      } else {
        const float2 apj = shfl_f2c(pick4(x, p >> 5), p & 31);
        nk = make_float2(fmaf(apj.x, r.x, -apj.y * r.y), fmaf(apj.x, r.y, apj.y * r.x));
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int i = lane + 32 * m;
        float2 v = x[m];
        v.x = fmaf(-f[m].x, nk.x, v.x);
        v.x = fmaf(f[m].y, nk.y, v.x);
        v.y = fmaf(-f[m].x, nk.y, v.y);
        v.y = fmaf(-f[m].y, nk.x, v.y);
        x[m] = (i == p) ? nk : v;
        if (i < N) col[i] = x[m];
      }
      if (j == k + 1) gj_pivot_publish_u(x, k + 1, N, cbn, recip, perm, misc, pos_of, row_at);
    }
    __syncthreads();
  }
  const int singular = misc[1];
  if (tid == 0) {
    for (int j = 0; j < N; ++j) cols[j] = j;
    if (!singular) {
      for (int k = N - 1; k >= 0; --k) {
        const int p = perm[k];
        const int t = cols[k];
        cols[k] = cols[p];
        cols[p] = t;
      }
    }
  }
  __syncthreads();
  for (int j = warp; j < N; j += nwarp) {
    const int cj = cols[j];
    for (int i = lane; i < N; i += 32) {
      const size_t e = (size_t)i + (size_t)j * N;
      if (singular) {
        G[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
      } else {
        const float2 v = sM[row_at[i] + (size_t)cj * N];
        G[e] = make_double2(f2d_bits(v.x), f2d_bits(v.y));
      }
    }
  }
  __syncthreads();
  return singular;
}

template <int R>
__device__ __forceinline__ float2 pick_f(const float2 (&x)[R], int m) {
  float2 v = x[0];
#pragma unroll
  for (int q = 1; q < R; ++q)
    if (q == m) v = x[q];
  return v;
}

__device__ __forceinline__ float2 shfl_f2(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// gj_pivot_publish_u for a column of R rows per lane (rows lane + 32 m): the
// multiplier column goes to cb, the reciprocal to *rslot, the pivot's row to
// prow[t]
template <int R>
__device__ __forceinline__ void gj_pivot_publish_ur(const float2 (&x)[R], int t, int N, float2* cb,
                                                 float2* rslot, int* perm, int* prow, int* misc,
                                                 int* pos_of, int* row_at) {
  const int lane = threadIdx.x & 31;
  int bkey = -1, bpos = 0x7fffffff, brow = N;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int i = lane + 32 * m;
    if (i < N) {
      const int ps = pos_of[i];
      const int key = __float_as_int(fabsf(x[m].x) + fabsf(x[m].y));
      if (ps >= t && (key > bkey || (key == bkey && ps < bpos))) {
        bkey = key;
        bpos = ps;
        brow = i;
      }
    }
  }
  {  // warp maximum of the key, then the smallest position among the lanes that hold it
    const unsigned kmax = __reduce_max_sync(0xffffffffu, (unsigned)(bkey + 1));
    const bool cand = (unsigned)(bkey + 1) == kmax;
    const int pmin = (int)__reduce_min_sync(0xffffffffu, cand ? (unsigned)bpos : 0xffffffffu);
    const int src = __ffs(__ballot_sync(0xffffffffu, cand && bpos == pmin)) - 1;
    brow = __shfl_sync(0xffffffffu, brow, src);
    bkey = (int)kmax - 1;
    bpos = pmin;
  }
  const float2 xp = shfl_f2(pick_f<R>(x, brow >> 5), brow & 31);
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int i = lane + 32 * m;
    if (i < N) cb[i] = x[m];
  }
  if (lane == 0) {
    perm[t] = bpos;
    prow[t] = brow;
    const int rk = row_at[t];
    row_at[bpos] = rk;
    pos_of[rk] = bpos;
    row_at[t] = brow;
    pos_of[brow] = t;
    if (bkey == 0) {
      misc[1] = 1;
    } else {
      const float inv_d = 1.0f / (xp.x * xp.x + xp.y * xp.y);
      *rslot = make_float2(xp.x * inv_d, -xp.y * inv_d);
    }
  }
}

// one Gauss-Jordan step k (pivot row p, reciprocal r, multiplier column cm in
// shared memory) applied to column j held in registers, rows in place
template <int R>
__device__ __forceinline__ void gj_step_col_u(float2 (&x)[R], const float2* __restrict__ cm, int N,
                                              int j, int k, int p, float2 r) {
  const int lane = threadIdx.x & 31;
  float2 nk = r;
  if (j == k) {
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = make_float2(0.f, 0.f);
  } else {
    const float2 apj = shfl_f2(pick_f<R>(x, p >> 5), p & 31);
    nk = make_float2(fmaf(apj.x, r.x, -apj.y * r.y), fmaf(apj.x, r.y, apj.y * r.x));
  }
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int i = lane + 32 * m;
    const float2 f = i < N ? cm[i] : make_float2(0.f, 0.f);
    float2 v = x[m];
    v.x = fmaf(-f.x, nk.x, v.x);
    v.x = fmaf(f.y, nk.y, v.x);
    v.y = fmaf(-f.x, nk.y, v.y);
    v.y = fmaf(-f.y, nk.x, v.y);
    x[m] = (i == p) ? nk : v;
  }
}

// As gj32_start for Ndim above the shared-memory limit: the FP32 matrix lives
// in global memory (Wf, N x N float2) and the pivot steps run in panels of
// MX_PANEL columns.  A panel's columns stay in registers (warp w owns panel
// column w, lane l rows l, l+32, ..., R rows per lane); each step updates them with
// one barrier, the owner of the next column publishing the next pivot and its
// multiplier column (look-ahead).  Then every other column is read once into
// registers, put through the panel's steps in order and written back.  Rows
// stay in place as in gj32_start.
template <int R>
__device__ __noinline__ int gj32_global(const double2* __restrict__ X, double2 w, int N, double2* Mi,
                           double2* G, float2* __restrict__ Wf, MxShared& s_) {
  const int T = blockDim.x, tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = T >> 5;
  float2* __restrict__ Cm = shm(s_, s_.mult);
  float2* __restrict__ recip = shm(s_, s_.recip);
  int* __restrict__ perm = shm(s_, s_.perm);
  int* __restrict__ cols = shm(s_, s_.cols);
  int* __restrict__ misc = shm(s_, s_.misc);
  int* const prow = cols;                        // pivot rows during the steps
  int* __restrict__ pos_of = shm(s_, s_.expA);   // the exponent arrays are free here
  int* __restrict__ row_at = shm(s_, s_.expB);
  for (int j = warp; j < N; j += nwarp) {
    for (int i = lane; i < N; i += 32) {
      const size_t e = (size_t)i + (size_t)j * N;
      const double2 x = X[e];
      double2 m = make_double2(-x.x, -x.y);
      if (i == j) m = make_double2(w.x - x.x, w.y - x.y);
      Mi[e] = m;
      Wf[e] = make_float2(d2f_bits(m.x), d2f_bits(m.y));
    }
  }
  for (int i = tid; i < N; i += T) {
    pos_of[i] = i;
    row_at[i] = i;
  }
  if (tid == 0) misc[1] = 0;
  __syncthreads();
  for (int k0 = 0; k0 < N; k0 += MX_PANEL) {
    const int pb = min(MX_PANEL, N - k0);
    float2 xc[2][R];                // this warp's panel columns warp, warp + nwarp
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      const int c = warp + cc * nwarp;
#pragma unroll
      for (int m = 0; m < R; ++m) {
        const int i = lane + 32 * m;
        xc[cc][m] = (c < pb && i < N) ? Wf[(size_t)(k0 + c) * N + i] : make_float2(0.f, 0.f);
      }
    }
    if (warp == 0) gj_pivot_publish_ur<R>(xc[0], k0, N, Cm, &recip[0], perm, prow, misc, pos_of, row_at);
    __syncthreads();
    for (int t = 0; t < pb; ++t) {
      if (misc[1]) break;
      const int k = k0 + t, p = prow[k];
      const float2 r = recip[t];
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const int c = warp + cc * nwarp;
        if (c < pb) {
          gj_step_col_u<R>(xc[cc], Cm + t * N, N, k0 + c, k, p, r);
          if (c == t + 1)
            gj_pivot_publish_ur<R>(xc[cc], k + 1, N, Cm + (t + 1) * N, &recip[t + 1], perm, prow, misc,
                                   pos_of, row_at);
        }
      }
      __syncthreads();
    }
    if (misc[1]) break;
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {       // panel columns back to memory
      const int c = warp + cc * nwarp;
      if (c < pb) {
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const int i = lane + 32 * m;
          if (i < N) Wf[(size_t)(k0 + c) * N + i] = xc[cc][m];
        }
      }
    }
    // every column outside the panel through the panel's steps, in registers
    for (int j = warp; j < N; j += nwarp) {
      if (j >= k0 && j < k0 + pb) continue;
      float2* col = Wf + (size_t)j * N;
      float2 x[R];
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int i = lane + 32 * q;
        x[q] = i < N ? col[i] : make_float2(0.f, 0.f);
      }
      for (int t = 0; t < pb; ++t) gj_step_col_u<R>(x, Cm + t * N, N, j, k0 + t, prow[k0 + t], recip[t]);
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int i = lane + 32 * q;
        if (i < N) col[i] = x[q];
      }
    }
    __syncthreads();
  }
  const int singular = misc[1];
  if (tid == 0) {
    for (int j = 0; j < N; ++j) cols[j] = j;
    if (!singular) {
      for (int k = N - 1; k >= 0; --k) {
        const int p = perm[k];
        const int t = cols[k];
        cols[k] = cols[p];
        cols[p] = t;
      }
    }
  }
  __syncthreads();
  for (int j = warp; j < N; j += nwarp) {
    const int cj = cols[j];
    for (int i = lane; i < N; i += 32) {
      const size_t e = (size_t)i + (size_t)j * N;
      if (singular) {
        G[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
      } else {
        const float2 v = Wf[row_at[i] + (size_t)cj * N];
        G[e] = make_double2(f2d_bits(v.x), f2d_bits(v.y));
      }
    }
  }
  __syncthreads();
  return singular;
}

// (w I - X)^-1 into *Gp: FP32 Gauss-Jordan, then Newton-Schulz steps
// G <- G + G (I - M G) on the split tensor-core products until the residual
// sum_ij |I - M G|_1 stops shrinking quadratically, or is at most brk N before
// an update (after which it is ~(brk N)^2; brk = 1e-7 puts it below the
// products' own rounding); at most ns_max steps.  Uses Mi, R, Gn as work;
// swaps *Gp and *Gn.
__device__ int mixed_inverse(const double2* X, double2 w, const MxPlan& pl, int ns_max,
                             double2** Gp, double2** Gnp, double2* Mi, double2* R, MxShared& s,
                             MxState& st, float brk = 1e-7f) {
  const int N = pl.N;
  float2* const Wf = reinterpret_cast<float2*>(R);
  const int sing = N <= MX_SMEM_GJ_N ? gj32_start(X, w, N, Mi, *Gp, s)
                   : N <= 160        ? gj32_global<5>(X, w, N, Mi, *Gp, Wf, s)
                   : N <= 224        ? gj32_global<7>(X, w, N, Mi, *Gp, Wf, s)
                                     : gj32_global<MX_ROWS>(X, w, N, Mi, *Gp, Wf, s);
  float prev = 3.0e38f;
  for (int t = 0; t < ns_max && !st.abort; ++t) {
    const float part = (float)oz_gemm<OZ_IMINUS>(Mi, *Gp, pl, R, nullptr, nullptr, s, st);  // R = I - M G
    const float res = block_sum_f(part, s);
    if (!(res < 0.25f * prev)) break;                 // no longer converging (or NaN)
    // Gn = G + G R: R is small, so 4 digits (28 bits) keep G R far below G's own error
    oz_gemm<OZ_ADDTO, -1, 4>(*Gp, R, mx_plan4(pl), *Gnp, nullptr, *Gp, s, st);
    double2* tmp = *Gp;
    *Gp = *Gnp;
    *Gnp = tmp;
    if (res <= brk * (float)N) break;                 // G + G R is then accurate enough
    prev = res;
  }
  return sing;
}

// tensor-memory allocation and mbarriers of a CTA (all threads)
__device__ void mx_setup(MxShared& s, MxState& st, unsigned spin_limit) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&s.mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&s.mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((tid >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(s.tslot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  st.tmem = *s.tslot;
  st.ncommit[0] = st.ncommit[1] = 0;
  st.nwaited[0] = st.nwaited[1] = 0;
  st.abort = 0;
  st.spin = spin_limit;
}

// every committed MMA must finish before tensor memory is released: these
// waits keep the built-in bound whatever a test set for the pipeline's waits
__device__ void mx_teardown(MxShared& s, MxState& st) {
  for (int b = 0; b < 2; ++b)
    if (st.ncommit[b] > st.nwaited[b]) mbar_wait(&s.mbar[b], (st.ncommit[b] - 1) & 1, 0u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(st.tmem), "r"(512));
}

// Decimation of one instance whose eps, eps_s, eps_t (= H00), alpha (= H01)
// and beta (= H01^dagger) already sit in workspace matrices 0..4 of W (11
// N x N matrices); the spectral sums go to emit(dl, dr, db, spin[6],
// iterations, status) in thread 0, the final inverses to gll / grr / gb when
// those are not null.  o has DecimArgs' member names (lists, tolerance, ...).
// The loop's products and inverses are the split-BF16 forms; the three final
// inverses (src/surfgreen.f90:127-134) are FP64 Gauss-Jordan, the FP64 form's
// own (gj_invert in shared memory up to MX_SMEM_GJ_N, gj_invert_global in
// workspace matrix 8 above), in an area that aliases the idle operand buffers.
template <class O, class Emit>
__device__ __forceinline__ void mixed_solve(const MxPlan& pl, double2 w, const O& o, int ns_iter,
                                            double2* gll, double2* grr, double2* gb, double2* W,
                                            MxShared& s, MxState& st, Emit emit) {
  const int N = pl.N, NN = N * N, tid = threadIdx.x;
  double2* E = W;
  double2* ES = W + (size_t)NN;
  double2* ET = W + (size_t)2 * NN;
  double2* Al = W + (size_t)3 * NN;
  double2* Be = W + (size_t)4 * NN;
  double2* G = W + (size_t)5 * NN;
  double2* M1 = W + (size_t)6 * NN;
  double2* M2 = W + (size_t)7 * NN;
  double2* Mi = W + (size_t)8 * NN;
  double2* R = W + (size_t)9 * NN;
  double2* Gn = W + (size_t)10 * NN;
  int stat = 0, it = 0;
  bool conv = false;
  for (int itc = 1; itc <= o.itermax && !st.abort; ++itc) {   // src/surfgreen.f90:86-122
    it = itc;
    // the refinement stops at a residual sum of 1e-4 Ndim (then ~1e-8 after its
    // update): the dense Fermi-arc check stays below 2e-6 against the FP64 oracle
    if (mixed_inverse(E, w, pl, ns_iter, &G, &Gn, Mi, R, s, st, 1e-4f)) stat |= PT_SINGULAR;
    // the reference's six products (:92-116), ordered so that each shares an
    // operand with the one before it and reuses its exponents; eps still
    // receives M1 beta before M2 alpha.  Where it takes fewer 128-row tiles
    // (Ndim mod 128 in 1..64: up to Ndim 64, or 129..192, 257..320), the
    // products with a common right factor run as one product whose rows are
    // those of the first and then those of the second: three products instead
    // of six.
    double part;
    if ((2 * N + 127) / 128 < 2 * ((N + 127) / 128)) {
      oz_gemm<OZ_STORE, OZ_STORE>(Al, G, pl, M1, nullptr, nullptr, s, st, 0,
                                  OzLower{Be, M2, nullptr, nullptr});               // :92, :95
      oz_gemm<OZ_ADD2, OZ_STORE>(M1, Be, pl, E, ES, nullptr, s, st, 0,
                                 OzLower{M2, R, nullptr, nullptr});                 // :98-102, :116
      part = oz_gemm<OZ_STORE_NORM, OZ_ADD2>(M1, Al, pl, Gn, nullptr, nullptr, s, st, REUSE_X,
                                             OzLower{M2, E, ET, nullptr});          // :113, :107-110
    } else {
      oz_gemm<OZ_STORE>(Al, G, pl, M1, nullptr, nullptr, s, st);                     // :92
      oz_gemm<OZ_STORE>(Be, G, pl, M2, nullptr, nullptr, s, st, REUSE_Y);            // :95
      oz_gemm<OZ_ADD2>(M1, Be, pl, E, ES, nullptr, s, st);                           // :98-102
      part = oz_gemm<OZ_STORE_NORM>(M1, Al, pl, Gn, nullptr, nullptr, s, st, REUSE_X);  // :113
      oz_gemm<OZ_ADD2>(M2, Al, pl, E, ET, nullptr, s, st, REUSE_Y);                  // :107-110
      oz_gemm<OZ_STORE>(M2, Be, pl, R, nullptr, nullptr, s, st, REUSE_X);            // :116
    }
    double2* t0 = Al;
    Al = Gn;
    Gn = t0;
    double2* t1 = Be;
    Be = R;
    R = t1;
    const double nrm = block_sum_d(part, s);     // :120-122, summed and tested in FP64
    if (nrm <= o.tol) {
      conv = true;
      break;
    }
  }
  if (!conv) stat |= PT_NOT_CONVERGED;

  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  const bool gsm = N <= MX_SMEM_GJ_N;
  const Shared fs = fp64_layout(smem_dyn, N, GJ_PANEL, gsm);
  // (w - X)^-1 in FP64, optionally stored un-permuted to dst; ginv reads the
  // result.  blk 1 / 2: only the leading / trailing nw x nw block (one principal
  // layer), by the Schur complement of the rest (schur_block_invert), where the
  // spectral sums read nothing else; a zero pivot there takes the full inverse.
  const int m = N - o.nw;
  // above MX_SMEM_GJ_N the elimination runs in workspace matrix 8 and the
  // block's inverse in shared memory, when the block fits the area
  const bool gblk = !gsm && schur_area_bytes(N, o.nw) <= MX_FP64_AREA;
  const Shared fb = schur_layout(smem_dyn, N, o.nw);
  int blk = 0;
  auto invert = [&](const double2* X, double2* dst, int want_blk) -> int {
    __syncthreads();                  // the area aliases buffers the loop just used
    blk = ((gsm || gblk) && !dst && m > 0) ? want_blk : 0;
    if (blk && !(gsm ? schur_block_invert(X, w, N, o.nw, blk == 1, fs)
                     : schur_block_invert_global(X, w, N, o.nw, blk == 1, Mi, fb)))
      return 0;
    blk = 0;
    int sing;
    if (gsm) {
      sing = gj_invert(X, w, N, fs);
      if (dst) gj_store(N, fs, dst);
    } else {
      sing = gj_invert_global(X, w, N, Mi, fs);
      if (dst) gj_store_global(N, Mi, fs, dst);
    }
    return sing;
  };
  auto ginv = [&](int i, int j) {
    if (blk) {                        // block entry (i, j): local indices in the block
      const int li = blk == 1 ? o.nw - 1 - i : i - m;
      const int lj = blk == 1 ? o.nw - 1 - j : j - m;
      return gsm ? fs.big[m + li + (size_t)(m + fs.cols[lj]) * N]
                 : fb.big[li + (size_t)fb.cols[lj] * o.nw];
    }
    return gsm ? fs.big[i + fs.cols[j] * N] : Mi[i + (size_t)fs.cols[j] * N];
  };
  double dl = 0.0, dr = 0.0, db = 0.0;
  double spin[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (invert(ES, gll, 1)) stat |= PT_SINGULAR;                // :127-128
  if (tid == 0) {
    for (int q = 0; q < o.ntop; ++q) {
      const int io = o.top[q] - 1;
      const double v = ginv(io, io).y;
      dl = o.divide_by_pi ? dl - v / PI_REF : dl - v;
    }
    if (o.spin[0]) spin_sums(ginv, o.nw, o.ntop, o.top, 0, o.divide_by_pi, spin[0], spin[1], spin[2]);
  }
  __syncthreads();
  // surfstat's spin sums read GRR's leading block as well (src/surfstat.f90:178-192)
  if (invert(ET, grr, (o.spin[0] && !o.spin_right_bottom) ? 0 : 2))    // :130-131
    stat |= PT_SINGULAR;
  if (tid == 0) {
    for (int q = 0; q < o.nbot; ++q) {
      const int io = N - o.nw + o.bot[q] - 1;
      const double v = ginv(io, io).y;
      dr = o.divide_by_pi ? dr - v / PI_REF : dr - v;
    }
    if (o.spin[0]) {
      if (o.spin_right_bottom)
        spin_sums(ginv, o.nw, o.nbot, o.bot, N - o.nw, o.divide_by_pi, spin[3], spin[4], spin[5]);
      else
        spin_sums(ginv, o.nw, o.ntop, o.top, 0, o.divide_by_pi, spin[3], spin[4], spin[5]);
    }
  }
  __syncthreads();
  if (invert(E, gb, 0)) stat |= PT_SINGULAR;                  // :133-134
  if (tid == 0) {
    for (int i = 0; i < N; ++i) {
      const double v = ginv(i, i).y;
      db = o.divide_by_pi ? db - v / PI_REF : db - v;
    }
    if (st.abort) stat |= PT_TIMEOUT;
    if (!isfinite(dl) || !isfinite(dr) || !isfinite(db)) stat |= PT_NONFINITE;
    emit(dl, dr, db, spin, it, stat);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(MX_T, 1) k_decimate_mixed(const __grid_constant__ DecimArgs a,
                                                            int ns_iter, unsigned spin_limit) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  const int N = a.N, NN = N * N, T = blockDim.x, tid = threadIdx.x;
  const MxPlan pl = mx_plan(N, a.w0);
  MxShared s = mx_layout(smraw, pl.wb);
  MxState st;
  mx_setup(s, st, spin_limit);
  double2* W = a.ws + (size_t)blockIdx.x * 11 * NN;
  for (;;) {
    if (tid == 0) s.misc[0] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int inst = s.misc[0];
    __syncthreads();
    if (inst >= a.n_inst) break;
    const int ik = inst / a.nomega, iw = inst % a.nomega;
    if (st.abort) {        // a wait gave up earlier: the rest of this CTA's points are not computed
      if (tid == 0) {
        const size_t oidx = (size_t)(a.k_offset + ik) + (size_t)iw * a.nk_total;
        const double nan = __longlong_as_double(0x7FF8000000000000LL);
        a.dos_l[oidx] = nan;
        a.dos_r[oidx] = nan;
        a.dos_bulk[oidx] = nan;
        if (a.spin[0])
          for (int c = 0; c < 6; ++c) a.spin[c][oidx] = nan;
        if (a.iters) a.iters[oidx] = 0;
        if (a.status) a.status[oidx] = (uint8_t)PT_TIMEOUT;
      }
      continue;
    }
    const double2* H00 = a.h + (size_t)ik * 2 * NN;
    const double2* H01 = H00 + NN;
    const double2 w = make_double2(a.omega[iw], a.eta);      // src/surfgreen.f90:82
    for (int e = tid; e < NN; e += T) {                       // :74-78
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
    mixed_solve(pl, w, a, ns_iter, a.gll ? a.gll + (size_t)inst * NN : nullptr,
                a.grr ? a.grr + (size_t)inst * NN : nullptr,
                a.gb ? a.gb + (size_t)inst * NN : nullptr, W, s, st,
                [&](double dl, double dr, double db, const double* spin, int it, int stat) {
                  a.dos_l[oidx] = dl;
                  a.dos_r[oidx] = dr;
                  a.dos_bulk[oidx] = db;
                  if (a.spin[0])
                    for (int c = 0; c < 6; ++c) a.spin[c][oidx] = spin[c];
                  if (a.iters) a.iters[oidx] = it;
                  if (a.status) a.status[oidx] = (uint8_t)stat;
                });
  }
  mx_teardown(s, st);
}

// options of one batch instance, with DecimArgs' member names
struct MxOpts {
  int nw;
  double tol;
  int itermax;
  int divide_by_pi;
  int ntop, nbot;
  const int* top;
  const int* bot;
  double* spin[6];
  int spin_right_bottom;
};

// Uneven batch in one persistent launch (mixed form): as k_batch_fp64, with the
// shared-memory layout sized for the widest B plane of the batch (a.wb).
__global__ void __launch_bounds__(MX_T, 1) k_batch_mixed(const __grid_constant__ BatchArgs a,
                                                         int ns_iter, unsigned spin_limit) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  const int tid = threadIdx.x;
  MxShared s = mx_layout(smraw, a.wb);
  MxState st;
  mx_setup(s, st, spin_limit);
  double2* W = a.ws + (size_t)blockIdx.x * a.ws_stride;
  const int npts = a.run ? a.run->npts : a.npts;
  const double tol = a.run ? a.run->tol : a.tol;
  const int itermax = a.run ? a.run->itermax : a.itermax;
  const int divide_by_pi = a.run ? a.run->divide_by_pi : a.divide_by_pi;
  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.counter, 1);
      s.misc[0] = q < npts ? a.order[q] : -1;
    }
    __syncthreads();
    const int p = s.misc[0];
    __syncthreads();
    if (p < 0 || st.abort) {
      if (p >= 0 && tid == 0) {       // a wait gave up earlier: not computed
        const double nan = __longlong_as_double(0x7FF8000000000000LL);
        a.dos_l[p] = nan;
        a.dos_r[p] = nan;
        a.dos_bulk[p] = nan;
        if (a.iters) a.iters[p] = 0;
        if (a.status) a.status[p] = PT_TIMEOUT;
      }
      if (p < 0) break;
      continue;
    }
    const BatchModel& m = a.models[a.pmodel[p]];
    MxPlan pl = mx_plan(m.N, m.w0);
    pl.wb = a.wb;
    fourier_fill(m, a.k[p], a.k[p + a.npts], W, reinterpret_cast<double2*>(smraw + a.ph_off));
    MxOpts o;
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
    mixed_solve(pl, make_double2(a.omega[p], a.eta[p]), o, ns_iter, nullptr, nullptr,
                nullptr, W, s, st,
                [&](double dl, double dr, double db, const double*, int it, int stat) {
                  a.dos_l[p] = dl;
                  a.dos_r[p] = dr;
                  a.dos_bulk[p] = db;
                  if (a.iters) a.iters[p] = it;
                  if (a.status) a.status[p] = (uint8_t)stat;
                });
  }
  mx_teardown(s, st);
}

// single complex product / inverse through the same device code (one CTA)
__global__ void __launch_bounds__(MX_T, 1) k_mixed_unit(int op, int N, const double2* X,
                                                        const double2* Y, double2* C, double2* ws,
                                                        int ns, int* status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  const MxPlan pl = mx_plan(N);
  const int NN = N * N;
  MxShared s = mx_layout(smraw, pl.wb);
  const int tid = threadIdx.x;
  MxState st;
  mx_setup(s, st, 0u);
  int sing = 0;
  if (op == 0) {
    oz_gemm<OZ_STORE>(X, Y, pl, C, nullptr, nullptr, s, st);
  } else {
    // C = X^-1: X given directly, so pass -X with w = 0 (M = 0*I - (-X) = X)
    double2* negX = ws + 4 * (size_t)NN;
    for (int e = tid; e < NN; e += blockDim.x) negX[e] = make_double2(-X[e].x, -X[e].y);
    __syncthreads();
    double2* G = ws;
    double2* Gn = ws + NN;
    sing = mixed_inverse(negX, make_double2(0.0, 0.0), pl, ns, &G, &Gn, ws + 2 * (size_t)NN,
                         ws + 3 * (size_t)NN, s, st);
    for (int e = tid; e < NN; e += blockDim.x) C[e] = G[e];
  }
  if (tid == 0) *status = (st.abort ? PT_TIMEOUT : 0) | (sing ? PT_SINGULAR : 0);
  mx_teardown(s, st);
}

size_t mixed_smem(int N, int wb = 0) {     // wb = 0: the built-in plan's width
  const MxPlan pl = mx_plan(N);
  // the FP32 Gauss-Jordan matrix ((N+1)*N float2, Ndim <= MX_SMEM_GJ_N), its
  // multiplier columns (MX_MAXN * MX_PANEL float2, reserved twice) and the FP64
  // area of the final inverses all fit the planes region
  static_assert((MX_SMEM_GJ_N + 1) * MX_SMEM_GJ_N * 8 <= MX_FP64_AREA, "FP32 GJ area");
  static_assert(2 * MX_MAXN * MX_PANEL * 8 <= MX_FP64_AREA, "FP32 GJ panel area");
  const size_t planes = (size_t)planes_bytes_of(wb > 0 ? wb : pl.w0);
  return planes + (size_t)MX_MAXN * 8 * 2 + MX_PANEL * 8 + (size_t)MX_MAXN * 4 * 5 + 32 * 4 +
         16 + 8 + 16;
}

}  // namespace

int decim_mixed_max_n() { return MX_MAXN; }

size_t decim_mixed_ws_matrices() { return 11; }

cudaError_t decim_mixed_config(int N, DecimConfig* cfg) {
  cfg->threads = MX_T;
  cfg->KC = 0;
  cfg->RP = 0;
  cfg->w0 = mx_plan(N, tile_value(1, N)).w0;
  // at least 116 KB so that two CTAs never share an SM (each allocates all 512 TMEM columns)
  const size_t sm = mixed_smem(N, cfg->w0);
  cfg->smem = sm > (size_t)(116 << 10) ? sm : (size_t)(116 << 10);
  cudaError_t e = cudaFuncSetAttribute(k_decimate_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)cfg->smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_decimate_mixed, MX_T, cfg->smem);
  if (e != cudaSuccess) return e;
  cfg->ctas_per_sm = occ > 1 ? 1 : occ;     // tensor memory is allocated whole (512 columns)
  return cudaSuccess;
}

cudaError_t launch_decimate_mixed(const DecimArgs& a, const DecimConfig& cfg, int grid,
                                  cudaStream_t s) {
  k_decimate_mixed<<<grid, cfg.threads, cfg.smem, s>>>(
      a, 6, (unsigned)test_option(WTG_TEST_MIXED_SPIN_LIMIT));
  return cudaGetLastError();
}

cudaError_t batch_mixed_config(int max_n, int* wb, DecimConfig* cfg) {
  if (max_n > MX_MAXN) return cudaErrorInvalidValue;
  int w = 16;
  size_t smem = 0;
  for (int n = 1; n <= max_n; ++n) {
    const int wn = mx_plan(n, tile_value(1, n)).w0;
    w = w > wn ? w : wn;
  }
  for (int n = 1; n <= max_n; ++n) {
    const size_t t = mixed_smem(n, w);
    smem = smem > t ? smem : t;
  }
  *wb = w;
  cfg->threads = MX_T;
  cfg->KC = 0;
  cfg->RP = 0;
  cfg->inv_global = 0;
  cfg->smem = smem > (size_t)(116 << 10) ? smem : (size_t)(116 << 10);
  cfg->ctas_per_sm = 1;
  return cudaSuccess;
}

// as batch_fp64_prepare
cudaError_t batch_mixed_prepare() {
  static std::mutex mu;
  static bool done[64];
  int dev = 0, optin = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && done[dev]) return cudaSuccess;
  cudaFuncAttributes fa;
  err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, k_batch_mixed);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_batch_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               optin - (int)fa.sharedSizeBytes);
  if (err == cudaSuccess && dev < 64) done[dev] = true;
  return err;
}

cudaError_t launch_batch_mixed(const BatchArgs& a, const DecimConfig& cfg, int grid,
                               cudaStream_t s) {
  k_batch_mixed<<<grid, cfg.threads, cfg.smem, s>>>(
      a, 6, (unsigned)test_option(WTG_TEST_MIXED_SPIN_LIMIT));
  return cudaGetLastError();
}

int batch_mixed_w0(int N) { return mx_plan(N, tile_value(1, N)).w0; }

int mixed_w0_default(int N) { return mx_plan(N).w0; }

int mixed_w0_max(int N) { return mx_wmax(N); }

cudaError_t launch_mixed_unit(int op, int N, const double2* X, const double2* Y, double2* C,
                              double2* ws, int ns, int* status, cudaStream_t s) {
  const size_t smem = mixed_smem(N) > (size_t)(116 << 10) ? mixed_smem(N) : (size_t)(116 << 10);
  cudaError_t e =
      cudaFuncSetAttribute(k_mixed_unit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_mixed_unit<<<1, MX_T, smem, s>>>(op, N, X, Y, C, ws, ns, status);
  return cudaGetLastError();
}

}  // namespace wtg
