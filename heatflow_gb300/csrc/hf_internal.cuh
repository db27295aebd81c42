// Internal declarations shared by the CUDA translation units of libheatflow_gb300.
//
// Data layout in HBM (per context, all instances concatenated, cell order x fastest):
//   static operator (FP64): diag, cx, cy, cz   -- geometric SoA form of the reference's COO H
//                                                 (c_a[I] = face to the + neighbour, periodic wrap)
//   scaled operator:         sinv = 1/sqrt|diag| (FP64), a64{x,y,z} = c_a[I]*sinv[I]*sinv[E_a(I)]
//                            (FP64) and the same in FP32 (a32{x,y,z}) for the mixed inner solve
//   static RHS terms (FP64): rhoc, ccat = tau'*rhoc, bvec (boundary vector B), optional heater
//                            arrays (int8 case, FP64 power, FP64 radiative coefficient)
//   state (FP64):            four temperature buffers whose roles (T^n, T^(n-1), x read,
//                            x write) rotate per instance without copies
//   solver (FP64/FP32):      b, y, r, p, q (FP64 CG on the scaled operator) or their FP32 twins
//
// Per-instance scalars live in device memory (InstScal) so that every kernel is launch-argument
// free of solver state and the step loop can be captured in a CUDA graph.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/heatflow_gb300.h"

namespace hf {

constexpr double kTiny = 1.0e-12;            // mod_constants.f90:17
constexpr double kPi = 3.141592653589793;    // mod_constants.f90:12
constexpr double kStefBoltz = 5.670373e-8;   // mod_constants.f90:16

constexpr int kBlock = 256;                  // threads per block of the cell kernels
constexpr int kCellsPerThread = 4;
constexpr int kTile = kBlock * kCellsPerThread;   // cells per tile (one block per tile)
constexpr int kNR = 8;
// Step kernels work on tasks: a block of 32 x kTY threads owns kXC*32 x kTY columns of one
// instance (one warp per row; lane L holds columns x0 + L + 32 j, j < kXC) and marches the task
// depth (InstDesc::zc planes, an option; kZC by default) along z.  (kXC > 1 trades occupancy for
// per-thread parallelism; on GB300 kXC = 1 is faster.)
constexpr int kXC = 1, kTX = 32 * kXC, kTY = 8, kZC = 32;
// Instances with more tasks than this have their task partials summed by a whole block, the
// others by one warp.
constexpr int kWarpSumMax = 512;
constexpr int kMinTaskDepth = 4;   // task buffers are sized for the shallowest task depth
// InstScal::status bit: some S was NaN; the failing vector is found by the diagnosis kernel.
constexpr int kStatusRhsNan = 1 << 16;                       // reduction slots per tile
// Instances are laid out at multiples of kTile cells, so tile t covers cells
// [t*kTile, (t+1)*kTile) of exactly one instance; cells past an instance's end are padding.

// Static description of one instance (read-only on the device).
struct InstDesc {
  int64_t off;        // first global cell
  int32_t nx, ny, nz, n;
  int64_t tile0;      // first tile
  int32_t ntiles;
  int32_t px, py, pz; // periodic flags
  int32_t icattaneo, isteady;
  int32_t heater;     // any iheater > 0 (heater() is called, mod_evolve.f90:79)
  int32_t has_power;  // per-cell POWER array present
  int32_t has_em;     // any emissivity != 0
  int32_t qdens_mode;
  int32_t has_case5;  // some cell uses heater case 5 (needs tau)
  double inv_dt, time_step, freq, power_in, time_pulse, t_bath, heated_volume, volume;
  double len[3];
  double mean_sinv;   // mean of 1/sqrt|H_II| (scaling of the FP32 inner right-hand side)
  int64_t task0;      // first task of the step kernels
  int32_t ntask;      // tasks of this instance
  int32_t zc;         // planes per task (the task depth)
  int64_t hoff;       // first cell in the compact host layout (instances back to back, no padding)
  // The FP32 vectors of the inner solve (a32x/y/z, y32, r32, p32, p232, q32) use their own layout:
  // rows of sx = nx rounded up to 4 cells (the padding cells hold zeros), so every grid takes the
  // 16-byte vector passes; instance at off4, a multiple of kTile cells.  sx = nx: the FP64 layout.
  int64_t off4;
  int32_t sx;
  int32_t pad4;
};

// Per-instance mutable scalars (device memory).
struct InstScal {
  double bb;          // ||b||^2 (unscaled S)
  double rr_true;     // ||b - H x||^2 of the last residual sweep
  double relres;      // sqrt(rr_true / bb)
  double gg0;         // ||g||^2 at the start of the current inner solve (scaled space)
  double rho;         // r.r (scaled) of the current inner iterate
  double pq;          // p.Ap
  double alpha, beta;
  double rr_w;        // unscaled recursive ||r||^2 (reference criterion)
  double err;         // criterion value at exit (reference `err`)
  double sigma;       // scale of the FP32 inner right-hand side
  double eta;         // relative reduction asked of the current inner solve
  int64_t iter;       // inner iterations of the current solve
  int64_t step_iters; // inner iterations of the current step
  int64_t tot_iters;  // FP64 inner iterations, all steps
  int64_t tot_inner;  // FP32 inner iterations, all steps
  int64_t tot_refine; // residual sweeps, all steps
  int64_t unconverged;
  int64_t itime;      // step index of the current step
  int64_t failed_step;
  int32_t inner_active; // inner CG running
  int32_t outer_active; // step not finished
  int32_t refine;       // refinement sweeps in this step
  int32_t x0flag;       // any(x0 - Tp < TINY) (mod_evolve.f90:141)
  int32_t status;       // bit k set: HF_ENAN_B + k raised
  int32_t devcheck;     // nonzero: a device-side consistency check failed
  int32_t tiny_pending; // x still needs the reference's +TINY (applied with the next update)
  int32_t phase;        // persistent solve: work of this instance in the current round (PH_*)
  int32_t role[4];      // temperature buffers: [0]=T^n, [1]=T^(n-1), [2]=x read, [3]=x write
  int32_t hx_role;      // hx[hx_role] = H T^n, hx[1 - hx_role] = H T^(n-1) (when hx_ok says so)
  int32_t hx_ok;        // how many of those two products are valid (trailing steps, 0..2)
  int32_t hx_fresh;     // this step's last sweep stored H x of its final x in hx[1 - hx_role]
  int32_t xw;           // fused x update: kXwAllowed | kXwThis | kXwDone bits
  double sigma_prev;    // scale used by the previous residual sweep
  double last_err, last_relres;   // of the last finished step
  int64_t last_iter;
};

// InstScal::xw.  kXwAllowed: the inner CG update may form x itself (true-residual criterion, rows
// of 4k cells: the vector form of the update, whose FP32 vectors index like x there).  kXwThis:
// the next CG update
// is predicted to be the inner solve's last and also forms x_new into role[3].  kXwDone: the last
// CG update did so and y has not changed since, so the separate x update is skipped.
constexpr int32_t kXwThis = 1, kXwDone = 2, kXwAllowed = 4;

// Device-side control of a captured step (CUDA graph with conditional nodes).
struct CtrlState {
  int64_t itime;      // step index of the next step
  int64_t loop_iter;  // body iterations of the current step's solve loop
  int64_t limit;      // bound on body iterations per step (termination guarantee)
  int32_t guard_hit;  // the bound was reached (reported as HF_EDEVICE)
  uint32_t fin_count; // finalize blocks arrived (last one sets the loop condition)
  int64_t launches;   // kernels the captured steps launched
  int64_t itime_end;  // one past the last step of a whole-loop graph launch
};

// Phases of an instance inside the persistent solve kernel (one per grid-wide round).
enum : int32_t {
  PH_IDLE = HF_PHASE_IDLE,          // step finished (or failed): nothing to do
  PH_START = HF_PHASE_START,        // reserved
  PH_RES_INIT = HF_PHASE_RES_INIT,  // r = S - H x0 (x0 + TINY), g, norms
  PH_CG_P = HF_PHASE_CG_P,          // p = r + beta p                      (FP64 inner solve)
  PH_CG_Q = HF_PHASE_CG_Q,          // q = Ah p, p.q                        (FP64 inner solve)
  PH_CG_PQ = HF_PHASE_CG_PQ,        // p = r + beta p and q = Ah p fused    (FP32 inner solve)
  PH_CG_B = HF_PHASE_CG_B,          // y += alpha p, r -= alpha q, r.r
  PH_XUPD = HF_PHASE_XUPD,          // x += sigma S^-1 y (+ TINY once)
  PH_RES = HF_PHASE_RES             // true residual of the updated x
};

// Control block of one launch of the persistent solve kernel (zeroed before every launch).
constexpr int kRoundLog = 512;                     // rounds whose end time is recorded
struct SolveCtl {
  unsigned count;          // blocks arrived at the current grid barrier
  unsigned gen;            // barrier generation (release/acquire)
  unsigned result[2];      // "some instance has work", published by barrier parity
  int32_t err;             // a barrier wait gave up (time limit): the launch was abandoned
  int32_t guard_hit;       // the round bound was reached
  int32_t pad;
  unsigned next_task[2];   // tasks handed out in the current round (by round parity)
  int64_t rounds;          // rounds run
  unsigned long long t_start;                 // %globaltimer at kernel start (ns)
  unsigned long long t_round[kRoundLog];      // %globaltimer when round r's barrier opened
  int32_t phase_log[kRoundLog];               // phase instance 0 ran in round r
};

// Options mirrored on the device.
struct DevOpts {
  int32_t precision, criterion;
  double tol;
  int64_t itmax;
  double inner_tol;
  int32_t inner_itmax, max_refine;
};

// Device pointers of a context (passed by value to kernels).
struct DevArrays {
  const InstDesc* inst;
  InstScal* scal;
  const int32_t* tile_inst;
  double* partials;       // ntasks * kNR partial sums, one fixed slot range per task
  unsigned int* counters; // per instance, last-block detection
  DevOpts opts;
  // static
  double *diag, *cx, *cy, *cz, *sinv, *a64x, *a64y, *a64z;
  double* rsum;           // H*1 per cell (residual of x0 + TINY from that of x0)
  float* sinv32;          // FP32 copy of sinv (scaling of FP32 right-hand sides/corrections)
  float *a32x, *a32y, *a32z;
  double *rhoc, *ccat, *bvec, *power, *emc;
  // -rho c / dt - 2 tau' rho c per cell (-rho c / dt in Fourier mode): S = T^n scoef + ccat T^(n-1)
  // - Qdens - B, the RHS's form under the true-residual criterion (fewer FP64 roundings)
  double* scoef;
  int8_t* icase;
  double* tau_s;          // tau/dt^2 (heater case 5)
  // state: four temperature-sized buffers, roles per instance in InstScal::role
  double* tbuf[4];
  // H T^n and H T^(n-1), stored by the final residual sweep of each step: the next step's first
  // residual is then S - H x0 = S - 2 H T^n + H T^(n-1), pointwise (x0 = 2 T^n - T^(n-1))
  double* hx[2];
  // step timeline: %globaltimer when the kernels of the latest step started (kStamp* slots)
  unsigned long long* stamps;
  // solver
  double *b, *y, *r, *p, *q, *p2;
  float *y32, *r32, *p32, *q32, *p232;   // p / p2: search directions, ping-pong by iteration
  const int8_t* task_heat;  // per task: some cell holds a heater
  const int4* tasks;        // (instance, x0, y0, z0) per task
  int64_t ncells, ntiles, ninst, ntasks;
  int64_t nsmall;           // instances with at most kWarpSumMax tasks (their partials: one warp)
  const int32_t* large;     // the other instances (block sums), nlarge of them
  int64_t nlarge;
  // index-check record of the checked build (HF_CHECKED): [0] failed checks, [1] site of the
  // first, [2] its index, [3] the extent it was checked against
  unsigned long long* check;
  // host-buffer steps (the graphs of hf_step_host_async only, null elsewhere): the residual
  // sweeps after an update also store x here, in the compact layout (InstDesc::hoff), so the
  // step's result needs no gather for its download
  double* xout;
};

// ---- index checks of the checked build ----------------------------------------------------------
// Compiled with -DHF_CHECKED (build_library(checked=True): a separate library for tests), every
// global load and store of the step kernels takes its index through HF_IX (one cell) or HF_IX4 (a
// 4-cell vector, which must also start on a multiple of 4 cells: a 16-byte boundary for FP32, two
// for FP64).  An index outside [0, n) -- n the extent of that array in the instance's layout -- is
// recorded in DevArrays::check and replaced by 0, so the access stays inside the array and the
// kernel goes on: no trap, no fault.  The host reports a record as HF_EDEVICE (the site is
// 100000 * file + line).  In the normal build both macros are the index itself.
#ifdef HF_CHECKED
__device__ __noinline__ inline long long hf_check_ix(unsigned long long* rec, int site, long long i,
                                                     long long n, int vec) {
  const bool ok = i >= 0 && i + vec <= n && (vec == 1 || (i & (vec - 1)) == 0);
  if (ok) return i;
  if (rec) {
    const unsigned long long k = atomicAdd(rec, 1ull);
    if (k == 0ull) {
      rec[1] = (unsigned long long)site;
      rec[2] = (unsigned long long)i;
      rec[3] = (unsigned long long)n;
    }
  }
  return 0;
}
#define HF_SITE (HF_FILE_ID * 100000 + __LINE__)
#define HF_IX(A, i, n) ((int)hf_check_ix((A).check, HF_SITE, (long long)(i), (long long)(n), 1))
#define HF_IX4(A, i, n) ((int)hf_check_ix((A).check, HF_SITE, (long long)(i), (long long)(n), 4))
#else
#define HF_IX(A, i, n) (i)
#define HF_IX4(A, i, n) (i)
#endif

// Slots of DevArrays::stamps: step begin, RHS start, RHS finalize start, solve start, end of the
// solve's last round, step end.
enum { kStampBegin = 0, kStampRhs, kStampFin, kStampSolve, kStampSolveEnd, kStampEnd, kStamps = 8 };

// Ask L2 for the line holding p (no register, no result): planes a pass streams in its next z
// steps, so their DRAM latency overlaps the current step's work at the persistent solve's 3 blocks
// per SM.  Only ever given addresses inside the arrays (planes the task itself reads next).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- helpers ---------------------------------------------------------------------------------
// IEEE-754 bit access through inline PTX, so that tests and format conversions stay integer
// instructions instead of being turned back into FP64 compares/conversions: on GB300 the FP64
// pipe (~1 TFLOP/s) is the scarce resource of every FP64 kernel.
__device__ __forceinline__ unsigned long long dbits(double v) {
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
  return b;
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
  double v;
  asm("mov.b64 %0, %1;" : "=d"(v) : "l"(b));
  return v;
}
__device__ __forceinline__ bool dbl_is_zero(double v) { return (dbits(v) << 1) == 0ull; }
__device__ __forceinline__ bool dbl_is_nan(double v) {
  const unsigned long long b = dbits(v);
  return ((b >> 52) & 0x7ffull) == 0x7ffull && (b & 0xfffffffffffffull) != 0ull;
}
// v < t for finite t > 0 and non-NaN v (sign-magnitude order of the bit patterns).
__device__ __forceinline__ bool dbl_lt_pos(double v, double t) {
  const long long b = (long long)dbits(v);
  return b < 0 || (unsigned long long)b < dbits(t);
}
// FP64 -> FP32 by truncation of the mantissa (integer instructions only).  Magnitudes outside
// the FP32 normal range saturate to 0 or infinity; NaN stays NaN.
__device__ __forceinline__ float f64_to_f32_trunc(double v) {
  const unsigned long long u = dbits(v);
  const unsigned sign = (unsigned)(u >> 63) << 31;
  const int e = (int)((u >> 52) & 0x7ffull);
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((u & 0xfffffffffffffull) ? 0x400000u : 0u));
  const int fe = e - 1023 + 127;
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)((u >> 29) & 0x7fffffull));
}
// v * 2^-k -> FP32 by truncation of the mantissa (integer instructions only); saturates like
// f64_to_f32_trunc.  For |v| 2^-k in the FP32 normal range the result is exactly
// f64_to_f32_trunc(v) 2^-k.
__device__ __forceinline__ float f64_to_f32_trunc_pow2(double v, int k) {
  const unsigned long long u = dbits(v);
  const unsigned sign = (unsigned)(u >> 63) << 31;
  const int e = (int)((u >> 52) & 0x7ffull);
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((u & 0xfffffffffffffull) ? 0x400000u : 0u));
  if (e == 0) return __uint_as_float(sign);
  const int fe = e - 1023 + 127 - k;
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)((u >> 29) & 0x7fffffull));
}
// 2^k as an FP64 value (-1022 <= k <= 1023).
__device__ __forceinline__ double pow2d(int k) { return bitsd((unsigned long long)(1023 + k) << 52); }

// FP32 -> FP64, exact (integer instructions only).
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned e = (u >> 23) & 0xffu;
  unsigned long long m = u & 0x7fffffu;
  if (e == 0xffu) return bitsd(sign | 0x7ff0000000000000ull | (m << 29));
  if (e == 0u) {
    if (m == 0ull) return bitsd(sign);
    const int p = 31 - __clz((int)m);                  // subnormal: normalise
    const unsigned long long mant = (m << (52 - p)) & 0xfffffffffffffull;
    return bitsd(sign | ((unsigned long long)(p - 149 + 1023) << 52) | mant);
  }
  return bitsd(sign | ((unsigned long long)(e - 127 + 1023) << 52) | (m << 29));
}

// 2^m as an FP32 value for m <= 0 (subnormal below 2^-126, 0 below 2^-149).
__device__ __forceinline__ float pow2f_neg(int m) {
  if (m >= -126) return __uint_as_float((unsigned)(m + 127) << 23);
  if (m >= -149) return __uint_as_float(1u << (m + 149));
  return 0.f;
}

// Sum of squares of one thread's FP64 values in FP32 over v 2^-k, with k kept within 30 of the
// largest exponent seen (the running sum is rescaled by an exact power of two when it moves), so
// no term leaves the FP32 range and terms below 2^-60 of the largest vanish, as they would at this
// precision anyway.  Integer and FP32 instructions only: for passes bound by the FP64 pipe, whose
// FP32/integer pipes are idle.  Relative error ~1e-6, enough for norms that scale or feed threshold
// tests.  NaN and infinity propagate.
struct SqSum {
  float s = 0.f;
  int k = -2000;                  // no nonzero value yet
  __device__ __forceinline__ void add(double v) {
    const int e = (int)((dbits(v) >> 52) & 0x7ffull);
    if (e == 0) return;           // zero or subnormal: nothing at this precision
    const int ev = e - 1023;      // 1024 for infinity and NaN
    if (ev > k + 30) {
      s = k == -2000 ? 0.f : s * pow2f_neg(2 * (k - ev));
      k = ev;
    }
    const float f = f64_to_f32_trunc_pow2(v, k);
    s = fmaf(f, f, s);
  }
  __device__ __forceinline__ double value() const {
    if (k == -2000) return 0.0;
    if (!isfinite(s)) return isnan(s) ? (double)NAN : (double)INFINITY;
    return f32_to_f64(s) * pow2d(k) * pow2d(k);
  }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-reduce kNR values (all threads get nothing back; thread 0 returns the sums in out).
template <int NRV>
__device__ __forceinline__ void block_sum(double (&v)[NRV], double* smem /* [32*NRV] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NRV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NRV; ++k) smem[warp * NRV + k] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NRV; ++k) {
      double t = lane < nw ? smem[lane * NRV + k] : 0.0;
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Write this tile's partial sums (fixed slot per tile; summed by a finalize kernel).
// FP64 values go through shared memory and only warp 0 adds them (8 + 5 adds per value per
// block): on GB300 every FP64 warp instruction costs the slow FP64 pipe, so a shuffle tree in
// all eight warps would cost more than the kernel's own arithmetic.
template <int NRV>
__device__ __forceinline__ void tile_store(double* dst, const double (&v)[NRV]);
template <int NRV>
__device__ __forceinline__ void tile_store(const DevArrays& A, int64_t tile, const double (&v)[NRV]) {
  tile_store<NRV>(A.partials + tile * kNR, v);
}
// dst: the kNR partial slots of one task
template <int NRV>
__device__ __forceinline__ void tile_store(double* dst, const double (&v)[NRV]) {
  static_assert(NRV <= kNR, "reduction slots");
  __shared__ double stage[NRV][kBlock];
  __syncthreads();   // the previous tile of this block has finished reading the stage
#pragma unroll
  for (int k = 0; k < NRV; ++k) stage[k][threadIdx.x] = v[k];
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NRV; ++k) {
      double t = stage[k][lane];
#pragma unroll
      for (int w = 1; w < kBlock / 32; ++w) t += stage[k][lane + 32 * w];
      t = warp_sum(t);
      if (lane == 0) dst[k] = t;
    }
  }
}

// The columns of a task that this thread owns.
struct TCell {
  int inst;
  int64_t off;
  int nx, ny, nz, nxy;
  bool px, py, pz;
  int x0, y, z0, z1, lane;
  int64_t off4;       // the FP32 vectors' layout (rows of sx cells)
  int sx, nxy4;
  __device__ int x(int j) const { return x0 + 32 * j + lane; }
  __device__ bool act(int j) const { return x(j) < nx && y < ny; }   // column inside the grid
  __device__ int base(int j) const { return y * nx + x(j); }          // local index of (x, y, 0)
  __device__ int base4(int j) const { return y * sx + x(j); }         // the same in the FP32 layout
  __device__ int n() const { return nxy * nz; }                       // cells of the instance
  __device__ int n4() const { return nxy4 * nz; }                     // ... in the FP32 layout
};
__device__ __forceinline__ TCell task_cell(const DevArrays& A, int64_t task) {
  const int4 t = A.tasks[task];
  const InstDesc& d = A.inst[t.x];
  TCell c;
  c.inst = t.x;
  c.off = d.off;
  c.nx = d.nx; c.ny = d.ny; c.nz = d.nz; c.nxy = d.nx * d.ny;
  c.px = d.px; c.py = d.py; c.pz = d.pz;
  c.lane = threadIdx.x & 31;
  c.x0 = t.y;
  c.y = t.z + (int)(threadIdx.x >> 5);
  c.z0 = t.w;
  c.z1 = min(t.w + d.zc, d.nz);
  c.off4 = d.off4;
  c.sx = d.sx;
  c.nxy4 = d.sx * d.ny;
  return c;
}

// ---- host-side launchers (defined in the .cu files) ------------------------------------------
struct Ctx;
cudaError_t launch_assemble(Ctx& c);
cudaError_t launch_coo(Ctx& c, int64_t instance, int64_t* d_counts, int64_t* d_irow,
                       int64_t* d_jcol, double* d_val, int64_t* d_pos, int phase);
cudaError_t launch_step_begin(Ctx& c, int64_t itime, int first_of_run);
cudaError_t launch_rhs(Ctx& c);
// The RHS of tasks [t0, t1) only (their cells' inputs placed; the finalize still sums all tasks).
cudaError_t launch_rhs_range(Ctx& c, int64_t t0, int64_t t1);
cudaError_t launch_task_heat(Ctx& c);
// Tabulated properties at the current T^n, then the operator rebuilt (4 kernels).
cudaError_t launch_tempdep(Ctx& c);
cudaError_t launch_subbox_gather(Ctx& c, int64_t inst, const int64_t* lo, const int64_t* hi,
                                 int which, double* dst);
// Temperature role buffer `which` of every instance <-> a compact device array, on `stream`;
// host_in drops the stored products H T of an instance whose state it changes.
cudaError_t launch_host_in(Ctx& c, const double* src, int which, cudaStream_t stream);
// The same for the device cells [glo, ghi) (whole z-slabs of instances, padding skipped).
cudaError_t launch_host_in_range(Ctx& c, const double* src, int which, int64_t glo, int64_t ghi,
                                 cudaStream_t stream);
cudaError_t launch_stage_fallback(Ctx& c);
// Bit-for-bit check of uploaded inputs (compact layout) against the device's T^n and T^(n-1) of
// the step that just ended (roles 1 and 2 after its rotation): a difference sets *first to
// min(*first, call).  Instances whose step failed are skipped.
cudaError_t launch_host_check(Ctx& c, const double* sp, const double* spp, int64_t call,
                              int64_t* first, cudaStream_t stream);
// Control block of a one-step graph launch queued without the host (async host-buffer steps).
cudaError_t launch_ctrl_init(Ctx& c, int64_t itime, int64_t limit);
cudaError_t launch_rhs_parts(Ctx& c, double* B, double* Q, double* Qd, double* Sc);
cudaError_t launch_rhs_diagnose(Ctx& c);
cudaError_t launch_adj_rhs(Ctx& c, const double* g, const double* l1, const double* l2, double* out);
cudaError_t launch_adj_grad(Ctx& c, const double* lam, const double* x, int64_t itime,
                            double* grad_logk, double* grad_src);
cudaError_t launch_sumsq(Ctx& c, const double* b, int64_t n);
cudaError_t launch_residual(Ctx& c, int mode, CtrlState* ctrl = nullptr,
                            cudaGraphConditionalHandle hw = 0, int graph = 0);
cudaError_t launch_inner_iteration(Ctx& c, int fp32, CtrlState* ctrl = nullptr,
                                   cudaGraphConditionalHandle hw = 0, int graph = 0);
cudaError_t launch_step_end(Ctx& c);
// Persistent solve: one cooperative launch runs the whole refinement loop of a step.
cudaError_t launch_solve(Ctx& c, unsigned long long wait_ns = 4000000000ull, int leaver = -1);
int solve_grid_blocks(Ctx& c, int fp32);
cudaError_t launch_apply(Ctx& c, const double* x, double* y);
cudaError_t launch_single(Ctx& c, int which);
cudaError_t launch_graph_step_begin(Ctx& c, CtrlState* ctrl, int launches_per_step);
cudaError_t launch_graph_step_end(Ctx& c, CtrlState* ctrl, const SolveCtl* sctl,
                                  cudaGraphConditionalHandle hloop = 0, int loop = 0);
cudaError_t launch_ctrl_select(Ctx& c, CtrlState* ctrl, cudaGraphConditionalHandle hs,
                               cudaGraphConditionalHandle hw);
// Finalize kernels: sum the tile partials of each instance and run the scalar epilogue of the
// kernel that produced them.  With graph != 0 the last block also sets the loop condition hw.
enum { FIN_RHS = 0, FIN_RHS_DIAG, FIN_RES_INIT, FIN_RES, FIN_SPMV, FIN_UPD };
cudaError_t launch_finalize(Ctx& c, int kind, CtrlState* ctrl, cudaGraphConditionalHandle hw,
                            int graph);
#ifdef HF_CHECKED
cudaError_t launch_check_probe(Ctx& c);   // one failed index check, no memory access
#endif

}  // namespace hf
