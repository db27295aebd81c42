// Linear solve of one implicit step, H x = S (linbcg, mod_Sparse.f90:372-434, replaced).
//
// Method.  H is symmetric negative definite, so the reference's Jacobi-preconditioned BiCG is,
// in exact arithmetic, Jacobi-PCG (rr == r, pp == p).  The GPU runs the same iteration as plain CG
// on the symmetrically scaled operator  Ah = S^-1 (-H) S^-1,  S = diag(sqrt|H_II|), whose diagonal
// is 1: identical iterates, no divisions and one coefficient array fewer per pass.
//
// Each step is a refinement loop:
//   x = x0                                                 (RHS kernel)
//   repeat:  r = S - H x (FP64, true residual), test ||r||/||S||        k_residual
//            g = -S^-1 r / sigma ; solve Ah y = g by CG   (FP64, or FP32 in mixed mode)
//            x += sigma S^-1 y                                           k_xupdate
// The reference adds TINY to every x0 when any x0 - T < TINY (mod_evolve.f90:141).  Here the
// first residual is that of x0 + TINY, formed as r(x0) - TINY * (H 1) from a stored row-sum
// vector, and the TINY itself joins x with the first update: the same iterate, without seven
// extra FP64 additions per cell.
//
// GB300 issues FP64 at ~1 TFLOP/s, so the FP64 kernels (residual, x update, FP64 CG) are bound by
// FP64 instructions: they spend them only on the arithmetic itself (no FP64 compares, no FP64
// accumulation of FP32 quantities).  The FP32 kernels accumulate in FP32 within a block.
//
// All solver state is per instance in device memory; tiles of instances that are not in the
// phase a kernel serves return at once (per-instance convergence masks).
#include <algorithm>

#include "hf_ctx.cuh"

#define HF_FILE_ID 3   // index-check sites of the checked build: 100000 * file + line

namespace hf {

template <typename T> struct Vec;
template <> struct Vec<double> {
  __device__ static double* y(const DevArrays& A) { return A.y; }
  __device__ static double* r(const DevArrays& A) { return A.r; }
  __device__ static double* p(const DevArrays& A) { return A.p; }
  __device__ static double* pb(const DevArrays& A, int64_t k) { return (k & 1) ? A.p2 : A.p; }
  __device__ static double* q(const DevArrays& A) { return A.q; }
  __device__ static const double* ax(const DevArrays& A) { return A.a64x; }
  __device__ static const double* ay(const DevArrays& A) { return A.a64y; }
  __device__ static const double* az(const DevArrays& A) { return A.a64z; }
};
template <> struct Vec<float> {
  __device__ static float* y(const DevArrays& A) { return A.y32; }
  __device__ static float* r(const DevArrays& A) { return A.r32; }
  __device__ static float* p(const DevArrays& A) { return A.p32; }
  __device__ static float* pb(const DevArrays& A, int64_t k) { return (k & 1) ? A.p232 : A.p32; }
  __device__ static float* q(const DevArrays& A) { return A.q32; }
  __device__ static const float* ax(const DevArrays& A) { return A.a32x; }
  __device__ static const float* ay(const DevArrays& A) { return A.a32y; }
  __device__ static const float* az(const DevArrays& A) { return A.a32z; }
};

// ---- step bookkeeping ------------------------------------------------------------------------
__device__ __forceinline__ void begin_step(InstScal& s, int64_t itime) {
  s.itime = itime;
  s.outer_active = (s.status == 0) ? 1 : 0;
  s.inner_active = 0;
  s.refine = 0;
  s.iter = 0;
  s.step_iters = 0;
  s.x0flag = 0;
  s.tiny_pending = 0;
  s.err = 0.0;
  s.hx_fresh = 0;
  s.xw = 0;
  s.phase = s.outer_active ? PH_RES_INIT : PH_IDLE;   // the persistent solve's first round
}

// Finished steps rotate the temperature roles: T^(n-1) <- T^n, T^n <- x (mod_evolve.f90:169-170).
// The stored H x of the final x becomes H T^n, the previous H T^n becomes H T^(n-1); a step that
// ended without a sweep of its final x (accepted at its first residual) leaves no valid product.
__device__ __forceinline__ void end_step(InstScal& s) {
  if (s.status != 0) {
    s.hx_ok = 0;
    return;
  }
  const int r0 = s.role[0], r1 = s.role[1], r2 = s.role[2], r3 = s.role[3];
  s.role[0] = r2;  // x
  s.role[1] = r0;  // old T^n
  s.role[2] = r1;  // free
  s.role[3] = r3;  // free
  if (s.hx_fresh) {
    s.hx_role ^= 1;
    s.hx_ok = s.hx_ok < 2 ? s.hx_ok + 1 : 2;
  } else {
    s.hx_ok = 0;
  }
  s.hx_fresh = 0;
}

__global__ void k_step_begin(DevArrays A, int64_t itime) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kStamps) A.stamps[i] = i == kStampBegin ? gtimer() : 0ull;
  if (i < A.ninst) begin_step(A.scal[i], itime);
}

__global__ void k_step_end(DevArrays A) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) A.stamps[kStampEnd] = gtimer();
  if (i < A.ninst) end_step(A.scal[i]);
}

// The reference adds TINY to every x0 when any x0 - T < TINY (mod_evolve.f90:140-141) so that its
// BiCG never starts from a zero residual.  The TINY moves only the starting point: the system and
// its solution are unchanged.  Under the reference's own stopping rule (HF_STOP_RECURSIVE) the
// iterates follow linbcg's, so the TINY is applied (in the first residual as -TINY * H1, in x with
// the first update).  Under HF_STOP_TRUE every step is accepted on the true residual of its final
// x, whatever the start, and this CG treats a zero residual itself, so the TINY is skipped: one
// FP64 instruction per cell less in the first residual and in the x update (GB300's FP64 pipe
// bounds both).
__device__ __forceinline__ bool tiny_applies(const DevArrays& A, const InstScal& s) {
  return s.x0flag != 0 && A.opts.criterion == HF_STOP_RECURSIVE;
}

// ---- neighbour access for the columns of a task ------------------------------------------------
// x neighbours come from the lanes of the same warp (shuffles); lanes at a task edge, periodic
// wraps and the y neighbours are loaded; the z neighbours roll through registers as the block
// marches along z.  Inactive lanes hold zeros, so every lane can take part in the shuffles.
constexpr unsigned kFull = 0xffffffffu;

// Value and z-face of plane z0-1 of chunk j (zeros at a non-periodic bottom face).
template <typename T, typename C, class V>
__device__ __forceinline__ void plane_below(const DevArrays& A, const TCell& c, int j, V v,
                                            const C* __restrict__ cz, T& vm, C& czm) {
  vm = T(0);
  czm = C(0);
  if (!c.act(j) || c.nz < 2) return;
  int l;
  if (c.z0 > 0) l = c.base(j) + (c.z0 - 1) * c.nxy;
  else if (c.pz) l = c.base(j) + (c.nz - 1) * c.nxy;
  else return;
  vm = v(l);
  czm = cz[HF_IX(A, l, c.n())];
}

template <typename T, class V>
__device__ __forceinline__ T plane_above(const TCell& c, int j, V v, int z) {
  if (!c.act(j) || c.nz < 2) return T(0);
  if (z + 1 < c.nz) return v(c.base(j) + (z + 1) * c.nxy);
  if (c.pz) return v(c.base(j));
  return T(0);
}

// FP32 block sum of one value into partial slot k of a task (one conversion per block).
__device__ __forceinline__ void task_store_f(double* dst, int k, float v) {
  __shared__ float red[kBlock / 32];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < kBlock / 32 ? red[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (lane == 0) dst[k] = (double)v;
  }
}

// ---- task bodies ---------------------------------------------------------------------------------
// Each body does one kernel's work for one task; the standalone kernels (host-polled loop, the
// conditional-node graph, kernel timing) and the persistent solve kernel call the same bodies, so
// every path computes the same bits.  Vectors that some phase of the persistent kernel writes
// (temperature buffers, CG vectors) are read through plain pointers: within one launch they change
// between rounds, so they must not be taken for read-only data.  The operator, S and the scalings
// do not change during a solve and are read through const __restrict__ pointers.
//
// Loads are issued ahead of their use by hand (next plane of a stencil, four planes of an
// element-wise pass), because the compiler may not move a load above a store to a vector it cannot
// prove distinct.

// x-neighbour loads of a column (offsets from the cell, or kNoNbr): lane 0 loads its west
// neighbour, lane 31 its east neighbour, and a last column of a periodic axis its wrap; all other
// x neighbours come from the adjacent lanes by shuffles.
constexpr int kNoNbr = -2147483647 - 1;
struct XEdge { int w, e; };
__device__ __forceinline__ XEdge x_edges(const TCell& c) {
  XEdge r{kNoNbr, kNoNbr};
  if (!c.act(0)) return r;
  const int x = c.x(0), nx = c.nx;
  if (c.lane == 0) {
    if (x > 0) r.w = -1;
    else if (c.px && nx > 1) r.w = nx - 1;
  }
  if (x + 1 < nx) {
    if (c.lane == 31) r.e = 1;
  } else if (c.px && nx > 1) {
    r.e = -(nx - 1);
  }
  return r;
}
// y-neighbour offsets (north = +y, south = -y) of an active column, or kNoNbr.
__device__ __forceinline__ int y_north(const TCell& c) {
  if (!c.act(0) || c.ny < 2) return kNoNbr;
  if (c.y + 1 < c.ny) return c.nx;
  return c.py ? -(c.ny - 1) * c.nx : kNoNbr;
}
__device__ __forceinline__ int y_south(const TCell& c) {
  if (!c.act(0) || c.ny < 2) return kNoNbr;
  if (c.y > 0) return -c.nx;
  return c.py ? (c.ny - 1) * c.nx : kNoNbr;
}

// First residual of a step from the products the last two steps stored: x0 = T^n + (T^n - T^(n-1))
// (mod_evolve.f90:141), so S - H x0 = S - 2 H T^n + H T^(n-1) up to the rounding of x0 (~1e-16 of
// the terms).  Pointwise: 40 B and 4 FP64 instructions per cell (mixed) instead of the stencil
// sweep's 64 B and 9.  The step's acceptance test stays the FP64 residual of the final x.
template <typename TR>
__device__ __forceinline__ void res_hx_task(const DevArrays& A, double* part, int64_t task,
                                            const InstScal& s) {
  const TCell c = task_cell(A, task);
  const int64_t off = c.off;
  const double* __restrict__ b = A.b + off;
  const double* __restrict__ yc = A.hx[s.hx_role] + off;
  const double* __restrict__ yp = A.hx[1 - s.hx_role] + off;
  const double* __restrict__ rsum = A.rsum + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const double* __restrict__ sinv = A.sinv + off;
  const bool f32 = sizeof(TR) == 4;           // FP32 g goes into the FP32 layout
  TR* R = Vec<TR>::r(A) + (f32 ? c.off4 : off);
  const float isig = (float)(1.0 / s.sigma);
  const bool tiny = tiny_applies(A, s);       // the residual of x0 + TINY: r(x0) - TINY * H1
  double rr = 0.0, gg64 = 0.0;
  float gg = 0.f;
  SqSum rq;                                    // mixed: ||r||^2 off the FP64 pipe
  if (c.act(0)) {
    const int nxy = c.nxy, base = c.base(0);
    const int rxy = f32 ? c.nxy4 : nxy, rbase = f32 ? c.base4(0) : base;
#pragma unroll 4
    for (int z = c.z0; z < c.z1; ++z) {
      const int l = base + z * nxy, lr = rbase + z * rxy;
      if (z + 4 < c.z1) {                       // four planes ahead
        prefetch_l2(b + l + 4 * nxy);
        prefetch_l2(yc + l + 4 * nxy);
        prefetch_l2(yp + l + 4 * nxy);
      }
      const int lc = HF_IX(A, l, c.n());
      double a = fma(-2.0, yc[lc], b[lc]);
      a = a + yp[lc];
      if (tiny) a = fma(-kTiny, rsum[lc], a);
      if (sizeof(TR) == 4) rq.add(a); else rr = fma(a, a, rr);
      if (sizeof(TR) == 4) {
        const float g = -sinv32[lc] * f64_to_f32_trunc(a) * isig;
        R[HF_IX(A, lr, c.n4())] = (TR)g;
        gg = fmaf(g, g, gg);
      } else {
        const double g = -sinv[lc] * a;
        R[HF_IX(A, lr, c.n())] = (TR)g;
        gg64 = fma(g, g, gg64);
      }
    }
  }
  if (sizeof(TR) == 4) rr = rq.value();
  if (sizeof(TR) == 4) {
    task_store_f(part + task * kNR, 1, gg);
    const double v[1] = {rr};
    tile_store<1>(part + task * kNR, v);
  } else {
    const double v[2] = {rr, gg64};
    tile_store<2>(part + task * kNR, v);
  }
}

__device__ __forceinline__ bool vec4_ok(const InstDesc& d);
template <typename TR>
__device__ __forceinline__ void res_hx4_task(const DevArrays& A, double* part, int64_t task,
                                             const InstScal& s);

// FP64 true residual of one task: r = S - H x with x in the x-read buffer (INIT: x0 from the RHS
// kernel) or, after an update, in the x-write buffer (the epilogue then swaps the roles).  Writes
// g = -S^-1 r / sigma into the inner residual (type TR).  FP64 work per cell: 7 FMA for S - Hx,
// 1 FMA for ||r||^2 on the FP64 path (the mixed path sums it in FP32, SqSum); after an update
// also H x = S - r into hx[1 - hx_role] (1 subtraction).
template <bool INIT, typename TR, bool XOUT = false>
__device__ __forceinline__ void res_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  if (INIT && s.hx_ok >= 2) {
    if (vec4_ok(A.inst[A.tasks[task].x])) res_hx4_task<TR>(A, part, task, s);
    else res_hx_task<TR>(A, part, task, s);
    return;
  }
  const TCell c = task_cell(A, task);
  const int64_t off = c.off;
  const double* X = A.tbuf[INIT ? s.role[2] : s.role[3]] + off;
  const double* __restrict__ diag = A.diag + off;
  const double* __restrict__ b = A.b + off;
  const double* __restrict__ cx = A.cx + off;
  const double* __restrict__ cy = A.cy + off;
  const double* __restrict__ cz = A.cz + off;
  const double* __restrict__ rsum = A.rsum + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const double* __restrict__ sinv = A.sinv + off;
  const bool f32 = sizeof(TR) == 4;           // FP32 g goes into the FP32 layout
  TR* R = Vec<TR>::r(A) + (f32 ? c.off4 : off);
  const int rxy = f32 ? c.nxy4 : c.nxy, rbase = f32 ? c.base4(0) : c.base(0);
  double* HX = A.hx[1 - s.hx_role] + off;
  // host-buffer steps (the persistent solve of their graphs): x into the result buffer too
  double* XO = (XOUT && !INIT) ? A.xout + A.inst[c.inst].hoff : nullptr;
  const float isig = (float)(1.0 / s.sigma);
  // mixed: ||r||^2 summed in FP32 over per-thread scaled r (one FP64 instruction less per cell on
  // this FP64-bound sweep)
  SqSum rq;
  // INIT: the residual of x0 + TINY (mod_evolve.f90:141) is r(x0) - TINY * H1
  const bool tiny = INIT && tiny_applies(A, s);
  const bool act = c.act(0);
  const int nz = c.nz, nxy = c.nxy, base = c.base(0);
  const XEdge xe = x_edges(c);
  const int yn = y_north(c), ys = y_south(c);
  const int n = c.n();
  auto xval = [&](int m) -> double { return X[HF_IX(A, m, n)]; };
  double xm, czm;
  plane_below<double>(A, c, 0, xval, cz, xm, czm);
  double xc = act ? xval(base + c.z0 * nxy) : 0.0;
  double rr = 0.0, gg64 = 0.0;
  float gg = 0.f;
  for (int z = c.z0; z < c.z1; ++z) {
    const int l = base + z * nxy;
    const double xn = plane_above<double>(c, 0, xval, z);
    double cxc = 0.0, a = 0.0, bl = 0.0, xwl = 0.0, cxwl = 0.0, xel = 0.0;
    double cyn = 0.0, xyn = 0.0, cys = 0.0, xys = 0.0, czc = 0.0;
    if (act) {
      if (z + 2 < c.z1) {                    // the plane after next: x, diag, b, cx, cy, cz
        const int lp = l + 2 * nxy;
        prefetch_l2(X + lp);
        prefetch_l2(diag + lp);
        prefetch_l2(b + lp);
        prefetch_l2(cx + lp);
        prefetch_l2(cy + lp);
        prefetch_l2(cz + lp);
      }
      const int lc = HF_IX(A, l, n);
      cxc = cx[lc];
      bl = b[lc];
      a = fma(-diag[lc], xc, bl);
      if (tiny) a = fma(-kTiny, rsum[lc], a);
      if (xe.w != kNoNbr) { xwl = xval(l + xe.w); cxwl = cx[HF_IX(A, l + xe.w, n)]; }
      if (xe.e != kNoNbr) xel = xval(l + xe.e);
      if (yn != kNoNbr) { cyn = cy[lc]; xyn = xval(l + yn); }
      if (ys != kNoNbr) { cys = cy[HF_IX(A, l + ys, n)]; xys = xval(l + ys); }
      czc = cz[lc];
    }
    const double up = __shfl_up_sync(kFull, xc, 1), cup = __shfl_up_sync(kFull, cxc, 1);
    const double dn = __shfl_down_sync(kFull, xc, 1);
    if (act) {
      const double xw = c.lane > 0 ? up : xwl, cxw = c.lane > 0 ? cup : cxwl;
      const double xeast = (c.x(0) + 1 < c.nx && c.lane < 31) ? dn : xel;
      a = fma(-cxc, xeast, a);
      a = fma(-cxw, xw, a);
      if (yn != kNoNbr) a = fma(-cyn, xyn, a);
      if (ys != kNoNbr) a = fma(-cys, xys, a);
      if (nz > 1) {
        a = fma(-czc, xn, a);
        a = fma(-czm, xm, a);
      }
      if (sizeof(TR) == 8) rr = fma(a, a, rr);
      else rq.add(a);
      const int lc = HF_IX(A, l, n);
      if (!INIT) HX[lc] = bl - a;
      if (XOUT && !INIT) XO[lc] = xc;
      if (sizeof(TR) == 4) {             // mixed: g in FP32, scaled by 1/sigma
        const float g = -sinv32[lc] * f64_to_f32_trunc(a) * isig;
        R[HF_IX(A, rbase + z * rxy, c.n4())] = (TR)g;
        gg = fmaf(g, g, gg);
      } else {                           // FP64 path: sigma = 1
        const double g = -sinv[lc] * a;
        R[HF_IX(A, rbase + z * rxy, n)] = (TR)g;
        gg64 = fma(g, g, gg64);
      }
    }
    czm = czc;
    xm = xc;
    xc = xn;
  }
  if (sizeof(TR) == 4) rr = rq.value();
  if (sizeof(TR) == 4) {
    task_store_f(part + task * kNR, 1, gg);
    const double v[1] = {rr};
    tile_store<1>(part + task * kNR, v);
  } else {
    const double v[2] = {rr, gg64};
    tile_store<2>(part + task * kNR, v);
  }
}

// Solution update of one task: x_new = x + sigma S^-1 y (+ TINY once).
template <typename TY>
__device__ __forceinline__ void xupd_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  const TCell c = task_cell(A, task);
  if (!c.act(0)) return;
  const int64_t off = c.off;
  const double* XR = A.tbuf[s.role[2]] + off;
  double* XW = A.tbuf[s.role[3]] + off;
  const bool f32 = sizeof(TY) == 4;           // FP32 y is read from the FP32 layout
  const TY* Y = Vec<TY>::y(A) + (f32 ? c.off4 : off);
  const double* __restrict__ sinv = A.sinv + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const bool use_y = s.iter > 0;
  const bool tiny = s.tiny_pending != 0;
  const float sig = (float)s.sigma_prev;
  const int nxy = c.nxy, base = c.base(0);
  const int yxy = f32 ? c.nxy4 : nxy, ybase = f32 ? c.base4(0) : base;
  for (int z0 = c.z0; z0 < c.z1; z0 += 4) {
    double xv[4], sv[4];
    float sv32[4];
    TY yv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int l = base + (z0 + u) * nxy;
      xv[u] = 0.0; yv[u] = TY(0); sv[u] = 0.0; sv32[u] = 0.f;
      if (z0 + u < c.z1) {
        const int lc = HF_IX(A, l, c.n());
        xv[u] = XR[lc];
        if (use_y) {
          yv[u] = Y[HF_IX(A, ybase + (z0 + u) * yxy, f32 ? c.n4() : c.n())];
          if (sizeof(TY) == 8) sv[u] = sinv[lc];
          else sv32[u] = sinv32[lc];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (z0 + u >= c.z1) continue;
      const int l = base + (z0 + u) * nxy;
      double x = xv[u];
      if (tiny) x = x + kTiny;
      if (use_y) {
        if (sizeof(TY) == 8) x = fma(sv[u], (double)yv[u], x);   // sigma = 1 on the FP64 path
        else x = x + f32_to_f64(sig * sv32[u] * (float)yv[u]);
      }
      XW[HF_IX(A, l, c.n())] = x;
    }
  }
}

// Direction update of one task: p_k = r + beta p_(k-1) (p_0 = r) into the buffer of parity k.
template <typename T>
__device__ __forceinline__ void cgp_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  const TCell c = task_cell(A, task);
  if (!c.act(0)) return;
  const int64_t k = s.iter;
  const bool first = (k == 0);
  const T beta = (T)s.beta;
  const T* R = Vec<T>::r(A) + c.off;
  const T* Po = Vec<T>::pb(A, k + 1) + c.off;
  T* Pn = Vec<T>::pb(A, k) + c.off;
  const int nxy = c.nxy, base = c.base(0);
  for (int z0 = c.z0; z0 < c.z1; z0 += 4) {
    T rv[4], pv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      rv[u] = T(0); pv[u] = T(0);
      if (z0 + u < c.z1) {
        const int l = HF_IX(A, base + (z0 + u) * nxy, c.n());
        rv[u] = R[l];
        if (!first) pv[u] = Po[l];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (z0 + u >= c.z1) continue;
      Pn[HF_IX(A, base + (z0 + u) * nxy, c.n())] = first ? rv[u] : fma(beta, pv[u], rv[u]);
    }
  }
}

// q = Ah p and p.q for one task.  FUSED: p is formed on the fly from r and the previous direction
// (p = r + beta p_old, the value the direction update would store) and written out beside q, so
// one pass replaces two.  One column per thread; the operands of plane z+1 (its coefficients, y
// neighbours, x-edge neighbours and plane z+2) are loaded while plane z is computed.
template <typename T, bool FUSED>
__device__ __forceinline__ void spmv_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  static_assert(kXC == 1, "one column per thread");
  const TCell c = task_cell(A, task);
  const int64_t off = c.off;
  const int64_t k = s.iter;
  const bool first = !FUSED || (k == 0);
  const T beta = (T)s.beta;
  // r, or p itself (p_0 = r: the first iteration reads r, its direction update has no round)
  const T* Src = (FUSED || k == 0) ? Vec<T>::r(A) + off : Vec<T>::pb(A, k) + off;
  const T* Po = Vec<T>::pb(A, k + 1) + off;
  T* Pn = Vec<T>::pb(A, k) + off;
  T* Q = Vec<T>::q(A) + off;
  const T* __restrict__ ax = Vec<T>::ax(A) + off;
  const T* __restrict__ ay = Vec<T>::ay(A) + off;
  const T* __restrict__ az = Vec<T>::az(A) + off;
  const bool act = c.act(0);
  const int nx = c.nx, nz = c.nz, nxy = c.nxy, base = c.base(0);
  const XEdge xe = x_edges(c);
  const int yn = y_north(c), ys = y_south(c);
  const bool east_shfl = act && (c.x(0) + 1 < nx) && c.lane < 31;
  // raw operands of one direction value: p = first ? a : beta * b + a
  struct RP { T a, b; };
  const int n = c.n();
  auto ld = [&](int m) -> RP {
    const int mc = HF_IX(A, m, n);
    return RP{Src[mc], first ? T(0) : Po[mc]};
  };
  auto pval = [&](const RP& v) -> T { return first ? v.a : fma(beta, v.b, v.a); };
  struct Plane { RP own, n, s, w, e; T axc, ayc, azc, ays, axw; };
  const RP z0v{T(0), T(0)};
  auto load = [&](int z, Plane& o) {
    o.own = z0v; o.n = z0v; o.s = z0v; o.w = z0v; o.e = z0v;
    o.axc = T(0); o.ayc = T(0); o.azc = T(0); o.ays = T(0); o.axw = T(0);
    if (!act) return;
    if (z >= nz) {                      // above the top plane: the periodic wrap, or nothing
      if (c.pz && nz > 1) o.own = ld(base);
      return;
    }
    const int l = base + z * nxy, lc = HF_IX(A, l, n);
    o.own = ld(l);
    o.axc = ax[lc]; o.ayc = ay[lc]; o.azc = az[lc];
    if (yn != kNoNbr) o.n = ld(l + yn);
    if (ys != kNoNbr) { o.s = ld(l + ys); o.ays = ay[HF_IX(A, l + ys, n)]; }
    if (xe.w != kNoNbr) { o.w = ld(l + xe.w); o.axw = ax[HF_IX(A, l + xe.w, n)]; }
    if (xe.e != kNoNbr) o.e = ld(l + xe.e);
  };
  // plane below the task (z0 - 1, or the periodic wrap to nz - 1)
  T pm = T(0), azm = T(0);
  if (act && nz > 1) {
    int lb = -1;
    if (c.z0 > 0) lb = base + (c.z0 - 1) * nxy;
    else if (c.pz) lb = base + (nz - 1) * nxy;
    if (lb >= 0) { pm = pval(ld(lb)); azm = az[HF_IX(A, lb, n)]; }
  }
  Plane cur, nxt;
  load(c.z0, cur);
  T pq = T(0);
  for (int z = c.z0; z < c.z1; ++z) {
    if (z + 1 < nz) load(z + 1, nxt);
    else load(nz, nxt);
    const int l = base + z * nxy;
    const T pc = pval(cur.own);
    const T up = __shfl_up_sync(kFull, pc, 1);
    const T cup = __shfl_up_sync(kFull, cur.axc, 1);
    const T dn = __shfl_down_sync(kFull, pc, 1);
    if (act) {
      const T pw = c.lane > 0 ? up : pval(cur.w);
      const T axw = c.lane > 0 ? cup : cur.axw;
      const T pe = east_shfl ? dn : pval(cur.e);
      T acc = pc;
      acc = fma(cur.axc, pe, acc);
      acc = fma(axw, pw, acc);
      if (c.ny > 1) {
        acc = fma(cur.ayc, pval(cur.n), acc);
        acc = fma(cur.ays, pval(cur.s), acc);
      }
      if (nz > 1) {
        acc = fma(cur.azc, pval(nxt.own), acc);
        acc = fma(azm, pm, acc);
      }
      const int lc = HF_IX(A, l, n);
      if (FUSED) Pn[lc] = pc;
      Q[lc] = acc;
      pq = fma(pc, acc, pq);
    }
    pm = pc; azm = cur.azc;
    cur = nxt;
  }
  if (sizeof(T) == 4) {
    task_store_f(part + task * kNR, 0, (float)pq);
  } else {
    const double v[1] = {(double)pq};
    tile_store<1>(part + task * kNR, v);
  }
}

// y += alpha p, r -= alpha q, r.r (and the unscaled ||r||^2 for the reference rule) of one task.
template <typename T>
__device__ __forceinline__ void upd_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  const TCell c = task_cell(A, task);
  const DevOpts& o = A.opts;
  const bool weighted = (o.criterion == HF_STOP_RECURSIVE);
  const T alpha = (T)s.alpha;
  const bool first = (s.iter == 0);
  const int64_t off = c.off;
  T* Y = Vec<T>::y(A) + off;
  T* R = Vec<T>::r(A) + off;
  const T* P = Vec<T>::pb(A, s.iter) + off;
  T* P0 = Vec<T>::pb(A, 0) + off;            // p_0 = r, left for p_1 (as in upd4_task)
  const T* Q = Vec<T>::q(A) + off;
  const double* __restrict__ diag = A.diag + off;
  const bool act = c.act(0);
  const int nxy = c.nxy, base = c.base(0);
  T rr = T(0);
  double rw = 0.0;
  if (act) {
    for (int z0 = c.z0; z0 < c.z1; z0 += 4) {
      T pv[4], qv[4], rv[4], yv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        pv[u] = T(0); qv[u] = T(0); rv[u] = T(0); yv[u] = T(0);
        if (z0 + u < c.z1) {
          const int l = HF_IX(A, base + (z0 + u) * nxy, c.n());
          qv[u] = Q[l]; rv[u] = R[l];
          pv[u] = first ? rv[u] : P[l];
          if (!first) yv[u] = Y[l];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (z0 + u >= c.z1) continue;
        const int l = HF_IX(A, base + (z0 + u) * nxy, c.n());
        Y[l] = first ? alpha * pv[u] : fma(alpha, pv[u], yv[u]);
        const T r = fma(-alpha, qv[u], rv[u]);
        R[l] = r;
        if (first) P0[l] = rv[u];
        rr = fma(r, r, rr);
        if (weighted) rw = fma(-diag[l] * (double)r, (double)r, rw);
      }
    }
  }
  if (sizeof(T) == 4 && !weighted) {
    task_store_f(part + task * kNR, 0, (float)rr);
  } else {
    const double v[2] = {(double)rr, rw};
    tile_store<2>(part + task * kNR, v);
  }
}

// ---- FP32 p + SpMV on 16-byte vectors ---------------------------------------------------------
// The FP32 vectors have rows of sx = nx rounded up to 4 cells (every row starts 16-byte aligned;
// the instances start at multiples of 1024 cells), so each thread owns 4 consecutive x cells and
// works on float4 vectors: a quarter of the scalar version's instructions per cell.  In a row's
// last quad the cells past nx are padding: their coefficients and p are zero, q is kept zero, and
// the last grid cell takes its east neighbour from a load (the periodic wrap) or has none.  Block layout over a
// 32 x 8 column tile: four z-groups of 64 threads, each marching its quarter of the task's planes;
// in a group, thread w owns row w / 8 and cells x0 + 4 (w % 8) .. + 3, so a warp holds 4 rows of
// 8 quads and the x neighbours across quads are shuffles.  Per plane a thread issues its ten
// vector loads (own r, p_old, three faces; the y-neighbour rows; the next plane's r, p_old) at
// once, which keeps ~40 KB per block in flight.  FUSED: p = r + beta p_old is formed on the fly and
// stored beside q (the persistent solve's pass); otherwise p is read (the standalone SpMV).  The
// per-cell arithmetic is the scalar version's; the p.q partial is summed per thread over its 4
// cells plane by plane, the same way in both uses.
__device__ __forceinline__ bool vec4_ok(const InstDesc& d) { return (d.nx & 3) == 0; }

// The quad (4 consecutive x cells) of thread w (0..63) of a z-group: 8 quads x 8 rows of the
// task's tile.  west_lane / east_lane: the neighbouring quad of the row is not in the adjacent
// lane of this warp.
struct QuadPos {
  int x, y;
  bool act, west_lane, east_lane;
};
__device__ __forceinline__ QuadPos quad_pos(const int4& tk, const InstDesc& d, int w) {
  QuadPos p;
  p.x = tk.y + 4 * (w & 7);
  p.y = tk.z + (w >> 3);
  p.act = p.x < d.nx && p.y < d.ny;
  p.west_lane = (w & 7) == 0;
  p.east_lane = (w & 7) == 7;
  return p;
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

__device__ __forceinline__ void st4(float* p, const float4& v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float f4(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

template <bool FUSED>
__device__ __forceinline__ void spmv4_task(const DevArrays& A, double* part, int64_t task,
                                           const InstScal& s) {
  const int4 tk = A.tasks[task];
  const InstDesc& d = A.inst[tk.x];
  const int nx = d.nx, ny = d.ny, nz = d.nz, sx = d.sx, nxy = sx * ny;
  const int64_t off = d.off4;
  const int tid = threadIdx.x, grp = tid >> 6, w = tid & 63;
  const QuadPos qp = quad_pos(tk, d, w);
  const int x = qp.x, y = qp.y;
  const int z0 = tk.w, z1 = min(z0 + d.zc, nz);
  const int per = (z1 - z0 + 3) >> 2;
  const int za = min(z0 + grp * per, z1), zb = min(za + per, z1);
  const bool act = qp.act;
  const int last = min(3, nx - 1 - x);   // the quad's last grid cell; cells past it are padding
  const int64_t k = s.iter;
  const bool first = !FUSED || k == 0;
  const float beta = (float)s.beta;
  const float* Src = (FUSED || k == 0) ? A.r32 + off : ((k & 1) ? A.p232 : A.p32) + off;
  const float* Po = (((k + 1) & 1) ? A.p232 : A.p32) + off;
  float* Pn = ((k & 1) ? A.p232 : A.p32) + off;
  float* Q = A.q32 + off;
  const float* __restrict__ ax = A.a32x + off;
  const float* __restrict__ ay = A.a32y + off;
  const float* __restrict__ az = A.a32z + off;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  // neighbour offsets (y rows, x edges, z wrap); has_* false: the face is absent (value 0)
  bool hn = false, hs = false;
  int dn = 0, ds = 0;
  if (ny > 1) {
    if (y + 1 < ny) { dn = sx; hn = true; } else if (d.py) { dn = -(ny - 1) * sx; hn = true; }
    if (y > 0) { ds = -sx; hs = true; } else if (d.py) { ds = (ny - 1) * sx; hs = true; }
  }
  const bool wload = (qp.west_lane || x == 0);     // west of cell 0 is loaded, not shuffled
  const bool eload = (qp.east_lane || x + 4 >= nx); // east of the last cell is loaded, not shuffled
  bool hw = false, he = false;
  int dw = 0, de = 0;
  if (x > 0) { dw = -1; hw = true; } else if (d.px && nx > 1) { dw = nx - 1; hw = true; }
  if (x + 4 < nx) { de = 4; he = true; } else if (d.px && nx > 1) { de = -x; he = true; }
  auto pv = [&](float a, float b) -> float { return first ? a : fmaf(beta, b, a); };
  auto pv4 = [&](const float4& a, const float4& b) -> float4 {
    return make_float4(pv(a.x, b.x), pv(a.y, b.y), pv(a.z, b.z), pv(a.w, b.w));
  };
  const int n4 = nxy * nz;               // the instance's cells in the FP32 layout
  auto ldp = [&](int l, float4& r, float4& po) {
    const int lc = HF_IX4(A, l, n4);
    r = ld4(Src + lc);
    po = first ? zero4 : ld4(Po + lc);
  };
  const int lxy = y * sx + x;
  // plane below the group (za - 1, or the periodic wrap to nz - 1), and the group's first plane
  float4 pm = zero4, azm = zero4, rc = zero4, poc = zero4;
  if (act && za < zb) {
    if (nz > 1) {
      int lb = -1;
      if (za > 0) lb = lxy + (za - 1) * nxy;
      else if (d.pz) lb = lxy + (nz - 1) * nxy;
      if (lb >= 0) {
        float4 rb, pob;
        ldp(lb, rb, pob);
        pm = pv4(rb, pob);
        azm = ld4(az + HF_IX4(A, lb, n4));
      }
    }
    ldp(lxy + za * nxy, rc, poc);
  }
  float pq = 0.f;
  for (int z = za; z < zb; ++z) {
    const int l = lxy + z * nxy;
    float4 ru = zero4, pou = zero4, axv = zero4, ayv = zero4, azv = zero4;
    float4 rn = zero4, pon = zero4, rs = zero4, pos = zero4, aysv = zero4;
    float rw = 0.f, pow_ = 0.f, axwl = 0.f, re = 0.f, poe = 0.f;
    if (act) {
      if (nz > 1) {
        if (z + 1 < nz) ldp(l + nxy, ru, pou);
        else if (d.pz) ldp(lxy, ru, pou);
      }
      const int lc = HF_IX4(A, l, n4);
      axv = ld4(ax + lc); ayv = ld4(ay + lc); azv = ld4(az + lc);
      if (z + 1 < zb) {
        prefetch_l2(ax + l + nxy);
        prefetch_l2(ay + l + nxy);
        prefetch_l2(az + l + nxy);
      }
      if (hn) ldp(l + dn, rn, pon);
      if (hs) { ldp(l + ds, rs, pos); aysv = ld4(ay + HF_IX4(A, l + ds, n4)); }
      if (wload && hw) {
        const int lw = HF_IX(A, l + dw, n4);
        rw = Src[lw];
        pow_ = first ? 0.f : Po[lw];
        axwl = ax[lw];
      }
      if (eload && he) {
        const int le = HF_IX(A, l + de, n4);
        re = Src[le];
        poe = first ? 0.f : Po[le];
      }
    }
    const float4 p = pv4(rc, poc);
    const float pw_sh = __shfl_up_sync(kFull, p.w, 1);
    const float axw_sh = __shfl_up_sync(kFull, axv.w, 1);
    const float pe_sh = __shfl_down_sync(kFull, p.x, 1);
    if (act) {
      const float pw0 = wload ? (hw ? pv(rw, pow_) : 0.f) : pw_sh;
      const float axw0 = wload ? (hw ? axwl : 0.f) : axw_sh;
      const float pe3 = eload ? (he ? pv(re, poe) : 0.f) : pe_sh;
      const float4 pu = pv4(ru, pou), pn = pv4(rn, pon), ps = pv4(rs, pos);
      float4 qv;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float pc = f4(p, i);
        const float pe = i < last ? f4(p, i + 1) : pe3;
        const float pw = i > 0 ? f4(p, i - 1) : pw0;
        const float axw = i > 0 ? f4(axv, i - 1) : axw0;
        float acc = pc;
        acc = fmaf(f4(axv, i), pe, acc);
        acc = fmaf(axw, pw, acc);
        if (ny > 1) {
          acc = fmaf(f4(ayv, i), f4(pn, i), acc);
          acc = fmaf(f4(aysv, i), f4(ps, i), acc);
        }
        if (nz > 1) {
          acc = fmaf(f4(azv, i), f4(pu, i), acc);
          acc = fmaf(f4(azm, i), f4(pm, i), acc);
        }
        if (i > last) acc = 0.f;       // padding: q stays 0 (its p is 0)
        pq = fmaf(pc, acc, pq);
        if (i == 0) qv.x = acc; else if (i == 1) qv.y = acc; else if (i == 2) qv.z = acc; else qv.w = acc;
      }
      const int ls = HF_IX4(A, l, n4);
      if (FUSED) st4(Pn + ls, p);
      st4(Q + ls, qv);
      pm = p;
      azm = azv;
      rc = ru;
      poc = pou;
    }
  }
  task_store_f(part + task * kNR, 0, pq);
}

// ---- element-wise passes on 4-cell vectors (rows of 4k cells) --------------------------------
// Same thread layout as spmv4_task (four z-groups of 64 threads, 4 consecutive x cells per
// thread); FP32 vectors are one 16-byte access, FP64 vectors two.  Two planes of loads are issued
// before they are used.  Reductions are summed per thread plane by plane, cells in x order.
template <typename T> struct V4 { T v[4]; };
__device__ __forceinline__ V4<float> ldv4(const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  return V4<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ V4<double> ldv4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  return V4<double>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void stv4(float* p, const V4<float>& v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void stv4(double* p, const V4<double>& v) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v.v[0], v.v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v.v[2], v.v[3]);
}

// A thread's quad.  F32: the pass's vectors are FP32 and live in the FP32 layout (rows of sx
// cells; voff, nxy, lxy index them); FP64 arrays beside them use the FP64 layout (off, dxy, dlxy).
// For FP64 vectors (F32 false) both are the FP64 layout.
struct Quad {
  int64_t off, voff;
  int nxy, lxy, dxy, dlxy, za, zb, nx, x;
  int vn, dn;        // cells of the instance in the vectors' layout and in the FP64 layout
  bool act, padded;
};
template <bool F32>
__device__ __forceinline__ Quad quad_cell(const DevArrays& A, int64_t task) {
  const int4 tk = A.tasks[task];
  const InstDesc& d = A.inst[tk.x];
  const int tid = threadIdx.x, grp = tid >> 6, w = tid & 63;
  const QuadPos qp = quad_pos(tk, d, w);
  const int x = qp.x, y = qp.y;
  const int z1 = min(tk.w + d.zc, d.nz);
  const int per = (z1 - tk.w + 3) >> 2;
  const int sx = F32 ? d.sx : d.nx;
  Quad c;
  c.off = d.off;
  c.voff = F32 ? d.off4 : d.off;
  c.nxy = sx * d.ny;
  c.lxy = y * sx + x;
  c.dxy = d.nx * d.ny;
  c.dlxy = y * d.nx + x;
  c.nx = d.nx;
  c.x = x;
  c.padded = sx != d.nx;
  c.za = min(tk.w + grp * per, z1);
  c.zb = min(c.za + per, z1);
  c.act = qp.act;
  c.vn = c.nxy * d.nz;
  c.dn = c.dxy * d.nz;
  return c;
}

// The FP64-layout diagonal of a quad's cells (zeros for padding cells).
__device__ __forceinline__ V4<double> diag4(const DevArrays& A, const double* __restrict__ diag,
                                            const Quad& c, int z) {
  const int l = c.dlxy + z * c.dxy;
  if (!c.padded) return ldv4(diag + HF_IX4(A, l, c.dn));
  V4<double> v{};
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (c.x + i < c.nx) v.v[i] = diag[HF_IX(A, l + i, c.dn)];
  return v;
}

template <typename T>
__device__ __forceinline__ void upd4_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  const Quad c = quad_cell<sizeof(T) == 4>(A, task);
  const bool weighted = (A.opts.criterion == HF_STOP_RECURSIVE);
  const T alpha = (T)s.alpha;
  const bool first = (s.iter == 0);
  T* Y = Vec<T>::y(A) + c.voff;
  T* R = Vec<T>::r(A) + c.voff;
  // p_0 = r has no round of its own: the first update takes p from r and leaves it in the
  // direction buffer of iteration 0 (p_1 = r_1 + beta p_0 reads it there)
  const T* P = Vec<T>::pb(A, s.iter) + c.voff;
  T* P0 = Vec<T>::pb(A, 0) + c.voff;
  const T* Q = Vec<T>::q(A) + c.voff;
  const double* __restrict__ diag = A.diag + c.off;
  T rr = T(0);
  double rw = 0.0;
  if (c.act && (s.xw & kXwThis)) {
    // The iteration predicted to end the inner solve also forms x_new = x + sigma S^-1 y_new, the
    // x update's arithmetic on the y it stores (rows of 4k cells: both layouts index alike).
    const double* XR = A.tbuf[s.role[2]] + c.off;
    double* XW = A.tbuf[s.role[3]] + c.off;
    const double* __restrict__ sinv = A.sinv + c.off;
    const float* __restrict__ sinv32 = A.sinv32 + c.off;
    const float sig = (float)s.sigma_prev;
    for (int z = c.za; z < c.zb; ++z) {
      const int l = HF_IX4(A, c.lxy + z * c.nxy, c.vn);
      const V4<T> qv = ldv4(Q + l), rv = ldv4(R + l);
      const V4<T> pv = first ? rv : ldv4(P + l);
      V4<T> yv{};
      if (!first) yv = ldv4(Y + l);
      V4<double> xv = ldv4(XR + l), sv{};
      V4<float> fv{};
      if (sizeof(T) == 8) sv = ldv4(sinv + l); else fv = ldv4(sinv32 + l);
      V4<T> yo, ro;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        yo.v[i] = first ? alpha * pv.v[i] : fma(alpha, pv.v[i], yv.v[i]);
        const T r = fma(-alpha, qv.v[i], rv.v[i]);
        ro.v[i] = r;
        rr = fma(r, r, rr);
        if (sizeof(T) == 8) xv.v[i] = fma(sv.v[i], (double)yo.v[i], xv.v[i]);
        else xv.v[i] = xv.v[i] + f32_to_f64(sig * fv.v[i] * (float)yo.v[i]);
      }
      stv4(Y + l, yo);
      stv4(R + l, ro);
      stv4(XW + l, xv);
      if (first) stv4(P0 + l, rv);
    }
  } else if (c.act) {
    for (int z = c.za; z < c.zb; z += 2) {
      const bool two = z + 1 < c.zb;
      const int l0 = HF_IX4(A, c.lxy + z * c.nxy, c.vn);
      const int l1 = two ? HF_IX4(A, l0 + c.nxy, c.vn) : 0;
      V4<T> q0 = ldv4(Q + l0), r0 = ldv4(R + l0), p0{}, y0{}, p1{}, q1{}, r1{}, y1{};
      p0 = first ? r0 : ldv4(P + l0);
      if (!first) y0 = ldv4(Y + l0);
      if (two) {
        q1 = ldv4(Q + l1); r1 = ldv4(R + l1);
        p1 = first ? r1 : ldv4(P + l1);
        if (!first) y1 = ldv4(Y + l1);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 1 && !two) break;
        const int l = h ? l1 : l0;
        const V4<T>& pv = h ? p1 : p0;
        const V4<T>& qv = h ? q1 : q0;
        const V4<T>& rv = h ? r1 : r0;
        const V4<T>& yv = h ? y1 : y0;
        V4<T> yo, ro;
        V4<double> dg{};
        if (weighted) dg = diag4(A, diag, c, z + h);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          yo.v[i] = first ? alpha * pv.v[i] : fma(alpha, pv.v[i], yv.v[i]);
          const T r = fma(-alpha, qv.v[i], rv.v[i]);
          ro.v[i] = r;
          rr = fma(r, r, rr);
          if (weighted) rw = fma(-dg.v[i] * (double)r, (double)r, rw);
        }
        stv4(Y + l, yo);
        stv4(R + l, ro);
        if (first) stv4(P0 + l, rv);
      }
    }
  }
  if (sizeof(T) == 4 && !weighted) {
    task_store_f(part + task * kNR, 0, (float)rr);
  } else {
    const double v[2] = {(double)rr, rw};
    tile_store<2>(part + task * kNR, v);
  }
}

template <typename T>
__device__ __forceinline__ void cgp4_task(const DevArrays& A, double* part, int64_t task,
                                          const InstScal& s) {
  const Quad c = quad_cell<sizeof(T) == 4>(A, task);
  if (!c.act) return;
  const int64_t k = s.iter;
  const bool first = (k == 0);
  const T beta = (T)s.beta;
  const T* R = Vec<T>::r(A) + c.voff;
  const T* Po = Vec<T>::pb(A, k + 1) + c.voff;
  T* Pn = Vec<T>::pb(A, k) + c.voff;
  for (int z = c.za; z < c.zb; z += 2) {
    const bool two = z + 1 < c.zb;
    const int l0 = HF_IX4(A, c.lxy + z * c.nxy, c.vn);
    const int l1 = two ? HF_IX4(A, l0 + c.nxy, c.vn) : 0;
    V4<T> r0 = ldv4(R + l0), o0{}, r1{}, o1{};
    if (!first) o0 = ldv4(Po + l0);
    if (two) {
      r1 = ldv4(R + l1);
      if (!first) o1 = ldv4(Po + l1);
    }
    V4<T> n0, n1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      n0.v[i] = first ? r0.v[i] : fma(beta, o0.v[i], r0.v[i]);
      n1.v[i] = first ? r1.v[i] : fma(beta, o1.v[i], r1.v[i]);
    }
    stv4(Pn + l0, n0);
    if (two) stv4(Pn + l1, n1);
  }
}

template <typename TY>
__device__ __forceinline__ void xupd4_task(const DevArrays& A, double* part, int64_t task,
                                           const InstScal& s) {
  const Quad c = quad_cell<false>(A, task);   // rows of 4k cells: the two layouts agree in shape
  if (!c.act) return;
  const double* XR = A.tbuf[s.role[2]] + c.off;
  double* XW = A.tbuf[s.role[3]] + c.off;
  const TY* Y = Vec<TY>::y(A) + (sizeof(TY) == 4 ? A.inst[A.tasks[task].x].off4 : c.off);
  const double* __restrict__ sinv = A.sinv + c.off;
  const float* __restrict__ sinv32 = A.sinv32 + c.off;
  const bool use_y = s.iter > 0;
  const bool tiny = s.tiny_pending != 0;
  const float sig = (float)s.sigma_prev;
  for (int z = c.za; z < c.zb; z += 2) {
    const bool two = z + 1 < c.zb;
    const int l0 = HF_IX4(A, c.lxy + z * c.nxy, c.vn);
    const int l1 = two ? HF_IX4(A, l0 + c.nxy, c.vn) : 0;
    V4<double> x0 = ldv4(XR + l0), x1{}, s0{}, s1{};
    V4<TY> y0{}, y1{};
    V4<float> f0{}, f1{};
    if (use_y) {
      y0 = ldv4(Y + l0);
      if (sizeof(TY) == 8) s0 = ldv4(sinv + l0); else f0 = ldv4(sinv32 + l0);
    }
    if (two) {
      x1 = ldv4(XR + l1);
      if (use_y) {
        y1 = ldv4(Y + l1);
        if (sizeof(TY) == 8) s1 = ldv4(sinv + l1); else f1 = ldv4(sinv32 + l1);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && !two) break;
      V4<double> xv = h ? x1 : x0;
      const V4<TY>& yv = h ? y1 : y0;
      const V4<double>& sv = h ? s1 : s0;
      const V4<float>& fv = h ? f1 : f0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        double x = xv.v[i];
        if (tiny) x = x + kTiny;
        if (use_y) {
          if (sizeof(TY) == 8) x = fma(sv.v[i], (double)yv.v[i], x);   // sigma = 1 on the FP64 path
          else x = x + f32_to_f64(sig * fv.v[i] * (float)yv.v[i]);
        }
        xv.v[i] = x;
      }
      stv4(XW + (h ? l1 : l0), xv);
    }
  }
}

// The step's first residual from the stored products (res_hx_task) on 4-cell vectors, for rows of
// 4k cells: the same per-cell arithmetic; ||r||^2 and ||g||^2 summed per thread plane by plane,
// cells in x order.  A quarter of the scalar form's load instructions keeps more bytes in flight
// on this FP64-bound round.
template <typename TR>
__device__ __forceinline__ void res_hx4_task(const DevArrays& A, double* part, int64_t task,
                                             const InstScal& s) {
  const Quad c = quad_cell<false>(A, task);   // rows of 4k cells: the two layouts agree in shape
  const int64_t off = c.off;
  const double* __restrict__ b = A.b + off;
  const double* __restrict__ yc = A.hx[s.hx_role] + off;
  const double* __restrict__ yp = A.hx[1 - s.hx_role] + off;
  const double* __restrict__ rsum = A.rsum + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const double* __restrict__ sinv = A.sinv + off;
  const bool f32 = sizeof(TR) == 4;
  TR* R = Vec<TR>::r(A) + (f32 ? A.inst[A.tasks[task].x].off4 : off);
  const float isig = (float)(1.0 / s.sigma);
  const bool tiny = tiny_applies(A, s);       // the residual of x0 + TINY: r(x0) - TINY * H1
  double rr = 0.0, gg64 = 0.0;
  float gg = 0.f;
  SqSum rq;                                    // mixed: ||r||^2 off the FP64 pipe
  if (c.act) {
    for (int z = c.za; z < c.zb; ++z) {
      const int l = HF_IX4(A, c.lxy + z * c.nxy, c.vn);
      const V4<double> bv = ldv4(b + l), cv = ldv4(yc + l), pv = ldv4(yp + l);
      V4<double> rs{}, s64{};
      V4<float> s32{};
      if (tiny) rs = ldv4(rsum + l);
      if (f32) s32 = ldv4(sinv32 + l);
      else s64 = ldv4(sinv + l);
      V4<TR> g4;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        double a = fma(-2.0, cv.v[i], bv.v[i]);
        a = a + pv.v[i];
        if (tiny) a = fma(-kTiny, rs.v[i], a);
        if (f32) rq.add(a); else rr = fma(a, a, rr);
        if (f32) {
          const float g = -s32.v[i] * f64_to_f32_trunc(a) * isig;
          g4.v[i] = (TR)g;
          gg = fmaf(g, g, gg);
        } else {
          const double g = -s64.v[i] * a;
          g4.v[i] = (TR)g;
          gg64 = fma(g, g, gg64);
        }
      }
      stv4(R + l, g4);
    }
  }
  if (f32) rr = rq.value();
  if (sizeof(TR) == 4) {
    task_store_f(part + task * kNR, 1, gg);
    const double v[1] = {rr};
    tile_store<1>(part + task * kNR, v);
  } else {
    const double v[2] = {rr, gg64};
    tile_store<2>(part + task * kNR, v);
  }
}

// Dispatch between the vector and the scalar form of a pass (same choice on every path).  The
// FP32 vectors are padded to rows of 4k cells, so their passes are always vector passes.
template <typename T>
__device__ __forceinline__ void upd_any(const DevArrays& A, double* part, int64_t task, const InstScal& s) {
  if constexpr (sizeof(T) == 4) upd4_task<T>(A, part, task, s);
  else if (vec4_ok(A.inst[A.tasks[task].x])) upd4_task<T>(A, part, task, s);
  else upd_task<T>(A, part, task, s);
}
template <typename T>
__device__ __forceinline__ void cgp_any(const DevArrays& A, double* part, int64_t task, const InstScal& s) {
  if constexpr (sizeof(T) == 4) cgp4_task<T>(A, part, task, s);
  else if (vec4_ok(A.inst[A.tasks[task].x])) cgp4_task<T>(A, part, task, s);
  else cgp_task<T>(A, part, task, s);
}
template <typename TY>
__device__ __forceinline__ void xupd_any(const DevArrays& A, double* part, int64_t task, const InstScal& s) {
  if (vec4_ok(A.inst[A.tasks[task].x])) xupd4_task<TY>(A, part, task, s);
  else xupd_task<TY>(A, part, task, s);
}

// The FP32 p + SpMV pass of one task (always the vector form: the FP32 layout has rows of 4k).
template <bool FUSED>
__device__ __forceinline__ void pq_f32_task(const DevArrays& A, double* part, int64_t task,
                                            const InstScal& s) {
  spmv4_task<FUSED>(A, part, task, s);
}

// ---- standalone kernels (host-polled loop, conditional-node graph, kernel timing) --------------
template <bool INIT, typename TR>
__global__ void __launch_bounds__(kBlock) k_residual(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.outer_active || s.inner_active) return;
  if (INIT != (s.refine == 0)) return;
  res_task<INIT, TR>(A, A.partials, blockIdx.x, s);
}

template <typename TY>
__global__ void __launch_bounds__(kBlock) k_xupdate(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.outer_active || s.inner_active || s.refine == 0 || (s.xw & kXwDone)) return;
  xupd_any<TY>(A, A.partials, blockIdx.x, s);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_p(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.inner_active || s.iter == 0) return;   // p_0 = r: the SpMV and the update read r
  cgp_any<T>(A, A.partials, blockIdx.x, s);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_spmv(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.inner_active) return;
  if constexpr (sizeof(T) == 4) pq_f32_task<false>(A, A.partials, blockIdx.x, s);
  else spmv_task<T, false>(A, A.partials, blockIdx.x, s);
}

// The persistent solve's fused FP32 pass on its own (timing and profiling).
__global__ void __launch_bounds__(kBlock) k_cg_pq_f32(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.inner_active) return;
  pq_f32_task<true>(A, A.partials, blockIdx.x, s);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_upd(DevArrays A) {
  const InstScal& s = A.scal[A.tasks[blockIdx.x].x];
  if (!s.inner_active) return;
  upd_any<T>(A, A.partials, blockIdx.x, s);
}

// ---- summation of an instance's task partials ------------------------------------------------
// The order depends only on the instance's task count, so every path (finalize kernels, the
// persistent solve's barrier epilogue) and every batch composition obtains the same bits: above
// kWarpSumMax tasks the whole block sums (thread-strided, then block_sum), otherwise warp 0 sums
// (lane-strided, then a shuffle tree).  The result is valid in thread 0.  Partials are read
// through L2 (written by other blocks of the same persistent launch).
// acc += the partials of tasks first, first + step, ... (< ntask) of an instance, in that order.
// The loads of kSumBatch tasks are issued before their adds (the same adds in the same order, so
// the same bits): a grid barrier's epilogue waits on this sum, and one L2 round trip per task
// made it several microseconds per round.
constexpr int kSumBatch = 8;
template <int NRV>
__device__ __forceinline__ void strided_sum(const double* part, int64_t task0, int64_t ntask,
                                            int64_t first, int step, double (&acc)[NRV]) {
  for (int64_t t0 = first; t0 < ntask; t0 += (int64_t)kSumBatch * step) {
    double v[kSumBatch][NRV];
#pragma unroll
    for (int u = 0; u < kSumBatch; ++u) {
      const int64_t t = t0 + (int64_t)u * step;
#pragma unroll
      for (int k = 0; k < NRV; ++k) v[u][k] = t < ntask ? __ldcg(&part[(task0 + t) * kNR + k]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kSumBatch; ++u) {
      if (t0 + (int64_t)u * step >= ntask) break;
#pragma unroll
      for (int k = 0; k < NRV; ++k) acc[k] += v[u][k];
    }
  }
}

template <int NRV>
__device__ __forceinline__ void warp_instance_sum(const double* part, const InstDesc& d, int lane,
                                                  double (&acc)[NRV]) {
#pragma unroll
  for (int k = 0; k < NRV; ++k) acc[k] = 0.0;
  strided_sum<NRV>(part, d.task0, d.ntask, lane, 32, acc);
#pragma unroll
  for (int k = 0; k < NRV; ++k) acc[k] = warp_sum(acc[k]);
}
// Block-uniform call (all threads of the block).
template <int NRV>
__device__ __forceinline__ void instance_sum(const double* part, const InstDesc& d,
                                             double (&acc)[NRV], double* red) {
  if (d.ntask > kWarpSumMax) {
#pragma unroll
    for (int k = 0; k < NRV; ++k) acc[k] = 0.0;
    strided_sum<NRV>(part, d.task0, d.ntask, threadIdx.x, (int)blockDim.x, acc);
    block_sum<NRV>(acc, red);
  } else if (threadIdx.x < 32) {
    warp_instance_sum<NRV>(part, d, (int)threadIdx.x, acc);
  }
}

// ---- finalize kernels: one block per instance sums the task partials in task order ----------
// (deterministic), then runs the scalar epilogue of the producing kernel.

// Epilogue of the RHS kernel (mod_evolve.f90:70-127 checks, initial scale of the FP32 rhs).
__device__ void epi_rhs(const DevArrays& A, int inst, const double* tot) {
  InstScal& s = A.scal[inst];
  const InstDesc& d = A.inst[inst];
  s.bb = tot[0];
  s.x0flag = tot[1] > 0.0 ? 1 : 0;
  if (isnan(tot[0])) {              // some S is NaN: which vector failed is diagnosed later
    s.status |= kStatusRhsNan;
    s.outer_active = 0;
    s.failed_step = s.itime;
    s.phase = PH_IDLE;
    return;
  }
  // scale of the first FP32 residual: a power of two near rms(S)/rms(|H_II|^(1/2)) * 1e-6
  const double rms = sqrt(tot[0] / (double)d.n) * d.mean_sinv * 1e-6;
  s.sigma = (A.opts.precision == HF_PREC_MIXED && rms > 0.0 && isfinite(rms))
                ? exp2(rint(log2(rms))) : 1.0;
}

// Epilogue of the diagnosis pass: the first failing vector in the reference's order.
__device__ void epi_rhs_diag(const DevArrays& A, int inst, const double* tot) {
  InstScal& s = A.scal[inst];
  int st = 0;
  if (tot[1] > 0) st = 1 << (HF_ENAN_Q - HF_ENAN_B);
  else if (tot[2] > 0) st = 1 << (HF_ENAN_QDENS - HF_ENAN_B);
  else if (tot[3] > 0) st = 1 << (HF_ENAN_SCAT - HF_ENAN_B);
  else if (tot[4] > 0) st = 1 << (HF_ENAN_S - HF_ENAN_B);
  s.status = st ? st : (1 << (HF_ENAN_S - HF_ENAN_B));
}

// Epilogue of a residual sweep: convergence test and set-up of the next inner solve.
template <bool INIT>
__device__ void epi_residual_s(InstScal& s, const InstDesc& G, const DevOpts& o, const double* tot) {
  s.xw = 0;                              // this sweep consumed any x formed by a CG update
  if (!INIT) {
    const int t = s.role[2]; s.role[2] = s.role[3]; s.role[3] = t;
    s.tiny_pending = 0;
  } else {
    s.tiny_pending = (o.criterion == HF_STOP_RECURSIVE) ? s.x0flag : 0;   // tiny_applies
  }
  s.rr_true = tot[0];
  s.relres = s.bb > 0.0 ? sqrt(tot[0] / s.bb) : (tot[0] > 0.0 ? INFINITY : 0.0);
  s.refine += 1;
  s.tot_refine += 1;
  if (isnan(tot[0])) {                   // x holds a NaN (mod_evolve.f90:153-158)
    s.status |= 1 << (HF_ENAN_X - HF_ENAN_B);
    s.failed_step = s.itime;
    s.outer_active = 0;
    return;
  }
  bool done, converged;
  if (o.criterion == HF_STOP_RECURSIVE) {
    done = (s.refine >= 2);              // the reference solves once; this sweep only forms x
    converged = true;
  } else {
    converged = (s.relres <= o.tol);
    done = (converged && !s.tiny_pending) || (s.refine > o.max_refine) ||
           (tot[0] == 0.0 && !s.tiny_pending);
  }
  if (done) {
    s.outer_active = 0;
    s.hx_fresh = INIT ? 0 : 1;           // a sweep after an update stored H x of the final x
    if (!converged) s.unconverged += 1;
    s.last_relres = s.relres;
    s.last_err = (o.criterion == HF_STOP_RECURSIVE) ? s.err : s.relres;
    s.last_iter = s.step_iters;
    return;
  }
  s.iter = 0;
  if (o.criterion != HF_STOP_RECURSIVE && converged) {   // only the +TINY is left to apply
    s.inner_active = 0;
    return;
  }
  s.inner_active = 1;
  s.gg0 = tot[1];
  s.rho = tot[1];
  s.beta = 0.0;
  s.sigma_prev = s.sigma;
  if (o.precision == HF_PREC_MIXED) {
    s.eta = fmax(o.inner_tol, 0.1 * o.tol / fmax(s.relres, 1e-300));
    const double rms = sqrt(tot[0] / (double)G.n) * G.mean_sinv;
    s.sigma = (rms > 0.0 && isfinite(rms)) ? exp2(rint(log2(rms))) : 1.0;
  } else {
    s.eta = fmax(0.1 * o.tol / fmax(s.relres, 1e-300), 1e-15);
    s.sigma = 1.0;
  }
  if (!(tot[1] > 0.0)) s.inner_active = 0;  // exact already: go straight to the update
  if (s.inner_active && o.criterion == HF_STOP_TRUE && (G.nx & 3) == 0) {
    const int64_t cap = (o.precision == HF_PREC_MIXED) ? (int64_t)o.inner_itmax : o.itmax;
    s.xw = kXwAllowed | (cap <= 1 ? kXwThis : 0);
  }
}


__device__ void epi_spmv_s(InstScal& s, const double* tot) {
  s.pq = tot[0];
  if (tot[0] > 0.0 && isfinite(tot[0])) {
    s.alpha = s.rho / tot[0];
  } else {            // breakdown (p = 0 or non-finite): stop this inner solve
    s.alpha = 0.0;
    s.inner_active = 0;
  }
}


template <typename T>
__device__ void epi_upd_s(InstScal& s, const DevOpts& o, const double* tot) {
  const bool weighted = (o.criterion == HF_STOP_RECURSIVE);
  const double rho_new = tot[0], rho_old = s.rho;
  s.beta = rho_new / s.rho;
  s.rho = rho_new;
  s.iter += 1;
  s.step_iters += 1;
  if (sizeof(T) == 8) s.tot_iters += 1; else s.tot_inner += 1;
  bool stop;
  if (weighted) {
    // err = ||r||/||b|| on the unscaled recursive residual r = -S rh sigma (mod_Sparse.f90:420)
    s.rr_w = tot[1];
    s.err = s.bb > 0.0 ? sqrt(tot[1]) * s.sigma_prev / sqrt(s.bb) : 0.0;
    stop = (s.err <= o.tol);
  } else {
    s.err = s.gg0 > 0.0 ? sqrt(rho_new / s.gg0) : 0.0;
    stop = (s.err <= s.eta);
  }
  const int64_t cap = (sizeof(T) == 8) ? o.itmax : (int64_t)o.inner_itmax;
  if (!stop && s.iter >= cap) {
    stop = true;
    if (weighted) s.unconverged += 1;
  }
  if (!(rho_new > 0.0)) stop = true;
  if (stop) s.inner_active = 0;
  // Fused x update: whether the update that just ran formed x, and whether the next one should.
  // The next iteration is predicted to end the solve when it reaches the iteration cap, or when
  // the criterion shrinks once more by this iteration's factor: err_k^2 (rho_k / rho_(k-1)) <= eta^2.
  const int32_t wrote = (s.xw & kXwThis) ? kXwDone : 0;
  s.xw = (s.xw & kXwAllowed) | wrote;
  if (!stop && (s.xw & kXwAllowed)) {
    const double next = (rho_new / s.gg0) * (rho_new / rho_old);
    if (s.iter + 1 >= cap || next <= s.eta * s.eta) s.xw |= kXwThis;
  }
}


template <bool INIT>
__device__ void epi_residual(const DevArrays& A, int inst, const double* tot) {
  epi_residual_s<INIT>(A.scal[inst], A.inst[inst], A.opts, tot);
}
__device__ void epi_spmv(const DevArrays& A, int inst, const double* tot) { epi_spmv_s(A.scal[inst], tot); }
template <typename T>
__device__ void epi_upd(const DevArrays& A, int inst, const double* tot) {
  epi_upd_s<T>(A.scal[inst], A.opts, tot);
}

// Whether instance s took part in the producing kernel (the producers' own entry tests).
template <int KIND>
__device__ __forceinline__ bool took_part(const InstScal& s) {
  switch (KIND) {
    case FIN_RHS: return s.outer_active != 0;
    case FIN_RHS_DIAG: return (s.status & kStatusRhsNan) != 0;
    case FIN_RES_INIT: return s.outer_active && !s.inner_active && s.refine == 0;
    case FIN_RES: return s.outer_active && !s.inner_active && s.refine != 0;
    default: return s.inner_active != 0;      // FIN_SPMV, FIN_UPD
  }
}

template <int KIND, bool FP32>
__global__ void __launch_bounds__(256) k_finalize(DevArrays A, CtrlState* ctrl,
                                                  cudaGraphConditionalHandle hw, int graph) {
  constexpr int NR = (KIND == FIN_RHS_DIAG) ? 5 : (KIND == FIN_SPMV ? 1 : 2);
  const int inst = blockIdx.x;
  if (KIND == FIN_RHS && inst == 0 && threadIdx.x == 0) A.stamps[kStampFin] = gtimer();
  const InstDesc& d = A.inst[inst];
  if (took_part<KIND>(A.scal[inst])) {
    double acc[NR];
    __shared__ double red[32 * NR];
    instance_sum<NR>(A.partials, d, acc, red);
    if (threadIdx.x == 0) {
      switch (KIND) {
        case FIN_RHS: epi_rhs(A, inst, acc); break;
        case FIN_RHS_DIAG: epi_rhs_diag(A, inst, acc); break;
        case FIN_RES_INIT: epi_residual<true>(A, inst, acc); break;
        case FIN_RES: epi_residual<false>(A, inst, acc); break;
        case FIN_SPMV: epi_spmv(A, inst, acc); break;
        default:
          if (FP32) epi_upd<float>(A, inst, acc); else epi_upd<double>(A, inst, acc);
          break;
      }
    }
  }
  // loop condition of the captured solve loop: set by the last instance block to finish
  if (graph && (KIND == FIN_RES_INIT || KIND == FIN_RES || KIND == FIN_UPD)) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned prev = atomicAdd(&ctrl->fin_count, 1u);
      last = (prev == gridDim.x - 1u);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
      __threadfence();
      int any_outer = 0;
      for (int64_t i = 0; i < A.ninst; ++i) any_outer |= __ldcg(&A.scal[i].outer_active);
      ctrl->fin_count = 0u;
      cudaGraphSetConditional(hw, any_outer ? 1u : 0u);
    }
  }
}

// ---- captured step: control kernels of the conditional nodes -----------------------------------
__global__ void k_graph_step_begin(DevArrays A, CtrlState* ctrl, int launches_per_step) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kStamps) A.stamps[i] = i == kStampBegin ? gtimer() : 0ull;
  if (i == 0) {
    ctrl->loop_iter = 0;
    ctrl->launches += launches_per_step;   // the step's kernels outside the solve loop
  }
  if (i < A.ninst) begin_step(A.scal[i], ctrl->itime);
}

// One block: every instance rotates, then the step counter advances.  A persistent solve that
// gave up (barrier time limit or round bound) is recorded in ctrl->guard_hit, which stays set.
// In a whole-loop graph (loop != 0) it also sets the WHILE condition: another step follows while
// the step counter is below itime_end and no solve has failed, so the loop always ends.
__global__ void k_graph_step_end(DevArrays A, CtrlState* ctrl, const SolveCtl* sctl,
                                 cudaGraphConditionalHandle hloop, int loop) {
  if (threadIdx.x == 0) A.stamps[kStampEnd] = gtimer();
  for (int64_t i = threadIdx.x; i < A.ninst; i += blockDim.x) end_step(A.scal[i]);
  __syncthreads();
  if (threadIdx.x == 0) {
    ctrl->itime += 1;
    if (sctl && (sctl->err || sctl->guard_hit)) ctrl->guard_hit |= sctl->err ? 2 : 1;
    if (loop) cudaGraphSetConditional(hloop, (ctrl->itime < ctrl->itime_end && !ctrl->guard_hit) ? 1u : 0u);
  }
}

// Branch of the solve loop body: 0 = one inner CG iteration, 1 = update + residual, 2 = nothing.
// It also bounds the loop: past ctrl->limit body iterations (or with nothing to do) it clears the
// loop condition, so the WHILE node always terminates.
__global__ void k_ctrl_select(DevArrays A, CtrlState* ctrl, cudaGraphConditionalHandle hs,
                              cudaGraphConditionalHandle hw) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int any_inner = 0, any_outer = 0;
  for (int64_t i = 0; i < A.ninst; ++i) {
    any_inner |= A.scal[i].inner_active;
    any_outer |= A.scal[i].outer_active;
  }
  unsigned branch = any_inner ? 0u : (any_outer ? 1u : 2u);
  const int64_t it = ctrl->loop_iter + 1;
  ctrl->loop_iter = it;
  if (it > ctrl->limit) {
    ctrl->guard_hit = 1;
    branch = 2u;
  }
  ctrl->launches += 1 + (branch == 0u ? 5 : (branch == 1u ? 3 : 0));
  if (branch == 2u) cudaGraphSetConditional(hw, 0u);
  cudaGraphSetConditional(hs, branch);
}

// ---- persistent solve ------------------------------------------------------------------------
// One cooperative launch runs a step's whole refinement loop.  Work proceeds in grid-wide rounds:
// in round r every task does the work of its instance's current phase (PH_*), writing its partial
// sums to its fixed slot; then every block arrives at a grid barrier.  The last block to arrive
// runs the epilogue of every instance -- it sums each instance's task partials in the fixed order
// of instance_sum (the order the finalize kernels use, so every path obtains the same bits) and
// updates the instance's scalars (alpha, beta, convergence test, next phase) in device memory --
// and only then opens the barrier.  Blocks read the scalars of the instances they work on through
// L2 at the start of each round.  Tasks are handed out one at a time from a per-round counter
// (SolveCtl::next_task), so blocks on busier SMs take fewer of them.  The kernel returns when the
// last epilogue reports that no instance has work left.
//
// Termination: every barrier wait is bounded in time (wait_ns, 4 s by default) and in polls; a block that
// gives up records SolveCtl::err and returns, and the blocks still waiting see the flag and return
// too.  The number of rounds is bounded by `limit`.  Co-residency of all blocks, which the barrier
// needs, is guaranteed by the cooperative launch (the grid never exceeds the occupancy bound).

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__device__ __forceinline__ int32_t phase_after(const InstScal& s) {
  if (!s.outer_active) return PH_IDLE;
  // the fused FP32 pass (PH_CG_PQ) measured slower; iteration 0 needs no direction update (p_0 = r)
  if (s.inner_active) return s.iter == 0 ? PH_CG_Q : PH_CG_P;
  return (s.xw & kXwDone) ? PH_RES : PH_XUPD;   // the last CG update may have formed x already
}
__device__ __forceinline__ int phase_partials(int32_t ph) {
  return (ph == PH_RES_INIT || ph == PH_RES || ph == PH_CG_B) ? 2
         : ((ph == PH_CG_Q || ph == PH_CG_PQ) ? 1 : 0);
}

constexpr int kScalWords = (int)(sizeof(InstScal) / 8);
static_assert(sizeof(InstScal) % 8 == 0 && kScalWords < kBlock, "scalar copy");

// Epilogue of one instance after a round (one thread): scalars read through L2, updated, stored.
// Returns whether the instance has work in the next round.
template <typename T>
__device__ int instance_epilogue(const DevArrays& A, int64_t inst, const double (&acc)[2]) {
  InstScal sc;
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(A.scal + inst);
  unsigned long long* w = reinterpret_cast<unsigned long long*>(&sc);
  for (int k = 0; k < kScalWords; ++k) w[k] = __ldcg(src + k);
  const InstDesc& d = A.inst[inst];
  switch (sc.phase) {
    case PH_RES_INIT:
      epi_residual_s<true>(sc, d, A.opts, acc);
      sc.phase = phase_after<T>(sc);
      break;
    case PH_RES:
      epi_residual_s<false>(sc, d, A.opts, acc);
      sc.phase = phase_after<T>(sc);
      break;
    case PH_CG_P: sc.phase = PH_CG_Q; break;
    case PH_CG_Q:
    case PH_CG_PQ:
      epi_spmv_s(sc, acc);
      sc.phase = sc.inner_active ? PH_CG_B : phase_after<T>(sc);
      break;
    case PH_CG_B:
      epi_upd_s<T>(sc, A.opts, acc);
      sc.phase = phase_after<T>(sc);
      break;
    case PH_XUPD: sc.phase = PH_RES; break;
    default: sc.phase = PH_IDLE; break;
  }
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(A.scal + inst);
  for (int k = 0; k < kScalWords; ++k) dst[k] = w[k];
  return sc.phase != PH_IDLE ? 1 : 0;
}

// Epilogues of all instances (the whole last-arriving block).  Large instances (block sums) one
// after the other.  Small ones kBlock at a time: each warp sums the partials of its instances
// (per instance exactly warp_instance_sum's order, as in the finalize kernels), kEpiUnroll
// instances' loads in flight at once, into shared memory; then one thread per instance runs the
// epilogues side by side (with many instances, one lane running them in turn set the round's
// length).  Returns (in every thread) whether any instance has work left.
constexpr int kEpiUnroll = 4;
constexpr int kPhaseCache = 1024;   // instances whose phases a solve block keeps in shared memory
template <typename T>
__device__ int all_epilogues(const DevArrays& A, double* red) {
  __shared__ double s_acc[kBlock][2];
  __shared__ int32_t s_ph[kBlock];
  int act = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t k = 0; k < A.nlarge; ++k) {     // a list: no serial walk over every instance
    const int64_t i = A.large[k];
    const InstDesc& d = A.inst[i];
    const int32_t ph = __ldcg(&A.scal[i].phase);
    double acc[2] = {0.0, 0.0};
    if (phase_partials(ph) > 0) instance_sum<2>(A.partials, d, acc, red);
    if (threadIdx.x == 0) act |= instance_epilogue<T>(A, i, acc);
    __syncthreads();
  }
  for (int64_t base = 0; A.nsmall > 0 && base < A.ninst; base += kBlock) {
    const int nb = (int)(A.ninst - base < kBlock ? A.ninst - base : kBlock);
    if ((int)threadIdx.x < nb) s_ph[threadIdx.x] = __ldcg(&A.scal[base + threadIdx.x].phase);
    __syncthreads();
    for (int j0 = warp * kEpiUnroll; j0 < nb; j0 += (kBlock / 32) * kEpiUnroll) {
      double acc[kEpiUnroll][2];
#pragma unroll
      for (int u = 0; u < kEpiUnroll; ++u) {
        acc[u][0] = 0.0;
        acc[u][1] = 0.0;
        const int j = j0 + u;
        if (j >= nb) continue;
        const InstDesc& d = A.inst[base + j];
        if (d.ntask > kWarpSumMax || phase_partials(s_ph[j]) == 0) continue;
        strided_sum<2>(A.partials, d.task0, d.ntask, lane, 32, acc[u]);
      }
#pragma unroll
      for (int u = 0; u < kEpiUnroll; ++u) {
        const double v0 = warp_sum(acc[u][0]), v1 = warp_sum(acc[u][1]);
        if (lane == 0 && j0 + u < nb) {
          s_acc[j0 + u][0] = v0;
          s_acc[j0 + u][1] = v1;
        }
      }
    }
    __syncthreads();
    if ((int)threadIdx.x < nb && A.inst[base + threadIdx.x].ntask <= kWarpSumMax) {
      const double acc[2] = {s_acc[threadIdx.x][0], s_acc[threadIdx.x][1]};
      act |= instance_epilogue<T>(A, base + threadIdx.x, acc);
    }
    __syncthreads();
  }
  return __syncthreads_or(act);
}

// Grid barrier whose last arriving block runs all epilogues before opening it.  Returns false if
// the wait gave up; `any` = some instance has work in the next round.
template <typename T>
__device__ bool grid_barrier_epilogue(const DevArrays& A, SolveCtl* ctl, unsigned nblocks,
                                      int64_t round, double* red, unsigned long long wait_ns,
                                      unsigned& any) {
  __shared__ unsigned s_gen, s_any;
  __shared__ int s_last, s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = ld_acquire_u32(&ctl->gen);   // cannot advance before this block arrives
    __threadfence();
    const unsigned arrived = atomicAdd(&ctl->count, 1u);
    s_gen = g;
    s_last = (arrived == nblocks - 1) ? 1 : 0;
    if (s_last) __threadfence();                   // every block's partials are visible now
  }
  __syncthreads();
  const unsigned g = s_gen;
  if (s_last) {
    if (threadIdx.x == 0 && round < kRoundLog) {
      int32_t ph = __ldcg(&A.scal[0].phase);
      if (ph == PH_RES_INIT && __ldcg(&A.scal[0].hx_ok) >= 2) ph = HF_PHASE_RES_INIT_HX;
      if (ph == PH_CG_B && (__ldcg(&A.scal[0].xw) & kXwThis)) ph = HF_PHASE_CG_BX;
      ctl->phase_log[round] = ph;
    }
    const int act = all_epilogues<T>(A, red);
    if (threadIdx.x == 0) {
      ctl->next_task[round & 1] = 0u;     // every block is done taking this round's tasks
      ctl->result[(g + 1) & 1] = act ? 1u : 0u;
      const unsigned long long t = gtimer();
      if (round < kRoundLog) ctl->t_round[round] = t;
      A.stamps[kStampSolveEnd] = t;
      ctl->rounds = round + 1;
      ctl->count = 0u;
      __threadfence();
      st_release_u32(&ctl->gen, g + 1);
      s_ok = 1;
    }
  } else if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long t0 = gtimer();
    unsigned polls = 0;
    while (ld_acquire_u32(&ctl->gen) == g) {
      if (*(volatile int*)&ctl->err) { ok = 0; break; }
      if ((++polls & 255u) == 0u && (gtimer() - t0 > wait_ns || polls > (1u << 27))) {
        atomicExch(&ctl->err, 1);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    s_ok = ok;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    s_any = s_ok ? *(volatile unsigned*)&ctl->result[(g + 1) & 1] : 0u;
  }
  __syncthreads();
  any = s_any;
  return s_ok != 0;
}

template <typename T, bool XOUT>
__device__ __forceinline__ void round_task(const DevArrays& A, double* part, int64_t task,
                                           const InstScal& s) {
  if constexpr (sizeof(T) == 4) {
    if (s.phase == PH_CG_PQ || s.phase == PH_CG_Q) {
      if (s.phase == PH_CG_PQ) pq_f32_task<true>(A, part, task, s);
      else pq_f32_task<false>(A, part, task, s);
      return;
    }
  } else {
    if (s.phase == PH_CG_Q) { spmv_task<T, false>(A, part, task, s); return; }
    if (s.phase == PH_CG_PQ) { spmv_task<T, true>(A, part, task, s); return; }
  }
  switch (s.phase) {
    case PH_RES_INIT: res_task<true, T>(A, part, task, s); break;
    case PH_RES: res_task<false, T, XOUT>(A, part, task, s); break;
    case PH_CG_P: cgp_any<T>(A, part, task, s); break;
    case PH_CG_B: upd_any<T>(A, part, task, s); break;
    case PH_XUPD: xupd_any<T>(A, part, task, s); break;
    default: break;
  }
}

// Blocks per SM: 3 (85 registers: the FP64 stencil and the FP32 vector pass need about that).
// XOUT: the instance used by the graphs of host-buffer steps, whose residual sweeps also store x
// into A.xout (a variant of its own, so the other solves carry none of it).
template <typename T, bool XOUT>
__global__ void __launch_bounds__(kBlock, 3)
    k_solve(DevArrays A, SolveCtl* ctl, int64_t limit, unsigned long long wait_ns, int leaver) {
  __shared__ InstScal sh;
  __shared__ double red[32 * 2];
  __shared__ int32_t s_phase[kPhaseCache];
  __shared__ unsigned s_next;
  const unsigned G = gridDim.x;
  const unsigned nt = (unsigned)A.ntasks;
  // several instances: every round starts with all their phases in shared memory, so tasks of
  // instances without work this round are passed over without reading their scalars
  const bool cache = A.ninst > 1 && A.ninst <= kPhaseCache;
  const bool single = A.ninst == 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) A.stamps[kStampSolve] = ctl->t_start = gtimer();
  for (int64_t r = 0;; ++r) {
    if (r >= limit) {
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->guard_hit = 1;
      return;
    }
    // odd rounds walk the tasks backwards, so a round starts on the data the previous round wrote
    // last, which is still in L2 (the partial sums have fixed slots: the order changes no bits)
    int cur = single ? 0 : -1;
    if (cache) {
      for (int i = threadIdx.x; i < (int)A.ninst; i += kBlock) s_phase[i] = __ldcg(&A.scal[i].phase);
    }
    // tasks are handed out one at a time from a counter, so a block on a busier SM takes fewer
    // (every SM holds the same number of blocks, but a round lasts as long as its slowest SM);
    // each block asks for its next task while it runs the current one.  With one instance its
    // scalars are loaded beside the first request (threads 1..kScalWords), not after it.
    if (threadIdx.x == 0) s_next = atomicAdd(&ctl->next_task[r & 1], 1u);
    if (single && threadIdx.x >= 1 && (int)threadIdx.x <= kScalWords)
      reinterpret_cast<unsigned long long*>(&sh)[threadIdx.x - 1] =
          __ldcg(reinterpret_cast<const unsigned long long*>(A.scal) + threadIdx.x - 1);
    __syncthreads();
    for (unsigned k = s_next; k < nt;) {
      __syncthreads();                       // every thread has read s_next
      if (threadIdx.x == 0) s_next = atomicAdd(&ctl->next_task[r & 1], 1u);
      const unsigned t = (r & 1) ? nt - 1 - k : k;
      const int inst = A.tasks[t].x;
      const bool skip = cache && s_phase[inst] == PH_IDLE;
      if (!skip) {
        if (inst != cur) {                   // this instance's scalars, through L2
          __syncthreads();
          if ((int)threadIdx.x < kScalWords)
            reinterpret_cast<unsigned long long*>(&sh)[threadIdx.x] =
                __ldcg(reinterpret_cast<const unsigned long long*>(A.scal + inst) + threadIdx.x);
          __syncthreads();
          cur = inst;
        }
        if (sh.phase != PH_IDLE) round_task<T, XOUT>(A, A.partials, t, sh);
      }
      __syncthreads();                       // s_next holds the block's next task
      k = s_next;
    }
    unsigned any = 0;
    // failure-path check only (leaver >= 0): that block leaves without arriving, so the others'
    // waits run out and record SolveCtl::err
    if ((int)blockIdx.x == leaver) return;
    if (!grid_barrier_epilogue<T>(A, ctl, G, r, red, wait_ns, any)) return;
    if (!any) return;
  }
}

// Largest co-resident grid of the persistent solve (cooperative launch bound), capped by tasks.
int solve_grid_blocks(Ctx& c, int fp32) {
  int& cached = c.solve_blocks[fp32 ? 1 : 0];
  if (cached > 0) return cached;
  int per_sm = 0, per_sm_x = 0, nsm = 0;
  cudaError_t e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve<float, false>, kBlock, 0)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve<double, false>, kBlock, 0);
  if (e != cudaSuccess) return -1;
  e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_x, k_solve<float, true>, kBlock, 0)
           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_x, k_solve<double, true>, kBlock, 0);
  if (e != cudaSuccess) return -1;
  if (per_sm_x < per_sm) per_sm = per_sm_x;    // one grid size for both variants
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess) return -1;
  // every SM holds the same number of blocks; tasks are handed out one at a time, so the blocks
  // of busier SMs take fewer of them
  int64_t g = (int64_t)per_sm * nsm;
  if (g > c.ntasks) g = c.ntasks;
  if (g < 1) return -1;
  cached = (int)g;
  return cached;
}

// Zero the control block, then launch the persistent solve cooperatively on the context stream.
cudaError_t launch_solve(Ctx& c, unsigned long long wait_ns, int leaver) {
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  const int g = solve_grid_blocks(c, fp32 ? 1 : 0);
  if (g < 1) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaMemsetAsync(c.d_sctl, 0, sizeof(SolveCtl), c.stream);
  if (e != cudaSuccess) return e;
  const int64_t per = fp32 ? c.opts.inner_itmax : c.opts.itmax;
  const int64_t limit = (int64_t)(c.opts.max_refine + 3) * (3 * per + 6) + 8;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)g);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (c.A.xout) {
    if (fp32) return cudaLaunchKernelEx(&cfg, k_solve<float, true>, c.A, c.d_sctl, limit, wait_ns, leaver);
    return cudaLaunchKernelEx(&cfg, k_solve<double, true>, c.A, c.d_sctl, limit, wait_ns, leaver);
  }
  if (fp32) return cudaLaunchKernelEx(&cfg, k_solve<float, false>, c.A, c.d_sctl, limit, wait_ns, leaver);
  return cudaLaunchKernelEx(&cfg, k_solve<double, false>, c.A, c.d_sctl, limit, wait_ns, leaver);
}

#ifdef HF_CHECKED
// One failed check and no memory access (the index is only compared with its range), so a test
// can see a failed check recorded and reported.
__global__ void k_check_probe(DevArrays A) { (void)HF_IX(A, -1, 1); }
cudaError_t launch_check_probe(Ctx& c) {
  k_check_probe<<<1, 1, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}
#endif

// ---- launchers ---------------------------------------------------------------------------------
cudaError_t launch_step_begin(Ctx& c, int64_t itime, int) {
  k_step_begin<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A, itime);
  return cudaGetLastError();
}

cudaError_t launch_step_end(Ctx& c) {
  k_step_end<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}

// mode 0: initial residual (+ finalize); mode 1: solution update + residual (+ finalize)
cudaError_t launch_residual(Ctx& c, int mode, CtrlState* ctrl, cudaGraphConditionalHandle hw,
                            int graph) {
  const unsigned nb = (unsigned)c.ntasks;
  const bool mixed = c.opts.precision == HF_PREC_MIXED;
  if (mode == 0) {
    if (mixed) k_residual<true, float><<<nb, kBlock, 0, c.stream>>>(c.A);
    else k_residual<true, double><<<nb, kBlock, 0, c.stream>>>(c.A);
    return launch_finalize(c, FIN_RES_INIT, ctrl, hw, graph);
  }
  if (mixed) {
    k_xupdate<float><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_residual<false, float><<<nb, kBlock, 0, c.stream>>>(c.A);
  } else {
    k_xupdate<double><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_residual<false, double><<<nb, kBlock, 0, c.stream>>>(c.A);
  }
  return launch_finalize(c, FIN_RES, ctrl, hw, graph);
}

cudaError_t launch_inner_iteration(Ctx& c, int fp32, CtrlState* ctrl,
                                   cudaGraphConditionalHandle hw, int graph) {
  const unsigned nb = (unsigned)c.ntasks;
  if (fp32) {
    k_cg_p<float><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_spmv<float><<<nb, kBlock, 0, c.stream>>>(c.A);
  } else {
    k_cg_p<double><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_spmv<double><<<nb, kBlock, 0, c.stream>>>(c.A);
  }
  cudaError_t e = launch_finalize(c, FIN_SPMV, ctrl, hw, graph);
  if (e != cudaSuccess) return e;
  if (fp32) k_cg_upd<float><<<nb, kBlock, 0, c.stream>>>(c.A);
  else k_cg_upd<double><<<nb, kBlock, 0, c.stream>>>(c.A);
  return launch_finalize(c, FIN_UPD, ctrl, hw, graph);
}

cudaError_t launch_graph_step_begin(Ctx& c, CtrlState* ctrl, int launches_per_step) {
  k_graph_step_begin<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A, ctrl,
                                                                               launches_per_step);
  return cudaGetLastError();
}
cudaError_t launch_graph_step_end(Ctx& c, CtrlState* ctrl, const SolveCtl* sctl,
                                  cudaGraphConditionalHandle hloop, int loop) {
  k_graph_step_end<<<1, 256, 0, c.stream>>>(c.A, ctrl, sctl, hloop, loop);
  return cudaGetLastError();
}
cudaError_t launch_ctrl_select(Ctx& c, CtrlState* ctrl, cudaGraphConditionalHandle hs,
                               cudaGraphConditionalHandle hw) {
  k_ctrl_select<<<1, 32, 0, c.stream>>>(c.A, ctrl, hs, hw);
  return cudaGetLastError();
}

cudaError_t launch_finalize(Ctx& c, int kind, CtrlState* ctrl, cudaGraphConditionalHandle hw,
                            int graph) {
  const unsigned nb = (unsigned)c.ninst;
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  switch (kind) {
    case FIN_RHS: k_finalize<FIN_RHS, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph); break;
    case FIN_RHS_DIAG: k_finalize<FIN_RHS_DIAG, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph); break;
    case FIN_RES_INIT: k_finalize<FIN_RES_INIT, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph); break;
    case FIN_RES: k_finalize<FIN_RES, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph); break;
    case FIN_SPMV: k_finalize<FIN_SPMV, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph); break;
    case FIN_UPD:
      if (fp32) k_finalize<FIN_UPD, true><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph);
      else k_finalize<FIN_UPD, false><<<nb, 256, 0, c.stream>>>(c.A, ctrl, hw, graph);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// One kernel of the step, for timing (hf_time_kernel).
cudaError_t launch_single(Ctx& c, int which) {
  const unsigned nb = (unsigned)c.ntasks;
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  switch (which) {
    case HF_KERNEL_RHS: return launch_rhs(c);
    case HF_KERNEL_RESIDUAL:
      if (fp32) k_residual<false, float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_residual<false, double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_RESIDUAL_INIT:
      if (fp32) k_residual<true, float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_residual<true, double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_XUPDATE:
      if (fp32) k_xupdate<float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_xupdate<double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_CG_P:
      if (fp32) k_cg_p<float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_cg_p<double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_CG_SPMV:
      if (fp32) k_cg_spmv<float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_cg_spmv<double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_CG_UPDATE:
      if (fp32) k_cg_upd<float><<<nb, kBlock, 0, c.stream>>>(c.A);
      else k_cg_upd<double><<<nb, kBlock, 0, c.stream>>>(c.A);
      break;
    case HF_KERNEL_CG_PQ:
      if (fp32) {
        k_cg_pq_f32<<<nb, kBlock, 0, c.stream>>>(c.A);
      } else {
        k_cg_p<double><<<nb, kBlock, 0, c.stream>>>(c.A);
        k_cg_spmv<double><<<nb, kBlock, 0, c.stream>>>(c.A);
      }
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hf
