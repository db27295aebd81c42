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
}

// Finished steps rotate the temperature roles: T^(n-1) <- T^n, T^n <- x (mod_evolve.f90:169-170).
__device__ __forceinline__ void end_step(InstScal& s) {
  if (s.status != 0) return;
  const int r0 = s.role[0], r1 = s.role[1], r2 = s.role[2], r3 = s.role[3];
  s.role[0] = r2;  // x
  s.role[1] = r0;  // old T^n
  s.role[2] = r1;  // free
  s.role[3] = r3;  // free
}

__global__ void k_step_begin(DevArrays A, int64_t itime) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.ninst) begin_step(A.scal[i], itime);
}

__global__ void k_step_end(DevArrays A) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.ninst) end_step(A.scal[i]);
}

// ---- neighbour access for the columns of a task ------------------------------------------------
// x neighbours come from the lanes of the same warp (shuffles; across chunk boundaries from the
// first/last lane of the next/previous chunk); lanes at a task edge, periodic wraps and the y
// neighbours are loaded; the z neighbours roll through registers as the block marches along z.
// Inactive lanes hold zeros, so every lane can take part in the shuffles.
constexpr unsigned kFull = 0xffffffffu;

// West/east values and west face of chunk j at local cell l.
template <typename T, typename C, class V>
__device__ __forceinline__ void x_nbrs(const TCell& c, int j, const T (&vc)[kXC],
                                       const C (&cxc)[kXC], int l, V v, const C* __restrict__ cx,
                                       T& vw, C& cxw, T& ve) {
  const T up = __shfl_up_sync(kFull, vc[j], 1);
  const C cup = __shfl_up_sync(kFull, cxc[j], 1);
  const T dn = __shfl_down_sync(kFull, vc[j], 1);
  const T prev_last = __shfl_sync(kFull, vc[j > 0 ? j - 1 : 0], 31);
  const C cprev_last = __shfl_sync(kFull, cxc[j > 0 ? j - 1 : 0], 31);
  const T next_first = __shfl_sync(kFull, vc[j + 1 < kXC ? j + 1 : j], 0);
  vw = T(0); cxw = C(0); ve = T(0);
  if (!c.act(j)) return;
  const int x = c.x(j), nx = c.nx;
  if (c.lane > 0) { vw = up; cxw = cup; }
  else if (j > 0) { vw = prev_last; cxw = cprev_last; }
  else if (x > 0) { vw = v(l - 1); cxw = cx[l - 1]; }
  else if (c.px && nx > 1) { vw = v(l + nx - 1); cxw = cx[l + nx - 1]; }
  if (x + 1 < nx) {
    if (c.lane < 31) ve = dn;
    else if (j + 1 < kXC) ve = next_first;
    else ve = v(l + 1);
  } else if (c.px && nx > 1) {
    ve = v(l - (nx - 1));
  }
}

// The y faces of cell l (chunk j active): fold(coef, value).
template <typename T, typename C, class V, class F>
__device__ __forceinline__ void y_faces(const TCell& c, int l, C cyc, V v, const C* __restrict__ cy,
                                        F fold) {
  if (c.ny < 2) return;
  const int nx = c.nx;
  if (c.y + 1 < c.ny) fold(cyc, v(l + nx));
  else if (c.py) fold(cyc, v(l - (c.ny - 1) * nx));
  if (c.y > 0) fold(cy[l - nx], v(l - nx));
  else if (c.py) fold(cy[l + (c.ny - 1) * nx], v(l + (c.ny - 1) * nx));
}

// Value and z-face of plane z0-1 of chunk j (zeros at a non-periodic bottom face).
template <typename T, typename C, class V>
__device__ __forceinline__ void plane_below(const TCell& c, int j, V v, const C* __restrict__ cz,
                                            T& vm, C& czm) {
  vm = T(0);
  czm = C(0);
  if (!c.act(j) || c.nz < 2) return;
  int l;
  if (c.z0 > 0) l = c.base(j) + (c.z0 - 1) * c.nxy;
  else if (c.pz) l = c.base(j) + (c.nz - 1) * c.nxy;
  else return;
  vm = v(l);
  czm = cz[l];
}

template <typename T, class V>
__device__ __forceinline__ T plane_above(const TCell& c, int j, V v, int z) {
  if (!c.act(j) || c.nz < 2) return T(0);
  if (z + 1 < c.nz) return v(c.base(j) + (z + 1) * c.nxy);
  if (c.pz) return v(c.base(j));
  return T(0);
}

// FP32 block sum of one value into partial slot k of a task (one conversion per block).
__device__ __forceinline__ void task_store_f(const DevArrays& A, int64_t task, int k, float v) {
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
    if (lane == 0) A.partials[task * kNR + k] = (double)v;
  }
}

// ---- FP64 true residual ------------------------------------------------------------------------
// r = S - H x with x in the x-read buffer (INIT: x0 from the RHS kernel) or, after an update, in
// the x-write buffer (the finalize then swaps the roles).  Writes g = -S^-1 r / sigma into the
// inner residual (type TR).  FP64 work per cell: 7 FMA for S - Hx, 1 FMA for ||r||^2.
template <bool INIT, typename TR>
__global__ void __launch_bounds__(kBlock) k_residual(DevArrays A) {
  const int64_t task = blockIdx.x;
  const TCell c = task_cell(A, task);
  const InstScal& s = A.scal[c.inst];
  if (!s.outer_active || s.inner_active) return;
  if (INIT != (s.refine == 0)) return;
  const int64_t off = c.off;
  const double* __restrict__ X = A.tbuf[INIT ? s.role[2] : s.role[3]] + off;
  const double* __restrict__ diag = A.diag + off;
  const double* __restrict__ b = A.b + off;
  const double* __restrict__ cx = A.cx + off;
  const double* __restrict__ cy = A.cy + off;
  const double* __restrict__ cz = A.cz + off;
  const double* __restrict__ rsum = A.rsum + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const double* __restrict__ sinv = A.sinv + off;
  TR* __restrict__ R = Vec<TR>::r(A) + off;
  const float isig = (float)(1.0 / s.sigma);
  // INIT: the residual of x0 + TINY (mod_evolve.f90:141) is r(x0) - TINY * H1
  const bool tiny = INIT && s.x0flag;
  auto xval = [&](int m) -> double { return X[m]; };
  double xm[kXC], czm[kXC], xc[kXC];
#pragma unroll
  for (int j = 0; j < kXC; ++j) {
    plane_below<double>(c, j, xval, cz, xm[j], czm[j]);
    xc[j] = c.act(j) ? X[c.base(j) + c.z0 * c.nxy] : 0.0;
  }
  double rr = 0.0, gg64 = 0.0;
  float gg = 0.f;
  for (int z = c.z0; z < c.z1; ++z) {
    double xn[kXC], cxc[kXC], acc[kXC];
#pragma unroll
    for (int j = 0; j < kXC; ++j) {
      const int l = c.base(j) + z * c.nxy;
      const bool a = c.act(j);
      xn[j] = plane_above<double>(c, j, xval, z);
      cxc[j] = a ? cx[l] : 0.0;
      acc[j] = 0.0;
      if (a) {
        acc[j] = fma(-diag[l], xc[j], b[l]);
        if (tiny) acc[j] = fma(-kTiny, rsum[l], acc[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < kXC; ++j) {
      const int l = c.base(j) + z * c.nxy;
      double xw, cxw, xe;
      x_nbrs(c, j, xc, cxc, l, xval, cx, xw, cxw, xe);
      if (!c.act(j)) continue;
      double a = acc[j];
      a = fma(-cxc[j], xe, a);
      a = fma(-cxw, xw, a);
      y_faces<double>(c, l, cy[l], xval, cy, [&](double cf, double xv) { a = fma(-cf, xv, a); });
      if (c.nz > 1) {
        a = fma(-cz[l], xn[j], a);
        a = fma(-czm[j], xm[j], a);
      }
      rr = fma(a, a, rr);
      if (sizeof(TR) == 4) {             // mixed: g in FP32, scaled by 1/sigma
        const float g = -sinv32[l] * f64_to_f32_trunc(a) * isig;
        R[l] = (TR)g;
        gg = fmaf(g, g, gg);
      } else {                           // FP64 path: sigma = 1
        const double g = -sinv[l] * a;
        R[l] = (TR)g;
        gg64 = fma(g, g, gg64);
      }
      czm[j] = cz[l];
    }
#pragma unroll
    for (int j = 0; j < kXC; ++j) { xm[j] = xc[j]; xc[j] = xn[j]; }
  }
  if (sizeof(TR) == 4) {
    task_store_f(A, task, 1, gg);
    const double v[1] = {rr};
    tile_store<1>(A, task, v);
  } else {
    const double v[2] = {rr, gg64};
    tile_store<2>(A, task, v);
  }
}

// ---- solution update: x_new = x + sigma S^-1 y (+ TINY once) -----------------------------------
template <typename TY>
__global__ void __launch_bounds__(kBlock) k_xupdate(DevArrays A) {
  const TCell c = task_cell(A, blockIdx.x);
  const InstScal& s = A.scal[c.inst];
  if (!s.outer_active || s.inner_active || s.refine == 0) return;
  const int64_t off = c.off;
  const double* __restrict__ XR = A.tbuf[s.role[2]] + off;
  double* __restrict__ XW = A.tbuf[s.role[3]] + off;
  const TY* __restrict__ Y = Vec<TY>::y(A) + off;
  const double* __restrict__ sinv = A.sinv + off;
  const float* __restrict__ sinv32 = A.sinv32 + off;
  const bool use_y = s.iter > 0;
  const bool tiny = s.tiny_pending != 0;
  const float sig = (float)s.sigma_prev;
  for (int z = c.z0; z < c.z1; ++z) {
#pragma unroll
    for (int j = 0; j < kXC; ++j) {
      if (!c.act(j)) continue;
      const int l = c.base(j) + z * c.nxy;
      double x = XR[l];
      if (tiny) x = x + kTiny;
      if (use_y) {
        if (sizeof(TY) == 8) x = fma(sinv[l], (double)Y[l], x);   // sigma = 1 on the FP64 path
        else x = x + f32_to_f64(sig * sinv32[l] * (float)Y[l]);
      }
      XW[l] = x;
    }
  }
}

// ---- inner CG on Ah (type T) -------------------------------------------------------------------
// The direction p_k = r + beta p_(k-1) (p_0 = r) is written to the buffer of parity k; the
// previous direction is read from the other buffer of the pair.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_p(DevArrays A) {
  const TCell c = task_cell(A, blockIdx.x);
  const InstScal& s = A.scal[c.inst];
  if (!s.inner_active) return;
  const int64_t k = s.iter;
  const bool first = (k == 0);
  const T beta = (T)s.beta;
  const T* __restrict__ R = Vec<T>::r(A) + c.off;
  const T* __restrict__ Po = Vec<T>::pb(A, k + 1) + c.off;
  T* __restrict__ Pn = Vec<T>::pb(A, k) + c.off;
#pragma unroll
  for (int j = 0; j < kXC; ++j) {
    if (!c.act(j)) continue;
#pragma unroll 4
    for (int z = c.z0; z < c.z1; ++z) {
      const int l = c.base(j) + z * c.nxy;
      Pn[l] = first ? R[l] : fma(beta, Po[l], R[l]);
    }
  }
}

// k_cg_spmv: q = Ah p_k and p_k.q.  One column per thread; the operands of plane z+1 (its
// coefficients, y neighbours and plane z+2) are loaded while plane z is computed, so each
// thread keeps two planes of loads in flight.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_spmv(DevArrays A) {
  static_assert(kXC == 1, "one column per thread");
  const int64_t task = blockIdx.x;
  const TCell c = task_cell(A, task);
  const InstScal& s = A.scal[c.inst];
  if (!s.inner_active) return;
  const int64_t off = c.off;
  const T* __restrict__ P = Vec<T>::pb(A, s.iter) + off;
  T* __restrict__ Q = Vec<T>::q(A) + off;
  const T* __restrict__ ax = Vec<T>::ax(A) + off;
  const T* __restrict__ ay = Vec<T>::ay(A) + off;
  const T* __restrict__ az = Vec<T>::az(A) + off;
  const bool act = c.act(0);
  const int nx = c.nx, ny = c.ny, nxy = c.nxy, base = c.base(0);
  auto pv = [&](int m) -> T { return P[m]; };
  // operands of one plane: own value, its faces, y neighbours (+ south face)
  struct Plane { T p, axc, ayc, azc, pnn, ps, ays; };
  auto load = [&](int z, Plane& o) {
    o = Plane{T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
    if (!act || z >= c.nz) return;
    const int l = base + z * nxy;
    o.p = P[l]; o.axc = ax[l]; o.ayc = ay[l]; o.azc = az[l];
    if (ny > 1) {
      if (c.y + 1 < ny) o.pnn = P[l + nx];
      else if (c.py) o.pnn = P[l - (ny - 1) * nx];
      if (c.y > 0) { o.ps = P[l - nx]; o.ays = ay[l - nx]; }
      else if (c.py) { o.ps = P[l + (ny - 1) * nx]; o.ays = ay[l + (ny - 1) * nx]; }
    }
  };
  T pm, azm;
  plane_below<T>(c, 0, pv, az, pm, azm);
  Plane cur, nxt;
  load(c.z0, cur);
  T pq = T(0);
  for (int z = c.z0; z < c.z1; ++z) {
    // plane z+1 (wrapping to 0 on a periodic z axis) is both the next plane and the z+ value
    if (z + 1 < c.nz) load(z + 1, nxt);
    else {
      nxt = Plane{T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
      if (act && c.pz && c.nz > 1) nxt.p = P[base];
    }
    const int l = base + z * nxy;
    T pcv[kXC] = {cur.p};
    T axv[kXC] = {cur.axc};
    T pw, axw, pe;
    x_nbrs(c, 0, pcv, axv, l, pv, ax, pw, axw, pe);
    if (act) {
      T acc = cur.p;
      acc = fma(cur.axc, pe, acc);
      acc = fma(axw, pw, acc);
      if (ny > 1) {
        acc = fma(cur.ayc, cur.pnn, acc);
        acc = fma(cur.ays, cur.ps, acc);
      }
      if (c.nz > 1) {
        acc = fma(cur.azc, nxt.p, acc);
        acc = fma(azm, pm, acc);
      }
      Q[l] = acc;
      pq = fma(cur.p, acc, pq);
    }
    pm = cur.p; azm = cur.azc;
    cur = nxt;
  }
  if (sizeof(T) == 4) {
    task_store_f(A, task, 0, (float)pq);
  } else {
    const double v[1] = {(double)pq};
    tile_store<1>(A, task, v);
  }
}

// k_cg_upd: y += alpha p, r -= alpha q, r.r (and the unscaled ||r||^2 for the reference rule)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_upd(DevArrays A) {
  const int64_t task = blockIdx.x;
  const TCell c = task_cell(A, task);
  const InstScal& s = A.scal[c.inst];
  if (!s.inner_active) return;
  const DevOpts& o = A.opts;
  const bool weighted = (o.criterion == HF_STOP_RECURSIVE);
  const T alpha = (T)s.alpha;
  const bool first = (s.iter == 0);
  const int64_t off = c.off;
  T* __restrict__ Y = Vec<T>::y(A) + off;
  T* __restrict__ R = Vec<T>::r(A) + off;
  const T* __restrict__ P = Vec<T>::pb(A, s.iter) + off;
  const T* __restrict__ Q = Vec<T>::q(A) + off;
  const double* __restrict__ diag = A.diag + off;
  T rr = T(0);
  double rw = 0.0;
  for (int z = c.z0; z < c.z1; ++z) {
#pragma unroll
    for (int j = 0; j < kXC; ++j) {
      if (!c.act(j)) continue;
      const int l = c.base(j) + z * c.nxy;
      const T pv = P[l];
      Y[l] = first ? alpha * pv : fma(alpha, pv, Y[l]);
      const T rv = fma(-alpha, Q[l], R[l]);
      R[l] = rv;
      rr = fma(rv, rv, rr);
      if (weighted) rw = fma(-diag[l] * (double)rv, (double)rv, rw);
    }
  }
  if (sizeof(T) == 4 && !weighted) {
    task_store_f(A, task, 0, (float)rr);
  } else {
    const double v[2] = {(double)rr, rw};
    tile_store<2>(A, task, v);
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
__device__ void epi_residual(const DevArrays& A, int inst, const double* tot) {
  InstScal& s = A.scal[inst];
  const InstDesc& G = A.inst[inst];
  const DevOpts& o = A.opts;
  if (!INIT) {
    const int t = s.role[2]; s.role[2] = s.role[3]; s.role[3] = t;
    s.tiny_pending = 0;
  } else {
    s.tiny_pending = s.x0flag;
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
}


__device__ void epi_spmv(const DevArrays& A, int inst, const double* tot) {
  InstScal& s = A.scal[inst];
  s.pq = tot[0];
  if (tot[0] > 0.0 && isfinite(tot[0])) {
    s.alpha = s.rho / tot[0];
  } else {            // breakdown (p = 0 or non-finite): stop this inner solve
    s.alpha = 0.0;
    s.inner_active = 0;
  }
}


template <typename T>
__device__ void epi_upd(const DevArrays& A, int inst, const double* tot) {
  InstScal& s = A.scal[inst];
  const DevOpts& o = A.opts;
  const bool weighted = (o.criterion == HF_STOP_RECURSIVE);
  const double rho_new = tot[0];
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
  const InstDesc& d = A.inst[inst];
  if (took_part<KIND>(A.scal[inst])) {
    double acc[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) acc[k] = 0.0;
    for (int64_t t = threadIdx.x; t < d.ntask; t += blockDim.x) {
#pragma unroll
      for (int k = 0; k < NR; ++k) acc[k] += A.partials[(d.task0 + t) * kNR + k];
    }
    __shared__ double red[32 * NR];
    block_sum<NR>(acc, red);
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
__global__ void k_graph_step_begin(DevArrays A, CtrlState* ctrl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    ctrl->loop_iter = 0;
    ctrl->launches += 6;   // step begin, RHS + finalize, initial residual + finalize, step end
  }
  if (i < A.ninst) begin_step(A.scal[i], ctrl->itime);
}

// One block: every instance rotates, then the step counter advances.
__global__ void k_graph_step_end(DevArrays A, CtrlState* ctrl) {
  for (int64_t i = threadIdx.x; i < A.ninst; i += blockDim.x) end_step(A.scal[i]);
  __syncthreads();
  if (threadIdx.x == 0) ctrl->itime += 1;
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

cudaError_t launch_graph_step_begin(Ctx& c, CtrlState* ctrl) {
  k_graph_step_begin<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A, ctrl);
  return cudaGetLastError();
}
cudaError_t launch_graph_step_end(Ctx& c, CtrlState* ctrl) {
  k_graph_step_end<<<1, 256, 0, c.stream>>>(c.A, ctrl);
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
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hf
