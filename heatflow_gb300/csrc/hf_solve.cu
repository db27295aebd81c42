// Linear solve of one implicit step, H x = S (linbcg, mod_Sparse.f90:372-434, replaced).
//
// Method.  H is symmetric negative definite, so the reference's Jacobi-preconditioned BiCG is,
// in exact arithmetic, Jacobi-PCG (rr == r, pp == p).  The GPU runs the same iteration as plain CG
// on the symmetrically scaled operator  Ah = S^-1 (-H) S^-1,  S = diag(sqrt|H_II|), whose diagonal
// is 1: identical iterates, no divisions and one coefficient array fewer per pass.
//
// Each step is a refinement loop:
//   x = x0 (+TINY)                                         k_residual<INIT>
//   repeat:  r = S - H x (FP64, true residual), test ||r||/||S||
//            g = -S^-1 r / sigma ; solve Ah y = g by CG       (FP64, or FP32 in mixed mode)
//            x += sigma S^-1 y                              k_residual<UPDATE> (fused with the next r)
// The FP64 path asks its CG for the whole reduction at once (one sweep normally suffices); the
// mixed path runs FP32 CG with FP32 SpMV accumulation and refines in FP64.
//
// All solver state is per instance in device memory; tiles of instances that are not in the
// phase a kernel serves return at once (per-instance convergence masks).
#include "hf_ctx.cuh"

namespace hf {

enum { RES_INIT = 0, RES_UPDATE = 1 };

// y = H x for local cell l (unscaled operator, FP64).  xv(n) yields x at local cell n.
template <class XF>
__device__ __forceinline__ double apply_H(const DevArrays& A, const InstDesc& d, int64_t g,
                                          int64_t l, const Coord& c, XF xv) {
  const int64_t nx = d.nx, nxy = (int64_t)d.nx * d.ny;
  double acc = A.diag[g] * xv(l);
  if (c.x + 1 < d.nx) acc = fma(A.cx[g], xv(l + 1), acc);
  else if (d.px && d.nx > 1) acc = fma(A.cx[g], xv(l - (nx - 1)), acc);
  if (c.x > 0) acc = fma(A.cx[g - 1], xv(l - 1), acc);
  else if (d.px && d.nx > 1) acc = fma(A.cx[g + nx - 1], xv(l + nx - 1), acc);
  if (c.y + 1 < d.ny) acc = fma(A.cy[g], xv(l + nx), acc);
  else if (d.py && d.ny > 1) acc = fma(A.cy[g], xv(l - (int64_t)(d.ny - 1) * nx), acc);
  if (c.y > 0) acc = fma(A.cy[g - nx], xv(l - nx), acc);
  else if (d.py && d.ny > 1) acc = fma(A.cy[g + (int64_t)(d.ny - 1) * nx], xv(l + (int64_t)(d.ny - 1) * nx), acc);
  if (c.z + 1 < d.nz) acc = fma(A.cz[g], xv(l + nxy), acc);
  else if (d.pz && d.nz > 1) acc = fma(A.cz[g], xv(l - (int64_t)(d.nz - 1) * nxy), acc);
  if (c.z > 0) acc = fma(A.cz[g - nxy], xv(l - nxy), acc);
  else if (d.pz && d.nz > 1) acc = fma(A.cz[g + (int64_t)(d.nz - 1) * nxy], xv(l + (int64_t)(d.nz - 1) * nxy), acc);
  return acc;
}

// q = Ah p for local cell l (unit diagonal, coefficients a already carry the minus sign).
template <typename T, class PF>
__device__ __forceinline__ T apply_Ah(const T* ax, const T* ay, const T* az, const InstDesc& d,
                                      int64_t g, int64_t l, const Coord& c, PF pv) {
  const int64_t nx = d.nx, nxy = (int64_t)d.nx * d.ny;
  T acc = pv(l);
  if (c.x + 1 < d.nx) acc = fma(ax[g], pv(l + 1), acc);
  else if (d.px && d.nx > 1) acc = fma(ax[g], pv(l - (nx - 1)), acc);
  if (c.x > 0) acc = fma(ax[g - 1], pv(l - 1), acc);
  else if (d.px && d.nx > 1) acc = fma(ax[g + nx - 1], pv(l + nx - 1), acc);
  if (c.y + 1 < d.ny) acc = fma(ay[g], pv(l + nx), acc);
  else if (d.py && d.ny > 1) acc = fma(ay[g], pv(l - (int64_t)(d.ny - 1) * nx), acc);
  if (c.y > 0) acc = fma(ay[g - nx], pv(l - nx), acc);
  else if (d.py && d.ny > 1) acc = fma(ay[g + (int64_t)(d.ny - 1) * nx], pv(l + (int64_t)(d.ny - 1) * nx), acc);
  if (c.z + 1 < d.nz) acc = fma(az[g], pv(l + nxy), acc);
  else if (d.pz && d.nz > 1) acc = fma(az[g], pv(l - (int64_t)(d.nz - 1) * nxy), acc);
  if (c.z > 0) acc = fma(az[g - nxy], pv(l - nxy), acc);
  else if (d.pz && d.nz > 1) acc = fma(az[g + (int64_t)(d.nz - 1) * nxy], pv(l + (int64_t)(d.nz - 1) * nxy), acc);
  return acc;
}

template <typename T> struct Vec;
template <> struct Vec<double> {
  __device__ static double* y(const DevArrays& A) { return A.y; }
  __device__ static double* r(const DevArrays& A) { return A.r; }
  __device__ static double* p(const DevArrays& A) { return A.p; }
  __device__ static double* q(const DevArrays& A) { return A.q; }
  __device__ static const double* ax(const DevArrays& A) { return A.a64x; }
  __device__ static const double* ay(const DevArrays& A) { return A.a64y; }
  __device__ static const double* az(const DevArrays& A) { return A.a64z; }
};
template <> struct Vec<float> {
  __device__ static float* y(const DevArrays& A) { return A.y32; }
  __device__ static float* r(const DevArrays& A) { return A.r32; }
  __device__ static float* p(const DevArrays& A) { return A.p32; }
  __device__ static float* q(const DevArrays& A) { return A.q32; }
  __device__ static const float* ax(const DevArrays& A) { return A.a32x; }
  __device__ static const float* ay(const DevArrays& A) { return A.a32y; }
  __device__ static const float* az(const DevArrays& A) { return A.a32z; }
};

// ---- step bookkeeping ------------------------------------------------------------------------
__global__ void k_step_begin(DevArrays A, int64_t itime) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ninst) return;
  InstScal& s = A.scal[i];
  s.itime = itime;
  s.outer_active = (s.status == 0) ? 1 : 0;
  s.inner_active = 0;
  s.refine = 0;
  s.iter = 0;
  s.step_iters = 0;
  s.x0flag = 0;
  s.err = 0.0;
}

// Finished steps rotate the temperature roles: T^(n-1) <- T^n, T^n <- x (mod_evolve.f90:169-170).
__global__ void k_step_end(DevArrays A) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ninst) return;
  InstScal& s = A.scal[i];
  if (s.status != 0) return;
  int r0 = s.role[0], r1 = s.role[1], r2 = s.role[2], r3 = s.role[3];
  s.role[0] = r2;  // x
  s.role[1] = r0;  // old T^n
  s.role[2] = r1;  // free
  s.role[3] = r3;  // free
}

// ---- FP64 residual sweep (+ solution update) ---------------------------------------------------
// MODE RES_INIT:   x = x0 + TINY*flag (mod_evolve.f90:140-141), x0 from the RHS kernel.
// MODE RES_UPDATE: x = x + sigma_prev * S^-1 y (y from the inner solve, type TY).
// Writes x (into the x-write buffer), g = -S^-1 (S - H x) / sigma into the inner residual r (type
// TR) and the inner solution is restarted from 0.
template <int MODE, typename TY, typename TR>
__global__ void __launch_bounds__(kBlock) k_residual(DevArrays A) {
  const int64_t tile = blockIdx.x;
  const int inst = A.tile_inst[tile];
  const InstDesc& d = A.inst[inst];
  InstScal& s = A.scal[inst];
  if (!s.outer_active || s.inner_active) return;
  if (MODE == RES_INIT && s.refine != 0) return;
  if (MODE == RES_UPDATE && s.refine == 0) return;
  const double* XR = A.tbuf[s.role[2]] + d.off;
  double* XW = A.tbuf[s.role[3]] + d.off;
  const double* sinv = A.sinv + d.off;
  const TY* Y = Vec<TY>::y(A) + d.off;
  TR* R = Vec<TR>::r(A) + d.off;
  const double tadd = s.x0flag ? kTiny : 0.0;
  const double sig_prev = s.sigma_prev;
  const double sig = s.sigma;
  const double isig = 1.0 / sig;
  const bool use_y = (s.iter > 0);   // the last inner solve produced a correction
  auto xv = [&](int64_t n) -> double {
    if (MODE == RES_INIT) return XR[n] + tadd;
    return use_y ? fma(sig_prev * sinv[n], (double)Y[n], XR[n]) : XR[n];
  };
  double acc[3] = {0, 0, 0};  // ||r||^2, ||g||^2, NaN count of x
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t g = tile * kTile + k * kBlock + threadIdx.x;
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const Coord c = coord_of(d, (int32_t)l);
    const double xc = xv(l);
    const double hx = apply_H(A, d, g, l, c, xv);
    const double rv = A.b[g] - hx;
    XW[l] = xc;
    const double gv = -sinv[l] * rv * isig;
    R[l] = (TR)gv;
    acc[0] = fma(rv, rv, acc[0]);
    acc[1] = fma(gv, gv, acc[1]);
    acc[2] += isnan(xc) ? 1.0 : 0.0;
  }
  double tot[3];
  if (!tile_reduce<3>(A, inst, tile, acc, tot)) return;
  if (threadIdx.x != 0) return;
  // epilogue: the instance's residual is complete
  const DevOpts& o = A.opts;
  int t = s.role[2]; s.role[2] = s.role[3]; s.role[3] = t;
  s.rr_true = tot[0];
  s.relres = s.bb > 0.0 ? sqrt(tot[0] / s.bb) : (tot[0] > 0.0 ? INFINITY : 0.0);
  s.refine += 1;
  s.tot_refine += 1;
  if (tot[2] > 0.0) {
    s.status |= 1 << (HF_ENAN_X - HF_ENAN_B);
    s.failed_step = s.itime;
    s.outer_active = 0;
    return;
  }
  bool done;
  bool converged;
  if (o.criterion == HF_STOP_RECURSIVE) {
    done = (s.refine >= 2);       // the reference solves once; this sweep only forms x
    converged = true;
  } else {
    converged = (s.relres <= o.tol);
    done = converged || (s.refine > o.max_refine) || (tot[0] == 0.0);
  }
  if (done) {
    s.outer_active = 0;
    if (!converged) s.unconverged += 1;
    s.last_relres = s.relres;
    s.last_err = (o.criterion == HF_STOP_RECURSIVE) ? s.err : s.relres;
    s.last_iter = s.step_iters;
    return;
  }
  s.inner_active = 1;
  s.iter = 0;
  s.gg0 = tot[1];
  s.rho = tot[1];
  s.beta = 0.0;
  s.sigma_prev = sig;
  if (o.precision == HF_PREC_MIXED) {
    s.eta = fmax(o.inner_tol, 0.1 * o.tol / fmax(s.relres, 1e-300));
    double rms = sqrt(tot[0] / (double)d.n) * d.mean_sinv;
    s.sigma = (rms > 0.0 && isfinite(rms)) ? exp2(rint(log2(rms))) : 1.0;
  } else {
    s.eta = fmax(0.1 * o.tol / fmax(s.relres, 1e-300), 1e-15);
    s.sigma = 1.0;
  }
  if (!(tot[1] > 0.0)) s.inner_active = 0;  // exact already: go straight to the update sweep
}

// ---- inner CG on Ah (type T) -------------------------------------------------------------------
// k_cg_p:    p = r + beta p  (beta = 0 on the first iteration)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_p(DevArrays A) {
  const int64_t tile = blockIdx.x;
  const int inst = A.tile_inst[tile];
  const InstDesc& d = A.inst[inst];
  const InstScal& s = A.scal[inst];
  if (!s.inner_active) return;
  const T beta = (T)s.beta;
  const bool first = (s.iter == 0);
  const T* R = Vec<T>::r(A) + d.off;
  T* P = Vec<T>::p(A) + d.off;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t g = tile * kTile + k * kBlock + threadIdx.x;
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    P[l] = first ? R[l] : fma(beta, P[l], R[l]);
  }
}

// k_cg_spmv: q = Ah p, p.q
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_spmv(DevArrays A) {
  const int64_t tile = blockIdx.x;
  const int inst = A.tile_inst[tile];
  const InstDesc& d = A.inst[inst];
  InstScal& s = A.scal[inst];
  if (!s.inner_active) return;
  const T* P = Vec<T>::p(A) + d.off;
  T* Q = Vec<T>::q(A) + d.off;
  const T* ax = Vec<T>::ax(A);
  const T* ay = Vec<T>::ay(A);
  const T* az = Vec<T>::az(A);
  auto pv = [&](int64_t n) -> T { return P[n]; };
  double acc[1] = {0.0};
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t g = tile * kTile + k * kBlock + threadIdx.x;
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const Coord c = coord_of(d, (int32_t)l);
    const T qv = apply_Ah<T>(ax, ay, az, d, g, l, c, pv);
    Q[l] = qv;
    acc[0] += (double)(P[l] * qv);
  }
  double tot[1];
  if (!tile_reduce<1>(A, inst, tile, acc, tot)) return;
  if (threadIdx.x != 0) return;
  s.pq = tot[0];
  if (tot[0] > 0.0 && isfinite(tot[0])) {
    s.alpha = s.rho / tot[0];
  } else {            // breakdown (p = 0 or non-finite): stop this inner solve
    s.alpha = 0.0;
    s.inner_active = 0;
  }
}

// k_cg_upd: y += alpha p, r -= alpha q, r.r (and the unscaled ||r||^2 for the reference rule)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_upd(DevArrays A) {
  const int64_t tile = blockIdx.x;
  const int inst = A.tile_inst[tile];
  const InstDesc& d = A.inst[inst];
  InstScal& s = A.scal[inst];
  if (!s.inner_active) return;
  const DevOpts& o = A.opts;
  const bool weighted = (o.criterion == HF_STOP_RECURSIVE);
  const T alpha = (T)s.alpha;
  const bool first = (s.iter == 0);
  T* Y = Vec<T>::y(A) + d.off;
  T* R = Vec<T>::r(A) + d.off;
  const T* P = Vec<T>::p(A) + d.off;
  const T* Q = Vec<T>::q(A) + d.off;
  double acc[2] = {0.0, 0.0};
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t g = tile * kTile + k * kBlock + threadIdx.x;
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const T pv = P[l];
    Y[l] = first ? alpha * pv : fma(alpha, pv, Y[l]);
    const T rv = fma(-alpha, Q[l], R[l]);
    R[l] = rv;
    acc[0] += (double)(rv * rv);
    if (weighted) acc[1] += -A.diag[g] * (double)rv * (double)rv;
  }
  double tot[2];
  if (!tile_reduce<2>(A, inst, tile, acc, tot)) return;
  if (threadIdx.x != 0) return;
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

// ---- launchers ---------------------------------------------------------------------------------
cudaError_t launch_step_begin(Ctx& c, int64_t itime, int) {
  k_step_begin<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A, itime);
  return cudaGetLastError();
}

cudaError_t launch_step_end(Ctx& c) {
  k_step_end<<<(unsigned)((c.ninst + 127) / 128), 128, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}

cudaError_t launch_residual(Ctx& c, int mode) {
  const unsigned nb = (unsigned)c.ntiles;
  const bool mixed = c.opts.precision == HF_PREC_MIXED;
  if (mode == RES_INIT) {
    if (mixed) k_residual<RES_INIT, float, float><<<nb, kBlock, 0, c.stream>>>(c.A);
    else k_residual<RES_INIT, double, double><<<nb, kBlock, 0, c.stream>>>(c.A);
  } else {
    if (mixed) k_residual<RES_UPDATE, float, float><<<nb, kBlock, 0, c.stream>>>(c.A);
    else k_residual<RES_UPDATE, double, double><<<nb, kBlock, 0, c.stream>>>(c.A);
  }
  return cudaGetLastError();
}

cudaError_t launch_inner_iteration(Ctx& c, int fp32) {
  const unsigned nb = (unsigned)c.ntiles;
  if (fp32) {
    k_cg_p<float><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_spmv<float><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_upd<float><<<nb, kBlock, 0, c.stream>>>(c.A);
  } else {
    k_cg_p<double><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_spmv<double><<<nb, kBlock, 0, c.stream>>>(c.A);
    k_cg_upd<double><<<nb, kBlock, 0, c.stream>>>(c.A);
  }
  return cudaGetLastError();
}

// One kernel of the step, for timing (hf_time_kernel).
cudaError_t launch_single(Ctx& c, int which) {
  const unsigned nb = (unsigned)c.ntiles;
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  switch (which) {
    case HF_KERNEL_RHS: return launch_rhs(c);
    case HF_KERNEL_RESIDUAL: return launch_residual(c, RES_UPDATE);
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
