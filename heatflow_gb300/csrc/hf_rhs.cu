// Per-step right-hand side: heater (mod_heating.f90:27-169), Cattaneo term
// (mod_cattaneo.f90:23-42), S and the initial guess (mod_evolve.f90:112-141), in one pass.
//
// GB300 executes FP64 at ~1 TFLOP/s (measured), so an FP64 pass over the grid is bound by FP64
// instructions, not by HBM.  This kernel therefore spends FP64 instructions only on the values
// the reference computes: S, x0 = T + (T - T_pp) and x0 - T, plus ||S||^2.  The x0 test and
// the NaN screening use integer operations on the IEEE bits: any NaN among Q, Qdens, S_cat
// propagates into S and so into ||S||^2, and only then does the host run the diagnosis variant
// (DIAG) that finds the first failing vector in the reference's check order.
//
// Compiled with -fmad=false so that S is rounded exactly as the reference writes it.
//
// Under the true-residual criterion (HF_STOP_TRUE) the step's pass forms the same S with fewer
// roundings: S = T^n * c1 + tau' rho c * T^(n-1) - Qdens - B, with c1 = -rho c / dt - 2 tau' rho c
// per cell (-rho c / dt in Fourier mode) held in DevArrays::scoef, and x0 = 2 T^n - T^(n-1) in one
// FMA -- 3 FP64 instructions per interior cell instead of 7, which takes the pass from the FP64
// pipe's bound to HBM's.  S then differs from the reference's rounding by a few units in the last
// place (1e-16 relative, against a solver tolerance of 1e-10), x0 is only the starting point, and
// the step is accepted on the true residual of its final x; the x0 - T < TINY flag is not formed
// (the TINY is not applied under this criterion).  Under the reference's own stopping rule, and in
// the parity probe (PARTS) and the NaN diagnosis (DIAG), S and x0 keep the reference's arithmetic.
#include <algorithm>

#include "hf_ctx.cuh"

#define HF_FILE_ID 2   // index-check sites of the checked build: 100000 * file + line

namespace hf {

// Heat of one cell for heater case cs at step itime (mod_heating.f90:59-117).
__device__ __forceinline__ double heat_case(int cs, double P, double tau, int64_t itime,
                                            const InstDesc& d) {
  const double time = d.time_step * (double)itime;
  switch (cs) {
    case 1: return P;
    case 2: return (time <= d.time_pulse) ? P : 0.0;
    case 3: {
      double x = time * 2.0 * kPi * d.freq;
      double x2 = d.time_step * 2.0 * kPi * d.freq;
      return P * 0.5 * ((x2) - sin(x + x2) * cos(x + x2) + sin(x) * cos(x)) / x2;
    }
    case 4: {
      double s = sin(time * 2.0 * kPi * d.freq);
      return P * (s * s);
    }
    case 5: {
      double s = sin(time * 2.0 * kPi * d.freq);
      return P * (s * s) + P * 2.0 * kPi * d.freq * tau * sin(2.0 * time * 2.0 * kPi * d.freq);
    }
    case 6: return (itime == 1) ? P : 0.0;
    default: return 0.0;
  }
}

// x0 - T < TINY (mod_evolve.f90:140-141) for x0 = RN(T + d), d = RN(T - T_old), decided from d with
// integer compares where the rounding of x0 cannot change the answer: d <= 0 gives x0 <= T; for
// 0 < T < 2048 the rounding of x0 and of x0 - T is below 0.23 TINY, so d <= TINY/2 and d >= 2 TINY
// decide it.  The FP64 subtraction remains for the band between and other temperatures; the
// result is that of dbl_lt_pos(x0 - T, TINY) in every case (a NaN d keeps its sign's answer).
__device__ __forceinline__ bool x0_below_tiny(double tp, double d, double x0) {
  const long long bd = (long long)dbits(d);
  if (bd <= 0) return true;
  const long long bt = (long long)dbits(tp);
  if (bt > 0 && bt < (long long)dbits(2048.0)) {
    if (bd <= (long long)dbits(0.5 * kTiny)) return true;
    if (bd >= (long long)dbits(2.0 * kTiny)) return false;
  }
  return dbl_lt_pos(x0 - tp, kTiny);
}

// The per-cell work of the step RHS (shared by the scalar and the vector forms): heater, S_cat,
// S and the initial guess of cell l; returns S and sets x0 and the x0 - T < TINY flag.
struct RhsCtx {
  bool heater, has_power, has_em, case5, cat, steady;
  bool fast;      // HF_STOP_TRUE, not steady: S from scoef (passed as rhoc), x0 in one FMA
  int qmode;
  double inv_dt, vol, hvol, power_in, tb4, dt2;
  int64_t itime;
};
// Heat density of cell l (the heater branch, out of line so the common heater-free tasks keep
// a small register footprint).
__device__ __noinline__ double rhs_qdens(const DevArrays& A, const InstDesc& d, const RhsCtx& r,
                                         int64_t off, int l, double tp) {
  double q = 0.0, qd = 0.0;
  {
    l = HF_IX(A, l, d.n);
    const int cs = A.icase[off + l];
    if (cs > 0 && cs < 7) {
      const double P = r.has_power ? A.power[off + l] : r.power_in;
      const double tau = r.case5 ? A.tau_s[off + l] * r.dt2 : 0.0;
      q = heat_case(cs, P, tau, r.itime, d);
    }
    if (r.has_em) q = q - A.emc[off + l] * (pow(tp, 4.0) - r.tb4);
    if (!dbl_is_zero(q)) {
      if (r.qmode == HF_QDENS_CELL_VOLUME) qd = q / r.vol;
      else if (r.hvol > 0.0) qd = q / r.hvol;
    }
  }
  return qd;
}

template <bool HEAT>
__device__ __forceinline__ double rhs_cell(const DevArrays& A, const InstDesc& d, const RhsCtx& r,
                                           int64_t off, int l, double tp, double tpp, double rhoc,
                                           double ccat, double B, double& x0, int& flag) {
  const double qd = HEAT ? rhs_qdens(A, d, r, off, l, tp) : 0.0;
  double S;
  if (r.fast) {                                     // rhoc holds scoef here
    S = r.cat ? fma(tp, rhoc, ccat * tpp) : tp * rhoc;
    if (!dbl_is_zero(qd)) S = S - qd;
    if (!dbl_is_zero(B)) S = S - B;
    x0 = fma(2.0, tp, -tpp);
    return S;
  }
  if (!r.steady) {
    S = -r.inv_dt * tp * rhoc;
    if (!dbl_is_zero(qd)) S = S - qd;
    if (!dbl_is_zero(B)) S = S - B;
    if (r.cat) S = S + fma(-2.0, tp, tpp) * ccat;   // (tpp - 2 tp) * ccat: 2 tp is exact
  } else {
    S = -qd;
    if (!dbl_is_zero(B)) S = S - B;
  }
  const double dt = tp - tpp;
  x0 = tp + dt;
  flag |= x0_below_tiny(tp, dt, x0) ? 1 : 0;
  return S;
}

// The common task of a step under the true-residual criterion, on rows of 4k cells: no heated
// cell, S = T^n scoef + ccat T^(n-1) - B and x0 = 2 T^n - T^(n-1) (3 FP64 instructions per cell),
// the arithmetic and summation order of rhs4_task's fast form.  Kept apart from the general forms
// (out of line) so that its operands stay in registers: with them in one body the kernel's 64
// registers spilled, and the pass ran on local-memory traffic as large as its HBM traffic (ncu).
// B is read only on the outer faces: boundary() (k_assemble, k_tempdep) gives it to no other
// cell, where it is +0.0.
__device__ __forceinline__ void rhs4_fast_task(const DevArrays& A, int64_t task, const InstDesc& d,
                                               const InstScal& s) {
  const int4 tk = A.tasks[task];
  const int tid = threadIdx.x, grp = tid >> 6, w = tid & 63;
  const int x = tk.y + 4 * (w & 7), y = tk.z + (w >> 3);
  const int z1 = min(tk.w + d.zc, d.nz);
  const int per = (z1 - tk.w + 3) >> 2;
  const int za = min(tk.w + grp * per, z1), zb = min(za + per, z1);
  const bool act = x < d.nx && y < d.ny;
  const bool face_col = x == 0 || x + 4 >= d.nx || y == 0 || y == d.ny - 1;
  const bool cat = d.icattaneo == 1;
  const int64_t off = d.off;
  const int nxy = d.nx * d.ny, lxy = y * d.nx + x;
  const double* Tp = A.tbuf[s.role[0]] + off;
  const double* Tpp = A.tbuf[s.role[1]] + off;
  double* X = A.tbuf[s.role[2]] + off;
  const double* __restrict__ sc = A.scoef + off;
  const double* __restrict__ ccat = A.ccat + off;
  const double* __restrict__ bvec = A.bvec + off;
  double* bout = A.b + off;
  SqSum sq;
  if (act) {
    for (int z = za; z < zb; ++z) {
      const int l = HF_IX4(A, lxy + z * nxy, d.n);
      const double2* tp2 = reinterpret_cast<const double2*>(Tp + l);
      const double2* tq2 = reinterpret_cast<const double2*>(Tpp + l);
      const double2* sc2 = reinterpret_cast<const double2*>(sc + l);
      const double2* cc2 = reinterpret_cast<const double2*>(ccat + l);
      const double2* bv2 = reinterpret_cast<const double2*>(bvec + l);
      const double2 t0 = tp2[0], t1 = tp2[1], u0 = tq2[0], u1 = tq2[1], h0 = sc2[0], h1 = sc2[1];
      double2 c0 = make_double2(0.0, 0.0), c1 = c0, b0 = c0, b1 = c0;
      if (cat) { c0 = cc2[0]; c1 = cc2[1]; }
      if (face_col || z == 0 || z == d.nz - 1) { b0 = bv2[0]; b1 = bv2[1]; }
      const double tp[4] = {t0.x, t0.y, t1.x, t1.y}, tpp[4] = {u0.x, u0.y, u1.x, u1.y};
      const double rh[4] = {h0.x, h0.y, h1.x, h1.y}, cc[4] = {c0.x, c0.y, c1.x, c1.y};
      const double bv[4] = {b0.x, b0.y, b1.x, b1.y};
      double S[4], x0[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        S[i] = cat ? fma(tp[i], rh[i], cc[i] * tpp[i]) : tp[i] * rh[i];
        if (!dbl_is_zero(bv[i])) S[i] = S[i] - bv[i];
        x0[i] = fma(2.0, tp[i], -tpp[i]);
        sq.add(S[i]);
      }
      reinterpret_cast<double2*>(bout + l)[0] = make_double2(S[0], S[1]);
      reinterpret_cast<double2*>(bout + l)[1] = make_double2(S[2], S[3]);
      reinterpret_cast<double2*>(X + l)[0] = make_double2(x0[0], x0[1]);
      reinterpret_cast<double2*>(X + l)[1] = make_double2(x0[2], x0[3]);
    }
  }
  const double bb = sq.value();
  if (threadIdx.x == 0) A.partials[task * kNR + 1] = 0.0;   // no x0 - T < TINY test here
  const double v[1] = {bb};
  tile_store<1>(A, task, v);
}

// Vector form for rows of 4k cells: each thread owns 4 consecutive x cells of a quarter of the
// task's planes (the layout of the solver's vector passes), so every thread has 4 independent
// cells of FP64 work in flight: the pass is bound by the FP64 pipe, and one cell per thread left
// it partly idle.  ||S||^2 is summed per thread plane by plane, cells in x order.
__device__ __noinline__ void rhs4_task(const DevArrays& A, int64_t task, const InstDesc& d,
                                       const InstScal& s, const RhsCtx& r) {
  const int4 tk = A.tasks[task];
  const int tid = threadIdx.x, grp = tid >> 6, w = tid & 63;
  const int x = tk.y + 4 * (w & 7), y = tk.z + (w >> 3);
  const int z1 = min(tk.w + d.zc, d.nz);
  const int per = (z1 - tk.w + 3) >> 2;
  const int za = min(tk.w + grp * per, z1), zb = min(za + per, z1);
  const bool act = x < d.nx && y < d.ny;
  // boundary() gives B only to cells on the outer faces (k_assemble, k_tempdep): elsewhere it is
  // +0.0, so a quad off the x/y faces reads B only in the first and last plane
  const bool face_col = x == 0 || x + 4 >= d.nx || y == 0 || y == d.ny - 1;
  const int64_t off = d.off;
  const int nxy = d.nx * d.ny, lxy = y * d.nx + x;
  const double* Tp = A.tbuf[s.role[0]] + off;
  const double* Tpp = A.tbuf[s.role[1]] + off;
  double* X = A.tbuf[s.role[2]] + off;
  const double* __restrict__ rhoc = (r.fast ? A.scoef : A.rhoc) + off;
  const double* __restrict__ ccat = A.ccat + off;
  const double* __restrict__ bvec = A.bvec + off;
  double* bout = A.b + off;
  double bb = 0.0;
  SqSum sq;
  int flag = 0;
  if (act) {
    for (int z = za; z < zb; ++z) {
      const int l = HF_IX4(A, lxy + z * nxy, d.n);
      const double2* tp2 = reinterpret_cast<const double2*>(Tp + l);
      const double2* tq2 = reinterpret_cast<const double2*>(Tpp + l);
      const double2* rc2 = reinterpret_cast<const double2*>(rhoc + l);
      const double2* cc2 = reinterpret_cast<const double2*>(ccat + l);
      const double2* bv2 = reinterpret_cast<const double2*>(bvec + l);
      const double2 t0 = tp2[0], t1 = tp2[1], u0 = tq2[0], u1 = tq2[1];
      const double2 h0 = rc2[0], h1 = rc2[1], c0 = cc2[0], c1 = cc2[1];
      double2 b0 = make_double2(0.0, 0.0), b1 = b0;
      if (face_col || z == 0 || z == d.nz - 1) { b0 = bv2[0]; b1 = bv2[1]; }
      const double tp[4] = {t0.x, t0.y, t1.x, t1.y}, tpp[4] = {u0.x, u0.y, u1.x, u1.y};
      const double rh[4] = {h0.x, h0.y, h1.x, h1.y}, cc[4] = {c0.x, c0.y, c1.x, c1.y};
      const double bv[4] = {b0.x, b0.y, b1.x, b1.y};
      double S[4], x0[4];
      if (r.heater) {               // unrolled too: a dynamic index would put the arrays in
#pragma unroll                      // local memory for both branches
        for (int i = 0; i < 4; ++i)
          S[i] = rhs_cell<true>(A, d, r, off, l + i, tp[i], tpp[i], rh[i], cc[i], bv[i], x0[i], flag);
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          S[i] = rhs_cell<false>(A, d, r, off, l + i, tp[i], tpp[i], rh[i], cc[i], bv[i], x0[i], flag);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) sq.add(S[i]);
      reinterpret_cast<double2*>(bout + l)[0] = make_double2(S[0], S[1]);
      reinterpret_cast<double2*>(bout + l)[1] = make_double2(S[2], S[3]);
      reinterpret_cast<double2*>(X + l)[0] = make_double2(x0[0], x0[1]);
      reinterpret_cast<double2*>(X + l)[1] = make_double2(x0[2], x0[3]);
    }
  }
  bb = sq.value();
  const int any_flag = __syncthreads_or(flag);
  if (threadIdx.x == 0) A.partials[task * kNR + 1] = any_flag ? 1.0 : 0.0;
  const double v[1] = {bb};
  tile_store<1>(A, task, v);
}

// One block per task.  PARTS: also write B, Q, Qdens and S_cat (parity probe hf_get_rhs).
// DIAG: count NaNs per vector (failure path only).
template <bool PARTS, bool DIAG>
__global__ void __launch_bounds__(kBlock, 4) k_rhs(DevArrays A, double* oB, double* oQ, double* oQd,
                                                double* oSc, int64_t task_base) {
  const int64_t task = task_base + blockIdx.x;
  if (!PARTS && !DIAG && task == 0 && threadIdx.x == 0) A.stamps[kStampRhs] = gtimer();
  if (!PARTS && !DIAG) {          // the step's pass: vector form where the rows allow it
    const int inst = A.tasks[task].x;
    const InstDesc& d = A.inst[inst];
    const InstScal& s = A.scal[inst];
    if ((d.nx & 3) == 0) {
      if (!s.outer_active) return;
      const bool heater = d.heater && (d.has_em || A.task_heat[task]);
      if (!heater && A.opts.criterion == HF_STOP_TRUE && d.isteady == 0) {
        rhs4_fast_task(A, task, d, s);
        return;
      }
      RhsCtx r;
      r.heater = heater;
      r.has_power = d.has_power; r.has_em = d.has_em; r.case5 = d.has_case5;
      r.cat = d.icattaneo == 1; r.steady = d.isteady != 0;
      r.qmode = d.qdens_mode;
      r.inv_dt = d.inv_dt; r.vol = d.volume; r.hvol = d.heated_volume; r.power_in = d.power_in;
      r.tb4 = d.has_em ? pow(d.t_bath, 4.0) : 0.0;
      r.dt2 = d.has_case5 ? pow(d.time_step, 2.0) : 0.0;
      r.itime = s.itime;
      r.fast = A.opts.criterion == HF_STOP_TRUE && !r.steady;
      rhs4_task(A, task, d, s, r);
      return;
    }
  }
  const TCell c = task_cell(A, task);
  const InstDesc& d = A.inst[c.inst];
  InstScal& s = A.scal[c.inst];
  if (!DIAG && !s.outer_active) return;
  if (DIAG && !(s.status & kStatusRhsNan)) return;
  const int64_t itime = DIAG ? s.failed_step : s.itime;
  const int64_t off = c.off;
  // heater() runs for every cell when any exists (mod_evolve.f90:79); with emissivity every cell
  // has a radiative term, otherwise only tasks holding a heated cell have nonzero Q
  const bool heater = d.heater && (d.has_em || A.task_heat[task]);
  const bool has_power = d.has_power, has_em = d.has_em, case5 = d.has_case5;
  const bool cat = d.icattaneo == 1, steady = d.isteady != 0;
  const int qmode = d.qdens_mode;
  const double inv_dt = d.inv_dt, vol = d.volume, hvol = d.heated_volume, power_in = d.power_in;
  // the step's pass under the true-residual criterion: S from scoef, x0 in one FMA (see above)
  const bool fast = !PARTS && !DIAG && A.opts.criterion == HF_STOP_TRUE && !steady;
  const double* __restrict__ Tp = A.tbuf[s.role[0]] + off;
  const double* __restrict__ Tpp = A.tbuf[s.role[1]] + off;
  double* __restrict__ X = A.tbuf[s.role[2]] + off;
  const double* __restrict__ rhoc = (fast ? A.scoef : A.rhoc) + off;
  const double* __restrict__ ccat = A.ccat + off;
  const double* __restrict__ bvec = A.bvec + off;
  double* __restrict__ bout = A.b + off;
  const double tb4 = has_em ? pow(d.t_bath, 4.0) : 0.0;
  const double dt2 = case5 ? pow(d.time_step, 2.0) : 0.0;
  double bb = 0.0;
  SqSum sq;
  int flag = 0;
  int nan_q = 0, nan_qd = 0, nan_sc = 0, nan_s = 0;
  for (int z = c.z0; z < c.z1; ++z) {
#pragma unroll
    for (int j = 0; j < kXC; ++j) {
      if (!c.act(j)) continue;
      const int l = HF_IX(A, c.base(j) + z * c.nxy, c.n());
      const double tp = Tp[l], tpp = Tpp[l];
      double q = 0.0, qd = 0.0;
      if (heater) {
        const int cs = A.icase[off + l];
        if (cs > 0 && cs < 7) {
          const double P = has_power ? A.power[off + l] : power_in;
          const double tau = case5 ? A.tau_s[off + l] * dt2 : 0.0;
          q = heat_case(cs, P, tau, itime, d);
        }
        if (has_em) q = q - A.emc[off + l] * (pow(tp, 4.0) - tb4);
        if (!dbl_is_zero(q)) {
          if (qmode == HF_QDENS_CELL_VOLUME) qd = q / vol;
          else if (hvol > 0.0) qd = q / hvol;
        }
        if (DIAG) { nan_q += dbl_is_nan(q); nan_qd += dbl_is_nan(qd); }
      }
      double sc = 0.0;
      if (cat && !fast) {
        sc = fma(-2.0, tp, tpp) * ccat[l];   // = (tpp - 2 tp) * ccat: 2 tp is exact
        if (DIAG) nan_sc += dbl_is_nan(sc);
      }
      const double B = bvec[l];
      double S, x0;
      if (fast) {
        S = cat ? fma(tp, rhoc[l], ccat[l] * tpp) : tp * rhoc[l];
        if (!dbl_is_zero(qd)) S = S - qd;
        if (!dbl_is_zero(B)) S = S - B;
        x0 = fma(2.0, tp, -tpp);
      } else {
        if (!steady) {
          S = -inv_dt * tp * rhoc[l];
          if (!dbl_is_zero(qd)) S = S - qd;
          if (!dbl_is_zero(B)) S = S - B;
          if (cat) S = S + sc;
        } else {
          S = -qd;
          if (!dbl_is_zero(B)) S = S - B;
        }
        const double dt = tp - tpp;
        x0 = tp + dt;
        flag |= x0_below_tiny(tp, dt, x0) ? 1 : 0;
      }
      if (DIAG) nan_s += dbl_is_nan(S);
      bout[l] = S;
      X[l] = x0;
      sq.add(S);
      if (PARTS) {
        oB[off + l] = B;
        oQ[off + l] = q;
        oQd[off + l] = qd;
        oSc[off + l] = sc;
      }
    }
  }
  bb = sq.value();
  const int any_flag = __syncthreads_or(flag);
  if (DIAG) {
    const int c1 = __syncthreads_count(nan_q), c2 = __syncthreads_count(nan_qd);
    const int c3 = __syncthreads_count(nan_sc), c4 = __syncthreads_count(nan_s);
    if (threadIdx.x == 0) {
      A.partials[task * kNR + 1] = (double)c1;
      A.partials[task * kNR + 2] = (double)c2;
      A.partials[task * kNR + 3] = (double)c3;
      A.partials[task * kNR + 4] = (double)c4;
    }
  } else if (threadIdx.x == 0) {
    A.partials[task * kNR + 1] = any_flag ? 1.0 : 0.0;
  }
  const double v[1] = {bb};
  tile_store<1>(A, task, v);
}

cudaError_t launch_rhs(Ctx& c) { return launch_rhs_range(c, 0, c.ntasks); }

cudaError_t launch_rhs_range(Ctx& c, int64_t t0, int64_t t1) {
  if (t1 <= t0) return cudaSuccess;
  k_rhs<false, false><<<(unsigned)(t1 - t0), kBlock, 0, c.stream>>>(c.A, nullptr, nullptr, nullptr,
                                                                    nullptr, t0);
  return cudaGetLastError();
}

cudaError_t launch_rhs_parts(Ctx& c, double* B, double* Q, double* Qd, double* Sc) {
  k_rhs<true, false><<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, B, Q, Qd, Sc, 0);
  return cudaGetLastError();
}

cudaError_t launch_rhs_diagnose(Ctx& c) {
  k_rhs<false, true><<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, nullptr, nullptr, nullptr,
                                                                  nullptr, 0);
  return cudaGetLastError();
}

}  // namespace hf

// ---- adjoint (no counterpart in the reference: HeatFlow computes no gradients) -----------------
// Forward step k:  H x_k = S_k,  S_k = a x_(k-1) + c x_(k-2) - Qdens_k - B   (per cell, diagonal a, c)
// with a = -rho c / dt - 2 tau' rho c, c = tau' rho c (Cattaneo; c = 0 in Fourier mode).
// Discrete adjoint, k = K..1:  H lambda_k = dJ/dx_k + a lambda_(k+1) + c lambda_(k+2)   (H = H^T),
// dJ/dtheta = sum_k lambda_k^T (dS_k/dtheta - dH/dtheta x_k).

namespace hf {

__global__ void k_adj_rhs(DevArrays A, const double* g, const double* l1, const double* l2,
                          double* out) {
  const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= A.ncells) return;
  const InstDesc& d = A.inst[A.tile_inst[gi / kTile]];
  const int64_t l = gi - d.off;
  if (l >= d.n) return;
  double v = g[l];
  if (d.isteady == 0) {
    const double cc = d.icattaneo == 1 ? A.ccat[gi] : 0.0;
    const double a = -d.inv_dt * A.rhoc[gi] - 2.0 * cc;
    v = fma(a, l1[l], v);
    if (d.icattaneo == 1) v = fma(cc, l2[l], v);
  }
  out[l] = v;
}

// d c / d log(kappa_i) of a harmonic-mean face between kappa_i and kappa_j of length L
// (c = 2 ki kj / ((ki + kj) L^2), times BR when ki != kj; mod_hmatrix.f90:289-314).
__device__ __forceinline__ double dface(double ki, double kj, double L, double br) {
  const double s = ki + kj;
  double v = 2.0 * ki * kj * kj / (s * s * L * L);
  return ki != kj ? v * br : v;
}

// grad_logk[i] += dJ/dlog(kappa_i) of step k; grad_src[i] += dJ/dP_i of step k (P: the cell's
// heater power), for lambda_k, x_k.
__global__ void k_adj_grad(DevArrays A, const InstBC* bcs, const double* kappa, const double* lam,
                           const double* x, int64_t itime, double* grad_logk, double* grad_src) {
  const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= A.ncells) return;
  const int inst = A.tile_inst[gi / kTile];
  const InstDesc& d = A.inst[inst];
  const InstBC& bc = bcs[inst];
  const int64_t l = gi - d.off;
  if (l >= d.n) return;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  const int64_t c3[3] = {l % nx, (l / nx) % ny, l / nxy};
  const int64_t n3[3] = {nx, ny, nz}, st[3] = {1, nx, nxy};
  const int per[3] = {d.px, d.py, d.pz};
  const double* cf[3] = {A.cx + d.off, A.cy + d.off, A.cz + d.off};
  const double* K = kappa + d.off;
  const double ki = K[l], li = lam[l], xi = x[l];
  double g = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double L = d.len[a];
    if (n3[a] == 1) {
      // a lone cell along this axis has two outside faces (none when periodic)
      if (!per[a]) {
        for (int f = 2 * a; f <= 2 * a + 1; ++f) {
          const double kb = bc.kb[f], s = kb + ki;
          g += li * (xi - bc.tb[f]) * (2.0 * kb * kb * ki / (s * s * L * L)) * (ki != kb ? bc.br : 1.0);
        }
      }
      continue;
    }
    // + face (stored at this cell)
    const bool has_p = c3[a] + 1 < n3[a] || per[a];
    if (has_p) {
      const int64_t j = c3[a] + 1 < n3[a] ? l + st[a] : l - (n3[a] - 1) * st[a];
      if (cf[a][l] != 0.0) g += -(li - lam[j]) * (x[j] - xi) * dface(ki, K[j], L, bc.br);
    } else {
      const int f = 2 * a + 1;
      const double kb = bc.kb[f], s = kb + ki;
      g += li * (xi - bc.tb[f]) * (2.0 * kb * kb * ki / (s * s * L * L)) * (ki != kb ? bc.br : 1.0);
    }
    // - face (stored at the - neighbour)
    const bool has_m = c3[a] > 0 || per[a];
    if (has_m) {
      const int64_t j = c3[a] > 0 ? l - st[a] : l + (n3[a] - 1) * st[a];
      if (cf[a][j] != 0.0) g += -(li - lam[j]) * (x[j] - xi) * dface(ki, K[j], L, bc.br);
    } else {
      const int f = 2 * a;
      const double kb = bc.kb[f], s = kb + ki;
      g += li * (xi - bc.tb[f]) * (2.0 * kb * kb * ki / (s * s * L * L)) * (ki != kb ? bc.br : 1.0);
    }
  }
  grad_logk[l] += g;
  if (grad_src && d.heater) {
    const int cs = A.icase[gi];
    if (cs > 0 && cs < 7) {
      const double tau = d.has_case5 ? A.tau_s[gi] * pow(d.time_step, 2.0) : 0.0;
      const double f = heat_case(cs, 1.0, tau, itime, d);
      const double vn = d.qdens_mode == HF_QDENS_CELL_VOLUME ? d.volume : d.heated_volume;
      grad_src[l] += -li * f / vn;
    }
  }
}

// Per task: does some cell hold a heater (any heater case != 0)?  The RHS skips the heater loads of
// the other tasks.
__global__ void k_task_heat(DevArrays A, int8_t* flag) {
  const int64_t task = blockIdx.x;
  const TCell c = task_cell(A, task);
  int any = 0;
  if (A.icase && c.act(0)) {
    for (int z = c.z0; z < c.z1; ++z) any |= A.icase[c.off + c.base(0) + (int64_t)z * c.nxy] != 0;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) flag[task] = (int8_t)(any ? 1 : 0);
}

cudaError_t launch_task_heat(Ctx& c) {
  k_task_heat<<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, const_cast<int8_t*>(c.A.task_heat));
  return cudaGetLastError();
}

// Pack the box lo..hi of one temperature field of instance `inst` (its current role, read on the
// device, so this works inside a stream of captured steps) into dst, x fastest.
__global__ void k_subbox_gather(DevArrays A, int inst, int which, int x0, int y0, int z0, int bx,
                                int by, int bz, double* dst) {
  const InstDesc& d = A.inst[inst];
  const double* T = A.tbuf[A.scal[inst].role[which]] + d.off;
  const int64_t n = (int64_t)bx * by * bz;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % bx), iy = (int)((i / bx) % by), iz = (int)(i / ((int64_t)bx * by));
    dst[i] = T[(int64_t)(z0 + iz) * d.nx * d.ny + (int64_t)(y0 + iy) * d.nx + (x0 + ix)];
  }
}

cudaError_t launch_subbox_gather(Ctx& c, int64_t inst, const int64_t* lo, const int64_t* hi,
                                 int which, double* dst) {
  const int bx = (int)(hi[0] - lo[0] + 1), by = (int)(hi[1] - lo[1] + 1), bz = (int)(hi[2] - lo[2] + 1);
  const int64_t n = (int64_t)bx * by * bz;
  const unsigned nb = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
  k_subbox_gather<<<nb, 256, 0, c.stream>>>(c.A, (int)inst, which, (int)lo[0], (int)lo[1], (int)lo[2],
                                            bx, by, bz, dst);
  return cudaGetLastError();
}

// ---- host-buffer steps: staging arrays <-> role buffers -----------------------------------------
// The copy engines move compact arrays (instance i's cells from InstDesc::hoff, no padding); these
// kernels place them into, or compare them with, the temperature role buffers, whose indices live
// on the device, so they can be queued behind the step that rotates the roles.  Placing compares
// bit patterns first: an input that is exactly the state already there (a caller feeding back the
// results it downloaded) keeps the stored products H T^n, H T^(n-1); any other drops them.
__global__ void k_host_in(DevArrays A, const double* __restrict__ src, int which, int64_t glo,
                          int64_t ghi) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g = glo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ghi; g += stride) {
    const int inst = A.tile_inst[g / kTile];
    const InstDesc& d = A.inst[inst];
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    double* dst = A.tbuf[A.scal[inst].role[which]];
    const double v = src[d.hoff + l];
    if (dbits(dst[g]) != dbits(v)) A.scal[inst].hx_ok = 0;
    dst[g] = v;
  }
}

__global__ void k_host_check(DevArrays A, const double* __restrict__ sp,
                             const double* __restrict__ spp, int64_t call, int64_t* first) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool diff = false;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < A.ncells; g += stride) {
    const int inst = A.tile_inst[g / kTile];
    const InstDesc& d = A.inst[inst];
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const InstScal& s = A.scal[inst];
    if (s.status != 0) continue;                 // the step failed: its error is reported instead
    diff |= dbits(sp[d.hoff + l]) != dbits(A.tbuf[s.role[1]][g]);
    diff |= dbits(spp[d.hoff + l]) != dbits(A.tbuf[s.role[2]][g]);
  }
  if (diff) atomicMin(reinterpret_cast<long long*>(first), (long long)call);
}

// The result of a host-buffer step for the instances whose last residual sweep did not store it
// in A.xout; runs after the solve, before the step end rotates the roles.  A step accepted at its
// first residual (no sweep after an update: hx_fresh = 0) has x = x0 in role 2; a failed step
// keeps T^n (role 0), which is what it returns.  The blocks first look whether any instance needs
// it, so the common step costs one short pass over the instances' scalars.
__global__ void k_stage_fallback(DevArrays A) {
  int need = 0;
  for (int64_t i = threadIdx.x; i < A.ninst; i += blockDim.x) {
    const InstScal& s = A.scal[i];
    need |= (s.status != 0 || s.hx_fresh == 0) ? 1 : 0;
  }
  if (!__syncthreads_or(need)) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < A.ncells; g += stride) {
    const int inst = A.tile_inst[g / kTile];
    const InstDesc& d = A.inst[inst];
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const InstScal& s = A.scal[inst];
    if (s.status == 0 && s.hx_fresh != 0) continue;
    A.xout[d.hoff + l] = A.tbuf[s.role[s.status != 0 ? 0 : 2]][g];
  }
}

// itime of the next one-step launch; the kernel count and the failure flag accumulate over the
// queued steps (reset = first step of a queue).
__global__ void k_ctrl_init(CtrlState* ctrl, int64_t itime, int64_t limit, int reset) {
  ctrl->itime = itime;
  ctrl->itime_end = itime + 1;
  ctrl->loop_iter = 0;
  ctrl->limit = limit;
  ctrl->fin_count = 0u;
  if (reset) {
    ctrl->guard_hit = 0;
    ctrl->launches = 0;
  }
}

static unsigned host_copy_blocks(Ctx& c) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((c.ncells + 255) / 256, 152 * 8));
}

cudaError_t launch_host_in(Ctx& c, const double* src, int which, cudaStream_t stream) {
  return launch_host_in_range(c, src, which, 0, c.ncells, stream);
}

cudaError_t launch_host_in_range(Ctx& c, const double* src, int which, int64_t glo, int64_t ghi,
                                 cudaStream_t stream) {
  if (ghi <= glo) return cudaSuccess;
  const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>((ghi - glo + 255) / 256, 152 * 8));
  k_host_in<<<nb, 256, 0, stream>>>(c.A, src, which, glo, ghi);
  return cudaGetLastError();
}

cudaError_t launch_host_check(Ctx& c, const double* sp, const double* spp, int64_t call,
                              int64_t* first, cudaStream_t stream) {
  k_host_check<<<host_copy_blocks(c), 256, 0, stream>>>(c.A, sp, spp, call, first);
  return cudaGetLastError();
}

cudaError_t launch_stage_fallback(Ctx& c) {
  k_stage_fallback<<<152, 256, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}

cudaError_t launch_ctrl_init(Ctx& c, int64_t itime, int64_t limit) {
  k_ctrl_init<<<1, 1, 0, c.stream>>>(c.d_ctrl, itime, limit, c.async_steps == 0 ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_adj_rhs(Ctx& c, const double* g, const double* l1, const double* l2, double* out) {
  k_adj_rhs<<<(unsigned)((c.ncells + 255) / 256), 256, 0, c.stream>>>(c.A, g, l1, l2, out);
  return cudaGetLastError();
}

cudaError_t launch_adj_grad(Ctx& c, const double* lam, const double* x, int64_t itime,
                            double* grad_logk, double* grad_src) {
  k_adj_grad<<<(unsigned)((c.ncells + 255) / 256), 256, 0, c.stream>>>(
      c.A, c.d_bc, c.asm_.kappa, lam, x, itime, grad_logk, grad_src);
  return cudaGetLastError();
}

}  // namespace hf

namespace hf {

// ||b||^2 of a single-instance device vector (for hf_solve_device): per-block partials in a
// fixed order, then one block sums them and sets the instance's ||S||^2 and FP32 scale.
__global__ void k_sumsq_partial(DevArrays A, const double* b, int64_t n) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc = fma(b[i], b[i], acc);
  const double v[1] = {acc};
  tile_store<1>(A, blockIdx.x, v);
}

__global__ void k_sumsq_final(DevArrays A, int nparts) {
  double acc = 0.0;
  for (int t = threadIdx.x; t < nparts; t += blockDim.x) acc += A.partials[(int64_t)t * kNR];
  __shared__ double red[32];
  double v[1] = {acc};
  block_sum<1>(v, red);
  if (threadIdx.x == 0) {
    InstScal& s = A.scal[0];
    const InstDesc& d = A.inst[0];
    s.bb = v[0];
    const double rms = sqrt(v[0] / (double)d.n) * d.mean_sinv * 1e-6;
    s.sigma = (A.opts.precision == HF_PREC_MIXED && rms > 0.0 && isfinite(rms))
                  ? exp2(rint(log2(rms))) : 1.0;
  }
}

cudaError_t launch_sumsq(Ctx& c, const double* b, int64_t n) {
  const int nparts = (int)std::min<int64_t>(std::min<int64_t>((n + 255) / 256, 1024), c.ntasks);
  k_sumsq_partial<<<nparts, kBlock, 0, c.stream>>>(c.A, b, n);
  k_sumsq_final<<<1, 256, 0, c.stream>>>(c.A, nparts);
  return cudaGetLastError();
}

}  // namespace hf
