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
#include "hf_ctx.cuh"

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

// One block per task.  PARTS: also write B, Q, Qdens and S_cat (parity probe hf_get_rhs).
// DIAG: count NaNs per vector (failure path only).
template <bool PARTS, bool DIAG>
__global__ void __launch_bounds__(kBlock) k_rhs(DevArrays A, double* oB, double* oQ, double* oQd,
                                                double* oSc) {
  const int64_t task = blockIdx.x;
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
  const double* __restrict__ Tp = A.tbuf[s.role[0]] + off;
  const double* __restrict__ Tpp = A.tbuf[s.role[1]] + off;
  double* __restrict__ X = A.tbuf[s.role[2]] + off;
  const double* __restrict__ rhoc = A.rhoc + off;
  const double* __restrict__ ccat = A.ccat + off;
  const double* __restrict__ bvec = A.bvec + off;
  double* __restrict__ bout = A.b + off;
  const double tb4 = has_em ? pow(d.t_bath, 4.0) : 0.0;
  const double dt2 = case5 ? pow(d.time_step, 2.0) : 0.0;
  double bb = 0.0;
  int flag = 0;
  int nan_q = 0, nan_qd = 0, nan_sc = 0, nan_s = 0;
  if (c.act) {
#pragma unroll 4
    for (int z = c.z0; z < c.z1; ++z) {
      const int l = c.base + z * c.nxy;
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
      if (cat) {
        sc = fma(-2.0, tp, tpp) * ccat[l];   // = (tpp - 2 tp) * ccat: 2 tp is exact
        if (DIAG) nan_sc += dbl_is_nan(sc);
      }
      const double B = bvec[l];
      double S;
      if (!steady) {
        S = -inv_dt * tp * rhoc[l];
        if (!dbl_is_zero(qd)) S = S - qd;
        if (!dbl_is_zero(B)) S = S - B;
        if (cat) S = S + sc;
      } else {
        S = -qd;
        if (!dbl_is_zero(B)) S = S - B;
      }
      if (DIAG) nan_s += dbl_is_nan(S);
      const double x0 = tp + (tp - tpp);
      flag |= dbl_lt_pos(x0 - tp, kTiny) ? 1 : 0;
      bout[l] = S;
      X[l] = x0;
      bb = fma(S, S, bb);
      if (PARTS) {
        oB[off + l] = B;
        oQ[off + l] = q;
        oQd[off + l] = qd;
        oSc[off + l] = sc;
      }
    }
  }
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

cudaError_t launch_rhs(Ctx& c) {
  k_rhs<false, false><<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, nullptr, nullptr, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_rhs_parts(Ctx& c, double* B, double* Q, double* Qd, double* Sc) {
  k_rhs<true, false><<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, B, Q, Qd, Sc);
  return cudaGetLastError();
}

cudaError_t launch_rhs_diagnose(Ctx& c) {
  k_rhs<false, true><<<(unsigned)c.ntasks, kBlock, 0, c.stream>>>(c.A, nullptr, nullptr, nullptr, nullptr);
  return cudaGetLastError();
}

}  // namespace hf
