// Per-step right-hand side: heater (mod_heating.f90:27-169), Cattaneo term
// (mod_cattaneo.f90:23-42), S and the initial guess (mod_evolve.f90:112-141), in one pass.
//
// Compiled with -fmad=false so that S is rounded exactly as the reference writes it; the kernel
// is HBM-bound, so separate rounding costs nothing.
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

// One block per tile.  PARTS: also write B, Q, Qdens and S_cat (parity probe hf_get_rhs).
template <bool PARTS>
__global__ void __launch_bounds__(kBlock) k_rhs(DevArrays A, double* oB, double* oQ, double* oQd,
                                                double* oSc) {
  const int64_t tile = blockIdx.x;
  const int inst = A.tile_inst[tile];
  const InstDesc& d = A.inst[inst];
  InstScal& s = A.scal[inst];
  if (!s.outer_active) return;
  const int64_t itime = s.itime;
  const double* Tp = A.tbuf[s.role[0]] + d.off;
  const double* Tpp = A.tbuf[s.role[1]] + d.off;
  double* X = A.tbuf[s.role[2]] + d.off;
  double acc[6] = {0, 0, 0, 0, 0, 0};  // bb, x0 flags, nan Q, nan Qdens, nan S_cat, nan S
  const double tb4 = d.has_em ? pow(d.t_bath, 4.0) : 0.0;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t g = tile * kTile + k * kBlock + threadIdx.x;
    const int64_t l = g - d.off;
    if (l >= d.n) continue;
    const double tp = Tp[l], tpp = Tpp[l];
    double q = 0.0, qd = 0.0;
    if (d.heater) {
      const double P = d.has_power ? A.power[g] : d.power_in;
      const double tau = d.has_case5 ? A.tau_s[g] * pow(d.time_step, 2.0) : 0.0;
      q = heat_case(A.icase[g], P, tau, itime, d);
      if (d.has_em) q = q - A.emc[g] * (pow(tp, 4.0) - tb4);
      if (d.qdens_mode == HF_QDENS_CELL_VOLUME) qd = q / d.volume;
      else if (d.heated_volume > 0.0) qd = q / d.heated_volume;
      acc[2] += isnan(q) ? 1.0 : 0.0;
      acc[3] += isnan(qd) ? 1.0 : 0.0;
    }
    double sc = 0.0;
    if (d.icattaneo == 1) {
      sc = (tpp - 2.0 * tp) * A.ccat[g];
      acc[4] += isnan(sc) ? 1.0 : 0.0;
    }
    const double B = A.bvec[g];
    double S;
    if (d.isteady == 0) {
      S = -d.inv_dt * tp * A.rhoc[g] - qd - B;
      if (d.icattaneo == 1) S = S + sc;
    } else {
      S = -qd - B;
    }
    acc[5] += isnan(S) ? 1.0 : 0.0;
    const double x0 = tp + (tp - tpp);
    acc[1] += (x0 - tp < kTiny) ? 1.0 : 0.0;
    A.b[g] = S;
    X[l] = x0;
    acc[0] += S * S;
    if (PARTS) {
      oB[g] = B;
      oQ[g] = q;
      oQd[g] = qd;
      oSc[g] = sc;
    }
  }
  double tot[6];
  if (!tile_reduce<6>(A, inst, tile, acc, tot)) return;
  if (threadIdx.x == 0) {
    s.bb = tot[0];
    s.x0flag = tot[1] > 0.0 ? 1 : 0;
    int st = 0;
    if (tot[2] > 0) st |= 1 << (HF_ENAN_Q - HF_ENAN_B);
    if (tot[3] > 0) st |= 1 << (HF_ENAN_QDENS - HF_ENAN_B);
    if (tot[4] > 0) st |= 1 << (HF_ENAN_SCAT - HF_ENAN_B);
    if (tot[5] > 0) st |= 1 << (HF_ENAN_S - HF_ENAN_B);
    if (st) {
      s.status |= st;
      s.outer_active = 0;
      s.failed_step = itime;
    }
    // scale of the first FP32 residual: a power of two near rms(S)/rms(|H_II|^(1/2)) * 1e-6
    double rms = sqrt(tot[0] / (double)d.n) * d.mean_sinv * 1e-6;
    s.sigma = (A.opts.precision == HF_PREC_MIXED && rms > 0.0 && isfinite(rms))
                  ? exp2(rint(log2(rms))) : 1.0;
  }
}

cudaError_t launch_rhs(Ctx& c) {
  k_rhs<false><<<(unsigned)c.ntiles, kBlock, 0, c.stream>>>(c.A, nullptr, nullptr, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_rhs_parts(Ctx& c, double* B, double* Q, double* Qd, double* Sc) {
  k_rhs<true><<<(unsigned)c.ntiles, kBlock, 0, c.stream>>>(c.A, B, Q, Qd, Sc);
  return cudaGetLastError();
}

}  // namespace hf
