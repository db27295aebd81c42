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
constexpr int kNR = 8;                       // reduction slots per tile
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
  int32_t role[4];      // temperature buffers: [0]=T^n, [1]=T^(n-1), [2]=x read, [3]=x write
  double sigma_prev;    // scale used by the previous residual sweep
  double last_err, last_relres;   // of the last finished step
  int64_t last_iter;
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
  double* partials;       // ntiles * kNR
  unsigned int* counters; // per instance, last-block detection
  DevOpts opts;
  // static
  double *diag, *cx, *cy, *cz, *sinv, *a64x, *a64y, *a64z;
  float *a32x, *a32y, *a32z;
  double *rhoc, *ccat, *bvec, *power, *emc;
  int8_t* icase;
  double* tau_s;          // tau/dt^2 (heater case 5)
  // state: four temperature-sized buffers, roles per instance in InstScal::role
  double* tbuf[4];
  // solver
  double *b, *y, *r, *p, *q;
  float *y32, *r32, *p32, *q32;
  int64_t ncells, ntiles, ninst;
};

// ---- helpers ---------------------------------------------------------------------------------
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

// Write this tile's partial sums; returns true (in all threads) for the last tile of the
// instance to arrive, which then holds the instance totals in tot[] (fixed summation order).
template <int NRV>
__device__ bool tile_reduce(const DevArrays& A, int inst, int64_t tile, double (&v)[NRV],
                            double (&tot)[NRV]) {
  __shared__ double red[32 * NRV];
  __shared__ bool last;
  block_sum<NRV>(v, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NRV; ++k) A.partials[tile * kNR + k] = v[k];
    __threadfence();
    unsigned prev = atomicAdd(&A.counters[inst], 1u);
    last = (prev == (unsigned)A.inst[inst].ntiles - 1u);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const InstDesc& d = A.inst[inst];
  double acc[NRV];
#pragma unroll
  for (int k = 0; k < NRV; ++k) acc[k] = 0.0;
  for (int64_t t = threadIdx.x; t < d.ntiles; t += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NRV; ++k) acc[k] += __ldcg(&A.partials[(d.tile0 + t) * kNR + k]);
  }
  block_sum<NRV>(acc, red);
  __shared__ double out[NRV];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NRV; ++k) out[k] = acc[k];
    A.counters[inst] = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NRV; ++k) tot[k] = out[k];
  return true;
}

// Coordinates of local cell l in an instance.
struct Coord {
  int32_t x, y, z;
};
__device__ __forceinline__ Coord coord_of(const InstDesc& d, int32_t l) {
  Coord c;
  uint32_t ul = (uint32_t)l;
  uint32_t row = ul / (uint32_t)d.nx;
  c.x = (int32_t)(ul - row * (uint32_t)d.nx);
  uint32_t pl = row / (uint32_t)d.ny;
  c.y = (int32_t)(row - pl * (uint32_t)d.ny);
  c.z = (int32_t)pl;
  return c;
}

// ---- host-side launchers (defined in the .cu files) ------------------------------------------
struct Ctx;
cudaError_t launch_assemble(Ctx& c);
cudaError_t launch_coo(Ctx& c, int64_t instance, int64_t* d_counts, int64_t* d_irow,
                       int64_t* d_jcol, double* d_val, int64_t* d_pos, int phase);
cudaError_t launch_step_begin(Ctx& c, int64_t itime, int first_of_run);
cudaError_t launch_rhs(Ctx& c);
cudaError_t launch_rhs_parts(Ctx& c, double* B, double* Q, double* Qd, double* Sc);
cudaError_t launch_residual(Ctx& c, int mode);
cudaError_t launch_inner_iteration(Ctx& c, int fp32);
cudaError_t launch_step_end(Ctx& c);
cudaError_t launch_apply(Ctx& c, const double* x, double* y);
cudaError_t launch_single(Ctx& c, int which);

}  // namespace hf
