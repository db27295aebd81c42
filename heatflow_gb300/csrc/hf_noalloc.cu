// Allocation-free residual: r = b - H x and (||r||^2, ||b||^2) on caller-owned device buffers.
//
// Some callers cannot call cudaMalloc: hosts that own all device memory through their own fixed
// arena (a Fortran driver that hands the library pre-allocated buffers and leaves no headroom in
// HBM), and loops that may not stall on the allocator, since cudaMalloc can synchronise the
// device.  This entry point takes every input and
// output from the caller and keeps its only scratch - the per-block partial sums of the two
// norms - in a file-scope static device array, so it allocates nothing.
//
// The first call on a device looks up the array's device address with cudaGetSymbolAddress, so
// it belongs before any stream capture begins.  The address is kept per device together with the
// id of the CUDA context it was looked up in; a call that finds another context current (the
// device was reset with cudaDeviceReset, which unloads the array with the old context) looks the
// address up again instead of handing the kernel a stale one.
// The static array is created when the library is loaded on a device and stays resident until
// the process exits (kNoAllocScratchBytes per device that loads the library).  Every call shares
// it and it keeps the last call's contents; calls whose kernels overlap on the GPU (two streams,
// or two host threads) race on it and must be serialised by the caller.  Nothing in it needs to
// start at zero: each call writes every slot it reads.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/heatflow_gb300.h"

namespace hf {
void set_last_error(const std::string& msg);   // hf_last_error() of the library (hf_abi.cu)
}

namespace {

constexpr int kNaBlock = 256;                    // threads per block
constexpr int kNaCellsPerThread = 4;             // cells per thread (one block: 1024 cells)
constexpr int kNaCellsPerBlock = kNaBlock * kNaCellsPerThread;
constexpr int64_t kNaMaxBlocks = HF_NOALLOC_MAX_CELLS / kNaCellsPerBlock;
constexpr size_t kNoAllocScratchBytes = sizeof(double) * 2 * kNaMaxBlocks;
static_assert(kNoAllocScratchBytes == 256 * 1024, "the header states 256 KiB of static scratch");

static __device__ __align__(256) double g_noalloc_scratch[2 * kNaMaxBlocks];

// Device address of g_noalloc_scratch on each device (the host-side symbol is only a stand-in),
// with the id of the context it belongs to.
std::mutex g_mu;
struct ScratchSlot {
  double* ptr = nullptr;
  unsigned long long ctx_id = 0;
};
ScratchSlot g_scratch[128];

// cuCtxGetId through the runtime's driver entry point (no link against the driver library): the
// id of the current context, unique for the life of the process.  False if no context is current.
using CtxIdFn = int (*)(void* ctx, unsigned long long* id);
bool current_ctx_id(unsigned long long* id) {
  static CtxIdFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxIdFn>(p);
  }();
  return fn && fn(nullptr, id) == 0;
}

struct Grid {
  int nx, ny, nz;
  int px, py, pz;
};

// r = b - H x for the geometric SoA operator (face to the + neighbour stored at each cell,
// periodic wrap on the last cell of a periodic axis); per-block partials of ||r||^2, ||b||^2.
__global__ void __launch_bounds__(kNaBlock) k_residual_noalloc(Grid G, const double* __restrict__ diag,
                                                               const double* __restrict__ cx,
                                                               const double* __restrict__ cy,
                                                               const double* __restrict__ cz,
                                                               const double* __restrict__ b,
                                                               const double* __restrict__ x,
                                                               double* __restrict__ r,
                                                               double* __restrict__ scratch) {
  const int64_t n = (int64_t)G.nx * G.ny * G.nz;
  const int64_t nx = G.nx, nxy = (int64_t)G.nx * G.ny;
  double rr = 0.0, bb = 0.0;
#pragma unroll
  for (int k = 0; k < kNaCellsPerThread; ++k) {
    const int64_t l = (int64_t)blockIdx.x * kNaCellsPerBlock + k * kNaBlock + threadIdx.x;
    if (l >= n) continue;
    const int64_t cxi = l % nx, cyi = (l / nx) % G.ny, czi = l / nxy;
    double acc = fma(-diag[l], x[l], b[l]);
    if (cxi + 1 < G.nx) acc = fma(-cx[l], x[l + 1], acc);
    else if (G.px && G.nx > 1) acc = fma(-cx[l], x[l - (nx - 1)], acc);
    if (cxi > 0) acc = fma(-cx[l - 1], x[l - 1], acc);
    else if (G.px && G.nx > 1) acc = fma(-cx[l + nx - 1], x[l + nx - 1], acc);
    if (cyi + 1 < G.ny) acc = fma(-cy[l], x[l + nx], acc);
    else if (G.py && G.ny > 1) acc = fma(-cy[l], x[l - (G.ny - 1) * nx], acc);
    if (cyi > 0) acc = fma(-cy[l - nx], x[l - nx], acc);
    else if (G.py && G.ny > 1) acc = fma(-cy[l + (G.ny - 1) * nx], x[l + (G.ny - 1) * nx], acc);
    if (czi + 1 < G.nz) acc = fma(-cz[l], x[l + nxy], acc);
    else if (G.pz && G.nz > 1) acc = fma(-cz[l], x[l - (G.nz - 1) * nxy], acc);
    if (czi > 0) acc = fma(-cz[l - nxy], x[l - nxy], acc);
    else if (G.pz && G.nz > 1) acc = fma(-cz[l + (G.nz - 1) * nxy], x[l + (G.nz - 1) * nxy], acc);
    r[l] = acc;
    rr = fma(acc, acc, rr);
    bb = fma(b[l], b[l], bb);
  }
  __shared__ double red[2][kNaBlock];
  red[0][threadIdx.x] = rr;
  red[1][threadIdx.x] = bb;
  __syncthreads();
  for (int s = kNaBlock / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    scratch[2 * blockIdx.x] = red[0][0];
    scratch[2 * blockIdx.x + 1] = red[1][0];
  }
}

// One block sums the per-block partials in block order and writes the two norms.
__global__ void __launch_bounds__(kNaBlock) k_norms_noalloc(const double* __restrict__ scratch,
                                                            int64_t nblocks, double* __restrict__ out) {
  double rr = 0.0, bb = 0.0;
  for (int64_t i = threadIdx.x; i < nblocks; i += kNaBlock) {
    rr += scratch[2 * i];
    bb += scratch[2 * i + 1];
  }
  __shared__ double red[2][kNaBlock];
  red[0][threadIdx.x] = rr;
  red[1][threadIdx.x] = bb;
  __syncthreads();
  for (int s = kNaBlock / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0][0];
    out[1] = red[1][0];
  }
}

// Device address of the static scratch on the current device, looked up once per device.
int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    hf::set_last_error(std::string("hf_residual_noalloc: no current CUDA device: ") + cudaGetErrorString(e));
    return HF_ECUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  ScratchSlot& slot = g_scratch[dev];
  unsigned long long id = 0;
  if (!slot.ptr || !current_ctx_id(&id) || id != slot.ctx_id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);   // makes the device's context current
    if (e != cudaSuccess || !p) {
      hf::set_last_error(std::string("hf_residual_noalloc: cudaGetSymbolAddress failed: ") +
                         cudaGetErrorString(e));
      return HF_ECUDA;
    }
    slot.ptr = static_cast<double*>(p);
    slot.ctx_id = current_ctx_id(&id) ? id : 0;
  }
  *out = slot.ptr;
  return HF_OK;
}

}  // namespace

extern "C" int hf_residual_noalloc(int64_t nx, int64_t ny, int64_t nz, const int32_t* periodic,
                                   const double* diag, const double* cx, const double* cy,
                                   const double* cz, const double* b, const double* x, double* r,
                                   double* norms2, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || !diag || !cx || !cy || !cz || !b || !x || !r || !norms2) {
    hf::set_last_error("hf_residual_noalloc: dimensions must be >= 1 and every pointer non-null");
    return HF_EARG;
  }
  // the cell count is formed only once it cannot overflow: each factor and each partial product
  // is held to the limit first
  const int64_t lim = HF_NOALLOC_MAX_CELLS;
  if (nx > lim || ny > lim / nx || nz > lim / (nx * ny)) {
    hf::set_last_error("hf_residual_noalloc: a grid of " + std::to_string((long long)nx) + " x " +
                       std::to_string((long long)ny) + " x " + std::to_string((long long)nz) +
                       " cells exceeds the static scratch limit HF_NOALLOC_MAX_CELLS = " +
                       std::to_string((long long)lim));
    return HF_EARG;
  }
  const int64_t n = nx * ny * nz;
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  Grid G{(int)nx, (int)ny, (int)nz, periodic ? periodic[0] != 0 : 0, periodic ? periodic[1] != 0 : 0,
         periodic ? periodic[2] != 0 : 0};
  const int64_t nblocks = (n + kNaCellsPerBlock - 1) / kNaCellsPerBlock;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_residual_noalloc<<<(unsigned)nblocks, kNaBlock, 0, st>>>(G, diag, cx, cy, cz, b, x, r, scratch);
  k_norms_noalloc<<<1, kNaBlock, 0, st>>>(scratch, nblocks, norms2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    hf::set_last_error(std::string("hf_residual_noalloc: launch failed: ") + cudaGetErrorString(e));
    return HF_ECUDA;
  }
  return HF_OK;
}
