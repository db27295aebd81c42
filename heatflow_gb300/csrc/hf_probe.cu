// Arithmetic throughput of this GPU, measured (FMA chains, CUDA-event timed).  The FP64 rate
// decides which kernels of the step are FP64-bound rather than HBM-bound, so bench.py reports
// it beside the HBM roofline.
#include <cuda_runtime.h>

#include "../../include/heatflow_gb300.h"

namespace {

template <typename T>
__global__ void k_fma_chain(T* out, T a, T b, int iters) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int rate(int iters, double* tflops) {
  int sms = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return HF_ECUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return HF_ECUDA;
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * threads) != cudaSuccess) return HF_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T><<<blocks, threads>>>(out, (T)0.999, (T)0.001, iters / 10);
  cudaEventRecord(e0);
  k_fma_chain<T><<<blocks, threads>>>(out, (T)0.999, (T)0.001, iters);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return HF_ECUDA;
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return HF_OK;
}

}  // namespace

extern "C" int hf_measure_fp_rates(double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return HF_EARG;
  int rc = rate<double>(2000, fp64_tflops);
  if (rc) return rc;
  return rate<float>(20000, fp32_tflops);
}
