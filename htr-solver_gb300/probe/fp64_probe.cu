// FP64 rate probe of the benchmark (not part of the library): the FP64 peak
// of the device is measured with a dependent-chain DFMA loop (8 independent
// chains per thread, enough blocks to fill every SM) and used as the
// denominator of the FP64 roofline fractions.  Built into libhtr_probe.so.
#include <cuda_runtime.h>

#include "htr_rhs.h"

namespace {
__global__ void dfma_loop(double *out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
         a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, b, c);
    a1 = fma(a1, b, c);
    a2 = fma(a2, b, c);
    a3 = fma(a3, b, c);
    a4 = fma(a4, b, c);
    a5 = fma(a5, b, c);
    a6 = fma(a6, b, c);
    a7 = fma(a7, b, c);
  }
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
}  // namespace

extern "C" int htr_probe_fp64_tflops(int iters, double *tflops) {
  if (tflops == nullptr || iters <= 0) return HTR_ERR_ARGUMENT;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return HTR_ERR_NO_DEVICE;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * (size_t)threads * blocks) != cudaSuccess) return HTR_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_loop<<<blocks, threads>>>(out, iters / 10 + 1, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  dfma_loop<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return HTR_ERR_CUDA;
  *tflops = 2.0 * 8.0 * (double)iters * threads * (double)blocks / (ms * 1e-3) / 1e12;
  return HTR_OK;
}
