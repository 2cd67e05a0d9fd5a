// Test harness: the table-driven exponential of the chemistry sources
// (htr-solver_gb300/csrc/fastexp.cuh) and the math library's exp on the same
// arguments, on the device.
#include <cuda_runtime.h>

#include "fastexp.cuh"

__global__ void fastexp_kernel(const double *x, double *fast, double *ref, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    fast[i] = htr::exp_table(x[i]);
    ref[i] = exp(x[i]);
  }
}

extern "C" int fastexp_check(const double *x, double *fast, double *ref, int n) {
  double *d = nullptr;
  const size_t b = sizeof(double) * (size_t)n;
  if (cudaMalloc(&d, 3 * b) != cudaSuccess) return 1;
  int rc = 0;
  if (cudaMemcpy(d, x, b, cudaMemcpyHostToDevice) != cudaSuccess) rc = 2;
  if (!rc) {
    fastexp_kernel<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * n, n);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = 3;
  }
  if (!rc && cudaMemcpy(fast, d + n, b, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
  if (!rc && cudaMemcpy(ref, d + 2 * n, b, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 5;
  cudaFree(d);
  return rc;
}
