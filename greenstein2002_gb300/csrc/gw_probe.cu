// Measured FP64 FMA peak of the device: independent DFMA chains on every SM.
// The FRU stage kernel is FP64-pipe bound and the pool's measured-peak file
// lists no FP64 figure, so the benchmark measures this denominator in-run.
#include <cuda_runtime.h>

#include "gw_kernels.h"

namespace gw {

__global__ void fp64_fma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 123.456) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

cudaError_t probe_fp64(int sms, double* tflops) {
  const int threads = 256, blocks = sms * 8, iters = 4096;
  double* out = nullptr;
  cudaEvent_t e0, e1;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * threads * blocks);
  if (e != cudaSuccess) return e;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0);
    fp64_fma_loop<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
    if (e == cudaSuccess && rep > 0 && ms > 0.f) best = fmax(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = best;
  return e;
}

}  // namespace gw
