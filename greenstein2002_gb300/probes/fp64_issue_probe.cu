// FP64 issue-cost probe on one SM: clock64()-timed chains of 4096 dependent
// (or 8 independent) operations -- DFMA with 32/16/4/1 active lanes and 1-16
// warps, a DDIV+DADD chain, an exp() chain and an FP32 FFMA chain.  Each
// kernel runs one block; the printed figure is cycles per operation of warp 0.
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_issue_probe fp64_issue_probe.cu
//   ./fp64_issue_probe
#include <cstdio>
#include <cuda_runtime.h>
__global__ void dep_fma(double* out, int n, int active, double a, double b) {
  if (threadIdx.x % 32 >= active) return;
  double x = threadIdx.x * 1e-6;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) x = fma(x, a, b);
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = x; out[1] = (double)(t1 - t0) / n; }
  else if (x == 1.2345) out[2] = x;
}
__global__ void ind_fma(double* out, int n, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) { x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b); }
  long long t1 = clock64();
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (threadIdx.x == 0) { out[0] = s; out[1] = (double)(t1 - t0) / (8.0 * n); }
  else if (s == 1.2345) out[2] = s;
}
__global__ void dep_div(double* out, int n, int active) {
  if (threadIdx.x % 32 >= active) return;
  double x = 1.0 + threadIdx.x * 1e-6;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) x = 1.0000001 + 1.0 / x;
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = x; out[1] = (double)(t1 - t0) / n; }
  else if (x == 1.2345) out[2] = x;
}
__global__ void dep_exp(double* out, int n, int active) {
  if (threadIdx.x % 32 >= active) return;
  double x = 0.1 + threadIdx.x * 1e-6;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) x = exp(-x) ;
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = x; out[1] = (double)(t1 - t0) / n; }
  else if (x == 1.2345) out[2] = x;
}
__global__ void dep_ffma(double* out, int n, float a, float b) {
  float x = threadIdx.x * 1e-6f;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) x = fmaf(x, a, b);
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = x; out[1] = (double)(t1 - t0) / n; }
  else if (x == 1.2345f) out[2] = x;
}
int main() {
  double *d, h[3];
  cudaMalloc(&d, 3 * sizeof(double));
  const int n = 4096;
  for (int act : {32, 16, 4, 1}) {
    dep_fma<<<1, 32>>>(d, n, act, 0.999999, 1e-7); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
    printf("dependent DFMA, 1 warp, %2d active lanes: %.1f cycles/op\n", act, h[1]);
  }
  for (int w : {1, 2, 4, 8}) {
    dep_fma<<<1, 32 * w>>>(d, n, 32, 0.999999, 1e-7); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
    printf("dependent DFMA, %d warps/SM, 32 lanes: %.1f cycles/op (warp 0)\n", w, h[1]);
  }
  for (int w : {1, 4, 16}) {
    ind_fma<<<1, 32 * w>>>(d, n, 0.999999, 1e-7); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
    printf("8 independent DFMA chains, %d warps/SM: %.1f cycles per DFMA per warp (warp 0)\n", w, h[1]);
  }
  for (int act : {32, 1}) {
    dep_div<<<1, 32>>>(d, n, act); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
    printf("dependent DDIV+DADD, %2d lanes: %.1f cycles/op\n", act, h[1]);
    dep_exp<<<1, 32>>>(d, n, act); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
    printf("dependent exp(), %2d lanes: %.1f cycles/op\n", act, h[1]);
  }
  dep_ffma<<<1, 32>>>(d, n, 0.999f, 1e-3f); cudaMemcpy(h, d, 24, cudaMemcpyDeviceToHost);
  printf("dependent FFMA, 1 warp: %.1f cycles/op\n", h[1]);
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return 0;
}
