// Standalone throughput probe (not part of the library): DFMA vs DMMA (mma.sync m8n8k4 f64) vs FFMA.
// Grid/indexing: each thread writes exactly one double to out[blockIdx.x*blockDim.x+threadIdx.x];
// out is allocated for grid*block doubles.  No other memory access.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void dfma_kernel(double* out, int iters, double a) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, 1e-9); x1 = fma(x1, a, 1e-9); x2 = fma(x2, a, 1e-9); x3 = fma(x3, a, 1e-9);
    x4 = fma(x4, a, 1e-9); x5 = fma(x5, a, 1e-9); x6 = fma(x6, a, 1e-9); x7 = fma(x7, a, 1e-9);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void ffma_kernel(double* out, int iters, float a) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, 1e-9f); x1 = fmaf(x1, a, 1e-9f); x2 = fmaf(x2, a, 1e-9f); x3 = fmaf(x3, a, 1e-9f);
    x4 = fmaf(x4, a, 1e-9f); x5 = fmaf(x5, a, 1e-9f); x6 = fmaf(x6, a, 1e-9f); x7 = fmaf(x7, a, 1e-9f);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d0), "+d"(d1) : "d"(a), "d"(b));
}
__global__ void dmma_kernel(double* out, int iters, double a) {
  double c[8][2];
  for (int i = 0; i < 8; ++i) c[i][0] = c[i][1] = 0.0;
  double b = a * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) dmma(c[j][0], c[j][1], a, b);
  }
  double s = 0;
  for (int i = 0; i < 8; ++i) s += c[i][0] + c[i][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
  int dev = 0, sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4, threads = 256, iters = 4096;
  double* out;
  cudaMalloc(&out, sizeof(double) * blocks * threads);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0);
    dfma_kernel<<<blocks, threads>>>(out, iters, 0.999);
    cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    double fl = 2.0 * 8 * iters * (double)blocks * threads;
    if (rep) printf("DFMA : %.1f GFLOP/s (%.3f ms)\n", fl / ms / 1e6, ms);
    cudaEventRecord(e0);
    ffma_kernel<<<blocks, threads>>>(out, iters, 0.999f);
    cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    if (rep) printf("FFMA : %.1f GFLOP/s (%.3f ms)\n", fl / ms / 1e6, ms);
    cudaEventRecord(e0);
    dmma_kernel<<<blocks, threads>>>(out, iters / 4, 0.999);
    cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    double flm = 2.0 * 256 * 8 * (iters / 4) * (double)blocks * (threads / 32);
    if (rep) printf("DMMA : %.1f GFLOP/s (%.3f ms)\n", flm / ms / 1e6, ms);
  }
  printf("SMs %d, err=%s\n", sms, cudaGetErrorString(cudaGetLastError()));
  cudaFree(out);
  return 0;
}
