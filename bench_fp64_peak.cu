// FP64 pipe peak microbenchmark (measurement infrastructure for the roofline; not a
// compute entry point). Independent DFMA chains in every lane of 8 x SM-count blocks of
// 256 threads; the result is the best of `reps` timed launches, in DFMA lane-operations
// per second (1 DFMA = 2 flops).
#include <cuda_runtime.h>

namespace {
__global__ void dfma_chains(double* out, int iters) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1.0 + 1e-9 * (threadIdx.x + k);
  const double b = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int sgdyn_probe_fp64_dfma_rate(int reps, double* dfma_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  const int blocks = sms * 8, threads = 256, iters = 2000;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < reps + 1; r++) {
    cudaEventRecord(e0);
    dfma_chains<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return -3;
  *dfma_per_s = double(blocks) * threads * iters * 8 / (best * 1e-3);
  return 0;
}
