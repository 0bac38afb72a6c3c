// Measured FP64 issue peak of the device (the roof of the FP64-bound sweep
// kernels): DFMA throughput with 8 independent dependency chains per thread
// and enough resident warps to hide the pipe latency.
#include <cuda_runtime.h>

#include "../../include/idefix_gb300.h"

namespace {

constexpr int kChains = 8;

__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace

extern "C" int idfx_measure_fp64_peak(double* gops, void* stream) {
  if (!gops) return IDFX_ERR_STATE;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return IDFX_ERR_CUDA;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_peak<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(e0, s);
    k_dfma_peak<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t rc = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (rc != cudaSuccess) return IDFX_ERR_CUDA;
  *gops = (double)blocks * threads * iters * kChains / (best * 1e-3) / 1e9;
  return IDFX_OK;
}
