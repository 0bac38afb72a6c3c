// Measured FP64 issue peak of the device (the roof of the FP64-bound sweep
// kernels): DFMA throughput with 8 independent dependency chains per thread
// and enough resident warps to hide the pipe latency.
#include <cuda_runtime.h>

#include "../../include/idefix_gb300.h"
#include "fpconv.cuh"
#include "intdiv.cuh"
#include "rdiv.cuh"

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

__device__ __forceinline__ unsigned long long mix(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// random operand pairs: full normal range, a moderate range, significands
// near 1 and 2, and quotients at the edges of the normal range
__global__ void k_check_division(long long n, unsigned long long seed, unsigned long long* bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long h1 = mix(seed ^ (2 * i)), h2 = mix(seed ^ (2 * i + 1)), h3 = mix(h1 ^ h2);
  const unsigned long long M = (1ull << 52) - 1;
  unsigned long long ea, eb, ma = h1 & M, mb = h2 & M;
  switch (h3 % 4) {
    case 0: ea = 1 + (h1 >> 53) % 2046; eb = 1 + (h2 >> 53) % 2046; break;
    case 1: ea = 900 + (h1 >> 53) % 250; eb = 900 + (h2 >> 53) % 250; break;
    case 2:
      ea = 1000 + (h1 >> 58) % 40;
      eb = 1000 + (h2 >> 58) % 40;
      if (h3 & 16) mb = (h3 & 32) ? (h2 >> 40) : M - (h2 >> 40);
      if (h3 & 64) ma = (h3 & 128) ? (h1 >> 40) : M - (h1 >> 40);
      break;
    default: ea = 1 + (h1 >> 58) % 60; eb = 1000 + (h2 >> 58) % 60; break;
  }
  const double a = __longlong_as_double((long long)(((h1 & (1ull << 63))) | (ea << 52) | ma));
  const double b = __longlong_as_double((long long)(((h2 & (1ull << 63))) | (eb << 52) | mb));
  const double r0 = a / b, r1 = idfx::div_rn(a, b);
  if (__double_as_longlong(r0) != __double_as_longlong(r1)) atomicAdd(bad, 1ull);
  // the reciprocal form of the flux sweeps (rdiv.cuh)
  const double r2 = idfx::div_r(a, idfx::recip(b));
  if (__double_as_longlong(r0) != __double_as_longlong(r2)) atomicAdd(bad, 1ull);
}

// f2d_exact on a stride of all binary32 patterns, d2f_rn on random binary64
// values (any pattern, the binary32 range and its edges, rounding ties)
__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long h1 = mix(seed ^ (2 * i)), h2 = mix(seed ^ (2 * i + 1));
  const float f = __uint_as_float((unsigned)h1);
  const double a0 = (double)f, a1 = idfx::f2d_exact(f);
  if (__double_as_longlong(a0) != __double_as_longlong(a1) && !(a0 != a0 && a1 != a1)) atomicAdd(bad, 1ull);
  unsigned long long u;
  switch (h2 % 3) {
    case 0: u = h1 ^ h2; break;
    case 1: u = (h2 & (1ull << 63)) | ((860 + (h1 >> 40) % 330) << 52) | (h2 & ((1ull << 52) - 1)); break;
    default: {
      const unsigned long long m = ((h1 & ((1ull << 23) - 1)) << 29) + (1ull << 28) + (h2 >> 61) - 2;
      u = (h2 & (1ull << 63)) | ((897 + (h1 >> 40) % 254) << 52) | (m & ((1ull << 52) - 1));
    }
  }
  const double x = __longlong_as_double((long long)u);
  const float b0 = __double2float_rn(x), b1 = idfx::d2f_rn(x);
  if (__float_as_uint(b0) != __float_as_uint(b1) && !(b0 != b0 && b1 != b1)) atomicAdd(bad, 1ull);
}

}  // namespace

extern "C" int idfx_check_conversions(long long n, unsigned long long seed, long long* mismatches) {
  if (!mismatches || n < 0) return IDFX_ERR_STATE;
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) return IDFX_ERR_CUDA;
  cudaMemset(bad, 0, sizeof(*bad));
  if (n > 0) k_check_conversions<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, bad);
  unsigned long long h = 0;
  const cudaError_t rc = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (rc != cudaSuccess || cudaGetLastError() != cudaSuccess) return IDFX_ERR_CUDA;
  *mismatches = (long long)h;
  return IDFX_OK;
}

extern "C" int idfx_check_division(long long n, unsigned long long seed, long long* mismatches) {
  if (!mismatches || n < 0) return IDFX_ERR_STATE;
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) return IDFX_ERR_CUDA;
  cudaMemset(bad, 0, sizeof(*bad));
  if (n > 0) k_check_division<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, bad);
  unsigned long long h = 0;
  const cudaError_t rc = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (rc != cudaSuccess || cudaGetLastError() != cudaSuccess) return IDFX_ERR_CUDA;
  *mismatches = (long long)h;
  return IDFX_OK;
}

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
