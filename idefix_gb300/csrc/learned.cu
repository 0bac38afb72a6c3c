// Learned interface-state correction (see learned.cuh): BF16 training
// kernels on the 5th-generation tensor cores (forward, backward; Adam), the
// training-data kernels (coarsening of fine snapshots, batch assembly) and
// the learned sweep of the ORDER 5 solver (network inference fused with the
// reconstruction, the Riemann solve and the flux difference), with their C
// ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/idefix_gb300.h"
#include "engine.hpp"
#include "learned.cuh"
#include "umma.cuh"

using namespace idfx;
using namespace idfx::learn;

namespace {

// ---------------------------------------------------------------------------
// BF16 GEMM of the training on the 5th-generation tensor cores:
// C[M][N] = op(A)[M][K] . op(B)[K][N], FP32 accumulation in tensor memory.
// A(m,k) = transA ? A[k*lda + m] : A[m*lda + k]
// B(k,n) = transB ? B[n*ldb + k] : B[k*ldb + n]
// CTA tile 128 x N (N <= 128, a multiple of 16); K in chunks of 64 staged
// in the canonical K-major layout by all threads, two stages (the next chunk
// is staged while the tensor core works on the current one); one thread
// issues the MMAs and commits them to the stage's mbarrier; the epilogue
// reads each row from tensor memory (thread = row).
// ---------------------------------------------------------------------------
enum Epi { kEpiF32 = 0, kEpiBiasSilu = 1, kEpiBias = 2, kEpiDsilu = 3 };

struct EpiArgs {
  int mode;
  const float* bias;   // [N]           (kEpiBiasSilu, kEpiBias)
  const float* zin;    // [M][ldo]      (kEpiDsilu: pre-activation)
  float* out_f;        // [M][ldo]      FP32 result (Z, Y, dW, dZ)
  __nv_bfloat16* out_b;  // [M][ldo]    BF16 result (H = silu(Z), dZ)
  int ldo;
};

constexpr int GT_M = 128, GT_N = 128, GT_KC = 64;

// One operand chunk (R rows x GT_KC columns of k) into the canonical K-major
// layout, zero outside rows < Rmax and k < K.  kcontig: element (r, k) at
// src[r * ld + k] - eight consecutive k are one 16-byte load and one 16-byte
// core-matrix row in shared memory; else at src[k * ld + r] - eight
// consecutive rows are one 16-byte load, scattered over a core matrix's rows.
// Vector loads where ld and the base allow them (ld a multiple of 8, base
// 16-byte aligned; chunk and tile origins are multiples of 8).
__device__ __forceinline__ void stage_tile(__nv_bfloat16* dst, const __nv_bfloat16* __restrict__ src, int ld,
                                           bool kcontig, int r0, int Rmax, int k0, int K, int R) {
  const bool vec = (ld & 7) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (kcontig) {
    for (int e = threadIdx.x; e < R * (GT_KC / 8); e += blockDim.x) {
      const int r = e / (GT_KC / 8), kv = (e % (GT_KC / 8)) * 8;
      const int gr = r0 + r, gk = k0 + kv;
      alignas(16) __nv_bfloat16 t[8];
      if (gr < Rmax && vec && gk + 8 <= K) {
        *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(src + (long long)gr * ld + gk);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) t[i] = (gr < Rmax && gk + i < K) ? src[(long long)gr * ld + gk + i] : zero;
      }
      *reinterpret_cast<uint4*>(dst + umma::kmajor_offset(r, kv, GT_KC) / 2) = *reinterpret_cast<const uint4*>(t);
    }
  } else {
    const int rg = R / 8;  // groups of eight rows; consecutive threads take consecutive groups
    for (int e = threadIdx.x; e < rg * GT_KC; e += blockDim.x) {
      const int rv = (e % rg) * 8, k = e / rg;
      const int gr = r0 + rv, gk = k0 + k;
      alignas(16) __nv_bfloat16 t[8];
      if (gk < K && vec && gr + 8 <= Rmax) {
        *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(src + (long long)gk * ld + gr);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) t[i] = (gk < K && gr + i < Rmax) ? src[(long long)gk * ld + gr + i] : zero;
      }
#pragma unroll
      for (int i = 0; i < 8; i++) dst[umma::kmajor_offset(rv + i, k, GT_KC) / 2] = t[i];
    }
  }
}
constexpr size_t GT_A = (size_t)GT_M * GT_KC * 2, GT_B = (size_t)GT_N * GT_KC * 2;
constexpr size_t GT_STAGE = GT_A + GT_B;
constexpr size_t GT_SMEM = 2 * GT_STAGE + 64;

__global__ void __launch_bounds__(128, 1) k_gemm_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                    int lda, int transA, const __nv_bfloat16* __restrict__ B,
                                                    int ldb, int transB, EpiArgs ep, int* status, int cps,
                                                    float* __restrict__ part) {
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * GT_STAGE);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
  const int nt = min(GT_N, N - n0);  // a multiple of 16
  uint32_t ncols = 32;
  while ((int)ncols < nt) ncols <<= 1;
  if (warp == 0) umma::tmem_alloc(slot, ncols);
  if (tid == 0) {
    umma::mbar_init1(bar);
    umma::mbar_init1(bar + 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t taddr = *slot;
  const uint32_t idesc = umma::idesc_bf16_f32(GT_M, nt);
  // split K (blockIdx.z): this CTA's chunks of GT_KC start at q0
  const int nq_all = (K + GT_KC - 1) / GT_KC;
  const int q0 = blockIdx.z * cps;
  const int nq = min(cps, nq_all - q0);
  bool ok = true;
  for (int q = 0; q < nq; q++) {
    const int st = q & 1;
    if (q >= 2) {  // stage st is free once the MMAs of chunk q - 2 have landed
      const bool w = umma::mbar_wait_bounded(bar + st, (uint32_t)(((q - 2) >> 1) & 1), umma::kMmaSpin);
      ok = __syncthreads_and(w);
      if (!ok) break;
    }
    __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(sm + st * GT_STAGE);
    __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(sm + st * GT_STAGE + GT_A);
    const int k0 = (q0 + q) * GT_KC;
    // A(m, k): k contiguous in memory unless transposed; B(k, n) as the
    // N x K operand: k contiguous when transposed
    stage_tile(As, A, lda, !transA, m0, M, k0, K, GT_M);
    stage_tile(Bs, B, ldb, transB != 0, n0, N, k0, K, nt);
    umma::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
      umma::mma_tile(taddr, umma::smem_addr(As), umma::smem_addr(Bs), GT_KC, idesc, q > 0);
      umma::mma_commit(bar + st);
    }
  }
  if (ok) {  // the last commit lands after every MMA issued before it
    const int q = nq - 1;
    const bool w = umma::mbar_wait_bounded(bar + (q & 1), (uint32_t)((q >> 1) & 1), umma::kMmaSpin);
    ok = __syncthreads_and(w);
  }
  umma::fence_after_sync();
  if (ok) {
    const int m = m0 + 32 * warp + lane;
    for (int c = 0; c < nt; c += 16) {
      float v[16];
      umma::tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
      if (m >= M) continue;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int n = n0 + c + i;
        if (n >= N) continue;
        const long long o = (long long)m * ep.ldo + n;
        float x = v[i];
        if (part) {  // split K: this split's partial product, summed by k_splitk_sum
          part[((long long)blockIdx.z * M + m) * N + n] = x;
          continue;
        }
        switch (ep.mode) {
          case kEpiF32:
            ep.out_f[o] = x;
            break;
          case kEpiBiasSilu:
            x += ep.bias[n];
            ep.out_f[o] = x;
            ep.out_b[o] = __float2bfloat16(silu_f(x));
            break;
          case kEpiBias:
            ep.out_f[o] = x + ep.bias[n];
            break;
          default:  // kEpiDsilu
            x *= dsilu_f(ep.zin[o]);
            ep.out_f[o] = x;
            ep.out_b[o] = __float2bfloat16(x);
            break;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(status, 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(taddr, ncols);
}

// out = sum over the S partial products, in split order (deterministic)
__global__ void k_splitk_sum(const float* __restrict__ part, int S, int M, int N, float* __restrict__ out, int ldo) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)M * N) return;
  float acc = 0.f;
  for (int z = 0; z < S; z++) acc += part[(long long)z * M * N + e];
  out[(e / N) * ldo + e % N] = acc;
}

constexpr int GT_MAX_SPLITS = 64;
// split-K workspace of a trainer: GT_MAX_SPLITS partial products of up to
// 256 x 128
constexpr size_t GT_WS_FLOATS = (size_t)GT_MAX_SPLITS * 256 * 128;

// N a multiple of 16 (every use: NH, NOUT); status: set when a bounded wait
// of the tensor-core pipeline gave up.  A product with few output tiles and
// a long K (the weight gradients: K = the batch) is split over K into up to
// GT_MAX_SPLITS CTAs per tile, the partial products summed in split order
// by a second kernel (ws: GT_WS_FLOATS floats).
void gemm(cudaStream_t s, int M, int N, int K, const __nv_bfloat16* A, int lda, int transA, const __nv_bfloat16* B,
          int ldb, int transB, const EpiArgs& ep, int* status, float* ws) {
  dim3 grid((N + GT_N - 1) / GT_N, (M + GT_M - 1) / GT_M, 1);
  const int nq = (K + GT_KC - 1) / GT_KC;
  const int tiles = (int)(grid.x * grid.y);
  int cps = nq;
  if (ws && ep.mode == kEpiF32 && tiles < 64 && nq >= 4 && (size_t)M * N <= 256 * 128) {
    int splits = std::min(std::min(GT_MAX_SPLITS, (128 + tiles - 1) / tiles), nq / 2);
    cps = (nq + splits - 1) / splits;
    grid.z = (unsigned)((nq + cps - 1) / cps);
  }
  float* part = grid.z > 1 ? ws : nullptr;
  k_gemm_tc<<<grid, 128, GT_SMEM, s>>>(M, N, K, A, lda, transA, B, ldb, transB, ep, status, cps, part);
  if (part) {
    const long long mn = (long long)M * N;
    k_splitk_sum<<<(unsigned)((mn + 255) / 256), 256, 0, s>>>(part, (int)grid.z, M, N, ep.out_f, ep.ldo);
  }
}

// column sums (bias gradients): out[n] = sum_m in[m][n]
__global__ void k_colsum(const float* __restrict__ in, int M, int N, float* __restrict__ out) {
  const int n = blockIdx.x;
  float s = 0.f;
  for (int m = threadIdx.x; m < M; m += blockDim.x) s += in[(long long)m * N + n];
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = red[0];
}

// masked squared error: dY = 2 (Y - T) / B (BF16 and FP32), loss += sum (Y - T)^2 / B
__global__ void k_loss(const float* __restrict__ Y, const float* __restrict__ T, int B, float* __restrict__ dYf,
                       __nv_bfloat16* __restrict__ dYb, double* __restrict__ loss) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (e < (long long)B * NOUT) {
    const int o = (int)(e % NOUT);
    const float r = loss_masked(o) ? 0.f : Y[e] - T[e];
    const float d = 2.f * r / (float)B;
    dYf[e] = d;
    dYb[e] = __float2bfloat16(d);
    l = (double)r * r / B;
  }
  for (int w = 16; w > 0; w >>= 1) l += __shfl_down_sync(0xffffffffu, l, w);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// Adam step over the packed FP32 parameters; refreshes the BF16 weights
// (W1b has K1 rows, the last K1 - NIN stay zero)
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                       float lr, float b1, float b2, float eps, float bc1, float bc2, __nv_bfloat16* __restrict__ W1b,
                       __nv_bfloat16* __restrict__ W2b, __nv_bfloat16* __restrict__ W3b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  const float gp = g[p];
  const float mp = b1 * m[p] + (1.f - b1) * gp;
  const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
  m[p] = mp;
  v[p] = vp;
  const float wp = w[p] - lr * (mp / bc1) / (sqrtf(vp / bc2) + eps);
  w[p] = wp;
  if (p < OB1) W1b[p - OW1] = __float2bfloat16(wp);
  else if (p >= OW2 && p < OB2) W2b[p - OW2] = __float2bfloat16(wp);
  else if (p >= OW3 && p < OB3) W3b[p - OW3] = __float2bfloat16(wp);
}

__global__ void k_refresh_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ W1b,
                               __nv_bfloat16* __restrict__ W2b, __nv_bfloat16* __restrict__ W3b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < K1 * NH) W1b[p] = __float2bfloat16(p < NIN * NH ? w[OW1 + p] : 0.f);
  if (p < NH * NH) W2b[p] = __float2bfloat16(w[OW2 + p]);
  if (p < NH * NOUT) W3b[p] = __float2bfloat16(w[OW3 + p]);
}

// ---------------------------------------------------------------------------
// Coarsening of a fine snapshot (ghosted reference layout, 3-D, periodic):
// conserved averages over r^3 cells, face fields over r^2 faces, cell field
// from the coarse faces, ConsToPrim; and the face targets: per direction d,
// the fine primitives extrapolated to the coarse cell's two faces from the
// two fine layers next to each face (1.5 x outer layer - 0.5 x next layer;
// the outer layer alone when r = 1), averaged over the face (rotated
// variable order).
// One thread per coarse cell.  Outputs (compact, C order z, y, x):
//   prim[8][nc^3], faces[3][nc^3] (left faces), tgt[3][16][nc^3]
// ---------------------------------------------------------------------------
__global__ void k_coarsen(const double* __restrict__ Vc, const double* __restrict__ Vs, int nf, int ng, int r,
                          double gamma, double* __restrict__ prim, double* __restrict__ faces,
                          double* __restrict__ tgt) {
  const int nc = nf / r;
  const long long ncell_c = (long long)nc * nc * nc;
  const long long cid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cid >= ncell_c) return;
  const int X = (int)(cid % nc), Y = (int)((cid / nc) % nc), Z = (int)(cid / ((long long)nc * nc));
  const int nt = nf + 2 * ng, ntv = nt + 1;
  const long long fcell = (long long)nt * nt * nt, fface = (long long)ntv * ntv * ntv;
  auto ci = [&](int k, int j, int i) { return ((long long)k * nt + j) * nt + i; };
  auto fi = [&](int k, int j, int i) { return ((long long)k * ntv + j) * ntv + i; };
  const double g1 = gamma - 1.0;
  double U[5] = {0, 0, 0, 0, 0};
  // face extrapolation weights of the fine layers along d (offset 0..r-1)
  const double wo = (r > 1) ? 1.5 : 1.0, wi = (r > 1) ? -0.5 : 0.0;
  double first[3][8], last[3][8];
  for (int d = 0; d < 3; d++)
    for (int n = 0; n < 8; n++) first[d][n] = last[d][n] = 0.0;
  for (int a = 0; a < r; a++)
    for (int b = 0; b < r; b++)
      for (int c = 0; c < r; c++) {
        const int k = ng + Z * r + a, j = ng + Y * r + b, i = ng + X * r + c;
        const long long q = ci(k, j, i);
        double V[8];
        for (int n = 0; n < 8; n++) V[n] = Vc[n * fcell + q];
        const double v2 = V[1] * V[1] + V[2] * V[2] + V[3] * V[3];
        const double b2 = V[5] * V[5] + V[6] * V[6] + V[7] * V[7];
        U[0] += V[0];
        U[1] += V[0] * V[1];
        U[2] += V[0] * V[2];
        U[3] += V[0] * V[3];
        U[4] += V[4] / g1 + 0.5 * V[0] * v2 + 0.5 * b2;
        const int off[3] = {c, b, a};
        for (int d = 0; d < 3; d++) {
          const double w0 = (off[d] == 0) ? wo : ((off[d] == 1 && r > 1) ? wi : 0.0);
          const double w1 = (off[d] == r - 1) ? wo : ((off[d] == r - 2 && r > 1) ? wi : 0.0);
          if (w0 != 0.0)
            for (int n = 0; n < 8; n++) first[d][n] += w0 * V[n];
          if (w1 != 0.0)
            for (int n = 0; n < 8; n++) last[d][n] += w1 * V[n];
        }
      }
  const double inv3 = 1.0 / ((double)r * r * r), inv2 = 1.0 / ((double)r * r);
  for (int n = 0; n < 5; n++) U[n] *= inv3;
  double Bf[3][2];
  for (int d = 0; d < 3; d++) {
    const double* vs = Vs + d * fface;
    for (int side = 0; side < 2; side++) {
      double s = 0.0;
      for (int a = 0; a < r; a++)
        for (int b = 0; b < r; b++) {
          int k, j, i;
          if (d == 0) {
            i = ng + (X + side) * r; j = ng + Y * r + b; k = ng + Z * r + a;
          } else if (d == 1) {
            j = ng + (Y + side) * r; i = ng + X * r + b; k = ng + Z * r + a;
          } else {
            k = ng + (Z + side) * r; i = ng + X * r + b; j = ng + Y * r + a;
          }
          s += vs[fi(k, j, i)];
        }
      Bf[d][side] = s * inv2;
    }
    faces[d * ncell_c + cid] = Bf[d][0];
  }
  double P[8];
  P[0] = U[0];
  for (int d = 0; d < 3; d++) P[1 + d] = U[1 + d] / U[0];
  for (int d = 0; d < 3; d++) P[5 + d] = 0.5 * (Bf[d][0] + Bf[d][1]);
  P[4] = g1 * (U[4] - 0.5 * U[0] * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]) -
               0.5 * (P[5] * P[5] + P[6] * P[6] + P[7] * P[7]));
  for (int n = 0; n < 8; n++) prim[n * ncell_c + cid] = P[n];
  for (int d = 0; d < 3; d++)
    for (int rv = 0; rv < 8; rv++) {
      const int sv = rot_var(rv, d);
      tgt[((long long)d * 16 + rv) * ncell_c + cid] = first[d][sv] * inv2;
      tgt[((long long)d * 16 + 8 + rv) * ncell_c + cid] = last[d][sv] * inv2;
    }
}

// order-preserving map of floats to unsigned keys (atomic min / max)
__device__ __forceinline__ unsigned fkey(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ inline float fkey_inv(unsigned k) {
  const unsigned b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  memcpy(&f, &b, sizeof(f));
  return f;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float vanleer_f(float dvp, float dvm) {
  return dvp * dvm > 0.f ? 2.f * dvp * dvm / (dvp + dvm) : 0.f;
}

// Batch assembly: sample i of the batch picks (snapshot, cell, direction)
// from a counter-based hash; X = BF16 stencil features (K1 columns, the last
// zero), T = normalised correction targets.  Optionally widens the trained
// feature range.  prims/tgt: FP32 [S][8][nc^3] and [S][3][16][nc^3].
__global__ void k_make_batch(const float* __restrict__ prims, const float* __restrict__ tgt, int S, int nc,
                             float gamma, unsigned long long seed, long long base, int B,
                             __nv_bfloat16* __restrict__ X, float* __restrict__ T, unsigned* __restrict__ kmin,
                             unsigned* __restrict__ kmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const long long ncell = (long long)nc * nc * nc;
  const unsigned long long h = mix64(seed ^ mix64((unsigned long long)(base + i)));
  const int snap = (int)(h % (unsigned long long)S);
  const long long cell = (long long)((h >> 16) % (unsigned long long)ncell);
  const int d = (int)((h >> 48) % 3ull);
  const float* P = prims + (long long)snap * 8 * ncell;
  const int cx[3] = {(int)(cell % nc), (int)((cell / nc) % nc), (int)(cell / ((long long)nc * nc))};
  auto at = [&](int rv, int o0, int o1, int o2) {
    int q[3] = {cx[0], cx[1], cx[2]};
    q[d] = (q[d] + o0 + nc) % nc;
    q[(d + 1) % 3] = (q[(d + 1) % 3] + o1 + nc) % nc;
    q[(d + 2) % 3] = (q[(d + 2) % 3] + o2 + nc) % nc;
    return P[rot_var(rv, d) * ncell + ((long long)q[2] * nc + q[1]) * nc + q[0]];
  };
  float cen[8];
  for (int rv = 0; rv < 8; rv++) cen[rv] = at(rv, 0, 0, 0);
  const float rho_c = cen[0], p_c = cen[4];
  const float cs = sqrtf(gamma * p_c / rho_c), sb = sqrtf(rho_c) * cs;
  const float sc[8] = {rho_c, cs, cs, cs, p_c, sb, sb, sb};
  __nv_bfloat16* xr = X + (long long)i * K1;
  for (int rv = 0; rv < 8; rv++)
    for (int o2 = -1; o2 <= 1; o2++)
      for (int o1 = -1; o1 <= 1; o1++)
        for (int o0 = -1; o0 <= 1; o0++) {
          const float s = at(rv, o0, o1, o2);
          float f;
          if (rv == 0 || rv == 4) f = s / cen[rv] - 1.f;
          else if (rv < 4) f = (s - cen[rv]) / cs;
          else f = s / sb;
          const int col = rv * 27 + (o2 + 1) * 9 + (o1 + 1) * 3 + (o0 + 1);
          xr[col] = __float2bfloat16(f);
          if (kmin) {
            atomicMin(kmin + col, fkey(f));
            atomicMax(kmax + col, fkey(f));
          }
        }
  for (int col = NIN; col < K1; col++) xr[col] = __float2bfloat16(0.f);
  const float* tg = tgt + ((long long)snap * 3 + d) * 16 * ncell + cell;
  for (int rv = 0; rv < 8; rv++) {
    const float w0 = at(rv, -1, 0, 0), w1 = cen[rv], w2 = at(rv, 1, 0, 0);
    const float dd = vanleer_f(w2 - w1, w1 - w0);
    T[(long long)i * NOUT + rv] = (tg[rv * ncell] - (w1 - 0.5f * dd)) / sc[rv];
    T[(long long)i * NOUT + 8 + rv] = (tg[(8 + rv) * ncell] - (w1 + 0.5f * dd)) / sc[rv];
  }
}

// ---------------------------------------------------------------------------
// Learned sweep (ORDER 5): reconstruction with the network's correction,
// Riemann solve and flux difference of one direction in one kernel, over
// tiles of 128 cells laid along the sweep's pencils (lines of cells along
// DIR: the active cells plus one ghost cell at each end, for every column
// of the other two directions including the CT extension).  Per tile:
//   1. stencil features of the 128 cells (BF16, canonical K-major layout);
//   2. the three layers on the 5th-generation tensor cores - one thread
//      issues tcgen05.mma over the shared-memory operands, the FP32
//      accumulators live in tensor memory, the epilogues (bias, SiLU) read
//      them back with tcgen05.ld and write the next layer's operand;
//   3. each cell's PLM (van Leer) states plus the correction, or the plain
//      PLM states where the stencil is outside the trained feature range or
//      a corrected density / pressure is not positive (the cell's two faces
//      together), kept in shared memory;
//   4. the HLLD solve of every face between two cells of the tile, its EMF
//      outputs, and the flux difference of every cell with both faces in the
//      tile (the march's expressions, so that with a zero correction the
//      sweep is bit-identical to the plain PLM march).
// Pencils of up to 128 cells are packed whole into a tile; longer pencils
// are cut into segments of 128 cells that overlap by two (the face between
// them is solved by both, with the same result).  Persistent CTAs of 256
// threads, the BF16 weights resident in shared memory.  With states != null
// the kernel writes the face states ([3][16][ncell]: direction, face
// (minus / plus) x variable) and stops before the Riemann solves.
// ---------------------------------------------------------------------------
constexpr int LT = 128;  // cells (rows) per tile
constexpr size_t LS_W1 = 0;                                  // W1: N 128 x K 224
constexpr size_t LS_W2 = LS_W1 + (size_t)NH * K1 * 2;        // W2: 128 x 128
constexpr size_t LS_W3 = LS_W2 + (size_t)NH * NH * 2;        // W3: 16 x 128
constexpr size_t LS_X = LS_W3 + (size_t)NOUT * NH * 2;       // features 128 x 224 (reused)
constexpr size_t LS_H = LS_X + (size_t)LT * K1 * 2;          // layer-1 output 128 x 128
constexpr size_t LS_B = LS_H + (size_t)LT * NH * 2;          // biases
constexpr size_t LS_R = LS_B + (size_t)(2 * NH + NOUT) * 4;  // trained range
constexpr size_t LS_F = LS_R + (size_t)2 * NIN * 4;          // per-row fallback flags
constexpr size_t LS_M = LS_F + (size_t)LT * 4;               // counter, mbarrier, TMEM slot
constexpr size_t SM_LEARN = LS_M + 32;
// inside the feature region once the network is done with it
constexpr size_t LX_Y = 0;                                   // outputs 128 x 16 FP32
constexpr size_t LX_S = LX_Y + (size_t)LT * NOUT * 4;        // face states 128 x 2 x 8 FP64
constexpr size_t LX_FA = LX_S + (size_t)LT * 16 * 8;         // flux x area 128 x 5 FP64
constexpr size_t LX_CM = LX_FA + (size_t)LT * 5 * 8;         // wave speed 128 FP64
static_assert(LX_CM + (size_t)LT * 8 <= (size_t)LT * K1 * 2, "tile outputs exceed the feature region");
static_assert(LS_X % 128 == 0 && LS_H % 128 == 0 && LS_W2 % 128 == 0 && LS_W3 % 128 == 0, "operand alignment");
static_assert(SM_LEARN <= 227 * 1024, "learned sweep does not fit in shared memory");

struct LearnedDev {
  const __nv_bfloat16* W1b;  // [K1][NH]
  const __nv_bfloat16* W2b;  // [NH][NH]
  const __nv_bfloat16* W3b;  // [NH][NOUT]
  const float* w;            // packed FP32 parameters (biases)
  const float* fmin;         // [NIN] trained feature range, or null
  const float* fmax;
};

// tiling of one direction's pencils into tiles of LT cells
struct LTiles {
  int L;              // cells per pencil: n[DIR] + 2
  int per_tile;       // pencils per tile when L <= LT, else 0
  int nseg;           // segments of LT cells per pencil when L > LT
  int nA;             // pencils along the first transverse direction (with the CT extension)
  long long npencil;  // pencils
  long long ntiles;
};

__host__ inline LTiles make_tiles(const Geo& g, int dir) {
  const int A = (dir == 0) ? 1 : 0, B = (dir == 2) ? 1 : 2;
  LTiles t{};
  t.L = g.n[dir] + 2;
  t.nA = g.n[A] + 2 * g.ext;
  t.npencil = (long long)t.nA * (g.n[B] + 2 * g.ext);
  if (t.L <= LT) {
    t.per_tile = LT / t.L;
    t.nseg = 1;
    t.ntiles = (t.npencil + t.per_tile - 1) / t.per_tile;
  } else {
    t.per_tile = 0;
    t.nseg = (t.L - 2 + (LT - 2) - 1) / (LT - 2);
    t.ntiles = t.npencil * t.nseg;
  }
  return t;
}

// element (r, k) of a BF16 operand tile with K columns
__device__ __forceinline__ void put_bf16(unsigned char* base, int r, int k, int K, float v) {
  reinterpret_cast<__nv_bfloat16*>(base)[umma::kmajor_offset(r, k, K) / 2] = __float2bfloat16(v);
}

template <int DIR>
__global__ void __launch_bounds__(256, 1) k_learned_sweep(Geo g, Fields f, LearnedDev L, const Ctl* ctl, LTiles T,
                                                          int invdt, int last_dir, double* __restrict__ states,
                                                          unsigned long long* __restrict__ counters) {
  if (ctl->done) return;
  constexpr int A = (DIR == 0) ? 1 : 0, B = (DIR == 2) ? 1 : 2;
  using v = Var<3>;
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned char* W1s = sm + LS_W1;
  unsigned char* W2s = sm + LS_W2;
  unsigned char* W3s = sm + LS_W3;
  unsigned char* Xs = sm + LS_X;
  unsigned char* Hs = sm + LS_H;
  float* bs = reinterpret_cast<float*>(sm + LS_B);
  float* rmin = reinterpret_cast<float*>(sm + LS_R);
  float* rmax = rmin + NIN;
  int* flag = reinterpret_cast<int*>(sm + LS_F);
  int* nfall = reinterpret_cast<int*>(sm + LS_M);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + LS_M + 8);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + LS_M + 16);
  float* Ys = reinterpret_cast<float*>(Xs + LX_Y);
  double* FS = reinterpret_cast<double*>(Xs + LX_S);
  double* FA = reinterpret_cast<double*>(Xs + LX_FA);
  double* CM = reinterpret_cast<double*>(Xs + LX_CM);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights as the B operands (N x K, K-major): element (n, k) of layer l
  for (int e = tid; e < K1 * NH; e += blockDim.x) {
    const int k = e / NH, n = e % NH;
    reinterpret_cast<__nv_bfloat16*>(W1s)[umma::kmajor_offset(n, k, K1) / 2] = L.W1b[e];
  }
  for (int e = tid; e < NH * NH; e += blockDim.x) {
    const int k = e / NH, n = e % NH;
    reinterpret_cast<__nv_bfloat16*>(W2s)[umma::kmajor_offset(n, k, NH) / 2] = L.W2b[e];
  }
  for (int e = tid; e < NH * NOUT; e += blockDim.x) {
    const int k = e / NOUT, n = e % NOUT;
    reinterpret_cast<__nv_bfloat16*>(W3s)[umma::kmajor_offset(n, k, NH) / 2] = L.W3b[e];
  }
  for (int e = tid; e < NH; e += blockDim.x) {
    bs[e] = L.w[OB1 + e];
    bs[NH + e] = L.w[OB2 + e];
  }
  if (tid < NOUT) bs[2 * NH + tid] = L.w[OB3 + tid];
  const bool ranged = L.fmin != nullptr;
  for (int e = tid; e < NIN; e += blockDim.x) {
    rmin[e] = ranged ? L.fmin[e] : 0.f;
    rmax[e] = ranged ? L.fmax[e] : 0.f;
  }
  if (warp == 0) umma::tmem_alloc(slot, 256);  // layer 1: columns 0-127, layer 2: 128-255, layer 3: 0-15
  if (tid == 0) umma::mbar_init1(bar);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *slot;
  uint32_t phase = 0;
  bool ok = true;
  const int row = tid & (LT - 1), half = tid >> 7;
  const int a1 = (DIR + 1) % 3, a2 = (DIR + 2) % 3;
  const long long sd = g.s[DIR], s1 = g.s[a1], s2 = g.s[a2];
  const double dtdV = ctl->dtdV;
  const double areaT = g.A[DIR];
  double run_max = 0.0;  // max of InvDt over this thread's cells
  // one MMA run of a layer, then every thread waits (bounded) for it
  auto layer = [&](uint32_t d_col, const unsigned char* a, const unsigned char* b, int K, int N) {
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      umma::mma_tile(tmem + d_col, umma::smem_addr(a), umma::smem_addr(b), K, umma::idesc_bf16_f32(LT, N), false);
      umma::mma_commit(bar);
    }
    const bool w = umma::mbar_wait_bounded(bar, phase, umma::kMmaSpin);
    phase ^= 1u;
    ok = __syncthreads_and(w) != 0;
    umma::fence_after_sync();
  };
  // hidden-layer epilogue: SiLU(acc + bias) -> BF16 operand of the next layer
  // (warp w: rows 32 (w % 4) .., columns 64 (w / 4) ..)
  auto hidden = [&](uint32_t d_col, const float* bias, unsigned char* out) {
    const int r = 32 * (warp & 3) + lane, c0 = 64 * (warp >> 2);
    for (int c = c0; c < c0 + 64; c += 16) {
      float x[16];
      umma::tmem_ld16(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + d_col + (uint32_t)c, x);
#pragma unroll
      for (int i = 0; i < 16; i++) put_bf16(out, r, c + i, NH, silu_f(x[i] + bias[c + i]));
    }
  };
  for (long long tile = blockIdx.x; tile < T.ntiles && ok; tile += gridDim.x) {
    // ---- this thread's row: pencil, cell along DIR, segment ends --------
    long long pencil;
    int pos;
    bool valid, first, last;
    if (T.per_tile) {
      const int q = row / T.L;
      pos = row - q * T.L;
      pencil = tile * T.per_tile + q;
      valid = q < T.per_tile && pencil < T.npencil;
      first = pos == 0;
      last = pos == T.L - 1;
    } else {
      pencil = tile / T.nseg;
      pos = (int)(tile % T.nseg) * (LT - 2) + row;
      valid = pos < T.L;
      first = row == 0;
      last = row == LT - 1 || pos == T.L - 1;
    }
    if (!valid) {
      pencil = 0;
      pos = 1;
    }
    int ix[3];
    ix[DIR] = g.beg[DIR] - 1 + pos;
    ix[A] = g.beg[A] - g.ext + (int)(pencil % T.nA);
    ix[B] = g.beg[B] - g.ext + (int)(pencil / T.nA);
    const bool active_col = ix[A] >= g.beg[A] && ix[A] < g.end[A] && ix[B] >= g.beg[B] && ix[B] < g.end[B];
    const long long cc = cidx(g, ix[2], ix[1], ix[0]);
    if (tid < LT) flag[tid] = valid ? 0 : 1;
    if (tid == 0) *nfall = 0;
    __syncthreads();
    // ---- 1. stencil features (half 0: rotated variables 0-3, half 1: 4-7)
    {
      float cen[8];
#pragma unroll
      for (int rv = 0; rv < 8; rv++) cen[rv] = (float)f.Vc[rot_var(rv, DIR) * g.ncell + cc];
      const float cs = sqrtf((float)g.gamma * cen[4] / cen[0]), sb = sqrtf(cen[0]) * cs;
      int bad = 0;
      for (int q = 0; q < 4; q++) {
        const int rv = half * 4 + q;
        const double* base = f.Vc + rot_var(rv, DIR) * g.ncell + cc;
        for (int o2 = -1; o2 <= 1; o2++)
          for (int o1 = -1; o1 <= 1; o1++)
            for (int o0 = -1; o0 <= 1; o0++) {
              const float sv = valid ? (float)base[o0 * sd + o1 * s1 + o2 * s2] : 0.f;
              float x;
              if (rv == 0 || rv == 4) x = sv / cen[rv] - 1.f;
              else if (rv < 4) x = (sv - cen[rv]) / cs;
              else x = sv / sb;
              const int col = rv * 27 + (o2 + 1) * 9 + (o1 + 1) * 3 + (o0 + 1);
              if (!valid) x = 0.f;
              if (ranged && !(x >= rmin[col] && x <= rmax[col])) bad = 1;
              put_bf16(Xs, row, col, K1, x);
            }
      }
      if (half == 1)
        for (int col = NIN; col < K1; col++) put_bf16(Xs, row, col, K1, 0.f);
      if (bad) atomicOr(flag + row, 1);
    }
    // ---- 2. the network on the tensor cores -----------------------------
    layer(0, Xs, W1s, K1, NH);  // layer 1 -> TMEM columns 0-127
    if (!ok) break;
    hidden(0, bs, Hs);
    layer(NH, Hs, W2s, NH, NH);  // layer 2 -> TMEM columns 128-255
    if (!ok) break;
    hidden(NH, bs + NH, Xs);     // layer-2 output over the features
    layer(0, Xs, W3s, NH, NOUT);  // layer 3 -> TMEM columns 0-15
    if (!ok) break;
    if (warp < 4) {
      float y[16];
      umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), y);
#pragma unroll
      for (int i = 0; i < 16; i++) Ys[row * NOUT + i] = y[i] + bs[2 * NH + i];
    }
    __syncthreads();
    // ---- 3. corrected face states (thread: cell row, face = half) -------
    {
      double cen[8], vl[8], vr[8], st[8];
      const double dxd = g.dx[DIR];
#pragma unroll
      for (int sv = 0; sv < 8; sv++) {
        const double* base = f.Vc + sv * g.ncell + cc;
        double w[3];
        w[0] = valid ? base[-sd] : 1.0;
        w[1] = valid ? base[0] : 1.0;
        w[2] = valid ? base[sd] : 1.0;
        cen[sv] = w[1];
        Recon<2>::cell<double>(w, dxd, sv == 0 || sv == 4, vl[sv], vr[sv]);
      }
      const double cs = sqrt(g.gamma * cen[4] / cen[0]), sb = sqrt(cen[0]) * cs;
      const double sc[8] = {cen[0], cs, cs, cs, cen[4], sb, sb, sb};
#pragma unroll
      for (int rv = 0; rv < 8; rv++) {
        const int sv = rot_var(rv, DIR);
        const double plm = half ? vr[sv] : vl[sv];
        st[sv] = plm;
        if (rv == 5) continue;  // normal field: the face value is used
        st[sv] = plm + (double)Ys[row * NOUT + half * 8 + rv] * sc[rv];
      }
      if (!(st[0] > 0.0) || !(st[4] > 0.0)) atomicOr(flag + row, 1);
      __syncthreads();
      const bool fall = flag[row] != 0;
      if (fall) {
#pragma unroll
        for (int sv = 0; sv < 8; sv++) st[sv] = half ? vr[sv] : vl[sv];
      }
#pragma unroll
      for (int sv = 0; sv < 8; sv++) FS[(row * 2 + half) * 8 + sv] = st[sv];
      if (valid && states) {
#pragma unroll
        for (int sv = 0; sv < 8; sv++) states[((long long)DIR * 16 + half * 8 + sv) * g.ncell + cc] = st[sv];
      }
      if (valid && half == 0 && fall) atomicAdd(nfall, 1);
    }
    __syncthreads();
    if (tid == 0 && counters) {
      long long nvalid;
      if (T.per_tile) {
        const long long left = T.npencil - tile * T.per_tile;
        nvalid = (long long)T.L * (left < T.per_tile ? left : T.per_tile);
      } else {
        const long long p0 = (tile % T.nseg) * (LT - 2);
        nvalid = (T.L - p0 < LT) ? (T.L - p0) : LT;
      }
      atomicAdd(counters, (unsigned long long)nvalid);
      atomicAdd(counters + 1, (unsigned long long)*nfall);
    }
    if (states) continue;
    // ---- 4. Riemann solve of the face between this row and the next -----
    if (tid < LT && valid && !last) {
      double vL[8], vR[8];
#pragma unroll
      for (int n = 0; n < 8; n++) {
        vL[n] = FS[(row * 2 + 1) * 8 + n];        // plus-face state of this cell
        vR[n] = FS[((row + 1) * 2 + 0) * 8 + n];  // minus-face state of the next
      }
      int jx[3] = {ix[0], ix[1], ix[2]};
      jx[DIR] += 1;
      const long long cn = cidx(g, jx[2], jx[1], jx[0]);  // the face is the next cell's minus face
      const double bn = f.Vs[DIR * g.nface + fidx(g, jx[2], jx[1], jx[0])];
      vL[v::BX1 + DIR] = bn;
      vR[v::BX1 + DIR] = bn;
      RiemannOut<3, double> r;
      riemann<3, DIR, kHLLD>(g.gamma, g.rgm1, vL, vR, r);
      store_emf<3, DIR>(g, f, cn, r, vL, vR);
      if (active_col) {
#pragma unroll
        for (int n = 0; n < v::BX1; n++) FA[row * 5 + n] = r.F[n] * areaT;
        CM[row] = r.cmax;
      }
    }
    __syncthreads();
    // ---- flux difference of the cells with both faces in the tile -------
    if (tid < LT && valid && !first && !last && active_col) {
#pragma unroll
      for (int n = 0; n < v::BX1; n++) {
        const double rhs = -dtdV * (FA[row * 5 + n] - FA[(row - 1) * 5 + n]);
        f.Uc[n * g.ncell + cc] = f.Uc[n * g.ncell + cc] + rhs;
      }
      if (invdt) {
        const double prev = (invdt == 1) ? 0.0 : f.InvDt[cc];
        const double inv = prev + div_r(0.5 * (CM[row] + CM[row - 1]), Recip{g.dx[DIR], g.rdx[DIR]});
        f.InvDt[cc] = inv;
        if (inv > run_max) run_max = inv;  // NaN never compares greater
      }
    }
    __syncthreads();  // the feature region is rewritten by the next tile
  }
  if (!ok && tid == 0) report_wait_timeout(ctl);
  if (last_dir && invdt && !states) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, run_max, o);
      if (w > run_max) run_max = w;
    }
    if (lane == 0 && run_max > 0.0) atomic_max_pos((unsigned long long*)&((Ctl*)ctl)->invdt_max_bits, run_max);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

__global__ void k_sumsq_targets(const float* __restrict__ T, int B, double* __restrict__ out) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (e < (long long)B * NOUT && !loss_masked((int)(e % NOUT))) l = (double)T[e] * T[e] / B;
  for (int w = 16; w > 0; w >>= 1) l += __shfl_down_sync(0xffffffffu, l, w);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(out, l);
}

__global__ void k_init_keys(unsigned* kmin, unsigned* kmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NIN) {
    kmin[i] = 0xffffffffu;
    kmax[i] = 0u;
  }
}

// ---------------------------------------------------------------------------
// Self-check of the tcgen05 building blocks (umma.cuh): one CTA of 128
// threads computes D[128][N] = A[128][K] . B[N][K]^T with BF16 operands staged
// in the canonical K-major layout, the FP32 accumulator in TMEM, and writes D
// from TMEM to global memory.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 1) k_umma_check(int N, int K, const __nv_bfloat16* __restrict__ A,
                                                       const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                       int* status) {
  extern __shared__ __align__(128) unsigned char sm[];
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(sm);
  __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(sm + 128 * K * 2);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 128 * K * 2 + N * K * 2);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < 128 * K; e += blockDim.x)
    As[umma::kmajor_offset(e / K, e % K, K) / 2] = A[e];
  for (int e = tid; e < N * K; e += blockDim.x)
    Bs[umma::kmajor_offset(e / K, e % K, K) / 2] = B[e];
  uint32_t ncols = 32;
  while ((int)ncols < N) ncols *= 2;
  if (warp == 0) umma::tmem_alloc(slot, ncols);
  if (tid == 0) umma::mbar_init1(bar);
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t taddr = *slot;
  if (tid == 0) {
    umma::mma_tile(taddr, umma::smem_addr(As), umma::smem_addr(Bs), K, umma::idesc_bf16_f32(128, N), false);
    umma::mma_commit(bar);
  }
  const bool ok = umma::mbar_wait_bounded(bar, 0, umma::kMmaSpin);
  umma::fence_after_sync();
  if (ok) {
    const int row = 32 * warp + lane;
    for (int c = 0; c < N; c += 16) {
      float v[16];
      umma::tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) D[row * N + c + i] = v[i];
    }
  } else if (lane == 0) {
    atomicExch(status, 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(taddr, ncols);
}

}  // namespace

// the network as the engine holds it (ORDER 5)
struct LearnedModel {
  __nv_bfloat16 *W1b = nullptr, *W2b = nullptr, *W3b = nullptr;
  float* w = nullptr;
  float *fmin = nullptr, *fmax = nullptr;
  unsigned long long* counters = nullptr;
  bool ranged = false;
};

namespace idfx {

// the learned sweeps of one stage, direction after direction (the same
// InvDt modes as the march: 1 first contribution, 2 accumulate; the last
// direction folds the CFL maximum); states: face states instead (see
// k_learned_sweep)
static void launch_learned(Engine& e, int invdt, int fold_max, double* states) {
  LearnedModel* m = static_cast<LearnedModel*>(e.learned);
  LearnedDev L{m->W1b, m->W2b, m->W3b, m->w, m->ranged ? m->fmin : nullptr, m->ranged ? m->fmax : nullptr};
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int d = 0; d < 3; d++) {
    if (e.only_dir >= 0 && e.only_dir != d) continue;
    const LTiles T = make_tiles(e.g, d);
    const int grid = (int)(T.ntiles < sms ? T.ntiles : sms);
    const int inv = (invdt == 0) ? 0 : (d == 0 ? invdt : 2);
    const int last = fold_max && d == 2;
    mark_begin(e, kKSweepX + d);
    if (d == 0) k_learned_sweep<0><<<grid, 256, SM_LEARN, e.stream>>>(e.g, e.f, L, e.ctl, T, inv, last, states, m->counters);
    if (d == 1) k_learned_sweep<1><<<grid, 256, SM_LEARN, e.stream>>>(e.g, e.f, L, e.ctl, T, inv, last, states, m->counters);
    if (d == 2) k_learned_sweep<2><<<grid, 256, SM_LEARN, e.stream>>>(e.g, e.f, L, e.ctl, T, inv, last, states, m->counters);
    mark_end(e);
  }
}

void launch_learned_sweeps(Engine& e, int invdt, int fold_max) { launch_learned(e, invdt, fold_max, nullptr); }

void free_learned(Engine& e) {
  LearnedModel* m = static_cast<LearnedModel*>(e.learned);
  if (!m) return;
  cudaFree(m->W1b);
  cudaFree(m->W2b);
  cudaFree(m->W3b);
  cudaFree(m->w);
  cudaFree(m->fmin);
  cudaFree(m->fmax);
  cudaFree(m->counters);
  delete m;
  e.learned = nullptr;
}

}  // namespace idfx

// trainer state
struct idfx_mlp {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int max_batch = 0;
  long long t = 0;  // Adam steps taken
  float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16 *W1b = nullptr, *W2b = nullptr, *W3b = nullptr;
  __nv_bfloat16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dYb = nullptr, *dZ2b = nullptr, *dZ1b = nullptr;
  float *T = nullptr, *Z1 = nullptr, *Z2 = nullptr, *Y = nullptr, *dYf = nullptr, *dZ2f = nullptr, *dZ1f = nullptr;
  double* loss = nullptr;
  unsigned *kmin = nullptr, *kmax = nullptr;
  int* status = nullptr;  // set by a GEMM whose bounded tensor-core wait gave up
  float* ws = nullptr;    // split-K partial products of the weight-gradient GEMMs
  const float* prims = nullptr;
  const float* tgt = nullptr;
  int nsnap = 0, nc = 0;
  double gamma = 5.0 / 3.0;
  std::vector<void*> allocs;
};

namespace {

template <typename P>
bool dalloc(idfx_mlp* h, P** p, size_t n) {
  if (cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(P)) != cudaSuccess) return false;
  h->allocs.push_back(*p);
  return cudaMemsetAsync(*p, 0, n * sizeof(P), h->stream) == cudaSuccess;
}

// forward + loss + backward of one batch held in h->X / h->T (loss added to *loss)
void fwd_bwd(idfx_mlp* h, int B, double* loss) {
  cudaStream_t s = h->stream;
  gemm(s, B, NH, K1, h->X, K1, 0, h->W1b, NH, 0, EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH}, h->status, h->ws);
  gemm(s, B, NH, NH, h->H1, NH, 0, h->W2b, NH, 0, EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH}, h->status, h->ws);
  gemm(s, B, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0, EpiArgs{kEpiBias, h->w + OB3, nullptr, h->Y, nullptr, NOUT}, h->status, h->ws);
  const int ne = B * NOUT;
  k_loss<<<(ne + 255) / 256, 256, 0, s>>>(h->Y, h->T, B, h->dYf, h->dYb, loss);
  gemm(s, NH, NOUT, B, h->H2, NH, 1, h->dYb, NOUT, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW3, nullptr, NOUT}, h->status, h->ws);
  k_colsum<<<NOUT, 256, 0, s>>>(h->dYf, B, NOUT, h->g + OB3);
  gemm(s, B, NH, NOUT, h->dYb, NOUT, 0, h->W3b, NOUT, 1, EpiArgs{kEpiDsilu, nullptr, h->Z2, h->dZ2f, h->dZ2b, NH}, h->status, h->ws);
  gemm(s, NH, NH, B, h->H1, NH, 1, h->dZ2b, NH, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW2, nullptr, NH}, h->status, h->ws);
  k_colsum<<<NH, 256, 0, s>>>(h->dZ2f, B, NH, h->g + OB2);
  gemm(s, B, NH, NH, h->dZ2b, NH, 0, h->W2b, NH, 1, EpiArgs{kEpiDsilu, nullptr, h->Z1, h->dZ1f, h->dZ1b, NH}, h->status, h->ws);
  gemm(s, NIN, NH, B, h->X, K1, 1, h->dZ1b, NH, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW1, nullptr, NH}, h->status, h->ws);
  k_colsum<<<NH, 256, 0, s>>>(h->dZ1f, B, NH, h->g + OB1);
}

int sync_ok(idfx_mlp* h) {
  if (cudaGetLastError() != cudaSuccess) return IDFX_ERR_CUDA;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return IDFX_ERR_CUDA;
  if (h->status) {  // a bounded tensor-core wait that gave up
    int st = 0;
    if (cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess || st) return IDFX_ERR_CUDA;
  }
  return IDFX_OK;
}

}  // namespace

extern "C" {

int idfx_gpu_set_learned(idfx_gpu* hg, const float* params, const float* fmin, const float* fmax) {
  if (!hg || !params) return IDFX_ERR_STATE;
  Engine& e = hg->e;
  if (e.g.order != IDFX_LEARNED) {
    e.err = "set_learned: the handle was not created with the learned reconstruction order";
    return IDFX_ERR_CONFIG;
  }
  if (cudaStreamSynchronize(e.stream) != cudaSuccess) return IDFX_ERR_CUDA;
  if (!e.learned) {
    LearnedModel* m = new (std::nothrow) LearnedModel();
    if (!m) return IDFX_ERR_STATE;
    e.learned = m;
    bool ok = cudaMalloc(&m->W1b, sizeof(__nv_bfloat16) * K1 * NH) == cudaSuccess;
    ok = ok && cudaMalloc(&m->W2b, sizeof(__nv_bfloat16) * NH * NH) == cudaSuccess;
    ok = ok && cudaMalloc(&m->W3b, sizeof(__nv_bfloat16) * NH * NOUT) == cudaSuccess;
    ok = ok && cudaMalloc(&m->w, sizeof(float) * NPARAM) == cudaSuccess;
    ok = ok && cudaMalloc(&m->fmin, sizeof(float) * NIN) == cudaSuccess;
    ok = ok && cudaMalloc(&m->fmax, sizeof(float) * NIN) == cudaSuccess;
    ok = ok && cudaMalloc(&m->counters, sizeof(unsigned long long) * 2) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_learned_sweep<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)SM_LEARN) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_learned_sweep<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)SM_LEARN) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_learned_sweep<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)SM_LEARN) == cudaSuccess;
    if (!ok) {
      free_learned(e);
      e.err = "set_learned: CUDA allocation failed";
      return IDFX_ERR_CUDA;
    }
  }
  LearnedModel* m = static_cast<LearnedModel*>(e.learned);
  m->ranged = fmin && fmax;
  bool ok = cudaMemcpyAsync(m->w, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, e.stream) == cudaSuccess;
  if (m->ranged) {
    ok = ok && cudaMemcpyAsync(m->fmin, fmin, sizeof(float) * NIN, cudaMemcpyHostToDevice, e.stream) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(m->fmax, fmax, sizeof(float) * NIN, cudaMemcpyHostToDevice, e.stream) == cudaSuccess;
  }
  ok = ok && cudaMemsetAsync(m->counters, 0, sizeof(unsigned long long) * 2, e.stream) == cudaSuccess;
  if (!ok) return IDFX_ERR_CUDA;
  k_refresh_bf16<<<(K1 * NH + 255) / 256, 256, 0, e.stream>>>(m->w, m->W1b, m->W2b, m->W3b);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(e.stream) != cudaSuccess) return IDFX_ERR_CUDA;
  return IDFX_OK;
}

int idfx_gpu_learned_states(idfx_gpu* hg, double* ls) {
  if (!hg || !ls || !hg->e.learned) return IDFX_ERR_STATE;
  Engine& e = hg->e;
  if (idfx_gpu_set_boundaries(hg) != IDFX_OK) return IDFX_ERR_CUDA;
  const size_t n = (size_t)48 * e.g.ncell;
  double* tmp = nullptr;
  if (cudaMalloc(&tmp, n * sizeof(double)) != cudaSuccess) return IDFX_ERR_CUDA;
  bool ok = cudaMemsetAsync(tmp, 0, n * sizeof(double), e.stream) == cudaSuccess;
  if (ok) {
    launch_learned(e, 0, 0, tmp);
    ok = cudaGetLastError() == cudaSuccess;
  }
  ok = ok && cudaMemcpyAsync(ls, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, e.stream) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(e.stream) == cudaSuccess;
  cudaFree(tmp);
  return ok ? IDFX_OK : IDFX_ERR_CUDA;
}

int idfx_gpu_learned_stats(idfx_gpu* hg, long long* cells, long long* fallbacks) {
  if (!hg || !hg->e.learned) return IDFX_ERR_STATE;
  Engine& e = hg->e;
  unsigned long long c[2];
  LearnedModel* m = static_cast<LearnedModel*>(e.learned);
  if (cudaMemcpyAsync(c, m->counters, sizeof(c), cudaMemcpyDeviceToHost, e.stream) != cudaSuccess ||
      cudaStreamSynchronize(e.stream) != cudaSuccess)
    return IDFX_ERR_CUDA;
  if (cells) *cells = (long long)c[0];
  if (fallbacks) *fallbacks = (long long)c[1];
  return IDFX_OK;
}

int idfx_check_umma(int N, int K, const float* A, const float* B, float* D) {
  if (!A || !B || !D || N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16) return IDFX_ERR_CONFIG;
  std::vector<__nv_bfloat16> a((size_t)128 * K), b((size_t)N * K);
  for (size_t i = 0; i < a.size(); i++) a[i] = __float2bfloat16(A[i]);
  for (size_t i = 0; i < b.size(); i++) b[i] = __float2bfloat16(B[i]);
  __nv_bfloat16 *da = nullptr, *db = nullptr;
  float* dd = nullptr;
  int* dst = nullptr;
  int st = 0;
  const size_t smem = (size_t)128 * K * 2 + (size_t)N * K * 2 + 16;
  bool ok = cudaMalloc(&da, a.size() * 2) == cudaSuccess && cudaMalloc(&db, b.size() * 2) == cudaSuccess &&
            cudaMalloc(&dd, (size_t)128 * N * 4) == cudaSuccess && cudaMalloc(&dst, sizeof(int)) == cudaSuccess;
  ok = ok && cudaMemcpy(da, a.data(), a.size() * 2, cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(db, b.data(), b.size() * 2, cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemset(dst, 0, sizeof(int)) == cudaSuccess && cudaMemset(dd, 0, (size_t)128 * N * 4) == cudaSuccess;
  ok = ok && cudaFuncSetAttribute(k_umma_check, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                 cudaSuccess;
  if (ok) {
    k_umma_check<<<1, 128, smem>>>(N, K, da, db, dd, dst);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  }
  ok = ok && cudaMemcpy(D, dd, (size_t)128 * N * 4, cudaMemcpyDeviceToHost) == cudaSuccess;
  ok = ok && cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(da);
  cudaFree(db);
  cudaFree(dd);
  cudaFree(dst);
  if (!ok) return IDFX_ERR_CUDA;
  return st ? IDFX_ERR_CUDA : IDFX_OK;
}

int idfx_mlp_create(int max_batch, void* stream, idfx_mlp** out) {
  if (!out || max_batch < 1) return IDFX_ERR_STATE;
  *out = nullptr;
  idfx_mlp* h = new (std::nothrow) idfx_mlp();
  if (!h) return IDFX_ERR_STATE;
  if (stream) {
    h->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete h;
      return IDFX_ERR_CUDA;
    }
    h->own_stream = true;
  }
  h->max_batch = max_batch;
  const size_t B = (size_t)max_batch;
  bool ok = dalloc(h, &h->w, NPARAM) && dalloc(h, &h->m, NPARAM) && dalloc(h, &h->v, NPARAM) &&
            dalloc(h, &h->g, NPARAM) && dalloc(h, &h->W1b, (size_t)K1 * NH) && dalloc(h, &h->W2b, (size_t)NH * NH) &&
            dalloc(h, &h->W3b, (size_t)NH * NOUT) && dalloc(h, &h->X, B * K1) && dalloc(h, &h->H1, B * NH) &&
            dalloc(h, &h->H2, B * NH) && dalloc(h, &h->dYb, B * NOUT) && dalloc(h, &h->dZ2b, B * NH) &&
            dalloc(h, &h->dZ1b, B * NH) && dalloc(h, &h->T, B * NOUT) && dalloc(h, &h->Z1, B * NH) &&
            dalloc(h, &h->Z2, B * NH) && dalloc(h, &h->Y, B * NOUT) && dalloc(h, &h->dYf, B * NOUT) &&
            dalloc(h, &h->dZ2f, B * NH) && dalloc(h, &h->dZ1f, B * NH) && dalloc(h, &h->loss, 2) &&
            dalloc(h, &h->kmin, NIN) && dalloc(h, &h->kmax, NIN) && dalloc(h, &h->status, 1) &&
            dalloc(h, &h->ws, GT_WS_FLOATS);
  ok = ok && cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GT_SMEM) ==
                 cudaSuccess;
  if (ok) {
    k_init_keys<<<1, 256, 0, h->stream>>>(h->kmin, h->kmax);
    ok = sync_ok(h) == IDFX_OK;
  }
  if (!ok) {
    idfx_mlp_destroy(h);
    return IDFX_ERR_CUDA;
  }
  *out = h;
  return IDFX_OK;
}

int idfx_mlp_destroy(idfx_mlp* h) {
  if (!h) return IDFX_ERR_STATE;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->allocs) cudaFree(p);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  delete h;
  return IDFX_OK;
}

int idfx_mlp_set_params(idfx_mlp* h, const float* params) {
  if (!h || !params) return IDFX_ERR_STATE;
  if (cudaMemcpyAsync(h->w, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return IDFX_ERR_CUDA;
  cudaMemsetAsync(h->m, 0, sizeof(float) * NPARAM, h->stream);
  cudaMemsetAsync(h->v, 0, sizeof(float) * NPARAM, h->stream);
  h->t = 0;
  k_refresh_bf16<<<(K1 * NH + 255) / 256, 256, 0, h->stream>>>(h->w, h->W1b, h->W2b, h->W3b);
  return sync_ok(h);
}

int idfx_mlp_get_params(idfx_mlp* h, float* params) {
  if (!h || !params) return IDFX_ERR_STATE;
  if (cudaMemcpyAsync(params, h->w, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return IDFX_ERR_CUDA;
  return sync_ok(h);
}

int idfx_mlp_set_dataset_device(idfx_mlp* h, const float* prims, const float* targets, int nsnap, int nc,
                                double gamma) {
  if (!h || !prims || !targets || nsnap < 1 || nc < 3) return IDFX_ERR_STATE;
  h->prims = prims;
  h->tgt = targets;
  h->nsnap = nsnap;
  h->nc = nc;
  h->gamma = gamma;
  return IDFX_OK;
}

int idfx_mlp_batch_device(idfx_mlp* h, int batch, unsigned long long seed, long long base, void* X, float* T) {
  if (!h || !h->prims || !X || !T || batch < 1) return IDFX_ERR_STATE;
  k_make_batch<<<(batch + 127) / 128, 128, 0, h->stream>>>(h->prims, h->tgt, h->nsnap, h->nc, (float)h->gamma, seed,
                                                           base, batch, static_cast<__nv_bfloat16*>(X), T, nullptr,
                                                           nullptr);
  return sync_ok(h);
}

int idfx_mlp_train(idfx_mlp* h, int steps, int batch, float lr, float lr_end, unsigned long long seed,
                   float* losses) {
  if (!h || !h->prims || batch < 1 || batch > h->max_batch || steps < 0) return IDFX_ERR_STATE;
  double* dl = nullptr;
  if (cudaMalloc(&dl, sizeof(double) * (steps > 0 ? steps : 1)) != cudaSuccess) return IDFX_ERR_CUDA;
  cudaMemsetAsync(dl, 0, sizeof(double) * (steps > 0 ? steps : 1), h->stream);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int s = 0; s < steps; s++) {
    const long long base = (h->t + s) * (long long)batch;
    k_make_batch<<<(batch + 127) / 128, 128, 0, h->stream>>>(h->prims, h->tgt, h->nsnap, h->nc, (float)h->gamma,
                                                             seed, base, batch, h->X, h->T, h->kmin, h->kmax);
    fwd_bwd(h, batch, dl + s);
    const double tt = (double)(h->t + s + 1);
    const float frac = steps > 1 ? (float)s / (float)(steps - 1) : 1.f;
    const float lr_s = lr_end + 0.5f * (lr - lr_end) * (1.f + cosf(3.14159265f * frac));
    k_adam<<<(NPARAM + 255) / 256, 256, 0, h->stream>>>(h->w, h->m, h->v, h->g, lr_s, b1, b2, eps,
                                                        (float)(1.0 - std::pow((double)b1, tt)),
                                                        (float)(1.0 - std::pow((double)b2, tt)), h->W1b, h->W2b,
                                                        h->W3b);
  }
  h->t += steps;
  int rc = sync_ok(h);
  if (!rc && losses && steps > 0) {
    std::vector<double> hl(steps);
    if (cudaMemcpy(hl.data(), dl, sizeof(double) * steps, cudaMemcpyDeviceToHost) != cudaSuccess) rc = IDFX_ERR_CUDA;
    for (int s = 0; s < steps; s++) losses[s] = (float)hl[s];
  }
  cudaFree(dl);
  return rc;
}

int idfx_mlp_eval(idfx_mlp* h, int batch, unsigned long long seed, double* loss, double* loss_zero) {
  if (!h || !h->prims || batch < 1 || batch > h->max_batch) return IDFX_ERR_STATE;
  cudaMemsetAsync(h->loss, 0, sizeof(double) * 2, h->stream);
  k_make_batch<<<(batch + 127) / 128, 128, 0, h->stream>>>(h->prims, h->tgt, h->nsnap, h->nc, (float)h->gamma, seed,
                                                           0, batch, h->X, h->T, nullptr, nullptr);
  gemm(h->stream, batch, NH, K1, h->X, K1, 0, h->W1b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH}, h->status, h->ws);
  gemm(h->stream, batch, NH, NH, h->H1, NH, 0, h->W2b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH}, h->status, h->ws);
  gemm(h->stream, batch, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0,
       EpiArgs{kEpiBias, h->w + OB3, nullptr, h->Y, nullptr, NOUT}, h->status, h->ws);
  const int ne = batch * NOUT;
  k_loss<<<(ne + 255) / 256, 256, 0, h->stream>>>(h->Y, h->T, batch, h->dYf, h->dYb, h->loss);
  k_sumsq_targets<<<(ne + 255) / 256, 256, 0, h->stream>>>(h->T, batch, h->loss + 1);
  double hl[2];
  if (cudaMemcpyAsync(hl, h->loss, sizeof(hl), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) return IDFX_ERR_CUDA;
  const int rc = sync_ok(h);
  if (loss) *loss = hl[0];
  if (loss_zero) *loss_zero = hl[1];
  return rc;
}

int idfx_mlp_feature_range(idfx_mlp* h, float* fmin, float* fmax) {
  if (!h || !fmin || !fmax) return IDFX_ERR_STATE;
  unsigned a[NIN], b[NIN];
  cudaMemcpyAsync(a, h->kmin, sizeof(a), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(b, h->kmax, sizeof(b), cudaMemcpyDeviceToHost, h->stream);
  const int rc = sync_ok(h);
  for (int i = 0; i < NIN; i++) {
    fmin[i] = fkey_inv(a[i]);
    fmax[i] = fkey_inv(b[i]);
  }
  return rc;
}

int idfx_mlp_grad_device(idfx_mlp* h, const void* X, const float* T, int batch, float* grad, double* loss) {
  if (!h || !X || !T || !grad || batch < 1 || batch > h->max_batch) return IDFX_ERR_STATE;
  cudaMemcpyAsync(h->X, X, sizeof(__nv_bfloat16) * (size_t)batch * K1, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(h->T, T, sizeof(float) * (size_t)batch * NOUT, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemsetAsync(h->loss, 0, sizeof(double), h->stream);
  fwd_bwd(h, batch, h->loss);
  cudaMemcpyAsync(grad, h->g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, h->stream);
  double hl = 0.0;
  cudaMemcpyAsync(&hl, h->loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  const int rc = sync_ok(h);
  if (loss) *loss = hl;
  return rc;
}

int idfx_mlp_forward_device(idfx_mlp* h, const void* X, int batch, float* Y) {
  if (!h || !X || !Y || batch < 1 || batch > h->max_batch) return IDFX_ERR_STATE;
  cudaMemcpyAsync(h->X, X, sizeof(__nv_bfloat16) * (size_t)batch * K1, cudaMemcpyDeviceToDevice, h->stream);
  gemm(h->stream, batch, NH, K1, h->X, K1, 0, h->W1b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH}, h->status, h->ws);
  gemm(h->stream, batch, NH, NH, h->H1, NH, 0, h->W2b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH}, h->status, h->ws);
  gemm(h->stream, batch, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0, EpiArgs{kEpiBias, h->w + OB3, nullptr, Y, nullptr,
                                                                           NOUT}, h->status, h->ws);
  return sync_ok(h);
}

int idfx_learn_coarsen_device(const double* Vc, const double* Vs, int nf, int nghost, int r, double gamma,
                              double* prim, double* faces, double* targets, void* stream) {
  if (!Vc || !Vs || !prim || !faces || !targets || r < 1 || nf < r || nf % r != 0 || nghost < 1)
    return IDFX_ERR_CONFIG;
  const long long nc = nf / r;
  const long long n = nc * nc * nc;
  k_coarsen<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(Vc, Vs, nf, nghost, r, gamma, prim, faces,
                                                                          targets);
  if (cudaGetLastError() != cudaSuccess) return IDFX_ERR_CUDA;
  return cudaStreamSynchronize((cudaStream_t)stream) == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
}

}  // extern "C"
