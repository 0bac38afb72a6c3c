// Learned interface-state correction (see learned.cuh): BF16 tensor-core
// training kernels (forward, backward, Adam), the training-data kernels
// (coarsening of fine snapshots, batch assembly) and the fused learned
// reconstruction used by the ORDER 5 sweeps, with their C ABI.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/idefix_gb300.h"
#include "engine.hpp"
#include "learned.cuh"

using namespace idfx;
using namespace idfx::learn;

namespace {

// ---------------------------------------------------------------------------
// Generic BF16 GEMM for training: C[M][N] = op(A)[M][K] . op(B)[K][N] with
// FP32 accumulation, 64x64 block tiles, BK = 32, 4 warps of 32x32.
// A(m,k) = transA ? A[k*lda + m] : A[m*lda + k]
// B(k,n) = transB ? B[n*ldb + k] : B[k*ldb + n]
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

constexpr int GB_M = 64, GB_N = 64, GB_K = 32, GB_LD = GB_K + 8;

__global__ void __launch_bounds__(128) k_gemm(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                              int transA, const __nv_bfloat16* __restrict__ B, int ldb, int transB,
                                              EpiArgs ep) {
  __shared__ __align__(16) __nv_bfloat16 As[GB_M * GB_LD];
  __shared__ __align__(16) __nv_bfloat16 Bs[GB_N * GB_LD];
  const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
  const int warp = threadIdx.x >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < K; k0 += GB_K) {
    // stage the tiles: As[m][k], Bs[n][k] (k contiguous)
    for (int e = threadIdx.x; e < GB_M * GB_K; e += blockDim.x) {
      int r, k;
      if (transA) {  // consecutive threads walk m (contiguous in memory)
        r = e % GB_M;
        k = e / GB_M;
      } else {
        r = e / GB_K;
        k = e % GB_K;
      }
      const int gm = m0 + r, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gm < M && gk < K) v = transA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk];
      As[r * GB_LD + k] = v;
    }
    for (int e = threadIdx.x; e < GB_N * GB_K; e += blockDim.x) {
      int n, k;
      if (transB) {
        n = e / GB_K;
        k = e % GB_K;
      } else {
        n = e % GB_N;
        k = e / GB_N;
      }
      const int gn = n0 + n, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gn < N && gk < K) v = transB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn];
      Bs[n * GB_LD + k] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GB_K; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int a = 0; a < 2; a++) load_a(af[a], As, GB_LD, wm + 16 * a, kk);
#pragma unroll
      for (int b = 0; b < 4; b++) load_b(bf[b], Bs, GB_LD, wn + 8 * b, kk);
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) mma_bf16(acc[a][b], af[a], bf[b]);
    }
    __syncthreads();
  }
  // epilogue: accumulator element (row, col) of the C fragment layout
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int m = m0 + wm + 16 * a + g + ((c & 2) ? 8 : 0);
        const int n = n0 + wn + 8 * b + 2 * t + (c & 1);
        if (m >= M || n >= N) continue;
        const long long o = (long long)m * ep.ldo + n;
        float v = acc[a][b][c];
        switch (ep.mode) {
          case kEpiF32:
            ep.out_f[o] = v;
            break;
          case kEpiBiasSilu:
            v += ep.bias[n];
            ep.out_f[o] = v;
            ep.out_b[o] = __float2bfloat16(silu_f(v));
            break;
          case kEpiBias:
            ep.out_f[o] = v + ep.bias[n];
            break;
          default:  // kEpiDsilu
            v *= dsilu_f(ep.zin[o]);
            ep.out_f[o] = v;
            ep.out_b[o] = __float2bfloat16(v);
            break;
        }
      }
}

void gemm(cudaStream_t s, int M, int N, int K, const __nv_bfloat16* A, int lda, int transA, const __nv_bfloat16* B,
          int ldb, int transB, const EpiArgs& ep) {
  dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M);
  k_gemm<<<grid, 128, 0, s>>>(M, N, K, A, lda, transA, B, ldb, transB, ep);
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
// Fused learned reconstruction (ORDER 5): for every cell with a full 3x3x3
// stencil and every direction, the PLM (van Leer) states of the cell plus
// the network's correction, or the plain PLM states where the stencil is
// outside the trained feature range or a corrected density / pressure is
// not positive.  Persistent CTAs of 256 threads over tiles of 128 cells; the
// BF16 weights stay in shared memory, the three layers run on the tensor
// cores (m16n8k16, FP32 accumulation).
// ls[(d * 16 + face * 8 + var) * ncell + cell]: face 0 minus, 1 plus.
// ---------------------------------------------------------------------------
constexpr int RT = 128;             // cells per tile
constexpr int LD1 = K1 + 8;         // row pitch (elements) of K1-wide operands
constexpr int LD2 = NH + 8;         // row pitch of 128-wide operands
constexpr int LDY = NOUT + 1;
constexpr size_t SM_W1 = (size_t)NH * LD1 * 2;
constexpr size_t SM_W2 = (size_t)NH * LD2 * 2;
constexpr size_t SM_W3 = (size_t)NOUT * LD2 * 2;
constexpr size_t SM_X = (size_t)RT * LD1 * 2;
constexpr size_t SM_H = (size_t)RT * LD2 * 2;
constexpr size_t SM_Y = (size_t)RT * LDY * 4;
constexpr size_t SM_B = (size_t)(NH + NH + NOUT) * 4;
constexpr size_t SM_R = (size_t)2 * NIN * 4;
constexpr size_t SM_F = (size_t)RT * 4 + 16;
constexpr size_t SM_LEARN = SM_W1 + SM_W2 + SM_W3 + SM_X + SM_H + SM_Y + SM_B + SM_R + SM_F;
static_assert(SM_LEARN <= 227 * 1024, "learned reconstruction does not fit in shared memory");

struct LearnedDev {
  const __nv_bfloat16* W1b;  // [K1][NH]
  const __nv_bfloat16* W2b;  // [NH][NH]
  const __nv_bfloat16* W3b;  // [NH][NOUT]
  const float* w;            // packed FP32 parameters (biases)
  const float* fmin;         // [NIN] trained feature range, or null
  const float* fmax;
};

__global__ void __launch_bounds__(256, 1) k_learned_recon(Geo g, const double* __restrict__ Vc, double* __restrict__ ls,
                                                          LearnedDev L, const Ctl* ctl,
                                                          unsigned long long* __restrict__ counters) {
  if (ctl && ctl->done) return;
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* W1t = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* W2t = reinterpret_cast<__nv_bfloat16*>(smem + SM_W1);
  __nv_bfloat16* W3t = reinterpret_cast<__nv_bfloat16*>(smem + SM_W1 + SM_W2);
  __nv_bfloat16* Xs = reinterpret_cast<__nv_bfloat16*>(smem + SM_W1 + SM_W2 + SM_W3);
  __nv_bfloat16* Hs = reinterpret_cast<__nv_bfloat16*>(smem + SM_W1 + SM_W2 + SM_W3 + SM_X);
  float* Ys = reinterpret_cast<float*>(smem + SM_W1 + SM_W2 + SM_W3 + SM_X + SM_H);
  float* bs = reinterpret_cast<float*>(smem + SM_W1 + SM_W2 + SM_W3 + SM_X + SM_H + SM_Y);
  float* rmin = bs + NH + NH + NOUT;
  float* rmax = rmin + NIN;
  int* flag = reinterpret_cast<int*>(rmax + NIN);
  int* nfall = flag + RT;
  __nv_bfloat16* H2s = Xs;  // layer-2 output reuses the input tile
  const int tid = threadIdx.x;
  // weights, transposed to [n][k] (k contiguous) for the B operand
  for (int e = tid; e < K1 * NH; e += blockDim.x) {
    const int k = e / NH, n = e % NH;
    W1t[n * LD1 + k] = L.W1b[e];
  }
  for (int e = tid; e < NH * NH; e += blockDim.x) {
    const int k = e / NH, n = e % NH;
    W2t[n * LD2 + k] = L.W2b[e];
  }
  for (int e = tid; e < NH * NOUT; e += blockDim.x) {
    const int k = e / NOUT, n = e % NOUT;
    W3t[n * LD2 + k] = L.W3b[e];
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
  const int m0 = g.nt[0] - 2, m1 = g.nt[1] - 2, m2 = g.nt[2] - 2;
  const long long nr = (long long)m0 * m1 * m2;
  const long long tiles_per_dir = (nr + RT - 1) / RT;
  const int warp = tid >> 5, lane = tid & 31, gq = lane >> 2, tq = lane & 3;
  for (long long tile = blockIdx.x; tile < 3 * tiles_per_dir; tile += gridDim.x) {
    const int d = (int)(tile / tiles_per_dir);
    const long long r0 = (tile % tiles_per_dir) * RT;
    const int slot = tid & (RT - 1), half = tid >> 7;
    const long long r = r0 + slot;
    const bool valid = r < nr;
    int ix[3] = {1, 1, 1};
    if (valid) {
      ix[0] = 1 + (int)(r % m0);
      ix[1] = 1 + (int)((r / m0) % m1);
      ix[2] = 1 + (int)(r / ((long long)m0 * m1));
    }
    const int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
    const long long sd = g.s[d], s1 = g.s[a1], s2 = g.s[a2];
    const long long cc = cidx(g, ix[2], ix[1], ix[0]);
    __syncthreads();  // previous tile done with flag / Ys / H2s
    if (tid < RT) flag[tid] = valid ? 0 : 1;
    if (tid == 0) *nfall = 0;
    __syncthreads();
    // ---- stencil features (half 0: rotated vars 0-3, half 1: 4-7) ----
    {
      float cen[8];
#pragma unroll
      for (int rv = 0; rv < 8; rv++) cen[rv] = (float)Vc[rot_var(rv, d) * g.ncell + cc];
      const float cs = sqrtf((float)g.gamma * cen[4] / cen[0]), sb = sqrtf(cen[0]) * cs;
      int bad = 0;
      __nv_bfloat16* xr = Xs + slot * LD1;
      for (int q = 0; q < 4; q++) {
        const int rv = half * 4 + q;
        const double* base = Vc + rot_var(rv, d) * g.ncell + cc;
        for (int o2 = -1; o2 <= 1; o2++)
          for (int o1 = -1; o1 <= 1; o1++)
            for (int o0 = -1; o0 <= 1; o0++) {
              const float sv = valid ? (float)base[o0 * sd + o1 * s1 + o2 * s2] : 0.f;
              float f;
              if (rv == 0 || rv == 4) f = sv / cen[rv] - 1.f;
              else if (rv < 4) f = (sv - cen[rv]) / cs;
              else f = sv / sb;
              const int col = rv * 27 + (o2 + 1) * 9 + (o1 + 1) * 3 + (o0 + 1);
              if (!valid) f = 0.f;
              if (ranged && !(f >= rmin[col] && f <= rmax[col])) bad = 1;
              xr[col] = __float2bfloat16(f);
            }
      }
      if (half == 1)
        for (int col = NIN; col < K1; col++) xr[col] = __float2bfloat16(0.f);
      if (bad) atomicOr(flag + slot, 1);
    }
    __syncthreads();
    // ---- layer 1: [128 x K1] . [K1 x 128], warp tile 32 x 64 ----
    {
      const int wm = (warp & 3) * 32, wn = (warp >> 2) * 64;
      float acc[2][8][4];
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 8; b++)
#pragma unroll
          for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
      for (int k0 = 0; k0 < K1; k0 += 16) {
        uint32_t af[2][4], bf[8][2];
#pragma unroll
        for (int a = 0; a < 2; a++) load_a(af[a], Xs, LD1, wm + 16 * a, k0);
#pragma unroll
        for (int b = 0; b < 8; b++) load_b(bf[b], W1t, LD1, wn + 8 * b, k0);
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
          for (int b = 0; b < 8; b++) mma_bf16(acc[a][b], af[a], bf[b]);
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 8; b++)
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const int m = wm + 16 * a + gq + ((c & 2) ? 8 : 0);
            const int n = wn + 8 * b + 2 * tq + (c & 1);
            Hs[m * LD2 + n] = __float2bfloat16(silu_f(acc[a][b][c] + bs[n]));
          }
    }
    __syncthreads();
    // ---- layer 2: [128 x 128] . [128 x 128] -> H2s (over the input tile) ----
    {
      const int wm = (warp & 3) * 32, wn = (warp >> 2) * 64;
      float acc[2][8][4];
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 8; b++)
#pragma unroll
          for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
      for (int k0 = 0; k0 < NH; k0 += 16) {
        uint32_t af[2][4], bf[8][2];
#pragma unroll
        for (int a = 0; a < 2; a++) load_a(af[a], Hs, LD2, wm + 16 * a, k0);
#pragma unroll
        for (int b = 0; b < 8; b++) load_b(bf[b], W2t, LD2, wn + 8 * b, k0);
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
          for (int b = 0; b < 8; b++) mma_bf16(acc[a][b], af[a], bf[b]);
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 8; b++)
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const int m = wm + 16 * a + gq + ((c & 2) ? 8 : 0);
            const int n = wn + 8 * b + 2 * tq + (c & 1);
            H2s[m * LD2 + n] = __float2bfloat16(silu_f(acc[a][b][c] + bs[NH + n]));
          }
    }
    __syncthreads();
    // ---- layer 3: [128 x 128] . [128 x 16], warp tile 16 x 16 ----
    {
      const int wm = warp * 16;
      float acc[2][4];
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[b][c] = 0.f;
      for (int k0 = 0; k0 < NH; k0 += 16) {
        uint32_t af[4], bf[2][2];
        load_a(af, H2s, LD2, wm, k0);
#pragma unroll
        for (int b = 0; b < 2; b++) load_b(bf[b], W3t, LD2, 8 * b, k0);
#pragma unroll
        for (int b = 0; b < 2; b++) mma_bf16(acc[b], af, bf[b]);
      }
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int m = wm + gq + ((c & 2) ? 8 : 0);
          const int n = 8 * b + 2 * tq + (c & 1);
          Ys[m * LDY + n] = acc[b][c] + bs[2 * NH + n];
        }
    }
    __syncthreads();
    // ---- corrected states (thread: cell slot, face = half) ----
    double st[8];
    {
      double cen[8], vl[8], vr[8];
      const double dxd = g.dx[d];
#pragma unroll
      for (int sv = 0; sv < 8; sv++) {
        const double* base = Vc + sv * g.ncell + cc;
        double w[3];
        w[0] = valid ? base[-sd] : 1.0;
        w[1] = valid ? base[0] : 1.0;
        w[2] = valid ? base[sd] : 1.0;
        cen[sv] = w[1];
        Recon<2>::cell<double>(w, dxd, sv == 0 || sv == 4, vl[sv], vr[sv]);
      }
      const double cs = sqrt(g.gamma * cen[4] / cen[0]), sb = sqrt(cen[0]) * cs;
      const double sc[8] = {cen[0], cs, cs, cs, cen[4], sb, sb, sb};
      int bad = 0;
#pragma unroll
      for (int rv = 0; rv < 8; rv++) {
        const int sv = rot_var(rv, d);
        const double plm = half ? vr[sv] : vl[sv];
        st[sv] = plm;
        if (rv == 5) continue;  // normal field: the face value is used
        st[sv] = plm + (double)Ys[slot * LDY + half * 8 + rv] * sc[rv];
      }
      if (!(st[0] > 0.0) || !(st[4] > 0.0)) bad = 1;
      if (bad) atomicOr(flag + slot, 1);
      __syncthreads();
      const bool fall = flag[slot] != 0;
      if (fall) {
#pragma unroll
        for (int sv = 0; sv < 8; sv++) st[sv] = half ? vr[sv] : vl[sv];
      }
      if (valid) {
#pragma unroll
        for (int sv = 0; sv < 8; sv++) ls[((long long)d * 16 + half * 8 + sv) * g.ncell + cc] = st[sv];
        if (half == 0 && fall) atomicAdd(nfall, 1);
      }
    }
    __syncthreads();
    if (tid == 0 && counters) {
      const long long nvalid = (nr - r0 < RT) ? (nr - r0) : RT;
      atomicAdd(counters, (unsigned long long)nvalid);
      atomicAdd(counters + 1, (unsigned long long)*nfall);
    }
  }
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

void launch_learned_recon(Engine& e) {
  LearnedModel* m = static_cast<LearnedModel*>(e.learned);
  LearnedDev L{m->W1b, m->W2b, m->W3b, m->w, m->ranged ? m->fmin : nullptr, m->ranged ? m->fmax : nullptr};
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long nr = (long long)(e.g.nt[0] - 2) * (e.g.nt[1] - 2) * (e.g.nt[2] - 2);
  const long long tiles = 3 * ((nr + RT - 1) / RT);
  const int grid = (int)(tiles < sms ? tiles : sms);
  mark_begin(e, kKLearned);
  k_learned_recon<<<grid, 256, SM_LEARN, e.stream>>>(e.g, e.f.Vc, e.f.ls, L, e.ctl, m->counters);
  mark_end(e);
}

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
  gemm(s, B, NH, K1, h->X, K1, 0, h->W1b, NH, 0, EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH});
  gemm(s, B, NH, NH, h->H1, NH, 0, h->W2b, NH, 0, EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH});
  gemm(s, B, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0, EpiArgs{kEpiBias, h->w + OB3, nullptr, h->Y, nullptr, NOUT});
  const int ne = B * NOUT;
  k_loss<<<(ne + 255) / 256, 256, 0, s>>>(h->Y, h->T, B, h->dYf, h->dYb, loss);
  gemm(s, NH, NOUT, B, h->H2, NH, 1, h->dYb, NOUT, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW3, nullptr, NOUT});
  k_colsum<<<NOUT, 256, 0, s>>>(h->dYf, B, NOUT, h->g + OB3);
  gemm(s, B, NH, NOUT, h->dYb, NOUT, 0, h->W3b, NOUT, 1, EpiArgs{kEpiDsilu, nullptr, h->Z2, h->dZ2f, h->dZ2b, NH});
  gemm(s, NH, NH, B, h->H1, NH, 1, h->dZ2b, NH, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW2, nullptr, NH});
  k_colsum<<<NH, 256, 0, s>>>(h->dZ2f, B, NH, h->g + OB2);
  gemm(s, B, NH, NH, h->dZ2b, NH, 0, h->W2b, NH, 1, EpiArgs{kEpiDsilu, nullptr, h->Z1, h->dZ1f, h->dZ1b, NH});
  gemm(s, NIN, NH, B, h->X, K1, 1, h->dZ1b, NH, 0, EpiArgs{kEpiF32, nullptr, nullptr, h->g + OW1, nullptr, NH});
  k_colsum<<<NH, 256, 0, s>>>(h->dZ1f, B, NH, h->g + OB1);
}

int sync_ok(idfx_mlp* h) {
  if (cudaGetLastError() != cudaSuccess) return IDFX_ERR_CUDA;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
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
    ok = ok && cudaFuncSetAttribute(k_learned_recon, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM_LEARN) ==
                   cudaSuccess;
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
  launch_learned_recon(e);
  const size_t n = (size_t)48 * e.g.ncell;
  if (cudaMemcpyAsync(ls, e.f.ls, n * sizeof(double), cudaMemcpyDeviceToHost, e.stream) != cudaSuccess ||
      cudaStreamSynchronize(e.stream) != cudaSuccess)
    return IDFX_ERR_CUDA;
  return IDFX_OK;
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
            dalloc(h, &h->kmin, NIN) && dalloc(h, &h->kmax, NIN);
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
       EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH});
  gemm(h->stream, batch, NH, NH, h->H1, NH, 0, h->W2b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH});
  gemm(h->stream, batch, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0,
       EpiArgs{kEpiBias, h->w + OB3, nullptr, h->Y, nullptr, NOUT});
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
       EpiArgs{kEpiBiasSilu, h->w + OB1, nullptr, h->Z1, h->H1, NH});
  gemm(h->stream, batch, NH, NH, h->H1, NH, 0, h->W2b, NH, 0,
       EpiArgs{kEpiBiasSilu, h->w + OB2, nullptr, h->Z2, h->H2, NH});
  gemm(h->stream, batch, NOUT, NH, h->H2, NH, 0, h->W3b, NOUT, 0, EpiArgs{kEpiBias, h->w + OB3, nullptr, Y, nullptr,
                                                                           NOUT});
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
