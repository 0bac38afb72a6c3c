// Learned interface-state correction: sizes, parameter packing and the
// BF16 tensor-core building blocks shared by the training kernels and the
// fused learned-reconstruction kernel (learned.cu).
//
// The network reads the 3x3x3 primitive stencil of a cell in the frame
// rotated so that the sweep direction is the first axis (cyclic permutation
// of axes and vector components), scaled by the centre cell, and returns
// normalised corrections of the cell's minus-face and plus-face PLM states:
//   216 -> 128 -> 128 -> 16, SiLU, BF16 operands, FP32 accumulation.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace idfx {
namespace learn {

constexpr int NVAR = 8;
constexpr int NIN = 216;  // 27 cells x 8 variables, index var * 27 + cell
constexpr int K1 = 224;   // NIN padded to a multiple of 16 (rows NIN.. of W1 are zero)
constexpr int NH = 128;
constexpr int NOUT = 16;  // minus-face 8 + plus-face 8 (rotated variable order)
// packed FP32 parameter vector: W1[NIN][NH] b1 W2[NH][NH] b2 W3[NH][NOUT] b3
constexpr int OW1 = 0;
constexpr int OB1 = OW1 + NIN * NH;
constexpr int OW2 = OB1 + NH;
constexpr int OB2 = OW2 + NH * NH;
constexpr int OW3 = OB2 + NH;
constexpr int OB3 = OW3 + NH * NOUT;
constexpr int NPARAM = OB3 + NOUT;
// rotated normal field components (taken from the face field by the solver)
__host__ __device__ constexpr bool loss_masked(int o) { return o == 5 || o == 13; }

// 3-D solver variable order: RHO, VX1..3, PRS, BX1..3.  Rotated variable r
// of direction d -> solver variable.
__host__ __device__ __forceinline__ int rot_var(int r, int d) {
  if (r == 0 || r == 4) return r;
  const int base = (r < 4) ? 1 : 5;
  return base + (d + (r - base)) % 3;
}

// one m16n8k16 BF16 MMA with FP32 accumulation (row-major A, column-major B)
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment of a 16x16 tile at (row0, k0) of a row-major BF16 array (ld in
// elements, even); lane layout of the m16n8k16 A operand
__device__ __forceinline__ void load_a(uint32_t* a, const __nv_bfloat16* A, int ld, int row0, int k0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const __nv_bfloat16* p = A + (row0 + g) * ld + k0 + 2 * t;
  a[0] = *reinterpret_cast<const uint32_t*>(p);
  a[1] = *reinterpret_cast<const uint32_t*>(p + 8 * ld);
  a[2] = *reinterpret_cast<const uint32_t*>(p + 8);
  a[3] = *reinterpret_cast<const uint32_t*>(p + 8 * ld + 8);
}

// B fragment of a 16x8 tile at (k0, n0) from Bt[n][k] (k contiguous)
__device__ __forceinline__ void load_b(uint32_t* b, const __nv_bfloat16* Bt, int ld, int n0, int k0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const __nv_bfloat16* p = Bt + (n0 + g) * ld + k0 + 2 * t;
  b[0] = *reinterpret_cast<const uint32_t*>(p);
  b[1] = *reinterpret_cast<const uint32_t*>(p + 8);
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

}  // namespace learn
}  // namespace idfx
