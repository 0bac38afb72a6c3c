// Learned interface-state correction: sizes, parameter packing and the
// activation functions shared by the training kernels and the learned sweep
// (learned.cu); the tensor-core building blocks are in umma.cuh.
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

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

}  // namespace learn
}  // namespace idfx
