// FP32 <-> FP64 conversions on the integer pipe.
//
// On this GPU the conversion instructions between FP32 and FP64 issue on the
// narrow FP64 pipe.  The mixed-precision path converts every primitive it
// hands to the FP32 sweeps and every FP32 EMF it hands to the FP64 face
// update; these two functions do it with integer operations on the bit
// patterns (IEEE-754 binary32 / binary64 layouts):
//   f2d_exact: binary32 -> binary64, exact (a rebias of the exponent and a
//              shift of the significand);
//   d2f_rn:    binary64 -> binary32, round to nearest, ties to even (the 29
//              dropped significand bits decide; a carry out of the significand
//              moves into the exponent, up to infinity as IEEE rounding does).
// Zeros take the integer path too; subnormal, infinite and NaN operands (and
// binary64 values outside the binary32 normal range) take the hardware
// conversion.  Both are checked bit for bit against the host's and CUDA's
// conversions.
#pragma once
#include <stdint.h>
#include <string.h>

#include "intdiv.cuh"  // dbits / dfrom, IDFX_HD

namespace idfx {

IDFX_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

IDFX_HD float ffrom(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

IDFX_HD double f2d_exact(float x) {
  const uint32_t u = fbits(x);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t s = (uint64_t)(u & 0x80000000u) << 32;
  if (e - 1u < 254u) return dfrom(s | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29));
  if ((u & 0x7fffffffu) == 0u) return dfrom(s);
  return (double)x;
}

IDFX_HD float d2f_rn(double x) {
  const uint64_t u = dbits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  const uint32_t s = (uint32_t)(u >> 32) & 0x80000000u;
  // binary32 normal range: biased exponent 1..254 <=> binary64 897..1150
  if (e - 897u < 254u) {
    const uint64_t m = u & ((1ull << 52) - 1ull);
    const uint32_t rest = (uint32_t)m & ((1u << 29) - 1u);
    uint32_t r = ((e - 896u) << 23) | (uint32_t)(m >> 29);
    const uint32_t half = 1u << 28;
    if (rest > half || (rest == half && (r & 1u))) r += 1u;
    return ffrom(s | r);
  }
  if ((u << 1) == 0ull) return ffrom(s);
  return (float)x;
}

}  // namespace idfx
