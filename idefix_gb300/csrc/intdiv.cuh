// Correctly rounded FP64 division on the integer pipe.
//
// GB300 issues FP64 at about 2 thread-operations per clock and SM, and a
// hardware-sequence FP64 division costs about nine of them; the integer
// pipe is much wider.  Its dependency chain is longer, so it pays in
// kernels with many resident warps (the memory-bound whole-array passes)
// and not in the low-occupancy flux sweeps, which keep the hardware division.  div_rn(a, b) returns the IEEE-754 round-to-nearest-
// even quotient, bit-identical to a / b, computing the significand quotient
// with 64-bit integer arithmetic:
//   * the divisor significand x in [2^52, 2^53) gets a reciprocal
//     R ~ 2^116 / x: a 24-bit seed (single-precision reciprocal) refined by
//     two Newton-Raphson steps R <- R + R (2^116 - x R) / 2^116 in 64/128-bit
//     fixed point (quadratic convergence: 2^-21 -> 2^-42 -> 2^-63);
//   * the quotient estimate q = floor(m R / 2^64) of the dividend
//     significand m (scaled so that m / x is in [1, 2)) is within a few
//     units of floor(m 2^52 / x); the exact remainder m 2^52 - q x (it fits
//     in 64 bits) corrects it, and rounds to nearest even.
// Operands that are zero, subnormal, infinite or NaN, and quotients outside
// the normal exponent range, take the hardware division.
// Written for this
// project from the textbook method (Newton-Raphson reciprocal refinement
// followed by an exact remainder correction, as in J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, ch. on division), and checked
// against IEEE division on the host and against CUDA's `/` on the GPU.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define IDFX_HD __host__ __device__ __forceinline__
#else
#define IDFX_HD inline
#endif

namespace idfx {

IDFX_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

IDFX_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

IDFX_HD double dfrom(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

// approximate reciprocal of a positive normal float (relative error < 2^-21)
IDFX_HD float rcp_seed(float f) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  return r;
#else
  return 1.0f / f;
#endif
}

// One Newton-Raphson step of R ~ 2^116 / x in fixed point.
IDFX_HD uint64_t nr_step(uint64_t x, uint64_t R) {
  const uint64_t p_hi = umulhi64(x, R);
  const uint64_t p_lo = x * R;
  // E = 2^116 - x R as a signed 128-bit (e_hi, e_lo); |E| < 2^96
  const uint64_t e_lo = 0ull - p_lo;
  const int64_t e_hi = (int64_t)((1ull << 52) - p_hi - (p_lo != 0 ? 1ull : 0ull));
  // e52 = E / 2^52 (arithmetic shift of the 128-bit value), |e52| < 2^44
  const int64_t e52 = (int64_t)(((uint64_t)e_hi << 12) | (e_lo >> 52));
  const uint64_t mag = e52 < 0 ? (uint64_t)(-e52) : (uint64_t)e52;
  const uint64_t c = umulhi64(R, mag);  // R |E| / 2^116, truncated
  return e52 < 0 ? R - c : R + c;
}

IDFX_HD double div_rn(double a, double b) {
  const uint64_t A = dbits(a), B = dbits(b);
  const uint32_t ea = (uint32_t)(A >> 52) & 0x7ffu, eb = (uint32_t)(B >> 52) & 0x7ffu;
  // zero, subnormal, infinite or NaN operands
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) return a / b;
  const uint64_t H = 1ull << 52, M = H - 1ull;
  uint64_t m = (A & M) | H;
  const uint64_t x = (B & M) | H;
  int e = (int)ea - (int)eb + 1023;
  if (m < x) {
    m <<= 1;
    e -= 1;
  }
  // the quotient's biased exponent must leave room for a rounding carry
  if ((uint32_t)(e - 1) >= 2045u) return a / b;
  const uint64_t sign = (A ^ B) & (1ull << 63);
  uint64_t q;
  int64_t rem;
  if (x == H) {  // divisor significand 1: exact
    q = m;
    rem = 0;
  } else {
    // seed: x truncated to 24 bits as a float in [2^52, 2^53), its
    // reciprocal scaled by 2^116 and read back as an integer in (2^63, 2^64)
    uint32_t fb = ((127u + 52u) << 23) | (uint32_t)((x >> 29) & 0x7fffffu);
    float xf;
    memcpy(&xf, &fb, 4);
    const float r = rcp_seed(xf);
    uint32_t rb;
    memcpy(&rb, &r, 4);
    // r * 2^116: add 116 to the exponent field
    const int re = (int)((rb >> 23) & 0xffu) + 116 - 127;  // unbiased exponent of R0
    const uint64_t rm = (uint64_t)((rb & 0x7fffffu) | 0x800000u);
    uint64_t R = (re >= 64) ? ~0ull : (rm << (re - 23));
    R = nr_step(x, R);
    R = nr_step(x, R);
    q = umulhi64(m, R);
    rem = (int64_t)((m << 52) - q * x);
    // bring the remainder into [0, x)
    for (int k = 0; k < 2; k++)
      if (rem < 0) {
        rem += (int64_t)x;
        q -= 1;
      }
    for (int k = 0; k < 4; k++)
      if (rem >= (int64_t)x) {
        rem -= (int64_t)x;
        q += 1;
      }
    if (rem < 0 || rem >= (int64_t)x) return a / b;  // not reached
  }
  // round to nearest, ties to even
  const uint64_t twice = (uint64_t)rem << 1;
  if (twice > x || (twice == x && (q & 1ull))) q += 1;
  if (q == (H << 1)) {
    q = H;
    e += 1;
  }
  return dfrom(sign | ((uint64_t)e << 52) | (q & M));
}

}  // namespace idfx
