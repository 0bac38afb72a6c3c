// FP64 division by a divisor whose correctly rounded reciprocal is known.
//
// The FP64 pipe of this GPU is narrow and the flux sweeps are bound by it;
// a hardware-sequence division costs several of its instructions.  When a
// divisor is a constant of the run (gamma - 1, a cell width) or is shared by
// several quotients of one Riemann problem, its reciprocal is formed once
// and each quotient takes three FP64 operations, bit-identical to a / b:
//   y = RN(1/b)            (host division, or the device's correctly rounded
//                           reciprocal __drcp_rn)
//   q = RN(a y)            (within one ulp of a / b)
//   r = a - b q            (exact, one FMA)
//   RN(q + r y) = RN(a/b)  (one FMA)
// This is Markstein's theorem on FMA-based division (P. W. Markstein, IBM J.
// Res. Dev. 34 (1990) 111-119; J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, chapter on division), which assumes no
// underflow or overflow: operands and quotients outside a safe exponent
// band, zeros and non-finite values take the hardware division instead.
// Checked bit for bit against a / b on the host and on the GPU.
#pragma once
#include <math.h>
#include <stdint.h>

#include "intdiv.cuh"  // dbits, IDFX_HD

namespace idfx {

struct Recip {
  double b, y;  // divisor, RN(1/b)
};

// correctly rounded reciprocal
IDFX_HD double rcp_rn(double b) {
#ifdef __CUDA_ARCH__
  return __drcp_rn(b);
#else
  return 1.0 / b;
#endif
}

IDFX_HD Recip recip(double b) { return Recip{b, rcp_rn(b)}; }

IDFX_HD double fma_rn(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return fma(a, b, c);
#endif
}

// a / R.b, correctly rounded
IDFX_HD double div_r(double a, const Recip& R) {
  const uint64_t A = dbits(a), B = dbits(R.b);
  const uint32_t ea = (uint32_t)(A >> 52) & 0x7ffu;
  const uint32_t eb = (uint32_t)(B >> 52) & 0x7ffu;
  if (eb - 64u < 1920u) {
    // |a|, |b| and |a / b| within 2^-959 .. 2^959 (biased exponents 64..1983)
    if (ea - 64u < 1920u && (ea + 1023u - eb) - 64u < 1920u) {
      const double q = a * R.y;
      const double r = fma_rn(-q, R.b, a);
      return fma_rn(r, R.y, q);
    }
    if ((A << 1) == 0ull) return dfrom((A ^ B) & (1ull << 63));  // +-0 / b
  }
  return a / R.b;
}

}  // namespace idfx
