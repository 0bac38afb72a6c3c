// Exact FP64 operations formed from the bit patterns on the integer pipe.
//
// The FP64 pipe of this GPU is narrow and the FP64 kernels are bound by it
// while the integer pipe idles; where an FP64 operation has an exact result
// that the bit pattern gives directly, these helpers form it with integer
// operations.  Each equals the IEEE-754 operation it replaces for every
// input (NaNs compare false and stay NaN), checked on the host over random
// bit patterns, zeros, subnormals and infinities.
#pragma once
#include <stdint.h>

#include "intdiv.cuh"  // dbits / dfrom, IDFX_HD

namespace idfx {

// Sign tests against zero from the bit pattern (FP64: integer pipe), equal
// to the IEEE comparisons for every x: zeros of either sign are neither > 0
// nor < 0, NaNs compare false.  FP32: the comparisons.
template <typename T>
IDFX_HD bool gt0(T x) {
  if constexpr (sizeof(T) == 8) {
    const int64_t b = (int64_t)dbits(x);
    return b > 0 && b <= 0x7FF0000000000000ll;
  } else {
    return x > T(0);
  }
}
template <typename T>
IDFX_HD bool lt0(T x) {
  if constexpr (sizeof(T) == 8) {
    const uint64_t m = dbits(x) & 0x7FFFFFFFFFFFFFFFull;  // |x|
    return (dbits(x) >> 63) && m != 0ull && m <= 0x7FF0000000000000ull;
  } else {
    return x < T(0);
  }
}
template <typename T>
IDFX_HD bool ge0(T x) {  // x >= 0: a zero or > 0
  if constexpr (sizeof(T) == 8) {
    return (dbits(x) << 1) == 0ull || gt0(x);
  } else {
    return x >= T(0);
  }
}
template <typename T>
IDFX_HD bool le0(T x) {
  if constexpr (sizeof(T) == 8) {
    return (dbits(x) << 1) == 0ull || lt0(x);
  } else {
    return x <= T(0);
  }
}

// x * s for a sign s = +-1 held as its sign bit (sb: 0 or the sign mask):
// on the FP64 path a sign-bit flip on the integer pipe, equal to the product
// for every non-NaN x; FP32 the product
template <typename T>
IDFX_HD T times_sign(T x, T s, uint64_t sb) {
  if constexpr (sizeof(T) == 8) {
    (void)s;
    return dfrom(dbits(x) ^ sb);
  } else {
    (void)sb;
    return x * s;
  }
}

// One upwind term of CalcContactAverage, (1 - w) a + w b with the weight w
// in {0, 1/2, 1} (storeFlux.hpp:40-43).  The FP64 path forms the two
// products exactly on the integer pipe - a product by 1 is the value, by 0 a
// zero of the value's sign, by 1/2 an exponent decrement - and 1 - w from
// w's bit pattern, so only the sum issues on the FP64 pipe; any other weight,
// and non-finite or subnormal values, take the FP64 expression.  Every case
// is bit-identical to the reference's expression.
IDFX_HD double zero_times(double x) {  // (+0) x
  const uint64_t u = dbits(x);
  if (((u >> 52) & 0x7ffu) != 0x7ffu) return dfrom(u & (1ull << 63));
  return 0.0 * x;
}
IDFX_HD double half_of(double x) {  // x / 2
  const uint64_t u = dbits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  if (e - 2u < 2045u) return dfrom(u - (1ull << 52));
  if ((u << 1) == 0ull) return x;
  return 0.5 * x;
}
template <typename E>
IDFX_HD E upwind_term(E w, E a, E b) {
  if constexpr (sizeof(E) == 8) {
    const uint64_t W = dbits(w);
    double p, q;
    if (W == 0ull) {  // (1 - 0) a + 0 b
      p = a;
      q = zero_times(b);
    } else if (W == 0x3FF0000000000000ull) {  // (1 - 1) a + 1 b
      p = zero_times(a);
      q = b;
    } else if (W == 0x3FE0000000000000ull) {  // halves
      p = half_of(a);
      q = half_of(b);
    } else {
      p = (1.0 - w) * a;
      q = w * b;
    }
    return p + q;
  } else {
    return (E(1) - w) * a + w * b;
  }
}

}  // namespace idfx
