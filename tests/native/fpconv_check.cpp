// Host check of idfx::f2d_exact and idfx::d2f_rn (idefix_gb300/csrc/
// fpconv.cuh) against the host's IEEE-754 conversions: every binary32 bit
// pattern (strided by argv[1]) for f2d, random binary64 values over the
// whole range, near the binary32 range limits and at rounding ties for d2f.
// Prints the number of mismatches.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../idefix_gb300/csrc/fpconv.cuh"

static unsigned long long mism = 0, total = 0;

static void check_d2f(double x) {
  const float a = (float)x, b = idfx::d2f_rn(x);
  total++;
  if (!((std::isnan(a) && std::isnan(b)) || idfx::fbits(a) == idfx::fbits(b))) {
    if (mism < 10) std::printf("d2f mismatch x=%a host=%a int=%a\n", x, (double)a, (double)b);
    mism++;
  }
}

int main(int argc, char** argv) {
  const unsigned stride = argc > 1 ? (unsigned)std::atol(argv[1]) : 1u;
  for (uint64_t u = 0; u < (1ull << 32); u += stride) {
    const float f = idfx::ffrom((uint32_t)u);
    const double a = (double)f, b = idfx::f2d_exact(f);
    total++;
    if (!((std::isnan(a) && std::isnan(b)) || idfx::dbits(a) == idfx::dbits(b))) {
      if (mism < 10) std::printf("f2d mismatch %08x host=%a int=%a\n", (unsigned)u, a, b);
      mism++;
    }
  }
  std::mt19937_64 rng(7);
  const long n = 4000000;
  for (long i = 0; i < n; i++) check_d2f(idfx::dfrom(rng()));  // any bit pattern
  for (long i = 0; i < n; i++) {  // around the binary32 normal range and its edges
    const uint64_t e = 860 + rng() % 330;
    check_d2f(idfx::dfrom((rng() & (1ull << 63)) | (e << 52) | (rng() & ((1ull << 52) - 1))));
  }
  for (long i = 0; i < n; i++) {  // ties and neighbours of ties
    const uint64_t e = 897 + rng() % 254;
    const uint64_t hi = rng() & ((1ull << 23) - 1);
    const int64_t d = (int64_t)(rng() % 5) - 2;
    const uint64_t m = (hi << 29) + (1ull << 28) + (uint64_t)d;
    check_d2f(idfx::dfrom((rng() & (1ull << 63)) | (e << 52) | (m & ((1ull << 52) - 1))));
  }
  // the largest binary32 and the rounding boundary to infinity
  const double fmax = 3.4028234663852886e38;
  for (int k = -3; k <= 3; k++) check_d2f(std::nextafter(fmax, k > 0 ? 1e300 : 0.0) * 1.0 + k * 1e22);
  check_d2f(0.0);
  check_d2f(-0.0);
  std::printf("%llu mismatches in %llu conversions\n", mism, total);
  return mism != 0;
}
