// Host check of idefix_gb300/csrc/exact_ops.cuh against the IEEE-754
// operations it replaces: sign tests against zero, products by +-1 (sign
// flips), by 0 and 1/2, and the uct_contact upwind term (1 - w) a + w b for
// w in {0, 1/2, 1}, over random bit patterns, zeros, subnormals, infinities
// and NaNs.  Prints the number of mismatches.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../idefix_gb300/csrc/exact_ops.cuh"

using idfx::dbits;
using idfx::dfrom;

static unsigned long long mism = 0, total = 0;

static bool same(double a, double b) { return (std::isnan(a) && std::isnan(b)) || dbits(a) == dbits(b); }

static void check(const char* what, bool ok, double x, double y = 0.0) {
  total++;
  if (!ok) {
    if (mism < 10) std::printf("%s mismatch x=%a y=%a\n", what, x, y);
    mism++;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 5000000;
  std::mt19937_64 rng(11);
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 1e-310, -1e-310, 4e-308, -4e-308,
                            1.0, -1.0, 0.5, 1.7976931348623157e308, -1.7976931348623157e308};
  auto value = [&](long i) {
    switch (i % 5) {
      case 0: return dfrom(rng());  // any bit pattern
      case 1: return special[rng() % (sizeof(special) / sizeof(special[0]))];
      case 2: return dfrom(rng() & 0x800FFFFFFFFFFFFFull);  // subnormals and zeros
      case 3: return (double)((int64_t)(rng() % 2001) - 1000) * 1e-3;
      default: return std::ldexp((double)(rng() >> 11), (int)(rng() % 2100) - 1100);
    }
  };
  const double weights[] = {0.0, 0.5, 1.0, 0.25, -0.0};
  for (long i = 0; i < n; i++) {
    const double x = value(i), y = value(i + 3);
    check("gt0", idfx::gt0(x) == (x > 0.0), x);
    check("lt0", idfx::lt0(x) == (x < 0.0), x);
    check("ge0", idfx::ge0(x) == (x >= 0.0), x);
    check("le0", idfx::le0(x) == (x <= 0.0), x);
    check("flip+", same(idfx::times_sign(x, 1.0, 0ull), x * 1.0) || std::isnan(x), x);
    check("flip-", same(idfx::times_sign(x, -1.0, 1ull << 63), x * -1.0) || std::isnan(x), x);
    check("zero", same(idfx::zero_times(x), 0.0 * x), x);
    check("half", same(idfx::half_of(x), 0.5 * x), x);
    const double w = weights[i % 5];
    check("upwind", same(idfx::upwind_term(w, x, y), (1.0 - w) * x + w * y), x, y);
  }
  std::printf("%llu mismatches in %llu checks\n", mism, total);
  return mism != 0;
}
