// Host check of idfx::div_rn (idefix_gb300/csrc/intdiv.cuh) against the
// host's IEEE-754 division: random operands over the whole normal range,
// significands near 1 and near 2, quotients at the edges of the normal range,
// and special operands.  Prints the number of mismatches.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <random>

#include "../../idefix_gb300/csrc/intdiv.cuh"
#include "../../idefix_gb300/csrc/rdiv.cuh"

static uint64_t mism = 0, total = 0;

static void check(double a, double b) {
  const double r0 = a / b, r1 = idfx::div_rn(a, b);
  total++;
  const bool same = (std::isnan(r0) && std::isnan(r1)) || idfx::dbits(r0) == idfx::dbits(r1);
  if (!same) {
    if (mism < 10)
      std::printf("mismatch a=%a b=%a ieee=%a int=%a\n", a, b, r0, r1);
    mism++;
  }
  // the reciprocal form with Markstein's correction (rdiv.cuh)
  const double r2 = idfx::div_r(a, idfx::recip(b));
  total++;
  if (!((std::isnan(r0) && std::isnan(r2)) || idfx::dbits(r0) == idfx::dbits(r2))) {
    if (mism < 10)
      std::printf("mismatch a=%a b=%a ieee=%a rcp=%a\n", a, b, r0, r2);
    mism++;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 rng(12345);
  auto rnd_double = [&](int emin, int emax) {
    const uint64_t mant = rng() & ((1ull << 52) - 1);
    const uint64_t e = (uint64_t)(emin + (long)(rng() % (uint64_t)(emax - emin + 1)));
    const uint64_t s = rng() & (1ull << 63);
    return idfx::dfrom(s | (e << 52) | mant);
  };
  for (long i = 0; i < n; i++) check(rnd_double(1, 2046), rnd_double(1, 2046));
  for (long i = 0; i < n; i++) check(rnd_double(900, 1150), rnd_double(900, 1150));
  // significands near 1 and near 2 (divisor and dividend)
  for (long i = 0; i < n / 4; i++) {
    const uint64_t lo = rng() % (1ull << 30), hi = ((1ull << 52) - 1) - (rng() % (1ull << 30));
    const uint64_t e1 = 1000 + rng() % 40, e2 = 1000 + rng() % 40;
    const uint64_t m1 = (rng() & 1) ? lo : hi, m2 = (rng() & 1) ? lo : hi;
    check(idfx::dfrom((e1 << 52) | m1), idfx::dfrom((e2 << 52) | m2));
    check(idfx::dfrom((e1 << 52) | (rng() & ((1ull << 52) - 1))), idfx::dfrom((e2 << 52) | m2));
  }
  // exact quotients and small integers
  for (int i = 1; i < 2000; i++)
    for (int j = 1; j < 200; j++) check((double)i, (double)j);
  // quotients near the edges of the normal range, and special operands
  const double sp[] = {0.0, -0.0, 1.0, -1.0, std::numeric_limits<double>::infinity(),
                       -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                       std::numeric_limits<double>::denorm_min(), std::numeric_limits<double>::min(),
                       std::numeric_limits<double>::max(), 3.0, 1e-300, 1e300, 0.1};
  for (double a : sp)
    for (double b : sp) check(a, b);
  for (long i = 0; i < n / 4; i++) {
    check(rnd_double(1, 60), rnd_double(1000, 1100));
    check(rnd_double(1990, 2046), rnd_double(1, 60));
  }
  std::printf("%llu mismatches of %llu\n", (unsigned long long)mism, (unsigned long long)total);
  return mism != 0;
}
