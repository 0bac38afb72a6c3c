/*
 * Floating-point operation count of the CPU oracle - TEST INFRASTRUCTURE ONLY.
 *
 * ofx.c is compiled here with every `double` replaced by `opc::R`, a scalar
 * that holds one double and counts each arithmetic operation done on it by
 * kind.  The arithmetic itself is unchanged (same expression trees, same
 * order, -ffp-contract=off), so the counting build gives results bit-
 * identical to libofx.so (checked by the tests), and the counts are those of
 * the reference algorithm on the actual data: branches (the HLLD fallbacks,
 * the limiter cases, the pressure floor) are taken as the data takes them.
 *
 * Built single-threaded (the counters are plain globals; the oracle's OpenMP
 * pragmas are ignored).  Exports the ofx API plus ofx_opcount_reset /
 * ofx_opcount_read; oracle/opcount.py turns the counts into FLOP per
 * zone-cycle.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

namespace opc {

/* add/sub, mul, div, sqrt, fmin/fmax, fabs, comparisons, negation */
enum { ADD = 0, MUL, DIV, SQRT, MINMAX, ABS, CMP, NEG, NCAT };
static long long counts[NCAT];

struct R {
  double v;
  R() = default;
  R(double x) : v(x) {}
  explicit operator double() const { return v; }

  friend R operator+(R a, R b) { counts[ADD]++; return R(a.v + b.v); }
  friend R operator-(R a, R b) { counts[ADD]++; return R(a.v - b.v); }
  friend R operator*(R a, R b) { counts[MUL]++; return R(a.v * b.v); }
  friend R operator/(R a, R b) { counts[DIV]++; return R(a.v / b.v); }
  friend R operator-(R a) { counts[NEG]++; return R(-a.v); }
  friend R operator+(R a) { return a; }
  R& operator+=(R b) { return *this = *this + b; }
  R& operator-=(R b) { return *this = *this - b; }
  R& operator*=(R b) { return *this = *this * b; }
  R& operator/=(R b) { return *this = *this / b; }

  friend bool operator<(R a, R b) { counts[CMP]++; return a.v < b.v; }
  friend bool operator>(R a, R b) { counts[CMP]++; return a.v > b.v; }
  friend bool operator<=(R a, R b) { counts[CMP]++; return a.v <= b.v; }
  friend bool operator>=(R a, R b) { counts[CMP]++; return a.v >= b.v; }
  friend bool operator==(R a, R b) { counts[CMP]++; return a.v == b.v; }
  friend bool operator!=(R a, R b) { counts[CMP]++; return a.v != b.v; }

  friend R sqrt(R a) { counts[SQRT]++; return R(std::sqrt(a.v)); }
  friend R fabs(R a) { counts[ABS]++; return R(std::fabs(a.v)); }
  friend R fmin(R a, R b) { counts[MINMAX]++; return R(std::fmin(a.v, b.v)); }
  friend R fmax(R a, R b) { counts[MINMAX]++; return R(std::fmax(a.v, b.v)); }
  friend bool isnan(R a) { return std::isnan(a.v); }
};
static_assert(sizeof(R) == sizeof(double), "R must have the layout of a double");

}  // namespace opc

#define double opc::R
#include "ofx.c"
#undef double

extern "C" {

void ofx_opcount_reset(void) {
  for (int c = 0; c < opc::NCAT; c++) opc::counts[c] = 0;
}

/* copies min(n, 8) counters: add/sub, mul, div, sqrt, min/max, abs, cmp, neg */
int ofx_opcount_read(long long* out, int n) {
  int m = n < opc::NCAT ? n : opc::NCAT;
  for (int c = 0; c < m; c++) out[c] = opc::counts[c];
  return opc::NCAT;
}

}  /* extern "C" */
