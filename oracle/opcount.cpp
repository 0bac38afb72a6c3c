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
 * pragmas are ignored).  Exports the ofx API plus ofx_opcount_reset,
 * ofx_opcount_read (totals) and ofx_opcount_read_phase (per phase of the
 * cycle, as ofx.c marks them with OFX_PHASE); oracle/opcount.py turns the
 * counts into FLOP per zone-cycle.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

namespace opc {

/* add/sub, mul, div, sqrt, fmin/fmax, fabs, comparisons, negation */
enum { ADD = 0, MUL, DIV, SQRT, MINMAX, ABS, CMP, NEG, NCAT };
/* per phase of the cycle (the OFX_PH_* of ofx.c, fewer than kMaxPhase) */
constexpr int kMaxPhase = 16;
static long long per_phase[kMaxPhase][NCAT];
static long long* counts = per_phase[0];
static void set_phase(int p) { counts = per_phase[(p >= 0 && p < kMaxPhase) ? p : 0]; }

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

#define OFX_PHASE(p) opc::set_phase(p)
#define double opc::R
#include "ofx.c"
#undef double
static_assert(OFX_NPH <= opc::kMaxPhase, "too many phases");

extern "C" {

void ofx_opcount_reset(void) {
  for (int p = 0; p < opc::kMaxPhase; p++)
    for (int c = 0; c < opc::NCAT; c++) opc::per_phase[p][c] = 0;
  opc::set_phase(OFX_PH_OTHER);
}

/* copies min(n, 8) counters summed over the phases: add/sub, mul, div,
   sqrt, min/max, abs, cmp, neg; returns the number of kinds */
int ofx_opcount_read(long long* out, int n) {
  int m = n < opc::NCAT ? n : opc::NCAT;
  for (int c = 0; c < m; c++) {
    long long t = 0;
    for (int p = 0; p < opc::kMaxPhase; p++) t += opc::per_phase[p][c];
    out[c] = t;
  }
  return opc::NCAT;
}

/* the same for one phase (OFX_PH_* of ofx.c); returns the number of phases */
int ofx_opcount_read_phase(int phase, long long* out, int n) {
  int m = n < opc::NCAT ? n : opc::NCAT;
  for (int c = 0; c < m; c++) out[c] = (phase >= 0 && phase < OFX_NPH) ? opc::per_phase[phase][c] : 0;
  return OFX_NPH;
}

}  /* extern "C" */
