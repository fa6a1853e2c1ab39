// Host check of the threshold form of sqrt(s) <= delta (perigrain_gb300/csrc/pg_sqrt_threshold.h,
// used by the bond builder and the contact test): s <= sqrt_le_max(delta) must decide exactly as
// sqrt(s) <= delta for deltas of every magnitude
// (grid spacings and random values, zero, negative, NaN, infinite) and s at and around delta^2
// (every double within 64 ulps), random s, and the special values a sum of squares can take
// (+0, +inf, NaN; never a negative number). Prints "bad 0" on success.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "pg_sqrt_threshold.h"

static uint64_t checked = 0, bad = 0;
static double from_bits(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }
static uint64_t bits(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }

static void check(double delta, double smax, double s) {
  ++checked;
  const bool want = std::sqrt(s) <= delta, got = s <= smax;
  if (want != got && bad++ < 10) std::printf("delta %a s %a: sqrt rule %d, threshold %a gives %d\n", delta, s, want, smax, got);
}

static void around(double delta) {
  const double smax = pg::sqrt_le_max(delta);
  // s is a sum of squares: +0 or more, +inf or NaN, never negative
  const double specials[] = {0.0, INFINITY, NAN, 5e-324, DBL_MAX};
  for (double s : specials) check(delta, smax, s);
  const double c = delta * delta;
  if (std::isfinite(c) && c > 0)
    for (int k = -64; k <= 64; ++k) check(delta, smax, from_bits(bits(c) + k));
  if (std::isfinite(smax) && smax > 0)
    for (int k = -3; k <= 3; ++k) check(delta, smax, from_bits(bits(smax) + k));
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 200000;
  std::mt19937_64 rng(11);
  const double fixed[] = {0.0, -0.0, -1.0, NAN, INFINITY, 1e-300, 5e-324, 1e154, 1.5e154, DBL_MAX, 1.0, 3e-4, 1e-3};
  for (double d : fixed) around(d);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (long i = 0; i < n; ++i) {
    // grid spacings h and horizons m h (m = 2..4, with and without a tiny jitter), mm to um scale
    const double h = std::ldexp(1.0 + u(rng), -(int)(rng() % 30));
    const double m = 2.0 + (double)(rng() % 3) + (rng() & 1 ? 0.0 : 1e-6 * u(rng));
    around(m * h);
    // random deltas over the whole exponent range
    const double d = from_bits((rng() & 0x7fefffffffffffffull) | 0x0010000000000000ull);
    around(d);
    const double smax = pg::sqrt_le_max(m * h);
    for (int k = 0; k < 4; ++k) check(m * h, smax, (m * h) * (m * h) * (0.5 + u(rng)));
  }
  std::printf("checked %" PRIu64 " bad %" PRIu64 "\n", checked, bad);
  return bad == 0 ? 0 : 1;
}
