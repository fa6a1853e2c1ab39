// Host check of the integer FP64 division, square root, addition, subtraction, multiplication and
// FP32 -> FP64 conversion (perigrain_gb300/csrc/pg_ieee64.cuh): their bits must equal the host's
// IEEE `a / b`, `sqrt(x)`, `a + b`, `a - b`, `a * b`, `(double)f` and `a > b` (b >= +0) on random
// operands of every exponent (including zeros, subnormals, infinities and NaNs, which take the
// hardware route),
// significands at the edges of the reciprocal estimate's range, quotients near 1 and near the
// overflow and underflow thresholds, exact squares and their neighbours, and divisors shared
// across several quotients. Usage: ieee64_check [cases] [seed]. Prints "bad 0" on success.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "pg_ieee64.cuh"

using pg::ieee64::bits;
using pg::ieee64::from_bits;

static uint64_t bad = 0, checked = 0, bad_div = 0, bad_sqrt = 0, bad_arith = 0;

static bool same(double x, double y) {
  if (std::isnan(x) && std::isnan(y)) return true;
  return bits(x) == bits(y);
}
static void check_div(double a, double b) {
  ++checked;
  const double want = a / b, got = pg::ieee64::div_rn(a, b);
  if (!same(want, got) && (++bad_div, bad++ < 10))
    std::printf("div %a / %a: want %a got %a\n", a, b, want, got);
}
static void check_arith(double a, double b) {
  checked += 3;
  const double w[3] = {a + b, a - b, a * b};
  const double g[3] = {pg::ieee64::add_rn(a, b), pg::ieee64::sub_rn(a, b), pg::ieee64::mul_rn(a, b)};
  const char* nm[3] = {"+", "-", "*"};
  for (int k = 0; k < 3; ++k)
    if (!same(w[k], g[k]) && (++bad_arith, bad++ < 10))
      std::printf("%a %s %a: want %a got %a\n", a, nm[k], b, w[k], g[k]);
}
static void check_widen(float x) {
  ++checked;
  const double w = (double)x, g = pg::ieee64::widen_f32(x);
  if (!same(w, g) && (++bad_arith, bad++ < 10)) std::printf("widen %a: want %a got %a\n", (double)x, w, g);
}
static void check_gt(double a, double b) {
  if (!pg::ieee64::gt_nonneg_ok(bits(b))) return;
  ++checked;
  if ((a > b) != pg::ieee64::gt_nonneg(a, bits(b)) && (++bad_arith, bad++ < 10))
    std::printf("%a > %a: want %d\n", a, b, (int)(a > b));
}
static void check_sqrt(double x) {
  ++checked;
  const double want = std::sqrt(x), got = pg::ieee64::sqrt_rn(x);
  if (!same(want, got) && (++bad_sqrt, bad++ < 10)) std::printf("sqrt %a: want %a got %a\n", x, want, got);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 rng(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 12345);
  auto frac = [&]() { return rng() & pg::ieee64::kFrac; };
  auto make = [](uint64_t sign, uint64_t e, uint64_t f) { return from_bits((sign << 63) | (e << 52) | f); };
  // significands that stress the estimate: smallest, largest, top-24-bit boundaries
  const uint64_t edge_frac[] = {0ull, 1ull, pg::ieee64::kFrac, pg::ieee64::kFrac - 1, (1ull << 29) - 1, 1ull << 29,
                                (1ull << 51), (1ull << 51) - 1, 0x5555555555555ull, 0xaaaaaaaaaaaaaull};
  for (uint64_t fa : edge_frac)
    for (uint64_t fb : edge_frac)
      for (int de = -3; de <= 3; ++de) {
        check_div(make(0, 1023 + de, fa), make(0, 1023, fb));
        check_div(make(1, 1023 + de, fa), make(0, 1023, fb));
      }
  for (uint64_t f : edge_frac)
    for (uint64_t e : {1ull, 2ull, 1022ull, 1023ull, 1024ull, 2045ull, 2046ull}) check_sqrt(make(0, e, f));
  const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 4.9e-324, 2.2250738585072014e-308,
                             1.7976931348623157e308, 1e-310, -1e-310};
  for (double a : specials) {
    check_sqrt(a);
    for (double b : specials) {
      check_div(a, b);
      check_arith(a, b);
      check_gt(a, b);
    }
  }
  for (uint64_t fa : edge_frac)
    for (uint64_t fb : edge_frac)
      for (int de = -60; de <= 60; ++de) {
        check_arith(make(0, 1023 + de, fa), make(0, 1023, fb));
        check_arith(make(1, 1023 + de, fa), make(0, 1023, fb));
      }
  const float fspec[] = {0.0f, -0.0f, INFINITY, -INFINITY, NAN, 1e-45f, -1e-40f, 1.17549435e-38f, 3.4028235e38f, 1.0f};
  for (float x : fspec) check_widen(x);
  for (long i = 0; i < n; ++i) {
    // normal operands with exponents near each other (the kernel's regime)
    const double a = make(rng() & 1, 1023 - 40 + rng() % 80, frac());
    const double b = make(rng() & 1, 1023 - 40 + rng() % 80, frac());
    check_div(a, b);
    check_sqrt(std::fabs(a));
    // any exponent, including zeros, subnormals, infinities, NaNs and over/underflowing quotients
    const double c = make(rng() & 1, rng() % 2048, frac());
    const double d = make(rng() & 1, rng() % 2048, frac());
    check_div(c, d);
    check_sqrt(c);
    // quotients just around the overflow and underflow thresholds
    check_div(make(0, 2046 - rng() % 3, frac()), make(0, 1022 + rng() % 3, frac()));
    check_div(make(0, 1 + rng() % 3, frac()), make(0, 1022 + rng() % 4, frac()));
    // sums, differences and products: any exponents, nearby exponents, near-cancellation,
    // products near the overflow and underflow thresholds
    check_arith(a, b);
    check_arith(c, d);
    check_gt(a, std::fabs(b));
    check_gt(c, std::fabs(d));
    check_gt(from_bits(bits(std::fabs(b)) + (rng() % 5) - 2), std::fabs(b));
    {
      const double x = make(rng() & 1, 1023 - 30 + rng() % 60, frac());
      const int de = (int)(rng() % 130) - 65;
      const double y = make(rng() & 1, (uint64_t)((int)((bits(x) >> 52) & 0x7ff) + de), frac());
      check_arith(x, y);
      const double z = from_bits(bits(x) + (rng() % 9) - 4);  // within a few ulps of x
      check_arith(x, z);
      check_arith(x, -z);
      check_arith(make(0, 1023 + 500 + rng() % 30, frac()), make(rng() & 1, 1023 + 500 + rng() % 30, frac()));
      check_arith(make(0, 1023 - 500 - rng() % 30, frac()), make(rng() & 1, 1023 - 500 - rng() % 30, frac()));
      check_arith(x, 0.0);
      check_arith(-0.0, x);
      // differences of tiny normals: subnormal and smallest-normal results
      const double t = make(rng() & 1, 1 + rng() % 3, frac());
      check_arith(t, from_bits(bits(t) + (rng() % 1025) - 512));
      check_arith(t, -make(0, 1 + rng() % 3, frac()));
    }
    {
      uint32_t u = (uint32_t)rng();
      float fx;
      std::memcpy(&fx, &u, 4);
      check_widen(fx);
    }
    // nearly equal significands (quotient significand near 1 from either side)
    const uint64_t fb = frac();
    const uint64_t fa = (fb + (rng() % 5) - 2) & pg::ieee64::kFrac;
    check_div(make(0, 1023, fa), make(0, 1023 + (rng() % 3) - 1, fb));
    // one divisor, several quotients
    const pg::ieee64::Divisor dv = pg::ieee64::make_divisor(b);
    for (int c3 = 0; c3 < 3; ++c3) {
      const double x = make(rng() & 1, 1023 - 20 + rng() % 40, frac());
      ++checked;
      const double want = x / b, got = pg::ieee64::div_rn(x, dv);
      if (!same(want, got) && (++bad_div, bad++ < 10)) std::printf("shared div %a / %a: want %a got %a\n", x, b, want, got);
    }
    // exact squares of 26-bit integers and their neighbours, at even and odd exponents
    const uint64_t s = (1ull << 25) + rng() % (1ull << 25);
    const double sq = std::ldexp((double)(s * s), (int)(rng() % 64) - 32);
    check_sqrt(sq);
    check_sqrt(from_bits(bits(sq) + 1));
    check_sqrt(from_bits(bits(sq) - 1));
    // products of two doubles rounded: near-tie square roots
    const double r = make(0, 1023, frac());
    check_sqrt(r * r);
    check_sqrt(from_bits(bits(r * r) + 1));
  }
  std::printf("checked %" PRIu64 " (division failures %" PRIu64 ", square root failures %" PRIu64
              ", add/sub/mul/widen failures %" PRIu64 ") bad %" PRIu64 "\n",
              checked, bad_div, bad_sqrt, bad_arith, bad);
  return bad == 0 ? 0 : 1;
}
