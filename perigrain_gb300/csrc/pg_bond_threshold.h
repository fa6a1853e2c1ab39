// Threshold form of the bond rule: the reference keeps the pair (i, j) when
// sqrt(s) <= delta, s the FP64 sum of squared coordinate differences (exp_dict.py:171-222). IEEE
// sqrt rounded to nearest is monotone in s, so the passing s form an interval [0, s_max]; the
// builder compares s <= s_max and decides every pair as the reference does without the square
// root. Host code (pg_bonds.cu computes s_max once per build).
#pragma once
#include <cfloat>
#include <cmath>

namespace pg {

// The largest double s with sqrt(s) <= delta: NaN for a NaN delta (no s passes), -inf for
// delta < 0 (sqrt(s) >= 0 > delta, and sqrt(-0) = -0 is not <= delta either), +inf for
// delta = +inf (every s but NaN passes).
inline double bond_s_max(double delta) {
  if (std::isnan(delta)) return NAN;
  if (delta < 0) return -INFINITY;
  if (std::isinf(delta)) return INFINITY;
  double t = delta * delta;
  if (std::isinf(t)) t = DBL_MAX;
  while (t < DBL_MAX && std::sqrt(std::nextafter(t, INFINITY)) <= delta) t = std::nextafter(t, INFINITY);
  while (t > 0 && !(std::sqrt(t) <= delta)) t = std::nextafter(t, 0.0);
  return t;
}

}  // namespace pg
