// Threshold form of a test sqrt(s) <= r in IEEE FP64: sqrt rounded to nearest is monotone in s,
// so the s that pass form an interval [0, sqrt_le_max(r)], and s <= sqrt_le_max(r) gives the same
// outcome for every s that a sum of squares can be (+0 or more, +inf, NaN; never negative) without
// the square root. Used by the bond builder for the reference's bond rule sqrt(s) <= delta
// (exp_dict.py:171-222) and by the force kernels to rule out contact, |x_q - x_p| <= R_c with
// R_c <= the contact radius (contact.h:737-741), before the distance itself is formed. Host code.
#pragma once
#include <cfloat>
#include <cmath>

namespace pg {

// The largest double s with sqrt(s) <= r: NaN for a NaN r (no s passes), -inf for r < 0
// (sqrt(s) >= 0 > r, and sqrt(-0) = -0 is not <= r either), +inf for r = +inf (every s but NaN
// passes).
inline double sqrt_le_max(double r) {
  if (std::isnan(r)) return NAN;
  if (r < 0) return -INFINITY;
  if (std::isinf(r)) return INFINITY;
  double t = r * r;
  if (std::isinf(t)) t = DBL_MAX;
  while (t < DBL_MAX && std::sqrt(std::nextafter(t, INFINITY)) <= r) t = std::nextafter(t, INFINITY);
  while (t > 0 && !(std::sqrt(t) <= r)) t = std::nextafter(t, 0.0);
  return t;
}

}  // namespace pg
