// Host check of the mixed path's hi/lo split (split_hl in perigrain_gb300/csrc/pg_kernels_mixed.cu):
// the integer route (hi and lo assembled from the FP64 bit pattern) must give the same bits as the
// FP64 route it replaces (hi = trunc_f32(x), lo = trunc_f32(x - hi)) on random bit patterns of
// every exponent, random magnitudes and mantissas near the FP32 range edges. The two functions
// below restate the device code with host bit-cast helpers. Prints "bad 0" on success.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <cmath>
static inline unsigned long long dbits(double x) { unsigned long long b; memcpy(&b, &x, 8); return b; }
static inline double bdouble(unsigned long long b) { double x; memcpy(&x, &b, 8); return x; }
static inline float ufloat(unsigned int u) { float f; memcpy(&f, &u, 4); return f; }
static inline unsigned int fbits(float f) { unsigned int u; memcpy(&u, &f, 4); return u; }
float trunc_f32(double x, double* as_double) {
  const unsigned long long b = dbits(x);
  const unsigned int hw = (unsigned int)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7ffu);
  const unsigned int sgn = hw & 0x80000000u;
  if (e < 1023 - 126) { *as_double = 0.0; return ufloat(sgn); }
  if (e > 1023 + 127) { *as_double = x; const bool nan = (e == 0x7ff) && ((b & 0xfffffffffffffull) != 0); return ufloat(sgn | 0x7f800000u | (nan ? 0x400000u : 0u)); }
  *as_double = bdouble(b & ~((1ull << 29) - 1));
  return ufloat(sgn | ((unsigned int)(e - 896) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
}
void split_ref(double x, float* hi, float* lo) { double hd, ld; *hi = trunc_f32(x, &hd); *lo = trunc_f32(x - hd, &ld); }
void split_int(double x, float* hi, float* lo) {
  const unsigned long long b = dbits(x);
  const unsigned int hw = (unsigned int)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7ffu);
  if (e < 1023 - 126 || e > 1023 + 127) { split_ref(x, hi, lo); return; }
  const unsigned int sgn = hw & 0x80000000u;
  *hi = ufloat(sgn | ((unsigned int)(e - 896) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
  const unsigned int r = (unsigned int)(b & ((1ull << 29) - 1));
  if (r == 0) { *lo = 0.0f; return; }
  const int p = 31 - __builtin_clz(r);
  const int ed = e + p - 52;
  if (ed < 1023 - 126) { *lo = ufloat(sgn); return; }
  const unsigned int frac = (p <= 23) ? ((r << (23 - p)) & 0x7fffffu) : ((r >> (p - 23)) & 0x7fffffu);
  *lo = ufloat(sgn | ((unsigned int)(ed - 896) << 23) | frac);
}
int main() {
  std::mt19937_64 rng(1);
  long bad = 0, n = 0;
  auto check = [&](double x) {
    float h1, l1, h2, l2; split_ref(x, &h1, &l1); split_int(x, &h2, &l2); ++n;
    if (fbits(h1) != fbits(h2) || fbits(l1) != fbits(l2)) { if (bad < 10) printf("x=%a ref %a %a int %a %a\n", x, h1, l1, h2, l2); ++bad; }
  };
  for (int k = 0; k < 2000000; ++k) check(bdouble(rng()));          // random bit patterns (all exponents)
  std::uniform_real_distribution<double> U(-1, 1);
  for (int k = 0; k < 2000000; ++k) check(U(rng) * std::pow(10.0, (int)(rng() % 40) - 20));
  for (int e = 880; e < 1160; ++e) for (int k = 0; k < 2000; ++k) {  // near the range edges, sparse mantissas
    unsigned long long m = rng() & ((1ull << 52) - 1); if (k % 3 == 0) m &= ~((1ull << 29) - 1); if (k % 3 == 1) m &= (1ull << (k % 29)) | (~((1ull << 29) - 1));
    check(bdouble(((unsigned long long)(rng() & 1) << 63) | ((unsigned long long)e << 52) | m)); }
  check(0.0); check(-0.0);
  printf("checked %ld bad %ld\n", n, bad);
}
