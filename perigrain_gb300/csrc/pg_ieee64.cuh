// Correctly rounded FP64 arithmetic computed on the integer and FP32 pipes: division and square
// root (used by the FP64 force kernel and the packing ascent), multiplication (the FP64 force
// kernel's squared bond length), addition, subtraction, FP32 -> FP64 conversion and an ordered
// compare against a non-negative threshold.
//
// GB300 executes FP64 arithmetic at about 1/64 of its FP32 rate, and an IEEE FP64 division or
// square root expands to about ten FP64 instructions, while the integer and FP32 pipes are some
// thirty to sixty times wider. These routines return exactly the IEEE round-to-nearest-even result,
// the bits of `a / b` and `sqrt(x)`, whenever operands and result are normal numbers, and for a
// zero dividend over a normal divisor; every other case (zero divisor or radicand, subnormal,
// infinite or NaN operands, a result outside the normal range) is passed to the FP64 hardware
// operation, so the functions are drop-in replacements bit for bit.
//
// Division (schoolbook long division with a reciprocal estimate, Knuth TAOCP vol. 2 section 4.3.1,
// in the form of division by a precomputed reciprocal of Granlund and Montgomery 1994). With
// ma, mb the 53-bit significands and k in {53, 54} chosen so that Q = floor(ma 2^k / mb) lies in
// [2^53, 2^54), Q is developed in three digits of 20, 20 and k - 40 bits. A 31-bit estimate
// y ~ 2^83 / mb (an FP32 reciprocal of the divisor's top 24 bits, relative error below 2^-21)
// gives each digit as floor(R y / 2^(83 - s)) from the running remainder R; the remainder update
// R <- R 2^s - q mb is exact in 64-bit two's complement arithmetic because its true value stays
// below 2 mb < 2^54 in magnitude. After the last digit the remainder lies in (-mb/64, 1.02 mb), so
// one correction step makes 0 <= R < mb. Q's lowest bit is the guard bit of the 53-bit result and
// R != 0 is the sticky bit, which settles round-to-nearest-even.
//
// Square root (two-stage integer square root with Newton refinement and remainder correction,
// Zimmermann, "Karatsuba square root", INRIA RR-3805, 1999, in a fixed two-level form). With
// M = m 2^k, k in {54, 55} making the exponent even, S = floor(sqrt(M)) lies in [2^53, 2^54).
// Stage one takes A = floor(sqrt(N)) of N = M / 2^44 (the low 44 bits of M are zero), an
// integer in [2^31, 2^32): FP32 estimate, one Newton step with the exact 64-bit remainder
// N - A^2, then one +-1 correction making 0 <= N - A^2 <= 2A. Stage two extends it by 22 bits:
// S ~ A 2^22 + (N - A^2) 2^21 / A (the next term of the binomial series is below 2^-10), the
// quotient taken in FP32; one more Newton step S += (M - S^2) / (2S) from the exact remainder
// (below 2^59 in magnitude while S is within eight units) and one +-1 correction make
// 0 <= M - S^2 <= 2S, and the remainder gives the sticky bit as for the quotient.
//
// Addition, subtraction and multiplication (add_rn, sub_rn, mul_rn) and the FP32 -> FP64
// conversion (widen_f32) are provided the same way. Measured in the FP64 force kernel's bond loop
// (bond vector e = (dj - dp) + (xj - xp)) and in the mixed path's position update, the integer
// sum was slower than the FP64 instruction it replaced (about 40 integer instructions with
// branches against one FP64 add); the nearly branch-free product pays off for the squares of the
// bond length, which is where the FP64 force kernel uses it.
//
// Host and device share the code, so the routines are tested bit for bit against the host's
// IEEE operations as well as against the GPU's.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {
namespace ieee64 {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

// The device read of the bits is opaque to the optimizer: the compiler takes the sign bit of
// fabs(x) as clear, while the GPU's FP64 absolute value keeps the sign of a NaN, and a check of the
// sign and exponent fields folded under that assumption sends such a NaN down the integer path.
PG_HD uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  uint64_t b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
PG_HD double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
// High 32 bits of a 32 x 32 bit product.
PG_HD uint32_t umulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
// FP32 reciprocal and reciprocal square root estimates (relative error about 2^-23). The host
// versions can be scaled by PG_IEEE64_EST_SCALE to check the correction margins against estimates
// worse than the GPU's.
#ifndef PG_IEEE64_EST_SCALE
#define PG_IEEE64_EST_SCALE 1.0f
#endif
PG_HD float rcp_est(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return (1.0f / x) * PG_IEEE64_EST_SCALE;
#endif
}
PG_HD float rsqrt_est(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return (1.0f / std::sqrt(x)) * PG_IEEE64_EST_SCALE;
#endif
}
// High 64 bits of a 64 x 64 bit product.
PG_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
// Leading zeros of a nonzero 64-bit word.
PG_HD int32_t clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}
// FP32 to int32, rounded to nearest.
PG_HD int32_t f2i_rn(float x) {
#ifdef __CUDA_ARCH__
  return __float2int_rn(x);
#else
  return (int32_t)std::nearbyint(x);
#endif
}
PG_HD double hw_div(double a, double b) { return a / b; }
PG_HD double hw_add(double a, double b) { return a + b; }
PG_HD double hw_sub(double a, double b) { return a - b; }
PG_HD double hw_mul(double a, double b) { return a * b; }
PG_HD double hw_sqrt(double x) {
#ifdef __CUDA_ARCH__
  return ::sqrt(x);
#else
  return std::sqrt(x);
#endif
}

// floor(r * y / 2^(32 + sh)) for |r| < 2^62 and 0 < y < 2^31.
PG_HD int64_t mul_shift(int64_t r, int32_t y, int sh) {
  const int32_t rh = (int32_t)(r >> 32);
  const uint32_t rl = (uint32_t)(uint64_t)r;
  const int64_t p = (int64_t)rh * (int64_t)y + (int64_t)umulhi32(rl, (uint32_t)y);
  return p >> sh;
}

// A divisor prepared once for several quotients.
struct Divisor {
  uint64_t m;  // significand with the hidden bit
  int32_t y;   // ~ 2^83 / m, relative error below 2^-21
  int32_t e;   // biased exponent; 0 routes every quotient to the hardware
  uint64_t s;  // sign bit
  double b;    // the divisor itself, for the hardware route
};

PG_HD Divisor make_divisor(double b) {
  const uint64_t bb = bits(b);
  Divisor d;
  d.b = b;
  d.s = bb & kSign;
  d.m = (bb & kFrac) | kHidden;
  const int32_t e = (int32_t)((bb >> 52) & 0x7ff);
  d.e = e == 0x7ff ? 0 : e;
  // top 24 bits of the significand, exact in FP32: x in [2^23, 2^24), y ~ 2^54 / x
  const float x = (float)(uint32_t)(d.m >> 29);
  float r = rcp_est(x) * 18014398509481984.0f;  // 2^54
  r = r < 2147483520.0f ? r : 2147483520.0f;    // largest FP32 below 2^31
  d.y = (int32_t)r;
  return d;
}

// IEEE round-to-nearest-even quotient a / d.b.
PG_HD double div_rn(double a, const Divisor& d) {
  const uint64_t ab = bits(a);
  const int32_t ea = (int32_t)((ab >> 52) & 0x7ff);
  const uint64_t ma = (ab & kFrac) | kHidden;
  const int32_t lt = ma < d.m ? 1 : 0;  // significand quotient below 1: develop one more bit
  const int32_t be = ea - d.e + 1023 - lt;
  if (ea == 0 || ea == 0x7ff || d.e == 0 || be < 1 || be > 2045) {
    // a zero over a normal divisor is a zero with the product of the signs
    if ((ab << 1) == 0 && d.e != 0) return from_bits((ab ^ d.s) & kSign);
    return hw_div(a, d.b);
  }
  const uint64_t mb = d.m;
  const int32_t s3 = 13 + lt;  // k - 40
  // digit 1: q ~ ma / mb 2^20
  int64_t q = mul_shift((int64_t)ma, d.y, 31);
  uint64_t r = (ma << 20) - (uint64_t)q * mb;
  // digit 2
  int64_t t = mul_shift((int64_t)r, d.y, 31);
  r = (r << 20) - (uint64_t)t * mb;
  q = (int64_t)(((uint64_t)q << 20) + (uint64_t)t);
  // digit 3
  t = mul_shift((int64_t)r, d.y, 51 - s3);
  r = (r << s3) - (uint64_t)t * mb;
  uint64_t Q = ((uint64_t)q << s3) + (uint64_t)t;
  // 0 <= r < mb
  if ((int64_t)r < 0) {
    Q -= 1;
    r += mb;
  } else if (r >= mb) {
    Q += 1;
    r -= mb;
  }
  // Q in [2^53, 2^54): 53-bit significand, guard bit, and the remainder as the sticky bit
  uint64_t M = Q >> 1;
  M += (Q & 1ull) & ((r != 0 ? 1ull : 0ull) | (M & 1ull));
  // a carry out of the significand (M == 2^53) moves into the exponent field
  return from_bits(((ab ^ d.s) & kSign) | (((uint64_t)be << 52) + M - kHidden));
}

PG_HD double div_rn(double a, double b) { return div_rn(a, make_divisor(b)); }

// IEEE round-to-nearest-even square root.
PG_HD double sqrt_rn(double x) {
  const uint64_t xb = bits(x);
  const int32_t ex = (int32_t)((xb >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff || (xb & kSign)) return hw_sqrt(x);
  const uint64_t m = (xb & kFrac) | kHidden;
  // x = m 2^(ex - 1075); k = 54, or 55 when ex - 1075 is odd, makes the exponent of M = m 2^k even
  const int32_t odd = (ex & 1) ^ 1;
  const int32_t k = 54 + odd;
  const int32_t be = (ex + 1023 - odd) >> 1;
  // stage one: A = floor(sqrt(N)), N = M / 2^44 in [2^62, 2^64)
  const uint64_t N = m << (10 + odd);
  const float nf = (float)(uint32_t)(N >> 32);
  float af = nf * rsqrt_est(nf) * 65536.0f;
  af = af < 4294967040.0f ? af : 4294967040.0f;  // largest FP32 below 2^32
  uint64_t A = (uint64_t)(uint32_t)af;
  int64_t D = (int64_t)(N - A * A);  // |D| < 2^44
  // Newton step A += D / (2A), the quotient in FP32
  const float df = (float)(int32_t)(D >> 16);
  A = (uint64_t)((int64_t)A + (int64_t)f2i_rn(df * (32768.0f * rcp_est(af))));
  D = (int64_t)(N - A * A);
  // A is within one of floor(sqrt N): the step lands within 1/2 + 2^-8 of sqrt N (rounded FP32
  // quotient, quadratic error below 2^-8)
  if (D < 0) {
    A -= 1;
    D += (int64_t)(2 * A + 1);
  } else if ((uint64_t)D > 2 * A) {
    D -= (int64_t)(2 * A + 1);
    A += 1;
  }
  // stage two: S ~ A 2^22 + D 2^21 / A, D in [0, 2A]
  const float ra = rcp_est((float)(uint32_t)A);
  uint64_t S = (A << 22) + (uint64_t)(uint32_t)((float)(uint32_t)((uint64_t)D >> 2) * (8388608.0f * ra));
  const uint64_t Mlo = m << k;
  int64_t R = (int64_t)(Mlo - S * S);  // M - S^2, exact: |M - S^2| < 2^59 while S is within 2^3
  // one more step S += R / (2S) from the exact remainder, rounded to nearest, lands within
  // 1/2 + 2^-8 of sqrt M, so S is within one of floor(sqrt M)
  S = (uint64_t)((int64_t)S + (int64_t)f2i_rn((float)(int32_t)(R >> 28) * (32.0f * ra)));
  R = (int64_t)(Mlo - S * S);
  if (R < 0) {
    S -= 1;
    R += (int64_t)(2 * S + 1);
  } else if ((uint64_t)R > 2 * S) {
    R -= (int64_t)(2 * S + 1);
    S += 1;
  }
  uint64_t Mt = S >> 1;
  Mt += (S & 1ull) & ((R != 0 ? 1ull : 0ull) | (Mt & 1ull));
  return from_bits(((uint64_t)be << 52) + Mt - kHidden);
}

// Core of the IEEE round-to-nearest-even sum of two doubles given by their bits (b's sign already
// flipped for a difference); `ok` is cleared, and the result is to be taken from the hardware,
// unless both operands are normal and so is the result, or b is a zero and a is normal.
// Method: the operand of larger magnitude keeps its exponent, the other significand is shifted
// right with the shifted-out bits jammed into its lowest bit (a sticky bit nine places below the
// guard bit), the significands are added or subtracted in 64-bit integers with the leading bit at
// bit 62, the sum is renormalised, and bits 9..0 round it to 53 bits (Goldberg, "What every
// computer scientist should know about floating-point arithmetic", 1991, section 1.4 on guard
// digits).
PG_HD uint64_t add_bits(uint64_t ab, uint64_t bb, bool* ok) {
  const uint64_t aa = ab & ~kSign, ba = bb & ~kSign;
  const bool sw = aa < ba;
  const uint64_t hb = sw ? bb : ab, lb = sw ? ab : bb;  // |h| >= |l|
  const uint64_t ha = sw ? ba : aa, la = sw ? aa : ba;
  const int32_t eh = (int32_t)(ha >> 52), el = (int32_t)(la >> 52);
  if (eh == 0x7ff || eh == 0 || el == 0) {
    *ok = la == 0 && eh != 0 && eh != 0x7ff;  // normal + zero is the normal operand
    return hb;
  }
  const uint64_t mh = ((ha & kFrac) | kHidden) << 10;
  const uint64_t ml = ((la & kFrac) | kHidden) << 10;
  const int32_t sh = eh - el;
  uint64_t mls = 1;  // only the sticky bit remains of a significand shifted by 64 or more
  if (sh < 64) {
    mls = ml >> sh;
    mls |= (mls << sh) != ml ? 1ull : 0ull;
  }
  int32_t e = eh;
  uint64_t m;
  if (((hb ^ lb) >> 63) == 0) {
    m = mh + mls;  // below 2^64
    if (m >> 63) {
      m = (m >> 1) | (m & 1ull);
      e += 1;
    }
  } else {
    m = mh - mls;
    if (m == 0) {
      *ok = true;
      return 0ull;  // an exact zero difference is +0 under round-to-nearest
    }
    const int32_t lz = clz64(m) - 1;
    m <<= lz;
    e -= lz;
  }
  *ok = e >= 1 && e <= 2045;
  const uint64_t r = m & 0x3ffull;
  uint64_t q = m >> 10;
  q += (r > 0x200ull ? 1ull : 0ull) | ((r == 0x200ull ? 1ull : 0ull) & q);
  return (hb & kSign) | (((uint64_t)e << 52) + q - kHidden);
}

// IEEE round-to-nearest-even a + b and a - b.
PG_HD double add_rn(double a, double b) {
  bool ok;
  const uint64_t r = add_bits(bits(a), bits(b), &ok);
  return ok ? from_bits(r) : hw_add(a, b);
}
PG_HD double sub_rn(double a, double b) {
  bool ok;
  const uint64_t r = add_bits(bits(a), bits(b) ^ kSign, &ok);
  return ok ? from_bits(r) : hw_sub(a, b);
}

// IEEE round-to-nearest-even a * b: the 106-bit product of the significands from a 64 x 64 bit
// multiplication, its top 53 bits rounded with the next bit and the rest as the sticky bit. A
// zero times a finite number is the signed zero; other zero, subnormal, infinite or NaN operands
// and results outside the normal range take the hardware operation.
PG_HD double mul_rn(double a, double b) {
  const uint64_t ab = bits(a), bb = bits(b);
  const int32_t ea = (int32_t)((ab >> 52) & 0x7ff), eb = (int32_t)((bb >> 52) & 0x7ff);
  const uint64_t sign = (ab ^ bb) & kSign;
  const uint64_t ma = (ab & kFrac) | kHidden, mb = (bb & kFrac) | kHidden;
  const uint64_t lo = ma * mb, hi = umulhi64(ma, mb);  // product in [2^104, 2^106)
  const int32_t top = (int32_t)(hi >> 41);               // 1 when the product is >= 2^105
  const int32_t e = ea + eb - 1023 + top;
  if (ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff || e < 1 || e > 2045) {
    if ((((ab << 1) == 0) && eb != 0x7ff) || (((bb << 1) == 0) && ea != 0x7ff)) return from_bits(sign);
    return hw_mul(a, b);
  }
  const int32_t sh = 52 + top;
  uint64_t q = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t g = (lo >> (sh - 1)) & 1ull;
  const uint64_t st = (lo & ((1ull << (sh - 1)) - 1ull)) != 0 ? 1ull : 0ull;
  q += g & (st | (q & 1ull));
  return from_bits(sign | (((uint64_t)e << 52) + q - kHidden));
}

// Exact FP32 -> FP64 conversion from the bits; subnormal, infinite and NaN inputs take the
// hardware conversion.
PG_HD double widen_f32(float x) {
#ifdef __CUDA_ARCH__
  uint32_t u;
  asm("mov.b32 %0, %1;" : "=r"(u) : "f"(x));
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
#endif
  const uint32_t ef = (u >> 23) & 0xffu;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  if (ef == 0 || ef == 0xff) {
    if ((u << 1) == 0) return from_bits(sign);
    return (double)x;
  }
  return from_bits(sign | ((uint64_t)(ef + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29));
}

// a > b for a threshold b that is +0 or more and not NaN (gt_nonneg_ok(b)), on the integer pipe:
// the bits of such numbers order as the numbers do, a NaN or negative a has bits above those of
// +inf, and a = -0 or +0 is not above any such b.
PG_HD bool gt_nonneg_ok(uint64_t b_bits) { return b_bits <= 0x7ff0000000000000ull; }
PG_HD bool gt_nonneg(double a, uint64_t b_bits) {
  const uint64_t ab = bits(a);
  return ab > b_bits && ab <= 0x7ff0000000000000ull;
}

}  // namespace ieee64
}  // namespace pg
