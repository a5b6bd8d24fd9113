// Float-float ("dd") arithmetic: a value is the unevaluated sum hi + lo of
// two floats with |lo| <= ulp(hi), about 48 significant bits. GB300 issues
// FP32 at about 58 times its FP64 rate, so the assembly kernels evaluate
// their FP64 formulas in this representation on the FP32 pipes.
//
// Algorithms: Knuth's two-sum and Dekker's fast two-sum (error-free
// additions), the FMA two-product, and the "sloppy" double-word addition
// and multiplication of the QD library (Hida, Li, Bailey 2001), applied to
// float pairs. Error bounds, with u = 2^-24:
//   add:  |err| <= 2 u^2 (|a| + |b|)      (relative to the operand sizes,
//                                          not to the possibly cancelling sum)
//   mul:  |err| <= 4 u^2 |a b|
//   rcp:  |err| <= 3 u^2 / |x|            (one Newton step from a float seed)
// Conversions from double keep the top 48 significand bits (the split error
// is <= 2^-48 relative); dd -> double rounds hi + lo once. The
// exponent range is the float range: |x| >= 2^128 becomes infinite, and
// below 2^-126 the precision degrades gradually (subnormal lo, then hi).
//
// The functions are host-callable too (the CPU tests check the bounds above
// against long double). Nothing here relies on reassociation; FMA
// contraction of a*b+c is harmless because every product is explicit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define NW_HD __host__ __device__ __forceinline__
#else
#define NW_HD inline
#endif

namespace nw {

struct dd {
  float hi, lo;
};

NW_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
NW_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
NW_HD uint64_t d2u(double d) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(d));
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
NW_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
NW_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
NW_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);  // never contracted into an FMA
#else
  return a + b;
#endif
}
NW_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
NW_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// s + e = a + b exactly (Knuth)
NW_HD dd two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
  return {s, e};
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
NW_HD dd fast_two_sum(float a, float b) {
  const float s = fadd(a, b);
  return {s, fsub(b, fsub(s, a))};
}

NW_HD dd dd_from_float(float f) { return {f, 0.0f}; }

NW_HD int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz(int(x));
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

// Exact widening of a float to double with integer operations only (no
// conversion instruction: on GB300 those issue on the FP64 pipe). Normal,
// zero, subnormal, infinite and NaN inputs are all handled by bit moves.
NW_HD double widen(float f) {
  const uint32_t u = f2u(f);
  const uint32_t ex = (u >> 23) & 0xffu;
  const uint32_t m = u & 0x7fffffu;
  const uint64_t sign = uint64_t(u & 0x80000000u) << 32;
  uint64_t bits;
  if (ex - 1u < 0xfeu) {  // normal
    bits = (uint64_t(ex + 896u) << 52) | (uint64_t(m) << 29);
  } else if (ex == 0xffu) {  // inf / nan
    bits = (uint64_t(0x7ffu) << 52) | (uint64_t(m) << 29);
  } else if (m == 0) {  // zero
    bits = 0;
  } else {  // subnormal: m 2^-149 with the top bit of m at position k
    const int k = 31 - clz32(m);
    bits = (uint64_t(uint32_t(k + 874)) << 52) | ((uint64_t(m) << (52 - k)) & ((uint64_t(1) << 52) - 1));
  }
  return u2d(sign | bits);
}

// hi + lo rounded to the nearest double: both halves widen exactly, so the
// one FP64 add rounds the exact sum once.
NW_HD double dd_to_double(dd a) { return widen(a.hi) + widen(a.lo); }

NW_HD int f2i_rn(float x) {
#ifdef __CUDA_ARCH__
  return __float2int_rn(x);
#else
  return int(std::nearbyint(x));  // the default rounding: to nearest, ties to even
#endif
}

// hi + lo as a double without an FP64 instruction, for the row kernels that
// widen every CSR entry (GB300 issues FP64 adds at about one lane per SM
// clock, so one add per entry bounds those kernels). double(hi) is a bit
// move; lo is scaled (exactly, by a power of two) to units in the last
// place of a double in hi's binade, rounded to an integer and added to the
// magnitude bits of double(hi) (subtracted when lo has the other sign). When hi is a power of two and lo has the other sign the sum
// lies one binade lower, where the unit is half as large: lo is scaled by
// one more factor of two and the subtraction borrows into the exponent
// field, which is the pattern of the lower binade. The low 29 bits of
// double(hi) are zero and a normalised lo (|lo| <= ulp(hi) / 2) is worth at
// most 2^28 of those units, so the add never carries out of hi's binade.
// Result: hi + lo rounded to the nearest double (ties to even), within one
// unit in the last place for pairs that are not normalised. Pairs outside
// that form (hi zero, subnormal, non-finite or below
// 2^-74; lo non-finite or worth 2^29 units or more) take dd_to_double.
NW_HD double dd_to_double_int(dd a) {
  const uint32_t hb = f2u(a.hi), lb = f2u(a.lo);
  const uint32_t eh = (hb >> 23) & 0xffu;
  if (eh - 53u > 201u || (lb & 0x7f800000u) == 0x7f800000u) return dd_to_double(a);
  const uint64_t dh = (uint64_t(hb & 0x80000000u) << 32) |
                      ((uint64_t(hb & 0x7fffffffu) << 29) + (uint64_t(896u) << 52));
  const bool down = ((hb ^ lb) & 0x80000000u) != 0 && (hb & 0x7fffffu) == 0;
  // 2^(52 - e) (2^(53 - e) one binade lower), e = eh - 127 the exponent of hi
  const float scale = u2f((306u - eh + (down ? 1u : 0u)) << 23);
  // lo's units with the sign taken relative to hi's: the pattern holds |hi|
  const float t = u2f(f2u(fmul(a.lo, scale)) ^ (hb & 0x80000000u));
  if (!(fabsf(t) < 536870912.0f)) return dd_to_double(a);  // 2^29
  return u2d(dh + uint64_t(int64_t(f2i_rn(t))));
}

// Split of a double into hi (top 24 significand bits) + lo (the next 24,
// rounded), with integer operations for |x| in [2^-62, 2^127); zeros are
// exact; anything else takes the conversion instructions.
NW_HD dd dd_from_double(double x) {
  const uint64_t b = d2u(x);
  const uint32_t hw = uint32_t(b >> 32), lw = uint32_t(b);
  const int ex = int((hw >> 20) & 0x7ffu);
  const uint32_t sign = hw & 0x80000000u;
  if (ex >= 961 && ex < 1150) {
    const float hi = u2f(sign | (uint32_t(ex - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    // the remaining 29 bits are worth rest * 2^(ex - 1075)
    const float rest = float(lw & 0x1fffffffu);  // exact up to 2^24, rounded above
    const float scale = u2f(uint32_t(ex - 1075 + 127) << 23);
    // |lo| < ulp(hi): the pair is used as it is (the double-word
    // operations only need |lo| below ulp(hi), not a rounded split)
    return {hi, u2f(f2u(fmul(rest, scale)) | sign)};
  }
  if ((b << 1) == 0) return {u2f(sign), 0.0f};
  const float hi = float(x);
  if (!(fabsf(hi) < INFINITY)) return {hi, 0.0f};  // beyond the float range
  return {hi, float(x - double(hi))};
}

NW_HD dd operator-(dd a) { return {-a.hi, -a.lo}; }

// sloppy double-word addition
NW_HD dd operator+(dd a, dd b) {
  const dd s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, fadd(s.lo, fadd(a.lo, b.lo)));
}
NW_HD dd operator-(dd a, dd b) { return a + (-b); }
NW_HD dd operator+(dd a, float b) {
  const dd s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, fadd(s.lo, a.lo));
}

NW_HD dd operator*(dd a, dd b) {
  const float p = fmul(a.hi, b.hi);
  float e = ffma(a.hi, b.hi, -p);
  e = ffma(a.hi, b.lo, e);
  e = ffma(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
NW_HD dd operator*(dd a, float b) {
  const float p = fmul(a.hi, b);
  float e = ffma(a.hi, b, -p);
  e = ffma(a.lo, b, e);
  return fast_two_sum(p, e);
}
// exact scaling by a power of two (no overflow / underflow assumed)
NW_HD dd scale2(dd a, float p2) { return {fmul(a.hi, p2), fmul(a.lo, p2)}; }

NW_HD dd dd_fma(dd a, dd b, dd c) { return a * b + c; }

// A running sum of float pairs with the renormalisation deferred to the
// end: s is the two-sum head, c the float sum of the heads' rounding errors
// and of the low parts (8 operations per term against 11 for the pair
// addition). After k terms the error is within about k^2 u^2 of the sum of
// |terms| (u = 2^-24), which the host test checks against long double.
struct dd_acc {
  float s = 0.0f, c = 0.0f;
};
NW_HD void acc_add(dd_acc& a, dd x) {
  const dd t = two_sum(a.s, x.hi);
  a.s = t.hi;
  a.c = fadd(a.c, fadd(t.lo, x.lo));
}
NW_HD dd acc_value(const dd_acc& a) { return fast_two_sum(a.s, a.c); }

// a0 b0 + a1 b1 + a2 b2: the three FMA two-products (head + error), the
// heads added with two error-free sums, every error term added in float,
// one final renormalisation. 31 float operations against 43 for three
// products and two additions; the error stays a few u^2 times the sum of
// |a_i b_i| (u = 2^-24), as for the separate operations.
NW_HD dd dd_dot3(dd a0, dd b0, dd a1, dd b1, dd a2, dd b2) {
  const float p0 = fmul(a0.hi, b0.hi), p1 = fmul(a1.hi, b1.hi), p2 = fmul(a2.hi, b2.hi);
  float e0 = ffma(a0.hi, b0.hi, -p0), e1 = ffma(a1.hi, b1.hi, -p1), e2 = ffma(a2.hi, b2.hi, -p2);
  e0 = ffma(a0.lo, b0.hi, ffma(a0.hi, b0.lo, e0));
  e1 = ffma(a1.lo, b1.hi, ffma(a1.hi, b1.lo, e1));
  e2 = ffma(a2.lo, b2.hi, ffma(a2.hi, b2.lo, e2));
  const dd s01 = two_sum(p0, p1);
  const dd s = two_sum(s01.hi, p2);
  const float err = fadd(fadd(fadd(e0, e1), e2), fadd(s01.lo, s.lo));
  return fast_two_sum(s.hi, err);
}

// 1/x: float seed refined by one Newton step in double-word arithmetic.
// x == 0 gives inf (as the FP64 reciprocal does); non-finite x its float
// reciprocal.
NW_HD dd dd_rcp(dd x) {
  x = fast_two_sum(x.hi, x.lo);  // |lo| <= ulp(hi)/2 keeps the seed within 2^-23
  const float r0 = 1.0f / x.hi;
  if (x.hi == 0.0f || !(fabsf(r0) < INFINITY)) return {r0, 0.0f};
  // e = 1 - x r0 with the product kept to 48 bits
  const float p = fmul(x.hi, r0);
  float pe = ffma(x.hi, r0, -p);
  pe = ffma(x.lo, r0, pe);
  const float e = fsub(fsub(1.0f, p), pe);
  return fast_two_sum(r0, fmul(r0, e));
}

NW_HD dd dd_abs(dd a) { return a.hi < 0.0f ? -a : a; }
NW_HD bool dd_gt0(dd a) { return a.hi > 0.0f; }
NW_HD bool dd_lt(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
NW_HD dd dd_min(dd a, dd b) { return dd_lt(b, a) ? b : a; }

}  // namespace nw
