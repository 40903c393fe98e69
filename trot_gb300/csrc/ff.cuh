// Float-float (pairs of FP32 values) arithmetic and conversions that avoid the FP64
// pipe, shared by the mixed-precision kernels (mixed.cu) and the CISD kernels (cisd.cu).
#pragma once
#include "common.cuh"

namespace trot {

struct ff { float hi, lo; };
// The error-free transformations below rely on the rounded value of every sum and
// product, so they use the _rn intrinsics, which the compiler never contracts into FMAs.
TROT_D ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
TROT_D ff ff_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
TROT_D ff ff_add(ff x, ff y) {
  ff s = ff_two_sum(x.hi, y.hi);
  return ff_fast(s.hi, __fadd_rn(__fadd_rn(s.lo, x.lo), y.lo));
}
TROT_D ff ff_sub(ff x, ff y) { return ff_add(x, ff{-y.hi, -y.lo}); }
TROT_D ff ff_mul(ff x, ff y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return ff_fast(p, e);
}
// float -> double by moving the bits (exact for normal floats; zero, subnormal, inf and
// NaN take the conversion instruction)
TROT_D double f2d_bits(float f) {
  const unsigned v = (unsigned)__float_as_int(f);
  const unsigned e = (v >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned long long d = ((unsigned long long)(v & 0x80000000u) << 32) |
                               ((unsigned long long)(e - 127u + 1023u) << 52) |
                               ((unsigned long long)(v & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}
TROT_D double ff_d(ff x) { return f2d_bits(x.hi) + f2d_bits(x.lo); }
// 2^e as a float for e in [-126, 127] (exact; the exponents here stay far inside)
TROT_D float pow2f(int e) { return __int_as_float((e + 127) << 23); }
TROT_D ff ff_shfl_xor(ff x, int o) {
  return ff{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)};
}
// acc += a b (float-float operands): exact product of the high parts (TwoProd) plus
// the cross terms; the high parts are summed with TwoSum and the low parts in plain
// FP32, renormalised once by the caller (ff_fast) after at most a few dozen terms.
TROT_D void ff_mad(ff& acc, ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const ff t = ff_two_sum(acc.hi, p);
  acc.hi = t.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t.lo, e));
}

struct ffc { ff re, im; };
// Split a double into float-float with integer operations only (conversions and
// double arithmetic run on the FP64 pipe, a few operations per clock per SM on this
// GPU): hi = the top 24 significant bits (truncated), lo = the next 29 bits rounded to
// a float, so hi + lo = x to 2^-48 relative.  Values below 2^-126 give 0; values past
// the float range give inf; NaN and inf pass through.
TROT_D ff ff_from_d(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex == 0x7FF) return ff{__double2float_rn(x), 0.f};
  const int ef = ex - 1023 + 127;
  if (ex == 0 || ef <= 0) return ff{__int_as_float((int)sign), 0.f};
  if (ef >= 255) return ff{__int_as_float((int)(sign | 0x7F800000u)), 0.f};
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  const float hi = __int_as_float((int)(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29)));
  const float r = __uint2float_rn((unsigned)(m & 0x1FFFFFFFull));
  const int sc = ex - 1075;  // rem * 2^(ex - 1023 - 52)
  float lo = sc >= -126 ? r * pow2f(sc) : ldexpf(r, sc);
  return ff{hi, sign ? -lo : lo};
}
TROT_D ff ff_fma(ff acc, ff a, ff b) { return ff_add(acc, ff_mul(a, b)); }

// Round-to-nearest-even double -> float by integer operations (the conversion instruction
// runs on the FP64 pipe); subnormal results flush to zero, NaN and inf pass through.
TROT_D float d2f_bits(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex == 0x7FF) return __double2float_rn(x);
  const int ef = ex - 1023 + 127;
  if (ex == 0 || ef <= 0) return __int_as_float((int)sign);
  if (ef >= 255) return __int_as_float((int)(sign | 0x7F800000u));
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  const unsigned long long r = m + 0x0FFFFFFFull + ((m >> 29) & 1ull);  // round half to even at bit 29
  // a carry out of the mantissa field increments the exponent field (up to inf)
  return __int_as_float((int)(sign | (((unsigned)ef << 23) + (unsigned)(r >> 29))));
}


// ---------------------------------------------------------------- fixed-point sums
// Integer sums are associative, so fixed-point reductions give the same bits in any
// order.  x 2^s rounded to the nearest int64 (the caller keeps |x 2^s| below 2^62);
// s is split into two float scalings so each factor stays a normal float.
TROT_D long long ff_to_fixed(ff x, int s) {
  const int s1 = max(-126, min(127, s >> 1)), s2 = max(-126, min(127, s - (s >> 1)));
  const float f1 = pow2f(s1), f2 = pow2f(s2);
  return __float2ll_rn(__fmul_rn(__fmul_rn(x.hi, f1), f2)) + __float2ll_rn(__fmul_rn(__fmul_rn(x.lo, f1), f2));
}
// Sum of an int64 over the 32 lanes of a warp (|v| < 2^57 per lane): three 21-bit
// chunks, each summed exactly by redux.sync.
TROT_D long long warp_sum_i64(long long v) {
  const int hi = (int)(v >> 42);
  const unsigned mid = (unsigned)((v >> 21) & 0x1FFFFF), lo = (unsigned)(v & 0x1FFFFF);
  const int shi = __reduce_add_sync(0xffffffffu, hi);
  const unsigned smid = __reduce_add_sync(0xffffffffu, mid), slo = __reduce_add_sync(0xffffffffu, lo);
  return ((long long)shi << 42) + ((long long)smid << 21) + (long long)slo;
}
// 2^e as a double for e in [-1022, 1023]
TROT_D double pow2d(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }

}  // namespace trot
