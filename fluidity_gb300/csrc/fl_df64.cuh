// fl_df64.cuh -- double-float ("df64") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The operations are the classical error-free
// transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the FMA-based
// TwoProduct (Ogita, Rump and Oishi, "Accurate sum and dot product", 2005),
// combined into the usual "sloppy" double-float add and multiply.  Every
// operation has an absolute error of a few units of 2^-48 of its operands'
// magnitudes, which is what a row-scaled 1e-12 tolerance needs.
//
// GB300 executes FP64 at about 1/60 of its FP32 rate, so element kernels that
// need ~1e-14 accuracy run their arithmetic here and keep FP64 for the few
// operations that must see every bit of a double input.  The compiler must
// not reassociate these operations (no fast-math), which is the default.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace fl {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ df df_fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return {s, e};
}

__device__ __forceinline__ df df_add(df x, df y) {
  const df s = df_two_sum(x.hi, y.hi);
  const float e = s.lo + (x.lo + y.lo);
  return df_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df df_neg(df x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return df_fast_two_sum(p, e);
}

// x*y - z*w with one renormalisation (cofactors).
__device__ __forceinline__ df df_mul_sub_mul(df x, df y, df z, df w) {
  const float p = x.hi * y.hi;
  const float q = z.hi * w.hi;
  float ep = fmaf(x.hi, y.hi, -p);
  float eq = fmaf(z.hi, w.hi, -q);
  ep = fmaf(x.hi, y.lo, ep);
  ep = fmaf(x.lo, y.hi, ep);
  eq = fmaf(z.hi, w.lo, eq);
  eq = fmaf(z.lo, w.hi, eq);
  const df s = df_two_sum(p, -q);
  return df_fast_two_sum(s.hi, s.lo + (ep - eq));
}

// a0*b0 + a1*b1 + a2*b2 with one renormalisation.
__device__ __forceinline__ df df_dot3(df a0, df b0, df a1, df b1, df a2, df b2) {
  const float p0 = a0.hi * b0.hi, p1 = a1.hi * b1.hi, p2 = a2.hi * b2.hi;
  float e = fmaf(a0.hi, b0.hi, -p0);
  e += fmaf(a1.hi, b1.hi, -p1);
  e += fmaf(a2.hi, b2.hi, -p2);
  e = fmaf(a0.hi, b0.lo, e);
  e = fmaf(a0.lo, b0.hi, e);
  e = fmaf(a1.hi, b1.lo, e);
  e = fmaf(a1.lo, b1.hi, e);
  e = fmaf(a2.hi, b2.lo, e);
  e = fmaf(a2.lo, b2.hi, e);
  const df s01 = df_two_sum(p0, p1);
  const df s = df_two_sum(s01.hi, p2);
  return df_fast_two_sum(s.hi, s.lo + (s01.lo + e));
}

__device__ __forceinline__ df df_abs(df x) { return x.hi < 0.0f ? df_neg(x) : x; }

// 1/x by one Newton step from the FP32 reciprocal: r1 = r0 + r0 (1 - x r0),
// with the residual 1 - x r0 formed exactly enough in double-float.
__device__ __forceinline__ df df_rcp(df x) {
  const float r0 = 1.0f / x.hi;
  const float p = x.hi * r0;
  const float pe = fmaf(x.hi, r0, -p);
  const float res = ((1.0f - p) - pe) - x.lo * r0;  // 1 - x r0
  return df_fast_two_sum(r0, r0 * res);
}

// Conversion path of df_from_double, kept out of line so that the common
// path carries no FP64 instruction (an inlined branch this short would be
// predicated and executed by every thread).
static __device__ __noinline__ df df_from_double_rare(double d) {
  const float hi = __double2float_rn(d);
  return {hi, __double2float_rn(d - (double)hi)};
}

// Exact-or-nearly split of a double into hi + lo by slicing its bits (no FP64
// or conversion-pipe instruction on the common path): hi keeps the leading 24
// significand bits, lo the remaining 29 rounded to 24 (exact when the double
// has at most 48 significant bits).  Zeros are split by bits too; magnitudes
// outside [2^-70, 2^100], infinities and NaNs take the conversion path.
__device__ __forceinline__ df df_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const int exp = (int)((hw >> 20) & 0x7ffu);
  if (exp < 1023 - 70 || exp > 1023 + 100) {
    if ((b << 1) == 0ull) return {__uint_as_float(hw & 0x80000000u), 0.0f};  // signed zero
    return df_from_double_rare(d);
  }
  const uint32_t sign = hw & 0x80000000u;
  const uint32_t fb = sign | ((uint32_t)(exp - 1023 + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  const float hi = __uint_as_float(fb);
  // lo = rem * 2^(exp - 1075) for the 29 remaining bits, rounded down to 23:
  // a float 2^E0 * (1 + m 2^-23) with m = rem >> 6 minus 2^E0 is exactly
  // m 2^(E0-23) (Sterbenz), so no normalisation instruction is needed.
  const uint32_t rem = lw & 0x1fffffffu;
  const uint32_t e0 = (uint32_t)(exp - 1046 + 127) << 23;
  float lo = __uint_as_float(e0 | (rem >> 6)) - __uint_as_float(e0);
  if (sign) lo = -lo;
  return {hi, lo};
}

// Host-side split of a double constant.
inline df df_host(double d) {
  const float hi = (float)d;
  return {hi, (float)(d - (double)hi)};
}

// Exact float -> double by bits (GB300 runs F2F conversions on the FP64 pipe at
// FP64 rate; this uses the integer pipe).  Zero and subnormal floats map to
// a signed zero (magnitudes below 2^-126 do not occur in assembled values).
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  const uint32_t sign = b & 0x80000000u;
  if (e == 0u) return __hiloint2double((int)sign, 0);
  if (e == 0xffu) return (double)f;  // inf / nan: keep IEEE semantics
  const uint32_t m = b & 0x7fffffu;
  const uint32_t hi = sign | ((e + 896u) << 20) | (m >> 3);
  const uint32_t lo = m << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// hi + lo as one double: exact conversions by bits, one FP64 add.
__device__ __forceinline__ double df_to_double(df x) { return f2d_bits(x.hi) + f2d_bits(x.lo); }

}  // namespace fl
