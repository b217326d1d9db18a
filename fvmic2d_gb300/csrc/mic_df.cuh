// mic_df.cuh -- double-float arithmetic on the FP32 pipe (product build).
//
// A value is the unevaluated sum hi + lo of two floats, about 48 significant bits.  The
// operations are the classical error-free transformations: TwoSum (Knuth) for a sum and its
// rounding error, TwoProd by a fused multiply-add (the FMA form of Dekker's product) for a product
// and its rounding error, and a FastTwoSum renormalisation (Dekker 1971).  A sum or product of
// double-floats is accurate to a few units of 2^-48 of its magnitude (of the larger operand's
// product, for a fused multiply-add).
//
// Why: GB300 issues 64 FP32 lanes for every FP64 lane, and the marker passes are bound by the FP64
// pipe.  Sums of products whose results need about 1e-14 relative accuracy (the bilinear velocity
// and vorticity interpolations of the advection, the RK4 combinations) run here on the FP32 pipe
// and enter FP64 once, by one FP64 addition of the two halves.  The range is FP32's: values below
// 2^-74 (5e-23) keep only hi's 24 bits, values below 2^-126 flush to zero.  Every operation is
// written with explicit-rounding intrinsics, so no compiler contraction can fuse a step of an
// error-free transformation.
#pragma once

#include "mic_internal.cuh"

namespace mic {

struct df {
  float hi, lo;
};

// v split into hi (its top 24 significant bits, truncated: f32_trunc) and lo (the remaining 29
// mantissa bits rounded to 24): hi + lo = v within a relative 2^-48.  Integer work and one
// integer-to-float conversion, no FP64 instruction.  Infinities and NaN give hi = v, lo = 0.
__device__ __forceinline__ df df_of(double v) {
  const long long b = dbits(v);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;  // v = 1.m 2^e
  df r;
  r.hi = f32_trunc(v);
  // the low 29 mantissa bits are worth 2^(e - 52) each: (m 2^-52) 2^e, exact scaling down to FP32's
  // subnormal range, where it rounds gradually
  const float m = __fmul_rn((float)(unsigned)(b & 0x1FFFFFFFLL), 0x1p-52f);
  float lo = (e >= -126 && e <= 127) ? __fmul_rn(m, __int_as_float((e + 127) << 23)) : 0.0f;
  r.lo = b < 0 ? -lo : lo;
  return r;
}
__device__ __forceinline__ df df_of(float v) { return {v, 0.0f}; }

// hi + lo as a double: the halves are exact doubles (bit-pattern conversions), one FP64 addition
__device__ __forceinline__ double df_to_f64(const df &a) { return f64_of(a.hi) + f64_of(a.lo); }

// TwoSum: s = fl(a + b) and the exact error a + b - s
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// FastTwoSum (|a| >= |b| or a = 0): renormalises a hi part and a small correction
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_add(const df &a, const df &b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df df_neg(const df &a) { return {-a.hi, -a.lo}; }
// exact scaling by a power of two
__device__ __forceinline__ df df_scale(const df &a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }

// a b (TwoProd of the high parts by FMA, the cross terms in FP32; lo lo dropped)
__device__ __forceinline__ df df_mul(const df &a, const df &b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return fast_two_sum(p, e);
}
// a b + c
__device__ __forceinline__ df df_fma(const df &a, const df &b, const df &c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  const df s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

}  // namespace mic
