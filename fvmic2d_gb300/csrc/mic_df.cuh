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
// With sat, finite values beyond FP32's range saturate to +-FLT_MAX (instead of infinity), so
// that a zero weight on such a value (a node an interpolation does not use) still contributes
// zero, as in FP64, not 0 x inf = NaN.
template <bool SAT = false>
__device__ __forceinline__ df df_of(double v) {
  const long long b = dbits(v);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;  // v = 1.m 2^e
  df r;
  r.hi = (SAT && e >= 128 && e < 1024) ? (b < 0 ? -3.402823466e38f : 3.402823466e38f) : f32_trunc(v);
  // the low 29 mantissa bits are worth 2^(e - 52) each: (m 2^-52) 2^e, exact scaling down to FP32's
  // subnormal range, where it rounds gradually
  const float m = __fmul_rn((float)(unsigned)(b & 0x1FFFFFFFLL), 0x1p-52f);
  float lo = (e >= -126 && e <= 127) ? __fmul_rn(m, __int_as_float((e + 127) << 23)) : 0.0f;
  r.lo = b < 0 ? -lo : lo;
  return r;
}
// the split of v 2^-k, an exact scaling by the exponent (for values whose squares would leave
// FP32's range); zero and FP64 subnormals give zero
__device__ __forceinline__ df df_of_scaled(double v, int k) {
  const long long b = dbits(v);
  const int eb = (int)((b >> 52) & 0x7FF);
  const int e = eb - 1023 - k;
  df r;
  r.hi = eb == 0 ? 0.0f : f32_trunc(v, k);
  const float m = __fmul_rn((float)(unsigned)(b & 0x1FFFFFFFLL), 0x1p-52f);
  float lo = (eb != 0 && e >= -126 && e <= 127) ? __fmul_rn(m, __int_as_float((e + 127) << 23)) : 0.0f;
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

// a < b for normalised double-floats (|lo| at most half an ulp of hi): lexicographic on (hi, lo)
__device__ __forceinline__ bool df_lt(const df &a, const df &b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// a / b: the FP32 quotient and one correction from the double-float remainder a - b q
__device__ __forceinline__ df df_div(const df &a, const df &b) {
  const float q = __fdiv_rn(a.hi, b.hi);
  const df r = df_fma(b, df{-q, 0.0f}, a);
  return fast_two_sum(q, __fdiv_rn(r.hi, b.hi));
}
// 1 / a: the FP32 reciprocal and one Newton step, y + y (1 - a y)
__device__ __forceinline__ df df_rcp(const df &a) {
  const float y = __frcp_rn(a.hi);
  const df e = df_fma(a, df{-y, 0.0f}, df{1.0f, 0.0f});
  return df_fma(df{y, 0.0f}, e, df{y, 0.0f});
}

// 2^(j/16) for j = 0 .. 15 as double-floats (hi, lo), from 60-digit arithmetic
__device__ const float2 kExp2Sixteenths[16] = {
    {1.0f, 0.0f},
    {1.0442737340927124f, 4.8334701574503924e-08f},
    {1.0905077457427979f, -1.3077539939843064e-08f},
    {1.1387885808944702f, 5.386222312608879e-08f},
    {1.1892070770263672f, 3.797635272917432e-08f},
    {1.2418577671051025f, 4.496838101886169e-08f},
    {1.2968395948410034f, -4.018999533172973e-08f},
    {1.3542555570602417f, -1.0123349269974824e-08f},
    {1.4142135381698608f, 2.4203234971764687e-08f},
    {1.4768261909484863f, -4.500898853621038e-08f},
    {1.5422108173370361f, 8.070904833346049e-09f},
    {1.610490322113037f, 9.836217174097328e-09f},
    {1.6817928552627563f, -2.4755326677450284e-08f},
    {1.7562521696090698f, -9.235770370707996e-09f},
    {1.8340080976486206f, -1.1239277952768134e-08f},
    {1.9152065515518188f, 9.845328108326612e-09f}};
// sqrt(a) for a >= 0 in FP32's normal range: the FP32 square root and one Newton correction
// from the double-float remainder, s + (a - s^2) / (2 s)
__device__ __forceinline__ df df_sqrt(const df &a) {
  if (!(a.hi > 0.0f)) return df{0.0f, 0.0f};
  const float s = __fsqrt_rn(a.hi);
  const df r = df_fma(df{-s, 0.0f}, df{s, 0.0f}, a);
  return fast_two_sum(s, __fdiv_rn(r.hi, 2.0f * s));
}

// sqrt(x^2 + y^2) (q = 0.5: sqrt(0.5 x^2 + 0.5 y^2 + z^2) with z given) for FP64 inputs of any
// magnitude: scaled by the largest one's binary exponent before the double-float squares, the
// result scaled back exactly
__device__ __forceinline__ double df_norm(double x, double y, double z, bool half_xy) {
  const int ex = exp2_of(fabs(x)), ey = exp2_of(fabs(y)), ez = exp2_of(fabs(z));
  const int k = max(ex, max(ey, ez));
  if (k < -1000 || k > 1000) return half_xy ? sqrt(0.5 * (x * x + y * y) + z * z) : sqrt(x * x + y * y + z * z);
  const df xs = df_of_scaled(x, k), ys = df_of_scaled(y, k), zs = df_of_scaled(z, k);
  df q = df_fma(xs, xs, df_mul(ys, ys));
  if (half_xy) q = df_scale(q, 0.5f);
  q = df_fma(zs, zs, q);
  const double r = df_to_f64(df_sqrt(q));
  // times 2^k, exactly: r is in [2^-1, 2^1] or zero
  return __longlong_as_double(dbits(r) == 0 ? 0LL : dbits(r) + ((long long)k << 52));
}

// interp_w (mic_internal.cuh) in double-float arithmetic: sum_k w_k f_k over the cell's four
// nodes in the same order, the weights given as double-floats, the node values split on load
__device__ __forceinline__ df interp_w_df(const double *__restrict__ f, int NX, int i, int j, const df w[4]) {
  const size_t r0 = (size_t)j * NX, r1 = r0 + NX;
  const int i1 = next_col(i, NX);
  df s = df_mul(w[0], df_of<true>(__ldg(f + r0 + i)));
  s = df_fma(w[1], df_of<true>(__ldg(f + r1 + i)), s);
  s = df_fma(w[2], df_of<true>(__ldg(f + r0 + i1)), s);
  return df_fma(w[3], df_of<true>(__ldg(f + r1 + i1)), s);
}
// the four corner weights of a W4 (w00, w01, w10, w11: interp_w's order) as double-floats
__device__ __forceinline__ void w4_df(const W4 &w, df out[4]) {
  out[0] = df_of(w.w00);
  out[1] = df_of(w.w01);
  out[2] = df_of(w.w10);
  out[3] = df_of(w.w11);
}

// ln 2 / 16 and ln 2 as double-floats
#define kLn2Over16 (df{0.043321698904037476f, -1.1904088825787085e-10f})
#define kLn2 (df{0.6931471824645996f, -1.9046542121259336e-09f})

// exp(x) for x in about [-87, 88] (the result in FP32's normal range), relative error near 1e-11
// (Tang's table-driven method): x = k ln2/16 + r with k = round(16 x / ln 2) and |r| <= ln2/32,
// exp(x) = 2^(k div 16) 2^((k mod 16) / 16) exp(r), 2^(j/16) from the table and exp(r) = 1 + r + t
// with the tail t = r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720) in FP32 (|t| < 2.4e-4: its
// rounding is below 2e-11, the truncation below 1e-15).
__device__ __forceinline__ df df_exp(const df &x) {
  // (callers keep x in range; the clamp only keeps the exponent arithmetic below valid)
  const float kf = fminf(fmaxf(rintf(__fmul_rn(x.hi, 23.083120346069336f)), -2016.0f), 2016.0f);
  const df r = df_fma(df{-kf, 0.0f}, kLn2Over16, x);
  const float h = r.hi;
  const float t = __fmul_rn(
      __fmul_rn(h, h),
      __fmaf_rn(h, __fmaf_rn(h, __fmaf_rn(h, __fmaf_rn(h, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f), 1.0f / 6.0f),
                0.5f));
  const df one_r = two_sum(1.0f, r.hi);
  const df e = fast_two_sum(one_r.hi, __fadd_rn(one_r.lo, __fadd_rn(r.lo, t)));
  const int k = (int)kf;
  const float2 tb = __ldg(&kExp2Sixteenths[k & 15]);
  const float p2 = __int_as_float(((k >> 4) + 127) << 23);  // 2^(k div 16), k div 16 in [-126, 126]
  return df_scale(df_mul(e, df{tb.x, tb.y}), p2);
}

}  // namespace mic
