// mic_creep.cuh -- composite ice creep (Goldsby & Kohlstedt 2001, as written in fvmic2d's
// viscosity.c:106-179) inverted for the stress at a given strain rate: material law 7.
//
// The reference evaluates the law forwards, stress -> strain rate:
//   rate(s) = C s                                          (s < 1 Pa, diffusion only)
//   rate(s) = C s + (1/B x^2.4 + 1/G x^1.8)^-1 + D x^4     (s >= 1 Pa),  x = s / 1e6
// with per-marker constants C (diffusion), G (grain-boundary sliding), B (basal slip) and
// D (dislocation creep) that depend on T, grain size d and pressure P only.  Law 7 needs the
// inverse: the stress s* at which rate(s*) equals the marker's strain-rate invariant.
//
// All powers of x come from p = x^0.2: x^1.8 = p^9, x^2.4 = p^12, x^4 = p^20, s = 1e6 p^5.
//
// Exact solve: the root of g(u) = ln rate(e^u) - ln edot, u = ln s.  g is increasing with
// slope between 1 and 4 and nearly linear.  The start is min(edot / C, 1e6 (edot / D)^(1/4))
// -- each term alone reaching edot bounds s* from above -- and a bracket is kept.
//   FMA-free parity build: Newton in u, one FP64 exp per iteration (the reference's arithmetic
//   throughout, for the bitwise comparisons of that build).
//   Product build: the iterate is p itself.  Each iteration evaluates the residual
//   rate(p) / edot - 1 exactly in FP64 (powers of p by multiplication, one division), and the
//   step -- a Halley step on g, third order -- is formed on the FP32 pipe from FP32 copies of
//   the terms; p moves by the factor exp(0.2 du), an FP64 polynomial for small steps.  Only the
//   residual decides convergence, so rounding in the step changes how fast the iterates
//   approach the root, never which root is accepted.  The FP64 pipe, the bound of this
//   solve on GB300 (2 FP64 instructions per SM per clock), then carries no transcendental
//   inside the loop.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mic_df.cuh"
#include "mic_internal.cuh"

namespace mic {

struct CreepCoef {
  double C;     // diffusion:   rate = C s
  double G;     // GBS:         rate = G x^1.8
  double B;     // basal slip:  rate = B x^2.4
  double D;     // dislocation: rate = D x^4
};

// the law's terms q = (C 1e6, G, B, D) / edot as double-floats (product build, the surrogate's
// coarse polish: creep_terms_df)
struct CreepTermsDF {
  df a, g, b, d;
};

// The per-marker grain column holds what creep_coef takes: the grain size d in the FMA-free
// parity build, d^-0.2 in the product build (1/d = g^5 and d^-1.4 = g^7 then cost multiplies,
// where d itself would cost a division, a log2 and an exp2 per marker and step).
__device__ __forceinline__ double grain_arg(double d) {
#ifdef MIC_EXACT
  return d;
#else
  return exp2(-0.2 * log2(d));
#endif
}
constexpr double kGrainDefault = 1e-3;  // metres, until mic_markers_set_grain_size

// viscosity.c:109-173: constants of the law at (T, grain argument g, P), with P clamped below at
// 1 Pa.  The FMA-free parity build evaluates each Arrhenius factor as the reference writes it.
// The product build factors exp((-Q + P V) / RT) = exp(-Q / RT) exp(P V / RT); the activation
// energies 49, 59.4, 60, 180 and 192 kJ/mol are whole multiples of 0.2 kJ/mol, so their factors
// are integer powers (245, 297, 300, 900, 960) of b = exp(-0.2 kJ/mol / RT) by repeated squaring
// and shared partial products (22 multiplies; relative error at most about one ulp of b per unit
// of the power, below 2.2e-13 for the largest, typically a quarter of that), and only b and the
// pressure factor take an exp: two exponentials instead of six (both temperature branches of a
// warp run) plus log2 and exp2.
__device__ __forceinline__ CreepCoef creep_coef(double T, double g, double P) {
  const double R = 8.3144621;
#ifdef MIC_EXACT
  if (P < 1.0) P = 1.0;
#else
  if (lt_pos(P, 1.0)) P = 1.0;  // the compares of this build by bit pattern (no FP64-pipe slot)
#endif
  const double RT = R * T;
  const double b = 4.52e-10, Vm = 1.97e-5, delta = 2.0 * b;
  const double V = -13e-6;
  CreepCoef k;
#ifdef MIC_EXACT
  const double d = g;
  const double Dv = 9.10e-4 * exp(-59.4e3 / RT);
  const double Db = 5.8e-4 * exp(-49.0e3 / RT);
  k.C = 42.0 * Vm / (RT * d * d) * (Dv + M_PI * delta / d * Db);
  const double Qg = (T < 255.0) ? 49.0e3 : 192.0e3, Ag = (T < 255.0) ? 3.9e-3 : 3.0e26;
  const double Qd = (T < 258.0) ? 60.0e3 : 180.0e3, Ad = (T < 258.0) ? 4.0e5 : 6.0e28;
  k.G = Ag / pow(d, 1.4) * exp((-Qg + P * V) / RT);
  k.D = Ad * exp((-Qd + P * V) / RT);
  k.B = 5.5e7 * exp((-60.0e3 + P * V) / RT);
#else
  const double iRT = 1.0 / RT;
  const double b1 = exp(-200.0 * iRT);
  const double b2 = b1 * b1, b4 = b2 * b2, b8 = b4 * b4, b16 = b8 * b8, b32 = b16 * b16, b64 = b32 * b32,
               b128 = b64 * b64, b256 = b128 * b128, b512 = b256 * b256;
  const double b296 = (b256 * b32) * b8;
  const double e594 = b296 * b1, e60 = b296 * b4;                          // 59.4 and 60 kJ/mol
  const double e49 = ((b128 * b64) * (b32 * b16)) * (b4 * b1);              // b^245
  const double b896 = (b512 * b256) * b128;
  const double e180 = b896 * b4, e192 = b896 * b64;                          // b^900, b^960
  const double eP = exp(P * V * iRT);
  const double Dv = 9.10e-4 * e594;
  const double Db = 5.8e-4 * e49;
  const double g2 = g * g, id = (g2 * g2) * g;  // 1/d
  k.C = 42.0 * Vm * iRT * id * id * fma(M_PI * delta * id, Db, Dv);
  const bool cold_g = lt_pos(T, 255.0), cold_d = lt_pos(T, 258.0);
  const double eg = (cold_g ? 3.9e-3 : 3.0e26) * (cold_g ? e49 : e192);
  const double ed = (cold_d ? 4.0e5 : 6.0e28) * (cold_d ? e60 : e180);
  k.G = eg * eP * (id * g2);  // d^-1.4
  k.D = ed * eP;
  k.B = 5.5e7 * e60 * eP;
#endif
  return k;
}

// rate and d(rate)/d(ln s) at s = 1e6 p^5 (s >= 1 Pa branch)
__device__ __forceinline__ void creep_rate_p(const CreepCoef &k, double p, double &f, double &df) {
  const double p2 = p * p, p4 = p2 * p2, p5 = p4 * p, p8 = p4 * p4, p9 = p8 * p, p12 = p8 * p4;
  const double p20 = p12 * p8;
  const double td = k.C * 1e6 * p5, tg = k.G * p9, tb = k.B * p12, tl = k.D * p20;
  const double isum = 1.0 / (tg + tb);  // one division for the series term and its derivative
  const double tc = tg * tb * isum;      // (1/tb + 1/tg)^-1
  f = td + tc + tl;
  df = td + tc * (2.4 * tg + 1.8 * tb) * isum + 4.0 * tl;
}

// ln r for the Newton function, with the series near 1 (no log call in the final iterations)
__device__ __forceinline__ double creep_lnratio(double r) {
  const double t = r - 1.0;
  if (fabs(t) < 1e-3) return t * fma(t, fma(t, fma(t, -0.25, 1.0 / 3.0), -0.5), 1.0);
  return log(r);
}

constexpr double kLn1e6 = 13.815510557964274;  // ln(1e6)

// Newton iterations from u (ln s) until |rate/edot - 1| <= tol or maxit; updates u, the
// bracket [ulo, uhi] (ulo may be -inf) and returns iterations used; *res = rate/edot - 1.
__device__ __forceinline__ int creep_newton(const CreepCoef &k, double edot, double &u, double &ulo, double &uhi,
                                            double tol, int maxit, double &res) {
  int it = 0;
  res = 1.0;
  const double iedot = 1.0 / edot;  // once per marker, not per iteration
  for (; it < maxit; ++it) {
    const double p = exp(0.2 * (u - kLn1e6));
    double f, df;
    creep_rate_p(k, p, f, df);
    const double r = f * iedot;
    res = r - 1.0;
    if (fabs(res) <= tol) break;
    if (res > 0.0)
      uhi = fmin(uhi, u);
    else
      ulo = fmax(ulo, u);
    double un = u - creep_lnratio(r) * f / df;
    if (!(un > ulo && un < uhi)) un = (ulo > -1e300) ? 0.5 * (ulo + uhi) : uhi - 2.0;  // safeguard
    u = un;
  }
  return it;
}

// Root u* = ln s* of the composite law (all four terms, no 1 Pa switch) by Newton from the upper
// bound min(edot / C, 1e6 (edot / D)^(1/4)); edot > 0.
__device__ __forceinline__ double creep_root_u(const CreepCoef &k, double edot, double tol, int maxit, int *iters,
                                               double *res_out) {
  const double s_lin = edot / k.C;
  const double s_dis = 1e6 * sqrt(sqrt(edot / k.D));
  double u = log(fmin(s_lin, s_dis));
  double ulo = -1e308, uhi = u + 1e-12;
  double res;
  *iters = creep_newton(k, edot, u, ulo, uhi, tol, maxit, res);
  *res_out = res;
  return u;
}

// Exact stress at strain rate edot (law 7), FMA-free parity build: returns s*, iterations in
// *iters.
__device__ __forceinline__ double creep_stress_exact_u(const CreepCoef &k, double edot, double tol, int maxit,
                                                       int *iters, double *res_out) {
  *iters = 0;
  *res_out = 0.0;
  if (!(edot > 0.0)) return 0.0;
  const double s_lin = edot / k.C;
  if (s_lin < 1.0) return s_lin;  // linear diffusion branch (viscosity.c:130-133)
  const double s = exp(creep_root_u(k, edot, tol, maxit, iters, res_out));
  // the rate jumps at s = 1 Pa where the non-linear terms switch on; a root in the jump is 1 Pa
  return s < 1.0 ? 1.0 : s;
}

// natural log of a positive normal double to FP32 accuracy, from its bit pattern: the exponent
// field, and __logf of the top 23 mantissa bits as a float in [1, 2) -- integer work and the
// FP32 pipe only (no FP64 instruction), over the whole double range, which FP32 lacks.  Zero
// gives about -709 (a huge negative log) instead of -inf; the callers take minima, where that
// acts the same.
__device__ __forceinline__ float ln_f(double v) {
  const long long b = dbits(v);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  const float mant = __int_as_float(0x3F800000 | (int)((b >> 29) & 0x7FFFFF));
  return fmaf((float)e, 0.693147181f, __logf(mant));
}

#ifndef MIC_EXACT
// ---- product-build solve: the iterate is p = (s / 1e6)^0.2 ----------------------------------

// rate(p) / edot = a p^5 + (1 / (g p^9) + 1 / (b p^12))^-1 + d p^20: the coefficients divided by
// edot once per marker, so no iteration divides by it
struct CreepTerms {
  double a, g, b, d;
};
__device__ __forceinline__ CreepTerms creep_terms(const CreepCoef &k, double iedot) {
  return {k.C * 1e6 * iedot, k.G * iedot, k.B * iedot, k.D * iedot};
}

// One evaluation at p, without a division: with S = tg + tb (the series' two terms) and
// N = (td + tl - 1) S + tg tb, the residual r - 1 is N / S, so |r - 1| <= tol is tested as
// |N| <= tol S, exactly in FP64 (the cancelling products are one FMA: their rounding is 1e-16 of
// tg tb / S <= 1).  The quotients the step needs come later, in FP32.
struct CreepEval {
  double N, S, tg, tb, td, tl, p5;
};
__device__ __forceinline__ void creep_eval(const CreepTerms &q, double p, CreepEval &e) {
  const double p2 = p * p, p4 = p2 * p2, p8 = p4 * p4;
  const double p12 = p8 * p4;
  e.tg = q.g * (p8 * p);
  e.tb = q.b * p12;
  e.p5 = p4 * p;
  e.td = q.a * e.p5;
  e.tl = q.d * (p12 * p8);
  // explicit roundings where a product meets a sum: the solve is shared by several kernels and
  // must not depend on how the compiler fuses it in each (the members of a batch and the
  // fallback of the surrogate modes reproduce the exact solve bit for bit)
  e.S = __dadd_rn(e.tg, e.tb);
  e.N = fma(__dadd_rn(__dadd_rn(e.td, e.tl), -1.0), e.S, e.tg * e.tb);
}
// |r - 1| <= tol as |N| <= tol S, compared by bit pattern (S > 0)
__device__ __forceinline__ bool creep_converged(const CreepEval &e, double tol) { return abs_le(e.N, tol * e.S); }
// the residual r - 1 (to FP32 accuracy: reported, and used for the step far from the root)
__device__ __forceinline__ double creep_residual(const CreepEval &e) { return e.N / e.S; }

// p exp(a) for a step a = 0.2 du formed in FP32: for |a| < 2^-5 as p + p d with d = exp(a) - 1
// from its series in FP32 (truncation below 2^-30 of d) and one FMA, else p times an FP32
// exponential.  The rounding of d (2^-24 of a step of at most 3 %) is below that of the FP32 step
// itself; the float-to-double conversions go by bit pattern.
__device__ __forceinline__ double creep_advance_f32(double p, float a) {
  if (fabsf(a) < 0.03125f) {
    const float d = a * fmaf(a, fmaf(a, fmaf(a, fmaf(a, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f), 0.5f), 1.0f);
    return fma(p, f64_of(d), p);
  }
  return p * f64_of(__expf(fminf(fmaxf(a, -80.0f), 80.0f)));
}

// One step from an evaluation: p exp(0.2 du) for the Halley step du in u = ln s on
// g(u) = ln r.  With r' and r'' the u-derivatives of r = td + tc + tl (term slopes 1,
// mc = 1.8 + 0.6 w for the series tc = tb w, w = tg / S, and 4; the series' log has curvature
// -0.36 w (1 - w)), g' = r'/r, g'' = r''/r - g'^2, and du = -2 g g' / (2 g'^2 - g g'').  The
// quotients come from FP32 copies (by bit pattern; N, S and tg scaled by S's binary exponent, so
// that the ratios N / S and tg / S stay in FP32 range however small the series' terms are): their
// rounding, about 1e-7 of the step, only perturbs the next iterate.  With `fine` (a tolerance
// FP32 steps cannot reach) and |r - 1| < 2^-16, g and g' are formed in FP64 from the exact N and
// S and the step decides the last digits; the small Halley correction stays FP32.
__device__ __forceinline__ double creep_advance(const CreepEval &e, double p, bool fine) {
  const int k = exp2_of(e.S);
  const float S = f32_trunc(e.S, k), tg = f32_trunc(e.tg, k), N = f32_trunc(e.N, k);
  const float tb = f32_trunc(e.tb), td = f32_trunc(e.td), tl = f32_trunc(e.tl);
  const float iS = 1.0f / S;
  const float w = tg * iS;
  const float tc = tb * w;
  const float resf = N * iS;
  const float mc = fmaf(0.6f, w, 1.8f);
  const float r1f = fmaf(tc, mc, fmaf(4.0f, tl, td));
  const float r2f = fmaf(tc, fmaf(mc, mc, -0.36f * w * (1.0f - w)), fmaf(16.0f, tl, td));
  if (!fine || !(fabsf(resf) < 0x1p-16f)) {
    const float r = __fadd_rn(__fadd_rn(td, tc), tl);
    if (!(r > 1e-30f && r < 1e30f && lt_pos(e.S, 1e30))) {
      // terms beyond FP32 range (an iterate far from the root): a step of -g / 4, which the
      // slope bound g' <= 4 keeps on the root's side
      return creep_advance_f32(p, -0.05f * ln_f(fabs(creep_residual(e) + 1.0)));
    }
    const float ir = 1.0f / r;
    const float g = fabsf(resf) < 0.5f ? log1pf(resf) : __logf(r);
    const float g1 = r1f * ir, g2 = fmaf(-g1, g1, r2f * ir);
    const float den = fmaf(-g, g2, 2.0f * g1 * g1);
    // Halley where its correction is moderate, Newton otherwise
    const float du = den > g1 * g1 ? -2.0f * g * g1 / den : -g / g1;
    return creep_advance_f32(p, 0.2f * du);
  }
  const double iS64 = 1.0 / e.S;
  const double t = e.N * iS64;
  const double g = t * fma(t, fma(t, fma(t, -0.25, 1.0 / 3.0), -0.5), 1.0);  // ln(1 + t), |t| < 2^-16
  const double w64 = e.tg * iS64;
  const double r1 = fma(e.tb * w64, fma(0.6, w64, 1.8), fma(4.0, e.tl, e.td));
  // r = 1 + t within 2^-16, so the correction g g'' / (2 g'^2) is formed with r = 1
  const float h = 1.0f - f32_trunc(g) * fmaf(-r1f, r1f, r2f) / (2.0f * r1f * r1f);
  const double a = -0.2 * (g * (1.0 + t)) / (r1 * f64_of(h));
  // exp(a) - 1 for |a| < 2e-5 to its third power (truncation below 1e-21)
  return fma(p, a * fma(a, fma(a, 1.0 / 6.0, 0.5), 1.0), p);
}

// Steps from p until |r - 1| <= tol or maxit steps were taken; [plo, phi] brackets the root
// (plo may be 0, phi infinite; compared by bit pattern, all non-negative) and a step leaving it
// bisects in ln p instead.  Returns the steps taken; conv, res and p5 belong to the final p (res
// to FP32 accuracy, at most tol in magnitude when conv).
__device__ __forceinline__ int creep_iterate(const CreepTerms &q, double &p, double plo, double phi, double tol,
                                             int maxit, bool &conv, double &res, double &p5) {
  const bool fine = tol < 1e-9;
  long long blo = dbits(plo), bhi = dbits(phi);
  CreepEval e;
  int it = 0;
  for (;; ++it) {
    creep_eval(q, p, e);
    conv = creep_converged(e, tol);
    if (conv || it >= maxit) break;
    const long long bp = dbits(p);
    if (dbits(e.N) > 0)
      bhi = min(bhi, bp);
    else
      blo = max(blo, bp);
    double pn = creep_advance(e, p, fine);
    const long long bn = dbits(pn);
    if (!(bn > blo && bn < bhi)) {
      const double lo = __longlong_as_double(blo), hi = __longlong_as_double(bhi);
      pn = (blo > 0) ? sqrt(lo * hi) : hi * 0.67032004603563930;  // e^-0.4
    }
    p = pn;
  }
  const int k = exp2_of(e.S);
  res = f64_of(f32_trunc(e.N, k) / f32_trunc(e.S, k));
  if (conv && !abs_le(res, tol)) res = copysign(tol, res);
  p5 = e.p5;
  return it;
}

// the exact solve from the upper bound min(x_lin, x_dis) (as p, FP32 logs, raised by 1e-4 so
// that their rounding cannot put it below the root); s >= 1 Pa branch
__device__ __forceinline__ double creep_solve_terms(const CreepTerms &q, double tol, int maxit, int *iters,
                                                    double *res_out) {
  const float lp = fminf(-0.2f * ln_f(q.a), -0.05f * ln_f(q.d));
  double p = f64_of(__expf(lp) * 1.0001f), res, p5;
  bool conv;
  *iters = creep_iterate(q, p, 0.0, INFINITY, tol, maxit, conv, res, p5);
  *res_out = res;
  const double s = 1e6 * p5;
  // the rate jumps at s = 1 Pa where the non-linear terms switch on; a root in the jump is 1 Pa
  return lt_pos(s, 1.0) ? 1.0 : s;
}

// ---- product build, surrogate polish at a coarse tolerance: double-float arithmetic --------
//
// The surrogate's polish stops at |rate/edot - 1| <= polish_tol (1e-7 by default: the stress is
// then within 1e-7 of the root).  For polish tolerances from kCoarseTol up, the law's terms and
// the polish run in double-float arithmetic on the FP32 pipe (mic_df.cuh), with no FP64
// instruction: the terms to a relative 1e-11 (which moves the root by no more than that, a
// hundredth of the smallest such tolerance) and the residual r - 1 to 1e-13.  A marker the
// polish does not bring below the tolerance, or whose terms leave FP32's range, takes the exact
// FP64 solve (its coefficients recomputed in FP64).
constexpr double kCoarseTol = 1e-9;

// q from (T, grain argument g, P, 1 / edot).  Each Arrhenius factor is one exponential of its
// whole exponent -- the log of its prefactor (the law's constants folded in), the binary
// exponent ke of 1/edot = m 2^ke (as ke ln 2) and (P V - Q) / RT -- so that every factor lies in
// FP32's range; the grain powers and m multiply after.  Logs of the prefactors in 60-digit
// arithmetic: ln(9.1e-4 42 Vm 1e6), ln(5.8e-4 42 Vm 1e6 pi delta) (viscosity.c:113-121), ln Ag,
// ln Ad, ln 5.5e7 of both temperature branches (viscosity.c:138-162); R and V as double-floats.
// Returns false when an exponent or a term leaves FP32's range.
__device__ __forceinline__ bool creep_terms_df(double T, double g, double P, double iedot, CreepTermsDF &q) {
  if (lt_pos(P, 1.0)) P = 1.0;
  const df iRT = df_rcp(df_mul(df_of(T), df{8.314461708068848f, 3.9193113821056613e-07f}));
  const df PV = df_mul(df_of(P), df{-1.2999999853491317e-05f, -1.4650868680136236e-13f});
  const df gd = df_of(g), g2 = df_mul(gd, gd), id = df_mul(df_mul(g2, g2), gd);  // 1/d = g^5
  const long long eb = dbits(iedot);
  const int ke = (int)((eb >> 52) & 0x7FF) - 1023;
  const df m = df_of(__longlong_as_double((eb & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL));
  const df kl = df_mul(df{(float)ke, 0.0f}, kLn2);
  const bool cold_g = lt_pos(T, 255.0), cold_d = lt_pos(T, 258.0);
  const df x0 = df_add(df_add(df{-0.28377771377563477f, 9.349567342553655e-09f}, kl),
                       df_mul(df{-59400.0f, 0.0f}, iRT));  // Dv (59.4 kJ/mol)
  const df x1 = df_add(df_add(df{-20.41365623474121f, 1.6465773455820454e-07f}, kl),
                       df_mul(df{-49000.0f, 0.0f}, iRT));  // Db (49 kJ/mol), with pi delta
  const df x2 = df_add(df_add(cold_g ? df{-5.546778678894043f, -4.695249344877084e-08f}
                                     : df{60.965824127197266f, 5.793160084976989e-07f},
                              kl),
                       df_mul(df_add(PV, df{cold_g ? -49000.0f : -192000.0f, 0.0f}), iRT));  // GBS
  const df x3 = df_add(df_add(cold_d ? df{12.899219512939453f, 3.1315067872128566e-07f}
                                     : df{66.26414489746094f, -2.824399643941433e-06f},
                              kl),
                       df_mul(df_add(PV, df{cold_d ? -60000.0f : -180000.0f, 0.0f}), iRT));  // dislocation
  const df x4 = df_add(df_add(df{17.822843551635742f, 1.915609999514345e-07f}, kl),
                       df_mul(df_add(PV, df{-60000.0f, 0.0f}), iRT));  // basal slip
  const bool ok = fabsf(x0.hi) <= 80.0f && fabsf(x1.hi) <= 80.0f && fabsf(x2.hi) <= 80.0f &&
                  fabsf(x3.hi) <= 80.0f && fabsf(x4.hi) <= 80.0f;
  q.a = df_mul(df_mul(iRT, df_mul(id, id)), df_mul(m, df_fma(id, df_exp(x1), df_exp(x0))));
  q.g = df_mul(df_mul(df_exp(x2), df_mul(id, g2)), m);  // d^-1.4 = g^7
  q.d = df_mul(df_exp(x3), m);
  q.b = df_mul(df_exp(x4), m);
  return ok && fabsf(q.a.hi) < 1e37f && fabsf(q.g.hi) < 1e37f && fabsf(q.d.hi) < 1e37f && fabsf(q.b.hi) < 1e37f;
}

// One evaluation at p: the residual r - 1 = td + tc + tl - 1 with the series term
// tc = tg (tb / (tg + tb)) (one double-float division; no product of the two terms, which could
// leave FP32's range), and FP32 copies of the terms for the step.
struct CreepEvalDF {
  df res, p5;
  float S, tg, tb, td, tl;
};
__device__ __forceinline__ void creep_eval_df(const CreepTermsDF &q, const df &p, CreepEvalDF &e) {
  const df p2 = df_mul(p, p), p4 = df_mul(p2, p2), p8 = df_mul(p4, p4), p12 = df_mul(p8, p4);
  const df tg = df_mul(q.g, df_mul(p8, p)), tb = df_mul(q.b, p12);
  e.p5 = df_mul(p4, p);
  const df td = df_mul(q.a, e.p5), tl = df_mul(q.d, df_mul(p12, p8));
  const df S = df_add(tg, tb);
  const df tc = S.hi > 0.0f ? df_mul(tg, df_div(tb, S)) : df{0.0f, 0.0f};
  e.res = df_add(df_add(td, tl), df_add(tc, df{-1.0f, 0.0f}));
  e.S = S.hi;
  e.tg = tg.hi;
  e.tb = tb.hi;
  e.td = td.hi;
  e.tl = tl.hi;
}

// The Halley step of creep_advance (FP32 branch) from an evaluation: returns a = 0.2 du, the
// exponent of the factor on p
__device__ __forceinline__ float creep_step_df(const CreepEvalDF &e) {
  const float w = e.S > 0.0f ? e.tg / e.S : 0.0f;
  const float tc = e.tb * w;
  const float resf = e.res.hi;
  const float mc = fmaf(0.6f, w, 1.8f);
  const float r1f = fmaf(tc, mc, fmaf(4.0f, e.tl, e.td));
  const float r2f = fmaf(tc, fmaf(mc, mc, -0.36f * w * (1.0f - w)), fmaf(16.0f, e.tl, e.td));
  const float r = __fadd_rn(__fadd_rn(e.td, tc), e.tl);
  if (!(r > 1e-30f && r < 1e30f)) {
    // terms beyond FP32 range (an iterate far from the root): a step of -g / 4, which the slope
    // bound g' <= 4 keeps on the root's side
    return -0.05f * __logf(fmaxf(fabsf(resf + 1.0f), 1e-30f));
  }
  const float ir = 1.0f / r;
  const float g = fabsf(resf) < 0.5f ? log1pf(resf) : __logf(r);
  const float g1 = r1f * ir, g2 = fmaf(-g1, g1, r2f * ir);
  const float den = fmaf(-g, g2, 2.0f * g1 * g1);
  // Halley where its correction is moderate, Newton otherwise
  return 0.2f * (den > g1 * g1 ? -2.0f * g * g1 / den : -g / g1);
}

// p exp(a): p + p d with d = exp(a) - 1 from its series in FP32 for |a| < 2^-5, else p times an
// FP32 exponential
__device__ __forceinline__ df creep_advance_df(const df &p, float a) {
  if (fabsf(a) < 0.03125f) {
    const float d = a * fmaf(a, fmaf(a, fmaf(a, fmaf(a, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f), 0.5f), 1.0f);
    return df_fma(p, df{d, 0.0f}, p);
  }
  return df_mul(p, df{__expf(fminf(fmaxf(a, -80.0f), 80.0f)), 0.0f});
}

// Polish steps from p until |r - 1| <= tolf or maxit steps were taken, with creep_iterate's
// bracket and bisection (the bracket compared as double-floats: a last step below an FP32 ulp of
// p must not read as leaving it).  Returns the steps taken; res (FP32) and p5 belong to the
// final p.
__device__ __forceinline__ int creep_iterate_df(const CreepTermsDF &q, df &p, float tolf, int maxit, bool &conv,
                                                float &res, df &p5) {
  df plo = {0.0f, 0.0f}, phi = {INFINITY, 0.0f};
  CreepEvalDF e;
  int it = 0;
  for (;; ++it) {
    creep_eval_df(q, p, e);
    conv = fabsf(e.res.hi) <= tolf;
    if (conv || it >= maxit) break;
    if (e.res.hi > 0.0f) {
      if (df_lt(p, phi)) phi = p;
    } else if (df_lt(plo, p)) {
      plo = p;
    }
    df pn = creep_advance_df(p, creep_step_df(e));
    if (!(df_lt(plo, pn) && df_lt(pn, phi)))
      pn = df{plo.hi > 0.0f ? sqrtf(plo.hi * phi.hi) : phi.hi * 0.67032004603563930f, 0.0f};
    p = pn;
  }
  res = e.res.hi;
  p5 = e.p5;
  return it;
}
#endif

// Exact stress at strain rate edot (law 7) given 1 / edot: returns s*, iterations in *iters.
__device__ __forceinline__ double creep_stress_exact(const CreepCoef &k, double edot, double iedot, double tol,
                                                     int maxit, int *iters, double *res_out) {
#ifdef MIC_EXACT
  (void)iedot;
  return creep_stress_exact_u(k, edot, tol, maxit, iters, res_out);
#else
  *iters = 0;
  *res_out = 0.0;
  if (!gt_zero(edot)) return 0.0;
  // linear diffusion branch, s = edot / C < 1 Pa (viscosity.c:130-133); edot, C > 0 compared by bits
  if (dbits(edot) < dbits(k.C)) return edot / k.C;
  return creep_solve_terms(creep_terms(k, iedot), tol, maxit, iters, res_out);
#endif
}
__device__ __forceinline__ double creep_stress_exact(const CreepCoef &k, double edot, double tol, int maxit,
                                                     int *iters, double *res_out) {
  return creep_stress_exact(k, edot, edot > 0.0 ? 1.0 / edot : 0.0, tol, maxit, iters, res_out);
}

// ---- surrogate network ------------------------------------------------------------------
// Inputs.  With x = s / 1e6, each mechanism alone reaches edot at its own stress:
//   ln x_lin = ln(edot / C) - ln 1e6,  ln x_g = ln(edot / G) / 1.8,
//   ln x_b = ln(edot / B) / 2.4,       ln x_d = ln(edot / D) / 4,
// and the composite root depends on these four only, equivariantly: adding c to all four adds c
// to ln x*.  So the network sees the four differences to a reference m = min(ln x_lin, ln x_d,
// max(ln x_g, ln x_b)) (the fastest parallel branch; basal slip and grain-boundary sliding act in
// series), clamped to +-12 and scaled to [-1, 1], and predicts ln x* - m (normalised by
// out_mu, out_sigma).  The temperature switches of the law (255 K, 258 K) and all of T, d and P
// enter only through the coefficients, so the function learned is continuous.
//
// An MLP 4 -> 64 -> 64 -> 1 with SiLU activations; parameters are one FP32 array:
constexpr int kH = 64;
constexpr int kOffW1 = 0;                // W1[64][4]
constexpr int kOffB1 = kOffW1 + kH * 4;  // b1[64]
constexpr int kOffW2 = kOffB1 + kH;      // W2[64][64], row = output neuron
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;      // w3[64]
constexpr int kOffB3 = kOffW3 + kH;      // b3
constexpr int kOffNorm = kOffB3 + 1;     // out_mu, out_sigma
constexpr int kNParams = kOffNorm + 2;   // 4547
constexpr int kNTrain = kOffNorm;        // trained parameters (normalisation excluded)
constexpr float kFeatClamp = 12.0f;

// The hidden layer's weights W2 are BF16 values: every reader rounds them to BF16 (round to
// nearest even) as it stages them, the tensor cores take them as one BF16 operand, and training
// is quantization-aware (its forward and backward passes use the rounded weights, the update
// goes to the FP32 master copy); the library rounds W2 when a network is set or trained.
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// features of (coefficients, edot > 0); returns the reference m (ln x units)
__device__ __forceinline__ float creep_features(const CreepCoef &k, double edot, float f[4]) {
  const float le = ln_f(edot);
  const float xl = le - ln_f(k.C) - 13.81551056f;
  const float xg = (le - ln_f(k.G)) * (1.0f / 1.8f);
  const float xb = (le - ln_f(k.B)) * (1.0f / 2.4f);
  const float xd = (le - ln_f(k.D)) * 0.25f;
  const float m = fminf(fminf(xl, xd), fmaxf(xg, xb));
  const float x[4] = {xl, xg, xb, xd};
#pragma unroll
  for (int i = 0; i < 4; ++i) f[i] = fminf(fmaxf(x[i] - m, -kFeatClamp), kFeatClamp) * (1.0f / kFeatClamp);
  return m;
}

#ifndef MIC_EXACT
// the same features from double-float terms q: ln x_lin = -ln q.a, ln x_g = -ln q.g / 1.8,
// ln x_b = -ln q.b / 2.4, ln x_d = -ln q.d / 4 (FP32 logs of the high parts)
__device__ __forceinline__ float creep_features_df(const CreepTermsDF &q, float f[4]) {
  const float xl = -__logf(q.a.hi);
  const float xg = -__logf(q.g.hi) * (1.0f / 1.8f);
  const float xb = -__logf(q.b.hi) * (1.0f / 2.4f);
  const float xd = -__logf(q.d.hi) * 0.25f;
  const float m = fminf(fminf(xl, xd), fmaxf(xg, xb));
  const float x[4] = {xl, xg, xb, xd};
#pragma unroll
  for (int i = 0; i < 4; ++i) f[i] = fminf(fmaxf(x[i] - m, -kFeatClamp), kFeatClamp) * (1.0f / kFeatClamp);
  return m;
}
#endif

// SiLU and its derivative with the fast reciprocal (__fdividef: two MUFU ops and a multiply,
// about 2 ulp) instead of the IEEE division sequence: 128 of these per marker at inference.  For
// z below about -87 the denominator overflows and both return 0, the limit.
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// FP32 forward pass on CUDA cores (reference path; W2 read from w2s, a shared-memory copy)
__device__ __forceinline__ float mlp_forward(const float *__restrict__ p, const float *__restrict__ w2s,
                                             const float f[4]) {
  float h1[kH];
#pragma unroll
  for (int n = 0; n < kH; ++n) {
    float z = p[kOffB1 + n];
#pragma unroll
    for (int i = 0; i < 4; ++i) z = fmaf(p[kOffW1 + 4 * n + i], f[i], z);
    h1[n] = silu(z);
  }
  float y = p[kOffB3];
  for (int n = 0; n < kH; ++n) {
    float z = p[kOffB2 + n];
#pragma unroll
    for (int k = 0; k < kH; ++k) z = fmaf(w2s[n * kH + k], h1[k], z);
    y = fmaf(p[kOffW3 + n], silu(z), y);
  }
  return y;
}


// Stress from a surrogate guess lx0 = ln(s / 1e6): polish steps until |rate/edot - 1| <=
// polish_tol within polish_iters steps, else the exact solve from its own start (*fb = 1).  The
// zero-rate and linear-diffusion cases are those of creep_stress_exact.
__device__ __forceinline__ double creep_stress_from_guess(const CreepCoef &k, double edot, double iedot, float lx0,
                                                          double tol, int maxit, int polish_iters, double polish_tol,
                                                          int *iters, double *res_out, int *fb) {
  *iters = 0;
  *res_out = 0.0;
  *fb = 0;
#ifdef MIC_EXACT
  if (!(edot > 0.0)) return 0.0;
  (void)iedot;
  const double s_lin = edot / k.C;
  if (s_lin < 1.0) return s_lin;
  if (isfinite(lx0)) {
    double u = (double)lx0 + kLn1e6, ulo = -1e308, uhi = 1e308, res;
    *iters = creep_newton(k, edot, u, ulo, uhi, polish_tol, polish_iters, res);
    if (fabs(res) <= polish_tol) {
      *res_out = res;
      const double s = exp(u);
      return s < 1.0 ? 1.0 : s;
    }
  }
  *fb = 1;
  int it2;
  const double s = creep_stress_exact_u(k, edot, tol, maxit, &it2, res_out);
  *iters += it2;
  return s;
#else
  if (!gt_zero(edot)) return 0.0;
  if (dbits(edot) < dbits(k.C)) return edot / k.C;
  const CreepTerms q = creep_terms(k, iedot);
  if (isfinite(lx0)) {
    double p = f64_of(__expf(0.2f * lx0)), res, p5;
    bool conv;
    *iters = creep_iterate(q, p, 0.0, INFINITY, polish_tol, polish_iters, conv, res, p5);
    if (conv) {
      *res_out = res;
      const double s = 1e6 * p5;
      return lt_pos(s, 1.0) ? 1.0 : s;
    }
  }
  *fb = 1;
  int it2;
  const double s = creep_solve_terms(q, tol, maxit, &it2, res_out);
  *iters += it2;
  return s;
#endif
}
__device__ __forceinline__ double creep_stress_from_guess(const CreepCoef &k, double edot, float lx0, double tol,
                                                          int maxit, int polish_iters, double polish_tol,
                                                          int *iters, double *res_out, int *fb) {
  return creep_stress_from_guess(k, edot, edot > 0.0 ? 1.0 / edot : 0.0, lx0, tol, maxit, polish_iters, polish_tol,
                                 iters, res_out, fb);
}

#ifndef MIC_EXACT
// Stress from a surrogate guess lx0 = ln(s / 1e6) at a coarse polish tolerance (from kCoarseTol):
// the polish in double-float arithmetic on the terms q (q_ok: creep_terms_df succeeded).  A marker
// on or within 1e-6 of the linear-diffusion branch (edot < C, i.e. q.a > 1e6) is decided and
// evaluated in FP64 exactly as the exact solve does it (s = edot / C); one whose terms are out of
// range or whose polish does not reach the tolerance takes the exact FP64 solve (*fb = 1).
// edot > 0.
__device__ __forceinline__ double creep_stress_coarse(const CreepTermsDF &q, bool q_ok, double T, double g, double P,
                                                      double edot, double iedot, float lx0, double tol, int maxit,
                                                      int polish_iters, double polish_tol, int *iters,
                                                      double *res_out, int *fb) {
  *iters = 0;
  *res_out = 0.0;
  *fb = 0;
  if (q_ok && !(q.a.hi > 0.999999e6f) && isfinite(lx0)) {
    const float tolf = f32_trunc(polish_tol);  // at most polish_tol
    df p = {__expf(0.2f * lx0), 0.0f}, p5;
    float res;
    bool conv;
    *iters = creep_iterate_df(q, p, tolf, polish_iters, conv, res, p5);
    if (conv) {
      *res_out = f64_of(res);
      const double s = 1e6 * df_to_f64(p5);
      return lt_pos(s, 1.0) ? 1.0 : s;
    }
  }
  const CreepCoef k = creep_coef(T, g, P);
  if (dbits(edot) < dbits(k.C)) return edot / k.C;  // linear diffusion branch (viscosity.c:130-133)
  *fb = 1;
  int it2;
  const double s = creep_solve_terms(creep_terms(k, iedot), tol, maxit, &it2, res_out);
  *iters += it2;
  return s;
}
#endif

// per-warp reduction of the creep counters into the device totals (all lanes of the warp)
__device__ __forceinline__ void creep_count(CreepCounters *cc, int active, int iters, double res, int fallback) {
  const unsigned full = 0xffffffffu;
  int a = active, it = iters, fb = fallback;
  long long rb = active ? nonneg_bits(fabs(res)) : 0;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(full, a, o);
    it += __shfl_down_sync(full, it, o);
    fb += __shfl_down_sync(full, fb, o);
    rb = max(rb, __shfl_down_sync(full, rb, o));
  }
  if ((threadIdx.x & 31) == 0 && a) {
    atomicAdd(&cc->markers, (unsigned long long)a);
    atomicAdd(&cc->iterations, (unsigned long long)it);
    if (fb) atomicAdd(&cc->fallbacks, (unsigned long long)fb);
    atomicMax(&cc->max_res_bits, (unsigned long long)rb);
  }
}

// network output and reference m -> guess of ln x* = ln(s* / 1e6)
__device__ __forceinline__ float creep_guess_lx(const float *__restrict__ p, float y, float m) {
  return m + fmaf(y, p[kOffNorm + 1], p[kOffNorm]);
}
}  // namespace mic
