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
// Exact solve: Newton on g(u) = ln rate(e^u) - ln edot, u = ln s.  g is increasing with
// slope between 1 and 4 and nearly linear, so Newton converges in a few steps; it starts from
// min(edot / C, 1e6 (edot / D)^(1/4)) -- each term alone reaching edot bounds s* from above --
// and keeps a bracket.  Powers of x come from one exp per iteration: p = x^0.2 gives
// x^1.8 = p^9, x^2.4 = p^12, x^4 = p^20, s = 1e6 p^5.
#pragma once

#include <cuda_runtime.h>

#include "mic_internal.cuh"

namespace mic {

struct CreepCoef {
  double C;     // diffusion:   rate = C s
  double G;     // GBS:         rate = G x^1.8
  double B;     // basal slip:  rate = B x^2.4
  double D;     // dislocation: rate = D x^4
};

// viscosity.c:109-173: constants of the law at (T, d, P), with P clamped below at 1 Pa.  The
// FMA-free parity build evaluates each Arrhenius factor as the reference writes it.  The product
// build factors exp((-Q + P V) / RT) = exp(-Q / RT) exp(P V / RT) and shares the factors whose
// activation energies coincide (grain-boundary diffusion and cold GBS: 49 kJ; basal slip and
// cold dislocation creep: 60 kJ): four exponentials instead of five plus pow for cold ice,
// agreeing with the reference's form to a few ulp.
__device__ __forceinline__ CreepCoef creep_coef(double T, double d, double P) {
  const double R = 8.3144621;
  if (P < 1.0) P = 1.0;
  const double RT = R * T;
  const double b = 4.52e-10, Vm = 1.97e-5, delta = 2.0 * b;
  const double V = -13e-6;
  CreepCoef k;
#ifdef MIC_EXACT
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
  const double e49 = exp(-49.0e3 * iRT), e60 = exp(-60.0e3 * iRT), eP = exp(P * V * iRT);
  const double Dv = 9.10e-4 * exp(-59.4e3 * iRT);
  const double Db = 5.8e-4 * e49;
  const double id = 1.0 / d;
  k.C = 42.0 * Vm * iRT * id * id * (Dv + M_PI * delta * id * Db);
  const double eg = (T < 255.0) ? 3.9e-3 * e49 : 3.0e26 * exp(-192.0e3 * iRT);
  const double ed = (T < 258.0) ? 4.0e5 * e60 : 6.0e28 * exp(-180.0e3 * iRT);
  k.G = eg * eP * exp2(-1.4 * log2(d));
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

// Exact stress at strain rate edot (law 7): returns s*, iterations in *iters.
__device__ __forceinline__ double creep_stress_exact(const CreepCoef &k, double edot, double tol, int maxit,
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

// natural log of a positive normal double to FP32 accuracy: exponent from frexp, __logf of the
// mantissa (the features need no more, and no FP64 transcendental is spent on them)
__device__ __forceinline__ float ln_f(double v) {
  int e;
  const double mant = frexp(v, &e);  // [0.5, 1)
  return (float)e * 0.693147181f + __logf((float)mant);
}

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

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
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


// Stress from a surrogate guess u0 (ln s): Newton polish until |rate/edot - 1| <= polish_tol
// within polish_iters steps, else the exact solve from its own start (*fb = 1).  The zero-rate
// and linear-diffusion cases are those of creep_stress_exact.
__device__ __forceinline__ double creep_stress_from_guess(const CreepCoef &k, double edot, double u0, double tol,
                                                          int maxit, int polish_iters, double polish_tol,
                                                          int *iters, double *res_out, int *fb) {
  *iters = 0;
  *res_out = 0.0;
  *fb = 0;
  if (!(edot > 0.0)) return 0.0;
  const double s_lin = edot / k.C;
  if (s_lin < 1.0) return s_lin;
  if (isfinite(u0)) {
    double u = u0, ulo = -1e308, uhi = 1e308, res;
    *iters = creep_newton(k, edot, u, ulo, uhi, polish_tol, polish_iters, res);
    if (fabs(res) <= polish_tol) {
      *res_out = res;
      const double s = exp(u);
      return s < 1.0 ? 1.0 : s;
    }
  }
  *fb = 1;
  int it2;
  const double s = creep_stress_exact(k, edot, tol, maxit, &it2, res_out);
  *iters += it2;
  return s;
}

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

// network output and reference m -> ln s guess
__device__ __forceinline__ double creep_guess_u(const float *__restrict__ p, float y, float m) {
  return kLn1e6 + (double)m + ((double)y * p[kOffNorm + 1] + p[kOffNorm]);
}
}  // namespace mic
