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

namespace mic {

struct CreepCoef {
  double C;     // diffusion:   rate = C s
  double G;     // GBS:         rate = G x^1.8
  double B;     // basal slip:  rate = B x^2.4
  double D;     // dislocation: rate = D x^4
};

// viscosity.c:109-173: constants of the law at (T, d, P), with P clamped below at 1 Pa
__device__ __forceinline__ CreepCoef creep_coef(double T, double d, double P) {
  const double R = 8.3144621;
  if (P < 1.0) P = 1.0;
  const double RT = R * T;
  const double b = 4.52e-10, Vm = 1.97e-5, delta = 2.0 * b;
  const double Dv = 9.10e-4 * exp(-59.4e3 / RT);
  const double Db = 5.8e-4 * exp(-49.0e3 / RT);
  CreepCoef k;
  k.C = 42.0 * Vm / (RT * d * d) * (Dv + M_PI * delta / d * Db);
  const double V = -13e-6;
  const double Qg = (T < 255.0) ? 49.0e3 : 192.0e3, Ag = (T < 255.0) ? 3.9e-3 : 3.0e26;
  const double Qd = (T < 258.0) ? 60.0e3 : 180.0e3, Ad = (T < 258.0) ? 4.0e5 : 6.0e28;
  k.G = Ag / pow(d, 1.4) * exp((-Qg + P * V) / RT);
  k.D = Ad * exp((-Qd + P * V) / RT);
  k.B = 5.5e7 * exp((-60.0e3 + P * V) / RT);
  return k;
}

// rate and d(rate)/d(ln s) at s = 1e6 p^5 (s >= 1 Pa branch)
__device__ __forceinline__ void creep_rate_p(const CreepCoef &k, double p, double &f, double &df) {
  const double p2 = p * p, p4 = p2 * p2, p5 = p4 * p, p8 = p4 * p4, p9 = p8 * p, p12 = p8 * p4;
  const double p20 = p12 * p8;
  const double td = k.C * 1e6 * p5, tg = k.G * p9, tb = k.B * p12, tl = k.D * p20;
  const double sum = tg + tb;
  const double tc = tg * tb / sum;  // (1/tb + 1/tg)^-1
  f = td + tc + tl;
  df = td + tc * (2.4 * tg + 1.8 * tb) / sum + 4.0 * tl;
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
  for (; it < maxit; ++it) {
    const double p = exp(0.2 * (u - kLn1e6));
    double f, df;
    creep_rate_p(k, p, f, df);
    const double r = f / edot;
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

// Exact stress at strain rate edot (law 7): returns s*, iterations in *iters.
__device__ __forceinline__ double creep_stress_exact(const CreepCoef &k, double edot, double tol, int maxit,
                                                     int *iters, double *res_out) {
  *iters = 0;
  *res_out = 0.0;
  if (!(edot > 0.0)) return 0.0;
  const double s_lin = edot / k.C;
  if (s_lin < 1.0) return s_lin;  // linear diffusion branch (viscosity.c:130-133)
  const double s_dis = 1e6 * sqrt(sqrt(edot / k.D));
  double u = log(fmin(s_lin, s_dis));
  double ulo = -1e308, uhi = u + 1e-12;
  double res;
  *iters = creep_newton(k, edot, u, ulo, uhi, tol, maxit, res);
  *res_out = res;
  const double s = exp(u);
  // the rate jumps at s = 1 Pa where the non-linear terms switch on; a root in the jump is 1 Pa
  return s < 1.0 ? 1.0 : s;
}

}  // namespace mic
