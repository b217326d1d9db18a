// mic_rheology.cuh -- computeRheology (viscosity.c:12-67) for one marker, with the composite
// creep law (law 7) of mic_creep.cuh; shared by the marker passes and density control.
#pragma once

#include <cmath>

#include "mic_creep.cuh"
#include "mic_internal.cuh"

namespace mic {

// Inputs of the composite creep law (law 7): the marker's strain rate, grain argument (the
// grain column: see grain_arg), pressure and (surrogate modes) the network's guess of
// ln(s* / 1e6); iteration count, residual and fallback flag of its stress solve come back in it.
struct CreepIn {
  double e11, e22, e12, grain, p;
  float lx_guess;
  int iters, fb;
  double res;
  int have_k;    // k, edot and iedot below already evaluated for this marker
  CreepCoef k;
  double edot;   // strain-rate invariant sqrt(0.5 (e11^2 + e22^2) + e12^2)
  double iedot;  // 1 / edot (product build)
  // product build, surrogate at a coarse polish tolerance: the law's terms in double-float
  // arithmetic (then k is not evaluated) and whether they are in range
  const CreepTermsDF *qdf;
  int q_ok;
};

__device__ __forceinline__ double strain_rate_invariant(double e11, double e22, double e12) {
  return sqrt(0.5 * (e11 * e11 + e22 * e22) + e12 * e12);
}

// The strain-rate invariant and its reciprocal.  The FMA-free parity build takes the square root
// (and divides by edot where the reference does; iedot is unused there).  The product build takes
// one reciprocal square root r of the invariant's square q, edot = q r and 1 / edot = r (at most
// about 1.5 ulp from the correctly rounded square root), where a square root and a division
// would each cost several FP64 instructions; q = 0 and q = +inf give edot = q.
__device__ __forceinline__ void strain_rate_and_inverse(double e11, double e22, double e12, double &edot,
                                                        double &iedot) {
#ifdef MIC_EXACT
  edot = strain_rate_invariant(e11, e22, e12);
  iedot = 0.0;
#else
  const double q = fma(e12, e12, 0.5 * fma(e11, e11, e22 * e22));
  const double r = rsqrt(q);
  const long long b = dbits(q);
  edot = (b == 0 || b == 0x7FF0000000000000LL) ? q : q * r;
  iedot = r;
#endif
}

// Law 7 (new): composite ice creep, eta = s* / (2 edot_II) with s* the stress at which the
// Goldsby-Kohlstedt strain rate (viscosity.c:106-179) equals the marker's strain-rate
// invariant; at zero strain rate the law's diffusion viscosity 0.5 / C (viscosity.c:130-133).
__device__ __forceinline__ double creep_viscosity(const CreepConfig &cfg, double T, CreepIn &ci) {
  double edot, iedot;  // once per marker: the solve and the viscosity share them
#ifndef MIC_EXACT
  if (ci.qdf) {  // the surrogate's coarse polish in double-float arithmetic (mic_creep.cuh)
    if (!gt_zero(ci.edot)) return 0.5 / creep_coef(T, ci.grain, ci.p).C;
    const double s = creep_stress_coarse(*ci.qdf, ci.q_ok != 0, T, ci.grain, ci.p, ci.edot, ci.iedot, ci.lx_guess,
                                         cfg.tol, cfg.maxit, cfg.polish_iters, cfg.polish_tol, &ci.iters, &ci.res,
                                         &ci.fb);
    return s * (0.5 * ci.iedot);
  }
#endif
  if (ci.have_k) {
    edot = ci.edot;
    iedot = ci.iedot;
  } else {
    strain_rate_and_inverse(ci.e11, ci.e22, ci.e12, edot, iedot);
  }
  const CreepCoef k = ci.have_k ? ci.k : creep_coef(T, ci.grain, ci.p);
#ifdef MIC_EXACT
  if (!(edot > 0.0)) return 0.5 / k.C;
#else
  if (!gt_zero(edot)) return 0.5 / k.C;
#endif
  const double s = (cfg.mode == 0) ? creep_stress_exact(k, edot, iedot, cfg.tol, cfg.maxit, &ci.iters, &ci.res)
                                   : creep_stress_from_guess(k, edot, iedot, ci.lx_guess, cfg.tol, cfg.maxit,
                                                             cfg.polish_iters, cfg.polish_tol, &ci.iters, &ci.res,
                                                             &ci.fb);
#ifdef MIC_EXACT
  return s / (2.0 * edot);
#else
  return s * (0.5 * iedot);
#endif
}

// computeRheology (viscosity.c:12-67) plus law 7; returns false for an undefined law
__device__ __forceinline__ bool rheology(const mic_materials &M, const mic_options &O, int k, double T, double X,
                                         double Y, double &eta, double &mu, const CreepConfig *cfg = nullptr,
                                         CreepIn *ci = nullptr) {
  mu = M.materialMu[k];
  switch (M.hasEtaT[k]) {
    case 7:
      if (!cfg || !ci) return false;
      eta = creep_viscosity(*cfg, T, *ci);
      return true;
    case 1: eta = M.materialEta[k] * exp(M.QonR[k] * (1.0 / T - 1.0 / M.Tref[k])); return true;
    case 2: {
      const double T0 = M.Tref[k];
      eta = M.materialEta[k] * exp(M.QonR[k] / T0 * (1.0 - (T - T0) / T0));
      return true;
    }
    case 3: eta = M.materialEta[k] * T; return true;
    case 5: eta = M.materialEta[k] * exp(-M.QonR[k] * T); return true;
    case 0: eta = M.materialEta[k]; return true;
    case 6: {
      double e = M.materialEta[k];
      const double edge = Y / tan(O.slabAngle);
      if (X > edge && X < (edge + O.decoupleThickness) && Y > O.minDecoupleDepth && Y < O.maxDecoupleDepth)
        e *= O.decoupleEtaScaler;
      eta = e;
      return true;
    }
    default: return false;
  }
}

}  // namespace mic
