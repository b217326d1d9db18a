// mic_marker_passes.cu -- K3..K5: the per-marker passes of the marker path and the
// deterministic node gathers of the subgrid corrections.
//
// Every marker kernel runs one thread per marker over the cell-sorted columns and skips
// markers outside the domain (cellX == -1), like the reference loops.  Floating-point
// expressions keep the reference's evaluation order; built without FMA contraction
// (-fmad=false) the results match the reference bit for bit except where a CUDA
// transcendental (exp, sin, cos, tan) differs from the host libm in the last place.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "mic_creep.cuh"
#include "mic_creep_tc.cuh"
#include "mic_df.cuh"
#include "mic_internal.cuh"
#include "mic_rheology.cuh"

using namespace mic;


namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

#ifndef MIC_EXACT  // product-build helpers
// cos, sin, sin 2t, cos 2t of the rotation angle t of markers.c:2158-2164.  Per-step rotations
// are small: for |t| <= 2^-6 truncated Taylor series (to t^7 / t^8, remainder below 2^-60
// relative) and the double-angle identities replace four transcendental calls; larger angles
// use sincos.
__device__ __forceinline__ void small_angle_rotation(double t, double &c, double &s, double &s2, double &c2) {
  if (fabs(t) <= 0.015625) {
    const double t2 = t * t;
    s = t * fma(t2, fma(t2, fma(t2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), 1.0);
    c = fma(t2, fma(t2, fma(t2, fma(t2, 1.0 / 40320.0, -1.0 / 720.0), 1.0 / 24.0), -0.5), 1.0);
  } else {
    sincos(t, &s, &c);
  }
  s2 = 2.0 * s * c;
  c2 = (c - s) * (c + s);
}
#endif

#ifdef MIC_EXACT
// Interpolation cell at cell centres (updateMarkerStrainPressure.c:137-150, updateMarkerStress.c:66-80,
// subgridStressChanges.c:179-190): staggered cell clamped to [1, cmax] x [1, NY-2].  Where the
// clamp leaves the staggered cell unchanged the offsets are the projection geometry.
__device__ __forceinline__ void centre_interp(const Params &P, int cx, int cy, int fl, double gx1, double gy1,
                                              double x, double y, int cmax, int &i, int &j, double &mdx,
                                              double &mdy) {
  const int sx = cx + (fl & 1), sy = cy + ((fl >> 1) & 1);
  i = clampi(sx, 1, cmax);
  j = clampi(sy, 1, P.NY - 2);
  mdx = (i == sx) ? gx1 : div_sp(x - P.xc[i], P.hxc[i], P.ixc[i]);
  mdy = (j == sy) ? gy1 : div_sp(y - P.yc[j], P.hyc[j], P.iyc[j]);
}
#endif

// Largest staggered interpolation cell of updateMarkerStrainPressure and updateMarkerStress
// (cellXMax: NX - 2, NX - 1 on a grid periodic in x; updateMarkerStrainPressure.c:137-147,
// updateMarkerStress.c:66-77).  subgridStressChanges keeps NX - 2 either way (its lines 92, 187).
__device__ __forceinline__ int centre_cmax(const Params &P) { return P.xper ? P.NX - 1 : P.NX - 2; }

// limitViscosity (viscosity.c:90-104) on one viscosity
__device__ __forceinline__ double limit_eta(double e, const mic_options &O) {
#ifdef MIC_EXACT
  if (e > O.etamax) return O.etamax;
  if (e < O.etamin) return O.etamin;
#else
  // the same two compares on order-preserving integer keys (a NaN viscosity stays NaN)
  if (nan_bits(dbits(e))) return e;
  const long long k = ordered_bits(e);
  if (k > ordered_bits(O.etamax)) return O.etamax;
  if (k < ordered_bits(O.etamin)) return O.etamin;
#endif
  return e;
}

struct YieldCols {
  const int *cellX, *mat;
  const double *X, *Y, *T, *p, *Eii, *exx, *eyy, *exy, *grain;
  double *eta, *mu, *sxx, *syy, *sxy;
};

// One marker of checkPlasticYielding (markers.c:1381-1505).  lx_guess: the surrogate's guess of
// ln(s* / 1e6) for a law-7 marker (surrogate modes); kc, kedot: its creep coefficients and
// strain-rate invariant when already evaluated.  Returns whether the marker yielded.  CREEP
// false: no material uses law 7, and its solver is left out (fewer registers, more resident
// warps).
template <bool CREEP = true>
__device__ __forceinline__ bool yield_marker(const YieldCols &c, const mic_materials &M, const mic_options &O,
                                             const CreepConfig &cfg, double dt, int64_t m, float lx_guess,
                                             const CreepCoef *kc, double kedot, double kiedot, Status *st,
                                             CreepIn &ci, int &creep_active, int limit,
                                             const CreepTermsDF *qdf = nullptr, int q_ok = 0) {
  bool yielded = false;
  const double eta_old = c.eta[m], mu_old = c.mu[m];
  const double e11 = c.exx[m], e22 = c.eyy[m], e12 = c.exy[m];
  const int k = c.mat[m];
  double eta, mu;
  ci = CreepIn{e11, e22, e12, c.grain[m], c.p[m], lx_guess, 0, 0, 0.0, kc != nullptr, {}, kedot, kiedot, qdf, q_ok};
  if (kc) ci.k = *kc;
  if (!(CREEP ? rheology(M, O, k, c.T[m], c.X[m], c.Y[m], eta, mu, &cfg, &ci)
              : rheology(M, O, k, c.T[m], c.X[m], c.Y[m], eta, mu))) {
    eta = eta_old;
    mu = mu_old;
    atomicAdd(&st->bad_law, 1ULL);
  }
  creep_active = M.hasEtaT[k] == 7;
  const int plast = M.hasPlasticity[k];
  if (plast) {
    // visco-elastic forecast with the old viscosity and modulus (markers.c:1397-1402); only the
    // yield test reads it (the rheology laws take no stress), so only plastic materials form it
    double s11 = c.sxx[m], s22 = c.syy[m], s12 = c.sxy[m];
    const double Xf = eta_old / (mu_old * dt + eta_old);
#ifdef MIC_EXACT
    const double fxx = s11 * Xf + 2 * eta_old * e11 * (1.0 - Xf);
    const double fyy = s22 * Xf + 2 * eta_old * e22 * (1.0 - Xf);
    const double fxy = s12 * Xf + 2 * eta_old * e12 * (1.0 - Xf);
#else
    const double ve = 2 * eta_old * (1.0 - Xf);  // shared by the three components
    const double fxx = fma(s11, Xf, ve * e11);
    const double fyy = fma(s22, Xf, ve * e22);
    const double fxy = fma(s12, Xf, ve * e12);
#endif
    const double sii = sqrt(0.5 * (fxx * fxx + fyy * fyy) + fxy * fxy);
    double sy;
    if (plast == 1) {
      sy = M.materialCohesion[k] + M.materialFriction[k] * c.p[m];
    } else if (plast == 2) {  // strain weakening (markers.c:1426-1448)
      const double E = c.Eii[m];
      double coh, fr;
      if (E < M.gamma[k][0]) {
        coh = M.C[k][0];
        fr = sin(M.F[k][0] / 180.0 * M_PI);
      } else if (E >= M.gamma[k][0] && E <= M.gamma[k][1]) {
        const double dg = (E - M.gamma[k][0]) / (M.gamma[k][1] - M.gamma[k][0]);
        coh = (M.C[k][1] - M.C[k][0]) * dg + M.C[k][0];
        fr = (sin(M.F[k][1] / 180.0 * M_PI) - sin(M.F[k][0] / 180.0 * M_PI)) * dg + sin(M.F[k][0] / 180.0 * M_PI);
      } else {
        coh = M.C[k][1];
        fr = sin(M.F[k][1] / 180.0 * M_PI);
      }
      sy = coh + fr * c.p[m];
    } else {
      sy = 0.0;
    }
    if (sy < 0.0) sy = 0.0;
    double etanew = eta_old;  // plastic materials keep the old viscosity unless they yield
    if (sii > sy) {
      const double eii = sqrt(0.5 * (e11 * e11 + e22 * e22) + e12 * e12);
      etanew = sy / 2.0 / eii;
      if (etanew / eta < O.fractionalEtamin) etanew = O.fractionalEtamin * eta;
      if (etanew < O.etamin)
        etanew = O.etamin;
      else if (etanew > O.etamax)
        etanew = O.etamax;
      const double sio = sqrt(0.5 * (s11 * s11 + s22 * s22) + s12 * s12);
      if (sio != 0.0) {
        s11 *= sy / sio;
        s22 *= sy / sio;
        s12 *= sy / sio;
        c.sxx[m] = s11;
        c.syy[m] = s22;
        c.sxy[m] = s12;
      }
      yielded = true;
    }
    eta = etanew;
  }
  if (limit) eta = limit_eta(eta, O);  // limitViscosity fused (the step runs it right after)
  c.eta[m] = eta;
  c.mu[m] = mu;
  return yielded;
}

// coefficients, strain-rate invariant and surrogate features of marker m when it follows law 7
// (false otherwise); *mref receives the features' reference
__device__ __forceinline__ bool creep_marker_features(const YieldCols &c, const mic_materials &M, int64_t m,
                                                      CreepCoef &k, double &edot, double &iedot, float f[4],
                                                      float *mref) {
  if (M.hasEtaT[c.mat[m]] != 7) return false;
  strain_rate_and_inverse(c.exx[m], c.eyy[m], c.exy[m], edot, iedot);
  k = creep_coef(c.T[m], c.grain[m], c.p[m]);
#ifdef MIC_EXACT
  if (!(edot > 0.0)) {
#else
  if (!gt_zero(edot)) {
#endif
    *mref = 0.f;
    f[0] = f[1] = f[2] = f[3] = 0.f;
    return true;
  }
  *mref = creep_features(k, edot, f);
  return true;
}

#ifndef MIC_EXACT
// creep_marker_features for the surrogate's coarse polish: the law's terms in double-float
// arithmetic (q_ok false when they leave FP32's range: the marker then takes the FP64 solve)
__device__ __forceinline__ bool creep_marker_features_df(const YieldCols &c, const mic_materials &M, int64_t m,
                                                         CreepTermsDF &q, int &q_ok, double &edot, double &iedot,
                                                         float f[4], float *mref) {
  if (M.hasEtaT[c.mat[m]] != 7) return false;
  strain_rate_and_inverse(c.exx[m], c.eyy[m], c.exy[m], edot, iedot);
  q_ok = gt_zero(edot) && creep_terms_df(c.T[m], c.grain[m], c.p[m], iedot, q);
  if (!q_ok) {
    *mref = 0.f;
    f[0] = f[1] = f[2] = f[3] = 0.f;
    return true;
  }
  *mref = creep_features_df(q, f);
  return true;
}
#endif

// One marker of checkPlasticYielding (the solo kernels and their batched forms share it).
// MODE 0: exact creep solve; MODE 1: surrogate guess on the CUDA cores (FP32, w2s: the hidden
// layer's weights in shared memory), polish and fallback; MODE 2: no material uses law 7.
// limit: limitViscosity fused in (every marker, out-of-domain ones included, viscosity.c:93-95).
// Every thread of a warp calls it (the creep counters reduce over the warp).
template <int MODE>
__device__ __forceinline__ bool yield_one(const YieldCols &c, const mic_materials &M, const mic_options &O,
                                          const CreepConfig &cfg, double dt, int64_t n, Status *st,
                                          CreepCounters *cc, int limit, const float *w2s, int64_t m) {
  bool yielded = false;
  int creep_active = 0;
  CreepIn ci = {};
  if (m < n && c.cellX[m] != -1) {
    float lx = 0.f, f[4], mref;
    double edot = 0.0, iedot = 0.0;
    CreepCoef k;
#ifndef MIC_EXACT
    CreepTermsDF q;
    int q_ok = 0;
    const bool coarse = MODE == 1 && !(cfg.polish_tol < kCoarseTol);  // uniform over the pass
    const bool law7 = MODE == 1 && (coarse ? creep_marker_features_df(c, M, m, q, q_ok, edot, iedot, f, &mref)
                                           : creep_marker_features(c, M, m, k, edot, iedot, f, &mref));
#else
    const bool coarse = false;
    const CreepTermsDF q{};
    const int q_ok = 0;
    const bool law7 = MODE == 1 && creep_marker_features(c, M, m, k, edot, iedot, f, &mref);
#endif
    if (law7) lx = creep_guess_lx(cfg.mlp, mlp_forward(cfg.mlp, w2s, f), mref);
    yielded = yield_marker<MODE != 2>(c, M, O, cfg, dt, m, lx, law7 && !coarse ? &k : nullptr, edot, iedot, st, ci,
                                      creep_active, limit, law7 && coarse ? &q : nullptr, q_ok);
  } else if (limit && m < n) {
    c.eta[m] = limit_eta(c.eta[m], O);
  }
  if (MODE != 2) creep_count(cc, creep_active, ci.iters, ci.res, ci.fb);
  return yielded;
}

// One 128-marker round of checkPlasticYielding with the surrogate's hidden layer on the tensor
// cores (all kTile threads of the block, block-uniform; thread t takes marker m0 + t).  Returns
// whether this thread's marker yielded.
__device__ __forceinline__ bool yield_tc_round(tc::Block &B, const YieldCols &c, const mic_materials &M,
                                               const mic_options &O, const CreepConfig &cfg, double dt, int64_t n,
                                               Status *st, CreepCounters *cc, int limit, int64_t m) {
  const bool live = m < n && c.cellX[m] != -1;
  float f[4] = {0.f, 0.f, 0.f, 0.f}, mref = 0.f;
  double edot = 0.0, iedot = 0.0;
  CreepCoef k;
#ifndef MIC_EXACT
  CreepTermsDF q;
  int q_ok = 0;
  const bool coarse = !(cfg.polish_tol < kCoarseTol);  // uniform over the pass
  const bool law7 = live && (coarse ? creep_marker_features_df(c, M, m, q, q_ok, edot, iedot, f, &mref)
                                    : creep_marker_features(c, M, m, k, edot, iedot, f, &mref));
#else
  const bool coarse = false;
  const CreepTermsDF q{};
  const int q_ok = 0;
  const bool law7 = live && creep_marker_features(c, M, m, k, edot, iedot, f, &mref);
#endif
  const float y = tc::guess(B, f, cfg.tc_wait_limit, &cc->tc_timeouts);
  int creep_active = 0;
  CreepIn ci = {};
  bool yielded = false;
  if (live)
    yielded = yield_marker(c, M, O, cfg, dt, m, creep_guess_lx(cfg.mlp, y, mref), law7 && !coarse ? &k : nullptr,
                           edot, iedot, st, ci, creep_active, limit, law7 && coarse ? &q : nullptr, q_ok);
  if (limit && !live && m < n) c.eta[m] = limit_eta(c.eta[m], O);
  creep_count(cc, creep_active, ci.iters, ci.res, ci.fb);
  return yielded;
}

// updateViscosity (viscosity.c:77-88): rheology from the current marker stress
__global__ void k_update_viscosity(YieldCols c, mic_materials M, mic_options O, CreepConfig cfg, int64_t n,
                                   Status *st) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n || c.cellX[m] == -1) return;
  double eta, mu;
  CreepIn ci = {c.exx[m], c.eyy[m], c.exy[m], c.grain[m], c.p[m], 0.0f, 0, 0, 0.0, 0, {}, 0.0};
  CreepConfig exact = cfg;  // no surrogate guess on this pass: exact solve
  exact.mode = 0;
  if (!rheology(M, O, c.mat[m], c.T[m], c.X[m], c.Y[m], eta, mu, &exact, &ci)) {
    atomicAdd(&st->bad_law, 1ULL);
    return;
  }
  c.eta[m] = eta;
  c.mu[m] = mu;
}

// limitViscosity (viscosity.c:90-104): every marker
__global__ void k_limit_viscosity(double *eta, double etamin, double etamax, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const double e = eta[m];
  if (e > etamax)
    eta[m] = etamax;
  else if (e < etamin)
    eta[m] = etamin;
}

// density update inline in main_subduction.c:255-264
// MAXT: also the maximum marker temperature of main:271-281 (in-domain markers, from 0; the bit
// patterns of non-negative doubles order as the values), one atomic per block into *maxT
// one marker; returns the bits of its temperature when it is in the domain and above 0, else 0
// (rho0, alpha: the materials' materialRho and materialAlpha)
__device__ __forceinline__ long long update_rho_one(const int *cellX, const int *mat, const double *T, double *rho,
                                                    double *rhodot, const double *rho0, const double *alpha,
                                                    int64_t n, int64_t m) {
  long long b = 0;  // bits of 0.0
  if (m < n && cellX[m] != -1) {
    const int k = mat[m];
    const double t = T[m];
    rho[m] = -rho0[k] * (alpha[k] * t);
    rhodot[m] = 0.0;
    if (t > 0.0) b = dbits(t);
  }
  return b;
}

// block maximum of non-negative double bit patterns, one atomic into *dst when above 0 (every
// thread of the block calls it; it may be called again right after)
__device__ __forceinline__ void block_max_to(long long b, unsigned long long *dst) {
  __shared__ long long wmax[32];
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_down_sync(0xffffffffu, b, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wmax[warp] = b;
  __syncthreads();
  if (warp == 0) {
    b = lane < (int)(blockDim.x >> 5) ? wmax[lane] : 0;
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_down_sync(0xffffffffu, b, o));
    if (lane == 0 && b > 0) atomicMax(dst, (unsigned long long)b);
  }
  __syncthreads();
}

struct Geo {
  const double *gx0, *gy0, *gx1, *gy1;
  const int *flags;
  const double *w0, *w1;  // stored corner weights (product build)
};

#ifndef MIC_EXACT
// Centre-cell weights of marker m: the stored ones, unless the interior clamp of centre_interp
// moved the cell (then formed from the offsets, as centre_interp forms them).
__device__ __forceinline__ W4 centre_w(const Params &P, const Geo &g, int64_t m, int cx, int cy,
                                       const double *__restrict__ X, const double *__restrict__ Y, int cmax, int &i,
                                       int &j) {
  const int fl = g.flags[m];
  const int sx = cx + (fl & 1), sy = cy + ((fl >> 1) & 1);
  i = clampi(sx, 1, cmax);
  j = clampi(sy, 1, P.NY - 2);
  if (i == sx && j == sy) return load_w4(g.w1, m);
  const double mdx = (i == sx) ? g.gx1[m] : div_sp(X[m] - P.xc[i], P.hxc[i], P.ixc[i]);
  const double mdy = (j == sy) ? g.gy1[m] : div_sp(Y[m] - P.yc[j], P.hyc[j], P.iyc[j]);
  return make_w4(mdx, mdy);
}
#endif

struct Nodal {
  const double *p, *exx, *exy, *soxx, *soyy, *soxy, *dsxx, *dsyy, *dsxy, *wxy;
};

struct StrainCols {
  const int *cellX, *cellY;
  const double *X, *Y, *eta, *mu;
  double *p, *exx, *eyy, *exy, *wxy, *srr;
  double *kxx, *kyy, *kxy;  // product build, when not null: the interpolated soxx, soyy, soxy kept
                            // for the sub-grid stress pass that follows in the same step
};

// updateMarkerStrainPressure (updateMarkerStrainPressure.c:131-306, non-TEXTURE branch)
// one marker (the marker-pass kernel k_batched runs it over a table of jobs)
__device__ __forceinline__ void strain_pressure_one(const Params &P, const StrainCols &c, const Geo &g,
                                                    const Nodal &nd, double dt, int64_t n, Status *st, int64_t m) {
  if (m >= n) return;
  const int cx = c.cellX[m], cy = c.cellY[m];
  if (cx == -1) return;
  // loaded ahead of the stores below (the compiler cannot tell the columns apart)
  const double eta = c.eta[m], mu = c.mu[m];
  int i, j;
  const int NX = P.NX;
#ifdef MIC_EXACT
  const double x = c.X[m], y = c.Y[m];
  double mdx, mdy;
  centre_interp(P, cx, cy, g.flags[m], g.gx1[m], g.gy1[m], x, y, centre_cmax(P), i, j, mdx, mdy);
  c.p[m] = interp_run(nd.p, NX, i, j, mdx, mdy);
  const double mexx = interp_run(nd.exx, NX, i, j, mdx, mdy);
  const double msxx = interp_run(nd.soxx, NX, i, j, mdx, mdy);
  const double msyy = interp_run(nd.soyy, NX, i, j, mdx, mdy);
  const double mdsxx = interp_run(nd.dsxx, NX, i, j, mdx, mdy);
  const double mdsyy = interp_run(nd.dsyy, NX, i, j, mdx, mdy);
  const double bx = g.gx0[m], by = g.gy0[m];
  c.wxy[m] = interp_run(nd.wxy, NX, cx, cy, bx, by);
  const double mexy = interp_run(nd.exy, NX, cx, cy, bx, by);
  const double msxy = interp_run(nd.soxy, NX, cx, cy, bx, by);
  const double mdsxy = interp_run(nd.dsxy, NX, cx, cy, bx, by);
#else
  // values that later enter a difference stay FP64: the strain-rate residual's (e11 - exx,
  // e12 - exy, with their sources) and the old stresses the sub-grid stress pass subtracts the
  // marker's from; pressure, dsyy and the vorticity in double-float arithmetic on the FP32 pipe
  // (mic_df.cuh)
  const W4 wc = centre_w(P, g, m, cx, cy, c.X, c.Y, centre_cmax(P), i, j);
  df wcd[4];
  w4_df(wc, wcd);
  c.p[m] = df_to_f64(interp_w_df(nd.p, NX, i, j, wcd));
  const double mexx = interp_w(nd.exx, NX, i, j, wc);
  const double msxx = interp_w(nd.soxx, NX, i, j, wc);
  const double msyy = interp_w(nd.soyy, NX, i, j, wc);
  const double mdsxx = interp_w(nd.dsxx, NX, i, j, wc);
  const df mdsyy = interp_w_df(nd.dsyy, NX, i, j, wcd);
  const W4 wb = load_w4(g.w0, m);
  df wbd[4];
  w4_df(wb, wbd);
  c.wxy[m] = df_to_f64(interp_w_df(nd.wxy, NX, cx, cy, wbd));
  const double mexy = interp_w(nd.exy, NX, cx, cy, wb);
  const double msxy = interp_w(nd.soxy, NX, cx, cy, wb);
  const double mdsxy = interp_w(nd.dsxy, NX, cx, cy, wb);
#endif
#ifdef MIC_EXACT
  const double e11 = msxx / 2.0 / eta + mdsxx / 2.0 / dt / mu;
  const double e22 = msyy / 2.0 / eta + mdsyy / 2.0 / dt / mu;
  const double e12 = msxy / 2.0 / eta + mdsxy / 2.0 / dt / mu;
#else
  // one division instead of nine: 1/(2 eta) and 1/(2 dt mu) from 1/(eta dt mu), shared by the
  // three components (within a few ulp of the reference's quotients)
  const double dtmu = dt * mu, den = eta * dtmu;
  double ie, idm;
  const unsigned ex = (unsigned)(dbits(den) >> 52) & 0x7ffu;  // den >= 0
  if (ex > 64u && ex < 1984u) {  // far from under- and overflow (an integer test)
    const double inv = 0.5 / den;
    ie = dtmu * inv;
    idm = eta * inv;
  } else {
    ie = 0.5 / eta;
    idm = 0.5 / dtmu;
  }
  const double e11 = fma(mdsxx, idm, msxx * ie);
  const double e22 = df_to_f64(df_fma(mdsyy, df_of(idm), df_mul(df_of(msyy), df_of(ie))));
  const double e12 = fma(mdsxy, idm, msxy * ie);
#endif
  c.exx[m] = e11;
  c.eyy[m] = e22;
  c.exy[m] = e12;
#ifndef MIC_EXACT
  if (c.kxx) {
    c.kxx[m] = msxx;
    c.kyy[m] = msyy;
    c.kxy[m] = msxy;
  }
#endif
  const double a = e11 - mexx, b = e12 - mexy;
#ifdef MIC_EXACT
  const double r = sqrt(a * a + b * b);  // pow(., 2.0) of the reference: the correctly rounded square
#else
  // the differences in FP64, their magnitude in double-float arithmetic (scaled)
  const double r = df_norm(a, b, 0.0, false);
#endif
  c.srr[m] = r;
  if (isnan(r)) atomicAdd(&st->nan_residual, 1ULL);
}

// area weighting of the projected residual (residual.c:23-38) and per-block partial sums
__global__ void k_residual_weight(Params P, double *srr, double *partial) {
  __shared__ double sh[kBlock];
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (q < (int64_t)P.NX * P.NY) {
    const int i = (int)(q % P.NX), j = (int)(q / P.NX);
    double s = srr[q];
    if (i > 0 && j > 0)
      s *= (P.x[i] - P.x[i - 1]) * (P.y[j] - P.y[j - 1]);
    else
      s = 0.0;
    srr[q] = s;
    v = s;
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double *partial, int np, double *out) {
  __shared__ double sh[1024];
  double v = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) v += partial[k];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

struct SubgridCols {
  const int *cellX, *cellY;
  const double *X, *Y, *eta, *mu;
  double *sxx, *syy, *sxy;
  double *dxy, *dxx, *dyy;  // per-marker stress changes (scratch)
};

// subgridStressChanges, marker part (subgridStressChanges.c:79-221)
// reuse (product build): dxx, dyy, dxy hold the nodal soxx, soyy, soxy interpolated at the
// marker by the strain-rate pass of this step (same nodes, weights and order: the same values)
// one marker (the marker-pass kernel k_batched runs it over a table of jobs)
__device__ __forceinline__ void subgrid_stress_one(const Params &P, const SubgridCols &c, const Geo &g,
                                                   const Nodal &nd, double dt, double D, int64_t n, int reuse,
                                                   int64_t m) {
  if (m >= n) return;
  const int cx = c.cellX[m], cy = c.cellY[m];
  if (cx == -1) return;
#ifdef MIC_EXACT
  const double sdm = c.eta[m] / c.mu[m];
  double sdif = -D * dt / sdm;
  if (sdif < -30.0) sdif = -30.0;
  sdif = 1.0 - exp(sdif);
  // the basic cell clamped to [0, NX-2] (subgridStressChanges.c:91-92): only a marker in the
  // last cell of a grid periodic in x moves, and its offset is formed again
  const int bxc = min(cx, P.NX - 2);
  const double bmdx = (bxc == cx) ? g.gx0[m] : div_sp(c.X[m] - P.x[bxc], P.hx[bxc], P.ix[bxc]);
  (void)reuse;
  double dsxy = interp_run(nd.soxy, P.NX, bxc, cy, bmdx, g.gy0[m]) - c.sxy[m];
  dsxy *= sdif;
  c.sxy[m] = c.sxy[m] + dsxy;
  int i, j;
  double mdx, mdy;
  centre_interp(P, cx, cy, g.flags[m], g.gx1[m], g.gy1[m], c.X[m], c.Y[m], P.NX - 2, i, j, mdx, mdy);
  double dsxx = interp_run(nd.soxx, P.NX, i, j, mdx, mdy) - c.sxx[m];
  dsxx *= sdif;
  c.sxx[m] = c.sxx[m] + dsxx;
  double dsyy = interp_run(nd.soyy, P.NX, i, j, mdx, mdy) - c.syy[m];
  dsyy *= sdif;
  c.syy[m] = c.syy[m] + dsyy;
#else
  // every marker load before the first store: the compiler cannot tell the columns apart, and a
  // load after a store would wait for it to issue
  const double s11 = c.sxx[m], s22 = c.syy[m], s12 = c.sxy[m];
  double mxy = 0.0, mxx = 0.0, myy = 0.0;
  if (reuse) {
    mxy = c.dxy[m];
    mxx = c.dxx[m];
    myy = c.dyy[m];
  }
  // the exponent -D dt mu / eta in double-float arithmetic (one FP64 add to bring it back); the
  // exponential and 1 - exp stay FP64, as the reference forms them
  double sdif = df_to_f64(df_div(df_mul(df_neg(df_mul(df_of(D), df_of(dt))), df_of(c.mu[m])), df_of(c.eta[m])));
  {
    const long long sb = dbits(sdif);  // sdif < -30 as an integer test (NaN stays NaN)
    if (sb < 0 && (sb & 0x7FFFFFFFFFFFFFFFLL) > dbits(30.0) && !nan_bits(sb)) sdif = -30.0;
  }
  sdif = 1.0 - exp(sdif);
  if (!reuse) {
    // the basic cell clamped to [0, NX-2] (subgridStressChanges.c:91-92): only a marker in the
    // last cell of a grid periodic in x moves, and its offset is formed again
    const int bxc = min(cx, P.NX - 2);
    mxy = interp_w(nd.soxy, P.NX, bxc, cy,
                   (bxc == cx) ? load_w4(g.w0, m) : make_w4(div_sp(c.X[m] - P.x[bxc], P.hx[bxc], P.ix[bxc]), g.gy0[m]));
    int i, j;
    const W4 wc = centre_w(P, g, m, cx, cy, c.X, c.Y, P.NX - 2, i, j);
    mxx = interp_w(nd.soxx, P.NX, i, j, wc);
    myy = interp_w(nd.soyy, P.NX, i, j, wc);
  }
  const double dsxy = (mxy - s12) * sdif, dsxx = (mxx - s11) * sdif, dsyy = (myy - s22) * sdif;
  c.sxy[m] = s12 + dsxy;
  c.sxx[m] = s11 + dsxx;
  c.syy[m] = s22 + dsyy;
#endif
  c.dxy[m] = dsxy;
  c.dxx[m] = dsxx;
  c.dyy[m] = dsyy;
}

#ifdef MIC_EXACT
// sums of local column L of node row j (the node's own column, or its periodic image)
__device__ __forceinline__ void subgrid_column(const Params &P, const int *__restrict__ cellX,
                                               const double *__restrict__ gx0, const double *__restrict__ gy0,
                                               const double *__restrict__ dxy, const double *__restrict__ dxx,
                                               const double *__restrict__ dyy, const int *__restrict__ cs, int L,
                                               int j, double &sxy, double &wxy, double &sxx, double &syy,
                                               double &wn) {
  const int NC = P.NCX;
  const long long half = 0x3FE0000000000000LL;
  const int cy0 = max(j - 1, 0), cy1 = min(j, P.NY - 2);
  const int cx0 = max(L - 1, 0), cx1 = min(L, NC - 1);
  if (cx0 <= cx1) {
    for (int cy = cy0; cy <= cy1; ++cy) {
      const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
      const int oy = j - cy;
      for (int m = mb; m < me; ++m) {
        const int ox = L - cellX[m];
        const double mx = gx0[m], my = gy0[m];
        const long long bx = nonneg_bits(mx), by = nonneg_bits(my);
        const bool inx = ox ? (bx >= half) : (bx <= half);
        const bool iny = oy ? (by >= half) : (by <= half);
        if (inx && iny) {
          const double w = (ox ? mx : (1.0 - mx)) * (oy ? my : (1.0 - my));
          sxy = sxy + w * dxy[m];
          wxy = wxy + w;
        }
      }
    }
  }
  if (L >= 1 && L - 1 < NC && j >= 1) {
    const int c = (j - 1) * NC + (L - 1);
    for (int m = cs[c]; m < cs[c + 1]; ++m) {
      const double w = (1.0 - fabs(0.5 - gx0[m])) * (1.0 - fabs(0.5 - gy0[m]));
      sxx += w * dxx[m];
      syy += w * dyy[m];
      wn += w;
    }
  }
}

// subgridStressChanges, node part (134-175 quadrant scatter, 227-233 centre scatter, 258-286
// divide and subtract) as a gather in marker order.  Periodic in x, nodes 0 and 1 add their seam
// image's sums after their own.
__global__ void __launch_bounds__(128) k_subgrid_stress_nodes(Params P, const int *__restrict__ cellX,
                                                              const double *__restrict__ gx0,
                                                              const double *__restrict__ gy0,
                                                              const double *__restrict__ dxy,
                                                              const double *__restrict__ dxx,
                                                              const double *__restrict__ dyy,
                                                              const int *__restrict__ cs, double *dsxx, double *dsyy,
                                                              double *dsxy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  double sxy = 0.0, wxy = 0.0, sxx = 0.0, syy = 0.0, wn = 0.0;
  double sxy2 = 0.0, wxy2 = 0.0, sxx2 = 0.0, syy2 = 0.0, wn2 = 0.0;
  subgrid_column(P, cellX, gx0, gy0, dxy, dxx, dyy, cs, i, j, sxy, wxy, sxx, syy, wn);
  if (P.xper && i + P.NX <= P.NCX + 1)
    subgrid_column(P, cellX, gx0, gy0, dxy, dxx, dyy, cs, i + P.NX, j, sxy2, wxy2, sxx2, syy2, wn2);
  const size_t q = (size_t)j * P.NX + i;
  const double W = (0.0 + wxy) + wxy2, Wn = (0.0 + wn) + wn2;
  const double gxy = (W != 0.0) ? ((0.0 + sxy) + sxy2) / W : 0.0;
  const double gxx = (Wn != 0.0) ? ((0.0 + sxx) + sxx2) / Wn : 0.0;
  const double gyy = (Wn != 0.0) ? ((0.0 + syy) + syy2) / Wn : 0.0;
  dsxx[q] = dsxx[q] + -1.0 * gxx;
  dsyy[q] = dsyy[q] + -1.0 * gyy;
  dsxy[q] = dsxy[q] + -1.0 * gxy;
}
#endif

#ifndef MIC_EXACT
// Product build: the same sums through per-cell partials.  One thread per basic cell walks the
// cell's markers once.  Each marker adds its dsxy to the corner node(s) its quadrant tests pick
// (both tests of subgridStressChanges.c:134-175 are inclusive, so a marker on a midline feeds two
// or four corners) in per-thread shared slots, and its dsxx, dsyy to the cell centre
// (227-233).  k_subgrid_combine then adds the four cells meeting at each node in a fixed order
// and divides.  Sums run in marker order within a cell; the cross-cell order differs from the
// reference's single loop (rounding at the last place), and is fixed, so runs reproduce.
// part[acc * ncells + cell]: corner k sxy at 2k, weight at 2k+1; centre sxx, syy, weight at 8..10.
constexpr int kSubgridBlocksPerSM = 4;
__global__ void __launch_bounds__(128) k_subgrid_partials(Params P, const double *__restrict__ gx0,
                                                          const double *__restrict__ gy0,
                                                          const double *__restrict__ wb,
                                                          const double *__restrict__ dxy,
                                                          const double *__restrict__ dxx,
                                                          const double *__restrict__ dyy,
                                                          const int *__restrict__ cs, double *__restrict__ part) {
  __shared__ double sloc[8][128];
  const int ncells = P.NCX * (P.NY - 1);
  const int t = threadIdx.x;
  // a persistent grid (kSubgridBlocksPerSM blocks of 128 per SM) walking the cells: each thread
  // streams its cell's markers from six columns, and with more warps per SM their sectors no
  // longer fit L1 (measured: 4.3 times the algorithmic DRAM bytes at the default occupancy)
  for (int c = blockIdx.x * blockDim.x + t; c < ncells; c += gridDim.x * blockDim.x) {
#pragma unroll
  for (int k = 0; k < 8; ++k) sloc[k][t] = 0.0;
  const long long half = 0x3FE0000000000000LL;
  double sxx = 0.0, syy = 0.0, wn = 0.0;
  const int mb = cs[c], me = cs[c + 1];
#pragma unroll 4
  for (int m = mb; m < me; ++m) {
    const double mx = gx0[m], my = gy0[m];
    const long long bx = nonneg_bits(mx), by = nonneg_bits(my);
    const int ox = bx > half, oy = by > half;  // the one corner off the midlines
    const double d = dxy[m];
    const W4 ww = load_w4(wb, m);  // (kx ? mx : 1 - mx) (ky ? my : 1 - my) for corner kx + 2 ky
    {
      const double w = w4_at(ww, ox + 2 * oy);
      double *L = &sloc[2 * (ox + 2 * oy)][t];
      L[0] = L[0] + w * d;
      L[128] = L[128] + w;
    }
    if (bx == half || by == half) {  // on a midline: the other corners whose tests hold too
      for (int k = 0; k < 4; ++k) {
        const int kx = k & 1, ky = k >> 1;
        if ((kx == ox && ky == oy) || (kx != ox && bx != half) || (ky != oy && by != half)) continue;
        const double w = w4_at(ww, k);
        double *L = &sloc[2 * k][t];
        L[0] = L[0] + w * d;
        L[128] = L[128] + w;
      }
    }
    const double wc = (1.0 - fabs(0.5 - mx)) * (1.0 - fabs(0.5 - my));
    sxx += wc * dxx[m];
    syy += wc * dyy[m];
    wn += wc;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) part[(size_t)k * ncells + c] = sloc[k][t];
  part[(size_t)8 * ncells + c] = sxx;
  part[(size_t)9 * ncells + c] = syy;
  part[(size_t)10 * ncells + c] = wn;
  }
}

// Node (i, j): dsxy sums of cells (i-1,j-1) corner 3, (i,j-1) corner 2, (i-1,j) corner 1, (i,j)
// corner 0; dsxx, dsyy from cell (i-1, j-1)'s centre; guarded divides and the subtraction of
// subgridStressChanges.c:258-286.
__global__ void __launch_bounds__(128) k_subgrid_combine(Params P, const double *__restrict__ part, double *dsxx,
                                                         double *dsyy, double *dsxy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  const int NC = P.NCX, ncells = NC * (P.NY - 1);
  double sxy = 0.0, wxy = 0.0, sxx = 0.0, syy = 0.0, wn = 0.0;
  // the node's own local column and, periodic in x, its seam image (nodes 0 and 1)
  const int nL = (P.xper && i + P.NX <= NC + 1) ? 2 : 1;
  for (int l = 0; l < nL; ++l) {
    const int L = i + l * P.NX;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int dx = r & 1, dy = r >> 1;
      const int cx = L - 1 + dx, cy = j - 1 + dy, k = (1 - dx) + 2 * (1 - dy);
      if (cx >= 0 && cx < NC && cy >= 0 && cy <= P.NY - 2) {
        const size_t cc = (size_t)cy * NC + cx;
        sxy += part[(size_t)(2 * k) * ncells + cc];
        wxy += part[(size_t)(2 * k + 1) * ncells + cc];
      }
    }
    if (L >= 1 && j >= 1 && L - 1 < NC && j <= P.NY - 1) {
      const size_t cc = (size_t)(j - 1) * NC + (L - 1);
      sxx += part[(size_t)8 * ncells + cc];
      syy += part[(size_t)9 * ncells + cc];
      wn += part[(size_t)10 * ncells + cc];
    }
  }
  const size_t q = (size_t)j * P.NX + i;
  const double W = 0.0 + wxy, Wn = 0.0 + wn;
  const double gxy = (W != 0.0) ? (0.0 + sxy) / W : 0.0;
  const double rn = (Wn != 0.0) ? 1.0 / Wn : 0.0;  // one division for the two centre sums
  const double gxx = (0.0 + sxx) * rn;
  const double gyy = (0.0 + syy) * rn;
  dsxx[q] = dsxx[q] + -1.0 * gxx;
  dsyy[q] = dsyy[q] + -1.0 * gyy;
  dsxy[q] = dsxy[q] + -1.0 * gxy;
}
#endif

struct StressCols {
  const int *cellX, *cellY;
  const double *X, *Y;
  double *sxx, *syy, *sxy;
};

// updateMarkerStress (updateMarkerStress.c:60-144)
// one marker (the marker-pass kernel k_batched runs it over a table of jobs)
__device__ __forceinline__ void update_stress_one(const Params &P, const StressCols &c, const Geo &g, const Nodal &nd,
                                                  int64_t n, Status *st, int64_t m) {
  if (m >= n) return;
  const int cx = c.cellX[m], cy = c.cellY[m];
  if (cx == -1) return;
  int i, j;
#ifdef MIC_EXACT
  double mdx, mdy;
  centre_interp(P, cx, cy, g.flags[m], g.gx1[m], g.gy1[m], c.X[m], c.Y[m], centre_cmax(P), i, j, mdx, mdy);
  const double mdsxx = interp_run(nd.dsxx, P.NX, i, j, mdx, mdy);
  const double mdsyy = interp_run(nd.dsyy, P.NX, i, j, mdx, mdy);
  c.sxx[m] = c.sxx[m] + mdsxx;
  c.syy[m] = c.syy[m] + mdsyy;
  const double mdsxy = interp_run(nd.dsxy, P.NX, cx, cy, g.gx0[m], g.gy0[m]);
  c.sxy[m] = c.sxy[m] + mdsxy;
#else
  // (FP64 interpolations: this pass does little FP64 work, and in double-float arithmetic it
  // measured slower, bound by its loads' latency.)  Every load before the first store: the
  // compiler cannot tell the columns apart, and a load after a store would wait for it to issue.
  const double s11 = c.sxx[m], s22 = c.syy[m], s12 = c.sxy[m];
  const W4 wb = load_w4(g.w0, m);
  const W4 wc = centre_w(P, g, m, cx, cy, c.X, c.Y, centre_cmax(P), i, j);
  const double mdsxx = interp_w(nd.dsxx, P.NX, i, j, wc);
  const double mdsyy = interp_w(nd.dsyy, P.NX, i, j, wc);
  const double mdsxy = interp_w(nd.dsxy, P.NX, cx, cy, wb);
  c.sxx[m] = s11 + mdsxx;
  c.syy[m] = s22 + mdsyy;
  c.sxy[m] = s12 + mdsxy;
#endif
  if (isnan(mdsxy)) atomicAdd(&st->nan_dsxy, 1ULL);
}

struct SubTCols {
  const int *cellX, *cellY;
  double *T, *Tdot;
  double *dTsub;
};

// subgridTemperatureChanges, first marker loop (subgridTemperatureChanges.c:45-70)
// one marker (the marker-pass kernel k_batched runs it over a table of jobs)
__device__ __forceinline__ void subgridT_markers_one(const Params &P, const SubTCols &c, const Geo &g, const double *__restrict__ Tn,
                                   const double *__restrict__ rn, const double *__restrict__ cpn,
                                   const double *__restrict__ kn, double rho0, double D, double dt, int64_t n, int64_t m) {
  if (m >= n) return;
  const int i = c.cellX[m], j = c.cellY[m];
  if (i == -1) return;
  const int NX = P.NX;
#ifdef MIC_EXACT
  // (node column i + 1 wraps to 0 across the seam of a grid periodic in x)
  const size_t k00 = (size_t)j * NX + i, k10 = (size_t)j * NX + next_col(i, NX), k01 = k00 + NX, k11 = k10 + NX;
  const double mdx = g.gx0[m], mdy = g.gy0[m];
  const double dx = P.x[i + 1] - P.x[i], dy = P.y[j + 1] - P.y[j];
  const double Tm = Tn[k00] * (1.0 - mdx) * (1.0 - mdy) + Tn[k10] * mdx * (1.0 - mdy) +
                    Tn[k01] * (1.0 - mdx) * (mdy) + Tn[k11] * mdx * mdy;
  const double rhom = rho0 + rn[k00] * (1.0 - mdx) * (1.0 - mdy) + rn[k10] * (mdx) * (1.0 - mdy) +
                      rn[k01] * (1.0 - mdx) * (mdy) + rn[k11] * mdx * mdy;
  const double cpm = cpn[k00] * (1.0 - mdx) * (1.0 - mdy) + cpn[k10] * (mdx) * (1.0 - mdy) +
                     cpn[k01] * (1.0 - mdx) * (mdy) + cpn[k11] * mdx * mdy;
  const double km = kn[k00] * (1.0 - mdx) * (1.0 - mdy) + kn[k10] * (mdx) * (1.0 - mdy) +
                    kn[k01] * (1.0 - mdx) * (mdy) + kn[k11] * mdx * mdy;
#else
  // the stored corner weights, shared by the four fields (the reference multiplies each value
  // by both factors in turn; the products agree to rounding)
  // T enters as the difference Tm - T: FP64; density, heat capacity and conductivity only form
  // the exponent, in double-float arithmetic on the FP32 pipe (mic_df.cuh)
  const W4 w = load_w4(g.w0, m);
  const double Tm = interp_w(Tn, NX, i, j, w);
  df wd[4];
  w4_df(w, wd);
  const df rhom = df_add(df_of(rho0), interp_w_df(rn, NX, i, j, wd));
  const df cpm = interp_w_df(cpn, NX, i, j, wd);
  const df km = interp_w_df(kn, NX, i, j, wd);
#endif
#ifdef MIC_EXACT
  const double tdiff = cpm * rhom / km / (2.0 / (dx * dx) + 2.0 / (dy * dy));
  c.dTsub[m] = (Tm - c.T[m]) * (1.0 - exp(-D * dt / tdiff));
#else
  // -D dt / tdiff = -D dt km 2 (1/dx^2 + 1/dy^2) / (cp rho), 1/dx and 1/dy from the reciprocal
  // tables; one FP64 add brings it back for the exponential
  const df ixx = df_of(P.ix[i]), iyy = df_of(P.iy[j]);
  const df h2 = df_scale(df_fma(ixx, ixx, df_mul(iyy, iyy)), 2.0f);
  const df num = df_mul(df_mul(df_neg(df_mul(df_of(D), df_of(dt))), km), h2);
  const double arg = df_to_f64(df_div(num, df_mul(cpm, rhom)));
  c.dTsub[m] = (Tm - c.T[m]) * (1.0 - exp(arg));
#endif
}

// nodal remainder thisT - lastT - projected subgrid change (VecAXPBYPCZ with alpha = 1)
__global__ void k_subgridT_nodes(const double *thisT, const double *lastT, const double *proj, double *dT,
                                 int64_t nn) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nn) return;
  dT[q] = thisT[q] + -1.0 * lastT[q] + -1.0 * proj[q];
}

// subgridTemperatureChanges, second marker loop (subgridTemperatureChanges.c:87-103)
// one marker (the marker-pass kernel k_batched runs it over a table of jobs)
__device__ __forceinline__ void subgridT_apply_one(const Params &P, const SubTCols &c, const Geo &g, const double *__restrict__ dT, double dt, int64_t n, int64_t m) {
  if (m >= n) return;
  const int i = c.cellX[m], j = c.cellY[m];
  if (i == -1) return;
#ifdef MIC_EXACT
  const size_t k00 = (size_t)j * P.NX + i, k10 = (size_t)j * P.NX + next_col(i, P.NX);
  const double mdx = g.gx0[m], mdy = g.gy0[m];
  const double dtm = (dT[k00] * (1.0 - mdy) * (1.0 - mdx) + dT[k00 + P.NX] * mdy * (1.0 - mdx) +
                      dT[k10] * (1.0 - mdy) * mdx + dT[k10 + P.NX] * mdy * mdx) +
                     c.dTsub[m];
#else
  const double dtm = interp_w(dT, P.NX, i, j, load_w4(g.w0, m)) + c.dTsub[m];
#endif
  c.T[m] = c.T[m] + dtm;
  c.Tdot[m] = dtm / dt;
}

#ifndef MIC_EXACT
// A nodal field's bilinear form on one cell in coefficient form, v = c0 + tx c1 + ty (c2 + tx c3)
// (corners 00, 10, 01, 11): three FMAs per evaluation instead of three subtractions
// and three FMAs.  The advection evaluates eleven of these per marker on three fields; forming
// the coefficients once per cell and step (a node kernel) moves the subtractions off the marker
// loop.  32-byte records: one cell's form is one aligned sector.
struct alignas(32) Bil4 {
  double c0, c1, c2, c3;
};
__device__ __forceinline__ Bil4 bil_coef(double f00, double f10, double f01, double f11) {
  Bil4 b;
  b.c0 = f00;
  b.c1 = f10 - f00;
  b.c2 = f01 - f00;
  b.c3 = (f11 - f01) - b.c1;
  return b;
}
// The advection's records hold the four coefficients as double-floats (hi, lo for c0 .. c3; the
// same 32 bytes): its marker loop evaluates them on the FP32 pipe (mic_df.cuh).
struct alignas(32) BilDF {
  float c0h, c0l, c1h, c1l, c2h, c2l, c3h, c3l;
};
__device__ __forceinline__ BilDF bil_coef_df(double f00, double f10, double f01, double f11) {
  const Bil4 b = bil_coef(f00, f10, f01, f11);
  const df c0 = df_of(b.c0), c1 = df_of(b.c1), c2 = df_of(b.c2), c3 = df_of(b.c3);
  return {c0.hi, c0.lo, c1.hi, c1.lo, c2.hi, c2.lo, c3.hi, c3.lo};
}
// c0 + tx c1 + ty (c2 + tx c3) in double-float arithmetic (two 16-byte loads, no FP64 instruction)
__device__ __forceinline__ df bil_eval_df(const BilDF *__restrict__ cells, size_t k, const df &tx, const df &ty) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(cells + k));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(cells + k) + 1);
  const df lower = df_fma(tx, df{a.z, a.w}, df{a.x, a.y});
  const df upper = df_fma(tx, df{b.z, b.w}, df{b.x, b.y});
  return df_fma(ty, upper, lower);
}

// The cells the advection interpolates on (markers.c:1978-2029), with the boundary ghosts it
// forms there: vx cells (NX-1 per row, rows vxY = -1 .. NY-2, the top ghost row from the top
// boundary condition), vy cells (NX per row, columns vyX = -1 .. NX-2, the left ghost column from
// the left boundary condition, rows 0 .. NY-2) and basic cells of the vorticity.
__global__ void k_advect_coef(const double *__restrict__ vx, const double *__restrict__ vy,
                              const double *__restrict__ wz, mic_bcinfo top, mic_bcinfo left, int NX, int NY,
                              BilDF *cvx, BilDF *cvy, BilDF *cwz) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < (int64_t)NY * (NX - 1)) {
    const int row = (int)(k / (NX - 1)), i = (int)(k % (NX - 1));
    const size_t r1 = (size_t)row * NX;
    double vul, vur;
    if (row == 0 && top.type[0] == 0) {
      vul = 2.0 * top.value[0] - vx[r1 + i];
      vur = 2.0 * top.value[0] - vx[r1 + i + 1];
    } else if (row == 0) {
      vul = vx[r1 + i];
      vur = vx[r1 + i + 1];
    } else {
      vul = vx[r1 - NX + i];
      vur = vx[r1 - NX + i + 1];
    }
    cvx[k] = bil_coef_df(vul, vur, vx[r1 + i], vx[r1 + i + 1]);
  }
  if (k < (int64_t)(NY - 1) * NX) {
    const int j = (int)(k / NX), col = (int)(k % NX);
    const size_t q0 = (size_t)j * NX, q1 = q0 + NX;
    double wul, wll;
    if (col == 0 && left.type[1] == 0) {
      wul = 2.0 * left.value[1] - vy[q0];
      wll = 2.0 * left.value[1] - vy[q1];
    } else if (col == 0) {
      wul = vy[q0];
      wll = vy[q1];
    } else {
      wul = vy[q0 + col - 1];
      wll = vy[q1 + col - 1];
    }
    cvy[k] = bil_coef_df(wul, vy[q0 + col], wll, vy[q1 + col]);
  }
  if (k < (int64_t)(NY - 1) * (NX - 1)) {
    const int j = (int)(k / (NX - 1)), i = (int)(k % (NX - 1));
    const size_t w0 = (size_t)j * NX + i;
    cwz[k] = bil_coef_df(wz[w0], wz[w0 + 1], wz[w0 + NX], wz[w0 + NX + 1]);
  }
}
#endif

struct AdvectCols {
  const int *cellX, *cellY;
  double *X, *Y, *VX, *VY, *wxy, *sxx, *syy, *sxy, *Eii;
  const double *exx, *eyy, *exy;
};

// advectMarkersRK (markers.c:1865-2250), non-periodic grid, non-JAUMANN rotation
// wz_known (product build): the marker's wxy column holds the vorticity k_strain_pressure of this
// step interpolated at the marker (the first stage's value: same nodes, weights and order)
// one in-domain marker m in stored cell (ci, cj); returns its rotated sxx
// (product build: cv holds the per-cell coefficient forms of vx, vy, wz, k_advect_coef)
struct AdvectCoef {
  const void *cvx, *cvy, *cwz;
};
__device__ __forceinline__ double advect_tail(const Params &P, const AdvectCols &c, double dt, int64_t m, double X0,
                                              double Y0, const double *mvx, const double *mvy, const double *mwz);
#ifndef MIC_EXACT
__device__ __forceinline__ double advect_tail_df(const Params &P, const AdvectCols &c, double dt, int64_t m, double X0,
                                                 double Y0, const df *mvx, const df *mvy, const df *mwz);
#endif

__device__ __forceinline__ double advect_marker(const Params &P, const AdvectCols &c, const Geo &g,
                                                const double *__restrict__ vx, const double *__restrict__ vy,
                                                const double *__restrict__ wz, const AdvectCoef &cv,
                                                const mic_bcinfo &top, const mic_bcinfo &left, double dt, int64_t m,
                                                int ci, int cj, int wz_known) {
#ifndef MIC_EXACT
  const BilDF *__restrict__ cvx = static_cast<const BilDF *>(cv.cvx);
  const BilDF *__restrict__ cvy = static_cast<const BilDF *>(cv.cvy);
  const BilDF *__restrict__ cwz = static_cast<const BilDF *>(cv.cwz);
#else
  (void)cv;
#endif
  const int NX = P.NX, NY = P.NY;
  const double X0 = c.X[m], Y0 = c.Y[m];
  double xcur = X0, ycur = Y0;
#ifdef MIC_EXACT
  double mvx[4], mvy[4], mwz[4];
#else
  // the stage values as double-floats (mic_df.cuh), and the half and full time steps
  df mvx[4], mvy[4], mwz[4];
  const df fdt = df_of(dt), hdt = df_scale(fdt, 0.5f);
#endif
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    // cell walk from the stored cell (markers.c:1928-1944) and the staggered-cell tests, all on
    // order-preserving integer images of the coordinates: same decisions as the FP64 compares
    // (a NaN coordinate compares false everywhere, as in the reference), none on the FP64 pipe
    const long long bx = ordered_bits(xcur), by = ordered_bits(ycur);
    const bool okx = !nan_bits(dbits(xcur)), oky = !nan_bits(dbits(ycur));
    int i = ci, j = cj;
    if (okx) {
      if (bx > P.xbits[i + 1]) {
        while (bx > P.xbits[i + 1] && i < NX - 2) i++;
      } else if (bx < P.xbits[i]) {
        while (bx < P.xbits[i] && i > 0) i--;
      }
    }
    if (oky) {
      if (by > P.ybits[j + 1]) {
        while (by > P.ybits[j + 1] && j < NY - 2) j++;
      } else if (by < P.ybits[j]) {
        while (by < P.ybits[j] && j > 0) j--;
      }
    }
    int vxX = i, vxY = j, vyX = i, vyY = j;
    if (vxY > -1 && oky && by < P.ycbits[vxY + 1]) vxY--;
    if (vyX > -1 && okx && bx < P.xcbits[vyX + 1]) vyX--;
    vxX = clampi(vxX, 0, NX - 2);
    vyX = clampi(vyX, -1, NX - 2);
    vxY = clampi(vxY, -1, NY - 2);
    vyY = clampi(vyY, 0, NY - 2);
#ifdef MIC_EXACT
    double ay = ycur - P.yc[vxY + 1];
    double ax = xcur - P.x[vxX];
    double hx = P.x[vxX + 1] - P.x[vxX];
    double hy = P.yc[vxY + 2] - P.yc[vxY + 1];
    const size_t r1 = (size_t)(vxY + 1) * NX;
    double vul, vur;
    if (vxY == -1 && top.type[0] == 0) {
      vul = 2.0 * top.value[0] - vx[r1 + vxX];
      vur = 2.0 * top.value[0] - vx[r1 + vxX + 1];
    } else if (vxY == -1) {
      vul = vx[r1 + vxX];
      vur = vx[r1 + vxX + 1];
    } else {
      vul = vx[r1 - NX + vxX];
      vur = vx[r1 - NX + vxX + 1];
    }
    const double vll = vx[r1 + vxX], vlr = vx[r1 + vxX + 1];
    double t = vul * (1.0 - ax / hx) * (1.0 - ay / hy);
    t += vur * (ax / hx) * (1.0 - ay / hy);
    t += vll * (1.0 - ax / hx) * (ay / hy);
    t += vlr * (ax * ay) / hx / hy;
    mvx[s] = t;
    const size_t q0 = (size_t)vyY * NX, q1 = q0 + NX;
    const double wur = vy[q0 + vyX + 1], wlr = vy[q1 + vyX + 1];
    double wul, wll;
    if (vyX == -1 && left.type[1] == 0) {
      wul = 2.0 * left.value[1] - vy[q0 + vyX + 1];
      wll = 2.0 * left.value[1] - vy[q1 + vyX + 1];
    } else if (vyX == -1) {
      wul = vy[q0 + vyX + 1];
      wll = vy[q1 + vyX + 1];
    } else {
      wul = vy[q0 + vyX];
      wll = vy[q1 + vyX];
    }
    ax = xcur - P.xc[vyX + 1];
    ay = ycur - P.y[vyY];
    hx = P.xc[vyX + 2] - P.xc[vyX + 1];
    hy = P.y[vyY + 1] - P.y[vyY];
    t = wul * (1.0 - ax / hx) * (1.0 - ay / hy);
    t += wur * (ax / hx) * (1.0 - ay / hy);
    t += wll * (1.0 - ax / hx) * (ay / hy);
    t += wlr * (ax * ay) / hx / hy;
    mvy[s] = t;
    const size_t w0 = (size_t)j * NX + i;
    const double mdx = div_sp(xcur - P.x[i], P.hx[i], P.ix[i]);
    const double mdy = div_sp(ycur - P.y[j], P.hy[j], P.iy[j]);
    t = (1.0 - mdx) * (1.0 - mdy) * wz[w0];
    t += (mdx) * (1.0 - mdy) * wz[w0 + 1];
    t += (1.0 - mdx) * (mdy)*wz[w0 + NX];
    t += (mdx) * (mdy)*wz[w0 + NX + 1];
    mwz[s] = t;
    if (s < 2) {
      xcur = X0 + dt / 2 * mvx[s];
      ycur = Y0 + dt / 2 * mvy[s];
    } else if (s == 2) {
      xcur = X0 + dt * mvx[s];
      ycur = Y0 + dt * mvy[s];
    }
#else
    // Fractions in the cells (they only weight interpolations: every cell decision above is on
    // integer images): the offset from the cell's line in FP64 (exact or within an ulp of the
    // offset), times the tabulated reciprocal spacing in double-float arithmetic.  vx sits on the
    // basic x lines and vy on the basic y lines: with vxX == i and vyY == j (the walk keeps i, j
    // inside the clamps) their fractions there are the basic cell's.  The first stage samples at
    // the marker itself, in its stored cell: its fractions are the binning geometry's (basic cell;
    // the vx cell's y and the vy cell's x fractions are those of the cell-centre cell, whose
    // stagger tests are the same).
    df fx, fy, fty, ftx;
    if (s == 0) {
      fx = df_of(g.gx0[m]);
      fy = df_of(g.gy0[m]);
      fty = df_of(g.gy1[m]);
      ftx = df_of(g.gx1[m]);
    } else {
      fx = df_mul(df_of(xcur - P.x[i]), df_of(P.ix[i]));
      fy = df_mul(df_of(ycur - P.y[j]), df_of(P.iy[j]));
      fty = df_mul(df_of(ycur - P.yc[vxY + 1]), df_of(P.iyc[vxY + 1]));
      ftx = df_mul(df_of(xcur - P.xc[vyX + 1]), df_of(P.ixc[vyX + 1]));
    }
    mvx[s] = bil_eval_df(cvx, (size_t)(vxY + 1) * (NX - 1) + vxX, fx, fty);
    mvy[s] = bil_eval_df(cvy, (size_t)vyY * NX + vyX + 1, ftx, fy);
    if (s == 0) {  // at the marker itself: the stored weights' form, as the strain pass forms it
      if (wz_known) {
        mwz[s] = df_of(c.wxy[m]);
      } else {
        df wbd[4];
        w4_df(load_w4(g.w0, m), wbd);
        mwz[s] = df_of(df_to_f64(interp_w_df(wz, NX, i, j, wbd)));
      }
    } else {
      mwz[s] = bil_eval_df(cwz, (size_t)j * (NX - 1) + i, fx, fy);
    }
    // the next stage's position: the displacement in double-float, added to the FP64 start
    if (s < 3) {
      const df h = (s < 2) ? hdt : fdt;
      xcur = X0 + df_to_f64(df_mul(h, mvx[s]));
      ycur = Y0 + df_to_f64(df_mul(h, mvy[s]));
    }
#endif
  }
#ifdef MIC_EXACT
  return advect_tail(P, c, dt, m, X0, Y0, mvx, mvy, mwz);
#else
  return advect_tail_df(P, c, dt, m, X0, Y0, mvx, mvy, mwz);
#endif
}

// The RK4 average of the four stages, the new position (wrapped across the seam of a grid
// periodic in x, markers.c:2225-2231), the stress rotation and the accumulated strain
// (markers.c:2120-2223).  Returns the rotated sxx.
__device__ __forceinline__ double advect_tail(const Params &P, const AdvectCols &c, double dt, int64_t m, double X0,
                                              double Y0, const double *mvx, const double *mvy, const double *mwz) {
#ifdef MIC_EXACT
  const double VX = div6(mvx[0] + 2 * mvx[1] + 2 * mvx[2] + mvx[3]);
  const double VY = div6(mvy[0] + 2 * mvy[1] + 2 * mvy[2] + mvy[3]);
  const double w = div6(mwz[0] + 2 * mwz[1] + 2 * mwz[2] + mwz[3]);
  c.VX[m] = VX;
  c.VY[m] = VY;
  c.wxy[m] = w;
  double Xn = X0 + dt * VX;
  c.Y[m] = Y0 + dt * VY;
#else
  const double inv6 = 0.16666666666666666;
  const double VX = (fma(2.0, mvx[2], fma(2.0, mvx[1], mvx[0])) + mvx[3]) * inv6;
  const double VY = (fma(2.0, mvy[2], fma(2.0, mvy[1], mvy[0])) + mvy[3]) * inv6;
  const double w = (fma(2.0, mwz[2], fma(2.0, mwz[1], mwz[0])) + mwz[3]) * inv6;
  c.VX[m] = VX;
  c.VY[m] = VY;
  c.wxy[m] = w;
  double Xn = fma(dt, VX, X0);
  c.Y[m] = fma(dt, VY, Y0);
#endif
  if (P.xper) {
    if (Xn > P.LX)
      Xn -= P.LX;
    else if (Xn < 0)
      Xn += P.LX;
  }
  c.X[m] = Xn;
  const double s11 = c.sxx[m], s22 = c.syy[m], s12 = c.sxy[m];
  double nsxx;
  if (P.jaumann) {
    // first-order Jaumann terms with wxy1 = wxy dt (markers.c:2147-2156)
    const double w1 = w * dt;
#ifdef MIC_EXACT
    nsxx = s11 + 2.0 * s12 * -w1;
    c.syy[m] = s22 + 2.0 * s12 * w1;
    c.sxy[m] = s12 + (s11 - s22) * w1;
#else
    nsxx = fma(2.0 * s12, -w1, s11);
    c.syy[m] = fma(2.0 * s12, w1, s22);
    c.sxy[m] = fma(s11 - s22, w1, s12);
#endif
    c.sxx[m] = nsxx;
  } else {
    const double th = -w * dt;
#ifdef MIC_EXACT
    const double ct = cos(th), st_ = sin(th), s2 = sin(2.0 * th), c2 = cos(2.0 * th);
    nsxx = s11 * (ct * ct) + s22 * (st_ * st_) - s12 * s2;
    c.sxx[m] = nsxx;
    c.syy[m] = s11 * (st_ * st_) + s22 * (ct * ct) + s12 * s2;
    c.sxy[m] = 0.5 * (s11 - s22) * s2 + s12 * c2;
#else
    double ct, st_, s2, c2;
    small_angle_rotation(th, ct, st_, s2, c2);
    const double cc = ct * ct, ss = st_ * st_;
    nsxx = fma(s11, cc, fma(s22, ss, -(s12 * s2)));
    c.sxx[m] = nsxx;
    c.syy[m] = fma(s11, ss, fma(s22, cc, s12 * s2));
    c.sxy[m] = fma(0.5 * (s11 - s22), s2, s12 * c2);
#endif
  }
#ifdef MIC_EXACT
  const double e11 = c.exx[m], e22 = c.eyy[m], e12 = c.exy[m];
  c.Eii[m] = c.Eii[m] + dt * sqrt(0.5 * (e11 * e11 + e22 * e22) + e12 * e12);
#else
  const double e11 = c.exx[m], e22 = c.eyy[m], e12 = c.exy[m];
  c.Eii[m] = fma(dt, sqrt(fma(e12, e12, 0.5 * fma(e11, e11, e22 * e22))), c.Eii[m]);
#endif
  return nsxx;
}

#ifndef MIC_EXACT
// sin^2 t and sin 2t of the rotation angle t of markers.c:2158-2164.  For |t| <= 2^-6 (an
// integer test) their Taylor series to t^8 (truncation below 1e-18 relative); sincos beyond.
__device__ __forceinline__ void rotation_terms(double t, double &ss, double &s2) {
  if (abs_le(t, 0.015625)) {
    const double t2 = t * t, u = 2.0 * t, u2 = 4.0 * t2;
    ss = t2 * fma(t2, fma(t2, fma(t2, -1.0 / 315.0, 2.0 / 45.0), -1.0 / 3.0), 1.0);
    s2 = u * fma(u2, fma(u2, fma(u2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), 1.0);
  } else {
    double sn, cs;
    sincos(t, &sn, &cs);
    ss = sn * sn;
    s2 = 2.0 * sn * cs;
  }
}

// The product build's tail of the advection on a grid not periodic in x: the RK4 averages of the
// double-float stage values (each entering FP64 once), the new position, the stress rotation and
// the accumulated strain (markers.c:2120-2223).  The exact rotation s' = R s R^T is written as
// its change: with d = s22 - s11, sxx' = sxx + (d sin^2 t - sxy sin 2t), syy' = syy minus the same,
// sxy' = sxy - (2 sxy sin^2 t + d sin 2t / 2) (cos^2 + sin^2 = 1), the changes formed in
// double-float arithmetic, so only the additions to the stresses are FP64.  Returns the rotated
// sxx.
__device__ __forceinline__ double advect_tail_df(const Params &P, const AdvectCols &c, double dt, int64_t m, double X0,
                                                 double Y0, const df *mvx, const df *mvy, const df *mwz) {
  // the marker's stresses and strain rates are loaded before the first store: the compiler
  // cannot tell the columns apart, and a load after a store would wait for it to issue
  const double s11 = c.sxx[m], s22 = c.syy[m], s12 = c.sxy[m];
  const double e11 = c.exx[m], e22 = c.eyy[m], e12 = c.exy[m], E0 = c.Eii[m];
  const df k6 = df_of(1.0 / 6.0);
  const df vxa = df_mul(df_add(df_add(mvx[0], mvx[3]), df_scale(df_add(mvx[1], mvx[2]), 2.0f)), k6);
  const df vya = df_mul(df_add(df_add(mvy[0], mvy[3]), df_scale(df_add(mvy[1], mvy[2]), 2.0f)), k6);
  const df wa = df_mul(df_add(df_add(mwz[0], mwz[3]), df_scale(df_add(mwz[1], mwz[2]), 2.0f)), k6);
  const double VX = df_to_f64(vxa), VY = df_to_f64(vya), w = df_to_f64(wa);
  c.VX[m] = VX;
  c.VY[m] = VY;
  c.wxy[m] = w;
  c.X[m] = fma(dt, VX, X0);
  c.Y[m] = fma(dt, VY, Y0);
  double nsxx;
  if (P.jaumann) {
    // first-order Jaumann terms with wxy1 = wxy dt (markers.c:2147-2156)
    const double w1 = w * dt;
    nsxx = fma(2.0 * s12, -w1, s11);
    c.syy[m] = fma(2.0 * s12, w1, s22);
    c.sxy[m] = fma(s11 - s22, w1, s12);
    c.sxx[m] = nsxx;
  } else {
    // (sin^2 t and sin 2t in FP64: forming them in double-float arithmetic as well measured slower,
    // the pass then being bound by instruction issue)
    double ss, s2;
    rotation_terms(-w * dt, ss, s2);
    const df d = df_of(s22 - s11), a = df_of(s12), dss = df_of(ss), ds2 = df_of(s2);
    const double c11 = df_to_f64(df_fma(d, dss, df_neg(df_mul(a, ds2))));
    const double c12 = df_to_f64(df_fma(df_scale(a, 2.0f), dss, df_scale(df_mul(d, ds2), 0.5f)));
    nsxx = s11 + c11;
    c.sxx[m] = nsxx;
    c.syy[m] = s22 - c11;
    c.sxy[m] = s12 - c12;
  }
  // accumulated strain: the invariant's square root as q / sqrt(q) by one reciprocal square root
  const double q = fma(e12, e12, 0.5 * fma(e11, e11, e22 * e22));
  const long long qb = dbits(q);
  const double rq = (qb == 0 || qb == 0x7FF0000000000000LL) ? q : q * rsqrt(q);
  c.Eii[m] = fma(dt, rq, E0);
  return nsxx;
}
#endif

// advectMarkersRK on a grid periodic in x (markers.c:1907-1913, 1928-1944, 1961-1966, 2014-2023):
// the cell walk runs over cells -1 .. NX-1 (line -1 and NX are the seam's images), the vx and vy
// cells are not clamped in x, node columns wrap, and the left wall has no ghost values.  The
// reference's own divisions, in both builds (periodic grids are small).
__device__ double advect_marker_periodic(const Params &P, const AdvectCols &c, const double *__restrict__ vx,
                                         const double *__restrict__ vy, const double *__restrict__ wz,
                                         const mic_bcinfo &top, double dt, int64_t m, int ci, int cj) {
  const int NX = P.NX, NY = P.NY;
  const double X0 = c.X[m], Y0 = c.Y[m];
  double xcur = X0, ycur = Y0;
  double mvx[4], mvy[4], mwz[4];
  for (int s = 0; s < 4; ++s) {
    int i = ci, j = cj;
    if (xcur > P.x[i + 1]) {
      while (xcur > P.x[i + 1] && i < NX - 1) i++;
    } else if (xcur < P.x[i]) {
      while (xcur < P.x[i] && i > -1) i--;
    }
    if (ycur > P.y[j + 1]) {
      while (ycur > P.y[j + 1] && j < NY - 2) j++;
    } else if (ycur < P.y[j]) {
      while (ycur < P.y[j] && j > 0) j--;
    }
    int vxX = i, vxY = j, vyX = i, vyY = j;
    if (vxY > -1 && ycur < P.yc[vxY + 1]) vxY--;
    if (vyX > -1 && xcur < P.xc[vyX + 1]) vyX--;
    vxY = clampi(vxY, -1, NY - 2);
    vyY = clampi(vyY, 0, NY - 2);
    const int a0 = wrap_col(vxX, NX), a1 = wrap_col(vxX + 1, NX);
    double deltaxm = xcur - P.x[vxX], deltaym = ycur - P.yc[vxY + 1];
    double dx = P.x[vxX + 1] - P.x[vxX], dy = P.yc[vxY + 2] - P.yc[vxY + 1];
    const size_t r1 = (size_t)(vxY + 1) * NX;
    double vul, vur;
    if (vxY == -1 && top.type[0] == 0) {
      vul = 2.0 * top.value[0] - vx[r1 + a0];
      vur = 2.0 * top.value[0] - vx[r1 + a1];
    } else if (vxY == -1) {
      vul = vx[r1 + a0];
      vur = vx[r1 + a1];
    } else {
      vul = vx[r1 - NX + a0];
      vur = vx[r1 - NX + a1];
    }
    const double vll = vx[r1 + a0], vlr = vx[r1 + a1];
    double t = vul * (1.0 - deltaxm / dx) * (1.0 - deltaym / dy);
    t += vur * (deltaxm / dx) * (1.0 - deltaym / dy);
    t += vll * (1.0 - deltaxm / dx) * (deltaym / dy);
    t += vlr * (deltaxm * deltaym) / dx / dy;
    mvx[s] = t;
    const int b0 = wrap_col(vyX, NX), b1 = wrap_col(vyX + 1, NX);
    const size_t q0 = (size_t)vyY * NX, q1 = q0 + NX;
    const double wul = vy[q0 + b0], wur = vy[q0 + b1], wll = vy[q1 + b0], wlr = vy[q1 + b1];
    deltaxm = xcur - P.xc[vyX + 1];
    deltaym = ycur - P.y[vyY];
    dx = P.xc[vyX + 2] - P.xc[vyX + 1];
    dy = P.y[vyY + 1] - P.y[vyY];
    t = wul * (1.0 - deltaxm / dx) * (1.0 - deltaym / dy);
    t += wur * (deltaxm / dx) * (1.0 - deltaym / dy);
    t += wll * (1.0 - deltaxm / dx) * (deltaym / dy);
    t += wlr * (deltaxm * deltaym) / dx / dy;
    mvy[s] = t;
    const int z0 = wrap_col(i, NX), z1 = wrap_col(i + 1, NX);
    const double mdx = (xcur - P.x[i]) / (P.x[i + 1] - P.x[i]);
    const double mdy = (ycur - P.y[j]) / (P.y[j + 1] - P.y[j]);
    const size_t k0 = (size_t)j * NX, k1 = k0 + NX;
    t = (1.0 - mdx) * (1.0 - mdy) * wz[k0 + z0];
    t += (mdx) * (1.0 - mdy) * wz[k0 + z1];
    t += (1.0 - mdx) * (mdy)*wz[k1 + z0];
    t += (mdx) * (mdy)*wz[k1 + z1];
    mwz[s] = t;
    if (s < 2) {
      xcur = X0 + dt / 2 * mvx[s];
      ycur = Y0 + dt / 2 * mvy[s];
    } else if (s == 2) {
      xcur = X0 + dt * mvx[s];
      ycur = Y0 + dt * mvy[s];
    }
  }
  return advect_tail(P, c, dt, m, X0, Y0, mvx, mvy, mwz);
}

// one marker; returns the bits of |sxx| after the rotation for an in-domain marker, else 0
__device__ __forceinline__ long long advect_one(const Params &P, const AdvectCols &c, const Geo &g,
                                                const double *__restrict__ vx, const double *__restrict__ vy,
                                                const double *__restrict__ wz, const AdvectCoef &cv,
                                                const mic_bcinfo &top, const mic_bcinfo &left, double dt, int64_t n,
                                                int wz_known, int64_t m) {
  long long b = 0;  // bits of 0.0
  if (m < n) {
    const int ci = c.cellX[m], cj = c.cellY[m];
    if (ci != -1) {
      const double a = fabs(P.xper ? advect_marker_periodic(P, c, vx, vy, wz, top, dt, m, ci, cj)
                                   : advect_marker(P, c, g, vx, vy, wz, cv, top, left, dt, m, ci, cj, wz_known));
      if (a > 0.0) b = dbits(a);
    }
  }
  return b;
}

// max over in-domain markers of v (or |v|), starting from 0 (main_subduction.c:271-281, 437-448)
__global__ void k_max(const int *cellX, const double *v, int absval, int64_t n, unsigned long long *out) {
  __shared__ long long sh[kBlock];
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  long long b = 0;  // bits of 0.0
  if (m < n && cellX[m] != -1) {
    double x = v[m];
    if (absval) x = fabs(x);
    if (x > 0.0) b = dbits(x);
  }
  sh[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] = max(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0 && sh[0] > 0) atomicMax(out, (unsigned long long)sh[0]);
}

// projectNodalFieldToMarkersS (markers.c:1670-1706)
__global__ void k_nodal_to_markers(Params P, const int *cellX, const int *cellY, Geo g, const double *f,
                                   double *dst, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const int i = cellX[m], j = cellY[m];
  if (i == -1) return;
  const double mdx = g.gx0[m], mdy = g.gy0[m];
  const size_t r0 = (size_t)j * P.NX, r1 = r0 + P.NX;
  const int i1 = next_col(i, P.NX);  // the seam image of column 0 on a grid periodic in x
  dst[m] = f[r0 + i] * (1 - mdx) * (1 - mdy) + f[r1 + i] * (1 - mdx) * mdy + f[r0 + i1] * (mdx) * (1 - mdy) +
           f[r1 + i1] * mdx * mdy;
}

Geo geo_of(mic_ctx *ctx) {
  Geo g;
  g.gx0 = ctx->geo[0];
  g.gy0 = ctx->geo[1];
  g.gx1 = ctx->geo[2];
  g.gy1 = ctx->geo[3];
  g.flags = ctx->geo_flags;
  g.w0 = ctx->wgt[0];
  g.w1 = ctx->wgt[1];
  return g;
}

Nodal nodal_of(mic_ctx *ctx) {
  Nodal d;
  d.p = ctx->nodal[MIC_NF_P];
  d.exx = ctx->nodal[MIC_NF_EDOTXX];
  d.exy = ctx->nodal[MIC_NF_EDOTXY];
  d.soxx = ctx->nodal[MIC_NF_SOXX];
  d.soyy = ctx->nodal[MIC_NF_SOYY];
  d.soxy = ctx->nodal[MIC_NF_SOXY];
  d.dsxx = ctx->nodal[MIC_NF_DSXX];
  d.dsyy = ctx->nodal[MIC_NF_DSYY];
  d.dsxy = ctx->nodal[MIC_NF_DSXY];
  d.wxy = ctx->nodal[MIC_NF_WXY];
  return d;
}

YieldCols yield_cols(mic_ctx *ctx) {
  YieldCols c;
  c.cellX = ctx->i32[C_CELLX];
  c.mat = ctx->i32[C_MAT];
  c.X = ctx->f64[C_X];
  c.Y = ctx->f64[C_Y];
  c.T = ctx->f64[C_T];
  c.p = ctx->f64[C_P];
  c.Eii = ctx->f64[C_EII];
  c.exx = ctx->f64[C_EXX];
  c.eyy = ctx->f64[C_EYY];
  c.exy = ctx->f64[C_EXY];
  c.grain = ctx->f64[C_GRAIN];
  c.eta = ctx->f64[C_ETA];
  c.mu = ctx->f64[C_MU];
  c.sxx = ctx->f64[C_SXX];
  c.syy = ctx->f64[C_SYY];
  c.sxy = ctx->f64[C_SXY];
  return c;
}

int read_status(mic_ctx *ctx) {
  MIC_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

int run_max(mic_ctx *ctx, int col, int absval, double *out) {
  unsigned long long *d = reinterpret_cast<unsigned long long *>(ctx->red_buf + 8);
  MIC_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n > 0) {
    {
      MIC_KERNEL(ctx, "k_max");
      k_max<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->i32[C_CELLX], ctx->f64[col], absval, ctx->n, d);
    }
    MIC_CUDA_TRY(cudaGetLastError());
  }
  if (out) {
    unsigned long long h = 0;
    MIC_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    double v;
    memcpy(&v, &h, sizeof(v));
    *out = v;
  }
  return MIC_OK;
}

// ---- marker-pass kernels over tables of jobs ---------------------------------------------
//
// A job is one context's launch of a marker pass (its columns, grid, settings).  Every marker
// pass runs as one kernel over a table of jobs: a single job when a context steps alone, every
// member's when an ensemble batches the pass.  Both launch the same kernel, so a member's markers
// go through the same machine code either way and come out bit for bit the same (the product
// build lets the compiler fuse multiplies and adds, and it may fuse the same source differently
// in two different kernels).  Each job's markers are cut into tiles of a fixed number of markers
// (a multiple of the block size); tile_start[j] is the first tile of job j (prefix sums, njobs + 1
// entries), so the table orders the tiles job-major in the order the jobs were added.  A block
// finds its tile's job by a binary search over tile_start, stages the job in shared memory and
// runs the per-marker code on the tile's markers; per-job reductions (flags, maxima) close at the
// end of each tile, since a tile never spans two jobs.

struct RhoJob {
  const int *cellX, *mat;
  const double *T;
  double *rho, *rhodot;
  double rho0[MIC_MAXMAT], alpha[MIC_MAXMAT];  // the materials' materialRho, materialAlpha
  int64_t n;
  unsigned long long *maxT;  // null: no maximum
};
struct YieldJob {
  YieldCols c;
  mic_materials M;
  mic_options O;
  CreepConfig cfg;
  double dt;
  int64_t n;
  Status *st;
  CreepCounters *cc;
  int limit;
};
struct StrainJob {
  Params P;
  StrainCols c;
  Geo g;
  Nodal nd;
  double dt;
  int64_t n;
  Status *st;
};
struct SubgridJob {
  Params P;
  SubgridCols c;
  Geo g;
  Nodal nd;
  double dt, D;
  int64_t n;
  int reuse;
};
struct StressJob {
  Params P;
  StressCols c;
  Geo g;
  Nodal nd;
  int64_t n;
  Status *st;
};
struct SubTJob {
  Params P;
  SubTCols c;
  Geo g;
  const double *Tn, *rn, *cpn, *kn;
  double rho0, D, dt;
  int64_t n;
};
struct SubTApplyJob {
  Params P;
  SubTCols c;
  Geo g;
  const double *dT;
  double dt;
  int64_t n;
};
struct AdvectJob {
  Params P;
  AdvectCols c;
  Geo g;
  const double *vx, *vy, *wz;
  AdvectCoef cv;
  mic_bcinfo top, left;
  double dt;
  int64_t n;
  int wz_known;
  unsigned long long *maxs;  // null: no maximum
};

constexpr int kBatchBlock = 256;  // threads per block of ensemble-batched passes (tensor-core yield: tc::kTile)

// the job of tile t: the last j with tile_start[j] <= t
__device__ __forceinline__ int tile_job(const int *__restrict__ ts, int njobs, int t) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(ts + mid) <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// How a block walks the tiles (block-uniform): walk 0 round-robin (tiles blockIdx.x, + gridDim.x,
// ...), 1 one contiguous run per block, 2 each block takes the next tile from a counter the grid
// shares (*ticket, 0 at launch): blocks that start late (other streams' kernels holding SMs) or
// meet costly markers take fewer tiles.
struct TileWalk {
  int first, end, step;
  unsigned int *ticket;  // walk 2
};
__device__ __forceinline__ TileWalk tile_walk(int ntiles, int walk, unsigned int *ticket) {
  TileWalk w;
  w.ticket = nullptr;
  if (walk == 2 && ticket) {
    w.first = 0;
    w.end = ntiles;
    w.step = 0;
    w.ticket = ticket;
  } else if (walk == 1) {
    w.first = (int)((long long)blockIdx.x * ntiles / gridDim.x);
    w.end = (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x);
    w.step = 1;
  } else {
    w.first = blockIdx.x;
    w.end = ntiles;
    w.step = gridDim.x;
  }
  return w;
}
__device__ __forceinline__ int walk_fetch(unsigned int *ticket) {
  __shared__ int s_next;
  if (threadIdx.x == 0) s_next = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int t = s_next;
  __syncthreads();  // every thread has read it before the next fetch overwrites it
  return t;
}
__device__ __forceinline__ int walk_start(const TileWalk &w) { return w.ticket ? walk_fetch(w.ticket) : w.first; }
__device__ __forceinline__ int walk_next(const TileWalk &w, int t) {
  return w.ticket ? walk_fetch(w.ticket) : t + w.step;
}

// the block's job j (or the kernel-argument job when the table is null) into shared memory;
// block-uniform, called between tiles
template <class Job>
__device__ __forceinline__ void stage_job(unsigned long long *sj, const Job *__restrict__ jobs, int j, const Job &one) {
  static_assert(sizeof(Job) % 8 == 0, "job records are whole 8-byte words");
  __syncthreads();
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(jobs ? jobs + j : &one);
  for (int w = threadIdx.x; w < (int)(sizeof(Job) / 8); w += blockDim.x) sj[w] = src[w];
  __syncthreads();
}

// Per-pass operations of the generic batched kernel: Acc is a thread's per-tile partial result,
// one() a marker, flush() closes a tile (every thread of the block calls it).
struct NoAcc {};
struct RhoOp {
  static constexpr int kMaxRegs = 64;
  using Job = RhoJob;
  using Acc = long long;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &a) {
    a = max(a, update_rho_one(J.cellX, J.mat, J.T, J.rho, J.rhodot, J.rho0, J.alpha, J.n, m));
  }
  static __device__ __forceinline__ void flush(const Job &J, Acc a) {
    if (J.maxT) block_max_to(a, J.maxT);
  }
};
template <int MODE>
struct YieldOp {
  static constexpr int kMaxRegs = 80;
  using Job = YieldJob;
  using Acc = int;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &a) {
    if (yield_one<MODE>(J.c, J.M, J.O, J.cfg, J.dt, J.n, J.st, J.cc, J.limit, nullptr, m)) a = 1;
  }
  static __device__ __forceinline__ void flush(const Job &J, Acc a) {
    if (__syncthreads_or(a) && threadIdx.x == 0) atomicOr(&J.st->is_yielding, 1);
  }
};
struct StrainOp {
  static constexpr int kMaxRegs = 64;
  using Job = StrainJob;
  using Acc = NoAcc;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &) {
    strain_pressure_one(J.P, J.c, J.g, J.nd, J.dt, J.n, J.st, m);
  }
  static __device__ __forceinline__ void flush(const Job &, Acc) {}
};
struct SubgridOp {
  static constexpr int kMaxRegs = 64;
  using Job = SubgridJob;
  using Acc = NoAcc;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &) {
    subgrid_stress_one(J.P, J.c, J.g, J.nd, J.dt, J.D, J.n, J.reuse, m);
  }
  static __device__ __forceinline__ void flush(const Job &, Acc) {}
};
struct StressOp {
  static constexpr int kMaxRegs = 48;
  using Job = StressJob;
  using Acc = NoAcc;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &) {
    update_stress_one(J.P, J.c, J.g, J.nd, J.n, J.st, m);
  }
  static __device__ __forceinline__ void flush(const Job &, Acc) {}
};
struct SubTOp {
  static constexpr int kMaxRegs = 64;
  using Job = SubTJob;
  using Acc = NoAcc;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &) {
    subgridT_markers_one(J.P, J.c, J.g, J.Tn, J.rn, J.cpn, J.kn, J.rho0, J.D, J.dt, J.n, m);
  }
  static __device__ __forceinline__ void flush(const Job &, Acc) {}
};
struct SubTApplyOp {
  static constexpr int kMaxRegs = 64;
  using Job = SubTApplyJob;
  using Acc = NoAcc;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &) {
    subgridT_apply_one(J.P, J.c, J.g, J.dT, J.dt, J.n, m);
  }
  static __device__ __forceinline__ void flush(const Job &, Acc) {}
};
struct AdvectOp {
  static constexpr int kMaxRegs = 64;
  using Job = AdvectJob;
  using Acc = long long;
  static __device__ __forceinline__ void one(const Job &J, int64_t m, Acc &a) {
    a = max(a, advect_one(J.P, J.c, J.g, J.vx, J.vy, J.wz, J.cv, J.top, J.left, J.dt, J.n, J.wz_known, m));
  }
  static __device__ __forceinline__ void flush(const Job &J, Acc a) {
    if (J.maxs) block_max_to(a, J.maxs);
  }
};

// One marker pass over every job of a table (tile_markers a multiple of blockDim.x, so every
// warp stays whole through the per-marker code and the tile's closing reduction).
// Op::kMaxRegs caps the registers (the job's fields otherwise stay in registers across the tile
// loop and halve the resident warps of the memory-bound passes); blocks of up to 512 threads.
// The caps were measured per pass on the 4,194,304-marker ice box: these passes wait mostly on
// loads, and the resident warps a lower cap buys outweigh the spills it costs (the advection at
// 64 registers spills about 0.5 KB per thread to L1 and runs 6% faster than at 80; at 48 its
// spills grow to 1.3 KB and it is slower again).
template <class Op>
__global__ void __maxnreg__(Op::kMaxRegs) k_batched(const typename Op::Job *__restrict__ jobs,
                                                         const int *__restrict__ ts, int njobs, int ntiles,
                                                         int tile_markers, int walk, unsigned int *ticket,
                                                         const __grid_constant__ typename Op::Job one) {
  using Job = typename Op::Job;
  __shared__ unsigned long long sj[sizeof(Job) / 8];
  const Job &J = *reinterpret_cast<const Job *>(sj);
  const TileWalk w = tile_walk(ntiles, walk, ticket);
  int cur = -1;
  for (int t = walk_start(w); t < w.end; t = walk_next(w, t)) {
    const int j = jobs ? tile_job(ts, njobs, t) : 0;
    if (j != cur) {  // the tile's job into shared memory (block-uniform)
      stage_job(sj, jobs, j, one);
      cur = j;
    }
    const int64_t base = (int64_t)(t - (jobs ? __ldg(ts + j) : 0)) * tile_markers;
    typename Op::Acc a{};
    for (int q = threadIdx.x; q < tile_markers; q += blockDim.x) Op::one(J, base + q, a);
    Op::flush(J, a);
  }
}

// checkPlasticYielding with the FP32 surrogate over a table: the hidden layer's weights are
// staged in shared memory again whenever a tile's member uses another network buffer.
__global__ void __launch_bounds__(512) k_yield_fp32_batched(const YieldJob *__restrict__ jobs,
                                                                    const int *__restrict__ ts, int njobs,
                                                                    int ntiles, int tile_markers, int walk,
                                                                    unsigned int *ticket,
                                                                    const __grid_constant__ YieldJob one) {
  __shared__ float w2s[kH * kH];
  __shared__ unsigned long long sj[sizeof(YieldJob) / 8];
  const YieldJob &J = *reinterpret_cast<const YieldJob *>(sj);
  const float *staged = nullptr;
  const TileWalk w = tile_walk(ntiles, walk, ticket);
  int cur = -1;
  for (int t = walk_start(w); t < w.end; t = walk_next(w, t)) {
    const int j = jobs ? tile_job(ts, njobs, t) : 0;
    if (j != cur) {
      stage_job(sj, jobs, j, one);
      cur = j;
    }
    if (J.cfg.mlp != staged) {
      staged = J.cfg.mlp;
      __syncthreads();
      for (int q = threadIdx.x; q < kH * kH; q += blockDim.x) w2s[q] = bf16_round(staged[kOffW2 + q]);
      __syncthreads();
    }
    const int64_t base = (int64_t)(t - (jobs ? __ldg(ts + j) : 0)) * tile_markers;
    int a = 0;
    for (int q = threadIdx.x; q < tile_markers; q += blockDim.x)
      if (yield_one<1>(J.c, J.M, J.O, J.cfg, J.dt, J.n, J.st, J.cc, J.limit, w2s, base + q)) a = 1;
    if (__syncthreads_or(a) && threadIdx.x == 0) atomicOr(&J.st->is_yielding, 1);
  }
}

// checkPlasticYielding with the tensor-core surrogate over a table (blocks of tc::kTile threads,
// tiles of multiples of tc::kTile markers).  The network is staged at the block's first tile
// and again when a tile's member reads another network buffer.  A block that gives up on the
// tensor path does so for the rest of its tiles (their markers take the exact solve); the drain
// timeout, if any, is counted on the member whose round gave up.
__global__ void __launch_bounds__(tc::kTile, tc::kBlocksPerSM) k_yield_tc_batched(const YieldJob *__restrict__ jobs,
                                                                const int *__restrict__ ts, int njobs, int ntiles,
                                                                int tile_markers, int walk, unsigned int *ticket,
                                                                const __grid_constant__ YieldJob one) {
  extern __shared__ unsigned char dyn[];
  __shared__ unsigned long long sj[sizeof(YieldJob) / 8];
  const YieldJob &J = *reinterpret_cast<const YieldJob *>(sj);
  const TileWalk w = tile_walk(ntiles, walk, ticket);
  int t = walk_start(w);
  if (t >= w.end) return;  // block-uniform, before any TMEM is taken
  tc::Block B;
  int cur = jobs ? tile_job(ts, njobs, t) : 0;
  stage_job(sj, jobs, cur, one);
  const float *staged = J.cfg.mlp;
  tc::setup(B, dyn, staged);
  CreepCounters *gave_up = nullptr;
  for (; t < w.end; t = walk_next(w, t)) {
    const int j = jobs ? tile_job(ts, njobs, t) : 0;
    if (j != cur) {
      stage_job(sj, jobs, j, one);
      cur = j;
    }
    if (J.cfg.mlp != staged) {
      staged = J.cfg.mlp;
      tc::restage(B, staged);
    }
    const int64_t base = (int64_t)(t - (jobs ? __ldg(ts + j) : 0)) * tile_markers;
    int a = 0;
    for (int q = 0; q < tile_markers; q += tc::kTile) {
      const int pending = B.pending;
      if (yield_tc_round(B, J.c, J.M, J.O, J.cfg, J.dt, J.n, J.st, J.cc, J.limit, base + q + threadIdx.x)) a = 1;
      if (!pending && B.pending) gave_up = J.cc;
    }
    if (__syncthreads_or(a) && threadIdx.x == 0) atomicOr(&J.st->is_yielding, 1);
  }
  tc::teardown(B, &(gave_up ? gave_up : J.cc)->tc_drain_timeouts);
}

constexpr size_t kJobBytes[BP_COUNT] = {sizeof(RhoJob),    sizeof(YieldJob),  sizeof(YieldJob), sizeof(YieldJob),
                                        sizeof(YieldJob),  sizeof(StrainJob), sizeof(SubgridJob), sizeof(StressJob),
                                        sizeof(SubTJob),   sizeof(SubTApplyJob), sizeof(AdvectJob)};
constexpr size_t kTableAlign = 256;

int batch_fail(cudaError_t e) { return mic_fail_cuda(nullptr, e); }

// the tensor-core yield kernel's shared memory (44 KB a block): the largest carveout, so that
// tc::kBlocksPerSM blocks fit an SM -- the occupancy calculator otherwise assumes the default split
cudaError_t tc_kernel_attributes() {
  cudaError_t e =
      cudaFuncSetAttribute(k_yield_tc_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kDynSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_yield_tc_batched, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  return e;
}

// resident blocks per SM of pass p's kernel at `block` threads (cached per device and shape)
int pass_occupancy(int dev, int pass, int block) {
  static int cache[64][BP_COUNT][5];
  const int bi = block / 128;
  if (dev < 0 || dev >= 64 || bi < 1 || bi > 4 || block % 128) return 1;
  int &c = cache[dev][pass][bi];
  if (c > 0) return c;
  int occ = 0;
  cudaError_t e;
  switch (pass) {
    case BP_RHO: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<RhoOp>, block, 0); break;
    case BP_YIELD_PLAIN: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<YieldOp<2>>, block, 0); break;
    case BP_YIELD_EXACT: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<YieldOp<0>>, block, 0); break;
    case BP_YIELD_FP32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_yield_fp32_batched, block, 0); break;
    case BP_YIELD_TC:
      e = tc_kernel_attributes();
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_yield_tc_batched, tc::kTile, tc::kDynSmem);
      break;
    case BP_STRAIN: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<StrainOp>, block, 0); break;
    case BP_SUBGRID: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<SubgridOp>, block, 0); break;
    case BP_STRESS: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<StressOp>, block, 0); break;
    case BP_SUBT: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<SubTOp>, block, 0); break;
    case BP_SUBT_APPLY: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<SubTApplyOp>, block, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched<AdvectOp>, block, 0); break;
  }
  if (e != cudaSuccess || occ < 1) occ = 1;
  c = occ;
  return c;
}

// pass p's kernel over a job table in device memory (jobs, ts), or over the single job `one`
// passed as a kernel argument (jobs null).  block: tc::kTile for the tensor-core yield.
template <class Job>
const Job &job_arg(const void *one) {
  static const Job zero{};
  return one ? *static_cast<const Job *>(one) : zero;
}

struct Walk {
  int walk;
  unsigned int *ticket;  // walk 2: zeroed on the stream before the launch
};

template <class Op>
void launch_generic(unsigned grid, int block, cudaStream_t s, const unsigned char *jobs, const int *ts, int nj,
                    int ntiles, int tm, Walk wk, const void *one) {
  using Job = typename Op::Job;
  k_batched<Op><<<grid, block, 0, s>>>(reinterpret_cast<const Job *>(jobs), ts, nj, ntiles, tm, wk.walk, wk.ticket,
                                       job_arg<Job>(one));
}

cudaError_t launch_pass(int pass, unsigned grid, int block, cudaStream_t s, const unsigned char *jobs, const int *ts,
                        int nj, int ntiles, int tm, Walk wk, const void *one) {
  if (wk.walk == 2) {
    const cudaError_t e = wk.ticket ? cudaMemsetAsync(wk.ticket, 0, sizeof(unsigned int), s) : cudaErrorInvalidValue;
    if (e != cudaSuccess) return e;
  }
  switch (pass) {
    case BP_RHO: launch_generic<RhoOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_YIELD_PLAIN: launch_generic<YieldOp<2>>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_YIELD_EXACT: launch_generic<YieldOp<0>>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_YIELD_FP32:
      k_yield_fp32_batched<<<grid, block, 0, s>>>(reinterpret_cast<const YieldJob *>(jobs), ts, nj, ntiles, tm,
                                                   wk.walk, wk.ticket, job_arg<YieldJob>(one));
      break;
    case BP_YIELD_TC: {
      const cudaError_t e = tc_kernel_attributes();
      if (e != cudaSuccess) return e;
      k_yield_tc_batched<<<grid, tc::kTile, tc::kDynSmem, s>>>(reinterpret_cast<const YieldJob *>(jobs), ts, nj,
                                                                ntiles, tm, wk.walk, wk.ticket,
                                                                job_arg<YieldJob>(one));
      break;
    }
    case BP_STRAIN: launch_generic<StrainOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_SUBGRID: launch_generic<SubgridOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_STRESS: launch_generic<StressOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_SUBT: launch_generic<SubTOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    case BP_SUBT_APPLY: launch_generic<SubTApplyOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
    default: launch_generic<AdvectOp>(grid, block, s, jobs, ts, nj, ntiles, tm, wk, one); break;
  }
  return cudaGetLastError();
}

// One context's marker pass: the pass kernel with the context's job as its argument -- one block
// per tile of one block's worth of markers (the tensor-core yield: the context's persistent
// tensor-core grid, each block taking the next tile from the context's counter for the pass).
template <class Job>
int solo_pass(mic_ctx *ctx, int pass, const Job &J, int block, const char *name) {
  const bool tcp = pass == BP_YIELD_TC;
  if (tcp) block = tc::kTile;
  const int64_t nt = (J.n + block - 1) / block;
  if (nt > 0x7fffffff) return MIC_ERR_ARG;
  const int ntiles = (int)nt;
  int64_t grid = tcp ? mic_creep_tc_blocks(ctx, J.n) : ntiles;
  if (grid < 1) grid = 1;
  MIC_KERNEL(ctx, name);
  const Walk wk = tcp ? Walk{2, ctx->tickets + pass} : Walk{0, nullptr};
  MIC_CUDA_TRY(launch_pass(pass, (unsigned)grid, block, ctx->stream, nullptr, nullptr, 1, ntiles, block, wk, &J));
  return MIC_OK;
}
}  // namespace

#define CHECK_CTX()                 \
  if (!ctx) return MIC_ERR_ARG;     \
  cudaSetDevice(ctx->device)

struct mic_batch {
  std::vector<unsigned char> jobs[BP_COUNT];  // job records of each pass, in the order added
  std::vector<int64_t> n[BP_COUNT];           // markers of each job
  // surrogate networks of the batch by content key: members holding the same network read one
  // copy of it, so a block of the batched yield pass stages it once
  std::vector<std::pair<unsigned long long, const float *>> nets;
  const float *shared_net(unsigned long long key, const float *own) {
    if (!key) return own;
    for (const auto &kv : nets)
      if (kv.first == key) return kv.second;
    nets.push_back({key, own});
    return own;
  }
  template <class J>
  int add(int pass, const J &job, int64_t markers) {
    std::vector<unsigned char> &v = jobs[pass];
    const size_t o = v.size();
    v.resize(o + sizeof(J));
    memcpy(v.data() + o, &job, sizeof(J));
    n[pass].push_back(markers);
    return MIC_OK;
  }
};

// with_max: the step's maximum marker temperature into the reduction slot as well (run_max's)
static int update_rho(mic_ctx *ctx, bool with_max, mic_batch *b = nullptr) {
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  unsigned long long *d = reinterpret_cast<unsigned long long *>(ctx->red_buf + 8);
  if (with_max) MIC_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n == 0) return MIC_OK;
  RhoJob J = {ctx->i32[C_CELLX], ctx->i32[C_MAT], ctx->f64[C_T], ctx->f64[C_RHO], ctx->f64[C_RHODOT], {}, {},
              ctx->n, with_max ? d : nullptr};
  for (int k = 0; k < MIC_MAXMAT; ++k) {
    J.rho0[k] = ctx->mat.materialRho[k];
    J.alpha[k] = ctx->mat.materialAlpha[k];
  }
  if (b) return b->add(BP_RHO, J, ctx->n);
  return solo_pass(ctx, BP_RHO, J, tuned_block(ctx, TU_UPDATE_RHO), "k_update_rho");
}

extern "C" int mic_update_marker_rho(mic_ctx *ctx) {
  CHECK_CTX();
  return update_rho(ctx, false);
}

extern "C" int mic_max_marker_T(mic_ctx *ctx, double *maxT) {
  CHECK_CTX();
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  return run_max(ctx, C_T, 0, maxT);
}

extern "C" int mic_max_abs_sxx(mic_ctx *ctx, double *v) {
  CHECK_CTX();
  return run_max(ctx, C_SXX, 1, v);
}

// limit: limitViscosity (viscosity.c:90-104) fused into the pass, for callers that run it next
static int yield_launch(mic_ctx *ctx, double dt, bool limit = false, mic_batch *b = nullptr) {
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  MIC_CUDA_TRY(cudaMemsetAsync(&ctx->d_status->is_yielding, 0, sizeof(int), ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(&ctx->d_status->bad_law, 0, sizeof(unsigned long long), ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(ctx->d_creep, 0, sizeof(CreepCounters), ctx->stream));
  if (ctx->n == 0) return MIC_OK;
  const int mode = ctx->creep.mlp ? ctx->creep.mode : 0;
  bool law7 = false;
  for (int k = 0; k < MIC_MAXMAT; ++k) law7 = law7 || ctx->mat.hasEtaT[k] == 7;
  YieldJob J = {yield_cols(ctx), ctx->mat,    ctx->opt,     ctx->creep,   dt,
                ctx->n,          ctx->d_status, ctx->d_creep, limit ? 1 : 0};
  const int pass = !law7 ? BP_YIELD_PLAIN : mode == 0 ? BP_YIELD_EXACT : mode == 1 ? BP_YIELD_FP32 : BP_YIELD_TC;
  if (b) {
    if (pass == BP_YIELD_FP32 || pass == BP_YIELD_TC) J.cfg.mlp = b->shared_net(ctx->mlp_key, J.cfg.mlp);
    return b->add(pass, J, ctx->n);
  }
  if (pass == BP_YIELD_PLAIN || pass == BP_YIELD_EXACT) return solo_pass(ctx, pass, J, tuned_block(ctx, TU_YIELD), "k_yield");
  if (pass == BP_YIELD_FP32) return solo_pass(ctx, pass, J, kBatchBlock, "k_yield_surrogate_fp32");
  return solo_pass(ctx, pass, J, tc::kTile, "k_yield_tc");
}

extern "C" int mic_check_plastic_yielding(mic_ctx *ctx, double dt, int *is_yielding, double elapsed_time) {
  CHECK_CTX();
  (void)elapsed_time;  // only read by the SANDBOX build of the reference
  int e = yield_launch(ctx, dt);
  if (e) return e;
  if ((e = read_status(ctx))) return e;
  if (is_yielding) *is_yielding = ctx->h_status->is_yielding;
  return ctx->h_status->bad_law ? MIC_ERR_LAW : MIC_OK;
}

extern "C" int mic_update_viscosity(mic_ctx *ctx) {
  CHECK_CTX();
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  MIC_CUDA_TRY(cudaMemsetAsync(&ctx->d_status->bad_law, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n > 0) {
    {
      MIC_KERNEL(ctx, "k_update_viscosity");
      k_update_viscosity<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(yield_cols(ctx), ctx->mat, ctx->opt,
                                                                       ctx->creep, ctx->n, ctx->d_status);
    }
    MIC_CUDA_TRY(cudaGetLastError());
  }
  if ((e = read_status(ctx))) return e;
  return ctx->h_status->bad_law ? MIC_ERR_LAW : MIC_OK;
}

extern "C" int mic_limit_viscosity(mic_ctx *ctx) {
  CHECK_CTX();
  if (ctx->n == 0) return MIC_OK;
  {
    MIC_KERNEL(ctx, "k_limit_viscosity");
    k_limit_viscosity<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->f64[C_ETA], ctx->opt.etamin,
                                                                    ctx->opt.etamax, ctx->n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

// keep: store the interpolated old stresses for a sub-grid stress pass that follows in this step
static int strain_launch(mic_ctx *ctx, double dt, bool keep = false, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  MIC_CUDA_TRY(cudaMemsetAsync(&ctx->d_status->nan_residual, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n == 0) return MIC_OK;
  StrainCols c;
  c.cellX = ctx->i32[C_CELLX];
  c.cellY = ctx->i32[C_CELLY];
  c.X = ctx->f64[C_X];
  c.Y = ctx->f64[C_Y];
  c.eta = ctx->f64[C_ETA];
  c.mu = ctx->f64[C_MU];
  c.p = ctx->f64[C_P];
  c.exx = ctx->f64[C_EXX];
  c.eyy = ctx->f64[C_EYY];
  c.exy = ctx->f64[C_EXY];
  c.wxy = ctx->f64[C_WXY];
  c.srr = ctx->f64[C_SRR];
  c.kxy = keep ? ctx->scr0 : nullptr;
  c.kxx = keep ? ctx->scr1 : nullptr;
  c.kyy = keep ? ctx->scr2 : nullptr;
  const StrainJob J = {ctx->P, c, geo_of(ctx), nodal_of(ctx), dt, ctx->n, ctx->d_status};
  if (b) return b->add(BP_STRAIN, J, ctx->n);
  return solo_pass(ctx, BP_STRAIN, J, tuned_block(ctx, TU_STRAIN), "k_strain_pressure");
}

extern "C" int mic_update_marker_strain_pressure(mic_ctx *ctx, double dt) {
  CHECK_CTX();
  int e = strain_launch(ctx, dt);
  if (e) return e;
  if ((e = read_status(ctx))) return e;
  return ctx->h_status->nan_residual ? MIC_ERR_NAN : MIC_OK;
}

static int residual_launch(mic_ctx *ctx, int iter, double *res_dev, cudaStream_t st = nullptr) {
  const cudaStream_t s = st ? st : ctx->stream;
  // binning first: a re-sort swaps the column buffers, so the srr column is taken after it
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  e = mic_project_scalar(ctx, ctx->f64[C_SRR], -1, ctx->nodal[MIC_NF_SRR], s);
  if (e) return e;
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  const int nb = (int)grid_for(nn);
  double *partial = ctx->node_scr[5];  // NX*NY >= number of blocks
  {
    MIC_KERNEL_ON(ctx, "k_residual_weight", s);
    k_residual_weight<<<nb, kBlock, 0, s>>>(ctx->P, ctx->nodal[MIC_NF_SRR], partial);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  {
    MIC_KERNEL_ON(ctx, "k_sum_partials", s);
    k_sum_partials<<<1, 1024, 0, s>>>(partial, nb, res_dev);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  (void)iter;
  return MIC_OK;
}

extern "C" int mic_update_global_strain_rate_residual(mic_ctx *ctx, int iter, double *residual) {
  CHECK_CTX();
  if (iter < 0) return MIC_ERR_ARG;
  double *d = ctx->red_buf + 16;
  int e = residual_launch(ctx, iter, d);
  if (e) return e;
  double s = 0.0;
  MIC_CUDA_TRY(cudaMemcpyAsync(&s, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  s /= (ctx->P.LX * ctx->P.LY);
  ctx->residuals[iter % 100] = s;
  if (residual) *residual = s;
  return MIC_OK;
}

// getGlobalStrainRateResidual / setGlobalStrainRateResidual (residual.c, residual.h:2-3): the
// stored residual of plasticity iteration iter (100 slots, as the reference's NRES)
extern "C" int mic_get_strain_rate_residual(mic_ctx *ctx, int iter, double *value) {
  if (!ctx || !value || iter < 0) return MIC_ERR_ARG;
  *value = ctx->residuals[iter % 100];
  return MIC_OK;
}
extern "C" int mic_set_strain_rate_residual(mic_ctx *ctx, int iter, double value) {
  if (!ctx || iter < 0) return MIC_ERR_ARG;
  ctx->residuals[iter % 100] = value;
  return MIC_OK;
}

// checkConvergence (residual.c:53-69)
extern "C" int mic_check_convergence(mic_ctx *ctx, double atol, double rtol, int iter, int *converged) {
  if (!ctx || !converged || iter < 0) return MIC_ERR_ARG;
  const double r = ctx->residuals[iter % 100];
  if (r < atol) {
    *converged = 1;
    return MIC_OK;
  }
  if (iter > 0) {
    const double last = ctx->residuals[(iter - 1) % 100];
    if (fabs((r - last) / last) < rtol) {
      *converged = 2;
      return MIC_OK;
    }
  }
  *converged = 0;
  return MIC_OK;
}

// subgridStressChanges, marker part.  reuse: k_strain_pressure of this step kept the
// interpolated old stresses in the scratch columns
static int subgrid_markers(mic_ctx *ctx, double dt, double D, bool reuse, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  if (ctx->n == 0) return MIC_OK;
  SubgridCols c;
  c.cellX = ctx->i32[C_CELLX];
  c.cellY = ctx->i32[C_CELLY];
  c.X = ctx->f64[C_X];
  c.Y = ctx->f64[C_Y];
  c.eta = ctx->f64[C_ETA];
  c.mu = ctx->f64[C_MU];
  c.sxx = ctx->f64[C_SXX];
  c.syy = ctx->f64[C_SYY];
  c.sxy = ctx->f64[C_SXY];
  c.dxy = ctx->scr0;
  c.dxx = ctx->scr1;
  c.dyy = ctx->scr2;
  const SubgridJob J = {ctx->P, c, geo_of(ctx), nodal_of(ctx), dt, D, ctx->n, reuse ? 1 : 0};
  if (b) return b->add(BP_SUBGRID, J, ctx->n);
  return solo_pass(ctx, BP_SUBGRID, J, tuned_block(ctx, TU_SUBGRID_STRESS), "k_subgrid_stress_markers");
}

// subgridStressChanges, node part: the nodal stress changes from the markers' ones
static int subgrid_nodes(mic_ctx *ctx) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  dim3 grid((ctx->P.NX + 127) / 128, ctx->P.NY);
#ifdef MIC_EXACT
  {
    MIC_KERNEL(ctx, "k_subgrid_stress_nodes");
    k_subgrid_stress_nodes<<<grid, 128, 0, ctx->stream>>>(ctx->P, ctx->i32[C_CELLX], ctx->geo[0], ctx->geo[1],
                                                          ctx->scr0, ctx->scr1, ctx->scr2, ctx->cell_start,
                                                          ctx->nodal[MIC_NF_DSXX], ctx->nodal[MIC_NF_DSYY],
                                                          ctx->nodal[MIC_NF_DSXY]);
  }
#else
  if (ctx->n > 0) {
    MIC_KERNEL(ctx, "k_subgrid_partials");
    const int64_t full = grid_for(ctx->ncells, 128), cap = (int64_t)kSubgridBlocksPerSM * sm_count(ctx);
    k_subgrid_partials<<<(unsigned)(full < cap ? full : cap), 128, 0, ctx->stream>>>(
        ctx->P, ctx->geo[0], ctx->geo[1], ctx->wgt[0], ctx->scr0, ctx->scr1, ctx->scr2, ctx->cell_start,
        ctx->part_b);
  } else {
    MIC_CUDA_TRY(cudaMemsetAsync(ctx->part_b, 0, sizeof(double) * 11 * (size_t)ctx->ncells, ctx->stream));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  {
    MIC_KERNEL(ctx, "k_subgrid_combine");
    k_subgrid_combine<<<grid, 128, 0, ctx->stream>>>(ctx->P, ctx->part_b, ctx->nodal[MIC_NF_DSXX],
                                                     ctx->nodal[MIC_NF_DSYY], ctx->nodal[MIC_NF_DSXY]);
  }
#endif
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

extern "C" int mic_subgrid_stress_changes(mic_ctx *ctx, double dt, double D) {
  CHECK_CTX();
  int e = subgrid_markers(ctx, dt, D, false);
  return e ? e : subgrid_nodes(ctx);
}

static int stress_launch(mic_ctx *ctx, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  MIC_CUDA_TRY(cudaMemsetAsync(&ctx->d_status->nan_dsxy, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n == 0) return MIC_OK;
  StressCols c;
  c.cellX = ctx->i32[C_CELLX];
  c.cellY = ctx->i32[C_CELLY];
  c.X = ctx->f64[C_X];
  c.Y = ctx->f64[C_Y];
  c.sxx = ctx->f64[C_SXX];
  c.syy = ctx->f64[C_SYY];
  c.sxy = ctx->f64[C_SXY];
  const StressJob J = {ctx->P, c, geo_of(ctx), nodal_of(ctx), ctx->n, ctx->d_status};
  if (b) return b->add(BP_STRESS, J, ctx->n);
  return solo_pass(ctx, BP_STRESS, J, tuned_block(ctx, TU_UPDATE_STRESS), "k_update_marker_stress");
}

extern "C" int mic_update_marker_stress(mic_ctx *ctx) {
  CHECK_CTX();
  return stress_launch(ctx);
}

static SubTCols subt_cols(mic_ctx *ctx) {
  SubTCols c;
  c.cellX = ctx->i32[C_CELLX];
  c.cellY = ctx->i32[C_CELLY];
  c.T = ctx->f64[C_T];
  c.Tdot = ctx->f64[C_TDOT];
  c.dTsub = ctx->scr0;
  return c;
}

// subgridTemperatureChanges in three parts: the markers' subgrid changes, their projection and
// the nodal remainder, and its interpolation back to the markers
static int subt_markers(mic_ctx *ctx, double dt, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  if (ctx->n == 0) return MIC_OK;
  const SubTJob J = {ctx->P,
                     subt_cols(ctx),
                     geo_of(ctx),
                     ctx->nodal[MIC_NF_LASTT],
                     ctx->nodal[MIC_NF_RHO],
                     ctx->nodal[MIC_NF_CP],
                     ctx->nodal[MIC_NF_KTHERMAL],
                     ctx->mat.materialRho[0],
                     ctx->opt.subgridTemperatureDiffusivity,
                     dt,
                     ctx->n};
  if (b) return b->add(BP_SUBT, J, ctx->n);
  return solo_pass(ctx, BP_SUBT, J, tuned_block(ctx, TU_SUBGRID_T), "k_subgridT_markers");
}

static int subt_nodes(mic_ctx *ctx) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  if ((e = mic_project_scalar(ctx, ctx->scr0, 0, ctx->node_scr[0]))) return e;
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  {
    MIC_KERNEL(ctx, "k_subgridT_nodes");
    k_subgridT_nodes<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->nodal[MIC_NF_THIST], ctx->nodal[MIC_NF_LASTT],
                                                               ctx->node_scr[0], ctx->node_scr[1], nn);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

static int subt_apply(mic_ctx *ctx, double dt, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  if (ctx->n == 0) return MIC_OK;
  const SubTApplyJob J = {ctx->P, subt_cols(ctx), geo_of(ctx), ctx->node_scr[1], dt, ctx->n};
  if (b) return b->add(BP_SUBT_APPLY, J, ctx->n);
  return solo_pass(ctx, BP_SUBT_APPLY, J, tuned_block(ctx, TU_SUBGRID_T_APPLY), "k_subgridT_apply");
}

extern "C" int mic_subgrid_temperature_changes(mic_ctx *ctx, double dt) {
  CHECK_CTX();
  int e;
  if ((e = subt_markers(ctx, dt)) || (e = subt_nodes(ctx)) || (e = subt_apply(ctx, dt))) return e;
  return MIC_OK;
}

// with_max: max |sxx| after the rotation into the reduction slot as well (run_max's)
static int advect_launch(mic_ctx *ctx, double dt, bool wz_known, bool with_max = false, mic_batch *b = nullptr) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  unsigned long long *d = reinterpret_cast<unsigned long long *>(ctx->red_buf + 8);
  if (with_max) MIC_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  if (ctx->n > 0) {
    AdvectCols c;
    c.cellX = ctx->i32[C_CELLX];
    c.cellY = ctx->i32[C_CELLY];
    c.X = ctx->f64[C_X];
    c.Y = ctx->f64[C_Y];
    c.VX = ctx->f64[C_VX];
    c.VY = ctx->f64[C_VY];
    c.wxy = ctx->f64[C_WXY];
    c.sxx = ctx->f64[C_SXX];
    c.syy = ctx->f64[C_SYY];
    c.sxy = ctx->f64[C_SXY];
    c.Eii = ctx->f64[C_EII];
    c.exx = ctx->f64[C_EXX];
    c.eyy = ctx->f64[C_EYY];
    c.exy = ctx->f64[C_EXY];
    AdvectCoef cv = {nullptr, nullptr, nullptr};
#ifndef MIC_EXACT
    if (!ctx->P.xper) {  // (the periodic advection interpolates the nodes directly)
      const int NX = ctx->P.NX, NY = ctx->P.NY;
      const size_t nn = (size_t)NX * NY;
      if (!ctx->adv_coef && cudaMalloc((void **)&ctx->adv_coef, 3 * nn * sizeof(BilDF)) != cudaSuccess) {
        ctx->adv_coef = nullptr;
        return MIC_ERR_NOMEM;
      }
      BilDF *cb = static_cast<BilDF *>(ctx->adv_coef);
      cv = {cb, cb + nn, cb + 2 * nn};
      MIC_KERNEL(ctx, "k_advect_coef");
      k_advect_coef<<<grid_for((int64_t)nn), kBlock, 0, ctx->stream>>>(
          ctx->nodal[MIC_NF_VX], ctx->nodal[MIC_NF_VY], ctx->nodal[MIC_NF_WXY], ctx->bcs.mechBCTop,
          ctx->bcs.mechBCLeft, NX, NY, cb, cb + nn, cb + 2 * nn);
    }
    MIC_CUDA_TRY(cudaGetLastError());
#endif
    const AdvectJob J = {ctx->P,
                         c,
                         geo_of(ctx),
                         ctx->nodal[MIC_NF_VX],
                         ctx->nodal[MIC_NF_VY],
                         ctx->nodal[MIC_NF_WXY],
                         cv,
                         ctx->bcs.mechBCTop,
                         ctx->bcs.mechBCLeft,
                         dt,
                         ctx->n,
                         wz_known ? 1 : 0,
                         with_max ? d : nullptr};
    if (b)
      b->add(BP_ADVECT, J, ctx->n);
    else if ((e = solo_pass(ctx, BP_ADVECT, J, tuned_block(ctx, TU_ADVECT), "k_advect")))
      return e;
  }
  // positions moved: cells, order and geometry are stale until the next binning
  ctx->sorted = 0;
  ctx->geo_valid = 0;
  return MIC_OK;
}

extern "C" int mic_advect_markers_rk(mic_ctx *ctx, double dt) {
  CHECK_CTX();
  return advect_launch(ctx, dt, false);
}

extern "C" int mic_project_nodal_field_to_markers(mic_ctx *ctx, int f, int off) {
  CHECK_CTX();
  if (f < 0 || f >= MIC_NF_COUNT) return MIC_ERR_ARG;
  const int col = mic_f64_column_of_offset(off);
  if (col < 0) return MIC_ERR_ARG;
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  if (ctx->n == 0) return MIC_OK;
  {
    MIC_KERNEL(ctx, "k_nodal_to_markers");
    k_nodal_to_markers<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->P, ctx->i32[C_CELLX], ctx->i32[C_CELLY],
                                                                     geo_of(ctx), ctx->nodal[f], ctx->f64[col], ctx->n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

// ---- step drivers ------------------------------------------------------------------

// One segment of a step (declared in mic_internal.cuh): the stages of main_subduction.c's time
// loop between one marker pass and the next, on the context's stream.
int mic_step_segment(mic_ctx *ctx, int seg, double dt_disp, double dt_thermal, int subgrid_stress, int wz_known,
                     mic_batch *b) {
  CHECK_CTX();
  int e;
  const bool sub = subgrid_stress && ctx->opt.subgridStressDiffusivity > 0.0;
#ifdef MIC_EXACT
  const bool keep = false;
#else
  // (not on a grid periodic in x: there the sub-grid pass clamps the marker's cells differently
  // from the strain-rate pass, subgridStressChanges.c:91-92, 186-187)
  const bool keep = sub && ctx->n > 0 && !ctx->P.xper;
#endif
  switch (seg) {
    case 0:
      // findMarkerCells (main:243, 247, 252): positions do not change between the three calls on
      // one rank without density control, so one binning gives all three results.  The density
      // update also finds the maximum temperature (main:271-281; the projection between changes no
      // marker temperature).
      if ((e = mic_bin_and_sort(ctx, nullptr))) return e;
      return update_rho(ctx, true, b);
    case 1:
#ifdef MIC_EXACT
      if ((e = mic_project_markers_nodes_all2(ctx))) return e;
      return yield_launch(ctx, dt_disp, false, b);
#else
      // The first projection (main:268) and the yield pass touch disjoint marker columns (rho, T,
      // materials against viscosity, modulus and stresses), and the first projection's viscosity
      // and stress fields are replaced by the second (main:303) before anything reads them: so it
      // forms only rho, k, T and Cp, on the second stream, beside the yield pass (which applies
      // the viscosity limit of main:297 to every marker as it stores the viscosities).
      if ((e = mic_ensure_geometry(ctx))) return e;
      MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[0], ctx->stream));
      MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->aux, ctx->aux_ev[0], 0));
      if ((e = mic_project_all2_first(ctx, ctx->aux))) return e;
      MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[1], ctx->aux));
      return yield_launch(ctx, dt_disp, /*limit=*/true, b);  // limitViscosity fused in
#endif
    case 2:
#ifdef MIC_EXACT
      if ((e = mic_limit_viscosity(ctx))) return e;
#else
      MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->aux_ev[1], 0));
#endif
      // the second projection: yielding and the limit changed viscosities and stresses only
      return mic_project_all2_viscous(ctx);
    case 3:
      return strain_launch(ctx, dt_disp, keep, b);
    case 4:
#ifdef MIC_EXACT
      if ((e = residual_launch(ctx, 0, ctx->red_buf + 16))) return e;
#else
      // the residual (a cell-centre projection of srr and its area-weighted sum) shares no buffer
      // with the sub-grid stress and stress-update passes: it runs on the second stream beside them
      if ((e = mic_ensure_geometry(ctx))) return e;
      MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[0], ctx->stream));
      MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->aux, ctx->aux_ev[0], 0));
      if ((e = residual_launch(ctx, 0, ctx->red_buf + 16, ctx->aux))) return e;  // leaves the scratch columns alone
      MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[1], ctx->aux));
#endif
      return sub ? subgrid_markers(ctx, dt_disp, ctx->opt.subgridStressDiffusivity, keep, b) : MIC_OK;
    case 5:
      if (sub && (e = subgrid_nodes(ctx))) return e;
      return stress_launch(ctx, b);
    case 6:
#ifndef MIC_EXACT
      MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->aux_ev[1], 0));
#endif
      return MIC_OK;
    case 7:
      return subt_markers(ctx, dt_thermal, b);
    case 8:
      if ((e = subt_nodes(ctx))) return e;
      return subt_apply(ctx, dt_thermal, b);
    case 9:
      // the advection also forms max |sxx| of the rotated stresses (main:437-448)
      return advect_launch(ctx, dt_thermal, wz_known != 0, true, b);
  }
  return MIC_ERR_ARG;
}

// segments [s0, s1) of a step, each marker pass launched on the context's stream
static int run_segments(mic_ctx *ctx, int s0, int s1, double dt_disp, double dt_thermal, int sub, int wz_known) {
  for (int k = s0; k < s1; ++k) {
    const int e = mic_step_segment(ctx, k, dt_disp, dt_thermal, sub, wz_known, nullptr);
    if (e) return e;
  }
  return MIC_OK;
}

static int read_max_slot(mic_ctx *ctx, double *out) {
  unsigned long long h = 0;
  MIC_CUDA_TRY(cudaMemcpyAsync(&h, ctx->red_buf + 8, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  memcpy(out, &h, sizeof(double));
  return MIC_OK;
}

extern "C" int mic_step_pre_stokes(mic_ctx *ctx, double dt_disp, int *is_yielding, double *max_T) {
  CHECK_CTX();
  int e;
  if ((e = run_segments(ctx, 0, 3, dt_disp, 0.0, 0, 0))) return e;
  if (is_yielding || max_T) {
    if ((e = read_status(ctx))) return e;
    if (is_yielding) *is_yielding = ctx->h_status->is_yielding;
    if (max_T && (e = read_max_slot(ctx, max_T))) return e;
  }
  return MIC_OK;
}

static int read_residual(mic_ctx *ctx, double *residual) {
  double s = 0.0;
  MIC_CUDA_TRY(cudaMemcpyAsync(&s, ctx->red_buf + 16, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  s /= (ctx->P.LX * ctx->P.LY);
  ctx->residuals[0] = s;
  *residual = s;
  return MIC_OK;
}

extern "C" int mic_step_post_stokes(mic_ctx *ctx, double dt_disp, int subgrid_stress, double *residual) {
  CHECK_CTX();
  int e;
  if ((e = run_segments(ctx, 3, 7, dt_disp, 0.0, subgrid_stress, 0))) return e;
  return residual ? read_residual(ctx, residual) : MIC_OK;
}

extern "C" int mic_step_post_thermal(mic_ctx *ctx, double dt_thermal, double *max_abs_sxx) {
  CHECK_CTX();
  int e;
  // the marker vorticity may be stale here: a caller between the calls may replace nodal fields
  if ((e = run_segments(ctx, 7, kStepSegments, 0.0, dt_thermal, 0, 0))) return e;
  return max_abs_sxx ? read_max_slot(ctx, max_abs_sxx) : MIC_OK;
}

extern "C" int mic_step(mic_ctx *ctx, double dt_disp, double dt_thermal, int subgrid_stress, double *residual) {
  CHECK_CTX();
  int e;
  if ((e = run_segments(ctx, 0, 7, dt_disp, dt_thermal, subgrid_stress, 0))) return e;
  if (residual && (e = read_residual(ctx, residual))) return e;
#ifdef MIC_EXACT
  const int wz_known = 0;
#else
  // the marker vorticity is this step's k_strain_pressure value on the nodal wxy the advection reads
  const int wz_known = ctx->n > 0;
#endif
  return run_segments(ctx, 7, kStepSegments, dt_disp, dt_thermal, subgrid_stress, wz_known);
}

// ---- batches --------------------------------------------------------------------------

mic_batch *mic_batch_new() { return new (std::nothrow) mic_batch(); }
void mic_batch_free(mic_batch *b) { delete b; }
void mic_batch_clear(mic_batch *b) {
  for (int p = 0; p < BP_COUNT; ++p) {
    b->jobs[p].clear();
    b->n[p].clear();
  }
  b->nets.clear();
}
bool mic_batch_empty(const mic_batch *b) {
  for (int p = 0; p < BP_COUNT; ++p)
    if (!b->n[p].empty()) return false;
  return true;
}


size_t mic_batch_table_bound(int n_members) {
  size_t per = sizeof(RhoJob) + sizeof(YieldJob) + sizeof(StrainJob) + sizeof(SubgridJob) + sizeof(StressJob) +
               sizeof(SubTJob) + sizeof(SubTApplyJob) + sizeof(AdvectJob);
  return (size_t)n_members * per + (size_t)BP_COUNT * (kTableAlign + sizeof(int) * ((size_t)n_members + 2)) +
         kTableAlign;
}

int mic_batch_launch(mic_batch *b, const BatchShape *shape, unsigned char *host_table, unsigned char *dev_table,
                     size_t *off, size_t cap, int copy, cudaStream_t s, long long *launches) {
  int dev = 0, nsm = 0;
  cudaError_t ce;
  if ((ce = cudaGetDevice(&dev)) != cudaSuccess) return batch_fail(ce);
  if ((ce = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return batch_fail(ce);
  int status = MIC_OK;
  for (int p = 0; p < BP_COUNT && status == MIC_OK; ++p) {
    const int nj = (int)b->n[p].size();
    if (nj == 0) continue;
    const bool tcp = p == BP_YIELD_TC;
    const int block = tcp ? tc::kTile : kBatchBlock;
    // the surrogate passes stage the network per block (and again when a tile's job reads another
    // copy): a persistent grid walking tiles of one block round-robin, as a context alone runs
    // them, which also spreads the markers' uneven solve costs over the blocks
    const bool surrogate = tcp || p == BP_YIELD_FP32;
    const int persistent = surrogate ? 1 : shape[p].persistent;
    const int walk = surrogate ? 2 : (persistent ? shape[p].chunked : 0);
    const int mult = surrogate ? 1 : (shape[p].mult < 1 ? 1 : (shape[p].mult > 64 ? 64 : shape[p].mult));
    const int tm = block * mult;
    std::vector<int> ts(nj + 2, 0);  // tile offsets, then the walk's ticket (zeroed before the launch)
    for (int j = 0; j < nj; ++j) {
      const int64_t t = (b->n[p][j] + tm - 1) / tm;
      if ((int64_t)ts[j] + t > 0x7fffffff) {
        status = MIC_ERR_ARG;
        break;
      }
      ts[j + 1] = ts[j] + (int)t;
    }
    if (status) break;
    const int ntiles = ts[nj];
    const size_t o = (*off + kTableAlign - 1) / kTableAlign * kTableAlign;
    const size_t jb = b->jobs[p].size(), tb = sizeof(int) * (size_t)(nj + 2);  // tile offsets, then the ticket
    if (jb != (size_t)nj * kJobBytes[p] || o + jb + tb > cap) {
      status = MIC_ERR_NOMEM;
      break;
    }
    memcpy(host_table + o, b->jobs[p].data(), jb);
    memcpy(host_table + o + jb, ts.data(), tb);
    if (copy && (ce = cudaMemcpyAsync(dev_table + o, host_table + o, jb + tb, cudaMemcpyHostToDevice, s)) != cudaSuccess) {
      status = batch_fail(ce);
      break;
    }
    *off = o + jb + tb;
    const unsigned char *dj = dev_table + o;
    const int *dts = reinterpret_cast<const int *>(dev_table + o + jb);
    unsigned int *ticket = reinterpret_cast<unsigned int *>(dev_table + o + jb) + nj + 1;
    int64_t grid = ntiles;
    if (persistent) {
      const int occ = pass_occupancy(dev, p, block);
      const int64_t g = (int64_t)nsm * (tcp && occ > tc::kGridBlocksPerSM ? tc::kGridBlocksPerSM : occ);
      if (g < grid) grid = g;
    }
    if (grid < 1) grid = 1;
    if ((ce = launch_pass(p, (unsigned)grid, block, s, dj, dts, nj, ntiles, tm, Walk{walk, ticket}, nullptr)) !=
        cudaSuccess) {
      status = batch_fail(ce);
      break;
    }
    if (launches) ++*launches;
  }
  mic_batch_clear(b);
  return status;
}
