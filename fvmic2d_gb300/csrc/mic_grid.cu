// mic_grid.cu -- the grid routines between the host solves, on the context's nodal arrays:
// nodalStressStrain (nodalStressStrain.c:6-486), limitDisplacementTimestep (limitTimestep.c:
// 6-133) and retrieveSolutions (retrieveSolutions.c:4-82).  With them on the device the
// Stokes solution goes up once (the solver's vector) and nothing comes back down for the
// marker passes that follow.
#include <climits>
#include <cmath>
#include <cstring>

#include "mic_internal.cuh"

using namespace mic;

namespace {

struct GridFields {
  const double *vx, *vy, *etaN, *muN, *etaS, *muS, *rho, *rhodot;
  double *exx, *eyy, *exy, *wxy, *soxx, *soyy, *soxy, *dsxx, *dsyy, *dsxy, *eii, *sii, *heat;
};

GridFields grid_fields(mic_ctx *ctx) {
  double **f = ctx->nodal;
  return GridFields{f[MIC_NF_VX], f[MIC_NF_VY], f[MIC_NF_ETAN], f[MIC_NF_MUN], f[MIC_NF_ETAS], f[MIC_NF_MUS],
                    f[MIC_NF_RHO], f[MIC_NF_RHODOT], f[MIC_NF_EDOTXX], f[MIC_NF_EDOTYY], f[MIC_NF_EDOTXY],
                    f[MIC_NF_WXY], f[MIC_NF_SOXX], f[MIC_NF_SOYY], f[MIC_NF_SOXY], f[MIC_NF_DSXX],
                    f[MIC_NF_DSYY], f[MIC_NF_DSXY], f[MIC_NF_EII], f[MIC_NF_SII], f[MIC_NF_HEATING]};
}

// The grid kernels are cheap (one thread per node): every operation is an IEEE intrinsic in
// the reference's order, so neither build contracts or rewrites anything and both give the
// reference's bits.
__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D(double a, double b) { return __ddiv_rn(a, b); }

// visco-elastic update of one stress component (nodalStressStrain.c:101-125 as vector ops):
// X = eta ./ (eta + dt mu) (0 for a zero divisor), X1 = eta (-2 X + 2), s = X1 e + X s_old,
// ds = s - s_old
__device__ __forceinline__ void ve_update(double eta, double mu, double dt, double e, double &so, double &ds) {
  const double den = A(eta, M(dt, mu));
  const double X = den != 0.0 ? D(eta, den) : 0.0;
  const double X1 = M(eta, A(M(-2.0, X), 2.0));
  const double et = M(X1, e);
  double st = M(X, so);
  st = A(st, M(1.0, et));
  ds = A(st, M(-1.0, so));
  so = st;
}

// per node: deviatoric strain rates at the cell centre (zero on the first row and column),
// vorticity and shear strain rate at the basic node (wall ghosts from the boundary values),
// and the stress updates of both
__global__ void k_nss_pointwise(Params P, GridFields g, mic_bcinfo left, mic_bcinfo top, double dt) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (k >= (int64_t)NX * NY) return;
  const int ix = (int)(k % NX), jy = (int)(k / NX);
  double exx = 0.0, eyy = 0.0;
  if (ix > 0 && jy > 0) {
    const double ux = S(g.vx[k - NX], g.vx[k - NX - 1]);  // vx[jy-1][ix] - vx[jy-1][ix-1]
    const double uy = S(g.vy[k - 1], g.vy[k - NX - 1]);   // vy[jy][ix-1] - vy[jy-1][ix-1]
    const double a = D(ux, P.hx[ix - 1]);                 // dx = x[ix] - x[ix-1]
    const double b = D(uy, P.hy[jy - 1]);
    const double divv = A(a, b);
    exx = S(a, D(divv, 3.0));
    eyy = S(b, D(divv, 3.0));
  }
  g.exx[k] = exx;
  g.eyy[k] = eyy;
  double so = g.soxx[k], ds;
  ve_update(g.etaN[k], g.muN[k], dt, exx, so, ds);
  g.soxx[k] = so;
  g.dsxx[k] = ds;
  so = g.soyy[k];
  ve_update(g.etaN[k], g.muN[k], dt, eyy, so, ds);
  g.soyy[k] = so;
  g.dsyy[k] = ds;
  // basic node (nodalStressStrain.c:150-230)
  const double vyp = g.vy[k], vxp = g.vx[k];
  const double vym = ix == 0 ? (left.type[1] == 0 ? S(M(2.0, left.value[1]), vyp) : vyp) : g.vy[k - 1];
  const double vxm = jy == 0 ? (top.type[0] == 0 ? S(M(2.0, top.value[0]), vxp) : vxp) : g.vx[k - NX];
  const double qy = D(S(vxp, vxm), P.hyc[jy]);  // dy = yc[jy+1] - yc[jy]
  const double qx = D(S(vyp, vym), P.hxc[ix]);
  g.wxy[k] = M(0.5, S(qy, qx));
  const double exy = M(0.5, A(qy, qx));
  g.exy[k] = exy;
  so = g.soxy[k];
  ve_update(g.etaS[k], g.muS[k], dt, exy, so, ds);
  g.soxy[k] = so;
  g.dsxy[k] = ds;
}

// shear heating and the second invariants at interior basic nodes (nodalStressStrain.c:
// 330-370), from the four surrounding cell centres; zero elsewhere
__global__ void k_nss_invariants(Params P, GridFields g) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (a >= (int64_t)NX * NY) return;
  const int ix = (int)(a % NX), jy = (int)(a / NX);
  double hs = 0.0, ei = 0.0, si = 0.0;
  if (ix >= 1 && ix <= NX - 2 && jy >= 1 && jy <= NY - 2) {
    const int64_t b = a + NX, r = a + 1, d = b + 1;
    const double *sxx = g.soxx, *syy = g.soyy, *sxy = g.soxy, *eN = g.etaN, *exx = g.exx, *eyy = g.eyy;
    // (v_a^2 / w_a + v_b^2 / w_b + v_r^2 / w_r + v_d^2 / w_d) / 8, left to right
    auto q4w = [&](const double *v, const double *w) {
      double t = D(M(v[a], v[a]), w[a]);
      t = A(t, D(M(v[b], v[b]), w[b]));
      t = A(t, D(M(v[r], v[r]), w[r]));
      t = A(t, D(M(v[d], v[d]), w[d]));
      return D(t, 8.0);
    };
    auto q4 = [&](const double *v) {
      double t = M(v[a], v[a]);
      t = A(t, M(v[b], v[b]));
      t = A(t, M(v[r], v[r]));
      t = A(t, M(v[d], v[d]));
      return D(t, 8.0);
    };
    hs = q4w(sxx, eN);
    hs = A(hs, q4w(syy, eN));
    hs = A(hs, D(M(sxy[a], sxy[a]), g.etaS[a]));
    hs = A(0.0, hs);  // the heating vector was zeroed, then accumulated into
    ei = __dsqrt_rn(A(A(q4(exx), q4(eyy)), M(g.exy[a], g.exy[a])));
    si = __dsqrt_rn(A(A(q4(sxx), q4(syy)), M(sxy[a], sxy[a])));
  }
  g.heat[a] = hs;
  g.eii[a] = ei;
  g.sii[a] = si;
}

// limitDisplacementTimestep candidates: min over nodes (order-preserving bits; NaN candidates
// never win, as the reference's `dt > dt1` test), and max |rhodot| over non-NaN entries
__global__ void k_limit_dt(Params P, GridFields g, double factor, unsigned long long *mins, unsigned long long *maxr,
                           int *nonnan) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (k >= (int64_t)NX * NY) return;
  const int ix = (int)(k % NX), jy = (int)(k / NX);
  long long best = LLONG_MAX;
  auto take = [&](double c) {
    if (!nan_bits(dbits(c))) best = min(best, ordered_bits(c));
  };
  double dx, dy;
  if (ix == 0) dx = P.x[1] - P.x[0];
  else if (ix == NX - 1) dx = P.x[NX - 1] - P.x[NX - 2];
  else {
    const double dx1 = P.x[ix + 1] - P.x[ix], dx2 = P.x[ix] - P.x[ix - 1];
    dx = (dx1 <= dx2) ? dx1 : dx2;
  }
  if (g.vx[k] != 0.0) take(M(D(dx, fabs(g.vx[k])), factor));
  if (jy == 0) dy = P.y[1] - P.y[0];
  else if (jy == NY - 1) dy = P.y[NY - 1] - P.y[NY - 2];
  else {
    const double dy1 = P.y[jy + 1] - P.y[jy], dy2 = P.y[jy] - P.y[jy - 1];
    dy = (dy1 <= dy2) ? dy1 : dy2;
  }
  if (g.vy[k] != 0.0) take(M(D(dy, fabs(g.vy[k])), factor));
  const double rd = g.rhodot[k];
  if (rd != 0.0) take(fabs(D(M(0.01, g.rho[k]), rd)));
  if (best != LLONG_MAX) atomicMin(reinterpret_cast<long long *>(mins), best);
  if (!nan_bits(dbits(rd))) {
    atomicMax(maxr, (unsigned long long)nonneg_bits(fabs(rd)));
    *nonnan = 1;
  }
}

__global__ void k_retrieve(const double *__restrict__ S, int64_t nn, double Kcont, double *p, double *vx,
                           double *vy) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nn) return;
  p[k] = M(S[3 * k + 2], Kcont);
  vx[k] = S[3 * k + 0];
  vy[k] = S[3 * k + 1];
}

// dx-weighted mean pressure of row 1 in the reference's order (retrieveSolutions.c:52-62)
__global__ void k_pressure_mean(Params P, const double *p, double *pm) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 1; i < P.NX; ++i) {
    const double dx = S(P.x[i], P.x[i - 1]);
    s = A(s, D(M(p[P.NX + i], dx), P.LX));
  }
  *pm = s;
}

__global__ void k_pressure_shift(Params P, double *p, const double *pm) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= (int64_t)P.NX * P.NY) return;
  if (k % P.NX >= 1 && k / P.NX >= 1) p[k] = S(p[k], *pm);
}

}  // namespace

extern "C" int mic_nodal_stress_strain(mic_ctx *ctx, double dt, double gy) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx) return MIC_ERR_ARG;
  (void)gy;  // the reference's gravity argument is not read in this routine
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  const GridFields g = grid_fields(ctx);
  {
    MIC_KERNEL(ctx, "k_nss_pointwise");
    k_nss_pointwise<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, g, ctx->bcs.mechBCLeft, ctx->bcs.mechBCTop,
                                                               dt);
  }
  {
    MIC_KERNEL(ctx, "k_nss_invariants");
    k_nss_invariants<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, g);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

extern "C" int mic_limit_displacement_timestep(mic_ctx *ctx, double factor, double *dt) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !dt) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  unsigned long long *d = reinterpret_cast<unsigned long long *>(ctx->red_buf + 24);  // min, max |rhodot|, flag
  const unsigned long long init[3] = {0x7FFFFFFFFFFFFFFFULL, 0ULL, 0ULL};
  MIC_CUDA_TRY(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
  {
    MIC_KERNEL(ctx, "k_limit_dt");
    k_limit_dt<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, grid_fields(ctx), factor, d, d + 1,
                                                          reinterpret_cast<int *>(d + 2));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  unsigned long long h[3];
  MIC_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  double t = *dt;
  if (h[0] != 0x7FFFFFFFFFFFFFFFULL) {  // smallest candidate, back from its ordered image
    long long b = (long long)h[0];
    if (b < 0) b = (long long)0x8000000000000000ULL - b;
    double c;
    memcpy(&c, &b, sizeof(c));
    if (t > c) t = c;
  }
  double mx;
  if (*reinterpret_cast<int *>(&h[2]))
    memcpy(&mx, &h[1], sizeof(mx));
  else
    mx = INFINITY;  // no non-NaN rhodot: VecMax / VecMin give -inf / inf
  if (mx * t > 0.01) t = 0.01 / mx;
  *dt = t;
  return MIC_OK;
}

extern "C" int mic_retrieve_solutions(mic_ctx *ctx, const double *S, double Kcont, int *foundnan) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || (!S && !ctx->solution)) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  if (!ctx->solution) {
    if (cudaMalloc((void **)&ctx->solution, sizeof(double) * 3 * nn) != cudaSuccess) return MIC_ERR_NOMEM;
  }
  // S = NULL: the solution mic_linear_solve left on the device
  if (S)
    MIC_CUDA_TRY(cudaMemcpyAsync(ctx->solution, S, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, ctx->stream));
  double *pm = ctx->red_buf + 28;
  {
    MIC_KERNEL(ctx, "k_retrieve");
    k_retrieve<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->solution, nn, Kcont, ctx->nodal[MIC_NF_P],
                                                          ctx->nodal[MIC_NF_VX], ctx->nodal[MIC_NF_VY]);
  }
  {
    MIC_KERNEL(ctx, "k_pressure_mean");
    k_pressure_mean<<<1, 32, 0, ctx->stream>>>(ctx->P, ctx->nodal[MIC_NF_P], pm);
  }
  {
    MIC_KERNEL(ctx, "k_pressure_shift");
    k_pressure_shift<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, ctx->nodal[MIC_NF_P], pm);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // the caller may reuse S on return
  if (foundnan) *foundnan = 0;  // the reference checks for NaN only in its TEXTURE build
  return MIC_OK;
}

// ---- diagnostics of main's time loop (post.c) -------------------------------------------------

namespace {

// nusseltNumber (post.c:5-46): the surface heat flux integral, summed in the reference's order by
// one thread (NX - 1 terms), every operation an IEEE intrinsic
__global__ void k_nusselt(Params P, const double *__restrict__ T, double dTbc, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int NX = P.NX;
  const double dz = S(P.y[1], P.y[0]);
  double integrand = 0.0;
  for (int ix = 0; ix < NX - 1; ++ix) {
    const double dT = D(S(A(S(T[NX + ix], T[ix]), T[NX + ix + 1]), T[ix + 1]), 2.0);
    const double dx = S(P.x[ix + 1], P.x[ix]);
    integrand = A(integrand, M(D(dT, dz), dx));
  }
  out[0] = M(D(D(P.LY, P.LX), dTbc), integrand);
}

// rmsVelocity (post.c:49-92): one term per cell, summed by a fixed tree (the reference sums the
// cells in order; the two agree to rounding)
__global__ void k_vrms_partial(Params P, const double *__restrict__ vx, const double *__restrict__ vy,
                               double *part) {
  __shared__ double sm[256];
  const int NX = P.NX, nc = (P.NX - 1) * (P.NY - 1);
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int ix = c % (NX - 1), jy = c / (NX - 1);
    const int64_t k = (int64_t)jy * NX + ix;
    const double dx = S(P.x[ix + 1], P.x[ix]), dy = S(P.y[jy + 1], P.y[jy]);
    const double vx2 = D(A(M(vx[k], vx[k]), M(vx[k + 1], vx[k + 1])), 2.0);
    const double vy2 = D(A(M(vy[k], vy[k]), M(vy[k + NX], vy[k + NX])), 2.0);
    acc = A(acc, M(M(A(vx2, vy2), dx), dy));
  }
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = A(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_vrms_final(Params P, const double *__restrict__ part, int nparts, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s = A(s, part[b]);
  out[0] = __dsqrt_rn(D(s, M(P.LX, P.LY)));
}

}  // namespace

extern "C" int mic_nusselt_number(mic_ctx *ctx, double bottom_T, double top_T, double *Nu) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !Nu) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  double *d = ctx->red_buf + 40;
  {
    MIC_KERNEL(ctx, "k_nusselt");
    k_nusselt<<<1, 32, 0, ctx->stream>>>(ctx->P, ctx->nodal[MIC_NF_THIST], bottom_T - top_T, d);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(Nu, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_rms_velocity(mic_ctx *ctx, double *vrms) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !vrms) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  constexpr int kParts = 64;
  double *part = ctx->red_buf + 64, *d = ctx->red_buf + 41;
  {
    MIC_KERNEL(ctx, "k_vrms_partial");
    k_vrms_partial<<<kParts, 256, 0, ctx->stream>>>(ctx->P, ctx->nodal[MIC_NF_VX], ctx->nodal[MIC_NF_VY], part);
  }
  {
    MIC_KERNEL(ctx, "k_vrms_final");
    k_vrms_final<<<1, 32, 0, ctx->stream>>>(ctx->P, part, kParts, d);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(vrms, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}
