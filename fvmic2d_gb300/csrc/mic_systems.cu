// mic_systems.cu -- the two linear systems of a time step, assembled on the device from the
// context's nodal arrays: the visco-elasto-plastic Stokes system (formVEPSystem,
// vep_system.c:12-726) and the implicit heat-diffusion system (formThermalSystem,
// formThermalSystem.c:6-249), with the thermal boundary values of the previous temperature
// (enforceThermalBCs1, enforceThermalBC.c:5-38).
//
// Rows follow the reference's global ordering: 3 (j NX + i) + dof for Stokes (dof 0 vx, 1 vy,
// 2 p) and j NX + i for temperature.  Each row is written by one thread as a short list of
// (column, value) entries (at most 12) in the order the reference inserts them; inserting a
// column twice replaces the value (INSERT_VALUES).  Columns of ghost points (local-to-global
// index -1) are dropped as PETSc drops negative indices.  Every operation is an IEEE intrinsic
// in the reference's order, so both builds give the reference's bits.
//
// The slab / plate geometry (benchmarkInitialConditions.c:75-145) enters through host tables
// evaluated with the C library, as the reference evaluates it: slab depth x tan(angle) and plate
// depth at every basic and centre x, the imposed slab velocity, and the boundary temperatures.
// The device only compares against them, so the decisions match the reference's bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mic_internal.cuh"
#include "mic_rheology.cuh"

using namespace mic;

namespace {

constexpr int kMaxEnt = 12;  // entries of the longest row (the 27-slot momentum stencils keep 11)

__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D(double a, double b) { return __ddiv_rn(a, b); }

struct Geo {  // device copies of the host tables
  const double *sd_x, *sd_xc;  // slab depth x tan(angle) at x[0..NX-1], xc[0..NX]
  const double *pd_x, *pd_xc;  // plate depth at x[0..NX-1], xc[0..NX]
  const double *t_left, *t_right;    // formThermalSystem boundary temperatures per row j
  const double *t_enf_left, *t_enf_right;  // enforceThermalBCs1 boundary temperatures per row j
  double pd_LX;                // plate_depth(LX)
  double svx, svy;             // slabVelocity cos(angle), slabVelocity sin(angle)
};

struct Rows {  // ELL rows
  int *cnt;
  int *col;
  double *val;
  double *rhs;
};

// one row under construction in registers
struct Row {
  int n;
  int c[kMaxEnt];
  double v[kMaxEnt];
  __device__ void set(int col, double val) {  // MatSetValue(..., INSERT_VALUES)
    if (col < 0) return;
    for (int k = 0; k < n; ++k)
      if (c[k] == col) {
        v[k] = val;
        return;
      }
    if (n < kMaxEnt) {
      c[n] = col;
      v[n] = val;
      ++n;
    }
  }
  __device__ void store(const Rows &R, int64_t row) const {
    R.cnt[row] = n;
    for (int k = 0; k < n; ++k) {
      R.col[row * kMaxEnt + k] = c[k];
      R.val[row * kMaxEnt + k] = v[k];
    }
  }
};

// in_slab / in_plate / in_either (benchmarkInitialConditions.c:100-145) against the tables
__device__ __forceinline__ bool in_slab(double y, double sd) { return y >= sd; }
__device__ __forceinline__ bool in_plate(double y, double sd, double pd) { return !(y >= sd) && y <= pd; }
__device__ __forceinline__ bool in_either(double y, double sd, double pd) {
  return in_slab(y, sd) || in_plate(y, sd, pd);
}

// a nodal field read through the reference's ghosted local vector: 0 on the ghost points
__device__ __forceinline__ double loc(const double *f, int NX, int NY, int j, int i) {
  return (i >= 0 && i < NX && j >= 0 && j < NY) ? f[(int64_t)j * NX + i] : 0.0;
}

__device__ __forceinline__ int sdof(int NX, int NY, int j, int i, int d) {
  return (i >= 0 && i < NX && j >= 0 && j < NY) ? 3 * (j * NX + i) + d : -1;
}

constexpr int kU = 0, kV = 1, kP = 2;  // DOF_U, DOF_V, DOF_P (fdcode.h:242-245)

// vep_system.c:60-96: viscosities with the visco-elastic factor, X = eta/(eta + dt mu) (0 for a
// zero divisor), etaZ = (1 - X) eta, as the reference's vector operations compute it
__global__ void k_vep_z(const double *__restrict__ etaN, const double *__restrict__ muN,
                        const double *__restrict__ etaS, const double *__restrict__ muS, int64_t nn, double dt,
                        double *etaNZ, double *etaSZ) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nn) return;
  double den = A(etaN[k], M(dt, muN[k]));
  double X = den != 0.0 ? D(etaN[k], den) : 0.0;
  etaNZ[k] = M(A(M(-1.0, X), 1.0), etaN[k]);
  den = A(etaS[k], M(dt, muS[k]));
  X = den != 0.0 ? D(etaS[k], den) : 0.0;
  etaSZ[k] = M(A(M(-1.0, X), 1.0), etaS[k]);
}

// VecMin (NaN entries skipped) of etaSZ, one block per slice, then one block over the slices
__global__ void k_min_partial(const double *__restrict__ v, int64_t nn, double *part) {
  __shared__ double sm[256];
  double m = INFINITY;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x)
    if (v[k] < m) m = v[k];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && sm[threadIdx.x + s] < sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// Kbond = 4 etamin / (dx + dy)^2, Kcont = 2 etamin / (dx + dy) (vep_system.c:112-119)
__global__ void k_vep_consts(Params P, const double *__restrict__ part, int nparts, double *K) {
  __shared__ double sm[256];
  double m = INFINITY;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x)
    if (part[k] < m) m = part[k];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && sm[threadIdx.x + s] < sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double etamin = sm[0];
    const double dx = S(P.x[1], P.x[0]), dy = S(P.y[1], P.y[0]);
    const double h = A(dx, dy);
    K[0] = D(M(4.0, etamin), M(h, h));
    K[1] = D(M(2.0, etamin), h);
  }
}

// the three rows of node (ix, jy): continuity (vep_system.c:243-284), x-momentum (288-395) and
// y-momentum (398-512); the ADD_VALUES pass after them (517-571) is disabled in the reference
__global__ void k_vep_rows(Params P, Geo G, const double *__restrict__ etaNZ, const double *__restrict__ etaSZ,
                           const double *__restrict__ rho, const double *__restrict__ Kd, double gx, double gy,
                           Rows R) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (k >= (int64_t)NX * NY) return;
  const int ix = (int)(k % NX), jy = (int)(k / NX);
  const double Kbond = Kd[0], Kcont = Kd[1];
  const double *x = P.x, *y = P.y, *xc = P.xc, *yc = P.yc;
  Row r;

  // ---- continuity ----
  {
    r.n = 0;
    const int row = sdof(NX, NY, jy, ix, kP);
    double rhs = 0.0;
    if (ix > 0 && jy > 0 && in_either(y[jy - 1], G.sd_xc[ix], G.pd_xc[ix]) &&
        in_either(y[jy], G.sd_xc[ix], G.pd_xc[ix]) && in_either(yc[jy], G.sd_x[ix], G.pd_x[ix]) &&
        in_either(yc[jy], G.sd_x[ix - 1], G.pd_x[ix - 1])) {
      r.set(row, M(1.0, Kbond));
    } else if (jy == 0) {  // ghost pressures follow the first row: a constant null space
      r.set(row, M(1.0, Kbond));
      r.set(sdof(NX, NY, jy + 1, ix, kP), M(-1.0, Kbond));
    } else if (ix == 0) {
      r.set(row, M(1.0, Kbond));
      r.set(sdof(NX, NY, jy, ix + 1, kP), M(-1.0, Kbond));
    } else if (ix == NX - 1 && jy > 0 && yc[jy] > G.pd_LX && yc[jy - 1] <= G.pd_LX) {  // FIX_PRESSURE
      r.set(row, M(1.0, Kbond));
    } else {
      const double dx = S(x[ix], x[ix - 1]);
      const double dy = S(y[jy], y[jy - 1]);
      r.set(sdof(NX, NY, jy - 1, ix, kU), D(Kcont, dx));
      r.set(sdof(NX, NY, jy - 1, ix - 1, kU), D(-Kcont, dx));
      r.set(sdof(NX, NY, jy, ix - 1, kV), D(Kcont, dy));
      r.set(sdof(NX, NY, jy - 1, ix - 1, kV), D(-Kcont, dy));
    }
    r.store(R, row);
    R.rhs[row] = rhs;
  }

  // ---- x-momentum ----
  {
    r.n = 0;
    const int row = sdof(NX, NY, jy, ix, kU);
    double rhs = 0.0;
    if (in_slab(yc[jy + 1], G.sd_x[ix])) {
      r.set(row, M(1.0, Kbond));
      rhs = M(Kbond, G.svx);
    } else if (in_plate(yc[jy + 1], G.sd_x[ix], G.pd_x[ix])) {
      r.set(row, M(1.0, Kbond));
    } else if (ix == NX - 1 && jy < NY - 1) {
      const double eta = loc(etaNZ, NX, NY, jy + 1, ix);
      const double dx = S(x[ix], x[ix - 1]);
      r.set(row, D(M(2.0, eta), dx));
      r.set(sdof(NX, NY, jy, ix - 1, kU), D(M(-2.0, eta), dx));
      r.set(sdof(NX, NY, jy + 1, ix, kP), -Kcont);
    } else if (jy == NY - 1 && ix < NX - 1) {  // bottom boundary
      const double dxc = S(xc[ix + 1], xc[ix]);
      const double dyc = S(yc[jy], yc[jy - 1]);
      r.set(row, M(D(1.0, dyc), Kcont));
      r.set(sdof(NX, NY, jy - 1, ix, kU), M(D(-1.0, dyc), Kcont));
      r.set(sdof(NX, NY, jy, ix, kV), M(D(1.0, dxc), Kcont));
      r.set(sdof(NX, NY, jy, ix - 1, kV), M(D(-1.0, dxc), Kcont));
    } else if (jy == NY - 1 && ix == NX - 1) {
      const double dyc = S(yc[NY], yc[NY - 1]);
      r.set(row, M(D(1.0, dyc), Kcont));
      r.set(sdof(NX, NY, jy - 1, ix, kU), M(D(-1.0, dyc), Kcont));
    } else {  // x-Stokes stencil
      const double v0000 = xc[ix], v0001 = Kcont, v0002 = x[ix], v0003 = y[jy];
      const double v0006 = loc(etaSZ, NX, NY, jy, ix);
      const double v0007 = xc[ix + 1], v0008 = y[jy + 1], v0009 = yc[jy + 1];
      const double v0010 = loc(etaSZ, NX, NY, jy + 1, ix);
      const double v0011 = loc(etaNZ, NX, NY, jy + 1, ix);
      const double v0012 = ix == NX - 1 ? v0011 : loc(etaNZ, NX, NY, jy + 1, ix + 1);
      const double v0013 = D(1.0, S(v0000, v0007));
      const double v0014 = ix == NX - 1 ? D(1.0, S(x[NX - 2], x[NX - 1])) : D(1.0, S(v0002, x[ix + 1]));
      const double v0015 = D(1.0, S(v0003, v0008));
      const double v0016 = D(1.0, A(-v0009, yc[jy]));
      const double v0017 = D(1.0, A(-v0002, x[ix - 1]));
      const double v0018 = D(1.0, S(v0009, yc[jy + 2]));
      r.set(sdof(NX, NY, jy, ix - 1, kU), D(M(M(M(4.0, v0011), v0013), v0017), 3.0));
      r.set(sdof(NX, NY, jy, ix - 1, kV), D(M(M(S(M(3.0, v0006), M(2.0, v0011)), v0013), v0015), 3.0));
      r.set(sdof(NX, NY, jy + 1, ix - 1, kV), D(M(M(A(M(-3.0, v0010), M(2.0, v0011)), v0013), v0015), 3.0));
      r.set(sdof(NX, NY, jy - 1, ix, kU), M(M(v0006, v0015), v0016));
      r.set(sdof(NX, NY, jy, ix, kU),
            A(S(D(M(M(M(-4.0, v0012), v0013), v0014), 3.0), D(M(M(M(4.0, v0011), v0013), v0017), 3.0)),
              D(A(M(v0006, v0016), M(v0010, v0018)), A(-v0003, v0008))));
      r.set(sdof(NX, NY, jy, ix, kV), D(M(M(A(M(-3.0, v0006), M(2.0, v0012)), v0013), v0015), 3.0));
      r.set(sdof(NX, NY, jy + 1, ix, kU), M(M(v0010, v0015), v0018));
      r.set(sdof(NX, NY, jy + 1, ix, kV), D(M(M(S(M(3.0, v0010), M(2.0, v0012)), v0013), v0015), 3.0));
      r.set(sdof(NX, NY, jy + 1, ix, kP), D(v0001, A(-v0000, v0007)));
      r.set(sdof(NX, NY, jy, ix + 1, kU), D(M(M(M(4.0, v0012), v0013), v0014), 3.0));
      r.set(sdof(NX, NY, jy + 1, ix + 1, kP), M(v0001, v0013));
      rhs = D(M(-gx, A(loc(rho, NX, NY, jy, ix), loc(rho, NX, NY, jy + 1, ix))), 2.0);
    }
    r.store(R, row);
    R.rhs[row] = rhs;
  }

  // ---- y-momentum ----
  {
    r.n = 0;
    const int row = sdof(NX, NY, jy, ix, kV);
    double rhs = 0.0;
    const bool plate_here = in_plate(y[jy], G.sd_x[ix], G.pd_x[ix]);
    if (in_slab(y[jy], G.sd_xc[ix + 1])) {
      r.set(row, Kbond);
      rhs = M(Kbond, G.svy);
    } else if (in_plate(y[jy], G.sd_xc[ix + 1], G.pd_xc[ix + 1])) {
      r.set(row, Kbond);
    } else if (jy == NY - 1 && ix < NX - 1) {
      // the reference reads etaNZ[jy][ixl+1] with the ghosted local index ixl = ix + 2
      const double eta = loc(etaNZ, NX, NY, jy, ix + 3);
      const double dy = S(y[jy], y[jy - 1]);
      r.set(row, D(M(2.0, eta), dy));
      r.set(sdof(NX, NY, jy - 1, ix, kV), D(M(-2.0, eta), dy));
      r.set(sdof(NX, NY, jy, ix + 1, kP), -Kcont);
    } else if (ix == NX - 1 && !plate_here) {  // zero shear stress on the right boundary
      const double dxc = S(xc[ix + 1], xc[ix]);
      const double dyc = S(yc[jy + 1], yc[jy]);
      r.set(sdof(NX, NY, jy, ix, kU), M(D(1.0, dyc), Kcont));
      r.set(sdof(NX, NY, jy - 1, ix, kU), M(D(-1.0, dyc), Kcont));
      r.set(row, M(D(1.0, dxc), Kcont));
      r.set(sdof(NX, NY, jy, ix - 1, kV), M(D(-1.0, dxc), Kcont));
    } else if (ix == NX - 1 && jy == NY - 1) {
      const double dxc = S(xc[NX], xc[NX - 1]);
      r.set(row, M(D(1.0, dxc), Kcont));
      r.set(sdof(NX, NY, jy, ix - 1, kV), M(D(-1.0, dxc), Kcont));
    } else {  // y-Stokes stencil
      const double v0000 = yc[jy], v0001 = Kcont, v0002 = y[jy];
      const double v0005 = loc(etaSZ, NX, NY, jy, ix);
      const double v0006 = yc[jy + 1], v0007 = xc[ix + 1];
      const double v0008 = loc(etaSZ, NX, NY, jy, ix + 1);
      const double v0009 = loc(etaNZ, NX, NY, jy, ix + 1);
      const double v0010 = jy == NY - 1 ? v0009 : loc(etaNZ, NX, NY, jy + 1, ix + 1);
      const double v0011 = D(1.0, S(v0000, v0006));
      const double v0012 = D(1.0, A(-v0000, v0006));
      const double v0013 = D(1.0, S(x[ix], x[ix + 1]));
      const double v0014 = jy == NY - 1 ? v0013 : D(1.0, S(v0002, y[jy + 1]));
      const double v0015 = D(1.0, A(-v0002, y[jy - 1]));
      const double v0016 = D(1.0, A(-v0007, xc[ix]));
      const double v0017 = D(1.0, S(v0007, xc[ix + 2]));
      r.set(sdof(NX, NY, jy, ix - 1, kV), M(M(v0005, v0013), v0016));
      r.set(sdof(NX, NY, jy - 1, ix, kU), D(M(M(S(M(3.0, v0005), M(2.0, v0009)), v0011), v0013), 3.0));
      r.set(sdof(NX, NY, jy - 1, ix, kV), D(M(M(M(4.0, v0009), v0011), v0015), 3.0));
      r.set(sdof(NX, NY, jy, ix, kU), D(M(M(A(M(-3.0, v0005), M(2.0, v0010)), v0011), v0013), 3.0));
      r.set(sdof(NX, NY, jy, ix, kV),
            S(S(D(M(M(4.0, v0012), A(M(v0010, v0014), M(v0009, v0015))), 3.0), M(M(v0005, v0013), v0016)),
              M(M(v0008, v0013), v0017)));
      r.set(sdof(NX, NY, jy + 1, ix, kV), D(M(M(M(4.0, v0010), v0011), v0014), 3.0));
      r.set(sdof(NX, NY, jy - 1, ix + 1, kU), D(M(M(A(M(-3.0, v0008), M(2.0, v0009)), v0011), v0013), 3.0));
      r.set(sdof(NX, NY, jy, ix + 1, kU), D(M(M(S(M(3.0, v0008), M(2.0, v0010)), v0011), v0013), 3.0));
      r.set(sdof(NX, NY, jy, ix + 1, kV), M(M(v0008, v0013), v0017));
      r.set(sdof(NX, NY, jy, ix + 1, kP), M(v0001, v0012));
      r.set(sdof(NX, NY, jy + 1, ix + 1, kP), M(v0001, v0011));
      rhs = D(M(-gy, A(loc(rho, NX, NY, jy, ix), loc(rho, NX, NY, jy, ix + 1))), 2.0);
    }
    r.store(R, row);
    R.rhs[row] = rhs;
  }
}

struct ThermalFields {
  const double *k, *rho, *Cp, *lastT, *vx, *heat;
};

// formThermalSystem.c:90-170 (rows, and the transient term added to the heating on the right-hand
// side) and 175-232 (boundary values inserted into the right-hand side)
__global__ void k_thermal_rows(Params P, Geo G, ThermalFields F, double rho0, double dt, int doSteady, int topType,
                               double topValue, Rows R) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (k >= (int64_t)NX * NY) return;
  const int ix = (int)(k % NX), jy = (int)(k / NX);
  const double *gx = P.x, *gy = P.y;
  Row r;
  r.n = 0;
  double rhs = F.heat[k];
  const bool right_fixed =
      ix == NX - 1 && (gy[jy] <= G.pd_LX || (jy > 0 && D(A(F.vx[k], F.vx[k - NX]), 2.0) < 0.0));
  if (ix == 0) {
    r.set((int)k, 1.0);
    rhs = G.t_left[jy];
  } else if (right_fixed) {
    r.set((int)k, 1.0);
    rhs = G.t_right[jy];
  } else if (ix == NX - 1) {
    r.set((int)k, 1.0);
    rhs = F.lastT[k];
  } else if (jy == 0) {
    if (topType == 0) {
      r.set((int)k, 1.0);
      rhs = topValue;
    } else if (topType == 1) {
      const double dyt1 = S(gy[jy + 1], gy[jy]);
      r.set((int)k, D(-1.0, dyt1));
      r.set((int)(k + NX), D(1.0, dyt1));
      rhs = 0.0;
    }
  } else if (jy == NY - 1) {
    r.set((int)k, 1.0);
    rhs = F.lastT[k];
  } else {
    const double kk = F.k[k];
    const double ka = D(A(kk, F.k[k - 1]), 2.0);
    const double kb = D(A(kk, F.k[k + 1]), 2.0);
    const double kc = D(A(kk, F.k[k - NX]), 2.0);
    const double kd = D(A(kk, F.k[k + NX]), 2.0);
    const double dx2 = S(gx[ix + 1], gx[ix]);
    const double dx1 = S(gx[ix], gx[ix - 1]);
    const double dy1 = S(gy[jy], gy[jy - 1]);
    const double dy2 = S(gy[jy + 1], gy[jy]);
    const double lap = A(M(D(2.0, A(dx2, dx1)), A(D(kb, dx2), D(ka, dx1))),
                         M(D(2.0, A(dy1, dy2)), A(D(kd, dy2), D(kc, dy1))));
    if (!doSteady) {
      const double c = D(M(A(rho0, F.rho[k]), F.Cp[k]), dt);
      rhs = A(rhs, M(c, F.lastT[k]));
      r.set((int)k, A(A(c, M(D(2.0, A(dx2, dx1)), A(D(kb, dx2), D(ka, dx1)))),
                      M(D(2.0, A(dy1, dy2)), A(D(kd, dy2), D(kc, dy1)))));
    } else {
      r.set((int)k, lap);
    }
    r.set((int)(k + 1), D(M(D(-2.0, A(dx1, dx2)), kb), dx2));
    r.set((int)(k - 1), D(M(D(-2.0, A(dx1, dx2)), ka), dx1));
    r.set((int)(k - NX), D(M(D(-2.0, A(dy1, dy2)), kc), dy1));
    r.set((int)(k + NX), D(M(D(-2.0, A(dy1, dy2)), kd), dy2));
  }
  r.store(R, k);
  R.rhs[k] = rhs;
}

// enforceThermalBCs1 (enforceThermalBC.c:15-33): top value, then the left wall's slab inflow
// temperature and the right wall's plate geotherm above the plate depth
__global__ void k_enforce_thermal_bcs(Params P, Geo G, double topValue, double *lastT) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int NX = P.NX, NY = P.NY;
  if (k >= (int64_t)NX * NY) return;
  const int ix = (int)(k % NX), jy = (int)(k / NX);
  if (jy == 0) lastT[k] = topValue;
  if (ix == 0)
    lastT[k] = G.t_enf_left[jy];
  else if (ix == NX - 1 && P.y[jy] <= G.pd_LX)
    lastT[k] = G.t_enf_right[jy];
}

// ---- host: the geometry of benchmarkInitialConditions.c, with the C library ----------------
// (this translation unit's host code is compiled without floating-point contraction)

double h_mantle_temperature() { return 1573.0; }

double h_plate_depth(double x, const mic_subduction_options &o) {
  const double plate_thickness = o.overridingPlateThickness;
  const double root_thickness = o.rootThickness;
  const double root_center_location = o.rootCenter;
  const double root_width = o.rootWidth;
  if (std::fabs(x - root_center_location) < root_width)
    return plate_thickness +
           root_thickness * std::pow(std::cos(M_PI * (x - root_center_location) / root_width / 2.0), 2.0);
  return plate_thickness;
}

double h_plate_geotherm(double x, double y, const mic_subduction_options &o) {
  return y / h_plate_depth(x, o) * (h_mantle_temperature() - 273.0) + 273.0;
}

double h_slab_depth(double x, double angle) { return x * std::tan(angle); }

double h_slab_inflow_temperature(double x, double y, double angle, double age) {
  const double Ts = 273, T0 = 1623, kappa = 0.7272e-6, s_in_year = 3.15576e7;
  const double slab_age_s = age * 1.0e6 * s_in_year;
  return Ts + (T0 - Ts) * std::erf((y - h_slab_depth(x, angle)) / (2.0 * std::sqrt(kappa * slab_age_s)));
}

struct Scratch {
  double *tables;  // sd_x, sd_xc, pd_x, pd_xc, t_left, t_right, t_enf_left, t_enf_right
  double *etaNZ, *etaSZ, *part, *K;
};

int ensure(void **buf, size_t *have, size_t need) {
  if (*have >= need) return MIC_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  if (cudaMalloc(buf, need) != cudaSuccess) return MIC_ERR_NOMEM;
  *have = need;
  return MIC_OK;
}

constexpr int kMinParts = 256;

int prepare(mic_ctx *ctx, const mic_subduction_options &o, Scratch &s, Geo &G) {
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const int64_t nn = (int64_t)NX * NY;
  const size_t nt = (size_t)4 * (NX + 1) + 4 * (size_t)NY;
  const size_t need = sizeof(double) * (nt + 2 * nn + kMinParts + 2) + 4 * 256;
  int e = ensure(&ctx->sys_scratch, &ctx->sys_scratch_bytes, need);
  if (e) return e;
  double *p = static_cast<double *>(ctx->sys_scratch);
  s.tables = p;
  s.etaNZ = p + nt;
  s.etaSZ = s.etaNZ + nn;
  s.part = s.etaSZ + nn;
  s.K = s.part + kMinParts;
  std::vector<double> h(nt);
  const double *x = ctx->h_x + 2, *xc = ctx->h_xc, *y = ctx->h_y;  // h_x is the buffer start (x[-2])
  const double tanA = std::tan(o.slabAngle);
  double *sd_x = h.data(), *sd_xc = sd_x + (NX + 1), *pd_x = sd_xc + (NX + 1), *pd_xc = pd_x + (NX + 1);
  double *tl = pd_xc + (NX + 1), *tr = tl + NY, *tel = tr + NY, *ter = tel + NY;
  for (int i = 0; i <= NX; ++i) {
    sd_x[i] = i < NX ? x[i] * tanA : 0.0;
    pd_x[i] = i < NX ? h_plate_depth(x[i], o) : 0.0;
    sd_xc[i] = xc[i] * tanA;
    pd_xc[i] = h_plate_depth(xc[i], o);
  }
  const double LX = ctx->P.LX;
  for (int j = 0; j < NY; ++j) {
    tl[j] = h_slab_inflow_temperature(x[0], y[j], o.slabAngle, o.slabAge);
    tr[j] = y[j] <= h_plate_depth(x[NX - 1], o) ? h_plate_geotherm(x[NX - 1], y[j], o) : 1573.0;
    tel[j] = h_slab_inflow_temperature(0.0, y[j], o.slabAngle, o.slabAge);
    ter[j] = h_plate_geotherm(LX, y[j], o);
  }
  MIC_CUDA_TRY(cudaMemcpyAsync(s.tables, h.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->stream));
  G.sd_x = s.tables;
  G.sd_xc = G.sd_x + (NX + 1);
  G.pd_x = G.sd_xc + (NX + 1);
  G.pd_xc = G.pd_x + (NX + 1);
  G.t_left = G.pd_xc + (NX + 1);
  G.t_right = G.t_left + NY;
  G.t_enf_left = G.t_right + NY;
  G.t_enf_right = G.t_enf_left + NY;
  G.pd_LX = h_plate_depth(LX, o);
  G.svx = o.slabVelocity * std::cos(o.slabAngle);
  G.svy = o.slabVelocity * std::sin(o.slabAngle);
  // the host vector must outlive the copy
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

int ensure_system(mic_ctx *ctx, int which, int64_t n) {
  mic_system_store &S = ctx->sys[which];
  if (S.n == n && S.cnt) return MIC_OK;
  cudaFree(S.cnt);
  cudaFree(S.col);
  cudaFree(S.val);
  cudaFree(S.rhs);
  if (S.lu_exec) cudaGraphExecDestroy(S.lu_exec);
  S = mic_system_store{};
  if (cudaMalloc(&S.cnt, sizeof(int) * n) != cudaSuccess || cudaMalloc(&S.col, sizeof(int) * n * kMaxEnt) != cudaSuccess ||
      cudaMalloc(&S.val, sizeof(double) * n * kMaxEnt) != cudaSuccess ||
      cudaMalloc(&S.rhs, sizeof(double) * n) != cudaSuccess)
    return MIC_ERR_NOMEM;
  S.n = n;
  S.width = kMaxEnt;
  return MIC_OK;
}

Rows rows_of(const mic_system_store &S) { return Rows{S.cnt, S.col, S.val, S.rhs}; }

// initialConditionsVanKeken (benchmarkInitialConditions.c:8-33) for one marker: temperature by
// region (slab: the half-space cooling profile; overriding plate: the linear geotherm; wedge:
// mantle temperature), material 0, density anomaly, viscosity and shear modulus
__global__ void k_van_keken(mic_materials M, mic_options O, CreepConfig cfg, double tanA, double slabAge,
                            double plate, double rootT, double rootC, double rootW, double *X, double *Y, double *T,
                            double *rho, double *rhodot, double *eta, double *mu, int *mat, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const double x = X[m], y = Y[m];
  const double sd = x * tanA;  // slab_depth
  double pd = plate;           // plate_depth
  if (fabs(x - rootC) < rootW) {
    const double c = cos(M_PI * (x - rootC) / rootW / 2.0);
    pd = plate + rootT * (c * c);
  }
  double t;
  if (y >= sd) {
    const double slab_age_s = slabAge * 1.0e6 * 3.15576e7;
    t = 273.0 + (1623.0 - 273.0) * erf((y - sd) / (2.0 * sqrt(0.7272e-6 * slab_age_s)));
  } else if (y <= pd) {
    t = y / pd * (1573.0 - 273.0) + 273.0;
  } else {
    t = 1573.0;
  }
  T[m] = t;
  mat[m] = 0;
  rhodot[m] = 0.0;
  rho[m] = -M.materialRho[0] * (M.materialAlpha[0] * t);
  double e, u;
  CreepIn ci = {0.0, 0.0, 0.0, kGrainArgDefault, 0.0, 0.0f, 0, 0, 0.0, 0, {}, 0.0};
  CreepConfig exact = cfg;
  exact.mode = 0;
  if (rheology(M, O, 0, t, x, y, e, u, &exact, &ci)) {  // updateMarkerViscosity(m, ..., 0.0)
    eta[m] = e;
    mu[m] = u;
  }
}

}  // namespace

extern "C" int mic_reset_nodal_fields(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const size_t bytes = sizeof(double) * ctx->P.NX * ctx->P.NY;
  for (int f = 0; f < MIC_NF_COUNT; ++f) MIC_CUDA_TRY(cudaMemsetAsync(ctx->nodal[f], 0, bytes, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_initial_conditions_van_keken(mic_ctx *ctx, const mic_subduction_options *o) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !o) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->n > 0) {
    MIC_KERNEL(ctx, "k_van_keken");
    k_van_keken<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(
        ctx->mat, ctx->opt, ctx->creep, std::tan(o->slabAngle), o->slabAge, o->overridingPlateThickness,
        o->rootThickness, o->rootCenter, o->rootWidth, ctx->f64[C_X], ctx->f64[C_Y], ctx->f64[C_T], ctx->f64[C_RHO],
        ctx->f64[C_RHODOT], ctx->f64[C_ETA], ctx->f64[C_MU], ctx->i32[C_MAT], ctx->n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  // boundary conditions for the prescribed slab velocity (benchmarkInitialConditions.c:36-46)
  mic_bcs b = ctx->bcs;
  b.mechBCLeft.type[0] = 0;
  b.mechBCLeft.type[1] = 0;
  b.mechBCLeft.value[0] = o->slabVelocity * std::cos(o->slabAngle);
  b.mechBCLeft.value[1] = o->slabVelocity * std::sin(o->slabAngle);
  b.mechBCTop.type[0] = 0;
  b.mechBCTop.value[0] = 0.0;
  b.mechBCTop.type[1] = 0;
  b.mechBCTop.value[1] = 0.0;
  int e = mic_set_bcs(ctx, &b);
  if (e) return e;
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_form_vep_system(mic_ctx *ctx, const mic_subduction_options *o, double dt, double *Kbond,
                                   double *Kcont) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !o) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const int64_t nn = (int64_t)NX * NY;
  Scratch s;
  Geo G;
  int e = prepare(ctx, *o, s, G);
  if (e) return e;
  if ((e = ensure_system(ctx, 0, 3 * nn))) return e;
  double **f = ctx->nodal;
  {
    MIC_KERNEL(ctx, "k_vep_z");
    k_vep_z<<<grid_for(nn), kBlock, 0, ctx->stream>>>(f[MIC_NF_ETAN], f[MIC_NF_MUN], f[MIC_NF_ETAS], f[MIC_NF_MUS],
                                                      nn, dt, s.etaNZ, s.etaSZ);
  }
  const int parts = (int)std::min<int64_t>(kMinParts, (nn + kBlock - 1) / kBlock);
  {
    MIC_KERNEL(ctx, "k_min_partial");
    k_min_partial<<<parts, 256, 0, ctx->stream>>>(s.etaSZ, nn, s.part);
  }
  {
    MIC_KERNEL(ctx, "k_vep_consts");
    k_vep_consts<<<1, 256, 0, ctx->stream>>>(ctx->P, s.part, parts, s.K);
  }
  {
    MIC_KERNEL(ctx, "k_vep_rows");
    k_vep_rows<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, G, s.etaNZ, s.etaSZ, f[MIC_NF_RHO], s.K, o->gx,
                                                         o->gy, rows_of(ctx->sys[0]));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  double K[2];
  MIC_CUDA_TRY(cudaMemcpyAsync(K, s.K, sizeof(K), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->sys[0].Kbond = K[0];
  ctx->sys[0].Kcont = K[1];
  ctx->sys[0].factored = 0;
  if (Kbond) *Kbond = K[0];
  if (Kcont) *Kcont = K[1];
  return MIC_OK;
}

extern "C" int mic_enforce_thermal_bcs(mic_ctx *ctx, const mic_subduction_options *o) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !o) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  Scratch s;
  Geo G;
  int e = prepare(ctx, *o, s, G);
  if (e) return e;
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  MIC_KERNEL(ctx, "k_enforce_thermal_bcs");
  k_enforce_thermal_bcs<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, G, o->thermalBCTopValue,
                                                                   ctx->nodal[MIC_NF_LASTT]);
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

extern "C" int mic_form_thermal_system(mic_ctx *ctx, const mic_subduction_options *o, double dt, int doSteady) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !o) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  Scratch s;
  Geo G;
  int e = prepare(ctx, *o, s, G);
  if (e) return e;
  if ((e = ensure_system(ctx, 1, nn))) return e;
  double **f = ctx->nodal;
  ThermalFields F{f[MIC_NF_KTHERMAL], f[MIC_NF_RHO], f[MIC_NF_CP], f[MIC_NF_LASTT], f[MIC_NF_VX], f[MIC_NF_HEATING]};
  {
    MIC_KERNEL(ctx, "k_thermal_rows");
    k_thermal_rows<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->P, G, F, ctx->mat.materialRho[0], dt, doSteady,
                                                             o->thermalBCTopType, o->thermalBCTopValue,
                                                             rows_of(ctx->sys[1]));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  ctx->sys[1].factored = 0;
  return MIC_OK;
}

extern "C" int mic_system_size(mic_ctx *ctx, int which, int64_t *nrows, int64_t *nnz) {
  if (!ctx || which < 0 || which > 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const mic_system_store &S = ctx->sys[which];
  if (!S.cnt) return MIC_ERR_ARG;
  std::vector<int> cnt(S.n);
  MIC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), S.cnt, sizeof(int) * S.n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int64_t t = 0;
  for (int c : cnt) t += c;
  if (nrows) *nrows = S.n;
  if (nnz) *nnz = t;
  return MIC_OK;
}

extern "C" int mic_system_get(mic_ctx *ctx, int which, int32_t *rowptr, int32_t *cols, double *vals, double *rhs) {
  if (!ctx || which < 0 || which > 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const mic_system_store &S = ctx->sys[which];
  if (!S.cnt) return MIC_ERR_ARG;
  const int64_t n = S.n;
  std::vector<int> cnt(n), col(n * kMaxEnt);
  std::vector<double> val(n * kMaxEnt);
  MIC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), S.cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(col.data(), S.col, sizeof(int) * n * kMaxEnt, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(val.data(), S.val, sizeof(double) * n * kMaxEnt, cudaMemcpyDeviceToHost, ctx->stream));
  if (rhs) MIC_CUDA_TRY(cudaMemcpyAsync(rhs, S.rhs, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int64_t at = 0;
  for (int64_t r = 0; r < n; ++r) {
    if (rowptr) rowptr[r] = (int32_t)at;
    std::vector<std::pair<int, double>> e;
    for (int k = 0; k < cnt[r]; ++k) e.emplace_back(col[r * kMaxEnt + k], val[r * kMaxEnt + k]);
    std::sort(e.begin(), e.end(), [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
      return a.first < b.first;
    });
    for (auto &pr : e) {
      if (cols) cols[at] = pr.first;
      if (vals) vals[at] = pr.second;
      ++at;
    }
  }
  if (rowptr) rowptr[n] = (int32_t)at;
  return MIC_OK;
}
