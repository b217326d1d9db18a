// mic_project.cu -- K2: marker -> node projection (projectMarkersNodesAll2 and
// projectMarkerFieldToNodes, markerProjection.c:11-250).
//
// Deterministic, atomic-free design.  With the columns sorted by cell, every node
// gathers its contributions itself: the markers of the (at most 3x3) cells that can
// touch it form three contiguous ranges (one per cell row), visited in sorted order.
// That is exactly the order in which the reference's sequential loop would add them
// if it ran over the sorted array, so each nodal sum is reproducible bit for bit.
//
// The per-marker fractional offsets (the divisions of markerProjection.c:127-154)
// are computed once per binning by k_geometry and shared by every projection and
// interpolation of the step; the node kernels only multiply and add.
//
// Node index NX or NY (the ghost column/row of fvmic2d's ghosted DMDA) receives no
// contribution (its ADD_VALUES would be dropped); a node whose weight sum is zero is
// set to zero.  On a grid periodic in x the ghost columns are the periodic images: local column
// NX adds into node column 0, NX + 1 into 1 and -1 into NX - 1, after the column's own sum (the
// order of DMLocalToGlobal's ADD on a periodic DMDA).  A node kernel then gathers each of its
// local columns L in {i, i + NX (, i - NX)} separately and adds them in that order.
//
// Staggered (cell-centre) cells sx run over [0, NCX] (NCX basic cells in x: NX - 1, or NX when
// periodic) and are stored with a row stride of NX + 1.
#include <climits>

#include "mic_df.cuh"
#include "mic_internal.cuh"

using namespace mic;

namespace {

__global__ void k_geometry(Params P, const double *__restrict__ X, const double *__restrict__ Y,
                           const int *__restrict__ cellX, const int *__restrict__ cellY, GeoOut o, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  geometry_marker(P, X[m], Y[m], cellX[m], cellY[m], o, m);
}

struct All2Out {
  double *rho, *rhodot, *etaN, *etaS, *muS, *muN, *k, *lastT, *Cp, *soxx, *soyy, *soxy;
};

struct MarkerView {
  const double *T, *eta, *rho, *sxx, *syy, *sxy;
  const int *mat, *cellX;
  const double *gx0, *gy0, *gx1, *gy1;
  const int *flags;
};

#ifdef MIC_EXACT  // the product build projects through per-cell partials (below)
struct All2Sums {
  double rho, etaS, k, T, Cp, w0, sxy, w3, etaN, w1, sxx, syy, w2;
};

// the sums of local column L (node column i, or its periodic image i + NX) of node row j, over
// the markers of the cells that can touch it, in marker order
__device__ __forceinline__ void all2_column(const Params &P, const MarkerView &mv, const int *__restrict__ cs,
                                            const mic_materials &mat, int L, int j, All2Sums &S) {
  const int NC = P.NCX;
  const int cy0 = max(j - 2, 0), cy1 = min(j, P.NY - 2);
  const int cx0 = max(L - 2, 0), cx1 = min(L, NC - 1);
  if (cx0 > cx1) return;
  for (int cy = cy0; cy <= cy1; ++cy) {
    const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
    for (int m = mb; m < me; ++m) {
      const int cx = mv.cellX[m];
      const int fl = mv.flags[m];
      // cell-centre node: staggered cell (sx, sy) = (cx + qx, cy + qy), corners sx..sx+1
      const int ox = L - (cx + (fl & 1)), oy = j - (cy + ((fl >> 1) & 1));
      if ((unsigned)ox <= 1u && (unsigned)oy <= 1u) {
        const double mx = mv.gx1[m], my = mv.gy1[m];
        const double w = (ox ? mx : (1.0 - mx)) * (oy ? my : (1.0 - my));
        S.etaN += w * mv.eta[m];
        S.w1 += w;
        if (ox == ((fl >> 4) & 1) && oy == ((fl >> 5) & 1)) {
          S.sxx += w * mv.sxx[m];
          S.syy += w * mv.syy[m];
          S.w2 += w;
        }
      }
      // basic node: cell (cx, cy) corners cx..cx+1
      const int bx = L - cx, by = j - cy;
      if ((unsigned)bx <= 1u && (unsigned)by <= 1u) {
        const double mx = mv.gx0[m], my = mv.gy0[m];
        const double w = (bx ? mx : (1.0 - mx)) * (by ? my : (1.0 - my));
        const int k = mv.mat[m];
        S.rho += w * mv.rho[m];
        S.etaS += w * mv.eta[m];
        S.k += w * mat.materialkThermal[k];
        S.T += w * mv.T[m];
        S.Cp += w * mat.materialCp[k];
        S.w0 += w;
        if (bx == ((fl >> 2) & 1) && by == ((fl >> 3) & 1)) {
          S.sxy += w * mv.sxy[m];
          S.w3 += w;
        }
      }
    }
  }
}

// One thread per node (i, j): basic-node sums (rho, etaS, k, T, Cp with ARITHMETIC weights;
// soxy with the nearest-node ARITHMETIC_LOCAL weight) and cell-centre sums (etaN ARITHMETIC;
// soxx, soyy ARITHMETIC_LOCAL) in the marker order of markerProjection.c:115-229.  Periodic in
// x, nodes 0 and 1 add their seam image's sums (local columns NX, NX + 1) after their own.
__global__ void __launch_bounds__(128) k_project_all2(Params P, MarkerView mv, const int *__restrict__ cs,
                                                       mic_materials mat, All2Out o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  All2Sums A = {}, B = {};
  all2_column(P, mv, cs, mat, i, j, A);
  if (P.xper && i + P.NX <= P.NCX + 1) all2_column(P, mv, cs, mat, i + P.NX, j, B);
  // global = 0 + the column's local sum (+ the seam image's), then a guarded divide
  const double W0 = (0.0 + A.w0) + B.w0, W1 = (0.0 + A.w1) + B.w1, W2 = (0.0 + A.w2) + B.w2,
               W3 = (0.0 + A.w3) + B.w3;
  const size_t q = (size_t)j * P.NX + i;
  o.rho[q] = (W0 != 0.0) ? ((0.0 + A.rho) + B.rho) / W0 : 0.0;
  o.etaS[q] = (W0 != 0.0) ? ((0.0 + A.etaS) + B.etaS) / W0 : 0.0;
  o.k[q] = (W0 != 0.0) ? ((0.0 + A.k) + B.k) / W0 : 0.0;
  o.lastT[q] = (W0 != 0.0) ? ((0.0 + A.T) + B.T) / W0 : 0.0;
  o.Cp[q] = (W0 != 0.0) ? ((0.0 + A.Cp) + B.Cp) / W0 : 0.0;
  o.soxy[q] = (W3 != 0.0) ? ((0.0 + A.sxy) + B.sxy) / W3 : 0.0;
  o.etaN[q] = (W1 != 0.0) ? ((0.0 + A.etaN) + B.etaN) / W1 : 0.0;
  o.soxx[q] = (W2 != 0.0) ? ((0.0 + A.sxx) + B.sxx) / W2 : 0.0;
  o.soyy[q] = (W2 != 0.0) ? ((0.0 + A.syy) + B.syy) / W2 : 0.0;
  o.rhodot[q] = 0.0;
  o.muS[q] = 1e99;
  o.muN[q] = 1e99;
}
#endif

// Single-field ARITHMETIC projection reusing the step geometry: STAG 0 -> basic nodes
// (projectMarkersNodesFromScalar, markers.c:1507-1594, and stagger (0,0)); STAG -1 ->
// cell centres (stagger (-1,-1), e.g. the strain-rate residual of residual.c:20).
template <int STAG>
__device__ __forceinline__ void geo_arith_column(const Params &P, const double *__restrict__ v,
                                                 const int *__restrict__ cellX, const double *__restrict__ gx,
                                                 const double *__restrict__ gy, const int *__restrict__ flags,
                                                 const int *__restrict__ cs, int L, int j, double &s, double &w_) {
  const int NC = P.NCX;
  const int R = (STAG == 0) ? 1 : 2;
  const int cy0 = max(j - R, 0), cy1 = min(j, P.NY - 2);
  const int cx0 = max(L - R, 0), cx1 = min(L, NC - 1);
  if (cx0 > cx1) return;
  for (int cy = cy0; cy <= cy1; ++cy) {
    const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
    for (int m = mb; m < me; ++m) {
      const int cx = cellX[m];
      int ox, oy;
      if (STAG == 0) {
        ox = L - cx;
        oy = j - cy;
      } else {
        const int fl = flags[m];
        ox = L - (cx + (fl & 1));
        oy = j - (cy + ((fl >> 1) & 1));
      }
      if ((unsigned)ox <= 1u && (unsigned)oy <= 1u) {
        const double mx = gx[m], my = gy[m];
        const double w = (ox ? mx : (1.0 - mx)) * (oy ? my : (1.0 - my));
        s += w * v[m];
        w_ += w;
      }
    }
  }
}

template <int STAG>
__global__ void __launch_bounds__(128) k_project_geo_arith(Params P, const double *__restrict__ v,
                                                            const int *__restrict__ cellX,
                                                            const double *__restrict__ gx,
                                                            const double *__restrict__ gy,
                                                            const int *__restrict__ flags,
                                                            const int *__restrict__ cs, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  double s = 0.0, w_ = 0.0, s2 = 0.0, w2 = 0.0;
  geo_arith_column<STAG>(P, v, cellX, gx, gy, flags, cs, i, j, s, w_);
  if (P.xper && i + P.NX <= P.NCX + 1) geo_arith_column<STAG>(P, v, cellX, gx, gy, flags, cs, i + P.NX, j, s2, w2);
  const double W = (0.0 + w_) + w2;
  out[(size_t)j * P.NX + i] = (W != 0.0) ? ((0.0 + s) + s2) / W : 0.0;
}

// Generic projectMarkerFieldToNodes for any stagger in {-1,0,1}^2 and method, computing the
// offsets from scratch (markerProjection.c:115-229): the sums of local column L of node row j,
// over candidate cells cx in [L-2, L+1].
__device__ __forceinline__ void generic_column(const Params &P, const double *__restrict__ X,
                                               const double *__restrict__ Y, const int *__restrict__ cellX,
                                               const double *__restrict__ v, const int *__restrict__ mat,
                                               const double *__restrict__ matprop_dev, int stagx, int stagy,
                                               int method, const int *__restrict__ cs, int L, int j, double &s,
                                               double &w_) {
  const int NC = P.NCX;
  const int cy0 = max(j - 2, 0), cy1 = min(j + 1, P.NY - 2);
  const int cx0 = max(L - 2, 0), cx1 = min(L + 1, NC - 1);
  if (cx0 > cx1) return;
  for (int cy = cy0; cy <= cy1; ++cy) {
    const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
    for (int m = mb; m < me; ++m) {
      const int cx = cellX[m];
      const double x = X[m], y = Y[m];
      int sx = cx, sy = cy;
      if (stagx == 1) {
        if (x < P.xc[cx + 1]) sx--;
      } else if (stagx == -1) {
        if (x >= P.xc[cx + 1]) sx++;
      }
      if (stagy == 1) {
        if (y < P.yc[cy + 1]) sy--;
      } else if (stagy == -1) {
        if (y >= P.yc[cy + 1]) sy++;
      }
      if (L - sx < 0 || L - sx > 1 || j - sy < 0 || j - sy > 1) continue;
      double mdx, mdy;
      if (stagx == -1)
        mdx = (x - P.xc[sx]) / (P.xc[sx + 1] - P.xc[sx]);
      else if (stagx == 0)
        mdx = (x - P.x[sx]) / (P.x[sx + 1] - P.x[sx]);
      else
        mdx = (x - P.xc[sx + 1]) / (P.xc[sx + 2] - P.xc[sx + 1]);
      if (stagy == -1)
        mdy = (y - P.yc[sy]) / (P.yc[sy + 1] - P.yc[sy]);
      else if (stagy == 0)
        mdy = (y - P.y[sy]) / (P.y[sy + 1] - P.y[sy]);
      else
        mdy = (y - P.yc[sy + 1]) / (P.yc[sy + 2] - P.yc[sy + 1]);
      const double val = matprop_dev ? matprop_dev[mat[m]] : v[m];
      const int ox = L - sx, oy = j - sy;
      if (method == MIC_ARITHMETIC) {
        const double w = (ox ? mdx : (1.0 - mdx)) * (oy ? mdy : (1.0 - mdy));
        s += w * val;
        w_ += w;
      } else {
        const int lx = mdx >= 0.5, ly = mdy >= 0.5;
        if (ox != lx || oy != ly) continue;
        if (method == MIC_ARITHMETIC_LOCAL) {
          const double w = (lx ? mdx : (1.0 - mdx)) * (ly ? mdy : (1.0 - mdy));
          s += w * val;
          w_ += w;
        } else {  // HARMONIC
          s += 1.0 / val;
          w_ += 1.0;
        }
      }
    }
  }
}

// One thread per node.  Periodic in x, node NX - 1 adds local column -1 (stagger +1 reaches it)
// and nodes 0, 1 add columns NX, NX + 1 after their own.
__global__ void __launch_bounds__(128) k_project_generic(Params P, const double *__restrict__ X,
                                                          const double *__restrict__ Y,
                                                          const int *__restrict__ cellX,
                                                          const double *__restrict__ v, const int *__restrict__ mat,
                                                          const double *__restrict__ matprop_dev, int stagx,
                                                          int stagy, int method, const int *__restrict__ cs,
                                                          double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  double s = 0.0, w_ = 0.0, s2 = 0.0, w2 = 0.0;
  generic_column(P, X, Y, cellX, v, mat, matprop_dev, stagx, stagy, method, cs, i, j, s, w_);
  if (P.xper) {
    const int L = (i == P.NX - 1) ? -1 : (i + P.NX <= P.NCX + 1 ? i + P.NX : INT_MIN);
    if (L != INT_MIN) generic_column(P, X, Y, cellX, v, mat, matprop_dev, stagx, stagy, method, cs, L, j, s2, w2);
  }
  const double a = (0.0 + s) + s2, W = (0.0 + w_) + w2;
  const size_t q = (size_t)j * P.NX + i;
  if (method == MIC_HARMONIC)
    out[q] = (a != 0.0) ? W / a : 0.0;
  else
    out[q] = (W != 0.0) ? a / W : 0.0;
}

inline dim3 node_grid(const Params &P) { return dim3((P.NX + 127) / 128, P.NY); }

#ifndef MIC_EXACT
// staggered cells: NCX + 1 per row
inline dim3 centre_grid(const Params &P) { return dim3((P.NCX + 1 + 127) / 128, P.NY); }

// ---- product build: divergence-free projection through per-cell corner partials ------
//
// One thread per cell runs over the cell's markers, whose quadrant runs are contiguous
// after the (cell, quadrant) sort, and accumulates each marker's weight into all four
// corners of its (basic or staggered) cell: every lane of a warp does useful FP64 work
// on every iteration, instead of one thread per node testing, and mostly discarding, the
// markers of nine cells.  A node kernel then adds the four cell partials that meet at
// each node in a fixed order and divides.  Summation order differs from the reference's
// sequential loop (rounding at the last place); the order is fixed, so results are
// reproducible run to run.  Corner k = ox + 2*oy; quadrant q = qx + 2*qy.

struct PartialView {
  const double *T, *eta, *rho, *sxx, *syy, *sxy, *scalar;
  const int *mat;
  const double *gx0, *gy0, *gx1, *gy1;
  const int *flags;
  const double *w0, *w1;  // stored corner weights of the basic and the cell-centre cell
};

// ALL2: rho, etaS, k, T, Cp, weight per corner (24) + nearest-node sxy, weight (8) = 32 sums.
// !ALL2: scalar, weight per corner = 8 sums.  part[acc * ncells + cell].  VISC (with ALL2): only
// the sums whose marker inputs yielding and the viscosity limit change (etaS per corner, the
// nearest-node sxy and its weight); the other slots keep the previous ALL2 pass's sums.  FIRST
// (with ALL2): only the others (rho, k, T, Cp and the weight per corner), for a projection whose
// viscosity and stress fields a VISC pass replaces before they are read.
//
// One loop over the cell's markers (its four quadrant runs back to back, the same order as
// quadrant by quadrant): a warp's lanes then wait for the longest cell of the warp once, not
// for the longest run of each quadrant four times.  The nearest-node sums go to a per-thread
// shared-memory slot picked by the marker's corner, so the loop has no corner branches.
template <bool ALL2, bool VISC = false, bool FIRST = false>
__global__ void __launch_bounds__(128) k_partials_basic(Params P, PartialView v, const int *__restrict__ qs,
                                                         mic_materials mat, double *__restrict__ part) {
  __shared__ double sloc[(ALL2 && !FIRST) ? 8 : 1][128];
  const int ncells = P.NCX * (P.NY - 1);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  constexpr int NA = ALL2 ? 6 : 2;
  const int t = threadIdx.x;
  // ALL2: rho (0), k (2) and Cp (4) sums in double-float arithmetic (slot f of accd); etaS (1,
  // whose own pass measured slower in double-float), T (3) and the weights (5), which later enter
  // differences (T against marker T in the sub-grid temperature pass), and the scalar
  // projections in FP64 (acc)
  double acc[4][NA];
  df accd[4][ALL2 ? 5 : 1];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int f = 0; f < NA; ++f) acc[k][f] = 0.0;
#pragma unroll
    for (int f = 0; f < (ALL2 ? 5 : 1); ++f) accd[k][f] = df{0.0f, 0.0f};
  }
  if (ALL2 && !FIRST) {
#pragma unroll
    for (int k = 0; k < 8; ++k) sloc[k][t] = 0.0;
  }
  const int mb = qs[4 * c], me = qs[4 * c + 4];
  for (int m = mb; m < me; ++m) {
    const W4 ww = load_w4(v.w0, m);
    const double w[4] = {ww.w00, ww.w10, ww.w01, ww.w11};
    if (ALL2 && VISC) {
      const double e = v.eta[m];
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[k][1] = fma(w[k], e, acc[k][1]);
    } else if (ALL2) {
      const double tt = v.T[m];
      const df r = df_of(v.rho[m]);
      const double e = FIRST ? 0.0 : v.eta[m];
      const int mt = v.mat[m];
      const df kk = df_of(mat.materialkThermal[mt]), cp = df_of(mat.materialCp[mt]);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const df wk = df_of(w[k]);
        accd[k][0] = df_fma(wk, r, accd[k][0]);
        if (!FIRST) acc[k][1] = fma(w[k], e, acc[k][1]);
        accd[k][2] = df_fma(wk, kk, accd[k][2]);
        acc[k][3] = fma(w[k], tt, acc[k][3]);
        accd[k][4] = df_fma(wk, cp, accd[k][4]);
        acc[k][5] += w[k];
      }
    }
    if (ALL2 && !FIRST) {
      // nearest basic node (mdx0 >= .5, mdy0 >= .5): the weight of that corner, as w[corner]
      const int fl = v.flags[m];
      const int corner = ((fl >> 2) & 1) | (((fl >> 3) & 1) << 1);
      const double wc = w4_at(ww, corner);
      double *L = &sloc[2 * corner][t];
      L[0] = fma(wc, v.sxy[m], L[0]);
      L[128] = __dadd_rn(L[128], wc);
    } else if (!ALL2) {
      const double sc = v.scalar[m];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        acc[k][0] = fma(w[k], sc, acc[k][0]);
        acc[k][1] += w[k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int f = 0; f < NA; ++f)
      if ((!VISC || f == 1) && (!FIRST || f != 1))
        part[(size_t)(k * NA + f) * ncells + c] =
            (ALL2 && (f == 0 || f == 2 || f == 4)) ? df_to_f64(accd[k][f]) : acc[k][f];
    if (ALL2 && !FIRST) {
      part[(size_t)(24 + 2 * k) * ncells + c] = sloc[2 * k][t];
      part[(size_t)(25 + 2 * k) * ncells + c] = sloc[2 * k + 1][t];
    }
  }
}

// Staggered (cell-centre) cell s = (sx, sy), sx in [0, NCX]: its markers are quadrant 3 of
// basic cell (sx-1, sy-1), quadrant 2 of (sx, sy-1), quadrant 1 of (sx-1, sy) and quadrant 0 of
// (sx, sy).  ALL2: etaN, weight per corner (8) + nearest-node sxx, syy, weight (12) = 20 sums;
// !ALL2: scalar, weight per corner = 8.  part[acc * (NX+1)*NY + s], s = sy (NX+1) + sx.
//
// The four runs are walked as one sequence (run 0's markers, then run 1's, ...) by one loop,
// for the same reason as in k_partials_basic; the nearest-centre sums use per-thread shared
// slots.
template <bool ALL2>
__global__ void __launch_bounds__(128) k_partials_centre(Params P, PartialView v, const int *__restrict__ qs,
                                                          double *__restrict__ part) {
  __shared__ double sloc[ALL2 ? 12 : 1][128];
  const int sx = blockIdx.x * blockDim.x + threadIdx.x;
  const int sy = blockIdx.y;
  if (sx > P.NCX || sy >= P.NY) return;
  const int NC = P.NCX;
  const int t = threadIdx.x;
  const size_t ns = (size_t)(P.NX + 1) * P.NY, s = (size_t)sy * (P.NX + 1) + sx;
  double acc[4][2];
#pragma unroll
  for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = 0.0;
  if (ALL2) {
#pragma unroll
    for (int k = 0; k < 12; ++k) sloc[k][t] = 0.0;
  }
  int rb[4], rn[4];  // run starts and lengths; a run outside the grid is empty
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int dx = r & 1, dy = r >> 1;         // basic cell (sx-1+dx, sy-1+dy) ...
    const int cx = sx - 1 + dx, cy = sy - 1 + dy;
    const int q = (1 - dx) + 2 * (1 - dy);      // ... contributes its quadrant q
    rb[r] = 0;
    rn[r] = 0;
    if (cx >= 0 && cx < NC && cy >= 0 && cy <= P.NY - 2) {
      const int qq = 4 * (cy * NC + cx) + q;
      rb[r] = qs[qq];
      rn[r] = qs[qq + 1] - qs[qq];
    }
  }
  const int e1 = rn[0], e2 = e1 + rn[1], e3 = e2 + rn[2], total = e3 + rn[3];
  for (int u = 0; u < total; ++u) {
    const int m = (u < e1) ? rb[0] + u : (u < e2) ? rb[1] + (u - e1) : (u < e3) ? rb[2] + (u - e2) : rb[3] + (u - e3);
    const W4 ww = load_w4(v.w1, m);
    const double w[4] = {ww.w00, ww.w10, ww.w01, ww.w11};
    const double e = ALL2 ? v.eta[m] : v.scalar[m];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      acc[k][0] = fma(w[k], e, acc[k][0]);
      acc[k][1] += w[k];
    }
    if (ALL2) {
      // nearest cell centre (mdx1 >= .5, mdy1 >= .5), weight as w[corner]
      const int fl = v.flags[m];
      const int corner = ((fl >> 4) & 1) | (((fl >> 5) & 1) << 1);
      const double wc = w4_at(ww, corner);
      double *L = &sloc[3 * corner][t];
      L[0] = fma(wc, v.sxx[m], L[0]);
      L[128] = fma(wc, v.syy[m], L[128]);
      L[256] = __dadd_rn(L[256], wc);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    part[(size_t)(2 * k) * ns + s] = acc[k][0];
    part[(size_t)(2 * k + 1) * ns + s] = acc[k][1];
    if (ALL2) {
      part[(size_t)(8 + 3 * k) * ns + s] = sloc[3 * k][t];
      part[(size_t)(9 + 3 * k) * ns + s] = sloc[3 * k + 1][t];
      part[(size_t)(10 + 3 * k) * ns + s] = sloc[3 * k + 2][t];
    }
  }
}

// Node (i, j): basic sums from cells (i-1,j-1) corner 3, (i,j-1) corner 2, (i-1,j) corner 1,
// (i,j) corner 0; centre sums from staggered cells with the same offsets.
__device__ __forceinline__ double guarded(double a, double w) { return (w != 0.0) ? a / w : 0.0; }
// 1/w for several sums over one weight (one division; each product within an ulp of the quotient)
__device__ __forceinline__ double guarded_rcp(double w) { return (w != 0.0) ? 1.0 / w : 0.0; }

// MODE 0 every field; 1 (VISC) only the viscosity and stress fields (etaS, soxy, etaN, soxx,
// soyy), rho, k, T, Cp and the constants keeping the previous full pass's values; 2 (FIRST) only
// the others, from basic-cell sums alone (pc unused).
template <int MODE>
__global__ void __launch_bounds__(128) k_combine_all2(Params P, const double *__restrict__ pb,
                                                       const double *__restrict__ pc, All2Out o) {
  constexpr bool VISC = MODE == 1, FIRST = MODE == 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  const int NC = P.NCX, ncells = NC * (P.NY - 1);
  const size_t ns = (size_t)(P.NX + 1) * P.NY;
  double b[8] = {0, 0, 0, 0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
  // local columns of this node: its own and, periodic, the seam image i + NX (nodes 0 and 1)
  const int nL = (P.xper && i + P.NX <= NC + 1) ? 2 : 1;
  for (int l = 0; l < nL; ++l) {
    const int L = i + l * P.NX;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int dx = r & 1, dy = r >> 1;
      const int cx = L - 1 + dx, cy = j - 1 + dy, k = (1 - dx) + 2 * (1 - dy);
      if (cx >= 0 && cx < NC && cy >= 0 && cy <= P.NY - 2) {
        const size_t cc = (size_t)cy * NC + cx;
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if ((!VISC || f == 1 || f == 5) && (!FIRST || f != 1)) b[f] += pb[(size_t)(k * 6 + f) * ncells + cc];
        if (!FIRST) {
          b[6] += pb[(size_t)(24 + 2 * k) * ncells + cc];
          b[7] += pb[(size_t)(25 + 2 * k) * ncells + cc];
        }
      }
      if (!FIRST && cx >= 0 && cx <= NC && cy >= 0) {  // staggered cells exist for sx in [0, NCX]
        const size_t ss = (size_t)cy * (P.NX + 1) + cx;
        c[0] += pc[(size_t)(2 * k) * ns + ss];
        c[1] += pc[(size_t)(2 * k + 1) * ns + ss];
        c[2] += pc[(size_t)(8 + 3 * k) * ns + ss];
        c[3] += pc[(size_t)(9 + 3 * k) * ns + ss];
        c[4] += pc[(size_t)(10 + 3 * k) * ns + ss];
      }
    }
  }
  const size_t q = (size_t)j * P.NX + i;
  const double r0 = guarded_rcp(b[5]);  // shared weight sums
  if (!FIRST) {
    const double r2 = guarded_rcp(c[4]);
    o.etaS[q] = b[1] * r0;
    o.soxy[q] = guarded(b[6], b[7]);
    o.etaN[q] = guarded(c[0], c[1]);
    o.soxx[q] = c[2] * r2;
    o.soyy[q] = c[3] * r2;
  }
  if (!VISC) {
    o.rho[q] = b[0] * r0;
    o.k[q] = b[2] * r0;
    o.lastT[q] = b[3] * r0;
    o.Cp[q] = b[4] * r0;
    o.rhodot[q] = 0.0;
    o.muS[q] = 1e99;
    o.muN[q] = 1e99;
  }
}

template <int STAG>
__global__ void __launch_bounds__(128) k_combine_scalar(Params P, const double *__restrict__ part,
                                                         double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  const int NC = P.NCX, ncells = NC * (P.NY - 1);
  const size_t ns = (size_t)(P.NX + 1) * P.NY;
  double a = 0.0, w = 0.0;
  const int nL = (P.xper && i + P.NX <= NC + 1) ? 2 : 1;
  for (int l = 0; l < nL; ++l) {
    const int L = i + l * P.NX;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int dx = r & 1, dy = r >> 1;
      const int cx = L - 1 + dx, cy = j - 1 + dy, k = (1 - dx) + 2 * (1 - dy);
      if (STAG == 0) {
        if (cx >= 0 && cx < NC && cy >= 0 && cy <= P.NY - 2) {
          const size_t cc = (size_t)cy * NC + cx;
          a += part[(size_t)(2 * k) * ncells + cc];
          w += part[(size_t)(2 * k + 1) * ncells + cc];
        }
      } else if (cx >= 0 && cx <= NC && cy >= 0) {
        const size_t ss = (size_t)cy * (P.NX + 1) + cx;
        a += part[(size_t)(2 * k) * ns + ss];
        w += part[(size_t)(2 * k + 1) * ns + ss];
      }
    }
  }
  out[(size_t)j * P.NX + i] = guarded(a, w);
}
#endif  // !MIC_EXACT

}  // namespace

int mic_ensure_geometry(mic_ctx *ctx) {
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  if (ctx->geo_valid) return MIC_OK;
  if (ctx->n > 0) {
    {
      MIC_KERNEL(ctx, "k_geometry");
      k_geometry<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->P, ctx->f64[C_X], ctx->f64[C_Y],
                                                               ctx->i32[C_CELLX], ctx->i32[C_CELLY], geo_out(ctx),
                                                               ctx->n);
    }
    MIC_CUDA_TRY(cudaGetLastError());
  }
  ctx->geo_valid = 1;
  return MIC_OK;
}

// Single-field ARITHMETIC projection of a sorted per-marker array (stagger 0 or -1).
int mic_project_scalar(mic_ctx *ctx, const double *v, int stag, double *out, cudaStream_t st) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
#ifndef MIC_EXACT
  {
    const cudaStream_t s = st ? st : ctx->stream;
    PartialView pv = {};
    pv.scalar = v;
    pv.gx0 = ctx->geo[0];
    pv.gy0 = ctx->geo[1];
    pv.gx1 = ctx->geo[2];
    pv.gy1 = ctx->geo[3];
    pv.flags = ctx->geo_flags;
    pv.w0 = ctx->wgt[0];
    pv.w1 = ctx->wgt[1];
    if (stag == 0) {
      {
        MIC_KERNEL_ON(ctx, "k_partials_basic<scalar>", s);
        k_partials_basic<false><<<grid_for(ctx->ncells, 128), 128, 0, s>>>(ctx->P, pv, ctx->quad_start, ctx->mat,
                                                                           ctx->part_b);
      }
      {
        MIC_KERNEL_ON(ctx, "k_combine_scalar<0>", s);
        k_combine_scalar<0><<<node_grid(ctx->P), 128, 0, s>>>(ctx->P, ctx->part_b, out);
      }
    } else {
      {
        MIC_KERNEL_ON(ctx, "k_partials_centre<scalar>", s);
        k_partials_centre<false><<<centre_grid(ctx->P), 128, 0, s>>>(ctx->P, pv, ctx->quad_start, ctx->part_c);
      }
      {
        MIC_KERNEL_ON(ctx, "k_combine_scalar<-1>", s);
        k_combine_scalar<-1><<<node_grid(ctx->P), 128, 0, s>>>(ctx->P, ctx->part_c, out);
      }
    }
    MIC_CUDA_TRY(cudaGetLastError());
    return MIC_OK;
  }
#else
  (void)st;  // the exact build projects on the context's stream
#endif
  if (stag == 0)
    {
      MIC_KERNEL(ctx, "k_project_geo_arith");
      k_project_geo_arith<0><<<node_grid(ctx->P), 128, 0, ctx->stream>>>(
          ctx->P, v, ctx->i32[C_CELLX], ctx->geo[0], ctx->geo[1], ctx->geo_flags, ctx->cell_start, out);
    }
  else
    {
      MIC_KERNEL(ctx, "k_project_geo_arith");
      k_project_geo_arith<-1><<<node_grid(ctx->P), 128, 0, ctx->stream>>>(
          ctx->P, v, ctx->i32[C_CELLX], ctx->geo[2], ctx->geo[3], ctx->geo_flags, ctx->cell_start, out);
    }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

// mode 0: every field.  1 (visc): the second projection of a step (main:303), after yielding and
// the viscosity limit changed only viscosities and stresses: the product build then forms only
// those sums and keeps the first projection's rho, k, T, Cp (same inputs, same order, so the
// same values).  2 (first, product build, on stream st): the step's first projection (main:268)
// when a visc pass follows before its viscosity and stress fields are read: only rho, k, T, Cp.
static int project_all2(mic_ctx *ctx, int mode, cudaStream_t st = nullptr) {
  const bool visc = mode == 1;
  cudaSetDevice(ctx->device);
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
  MarkerView mv;
  mv.T = ctx->f64[C_T];
  mv.eta = ctx->f64[C_ETA];
  mv.rho = ctx->f64[C_RHO];
  mv.sxx = ctx->f64[C_SXX];
  mv.syy = ctx->f64[C_SYY];
  mv.sxy = ctx->f64[C_SXY];
  mv.mat = ctx->i32[C_MAT];
  mv.cellX = ctx->i32[C_CELLX];
  mv.gx0 = ctx->geo[0];
  mv.gy0 = ctx->geo[1];
  mv.gx1 = ctx->geo[2];
  mv.gy1 = ctx->geo[3];
  mv.flags = ctx->geo_flags;
  All2Out o;
  o.rho = ctx->nodal[MIC_NF_RHO];
  o.rhodot = ctx->nodal[MIC_NF_RHODOT];
  o.etaN = ctx->nodal[MIC_NF_ETAN];
  o.etaS = ctx->nodal[MIC_NF_ETAS];
  o.muS = ctx->nodal[MIC_NF_MUS];
  o.muN = ctx->nodal[MIC_NF_MUN];
  o.k = ctx->nodal[MIC_NF_KTHERMAL];
  o.lastT = ctx->nodal[MIC_NF_LASTT];
  o.Cp = ctx->nodal[MIC_NF_CP];
  o.soxx = ctx->nodal[MIC_NF_SOXX];
  o.soyy = ctx->nodal[MIC_NF_SOYY];
  o.soxy = ctx->nodal[MIC_NF_SOXY];
#ifdef MIC_EXACT
  (void)visc;  // the exact build gathers every field in reference order each time
  (void)st;
  {
    MIC_KERNEL(ctx, "k_project_all2");
    k_project_all2<<<node_grid(ctx->P), 128, 0, ctx->stream>>>(ctx->P, mv, ctx->cell_start, ctx->mat, o);
  }
#else
  PartialView pv = {};
  pv.T = mv.T;
  pv.eta = mv.eta;
  pv.rho = mv.rho;
  pv.sxx = mv.sxx;
  pv.syy = mv.syy;
  pv.sxy = mv.sxy;
  pv.mat = mv.mat;
  pv.gx0 = mv.gx0;
  pv.gy0 = mv.gy0;
  pv.gx1 = mv.gx1;
  pv.gy1 = mv.gy1;
  pv.flags = mv.flags;
  pv.w0 = ctx->wgt[0];
  pv.w1 = ctx->wgt[1];
  if (mode == 2) {
    const cudaStream_t s = st ? st : ctx->stream;
    {
      MIC_KERNEL_ON(ctx, "k_partials_basic<first>", s);
      k_partials_basic<true, false, true><<<grid_for(ctx->ncells, 128), 128, 0, s>>>(ctx->P, pv, ctx->quad_start,
                                                                                     ctx->mat, ctx->part_b);
    }
    {
      MIC_KERNEL_ON(ctx, "k_combine_all2<first>", s);
      k_combine_all2<2><<<node_grid(ctx->P), 128, 0, s>>>(ctx->P, ctx->part_b, ctx->part_c, o);
    }
    MIC_CUDA_TRY(cudaGetLastError());
    return MIC_OK;
  }
  // the cell-centre sums on the second stream, beside the basic-cell sums: both only read the
  // markers and each runs at a fraction of the SMs' warp slots
  MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[0], ctx->stream));
  MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->aux, ctx->aux_ev[0], 0));
  {
    MIC_KERNEL_ON(ctx, "k_partials_centre", ctx->aux);
    k_partials_centre<true><<<centre_grid(ctx->P), 128, 0, ctx->aux>>>(ctx->P, pv, ctx->quad_start, ctx->part_c);
  }
  MIC_CUDA_TRY(cudaEventRecord(ctx->aux_ev[1], ctx->aux));
  if (visc) {
    MIC_KERNEL(ctx, "k_partials_basic<visc>");
    k_partials_basic<true, true><<<grid_for(ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->P, pv, ctx->quad_start,
                                                                                      ctx->mat, ctx->part_b);
  } else {
    MIC_KERNEL(ctx, "k_partials_basic");
    k_partials_basic<true><<<grid_for(ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->P, pv, ctx->quad_start,
                                                                                ctx->mat, ctx->part_b);
  }
  MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->aux_ev[1], 0));  // the cell-centre sums
  if (visc) {
    MIC_KERNEL(ctx, "k_combine_all2<visc>");
    k_combine_all2<1><<<node_grid(ctx->P), 128, 0, ctx->stream>>>(ctx->P, ctx->part_b, ctx->part_c, o);
  } else {
    MIC_KERNEL(ctx, "k_combine_all2");
    k_combine_all2<0><<<node_grid(ctx->P), 128, 0, ctx->stream>>>(ctx->P, ctx->part_b, ctx->part_c, o);
  }
#endif
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

extern "C" int mic_project_markers_nodes_all2(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
  return project_all2(ctx, 0);
}

int mic_project_all2_viscous(mic_ctx *ctx) { return project_all2(ctx, 1); }

int mic_project_all2_first(mic_ctx *ctx, cudaStream_t s) {
#ifdef MIC_EXACT
  (void)s;
  return project_all2(ctx, 0);
#else
  return project_all2(ctx, 2, s);
#endif
}

extern "C" int mic_project_marker_field_to_nodes(mic_ctx *ctx, int off, const double *matprop, int out_field,
                                                 int stagx, int stagy, int method) {
  if (!ctx || out_field < 0 || out_field >= MIC_NF_COUNT) return MIC_ERR_ARG;
  if (stagx < -1 || stagx > 1 || stagy < -1 || stagy > 1) return MIC_ERR_ARG;
  if (method != MIC_ARITHMETIC && method != MIC_ARITHMETIC_LOCAL && method != MIC_HARMONIC) return MIC_ERR_ARG;
  int col = -1;
  if (!matprop) {
    col = mic_f64_column_of_offset(off);
    if (col < 0) return MIC_ERR_ARG;
  }
  cudaSetDevice(ctx->device);
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  double *mp = nullptr;
  if (matprop) {
    mp = ctx->red_buf;  // MIC_MAXMAT values
    MIC_CUDA_TRY(cudaMemcpyAsync(mp, matprop, sizeof(double) * MIC_MAXMAT, cudaMemcpyHostToDevice, ctx->stream));
  }
  {
    MIC_KERNEL(ctx, "k_project_generic");
    k_project_generic<<<node_grid(ctx->P), 128, 0, ctx->stream>>>(
        ctx->P, ctx->f64[C_X], ctx->f64[C_Y], ctx->i32[C_CELLX], col >= 0 ? ctx->f64[col] : nullptr, ctx->i32[C_MAT],
        mp, stagx, stagy, method, ctx->cell_start, ctx->nodal[out_field]);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// projectMarkersNodesFromScalar (markers.c:1507-1594): a per-marker array in the caller's order
// projected onto the basic nodes (the bilinear weights of each marker's basic cell), divided by
// the weights; zero where nothing contributes
extern "C" int mic_project_markers_nodes_from_scalar(mic_ctx *ctx, const double *values, int out_field) {
  if (!ctx || (!values && ctx->n > 0) || out_field < 0 || out_field >= MIC_NF_COUNT) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  if (ctx->n > 0) {
    MIC_CUDA_TRY(cudaMemcpyAsync(ctx->scr1, values, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->stream));
    if ((e = mic_gather_by_id(ctx, ctx->scr1, ctx->scr2))) return e;
  }
  if ((e = mic_project_scalar(ctx, ctx->scr2, 0, ctx->nodal[out_field]))) return e;
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}
