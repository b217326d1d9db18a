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
// set to zero.
#include "mic_internal.cuh"

using namespace mic;

namespace {

__global__ void k_geometry(Params P, const double *__restrict__ X, const double *__restrict__ Y,
                           const int *__restrict__ cellX, const int *__restrict__ cellY, double *__restrict__ gx0,
                           double *__restrict__ gy0, double *__restrict__ gx1, double *__restrict__ gy1,
                           int *__restrict__ flags, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const int cx = cellX[m], cy = cellY[m];
  if (cx < 0) {
    flags[m] = 0;
    return;
  }
  const double x = X[m], y = Y[m];
  // basic cell (markerProjection.c:131-146, stagger 0)
  const double mdx0 = (x - P.x[cx]) / (P.x[cx + 1] - P.x[cx]);
  const double mdy0 = (y - P.y[cy]) / (P.y[cy + 1] - P.y[cy]);
  // cell-centre cell (findCellStag2D stagger -1, markerProjection.c:260-267, 128-143)
  const int qx = nonneg_bits(x) >= nonneg_bits(P.xc[cx + 1]);
  const int qy = nonneg_bits(y) >= nonneg_bits(P.yc[cy + 1]);
  const int sx = cx + qx, sy = cy + qy;
  const double mdx1 = (x - P.xc[sx]) / (P.xc[sx + 1] - P.xc[sx]);
  const double mdy1 = (y - P.yc[sy]) / (P.yc[sy + 1] - P.yc[sy]);
  const long long half = 0x3FE0000000000000LL;  // bits of 0.5; all offsets here are >= 0
  int f = qx | (qy << 1);
  f |= (nonneg_bits(mdx0) >= half) << 2;
  f |= (nonneg_bits(mdy0) >= half) << 3;
  f |= (nonneg_bits(mdx1) >= half) << 4;
  f |= (nonneg_bits(mdy1) >= half) << 5;
  gx0[m] = mdx0;
  gy0[m] = mdy0;
  gx1[m] = mdx1;
  gy1[m] = mdy1;
  flags[m] = f;
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

// One thread per node (i, j): basic-node sums (rho, etaS, k, T, Cp with ARITHMETIC weights;
// soxy with the nearest-node ARITHMETIC_LOCAL weight) and cell-centre sums (etaN ARITHMETIC;
// soxx, soyy ARITHMETIC_LOCAL) in the marker order of markerProjection.c:115-229.
__global__ void __launch_bounds__(128) k_project_all2(Params P, MarkerView mv, const int *__restrict__ cs,
                                                       mic_materials mat, All2Out o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P.NX || j >= P.NY) return;
  const int NC = P.NX - 1;
  double sRho = 0.0, sEtaS = 0.0, sK = 0.0, sT = 0.0, sCp = 0.0, w0 = 0.0, sSxy = 0.0, w3 = 0.0;
  double sEtaN = 0.0, w1 = 0.0, sSxx = 0.0, sSyy = 0.0, w2 = 0.0;
  const int cy0 = max(j - 2, 0), cy1 = min(j, P.NY - 2);
  const int cx0 = max(i - 2, 0), cx1 = min(i, P.NX - 2);
  for (int cy = cy0; cy <= cy1; ++cy) {
    const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
    for (int m = mb; m < me; ++m) {
      const int cx = mv.cellX[m];
      const int fl = mv.flags[m];
      // cell-centre node: staggered cell (sx, sy) = (cx + qx, cy + qy), corners sx..sx+1
      const int ox = i - (cx + (fl & 1)), oy = j - (cy + ((fl >> 1) & 1));
      if ((unsigned)ox <= 1u && (unsigned)oy <= 1u) {
        const double mx = mv.gx1[m], my = mv.gy1[m];
        const double w = (ox ? mx : (1.0 - mx)) * (oy ? my : (1.0 - my));
        sEtaN += w * mv.eta[m];
        w1 += w;
        if (ox == ((fl >> 4) & 1) && oy == ((fl >> 5) & 1)) {
          sSxx += w * mv.sxx[m];
          sSyy += w * mv.syy[m];
          w2 += w;
        }
      }
      // basic node: cell (cx, cy) corners cx..cx+1
      const int bx = i - cx, by = j - cy;
      if ((unsigned)bx <= 1u && (unsigned)by <= 1u) {
        const double mx = mv.gx0[m], my = mv.gy0[m];
        const double w = (bx ? mx : (1.0 - mx)) * (by ? my : (1.0 - my));
        const int k = mv.mat[m];
        sRho += w * mv.rho[m];
        sEtaS += w * mv.eta[m];
        sK += w * mat.materialkThermal[k];
        sT += w * mv.T[m];
        sCp += w * mat.materialCp[k];
        w0 += w;
        if (bx == ((fl >> 2) & 1) && by == ((fl >> 3) & 1)) {
          sSxy += w * mv.sxy[m];
          w3 += w;
        }
      }
    }
  }
  const size_t q = (size_t)j * P.NX + i;
  // global = 0 + local sum (DMLocalToGlobal ADD into a zeroed vector), then a guarded divide
  const double W0 = 0.0 + w0, W1 = 0.0 + w1, W2 = 0.0 + w2, W3 = 0.0 + w3;
  o.rho[q] = (W0 != 0.0) ? (0.0 + sRho) / W0 : 0.0;
  o.etaS[q] = (W0 != 0.0) ? (0.0 + sEtaS) / W0 : 0.0;
  o.k[q] = (W0 != 0.0) ? (0.0 + sK) / W0 : 0.0;
  o.lastT[q] = (W0 != 0.0) ? (0.0 + sT) / W0 : 0.0;
  o.Cp[q] = (W0 != 0.0) ? (0.0 + sCp) / W0 : 0.0;
  o.soxy[q] = (W3 != 0.0) ? (0.0 + sSxy) / W3 : 0.0;
  o.etaN[q] = (W1 != 0.0) ? (0.0 + sEtaN) / W1 : 0.0;
  o.soxx[q] = (W2 != 0.0) ? (0.0 + sSxx) / W2 : 0.0;
  o.soyy[q] = (W2 != 0.0) ? (0.0 + sSyy) / W2 : 0.0;
  o.rhodot[q] = 0.0;
  o.muS[q] = 1e99;
  o.muN[q] = 1e99;
}

// Single-field ARITHMETIC projection reusing the step geometry: STAG 0 -> basic nodes
// (projectMarkersNodesFromScalar, markers.c:1507-1594, and stagger (0,0)); STAG -1 ->
// cell centres (stagger (-1,-1), e.g. the strain-rate residual of residual.c:20).
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
  const int NC = P.NX - 1;
  const int R = (STAG == 0) ? 1 : 2;
  double s = 0.0, w_ = 0.0;
  const int cy0 = max(j - R, 0), cy1 = min(j, P.NY - 2);
  const int cx0 = max(i - R, 0), cx1 = min(i, P.NX - 2);
  for (int cy = cy0; cy <= cy1; ++cy) {
    const int mb = cs[cy * NC + cx0], me = cs[cy * NC + cx1 + 1];
    for (int m = mb; m < me; ++m) {
      const int cx = cellX[m];
      int ox, oy;
      if (STAG == 0) {
        ox = i - cx;
        oy = j - cy;
      } else {
        const int fl = flags[m];
        ox = i - (cx + (fl & 1));
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
  const double W = 0.0 + w_;
  out[(size_t)j * P.NX + i] = (W != 0.0) ? (0.0 + s) / W : 0.0;
}

// Generic projectMarkerFieldToNodes for any stagger in {-1,0,1}^2 and method, computing the
// offsets from scratch (markerProjection.c:115-229).  Candidate cells cx in [i-2, i+1].
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
  const int NC = P.NX - 1;
  double s = 0.0, w_ = 0.0;
  const int cy0 = max(j - 2, 0), cy1 = min(j + 1, P.NY - 2);
  const int cx0 = max(i - 2, 0), cx1 = min(i + 1, P.NX - 2);
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
      if (i - sx < 0 || i - sx > 1 || j - sy < 0 || j - sy > 1) continue;
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
      const int ox = i - sx, oy = j - sy;
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
  const double a = 0.0 + s, W = 0.0 + w_;
  const size_t q = (size_t)j * P.NX + i;
  if (method == MIC_HARMONIC)
    out[q] = (a != 0.0) ? W / a : 0.0;
  else
    out[q] = (W != 0.0) ? a / W : 0.0;
}

inline dim3 node_grid(const Params &P) { return dim3((P.NX + 127) / 128, P.NY); }

}  // namespace

int mic_ensure_geometry(mic_ctx *ctx) {
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  if (ctx->geo_valid) return MIC_OK;
  if (ctx->n > 0) {
    {
      MIC_KERNEL(ctx, "k_geometry");
      k_geometry<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->P, ctx->f64[C_X], ctx->f64[C_Y],
                                                               ctx->i32[C_CELLX], ctx->i32[C_CELLY], ctx->geo[0],
                                                               ctx->geo[1], ctx->geo[2], ctx->geo[3],
                                                               ctx->geo_flags, ctx->n);
    }
    MIC_CUDA_TRY(cudaGetLastError());
  }
  ctx->geo_valid = 1;
  return MIC_OK;
}

// Single-field ARITHMETIC projection of a sorted per-marker array (stagger 0 or -1).
int mic_project_scalar(mic_ctx *ctx, const double *v, int stag, double *out) {
  int e = mic_ensure_geometry(ctx);
  if (e) return e;
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

extern "C" int mic_project_markers_nodes_all2(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
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
  {
    MIC_KERNEL(ctx, "k_project_all2");
    k_project_all2<<<node_grid(ctx->P), 128, 0, ctx->stream>>>(ctx->P, mv, ctx->cell_start, ctx->mat, o);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
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
