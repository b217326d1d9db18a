/*
 * mic_oracle.c -- CPU restatement of fvmic2d's marker-in-cell transfer path.
 * TEST INFRASTRUCTURE ONLY (see mic_oracle.h).  Reference citations are
 * file:line in the fvmic2d tree.
 *
 * Single-rank DMDA semantics restated here: scatter-adds that land on a node
 * index NX or NY (the ghost column/row of a ghosted, non-periodic DMDA) are
 * dropped; a zero weight sum divides to zero (VecPointwiseDivide with a guarded
 * divisor); ghost values are never read because boundary types other than
 * prescribed (0) and free slip (1) are rejected.
 */
#include "mic_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc_ctx {
  const double *grain;     /* per-marker grain size for the composite creep law (law 7) */
  int64_t ngrain;
  int NX, NY;
  double LX, LY;
  double *buf;
  double *x, *y, *xc, *yc; /* ghost offset 2 */
  mic_materials mat;
  mic_options opt;
  mic_bcs bcs;
  double *nodal[MIC_NF_COUNT];
  double *scratch;         /* per-marker scratch (subgrid temperature change) */
  int64_t scratch_n;
  double residuals[100];   /* residual.c:9-10 ring of stored residuals */
  const mic_marker *mk_base; /* marker array of the current call (indexes the grain sizes) */
  int jaumann;             /* stress rotation: the reference built with -DJAUMANN (markers.c:2147-2156) */
};

#define NODE(c, f, i, j) ((c)->nodal[f][(size_t)(j) * (size_t)(c)->NX + (size_t)(i)])

orc_ctx *orc_create(int NX, int NY, double LX, double LY, const double *x, const double *y) {
  if (NX < 3 || NY < 3) return NULL;
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  if (!c) return NULL;
  c->NX = NX;
  c->NY = NY;
  c->LX = LX;
  c->LY = LY;
  size_t nx4 = (size_t)NX + 4, ny4 = (size_t)NY + 4;
  c->buf = (double *)malloc((2 * nx4 + 2 * ny4) * sizeof(double));
  for (size_t k = 0; k < 2 * nx4 + 2 * ny4; ++k) c->buf[k] = NAN;
  c->x = c->buf + 2;
  c->xc = c->buf + nx4 + 2;
  c->y = c->buf + 2 * nx4 + 2;
  c->yc = c->buf + 2 * nx4 + ny4 + 2;
  for (int i = 0; i < NX; ++i) c->x[i] = x[i];
  for (int j = 0; j < NY; ++j) c->y[j] = y[j];
  /* getCellCenters (gridSpacing.c:150-157) */
  for (int i = 1; i < NX; ++i) c->xc[i] = (c->x[i - 1] + c->x[i]) / 2.0;
  c->xc[0] = -c->xc[1];
  c->xc[NX] = 2.0 * LX - c->xc[NX - 1];
  for (int j = 1; j < NY; ++j) c->yc[j] = (c->y[j - 1] + c->y[j]) / 2.0;
  c->yc[0] = -c->yc[1];
  c->yc[NY] = 2.0 * LY - c->yc[NY - 1];
  for (int f = 0; f < MIC_NF_COUNT; ++f) c->nodal[f] = (double *)calloc((size_t)NX * NY, sizeof(double));
  for (int b = 0; b < 4; ++b) {
    mic_bcinfo *s = &((mic_bcinfo *)&c->bcs)[b];
    for (int k = 0; k < 3; ++k) s->type[k] = 1;
  }
  return c;
}

void orc_destroy(orc_ctx *c) {
  if (!c) return;
  for (int f = 0; f < MIC_NF_COUNT; ++f) free(c->nodal[f]);
  free(c->scratch);
  free(c->buf);
  free(c);
}

void orc_get_grid(const orc_ctx *c, double *xc, double *yc) {
  for (int i = 0; i <= c->NX; ++i) xc[i] = c->xc[i];
  for (int j = 0; j <= c->NY; ++j) yc[j] = c->yc[j];
}

void orc_set_materials(orc_ctx *c, const mic_materials *m) { c->mat = *m; }
void orc_set_options(orc_ctx *c, const mic_options *o) { c->opt = *o; }
void orc_set_jaumann(orc_ctx *c, int on) { c->jaumann = on != 0; }

int orc_set_bcs(orc_ctx *c, const mic_bcs *b) {
  /* markers.c:1986-2023 reads ghost velocities unless the top vx / left vy boundary is 0 or 1 */
  if (b->mechBCTop.type[0] != 0 && b->mechBCTop.type[0] != 1) return ORC_ERR_BC;
  if (b->mechBCLeft.type[1] != 0 && b->mechBCLeft.type[1] != 1) return ORC_ERR_BC;
  c->bcs = *b;
  return ORC_OK;
}

int orc_set_nodal(orc_ctx *c, int f, const double *v) {
  if (f < 0 || f >= MIC_NF_COUNT) return ORC_ERR_ARG;
  memcpy(c->nodal[f], v, sizeof(double) * (size_t)c->NX * c->NY);
  return ORC_OK;
}

int orc_get_nodal(const orc_ctx *c, int f, double *v) {
  if (f < 0 || f >= MIC_NF_COUNT) return ORC_ERR_ARG;
  memcpy(v, c->nodal[f], sizeof(double) * (size_t)c->NX * c->NY);
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* cell location                                                              */

/* Largest i in [0, n-2] with g[i] <= v, by bisection (markers.c:47-69). */
static int bisect_cell(const double *g, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (v >= g[mid])
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

/* findMarkerCell / findMarkerCells (markers.c:41-106) */
int64_t orc_find_marker_cells(orc_ctx *c, mic_marker *mk, int64_t n, int *err) {
  int64_t nout = 0;
  *err = ORC_OK;
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->X >= 0.0 && p->Y >= 0.0 && p->X <= c->LX && p->Y <= c->LY) {
      p->cellX = bisect_cell(c->x, c->NX, p->X);
      p->cellY = bisect_cell(c->y, c->NY, p->Y);
      if (p->cellX < 0 || p->cellX > c->NX - 2 || p->cellY < 0 || p->cellY > c->NY - 2) *err = ORC_ERR_CELL;
    } else {
      p->cellX = -1;
      p->cellY = -1;
    }
    p->cpu = 0;
    if (p->cellX == -1) nout++;
  }
  return nout;
}

/* main_subduction.c:255-264 */
void orc_update_marker_rho(orc_ctx *c, mic_marker *mk, int64_t n) {
  for (int64_t m = 0; m < n; ++m) {
    if (mk[m].cellX == -1) continue;
    int k = mk[m].Mat;
    mk[m].rho = -c->mat.materialRho[k] * (c->mat.materialAlpha[k] * mk[m].T);
    mk[m].rhodot = 0.0;
  }
}

/* main_subduction.c:271-281 */
double orc_max_marker_T(const orc_ctx *c, const mic_marker *mk, int64_t n) {
  (void)c;
  double t = 0.0;
  for (int64_t m = 0; m < n; ++m)
    if (mk[m].cellX != -1 && mk[m].T > t) t = mk[m].T;
  return t;
}

/* main_subduction.c:437-448 */
double orc_max_abs_sxx(const orc_ctx *c, const mic_marker *mk, int64_t n) {
  (void)c;
  double s = 0.0;
  for (int64_t m = 0; m < n; ++m)
    if (mk[m].cellX != -1 && fabs(mk[m].s.T11) > s) s = fabs(mk[m].s.T11);
  return s;
}

/* ------------------------------------------------------------------------- */
/* marker -> node projection                                                  */

static double field_at(const mic_marker *m, int off) { return *(const double *)((const char *)m + off); }

/* Staggered cell (findCellStag2D, markerProjection.c:252-269) and the fractional
 * offsets of markerProjection.c:127-154. */
static void stag_cell(const orc_ctx *c, const mic_marker *p, int stagx, int stagy, int *cx, int *cy, double *mdx,
                      double *mdy) {
  int i = p->cellX, j = p->cellY;
  if (stagx == 1) {
    if (p->X < c->xc[p->cellX + 1]) i--;
  } else if (stagx == -1) {
    if (p->X >= c->xc[p->cellX + 1]) i++;
  }
  if (stagy == 1) {
    if (p->Y < c->yc[p->cellY + 1]) j--;
  } else if (stagy == -1) {
    if (p->Y >= c->yc[p->cellY + 1]) j++;
  }
  if (stagx == -1)
    *mdx = (p->X - c->xc[i]) / (c->xc[i + 1] - c->xc[i]);
  else if (stagx == 0)
    *mdx = (p->X - c->x[i]) / (c->x[i + 1] - c->x[i]);
  else
    *mdx = (p->X - c->xc[i + 1]) / (c->xc[i + 2] - c->xc[i + 1]);
  if (stagy == -1)
    *mdy = (p->Y - c->yc[j]) / (c->yc[j + 1] - c->yc[j]);
  else if (stagy == 0)
    *mdy = (p->Y - c->y[j]) / (c->y[j + 1] - c->y[j]);
  else
    *mdy = (p->Y - c->yc[j + 1]) / (c->yc[j + 2] - c->yc[j + 1]);
  *cx = i;
  *cy = j;
}

/* accumulate into an interior node; node index NX or NY is a ghost of the DMDA and is dropped */
static inline void acc2(double *nf, double *wt, int NX, int NY, int i, int j, double w, double v) {
  if (i < 0 || j < 0 || i >= NX || j >= NY) return;
  size_t k = (size_t)j * NX + i;
  nf[k] += w * v;
  wt[k] += w;
}

/* projectMarkerFieldToNodes (markerProjection.c:71-250) */
int orc_project_marker_field(orc_ctx *c, const mic_marker *mk, int64_t n, int field_offset, const double *matprop,
                             int out_field, int stagx, int stagy, int method) {
  if (out_field < 0 || out_field >= MIC_NF_COUNT) return ORC_ERR_ARG;
  if (stagx < -1 || stagx > 1 || stagy < -1 || stagy > 1) return ORC_ERR_ARG;
  if (method != MIC_ARITHMETIC && method != MIC_ARITHMETIC_LOCAL && method != MIC_HARMONIC) return ORC_ERR_ARG;
  const int NX = c->NX, NY = c->NY;
  const size_t nn = (size_t)NX * NY;
  double *nf = (double *)calloc(nn, sizeof(double));
  double *wt = (double *)calloc(nn, sizeof(double));
  for (int64_t m = 0; m < n; ++m) {
    const mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const double v = matprop ? matprop[p->Mat] : field_at(p, field_offset);
    int i, j;
    double mdx, mdy;
    stag_cell(c, p, stagx, stagy, &i, &j, &mdx, &mdy);
    if (method == MIC_ARITHMETIC) {
      acc2(nf, wt, NX, NY, i, j, (1.0 - mdx) * (1.0 - mdy), v);
      acc2(nf, wt, NX, NY, i + 1, j, mdx * (1.0 - mdy), v);
      acc2(nf, wt, NX, NY, i, j + 1, (1.0 - mdx) * (mdy), v);
      acc2(nf, wt, NX, NY, i + 1, j + 1, mdx * mdy, v);
    } else if (method == MIC_ARITHMETIC_LOCAL) {
      double w = 1.0;
      if (mdx >= 0.5) {
        i++;
        w *= mdx;
      } else {
        w *= (1.0 - mdx);
      }
      if (mdy >= 0.5) {
        j++;
        w *= mdy;
      } else {
        w *= (1.0 - mdy);
      }
      acc2(nf, wt, NX, NY, i, j, w, v);
    } else {
      if (mdx >= 0.5) i++;
      if (mdy >= 0.5) j++;
      if (i < NX && j < NY) {
        nf[(size_t)j * NX + i] += 1.0 / v;
        wt[(size_t)j * NX + i] += 1.0;
      }
    }
  }
  double *out = c->nodal[out_field];
  for (size_t k = 0; k < nn; ++k) {
    double a = 0.0 + nf[k], b = 0.0 + wt[k];
    if (method == MIC_HARMONIC)
      out[k] = (a != 0.0) ? b / a : 0.0;
    else
      out[k] = (b != 0.0) ? a / b : 0.0;
  }
  free(nf);
  free(wt);
  return ORC_OK;
}

/* projectMarkersNodesAll2 (markerProjection.c:11-68) */
int orc_project_markers_nodes_all2(orc_ctx *c, const mic_marker *mk, int64_t n) {
  const int o_rho = (int)offsetof(mic_marker, rho), o_eta = (int)offsetof(mic_marker, eta);
  const int o_T = (int)offsetof(mic_marker, T);
  const int o_s11 = (int)offsetof(mic_marker, s.T11), o_s22 = (int)offsetof(mic_marker, s.T22);
  const int o_s12 = (int)offsetof(mic_marker, s.T12);
  int e = 0;
  e |= orc_project_marker_field(c, mk, n, o_rho, NULL, MIC_NF_RHO, 0, 0, MIC_ARITHMETIC);
  memset(c->nodal[MIC_NF_RHODOT], 0, sizeof(double) * (size_t)c->NX * c->NY);
  e |= orc_project_marker_field(c, mk, n, o_eta, NULL, MIC_NF_ETAN, -1, -1, MIC_ARITHMETIC);
  e |= orc_project_marker_field(c, mk, n, o_eta, NULL, MIC_NF_ETAS, 0, 0, MIC_ARITHMETIC);
  for (size_t k = 0; k < (size_t)c->NX * c->NY; ++k) {
    c->nodal[MIC_NF_MUS][k] = 1e99;
    c->nodal[MIC_NF_MUN][k] = 1e99;
  }
  e |= orc_project_marker_field(c, mk, n, -1, c->mat.materialkThermal, MIC_NF_KTHERMAL, 0, 0, MIC_ARITHMETIC);
  e |= orc_project_marker_field(c, mk, n, o_T, NULL, MIC_NF_LASTT, 0, 0, MIC_ARITHMETIC);
  e |= orc_project_marker_field(c, mk, n, -1, c->mat.materialCp, MIC_NF_CP, 0, 0, MIC_ARITHMETIC);
  e |= orc_project_marker_field(c, mk, n, o_s11, NULL, MIC_NF_SOXX, -1, -1, MIC_ARITHMETIC_LOCAL);
  e |= orc_project_marker_field(c, mk, n, o_s22, NULL, MIC_NF_SOYY, -1, -1, MIC_ARITHMETIC_LOCAL);
  e |= orc_project_marker_field(c, mk, n, o_s12, NULL, MIC_NF_SOXY, 0, 0, MIC_ARITHMETIC_LOCAL);
  return e ? ORC_ERR_ARG : ORC_OK;
}

/* projectNodalFieldToMarkersS (markers.c:1670-1706): basic-node bilinear value */
int orc_project_nodal_to_markers(orc_ctx *c, mic_marker *mk, int64_t n, int f, int field_offset) {
  if (f < 0 || f >= MIC_NF_COUNT) return ORC_ERR_ARG;
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    int i = p->cellX, j = p->cellY;
    double mdx = (p->X - c->x[i]) / (c->x[i + 1] - c->x[i]);
    double mdy = (p->Y - c->y[j]) / (c->y[j + 1] - c->y[j]);
    double val = NODE(c, f, i, j) * (1 - mdx) * (1 - mdy) + NODE(c, f, i, j + 1) * (1 - mdx) * mdy +
                 NODE(c, f, i + 1, j) * (mdx) * (1 - mdy) + NODE(c, f, i + 1, j + 1) * mdx * mdy;
    *(double *)((char *)p + field_offset) = val;
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* rheology                                                                   */

/* computeRheology (viscosity.c:12-67) */
int orc_compute_rheology(const orc_ctx *c, const mic_marker *p, double *eta, double *mu) {
  const int k = p->Mat;
  const mic_materials *M = &c->mat;
  *mu = M->materialMu[k];
  switch (M->hasEtaT[k]) {
    case 1:
      *eta = M->materialEta[k] * exp(M->QonR[k] * (1.0 / p->T - 1.0 / M->Tref[k]));
      return ORC_OK;
    case 2: {
      double T0 = M->Tref[k];
      *eta = M->materialEta[k] * exp(M->QonR[k] / T0 * (1.0 - (p->T - T0) / T0));
      return ORC_OK;
    }
    case 3:
      *eta = M->materialEta[k] * p->T;
      return ORC_OK;
    case 5:
      *eta = M->materialEta[k] * exp(-M->QonR[k] * p->T);
      return ORC_OK;
    case 0:
      *eta = M->materialEta[k];
      return ORC_OK;
    case 6: {
      double depth = p->Y, dist = p->X, e = M->materialEta[k];
      double edge = depth / tan(c->opt.slabAngle);
      if (dist > edge && dist < (edge + c->opt.decoupleThickness) && depth > c->opt.minDecoupleDepth &&
          depth < c->opt.maxDecoupleDepth)
        e *= c->opt.decoupleEtaScaler;
      *eta = e;
      return ORC_OK;
    }
    case 7: {
      /* composite ice creep: the stress at which the Goldsby-Kohlstedt strain rate
       * (viscosity.c:106-179) equals the marker's strain-rate invariant */
      const int64_t m = p - c->mk_base;
      if (!c->grain || m < 0 || m >= c->ngrain) return ORC_ERR_LAW;
      const double e2 = 0.5 * (p->e.T11 * p->e.T11 + p->e.T22 * p->e.T22) + p->e.T12 * p->e.T12;
      const double edot = sqrt(e2);
      double sst;
      int it;
      orc_creep_stress(edot, p->T, c->grain[m], p->p, 1e-14, &sst, &it);
      *eta = (edot > 0.0) ? sst / (2.0 * edot) : orc_gk_viscosity(0.0, p->T, c->grain[m], p->p);
      return ORC_OK;
    }
    default:
      return ORC_ERR_LAW;
  }
}

/* checkPlasticYielding (markers.c:1381-1505) */
int orc_check_plastic_yielding(orc_ctx *c, mic_marker *mk, int64_t n, double dt, int *is_yielding) {
  const mic_materials *M = &c->mat;
  c->mk_base = mk;
  const double etamin = c->opt.etamin, etamax = c->opt.etamax, frac = c->opt.fractionalEtamin;
  int err = ORC_OK;
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const double eta_old = p->eta;
    double etanew = eta_old;
    /* visco-elastic stress forecast with the old viscosity (markers.c:1397-1402) */
    const double X = p->eta / (p->mu * dt + p->eta);
    const double sxx = p->s.T11 * X + 2 * p->eta * p->e.T11 * (1.0 - X);
    const double syy = p->s.T22 * X + 2 * p->eta * p->e.T22 * (1.0 - X);
    const double sxy = p->s.T12 * X + 2 * p->eta * p->e.T12 * (1.0 - X);
    const double sii = sqrt(0.5 * (sxx * sxx + syy * syy) + sxy * sxy);
    (void)sii;
    double eta, mu;
    if (orc_compute_rheology(c, p, &eta, &mu) != ORC_OK) err = ORC_ERR_LAW;
    p->eta = eta;
    p->mu = mu;
    const int k = p->Mat;
    const int plast = M->hasPlasticity[k];
    if (!plast) continue;
    double sy;
    if (plast == 1) {
      sy = M->materialCohesion[k] + M->materialFriction[k] * p->p;
    } else if (plast == 2) {
      /* linear strain weakening between gamma[0] and gamma[1] (markers.c:1426-1448) */
      const double E = p->Eii;
      double coh, fr;
      if (E < M->gamma[k][0]) {
        coh = M->C[k][0];
        fr = sin(M->F[k][0] / 180.0 * M_PI);
      } else if (E >= M->gamma[k][0] && E <= M->gamma[k][1]) {
        const double dg = (E - M->gamma[k][0]) / (M->gamma[k][1] - M->gamma[k][0]);
        coh = (M->C[k][1] - M->C[k][0]) * dg + M->C[k][0];
        fr = (sin(M->F[k][1] / 180.0 * M_PI) - sin(M->F[k][0] / 180.0 * M_PI)) * dg + sin(M->F[k][0] / 180.0 * M_PI);
      } else {
        coh = M->C[k][1];
        fr = sin(M->F[k][1] / 180.0 * M_PI);
      }
      sy = coh + fr * p->p;
    } else {
      sy = 0.0;
    }
    if (sy < 0.0) sy = 0.0;
    if (sii > sy) {
      const double exx = p->e.T11, eyy = p->e.T22, exy = p->e.T12;
      const double eii = sqrt(0.5 * (exx * exx + eyy * eyy) + exy * exy);
      etanew = sy / 2.0 / eii;
      if (etanew / p->eta < frac) etanew = frac * p->eta;
      if (etanew < etamin)
        etanew = etamin;
      else if (etanew > etamax)
        etanew = etamax;
      const double sio = sqrt(0.5 * (p->s.T11 * p->s.T11 + p->s.T22 * p->s.T22) + p->s.T12 * p->s.T12);
      if (sio != 0.0) {
        p->s.T11 *= sy / sio;
        p->s.T22 *= sy / sio;
        p->s.T12 *= sy / sio;
      }
      *is_yielding = 1;
    }
    /* plastic materials keep the pre-update viscosity unless they yield (markers.c:1397, 1493) */
    p->eta = etanew;
  }
  return err;
}

/* limitViscosity / limitMarkerViscosity (viscosity.c:90-104): every marker, in domain or not */
void orc_limit_viscosity(orc_ctx *c, mic_marker *mk, int64_t n) {
  for (int64_t m = 0; m < n; ++m) {
    if (mk[m].eta > c->opt.etamax)
      mk[m].eta = c->opt.etamax;
    else if (mk[m].eta < c->opt.etamin)
      mk[m].eta = c->opt.etamin;
  }
}

/* ------------------------------------------------------------------------- */
/* node -> marker                                                             */

/* Pressure-cell (cell-centre) lookup with the bounds of updateMarkerStrainPressure.c:137-147:
 * step right when X >= xc[cellX+1] (only while cellX < xlim), down when Y >= yc[cellY+1] (while
 * cellY < NY-1), then clamp to the interior [1, NX-2] x [1, NY-2]. */
static void centre_cell(const orc_ctx *c, const mic_marker *p, int xlim, int *cx, int *cy, double *mdx, double *mdy) {
  int i = p->cellX, j = p->cellY;
  if (i < xlim && p->X >= c->xc[i + 1]) i++;
  if (j < c->NY - 1 && p->Y >= c->yc[j + 1]) j++;
  if (j < 1)
    j = 1;
  else if (j > c->NY - 2)
    j = c->NY - 2;
  if (i < 1)
    i = 1;
  else if (i > c->NX - 2)
    i = c->NX - 2;
  *mdx = (p->X - c->xc[i]) / (c->xc[i + 1] - c->xc[i]);
  *mdy = (p->Y - c->yc[j]) / (c->yc[j + 1] - c->yc[j]);
  *cx = i;
  *cy = j;
}

/* Basic cell clamped to [0, NX-2] x [0, NY-2] (updateMarkerStrainPressure.c:208-215). */
static void basic_cell(const orc_ctx *c, const mic_marker *p, int *cx, int *cy, double *mdx, double *mdy) {
  int i = p->cellX, j = p->cellY;
  if (j < 0)
    j = 0;
  else if (j > c->NY - 2)
    j = c->NY - 2;
  if (i < 0)
    i = 0;
  else if (i > c->NX - 2)
    i = c->NX - 2;
  *mdx = (p->X - c->x[i]) / (c->x[i + 1] - c->x[i]);
  *mdy = (p->Y - c->y[j]) / (c->y[j + 1] - c->y[j]);
  *cx = i;
  *cy = j;
}

/* Running bilinear sum in the order 00, 01, 10, 11 used by updateMarkerStrainPressure.c,
 * subgridStressChanges.c and updateMarkerStress.c. */
static inline double interp_run(const orc_ctx *c, int f, int i, int j, double mdx, double mdy) {
  double s = 0.0;
  s += (1.0 - mdx) * (1.0 - mdy) * NODE(c, f, i, j);
  s += (1.0 - mdx) * mdy * NODE(c, f, i, j + 1);
  s += mdx * (1.0 - mdy) * NODE(c, f, i + 1, j);
  s += mdx * mdy * NODE(c, f, i + 1, j + 1);
  return s;
}

/* updateMarkerStrainPressure (updateMarkerStrainPressure.c:131-339, non-TEXTURE branch) */
int orc_update_marker_strain_pressure(orc_ctx *c, mic_marker *mk, int64_t n, double dt) {
  int err = ORC_OK;
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    int i, j;
    double mdx, mdy;
    centre_cell(c, p, c->NX - 2, &i, &j, &mdx, &mdy);
    p->p = interp_run(c, MIC_NF_P, i, j, mdx, mdy);
    const double mexx = interp_run(c, MIC_NF_EDOTXX, i, j, mdx, mdy);
    const double msxx = interp_run(c, MIC_NF_SOXX, i, j, mdx, mdy);
    const double msyy = interp_run(c, MIC_NF_SOYY, i, j, mdx, mdy);
    const double mdsxx = interp_run(c, MIC_NF_DSXX, i, j, mdx, mdy);
    const double mdsyy = interp_run(c, MIC_NF_DSYY, i, j, mdx, mdy);
    basic_cell(c, p, &i, &j, &mdx, &mdy);
    p->wxy = interp_run(c, MIC_NF_WXY, i, j, mdx, mdy);
    const double mexy = interp_run(c, MIC_NF_EDOTXY, i, j, mdx, mdy);
    const double msxy = interp_run(c, MIC_NF_SOXY, i, j, mdx, mdy);
    const double mdsxy = interp_run(c, MIC_NF_DSXY, i, j, mdx, mdy);
    /* Gerya's method 1: viscous + elastic strain rate from nodal stress and stress change */
    p->e.T11 = msxx / 2.0 / p->eta + mdsxx / 2.0 / dt / p->mu;
    p->e.T22 = msyy / 2.0 / p->eta + mdsyy / 2.0 / dt / p->mu;
    p->e.T12 = msxy / 2.0 / p->eta + mdsxy / 2.0 / dt / p->mu;
    p->strainRateResidual = sqrt(pow(p->e.T11 - mexx, 2.0) + pow(p->e.T12 - mexy, 2.0));
    if (isnan(p->strainRateResidual)) err = ORC_ERR_NAN;
  }
  return err;
}

/* updateGlobalStrainRateResidual (residual.c:12-51) */
double orc_update_global_strain_rate_residual(orc_ctx *c, const mic_marker *mk, int64_t n, int iter) {
  orc_project_marker_field(c, mk, n, (int)offsetof(mic_marker, strainRateResidual), NULL, MIC_NF_SRR, -1, -1,
                           MIC_ARITHMETIC);
  double *srr = c->nodal[MIC_NF_SRR];
  for (int j = 0; j < c->NY; ++j)
    for (int i = 0; i < c->NX; ++i) {
      size_t k = (size_t)j * c->NX + i;
      if (i > 0 && j > 0)
        srr[k] *= (c->x[i] - c->x[i - 1]) * (c->y[j] - c->y[j - 1]);
      else
        srr[k] = 0.0;
    }
  double sum = 0.0;
  for (size_t k = 0; k < (size_t)c->NX * c->NY; ++k) sum += srr[k];
  sum /= (c->LX * c->LY);
  c->residuals[iter % 100] = sum;
  return sum;
}

/* subgridStressChanges (subgridStressChanges.c:5-318) */
int orc_subgrid_stress_changes(orc_ctx *c, mic_marker *mk, int64_t n, double dt, double D) {
  const int NX = c->NX, NY = c->NY;
  const size_t nn = (size_t)NX * NY;
  double *dxy = (double *)calloc(nn, sizeof(double)), *wxy = (double *)calloc(nn, sizeof(double));
  double *dxx = (double *)calloc(nn, sizeof(double)), *dyy = (double *)calloc(nn, sizeof(double));
  double *wn = (double *)calloc(nn, sizeof(double));
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    /* relaxation factor 1 - exp(-D dt mu / eta), exponent floored at -30 (subgridStressChanges.c:81-85) */
    const double sdm = p->eta / p->mu;
    double sdif = -D * dt / sdm;
    if (sdif < -30.0) sdif = -30.0;
    sdif = 1.0 - exp(sdif);
    int i, j;
    double mdx, mdy;
    basic_cell(c, p, &i, &j, &mdx, &mdy);
    double dsxy = interp_run(c, MIC_NF_SOXY, i, j, mdx, mdy) - p->s.T12;
    dsxy *= sdif;
    p->s.T12 += dsxy;
    /* quadrant scatter of the shear change; a marker on a half line feeds both sides (134-175) */
    i = p->cellX;
    j = p->cellY;
    mdx = (p->X - c->x[i]) / (c->x[i + 1] - c->x[i]);
    mdy = (p->Y - c->y[j]) / (c->y[j + 1] - c->y[j]);
    if (mdx <= 0.5 && mdy <= 0.5) {
      size_t k = (size_t)j * NX + i;
      dxy[k] = dxy[k] + (1.0 - mdx) * (1.0 - mdy) * dsxy;
      wxy[k] = wxy[k] + (1.0 - mdx) * (1.0 - mdy);
    }
    if (mdx <= 0.5 && mdy >= 0.5) {
      size_t k = (size_t)(j + 1) * NX + i;
      dxy[k] = dxy[k] + (1.0 - mdx) * (mdy)*dsxy;
      wxy[k] = wxy[k] + (1.0 - mdx) * (mdy);
    }
    if (mdx >= 0.5 && mdy <= 0.5) {
      size_t k = (size_t)j * NX + i + 1;
      dxy[k] = dxy[k] + (mdx) * (1.0 - mdy) * dsxy;
      wxy[k] = wxy[k] + (mdx) * (1.0 - mdy);
    }
    if (mdx >= 0.5 && mdy >= 0.5) {
      size_t k = (size_t)(j + 1) * NX + i + 1;
      dxy[k] = dxy[k] + (mdx) * (mdy)*dsxy;
      wxy[k] = wxy[k] + (mdx) * (mdy);
    }
    /* normal components at the pressure cell (178-210) */
    centre_cell(c, p, NX - 1, &i, &j, &mdx, &mdy);
    double dsxx = interp_run(c, MIC_NF_SOXX, i, j, mdx, mdy) - p->s.T11;
    dsxx *= sdif;
    p->s.T11 += dsxx;
    double dsyy = interp_run(c, MIC_NF_SOYY, i, j, mdx, mdy) - p->s.T22;
    dsyy *= sdif;
    p->s.T22 += dsyy;
    /* scatter to the cell's own centre node with a tent weight (222-233) */
    i = p->cellX;
    j = p->cellY;
    mdy = (p->Y - c->y[j]) / (c->y[j + 1] - c->y[j]);
    mdx = (p->X - c->x[i]) / (c->x[i + 1] - c->x[i]);
    {
      size_t k = (size_t)(j + 1) * NX + i + 1;
      dxx[k] += (1.0 - fabs(0.5 - mdx)) * (1.0 - fabs(0.5 - mdy)) * dsxx;
      dyy[k] += (1.0 - fabs(0.5 - mdx)) * (1.0 - fabs(0.5 - mdy)) * dsyy;
      wn[k] += (1.0 - fabs(0.5 - mdx)) * (1.0 - fabs(0.5 - mdy));
    }
  }
  /* divide by the weights and remove the subgrid part from the nodal stress changes (258-286) */
  for (size_t k = 0; k < nn; ++k) {
    double a = 0.0 + dxy[k], w = 0.0 + wxy[k];
    double gxy = (w != 0.0) ? a / w : 0.0;
    double wn_ = 0.0 + wn[k];
    double gxx = (wn_ != 0.0) ? (0.0 + dxx[k]) / wn_ : 0.0;
    double gyy = (wn_ != 0.0) ? (0.0 + dyy[k]) / wn_ : 0.0;
    c->nodal[MIC_NF_DSXX][k] = c->nodal[MIC_NF_DSXX][k] + -1.0 * gxx;
    c->nodal[MIC_NF_DSYY][k] = c->nodal[MIC_NF_DSYY][k] + -1.0 * gyy;
    c->nodal[MIC_NF_DSXY][k] = c->nodal[MIC_NF_DSXY][k] + -1.0 * gxy;
  }
  free(dxy);
  free(wxy);
  free(dxx);
  free(dyy);
  free(wn);
  return ORC_OK;
}

/* updateMarkerStress (updateMarkerStress.c:5-163) */
int orc_update_marker_stress(orc_ctx *c, mic_marker *mk, int64_t n, int64_t *nan_count) {
  int64_t nans = 0;
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    int i, j;
    double mdx, mdy;
    centre_cell(c, p, c->NX - 2, &i, &j, &mdx, &mdy);
    const double mdsxx = interp_run(c, MIC_NF_DSXX, i, j, mdx, mdy);
    const double mdsyy = interp_run(c, MIC_NF_DSYY, i, j, mdx, mdy);
    p->s.T11 += mdsxx;
    p->s.T22 += mdsyy;
    basic_cell(c, p, &i, &j, &mdx, &mdy);
    const double mdsxy = interp_run(c, MIC_NF_DSXY, i, j, mdx, mdy);
    p->s.T12 += mdsxy;
    if (isnan(mdsxy)) nans++;
  }
  if (nan_count) *nan_count = nans;
  return ORC_OK;
}

/* subgridTemperatureChanges (subgridTemperatureChanges.c:5-124) with the marker-to-node
 * projection of the subgrid change (projectMarkersNodesFromScalar, markers.c:1507-1594). */
int orc_subgrid_temperature_changes(orc_ctx *c, mic_marker *mk, int64_t n, double dt) {
  const int NX = c->NX, NY = c->NY;
  const size_t nn = (size_t)NX * NY;
  const double D = c->opt.subgridTemperatureDiffusivity;
  if (c->scratch_n < n) {
    free(c->scratch);
    c->scratch = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    c->scratch_n = n;
  }
  double *dTsub = c->scratch;
  const double *Tn = c->nodal[MIC_NF_LASTT], *rn = c->nodal[MIC_NF_RHO];
  const double *cpn = c->nodal[MIC_NF_CP], *kn = c->nodal[MIC_NF_KTHERMAL];
  for (int64_t m = 0; m < n; ++m) {
    const mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const int i = p->cellX, j = p->cellY;
    const size_t k00 = (size_t)j * NX + i, k10 = k00 + 1, k01 = k00 + NX, k11 = k01 + 1;
    const double dx = c->x[i + 1] - c->x[i], dy = c->y[j + 1] - c->y[j];
    const double mdx = (p->X - c->x[i]) / dx, mdy = (p->Y - c->y[j]) / dy;
    const double Tm = Tn[k00] * (1.0 - mdx) * (1.0 - mdy) + Tn[k10] * mdx * (1.0 - mdy) +
                      Tn[k01] * (1.0 - mdx) * (mdy) + Tn[k11] * mdx * mdy;
    const double rhom = c->mat.materialRho[0] + rn[k00] * (1.0 - mdx) * (1.0 - mdy) + rn[k10] * (mdx) * (1.0 - mdy) +
                        rn[k01] * (1.0 - mdx) * (mdy) + rn[k11] * mdx * mdy;
    const double cpm = cpn[k00] * (1.0 - mdx) * (1.0 - mdy) + cpn[k10] * (mdx) * (1.0 - mdy) +
                       cpn[k01] * (1.0 - mdx) * (mdy) + cpn[k11] * mdx * mdy;
    const double km = kn[k00] * (1.0 - mdx) * (1.0 - mdy) + kn[k10] * (mdx) * (1.0 - mdy) +
                      kn[k01] * (1.0 - mdx) * (mdy) + kn[k11] * mdx * mdy;
    /* diffusion time of one cell, Gerya's eq. 10.16 */
    const double tdiff = cpm * rhom / km / (2.0 / (dx * dx) + 2.0 / (dy * dy));
    dTsub[m] = (Tm - p->T) * (1.0 - exp(-D * dt / tdiff));
  }
  /* project the subgrid change onto basic nodes */
  double *nf = (double *)calloc(nn, sizeof(double)), *wt = (double *)calloc(nn, sizeof(double));
  for (int64_t m = 0; m < n; ++m) {
    const mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const int i = p->cellX, j = p->cellY;
    const double dx = c->x[i + 1] - c->x[i], dy = c->y[j + 1] - c->y[j];
    const double mdx = (p->X - c->x[i]) / dx, mdy = (p->Y - c->y[j]) / dy;
    const size_t k00 = (size_t)j * NX + i;
    double w = (1.0 - mdx) * (1.0 - mdy);
    wt[k00] += w;
    nf[k00] += w * dTsub[m];
    w = mdx * (1.0 - mdy);
    wt[k00 + 1] += w;
    nf[k00 + 1] += w * dTsub[m];
    w = (1.0 - mdx) * mdy;
    wt[k00 + NX] += w;
    nf[k00 + NX] += w * dTsub[m];
    w = mdx * mdy;
    wt[k00 + NX + 1] += w;
    nf[k00 + NX + 1] += w * dTsub[m];
  }
  /* remaining nodal change: thisT - lastT - projected subgrid change (VecAXPBYPCZ, alpha = 1) */
  const double *thisT = c->nodal[MIC_NF_THIST];
  for (size_t k = 0; k < nn; ++k) {
    double w = 0.0 + wt[k];
    double proj = (w != 0.0) ? (0.0 + nf[k]) / w : 0.0;
    nf[k] = thisT[k] + -1.0 * Tn[k] + -1.0 * proj;
  }
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const int i = p->cellX, j = p->cellY;
    const double dx = c->x[i + 1] - c->x[i], dy = c->y[j + 1] - c->y[j];
    const double mdx = (p->X - c->x[i]) / dx, mdy = (p->Y - c->y[j]) / dy;
    const size_t k00 = (size_t)j * NX + i;
    const double dtm = (nf[k00] * (1.0 - mdy) * (1.0 - mdx) + nf[k00 + NX] * mdy * (1.0 - mdx) +
                        nf[k00 + 1] * (1.0 - mdy) * mdx + nf[k00 + NX + 1] * mdy * mdx) +
                       dTsub[m];
    p->T += dtm;
    p->Tdot = dtm / dt;
  }
  free(nf);
  free(wt);
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* advection                                                                  */

/* advectMarkersRK (markers.c:1865-2250), non-periodic grid; the stress rotation of the default
 * build or of -DJAUMANN (orc_set_jaumann) */
int orc_advect_markers_rk(orc_ctx *c, mic_marker *mk, int64_t n, double dt) {
  const int NX = c->NX, NY = c->NY;
  const double *vx = c->nodal[MIC_NF_VX], *vy = c->nodal[MIC_NF_VY], *wz = c->nodal[MIC_NF_WXY];
  const mic_bcinfo *top = &c->bcs.mechBCTop, *left = &c->bcs.mechBCLeft;
#define VXN(i, j) vx[(size_t)(j) * NX + (i)]
#define VYN(i, j) vy[(size_t)(j) * NX + (i)]
#define WZN(i, j) wz[(size_t)(j) * NX + (i)]
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    double xcur = p->X, ycur = p->Y;
    double mvx[4], mvy[4], mwz[4];
    for (int s = 0; s < 4; ++s) {
      /* walk from the stored cell to the cell holding the stage position (1928-1944) */
      int i = p->cellX, j = p->cellY;
      if (xcur > c->x[i + 1]) {
        while (xcur > c->x[i + 1] && i < NX - 2) i++;
      } else if (xcur < c->x[i]) {
        while (xcur < c->x[i] && i > 0) i--;
      }
      if (ycur > c->y[j + 1]) {
        while (ycur > c->y[j + 1] && j < NY - 2) j++;
      } else if (ycur < c->y[j]) {
        while (ycur < c->y[j] && j > 0) j--;
      }
      /* staggered vx cell (x[i], yc[j+1]) and vy cell (xc[i+1], y[j]) (1946-1974) */
      int vxX = i, vxY = j, vyX = i, vyY = j;
      if (vxY > -1 && ycur < c->yc[vxY + 1]) vxY--;
      if (vyX > -1 && xcur < c->xc[vyX + 1]) vyX--;
      if (vxX < 0)
        vxX = 0;
      else if (vxX > NX - 2)
        vxX = NX - 2;
      if (vyX < -1)
        vyX = -1;
      else if (vyX > NX - 2)
        vyX = NX - 2;
      if (vxY < -1)
        vxY = -1;
      else if (vxY > NY - 2)
        vxY = NY - 2;
      if (vyY < 0)
        vyY = 0;
      else if (vyY > NY - 2)
        vyY = NY - 2;
      double ax = xcur - c->x[vxX];
      double ay = ycur - c->yc[vxY + 1];
      double hx = c->x[vxX + 1] - c->x[vxX];
      double hy = c->yc[vxY + 2] - c->yc[vxY + 1];
      double vul, vur;
      if (vxY == -1 && top->type[0] == 0) { /* prescribed velocity on the top wall (1986-1991) */
        vul = 2.0 * top->value[0] - VXN(vxX, vxY + 1);
        vur = 2.0 * top->value[0] - VXN(vxX + 1, vxY + 1);
      } else if (vxY == -1) { /* free slip */
        vul = VXN(vxX, vxY + 1);
        vur = VXN(vxX + 1, vxY + 1);
      } else {
        vul = VXN(vxX, vxY);
        vur = VXN(vxX + 1, vxY);
      }
      double vll = VXN(vxX, vxY + 1), vlr = VXN(vxX + 1, vxY + 1);
      mvx[s] = vul * (1.0 - ax / hx) * (1.0 - ay / hy);
      mvx[s] += vur * (ax / hx) * (1.0 - ay / hy);
      mvx[s] += vll * (1.0 - ax / hx) * (ay / hy);
      mvx[s] += vlr * (ax * ay) / hx / hy;
      double wur = VYN(vyX + 1, vyY), wlr = VYN(vyX + 1, vyY + 1), wul, wll;
      if (vyX == -1 && left->type[1] == 0) { /* prescribed velocity on the left wall (2009-2023) */
        wul = 2.0 * left->value[1] - VYN(vyX + 1, vyY);
        wll = 2.0 * left->value[1] - VYN(vyX + 1, vyY + 1);
      } else if (vyX == -1) {
        wul = VYN(vyX + 1, vyY);
        wll = VYN(vyX + 1, vyY + 1);
      } else {
        wul = VYN(vyX, vyY);
        wll = VYN(vyX, vyY + 1);
      }
      ax = xcur - c->xc[vyX + 1];
      ay = ycur - c->y[vyY];
      hx = c->xc[vyX + 2] - c->xc[vyX + 1];
      hy = c->y[vyY + 1] - c->y[vyY];
      mvy[s] = wul * (1.0 - ax / hx) * (1.0 - ay / hy);
      mvy[s] += wur * (ax / hx) * (1.0 - ay / hy);
      mvy[s] += wll * (1.0 - ax / hx) * (ay / hy);
      mvy[s] += wlr * (ax * ay) / hx / hy;
      /* vorticity at basic nodes of the walked cell (2089-2094) */
      const double mdx = (xcur - c->x[i]) / (c->x[i + 1] - c->x[i]);
      const double mdy = (ycur - c->y[j]) / (c->y[j + 1] - c->y[j]);
      mwz[s] = (1.0 - mdx) * (1.0 - mdy) * WZN(i, j);
      mwz[s] += (mdx) * (1.0 - mdy) * WZN(i + 1, j);
      mwz[s] += (1.0 - mdx) * (mdy)*WZN(i, j + 1);
      mwz[s] += (mdx) * (mdy)*WZN(i + 1, j + 1);
      if (s < 2) {
        xcur = p->X + dt / 2 * mvx[s];
        ycur = p->Y + dt / 2 * mvy[s];
      } else if (s == 2) {
        xcur = p->X + dt * mvx[s];
        ycur = p->Y + dt * mvy[s];
      }
    }
    p->VX = (mvx[0] + 2 * mvx[1] + 2 * mvx[2] + mvx[3]) / 6;
    p->VY = (mvy[0] + 2 * mvy[1] + 2 * mvy[2] + mvy[3]) / 6;
    p->wxy = (mwz[0] + 2 * mwz[1] + 2 * mwz[2] + mwz[3]) / 6.0;
    p->X += dt * p->VX;
    p->Y += dt * p->VY;
    const double s11 = p->s.T11, s22 = p->s.T22, s12 = p->s.T12;
    if (c->jaumann) {
      /* first-order Jaumann terms, wxy1 = wxy dt (2147-2156) */
      const double w1 = p->wxy * dt;
      p->s.T11 += 2.0 * s12 * -w1;
      p->s.T22 += 2.0 * s12 * w1;
      p->s.T12 += (s11 - s22) * w1;
    } else {
      /* finite rotation of the stress tensor by -wxy dt (2158-2164) */
      const double th = -p->wxy * dt;
      p->s.T11 = s11 * pow(cos(th), 2.0) + s22 * pow(sin(th), 2.0) - s12 * sin(2.0 * th);
      p->s.T22 = s11 * pow(sin(th), 2.0) + s22 * pow(cos(th), 2.0) + s12 * sin(2.0 * th);
      p->s.T12 = 0.5 * (s11 - s22) * sin(2.0 * th) + s12 * cos(2.0 * th);
    }
    p->Eii += dt * sqrt(0.5 * (p->e.T11 * p->e.T11 + p->e.T22 * p->e.T22) + p->e.T12 * p->e.T12);
  }
#undef VXN
#undef VYN
#undef WZN
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
int orc_step(orc_ctx *c, mic_marker *mk, int64_t n, double dt_disp, double dt_thermal, int do_subgrid_stress,
             double *residual) {
  int err = ORC_OK, e;
  orc_find_marker_cells(c, mk, n, &e);
  if (e) return e;
  orc_update_marker_rho(c, mk, n);
  orc_project_markers_nodes_all2(c, mk, n);
  (void)orc_max_marker_T(c, mk, n);
  int yielding = 0;
  if ((e = orc_check_plastic_yielding(c, mk, n, dt_disp, &yielding))) return e;
  orc_limit_viscosity(c, mk, n);
  orc_project_markers_nodes_all2(c, mk, n);
  if ((e = orc_update_marker_strain_pressure(c, mk, n, dt_disp))) err = e;
  double r = orc_update_global_strain_rate_residual(c, mk, n, 0);
  if (residual) *residual = r;
  if (do_subgrid_stress) orc_subgrid_stress_changes(c, mk, n, dt_disp, c->opt.subgridStressDiffusivity);
  orc_update_marker_stress(c, mk, n, NULL);
  orc_subgrid_temperature_changes(c, mk, n, dt_thermal);
  orc_advect_markers_rk(c, mk, n, dt_thermal);
  (void)orc_max_abs_sxx(c, mk, n);
  return err;
}

/* ------------------------------------------------------------------------- */
/* Goldsby & Kohlstedt (2001) composite ice creep, as in viscosity.c:106-179    */
double orc_gk_viscosity(double s, double T, double d, double P) {
  const double R = 8.3144621;
  if (P < 1.0) P = 1.0;
  const double b = 4.52e-10, Vm = 1.97e-5, Qv = 59.4 * 1000.0, delta = 2.0 * b, Qb = 49 * 1000.0;
  const double D0v = 9.10e-4, D0b = 5.8e-4;
  const double Dv = D0v * exp(-Qv / (R * T));
  const double Db = D0b * exp(-Qb / (R * T));
  double ediff = 42.0 * Vm / (R * T * d * d) * (Dv + M_PI * delta / d * Db);
  if (s < 1e0) return 0.5 / ediff;
  ediff *= s;
  double A, nn, Q;
  const double V = -13e-6;
  if (T < 255) {
    A = 3.9e-3;
    nn = 1.8;
    Q = 49 * 1000.0;
  } else {
    A = 3.0e26;
    nn = 1.8;
    Q = 192 * 1000.0;
  }
  const double egbs = A * pow(s / 1e6, nn) / pow(d, 1.4) * exp((-Q + P * V) / (R * T));
  if (T < 258) {
    A = 4.0e5;
    nn = 4.0;
    Q = 60 * 1000.0;
  } else {
    A = 6.0e28;
    nn = 4.0;
    Q = 180 * 1000.0;
  }
  const double edisl = A * pow(s / 1e6, nn) * exp((-Q + P * V) / (R * T));
  const double ebs = 5.5e7 * pow(s / 1e6, 2.4) * exp((-60.0 * 1000.0 + P * V) / (R * T));
  const double etot = ediff + 1.0 / (1.0 / ebs + 1.0 / egbs) + edisl;
  return s / 2.0 / etot;
}

/* sizes of the boundary structs as this compiler lays them out (checked against the
 * ctypes mirrors by the tests) */
int64_t orc_sizeof(int which) {
  switch (which) {
    case 0: return (int64_t)sizeof(mic_marker);
    case 1: return (int64_t)sizeof(mic_materials);
    case 2: return (int64_t)sizeof(mic_bcs);
    case 3: return (int64_t)sizeof(mic_options);
    case 4: return (int64_t)offsetof(mic_marker, cellX);
    case 5: return (int64_t)offsetof(mic_materials, Tref);
    default: return -1;
  }
}

void orc_set_grain(orc_ctx *c, const double *d, int64_t n) {
  c->grain = d;
  c->ngrain = n;
}

/* Strain rate of the Goldsby-Kohlstedt law at stress s: s / (2 eta(s)) with eta from
 * viscosity.c:106-179 exactly as the reference evaluates it. */
double orc_gk_strain_rate(double s, double T, double d, double P) {
  return s / 2.0 / orc_gk_viscosity(s, T, d, P);
}

/* Stress s* >= 0 with gk_strain_rate(s*) = edot, to relative residual rtol: safeguarded
 * secant on ln(strain rate) against ln(s), which is nearly linear (local exponent 1 to 4),
 * inside a bracket that always holds the root; bisection when the secant step leaves it.
 * Below 1 Pa the law is linear diffusion creep and the root is edot / C. */
int orc_creep_stress(double edot, double T, double d, double P, double rtol, double *s_out, int *iters) {
  *iters = 0;
  if (!(edot > 0.0)) {
    *s_out = 0.0;
    return ORC_OK;
  }
  const double C = 0.5 / orc_gk_viscosity(0.5, T, d, P); /* linear coefficient, eta = 0.5 / C */
  double s_lin = edot / C;
  if (s_lin < 1.0) {
    *s_out = s_lin;
    return ORC_OK;
  }
  const double le = log(edot);
  double ulo = 0.0, flo = log(orc_gk_strain_rate(1.0, T, d, P)) - le;
  if (flo >= 0.0) { /* the rate jumps past edot at s = 1 Pa: the root is the jump point */
    *s_out = 1.0;
    return ORC_OK;
  }
  double uhi = log(s_lin), fhi = log(orc_gk_strain_rate(s_lin, T, d, P)) - le;
  while (fhi < 0.0 && *iters < 200) { /* only reached if the linear estimate undershoots */
    ulo = uhi;
    flo = fhi;
    uhi += 2.0;
    fhi = log(orc_gk_strain_rate(exp(uhi), T, d, P)) - le;
    (*iters)++;
  }
  double u = uhi, f = fhi;
  for (int it = 0; it < 200; ++it) {
    (*iters)++;
    if (fabs(f) <= rtol) break;
    double un = (flo != fhi) ? uhi - fhi * (uhi - ulo) / (fhi - flo) : 0.5 * (ulo + uhi);
    if (!(un > ulo && un < uhi)) un = 0.5 * (ulo + uhi);
    const double fn = log(orc_gk_strain_rate(exp(un), T, d, P)) - le;
    if (fn > 0.0) {
      uhi = un;
      fhi = fn;
    } else {
      ulo = un;
      flo = fn;
    }
    u = un;
    f = fn;
    if (uhi - ulo <= 1e-15 * fabs(uhi)) break;
  }
  *s_out = exp(u);
  return ORC_OK;
}

/* orc_creep_stress over arrays (test access: large strided samples in one call) */
int orc_creep_stress_batch(const double *edot, const double *T, const double *d, const double *P, int64_t n,
                           double rtol, double *s_out, int *iters) {
  for (int64_t m = 0; m < n; ++m) {
    int it = 0;
    orc_creep_stress(edot[m], T[m], d[m], P[m], rtol, &s_out[m], &it);
    if (iters) iters[m] = it;
  }
  return ORC_OK;
}

/* ---- marker lifecycle -------------------------------------------------------------- */

/* resetMarker (markers.c:255-330): the fields the reference zeroes; mu, cellX, cellY, cpu and
 * strainRateResidual are left as they are. */
void orc_reset_markers(mic_marker *mk, int64_t n) {
  for (int64_t m = 0; m < n; ++m) {
    mic_marker *p = &mk[m];
    p->X = -1;
    p->Y = -1;
    p->VX = 0;
    p->VY = 0;
    p->p = 0.0;
    p->Mat = -1;
    p->T = 0.0;
    p->Tdot = 0.0;
    p->eta = 0.0;
    p->s.T11 = p->s.T22 = p->s.T12 = 0.0;
    p->e.T11 = p->e.T22 = p->e.T12 = 0.0;
    p->rho = 0.0;
    p->rhodot = 0.0;
    p->E.T11 = p->E.T22 = p->E.T12 = 0.0;
    p->Eii = 0.0;
    p->wxy = 0.0;
    p->isYielding = 0;
  }
}

/* The random stream of the single-rank PETSc stand-in: PetscRandomSetSeed(r, s) sets the 48-bit
 * state to (s << 16) | 0x330E, and each value is lo + (hi - lo) * u with u = X / 2^48 after the
 * LCG step X <- (0x5DEECE66D X + 11) mod 2^48 (the erand48 recurrence). */
static double orc_rand48(uint64_t *state, double lo, double hi) {
  *state = (0x5DEECE66DULL * *state + 0xBULL) & 0xFFFFFFFFFFFFULL;
  const double u = (double)*state / 281474976710656.0;
  return lo + (hi - lo) * u;
}

/* distributeMarkersUniformInDomain (markers.c:342-400), one rank: NMX x NMY markers per basic
 * cell on the domain-wide lattice, each jittered by U(-mdx/4, mdx/4) x U(-mdy/4, mdy/4) from the
 * stream seeded with `seed` (the reference seeds 0).  Returns the number of markers placed
 * (-1 if more than cap). */
int64_t orc_distribute_uniform(const orc_ctx *c, mic_marker *mk, int64_t cap, int NMX, int NMY, unsigned long seed) {
  const double mdx = c->LX / (NMX * (c->NX - 1));
  const double mdy = c->LY / (NMY * (c->NY - 1));
  const int nxl = (int)((c->x[c->NX - 1] - c->x[0]) / mdx);
  const int nyl = (int)((c->y[c->NY - 1] - c->y[0]) / mdy);
  if ((int64_t)nxl * nyl > cap) return -1;
  uint64_t state = ((uint64_t)(seed & 0xFFFFFFFFUL) << 16) | 0x330EULL;
  int64_t idx = 0;
  for (int k = 0; k < nxl; ++k) {
    for (int l = 0; l < nyl; ++l) {
      double tmp = orc_rand48(&state, -mdx / 4.0, mdx / 4.0);
      mk[idx].X = c->x[0] + mdx * (0.5 + (double)k) + tmp;
      tmp = orc_rand48(&state, -mdy / 4.0, mdy / 4.0);
      mk[idx].Y = c->y[0] + mdy * (0.5 + (double)l) + tmp;
      ++idx;
    }
  }
  return idx;
}

/* ---- marker density control: checkMarkerDensity (markers.c:455-781) ------------------- */

/* the C library's drand48 recurrence on an explicit state (the stream the reference's
 * drand48() calls and its PETSCRAND48 object share) */
static double orc_drand48(uint64_t *state) {
  *state = (0x5DEECE66DULL * *state + 0xBULL) & 0xFFFFFFFFFFFFULL;
  return (double)*state / 281474976710656.0;
}

uint64_t orc_srand48_state(long seed) { return ((uint64_t)(seed & 0xFFFFFFFFL) << 16) | 0x330EULL; }

/* benchmarkInitialConditions.c:80-91, 124-134, 72-75 */
static double orc_plate_depth(double x, const mic_density_options *d) {
  if (fabs(x - d->rootCenter) < d->rootWidth)
    return d->overridingPlateThickness + d->rootThickness * pow(cos(M_PI * (x - d->rootCenter) / d->rootWidth / 2.0), 2.0);
  return d->overridingPlateThickness;
}
static double orc_slab_inflow_temperature(double x, double y, double angle, double age) {
  const double Ts = 273, T0 = 1623, kappa = 0.7272e-6, s_in_year = 3.15576e7;
  const double slab_age_s = age * 1.0e6 * s_in_year;
  return Ts + (T0 - Ts) * erf((y - x * tan(angle)) / (2.0 * sqrt(kappa * slab_age_s)));
}

/* new_slab_marker / new_inflow_marker (benchmarkInitialConditions.c:44-66) + findMarkerCell;
 * the reference leaves cpu and strainRateResidual of such markers uninitialised: 0 here */
static void orc_new_inflow_marker(const orc_ctx *c, mic_marker *p, double x, double y, double T) {
  memset(p, 0, sizeof(*p));
  orc_reset_markers(p, 1);
  p->X = x;
  p->Y = y;
  p->Mat = 0;
  p->T = T;
  double eta, mu;
  orc_compute_rheology(c, p, &eta, &mu);
  p->eta = eta;
  p->mu = mu;
  if (p->X >= 0.0 && p->Y >= 0.0 && p->X <= c->LX && p->Y <= c->LY) {
    p->cellX = bisect_cell(c->x, c->NX, p->X);
    p->cellY = bisect_cell(c->y, c->NY, p->Y);
  } else {
    p->cellX = p->cellY = -1;
  }
}

/* Returns the new marker count, or -1 where the reference aborts (a quarter cell that would
 * get a non-positive number of markers; more markers than cap), -2 for a removal from a
 * quarter cell with no marker inside its bounds.  *state is the drand48 stream. */
int64_t orc_check_marker_density(orc_ctx *c, mic_marker *mk, int64_t n, int64_t cap, const mic_density_options *d,
                                 uint64_t *state, int64_t *n_added, int64_t *n_removed) {
  const int NX = c->NX, NY = c->NY, m = NX - 1, nn = NY - 1;
  const int nq = 4 * m * nn;
  const int64_t nMark = n;
  int64_t *cnt = (int64_t *)calloc((size_t)nq, sizeof(int64_t));
  int64_t *isout = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  int64_t nOut = 0, ret = 0;
  *n_added = *n_removed = 0;
  for (int64_t m1 = 0; m1 < n; ++m1) {
    if (mk[m1].cellX != -1) {
      int cx = mk[m1].cellX, cy = mk[m1].cellY;
      cx = 2 * cx + (mk[m1].X >= c->xc[cx + 1] ? 1 : 0);
      cy = 2 * cy + (mk[m1].Y >= c->yc[cy + 1] ? 1 : 0);
      cnt[cx + cy * 2 * m] += 1;
    } else {
      isout[nOut++] = m1;
    }
  }
  int64_t maxQC = 0;
  for (int q = 0; q < nq; ++q)
    if (cnt[q] > maxQC) maxQC = cnt[q];
  int64_t nAdd = 0, nRemove = 0;
  for (int j = 0; j < 2 * nn; ++j) {
    for (int i = 0; i < 2 * m; ++i) {
      const int q = i + 2 * m * j;
      if (cnt[q] < d->minMarkers) {
        double dy = c->y[j / 2 + 1] - c->y[j / 2];
        double dx = c->x[i / 2 + 1] - c->x[i / 2];
        dx /= 2.0;
        dy /= 2.0;
        const int64_t mynmx = (int64_t)ceil(d->NMX * (NX - 1) / 2.0 * dx / c->LX);
        const int64_t mynmy = (int64_t)ceil(d->NMY * (NY - 1) / 2.0 * dy / c->LY);
        const int64_t mynadd = mynmx * mynmy - cnt[q];
        if (mynadd <= 0) {
          ret = -1;
          goto done;
        }
        nAdd += mynadd;
        cnt[q] = mynadd;
      } else if (cnt[q] > d->maxMarkers) {
        const int64_t t = cnt[q] - d->maxMarkers;
        nRemove += t;
        cnt[q] = -t;
      } else {
        cnt[q] = 0;
      }
    }
  }
  if (nRemove > 0) {
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(maxQC + 1));
    double *rnd = (double *)malloc(sizeof(double) * (size_t)(maxQC + 1));
    isout = (int64_t *)realloc(isout, sizeof(int64_t) * (size_t)(n + nRemove + 1));
    for (int j = 0; j < 2 * nn && ret == 0; ++j) {
      const double ymin = !(j % 2) ? c->y[j / 2] : c->yc[(j + 1) / 2];
      const double ymax = !(j % 2) ? c->yc[j / 2 + 1] : c->y[(j + 1) / 2];
      for (int i = 0; i < 2 * m; ++i) {
        const double xmin = !(i % 2) ? c->x[i / 2] : c->xc[(i + 1) / 2];
        const double xmax = !(i % 2) ? c->xc[i / 2 + 1] : c->x[(i + 1) / 2];
        const int q = 2 * m * j + i;
        if (cnt[q] >= 0) continue;
        const int64_t toRemove = -cnt[q];
        int64_t nCell = 0;
        for (int64_t im = 0; im < n; ++im)
          if (mk[im].X >= xmin && mk[im].X < xmax && mk[im].Y >= ymin && mk[im].Y < ymax) {
            if (nCell > maxQC) break;
            idx[nCell++] = im;
          }
        if (nCell == 0 || nCell > maxQC) {
          ret = -2;
          break;
        }
        for (int64_t k = 0; k < nCell; ++k) rnd[k] = orc_drand48(state);
        for (int64_t r = 0; r < toRemove; ++r) {
          double minv = 1.0;
          int64_t minidx = 0;
          for (int64_t k = 0; k < nCell; ++k)
            if (rnd[k] < minv) {
              minv = rnd[k];
              minidx = k;
            }
          rnd[minidx] = 1.0;
          mic_marker *p = &mk[idx[minidx]];
          p->X = -1.0;
          p->Y = -1.0;
          p->cellX = -1;
          p->cellY = -1;
          isout[nOut++] = idx[minidx];
        }
      }
    }
    free(idx);
    free(rnd);
    if (ret) goto done;
    *n_removed = nRemove;
  }
  if (nAdd > 0 && (nAdd + n - nOut) < cap) {
    double *nx = (double *)malloc(sizeof(double) * (size_t)nAdd), *ny = (double *)malloc(sizeof(double) * (size_t)nAdd);
    int64_t iMark = 0;
    for (int j = 0; j < 2 * nn; ++j) {
      for (int i = 0; i < 2 * m; ++i) {
        const int q = 2 * m * j + i;
        for (int64_t k = 0; k < cnt[q]; ++k) {
          const double xlo = !(i % 2) ? c->x[i / 2] : c->xc[(i + 1) / 2];
          const double xhi = !(i % 2) ? c->xc[i / 2 + 1] : c->x[(i + 1) / 2];
          nx[iMark] = xlo + (xhi - xlo) * orc_drand48(state);
          const double ylo = !(j % 2) ? c->y[j / 2] : c->yc[(j + 1) / 2];
          const double yhi = !(j % 2) ? c->yc[j / 2 + 1] : c->y[(j + 1) / 2];
          ny[iMark] = ylo + (yhi - ylo) * orc_drand48(state);
          ++iMark;
        }
      }
    }
    for (int64_t a = 0; a < nAdd; ++a) {
      int64_t id;
      if (nOut > 0) {
        id = isout[nOut - 1];
        nOut--;
      } else {
        id = n;
        n++;
      }
      if (nx[a] < c->x[1]) {
        orc_new_inflow_marker(c, &mk[id], nx[a], ny[a], orc_slab_inflow_temperature(nx[a], ny[a], d->slabAngle, d->slabAge));
      } else if (nx[a] >= c->x[NX - 2] && ny[a] >= orc_plate_depth(c->LX, d)) {
        orc_new_inflow_marker(c, &mk[id], nx[a], ny[a], 1573.0);
      } else {
        double mindist = c->LX * c->LY;
        int64_t minidx = -1;
        for (int64_t m1 = 0; m1 < nMark; ++m1) {
          if (m1 != id && mk[m1].cellX != -1) {
            if (fabs(mk[m1].X - nx[a]) <= (c->x[mk[m1].cellX + 1] - c->x[mk[m1].cellX]) &&
                fabs(mk[m1].Y - ny[a]) <= (c->y[mk[m1].cellY + 1] - c->y[mk[m1].cellY])) {
              const double x1 = mk[m1].X - nx[a], y1 = mk[m1].Y - ny[a];
              const double r1 = sqrt(x1 * x1 + y1 * y1);
              if (r1 < mindist) {
                mindist = r1;
                minidx = m1;
              }
            }
          }
        }
        if (minidx != -1) {
          mk[id] = mk[minidx];
          mk[id].X = nx[a];
          mk[id].Y = ny[a];
        }
      }
    }
    free(nx);
    free(ny);
    *n_added = nAdd;
  } else if ((nAdd + n - nOut) > cap) {
    ret = -1;
    goto done;
  }
  ret = n;
done:
  free(cnt);
  free(isout);
  return ret;
}

/* ---- grid routines between the solves ------------------------------------------------ */

#define NF(c, f, i, j) ((c)->nodal[f][(size_t)(j) * (size_t)(c)->NX + (size_t)(i)])

/* nodalStressStrain (nodalStressStrain.c:6-486), one rank, non-periodic x.  The reference's
 * vector operations (X = etaN ./ (etaN + dt muN) with the zero-divisor guard, X1 = etaN (2 - 2X),
 * s_new = X1 e + X s_old, ds = s_new - s_old) are restated elementwise in their order. */
void orc_nodal_stress_strain(orc_ctx *c, double dt) {
  const int NX = c->NX, NY = c->NY;
  double *exx = c->nodal[MIC_NF_EDOTXX], *eyy = c->nodal[MIC_NF_EDOTYY];
  for (int ix = 0; ix < NX; ++ix) {
    for (int jy = 0; jy < NY; ++jy) {
      const size_t k = (size_t)jy * NX + ix;
      if (ix == 0 || jy == 0) {
        exx[k] = 0.0;
        eyy[k] = 0.0;
      } else {
        const double dx = c->x[ix] - c->x[ix - 1];
        const double dy = c->y[jy] - c->y[jy - 1];
        const double divv = (NF(c, MIC_NF_VX, ix, jy - 1) - NF(c, MIC_NF_VX, ix - 1, jy - 1)) / dx +
                            (NF(c, MIC_NF_VY, ix - 1, jy) - NF(c, MIC_NF_VY, ix - 1, jy - 1)) / dy;
        exx[k] = (NF(c, MIC_NF_VX, ix, jy - 1) - NF(c, MIC_NF_VX, ix - 1, jy - 1)) / dx - divv / 3.0;
        eyy[k] = (NF(c, MIC_NF_VY, ix - 1, jy) - NF(c, MIC_NF_VY, ix - 1, jy - 1)) / dy - divv / 3.0;
      }
    }
  }
  const size_t nn = (size_t)NX * NY;
  for (size_t k = 0; k < nn; ++k) {  /* cell-centred stresses */
    const double eta = c->nodal[MIC_NF_ETAN][k], mu = c->nodal[MIC_NF_MUN][k];
    const double den = eta + dt * mu;
    const double X = den != 0.0 ? eta / den : 0.0;
    const double X1 = eta * (-2.0 * X + 2.0);
    const int so[2] = {MIC_NF_SOXX, MIC_NF_SOYY}, ds[2] = {MIC_NF_DSXX, MIC_NF_DSYY};
    const double *e[2] = {exx, eyy};
    for (int q = 0; q < 2; ++q) {
      const double et = X1 * e[q][k];
      double st = X * c->nodal[so[q]][k];
      st = st + 1.0 * et;
      c->nodal[ds[q]][k] = st + -1.0 * c->nodal[so[q]][k];
      c->nodal[so[q]][k] = st;
    }
  }
  for (int jy = 0; jy < NY; ++jy) {  /* basic nodes: vorticity and shear strain rate */
    for (int ix = 0; ix < NX; ++ix) {
      double vxm, vym, vxp, vyp;
      if (ix == 0)
        vym = (c->bcs.mechBCLeft.type[1] == 0) ? 2.0 * c->bcs.mechBCLeft.value[1] - NF(c, MIC_NF_VY, ix, jy)
                                               : NF(c, MIC_NF_VY, ix, jy);
      else
        vym = NF(c, MIC_NF_VY, ix - 1, jy);
      vyp = NF(c, MIC_NF_VY, ix, jy);
      if (jy == 0)
        vxm = (c->bcs.mechBCTop.type[0] == 0) ? 2.0 * c->bcs.mechBCTop.value[0] - NF(c, MIC_NF_VX, ix, jy)
                                              : NF(c, MIC_NF_VX, ix, jy);
      else
        vxm = NF(c, MIC_NF_VX, ix, jy - 1);
      vxp = NF(c, MIC_NF_VX, ix, jy);
      const double dx = c->xc[ix + 1] - c->xc[ix];
      const double dy = c->yc[jy + 1] - c->yc[jy];
      NF(c, MIC_NF_WXY, ix, jy) = 0.5 * ((vxp - vxm) / dy - (vyp - vym) / dx);
      NF(c, MIC_NF_EDOTXY, ix, jy) = 0.5 * ((vxp - vxm) / dy + (vyp - vym) / dx);
    }
  }
  for (size_t k = 0; k < nn; ++k) {  /* basic-node shear stress */
    const double eta = c->nodal[MIC_NF_ETAS][k], mu = c->nodal[MIC_NF_MUS][k];
    const double den = eta + dt * mu;
    const double X = den != 0.0 ? eta / den : 0.0;
    const double X1 = eta * (-2.0 * X + 2.0);
    const double et = X1 * c->nodal[MIC_NF_EDOTXY][k];
    double st = X * c->nodal[MIC_NF_SOXY][k];
    st = st + 1.0 * et;
    c->nodal[MIC_NF_DSXY][k] = st + -1.0 * c->nodal[MIC_NF_SOXY][k];
    c->nodal[MIC_NF_SOXY][k] = st;
  }
  double *hs_out = c->nodal[MIC_NF_HEATING], *eii = c->nodal[MIC_NF_EII], *sii = c->nodal[MIC_NF_SII];
  memset(hs_out, 0, sizeof(double) * nn);
  memset(eii, 0, sizeof(double) * nn);
  memset(sii, 0, sizeof(double) * nn);
  const double *sxx = c->nodal[MIC_NF_SOXX], *syy = c->nodal[MIC_NF_SOYY], *sxy = c->nodal[MIC_NF_SOXY];
  const double *eN = c->nodal[MIC_NF_ETAN], *eS = c->nodal[MIC_NF_ETAS], *exy = c->nodal[MIC_NF_EDOTXY];
  for (int jy = 1; jy < NY - 1; ++jy) {
    for (int ix = 1; ix < NX - 1; ++ix) {
      const size_t a = (size_t)jy * NX + ix, b = a + NX, r = a + 1, d = b + 1;
      double hs = (sxx[a] * sxx[a] / eN[a] + sxx[b] * sxx[b] / eN[b] + sxx[r] * sxx[r] / eN[r] + sxx[d] * sxx[d] / eN[d]) / 8.0;
      hs += (syy[a] * syy[a] / eN[a] + syy[b] * syy[b] / eN[b] + syy[r] * syy[r] / eN[r] + syy[d] * syy[d] / eN[d]) / 8.0;
      hs += sxy[a] * sxy[a] / eS[a];
      hs_out[a] += hs;
      eii[a] = sqrt((exx[a] * exx[a] + exx[b] * exx[b] + exx[r] * exx[r] + exx[d] * exx[d]) / 8.0 +
                    (eyy[a] * eyy[a] + eyy[b] * eyy[b] + eyy[r] * eyy[r] + eyy[d] * eyy[d]) / 8.0 + exy[a] * exy[a]);
      sii[a] = sqrt((sxx[a] * sxx[a] + sxx[b] * sxx[b] + sxx[r] * sxx[r] + sxx[d] * sxx[d]) / 8.0 +
                    (syy[a] * syy[a] + syy[b] * syy[b] + syy[r] * syy[r] + syy[d] * syy[d]) / 8.0 + sxy[a] * sxy[a]);
    }
  }
}

/* limitDisplacementTimestep (limitTimestep.c:6-133): the smallest of dt, factor times the
 * time to cross the smaller adjacent cell at each nodal vx / vy, 1% of rho / rhodot per node,
 * and 0.01 / max |rhodot| */
double orc_limit_displacement_timestep(const orc_ctx *c, double dt, double factor) {
  const int NX = c->NX, NY = c->NY;
  const double *vx = c->nodal[MIC_NF_VX], *vy = c->nodal[MIC_NF_VY];
  const double *rho = c->nodal[MIC_NF_RHO], *rhodot = c->nodal[MIC_NF_RHODOT];
  for (int ix = 0; ix < NX; ++ix) {
    for (int jy = 0; jy < NY; ++jy) {
      const size_t k = (size_t)jy * NX + ix;
      double dx, dy, dt1;
      const double dx1 = c->x[ix + 1] - c->x[ix], dx2 = c->x[ix] - c->x[ix - 1];
      if (ix == 0) dx = dx1;
      else if (ix == NX - 1) dx = dx2;
      else dx = (dx1 <= dx2) ? dx1 : dx2;
      dt1 = (vx[k] != 0.0) ? dx / (fabs(vx[k])) * factor : dt;
      if (dt > dt1) dt = dt1;
      const double dy1 = c->y[jy + 1] - c->y[jy], dy2 = c->y[jy] - c->y[jy - 1];
      if (jy == 0) dy = dy1;
      else if (jy == NY - 1) dy = dy2;
      else dy = (dy1 <= dy2) ? dy1 : dy2;
      dt1 = (vy[k] != 0.0) ? dy / (fabs(vy[k])) * factor : dt;
      if (dt > dt1) dt = dt1;
      if (rhodot[k] != 0.0) dt1 = fabs(0.01 * rho[k] / rhodot[k]);
      if (dt > dt1) dt = dt1;
    }
  }
  double mx = -INFINITY, mn = INFINITY;
  for (size_t k = 0; k < (size_t)NX * NY; ++k) {
    if (rhodot[k] > mx) mx = rhodot[k];
    if (rhodot[k] < mn) mn = rhodot[k];
  }
  mx = fabs(mx);
  mn = fabs(mn);
  if (mn > mx) mx = mn;
  if (mx * dt > 0.01) dt = 0.01 / mx;
  return dt;
}

/* retrieveSolutions (retrieveSolutions.c:4-82): vx, vy, p from S[(j NX + i) 3 + {0,1,2}],
 * pressure scaled by Kcont, minus the dx-weighted mean of row 1 (i >= 1) on every j, i >= 1 */
void orc_retrieve_solutions(orc_ctx *c, const double *S, double Kcont) {
  const int NX = c->NX, NY = c->NY;
  for (int j = 0; j < NY; ++j)
    for (int i = 0; i < NX; ++i) {
      const size_t k = (size_t)j * NX + i;
      c->nodal[MIC_NF_P][k] = S[3 * k + 2] * Kcont;
      c->nodal[MIC_NF_VX][k] = S[3 * k + 0];
      c->nodal[MIC_NF_VY][k] = S[3 * k + 1];
    }
  double pm = 0.0;
  for (int i = 1; i < NX; ++i) {
    const double dx = c->x[i] - c->x[i - 1];
    pm += NF(c, MIC_NF_P, i, 1) * dx / c->LX;
  }
  for (int j = 1; j < NY; ++j)
    for (int i = 1; i < NX; ++i) NF(c, MIC_NF_P, i, j) -= pm;
}

/* ---- marker checkpoint: saveMarkersBinary (io.c:299-402) / restartFromMarkers (restart.c:8-125) */

#include <stdio.h>

/* fields of the file after the header (int32 count, float64 elapsed time), each over the
 * in-domain markers in array order: kind 'i' int32, 'd' float64, at the given record offset */
typedef struct { char kind; int off; } orc_io_field;
static const orc_io_field ORC_IO_FIELDS[] = {
    {'i', offsetof(mic_marker, cpu)},   {'i', offsetof(mic_marker, cellX)}, {'i', offsetof(mic_marker, cellY)},
    {'d', offsetof(mic_marker, X)},     {'d', offsetof(mic_marker, Y)},     {'d', offsetof(mic_marker, VX)},
    {'d', offsetof(mic_marker, VY)},    {'i', offsetof(mic_marker, Mat)},   {'d', offsetof(mic_marker, T)},
    {'d', offsetof(mic_marker, Tdot)},  {'d', offsetof(mic_marker, eta)},   {'d', offsetof(mic_marker, mu)},
    {'d', offsetof(mic_marker, e.T11)}, {'d', offsetof(mic_marker, e.T12)}, {'d', offsetof(mic_marker, Eii)},
    {'d', offsetof(mic_marker, s.T11)}, {'d', offsetof(mic_marker, s.T22)}, {'d', offsetof(mic_marker, s.T12)},
    {'d', offsetof(mic_marker, p)},     {'d', offsetof(mic_marker, rho)},   {'d', offsetof(mic_marker, rhodot)}};
#define ORC_IO_NFIELDS ((int)(sizeof(ORC_IO_FIELDS) / sizeof(ORC_IO_FIELDS[0])))

int orc_save_markers_binary(const char *path, const mic_marker *mk, int64_t n, double elapsed) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  int32_t cnt = 0;
  for (int64_t m = 0; m < n; ++m) cnt += mk[m].cellX != -1;
  fwrite(&cnt, sizeof(int32_t), 1, f);
  fwrite(&elapsed, sizeof(double), 1, f);
  for (int k = 0; k < ORC_IO_NFIELDS; ++k)
    for (int64_t m = 0; m < n; ++m) {
      if (mk[m].cellX == -1) continue;
      const char *rec = (const char *)&mk[m] + ORC_IO_FIELDS[k].off;
      fwrite(rec, ORC_IO_FIELDS[k].kind == 'i' ? 4 : 8, 1, f);
    }
  return fclose(f) == 0 ? 0 : -1;
}

/* reads into mk (capacity cap, reset first as allocateMarkers does), then finds cells;
 * returns the marker count or -1 */
int64_t orc_restart_from_markers(orc_ctx *c, const char *path, mic_marker *mk, int64_t cap, double *elapsed) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  int32_t cnt = 0;
  if (fread(&cnt, sizeof(int32_t), 1, f) != 1 || fread(elapsed, sizeof(double), 1, f) != 1 || cnt < 0 || cnt > cap) {
    fclose(f);
    return -1;
  }
  orc_reset_markers(mk, cap);
  for (int k = 0; k < ORC_IO_NFIELDS; ++k)
    for (int32_t m = 0; m < cnt; ++m) {
      char *rec = (char *)&mk[m] + ORC_IO_FIELDS[k].off;
      if (fread(rec, ORC_IO_FIELDS[k].kind == 'i' ? 4 : 8, 1, f) != 1) {
        fclose(f);
        return -1;
      }
    }
  fclose(f);
  int err = 0;
  orc_find_marker_cells(c, mk, cnt, &err);
  return err ? -1 : cnt;
}

/* projectMarkersNodesFromScalar (markers.c:1507-1594): a per-marker array (caller order)
 * projected bilinearly onto the basic nodes of each marker's cell, divided by the weights
 * (zero where no marker contributes) */
int orc_project_from_scalar(orc_ctx *c, const mic_marker *mk, int64_t n, const double *v, int field) {
  if (field < 0 || field >= MIC_NF_COUNT) return ORC_ERR_ARG;
  const int NX = c->NX;
  const size_t nn = (size_t)c->NX * c->NY;
  double *nf = (double *)calloc(nn, sizeof(double)), *wt = (double *)calloc(nn, sizeof(double));
  for (int64_t m = 0; m < n; ++m) {
    const mic_marker *p = &mk[m];
    if (p->cellX == -1) continue;
    const int i = p->cellX, j = p->cellY;
    const double dx = c->x[i + 1] - c->x[i], dy = c->y[j + 1] - c->y[j];
    const double mdx = (p->X - c->x[i]) / dx, mdy = (p->Y - c->y[j]) / dy;
    const size_t k00 = (size_t)j * NX + i;
    double w = (1.0 - mdx) * (1.0 - mdy);
    wt[k00] += w;
    nf[k00] += w * v[m];
    w = mdx * (1.0 - mdy);
    wt[k00 + 1] += w;
    nf[k00 + 1] += w * v[m];
    w = (1.0 - mdx) * mdy;
    wt[k00 + NX] += w;
    nf[k00 + NX] += w * v[m];
    w = mdx * mdy;
    wt[k00 + NX + 1] += w;
    nf[k00 + NX + 1] += w * v[m];
  }
  double *out = c->nodal[field];
  for (size_t k = 0; k < nn; ++k) {
    const double w = 0.0 + wt[k];
    out[k] = (w != 0.0) ? (0.0 + nf[k]) / w : 0.0;
  }
  free(nf);
  free(wt);
  return ORC_OK;
}
