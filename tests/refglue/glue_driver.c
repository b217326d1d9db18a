/*
 * glue_driver.c -- drives the reference-side binding (fvmic2d_gb300/refglue/fvmic2d_glue.c) the
 * way fvmic2d's main() would, through the routines' own names and signatures, on a grid, a
 * MarkerSet and PETSc Vecs built with the single-rank petsc_lite stand-in.  TEST INFRASTRUCTURE
 * ONLY: tests/refglue/gluepy.py loads it with ctypes; the calls mirror oracle/ref_bridge.c, which
 * drives the reference's own routines the same way.
 */
#include <math.h>
#include <string.h>

#include "fdcode.h"
#include "markerProjection.h"
#include "markers.h"
#include "residual.h"
#include "subgridStressChanges.h"
#include "subgridTemperatureChanges.h"
#include "updateMarkerStrainPressure.h"
#include "updateMarkerStress.h"
#include "viscosity.h"

#include "fvmic2d_glue.h"
#include "mic_types.h"

typedef struct {
  GridData grid;
  NodalFields nf;
  Materials mat;
  Options opt;
  BoundaryValues bv;
  MarkerSet ms;
  Vec thisT;
  double *gbuf;
} gdrv;

static Vec *field_vec(gdrv *p, int id) {
  switch (id) {
    case MIC_NF_RHO: return &p->nf.rho;
    case MIC_NF_RHODOT: return &p->nf.rhodot;
    case MIC_NF_ETAS: return &p->nf.etaS;
    case MIC_NF_ETAN: return &p->nf.etaN;
    case MIC_NF_THIST: return &p->thisT;
    case MIC_NF_LASTT: return &p->nf.lastT;
    case MIC_NF_KTHERMAL: return &p->nf.kThermal;
    case MIC_NF_CP: return &p->nf.Cp;
    case MIC_NF_EDOTXX: return &p->nf.edotxx;
    case MIC_NF_EDOTXY: return &p->nf.edotxy;
    case MIC_NF_EDOTYY: return &p->nf.edotyy;
    case MIC_NF_SOXX: return &p->nf.soxx;
    case MIC_NF_SOXY: return &p->nf.soxy;
    case MIC_NF_SOYY: return &p->nf.soyy;
    case MIC_NF_DSXX: return &p->nf.dsxx;
    case MIC_NF_DSYY: return &p->nf.dsyy;
    case MIC_NF_DSXY: return &p->nf.dsxy;
    case MIC_NF_MUS: return &p->nf.muS;
    case MIC_NF_MUN: return &p->nf.muN;
    case MIC_NF_VX: return &p->nf.vx;
    case MIC_NF_VY: return &p->nf.vy;
    case MIC_NF_P: return &p->nf.p;
    case MIC_NF_WXY: return &p->nf.wxy;
    case MIC_NF_SRR: return &p->nf.strainRateResidual;
    case MIC_NF_EII: return &p->nf.eii;
    case MIC_NF_SII: return &p->nf.sii;
    case MIC_NF_HEATING: return &p->nf.nodalHeating;
    default: return NULL;
  }
}

/* x[NX], y[NY]: basic gridlines, stored with two ghost entries on each side like fvmic2d's grid
 * arrays; cap: the marker set's capacity (allocateMarkers) */
gdrv *gd_create(int NX, int NY, double LX, double LY, const double *x, const double *y, int cap) {
  gdrv *p = (gdrv *)calloc(1, sizeof(gdrv));
  if (!p) return NULL;
  const size_t nx4 = (size_t)NX + 4, ny4 = (size_t)NY + 4;
  p->gbuf = (double *)malloc((2 * nx4 + 2 * ny4) * sizeof(double));
  for (size_t i = 0; i < 2 * nx4 + 2 * ny4; ++i) p->gbuf[i] = NAN;
  p->grid.x = p->gbuf + 2;
  p->grid.xc = p->gbuf + nx4 + 2;
  p->grid.y = p->gbuf + 2 * nx4 + 2;
  p->grid.yc = p->gbuf + 2 * nx4 + ny4 + 2;
  for (int i = 0; i < NX; ++i) p->grid.x[i] = x[i];
  for (int j = 0; j < NY; ++j) p->grid.y[j] = y[j];
  p->grid.NX = NX;
  p->grid.NY = NY;
  p->grid.LX = LX;
  p->grid.LY = LY;
  plite_DMDACreate(NX, NY, &p->grid.da);
  plite_DMDACreateDOF(NX, NY, 3, &p->grid.vda);
  for (int id = 0; id < MIC_NF_COUNT; ++id) DMCreateGlobalVector(p->grid.da, field_vec(p, id));
  if (allocateMarkers(cap, &p->ms, &p->opt)) {
    free(p->gbuf);
    free(p);
    return NULL;
  }
  p->ms.nMark = 0;
  return p;
}

void gd_destroy(gdrv *p) {
  if (!p) return;
  destroyMarkers(&p->ms, &p->opt);
  for (int id = 0; id < MIC_NF_COUNT; ++id) VecDestroy(field_vec(p, id));
  plite_DMDestroy(&p->grid.da);
  plite_DMDestroy(&p->grid.vda);
  free(p->gbuf);
  free(p);
}

void gd_set_materials(gdrv *p, const mic_materials *m) { memcpy(&p->mat, m, sizeof(Materials)); }
void gd_set_bcs(gdrv *p, const mic_bcs *b) { memcpy(&p->bv, b, sizeof(BoundaryValues)); }
void gd_set_options(gdrv *p, const mic_options *o) {
  p->opt.etamin = o->etamin;
  p->opt.etamax = o->etamax;
  p->opt.fractionalEtamin = o->fractionalEtamin;
  p->opt.subgridStressDiffusivity = o->subgridStressDiffusivity;
  p->opt.subgridTemperatureDiffusivity = o->subgridTemperatureDiffusivity;
  p->opt.slabAngle = o->slabAngle;
  p->opt.decoupleThickness = o->decoupleThickness;
  p->opt.minDecoupleDepth = o->minDecoupleDepth;
  p->opt.maxDecoupleDepth = o->maxDecoupleDepth;
  p->opt.decoupleEtaScaler = o->decoupleEtaScaler;
}

/* host code writing the marker array, as fvmic2d's initial conditions do: current copy to the
 * host first (micMarkersToHost), then the write */
int gd_set_markers(gdrv *p, const mic_marker *m, int n) {
  if (n > p->ms.maxMark) return -1;
  if (micMarkersToHost(&p->ms)) return -2;
  memcpy(p->ms.markers, m, sizeof(Marker) * (size_t)n);
  p->ms.nMark = n;
  return 0;
}

int gd_get_markers(gdrv *p, mic_marker *out, int max) {
  if (micMarkersToHost(&p->ms)) return -2;
  const int n = p->ms.nMark < max ? p->ms.nMark : max;
  memcpy(out, p->ms.markers, sizeof(Marker) * (size_t)n);
  return p->ms.nMark;
}

int gd_marker_count(gdrv *p) { return p->ms.nMark; }

int gd_set_nodal(gdrv *p, int id, const double *v) {
  Vec *f = field_vec(p, id);
  if (!f) return 1;
  PetscScalar *a;
  VecGetArray(*f, &a);
  memcpy(a, v, sizeof(double) * (size_t)p->grid.NX * (size_t)p->grid.NY);
  VecRestoreArray(*f, &a);
  return 0;
}

int gd_get_nodal(gdrv *p, int id, double *v) {
  Vec *f = field_vec(p, id);
  if (!f) return 1;
  PetscScalar *a;
  VecGetArray(*f, &a);
  memcpy(v, a, sizeof(double) * (size_t)p->grid.NX * (size_t)p->grid.NY);
  VecRestoreArray(*f, &a);
  return 0;
}

int gd_last_error(void) { return micGlueLastError(); }

void gd_resetMarkers(gdrv *p) { resetMarkers(&p->ms, &p->opt); }

int gd_distributeMarkersUniformInDomain(gdrv *p, int NMX, int NMY) {
  p->opt.NMX = NMX;
  p->opt.NMY = NMY;
  if (distributeMarkersUniformInDomain(&p->ms, &p->opt, &p->grid)) return -1;
  return p->ms.nMark;
}

int gd_findMarkerCells(gdrv *p) {
  findMarkerCells(&p->ms, &p->grid);
  return p->ms.nOut;
}

int gd_updateMarkerRho(gdrv *p) { return micUpdateMarkerRho(&p->ms, &p->mat); }
double gd_maxMarkerT(gdrv *p) { return micMaxMarkerT(&p->ms); }
double gd_maxAbsSxx(gdrv *p) { return micMaxAbsSxx(&p->ms); }

int gd_projectMarkersNodesAll2(gdrv *p) { return projectMarkersNodesAll2(&p->ms, &p->grid, &p->nf, &p->mat, &p->opt); }

/* field_offset: byte offset of a double inside Marker, or -1 with matprop != NULL */
int gd_projectMarkerFieldToNodes(gdrv *p, int field_offset, double *matprop, int out_id, int stagx, int stagy,
                                 int method) {
  PetscScalar *mf = NULL;
  if (field_offset >= 0) mf = (PetscScalar *)((char *)p->ms.markers + field_offset);
  return projectMarkerFieldToNodes(&p->grid, &p->ms, matprop, mf, *field_vec(p, out_id), stagx, stagy,
                                   (PROJECTION_METHOD)method);
}

int gd_projectNodalFieldToMarkersS(gdrv *p, int nodal_id, int field_offset) {
  return projectNodalFieldToMarkersS(&p->nf, *field_vec(p, nodal_id), &p->ms,
                                     (PetscScalar *)((char *)p->ms.markers + field_offset), &p->grid);
}

int gd_projectMarkersNodesFromScalar(gdrv *p, double *values, int out_id) {
  return projectMarkersNodesFromScalar(&p->ms, &p->grid, values, *field_vec(p, out_id));
}

int gd_checkPlasticYielding(gdrv *p, double dt, double t) {
  PetscInt isYielding = 0;
  if (checkPlasticYielding(&p->grid, &p->ms, &p->mat, dt, &isYielding, &p->opt, t)) return -1;
  return isYielding;
}

void gd_limitViscosity(gdrv *p) { limitViscosity(&p->ms, &p->opt, &p->mat); }
void gd_updateViscosity(gdrv *p) { updateViscosity(&p->ms, &p->opt, &p->mat); }

int gd_updateMarkerStrainPressure(gdrv *p, double dt) {
  return updateMarkerStrainPressure(&p->grid, &p->nf, &p->ms, &p->mat, &p->opt, dt);
}

double gd_updateGlobalStrainRateResidual(gdrv *p, int iter) {
  updateGlobalStrainRateResidual(&p->grid, &p->ms, iter);
  return getGlobalStrainRateResidual(iter);
}

void gd_setGlobalStrainRateResidual(int iter, double v) { setGlobalStrainRateResidual(iter, v); }
int gd_checkConvergence(double atol, double rtol, int iter) { return checkConvergence(atol, rtol, iter); }

int gd_subgridStressChanges(gdrv *p, double dt, double D) {
  return subgridStressChanges(&p->grid, &p->nf, &p->ms, &p->mat, dt, D);
}

int gd_updateMarkerStress(gdrv *p) { return updateMarkerStress(&p->grid, &p->nf, &p->ms, &p->mat); }

int gd_subgridTemperatureChanges(gdrv *p, double dt) {
  return subgridTemperatureChanges(p->thisT, &p->grid, &p->nf, &p->ms, &p->mat, dt, &p->opt);
}

int gd_advectMarkersRK(gdrv *p, double dt) { return advectMarkersRK(&p->ms, &p->nf, &p->grid, &p->opt, &p->bv, dt); }

/* checkMarkerDensity with the density-control settings (the Options fields it reads) */
int gd_checkMarkerDensity(gdrv *p, const mic_density_options *d) {
  static Problem prob;
  memset(&prob, 0, sizeof(prob));
  prob.materials = p->mat;
  p->opt.NMX = d->NMX;
  p->opt.NMY = d->NMY;
  p->opt.minMarkers = d->minMarkers;
  p->opt.maxMarkers = d->maxMarkers;
  p->opt.slabAngle = d->slabAngle;
  p->opt.slabAge = d->slabAge;
  p->opt.overridingPlateThickness = d->overridingPlateThickness;
  p->opt.rootThickness = d->rootThickness;
  p->opt.rootCenter = d->rootCenter;
  p->opt.rootWidth = d->rootWidth;
  if (checkMarkerDensity(&prob, &p->ms, &p->grid, &p->opt, NULL)) return -1;
  return p->ms.nMark;
}
