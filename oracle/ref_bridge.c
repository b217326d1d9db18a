/*
 * ref_bridge.c -- ctypes-friendly wrappers that drive fvmic2d's OWN hot-path
 * functions (compiled unmodified from the reference tree against petsc_lite)
 * on caller-provided grids, markers and nodal fields.
 *
 * TEST INFRASTRUCTURE ONLY.  It is linked into oracle/_ref/libfvmic2d_ref.so
 * by oracle/build_ref.sh; the library is used to pin the project's C
 * restatement (oracle/mic_oracle.c) and to generate golden vectors.
 *
 * Nothing here re-implements reference arithmetic except the three marker
 * loops that live inline in main_subduction.c (density update, main:255-264;
 * maximum temperature, main:271-289; maximum |sxx|, main:437-448), restated as
 * small loops because main() itself cannot be linked.
 */
#include "fdcode.h"
#include "markers.h"
#include "markerProjection.h"
#include "viscosity.h"
#include "updateMarkerStrainPressure.h"
#include "subgridStressChanges.h"
#include "updateMarkerStress.h"
#include "subgridTemperatureChanges.h"
#include "residual.h"
#include "profile.h"
#include "gridSpacing.h"
#include "nodalStressStrain.h"
#include "limitTimestep.h"
#include "retrieveSolutions.h"
#include "io.h"
#include "restart.h"
#include "vep_system.h"
#include "adiabaticHeating.h"
#include "post.h"
#include "thermalSystem.h"
#include "mic_types.h"

PetscErrorCode plite_DMDACreate(PetscInt NX, PetscInt NY, DM *da);
PetscErrorCode plite_DMDestroy(DM *da);
PetscScalar goldsbyKohlstedt(PetscScalar, PetscScalar, PetscScalar, PetscScalar);

_Static_assert(sizeof(Marker) == sizeof(mic_marker), "marker layout");
_Static_assert(offsetof(Marker, cellX) == offsetof(mic_marker, cellX), "marker layout");
_Static_assert(offsetof(Marker, isYielding) == offsetof(mic_marker, isYielding), "marker layout");
_Static_assert(sizeof(Materials) == sizeof(mic_materials), "materials layout");
_Static_assert(offsetof(Materials, Tref) == offsetof(mic_materials, Tref), "materials layout");
_Static_assert(sizeof(BoundaryValues) == sizeof(mic_bcs), "bc layout");

typedef struct {
  GridData grid;
  NodalFields nf;
  Materials mat;
  Options opt;
  BoundaryValues bv;
  MarkerSet ms;
  Vec thisT;
  Vec srr;
  Vec heat;
  double *gbuf;
} refp;

static int g_logging = 0;

static Vec *field_vec(refp *p, int id) {
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
    case MIC_NF_SRR: return &p->srr;
    case MIC_NF_EII: return &p->nf.eii;
    case MIC_NF_SII: return &p->nf.sii;
    case MIC_NF_HEATING: return &p->heat;
    default: return NULL;
  }
}

/* x[NX], y[NY]: basic gridlines.  Cell centres follow getCellCenters (gridSpacing.c:150-157).
 * Ghost entries that the reference leaves uninitialised are set to NaN so that any read shows. */
refp *ref_create(int NX, int NY, double LX, double LY, const double *x, const double *y) {
  if (!g_logging) {
    initializeLogging();
    g_logging = 1;
  }
  refp *p = (refp *)calloc(1, sizeof(refp));
  if (!p) return NULL;
  size_t nx4 = (size_t)NX + 4, ny4 = (size_t)NY + 4;
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
  p->grid.xperiodic = 0;
  p->grid.yperiodic = 0;
  getCellCenters(p->grid.x, p->grid.xc, LX, NX);
  getCellCenters(p->grid.y, p->grid.yc, LY, NY);
  plite_DMDACreate(NX, NY, &p->grid.da);
  plite_DMDACreateDOF(NX, NY, 3, &p->grid.vda);
  for (int id = 0; id < MIC_NF_COUNT; ++id) DMCreateGlobalVector(p->grid.da, field_vec(p, id));
  DMCreateGlobalVector(p->grid.da, &p->nf.ha);
  return p;
}

/* periodic x (gridGenerator.c:67-68, 82-84 and 97-110; nodalFields.c:11-19): the gridlines and
 * cell centres through the reference's own makePeriodic (gridSpacing.c:159-168), both DMDAs
 * periodic in x.  The caller's x holds NX uniform lines of the NX+1 from 0 to LX. */
void ref_set_periodic_x(refp *p) {
  p->grid.xperiodic = 1;
  makePeriodic(p->grid.x, p->grid.xc, p->grid.LX, p->grid.NX);
  plite_DMDASetPeriodicX(p->grid.da, 1);
  plite_DMDASetPeriodicX(p->grid.vda, 1);
}

void ref_destroy(refp *p) {
  if (!p) return;
  for (int id = 0; id < MIC_NF_COUNT; ++id) VecDestroy(field_vec(p, id));
  VecDestroy(&p->nf.ha);
  plite_DMDestroy(&p->grid.da);
  plite_DMDestroy(&p->grid.vda);
  free(p->gbuf);
  free(p);
}

void ref_get_grid(refp *p, double *xc, double *yc) {
  for (int i = 0; i <= p->grid.NX; ++i) xc[i] = p->grid.xc[i];  /* periodic: xc[NX] from makePeriodic */
  for (int j = 0; j <= p->grid.NY; ++j) yc[j] = p->grid.yc[j];
}

void ref_set_materials(refp *p, const mic_materials *m) { memcpy(&p->mat, m, sizeof(Materials)); }
void ref_set_bcs(refp *p, const mic_bcs *b) { memcpy(&p->bv, b, sizeof(BoundaryValues)); }
void ref_set_options(refp *p, const mic_options *o) {
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

/* markers stay owned by the caller (a numpy structured array with the Marker layout) */
void ref_set_markers(refp *p, mic_marker *m, int n) {
  p->ms.markers = (Marker *)m;
  p->ms.nMark = n;
  p->ms.maxMark = n;
  p->ms.nOut = 0;
}

int ref_set_nodal(refp *p, int id, const double *v) {
  Vec *f = field_vec(p, id);
  if (!f) return 1;
  PetscScalar *a;
  VecGetArray(*f, &a);
  memcpy(a, v, sizeof(double) * (size_t)p->grid.NX * (size_t)p->grid.NY);
  return 0;
}

int ref_get_nodal(refp *p, int id, double *v) {
  Vec *f = field_vec(p, id);
  if (!f) return 1;
  PetscScalar *a;
  VecGetArray(*f, &a);
  memcpy(v, a, sizeof(double) * (size_t)p->grid.NX * (size_t)p->grid.NY);
  return 0;
}

int ref_findMarkerCells(refp *p) {
  findMarkerCells(&p->ms, &p->grid);
  return p->ms.nOut;
}

/* main_subduction.c:255-264 */
void ref_updateMarkerRho(refp *p) {
  Marker *mk = p->ms.markers;
  for (int m = 0; m < p->ms.nMark; ++m) {
    if (mk[m].cellX != -1) {
      mk[m].rho = -p->mat.materialRho[mk[m].Mat] * (p->mat.materialAlpha[mk[m].Mat] * mk[m].T);
      mk[m].rhodot = 0.0;
    }
  }
}

/* main_subduction.c:271-281 */
double ref_maxMarkerT(refp *p) {
  double maxT = 0.0;
  Marker *mk = p->ms.markers;
  for (int m = 0; m < p->ms.nMark; ++m)
    if (mk[m].cellX != -1 && mk[m].T > maxT) maxT = mk[m].T;
  return maxT;
}

/* main_subduction.c:437-448 */
double ref_maxAbsSxx(refp *p) {
  double sxxmax = 0.0;
  Marker *mk = p->ms.markers;
  for (int m = 0; m < p->ms.nMark; ++m)
    if (mk[m].cellX != -1 && fabs(mk[m].s.T11) > sxxmax) sxxmax = fabs(mk[m].s.T11);
  return sxxmax;
}

int ref_projectMarkersNodesAll2(refp *p) {
  return projectMarkersNodesAll2(&p->ms, &p->grid, &p->nf, &p->mat, &p->opt);
}

/* field_offset: byte offset of a double inside Marker, or -1 with matprop != NULL */
int ref_projectMarkerFieldToNodes(refp *p, int field_offset, double *matprop, int out_id, int stagx, int stagy,
                                  int method) {
  PetscScalar *mf = NULL;
  if (field_offset >= 0) mf = (PetscScalar *)((char *)p->ms.markers + field_offset);
  return projectMarkerFieldToNodes(&p->grid, &p->ms, matprop, mf, *field_vec(p, out_id), stagx, stagy,
                                   (PROJECTION_METHOD)method);
}

int ref_projectNodalFieldToMarkersS(refp *p, int nodal_id, int field_offset) {
  return projectNodalFieldToMarkersS(&p->nf, *field_vec(p, nodal_id), &p->ms,
                                     (PetscScalar *)((char *)p->ms.markers + field_offset), &p->grid);
}

int ref_checkPlasticYielding(refp *p, double dt, double t) {
  PetscInt isYielding = 0;
  checkPlasticYielding(&p->grid, &p->ms, &p->mat, dt, &isYielding, &p->opt, t);
  return isYielding;
}

void ref_limitViscosity(refp *p) { limitViscosity(&p->ms, &p->opt, &p->mat); }
void ref_updateViscosity(refp *p) { updateViscosity(&p->ms, &p->opt, &p->mat); }

int ref_updateMarkerStrainPressure(refp *p, double dt) {
  return updateMarkerStrainPressure(&p->grid, &p->nf, &p->ms, &p->mat, &p->opt, dt);
}

double ref_updateGlobalStrainRateResidual(refp *p, int iter) {
  updateGlobalStrainRateResidual(&p->grid, &p->ms, iter);
  return getGlobalStrainRateResidual(iter);
}

int ref_checkConvergence(double atol, double rtol, int iter) { return checkConvergence(atol, rtol, iter); }

int ref_subgridStressChanges(refp *p, double dt, double D) {
  return subgridStressChanges(&p->grid, &p->nf, &p->ms, &p->mat, dt, D);
}

int ref_updateMarkerStress(refp *p) { return updateMarkerStress(&p->grid, &p->nf, &p->ms, &p->mat); }

int ref_subgridTemperatureChanges(refp *p, double dt) {
  return subgridTemperatureChanges(p->thisT, &p->grid, &p->nf, &p->ms, &p->mat, dt, &p->opt);
}

int ref_advectMarkersRK(refp *p, double dt) { return advectMarkersRK(&p->ms, &p->nf, &p->grid, &p->opt, &p->bv, dt); }

double ref_goldsbyKohlstedt(double s, double T, double d, double P) { return goldsbyKohlstedt(s, T, d, P); }

void ref_goldsbyKohlstedt_many(const double *s, const double *T, const double *d, const double *P, double *eta, int n) {
  for (int i = 0; i < n; ++i) eta[i] = goldsbyKohlstedt(s[i], T[i], d[i], P[i]);
}

/* Per-stage CPU time, profile.h:5-22 numbering. */
double ref_stage_seconds(int stage) {
  extern double plite_stage_seconds(int);
  return plite_stage_seconds(stage);
}
void ref_stage_reset(void) {
  extern void plite_stage_reset(void);
  plite_stage_reset();
}

/* resetMarkers + distributeMarkersUniformInDomain (markers.c:332-400) on a caller-owned array of
 * capacity cap; returns the reference's nMark.  The PETSc random stream is the stand-in's. */
int ref_resetMarkers(refp *p, mic_marker *m, int cap) {
  p->ms.markers = (Marker *)m;
  p->ms.maxMark = cap;
  resetMarkers(&p->ms, &p->opt);
  return 0;
}

int ref_distributeMarkersUniformInDomain(refp *p, mic_marker *m, int cap, int NMX, int NMY) {
  p->ms.markers = (Marker *)m;
  p->ms.maxMark = cap;
  p->opt.NMX = NMX;
  p->opt.NMY = NMY;
  if (distributeMarkersUniformInDomain(&p->ms, &p->opt, &p->grid)) return -1;
  return p->ms.nMark;
}

/* checkMarkerDensity (markers.c:455-781) on the caller's marker array (capacity cap, nMark
 * markers, cells current).  The PETSc random object is the reference's (PETSCRAND48, seeded
 * with srand48(seed) before the call when seed >= 0; seed < 0 continues the current global
 * drand48 stream).  Returns the new nMark; *rng_state receives the drand48 state afterwards. */
int ref_checkMarkerDensity(refp *p, mic_marker *m, int n, int cap, int NMX, int NMY, int minMarkers,
                           int maxMarkers, const double *slab, long seed, unsigned short *rng_state) {
  p->ms.markers = (Marker *)m;
  p->ms.nMark = n;
  p->ms.maxMark = cap;
  p->opt.NMX = NMX;
  p->opt.NMY = NMY;
  p->opt.minMarkers = minMarkers;
  p->opt.maxMarkers = maxMarkers;
  /* slab: slabAngle, slabAge, overridingPlateThickness, rootThickness, rootCenter, rootWidth */
  p->opt.slabAngle = slab[0];
  p->opt.slabAge = slab[1];
  p->opt.overridingPlateThickness = slab[2];
  p->opt.rootThickness = slab[3];
  p->opt.rootCenter = slab[4];
  p->opt.rootWidth = slab[5];
  static Problem prob;
  memset(&prob, 0, sizeof(prob));
  prob.materials = p->mat;
  PetscRandom r;
  PetscRandomCreate(PETSC_COMM_WORLD, &r);
  PetscRandomSetType(r, PETSCRAND48);
  if (seed >= 0) {
    PetscRandomSetSeed(r, (unsigned long)seed);
    PetscRandomSeed(r);
  }
  int e = checkMarkerDensity(&prob, &p->ms, &p->grid, &p->opt, r);
  PetscRandomDestroy(&r);
  if (rng_state) {
    unsigned short *st = seed48((unsigned short[3]){0, 0, 0}); /* read the state back ... */
    rng_state[0] = st[0];
    rng_state[1] = st[1];
    rng_state[2] = st[2];
    seed48(rng_state); /* ... and restore it */
  }
  if (e) return -1;
  return p->ms.nMark;
}

/* nodalStressStrain (nodalStressStrain.c:6): new nodal strain rates, vorticity, stresses and
 * stress changes from vx, vy, etaN/S, muN/S, soxx/yy/xy; shear heating into MIC_NF_HEATING */
int ref_nodalStressStrain(refp *p, double dt, double gy) {
  return nodalStressStrain(&p->grid, &p->nf, &p->opt, &p->bv, dt, p->heat, gy);
}

/* limitDisplacementTimestep (limitTimestep.c:6) starting from dt */
double ref_limitDisplacementTimestep(refp *p, double dt, double factor) {
  p->opt.displacementStepLimit = factor;
  PetscScalar d = dt;
  limitDisplacementTimestep(&p->grid, &p->nf, &d, &p->opt);
  return d;
}

/* retrieveSolutions (retrieveSolutions.c:4) from a solution vector S[(j NX + i) 3 + dof]
 * (copied; the reference scales the pressure entries of S in place) */
int ref_retrieveSolutions(refp *p, const double *S, double Kcont) {
  Vec v;
  DMCreateGlobalVector(p->grid.vda, &v);
  PetscScalar *a;
  VecGetArray(v, &a);
  memcpy(a, S, sizeof(double) * 3 * (size_t)p->grid.NX * (size_t)p->grid.NY);
  PetscInt nan = 0;
  int e = retrieveSolutions(&p->grid, &p->nf, v, Kcont, &nan);
  VecDestroy(&v);
  return e ? -1 : nan;
}

/* saveMarkersBinary (io.c:299) of the caller's markers: writes output/Markers.<iMonte>.<iTime>
 * under the current directory; nOut from the markers' cells */
int ref_saveMarkersBinary(refp *p, mic_marker *m, int n, int iMonte, int iTime, double elapsed) {
  p->ms.markers = (Marker *)m;
  p->ms.nMark = n;
  p->ms.maxMark = n;
  int nout = 0;
  for (int k = 0; k < n; ++k) nout += m[k].cellX == -1;
  p->ms.nOut = nout;
  return saveMarkersBinary(&p->ms, iMonte, iTime, elapsed);
}

/* restartFromMarkers (restart.c:8): reads output/Markers.<iMonte>.<iTime>, allocates with
 * maxMarkFactor, bins; copies up to cap markers out; returns nMark (or -1) */
int ref_restartFromMarkers(refp *p, int iMonte, int iTime, double maxMarkFactor, mic_marker *out, int cap,
                           double *elapsed) {
  MarkerSet ms;
  memset(&ms, 0, sizeof(ms));
  p->opt.maxMarkFactor = maxMarkFactor;
  PetscScalar t = 0.0;
  if (restartFromMarkers(&ms, &p->grid, &p->mat, &p->opt, iMonte, iTime, &t)) return -1;
  *elapsed = t;
  const int n = ms.nMark < cap ? ms.nMark : cap;
  memcpy(out, ms.markers, sizeof(Marker) * (size_t)n);
  const int total = ms.nMark;
  free(ms.markers);
  return total;
}

/* projectMarkersNodesFromScalar (markers.c:1507) of a per-marker array into a nodal field */
int ref_projectMarkersNodesFromScalar(refp *p, double *values, int out_id) {
  Vec *f = field_vec(p, out_id);
  if (!f) return -1;
  return projectMarkersNodesFromScalar(&p->ms, &p->grid, values, *f);
}

/* ---- the two linear systems (vep_system.c:12, formThermalSystem.c:6, enforceThermalBC.c:5) ---- */

PetscErrorCode plite_DMDACreateDOF(PetscInt NX, PetscInt NY, PetscInt dof, DM *da);

static void set_subduction(refp *p, const mic_subduction_options *so) {
  p->opt.gx = so->gx;
  p->opt.gy = so->gy;
  p->opt.slabVelocity = so->slabVelocity;
  p->opt.slabAngle = so->slabAngle;
  p->opt.slabAge = so->slabAge;
  p->opt.overridingPlateThickness = so->overridingPlateThickness;
  p->opt.rootThickness = so->rootThickness;
  p->opt.rootCenter = so->rootCenter;
  p->opt.rootWidth = so->rootWidth;
  p->opt.thermalBCTop.type[0] = so->thermalBCTopType;
  p->opt.thermalBCTop.value[0] = so->thermalBCTopValue;
}

typedef struct {
  PetscInt n, nnz;
  PetscInt *rowptr, *cols;
  PetscScalar *vals, *rhs;
} ref_system;

static ref_system g_sys[2];  /* 0: Stokes, 1: thermal (the last assembly of each) */

static void keep_system(int which, Mat A, Vec rhs) {
  ref_system *s = &g_sys[which];
  free(s->rowptr);
  free(s->cols);
  free(s->vals);
  free(s->rhs);
  s->nnz = plite_MatGetCSR(A, &s->rowptr, &s->cols, &s->vals);
  VecGetSize(rhs, &s->n);
  s->rhs = (PetscScalar *)malloc(sizeof(PetscScalar) * (size_t)s->n);
  PetscScalar *a;
  VecGetArray(rhs, &a);
  memcpy(s->rhs, a, sizeof(PetscScalar) * (size_t)s->n);
}

/* formVEPSystem on the nodal fields with gy = so->gy and P = NULL (no preconditioner matrix) */
int ref_formVEPSystem(refp *p, const mic_subduction_options *so, double dt, double *Kbond, double *Kcont) {
  set_subduction(p, so);
  Mat A;
  Vec rhs;
  plite_MatCreate(3 * p->grid.NX * p->grid.NY, &A);
  DMCreateGlobalVector(p->grid.vda, &rhs);
  int e = formVEPSystem(&p->nf, &p->grid, A, NULL, rhs, Kbond, Kcont, so->gy, dt, &p->opt, &p->bv);
  if (!e) keep_system(0, A, rhs);
  MatDestroy(&A);
  VecDestroy(&rhs);
  return e;
}

/* enforceThermalBCs1 on lastT (main_subduction.c:383) */
int ref_enforceThermalBCs1(refp *p, const mic_subduction_options *so) {
  set_subduction(p, so);
  return enforceThermalBCs1(&p->grid, &p->opt, &p->nf);
}

/* formThermalSystem with the right-hand side starting as a copy of the heating field
 * (main_subduction.c:381, VecCopy(nodal_heating, rhs)) */
int ref_formThermalSystem(refp *p, const mic_subduction_options *so, double dt, int doSteady) {
  set_subduction(p, so);
  Problem pr;
  memset(&pr, 0, sizeof(pr));
  pr.materials = p->mat;
  Mat A;
  Vec rhs;
  plite_MatCreate(p->grid.NX * p->grid.NY, &A);
  DMCreateGlobalVector(p->grid.da, &rhs);
  VecCopy(p->heat, rhs);
  int e = formThermalSystem(&pr, &p->grid, &p->nf, A, rhs, dt, &p->opt, doSteady);
  if (!e) keep_system(1, A, rhs);
  MatDestroy(&A);
  VecDestroy(&rhs);
  return e;
}

long ref_system_nnz(int which, long *nrows) {
  if (nrows) *nrows = g_sys[which].n;
  return g_sys[which].nnz;
}

void ref_system_get(int which, int *rowptr, int *cols, double *vals, double *rhs) {
  const ref_system *s = &g_sys[which];
  memcpy(rowptr, s->rowptr, sizeof(int) * (size_t)(s->n + 1));
  memcpy(cols, s->cols, sizeof(int) * (size_t)s->nnz);
  memcpy(vals, s->vals, sizeof(double) * (size_t)s->nnz);
  memcpy(rhs, s->rhs, sizeof(double) * (size_t)s->n);
}

/* adiabaticHeating (adiabaticHeating.c:7) with gy, then main's VecAXPY(nodal_heating, 1.0, ha)
 * (main_subduction.c:377) */
int ref_adiabaticHeating(refp *p, double gy) {
  p->opt.gy = gy;
  int e = adiabaticHeating(&p->grid, &p->ms, &p->nf, &p->mat, &p->opt);
  if (!e) e = VecAXPY(p->heat, 1.0, p->nf.ha);
  return e;
}

/* nusseltNumber (post.c:5) of thisT with the bottom and top boundary temperatures */
double ref_nusseltNumber(refp *p, double bottom, double top) {
  p->opt.thermalBCBottom.value[0] = bottom;
  p->opt.thermalBCTop.value[0] = top;
  PetscScalar Nu = 0.0;
  nusseltNumber(&p->grid, &p->opt, p->thisT, &Nu);
  return Nu;
}

/* rmsVelocity (post.c:49) of the nodal vx, vy */
double ref_rmsVelocity(refp *p) {
  PetscScalar v = 0.0;
  rmsVelocity(&p->grid, &p->nf, &v);
  return v;
}

/* initialConditionsVanKeken (benchmarkInitialConditions.c:8) on the caller's markers; the
 * boundary conditions it sets in Options come back in bcs */
int ref_initialConditionsVanKeken(refp *p, mic_marker *m, int n, const mic_subduction_options *so, mic_bcs *bcs) {
  set_subduction(p, so);
  p->ms.markers = (Marker *)m;
  p->ms.nMark = n;
  p->ms.maxMark = n;
  int e = initialConditionsVanKeken(&p->ms, &p->opt, &p->mat, &p->grid);
  bcs->mechBCLeft = *(const mic_bcinfo *)&p->opt.mechBCLeft;
  bcs->mechBCRight = *(const mic_bcinfo *)&p->opt.mechBCRight;
  bcs->mechBCTop = *(const mic_bcinfo *)&p->opt.mechBCTop;
  bcs->mechBCBottom = *(const mic_bcinfo *)&p->opt.mechBCBottom;
  return e;
}
