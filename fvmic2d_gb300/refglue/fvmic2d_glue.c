/*
 * fvmic2d_glue.c -- the reference-side binding of libmic_gb300: fvmic2d's marker routines under
 * their own names and signatures, each a thin call into the library's C ABI.
 *
 * A maintainer compiles this file into fvmic2d's build (one rank, one GPU) in place of
 *   markerProjection.c, updateMarkerStrainPressure.c, subgridStressChanges.c,
 *   updateMarkerStress.c, subgridTemperatureChanges.c and residual.c (whole files),
 * and of these functions of markers.c and viscosity.c (the rest of those files -- per-marker
 * helpers such as findMarkerCell, resetMarker, computeRheology, updateMarkerViscosity,
 * limitMarkerViscosity, exchangeMarkers -- stay the reference's host code):
 *   allocateMarkers, destroyMarkers, resetMarkers, distributeMarkersUniformInDomain,
 *   findMarkerCells, checkPlasticYielding, checkMarkerDensity, advectMarkersRK,
 *   projectMarkersNodesFromScalar, projectNodalFieldToMarkersS, updateViscosity, limitViscosity.
 * It links -lmic_gb300.  Arithmetic happens in the library; this file moves pointers, nodal
 * fields and the marker array.
 *
 * Markers.  MarkerSet.markers stays a host array of capacity maxMark, allocated here as the
 * reference allocates it.  The library keeps a device copy; exactly one of the two is current
 * (fvmic2d_glue.h says when each is).  The device context is created by the first routine that
 * knows the grid, with the marker set's capacity.
 *
 * Nodal fields.  PETSc global Vecs on one rank hold the NX*NY values in the library's own layout
 * ([j][i], x fastest), so a Vec's array is uploaded or downloaded as it is.  Each routine
 * uploads the fields it reads (host code between the routines -- the Stokes and thermal solves,
 * nodalStressStrain -- may have changed any of them) and downloads the fields it writes.
 *
 * Errors.  Library codes come back as the routines' PetscErrorCode (0 = success).  Where the
 * reference aborts (an impossible cell, a NaN strain-rate residual, an undefined viscosity law, a
 * full marker array) the library returns MIC_ERR_CELL, MIC_ERR_NAN, MIC_ERR_LAW or
 * MIC_ERR_CAPACITY instead; routines whose reference signature returns void record the code for
 * micGlueLastError.
 */
#include <stddef.h>
#include <stdlib.h>
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
#include "mic_gb300.h"

/* the records the library takes are the reference's own (include/mic_types.h) */
typedef char glue_marker_layout[(sizeof(Marker) == sizeof(mic_marker) &&
                                 offsetof(Marker, isYielding) == offsetof(mic_marker, isYielding)) ? 1 : -1];
typedef char glue_materials_layout[(sizeof(Materials) == sizeof(mic_materials)) ? 1 : -1];
typedef char glue_bc_layout[(sizeof(BoundaryValues) == sizeof(mic_bcs)) ? 1 : -1];

enum { ON_HOST = 0, ON_DEVICE = 1 };

static struct {
  mic_ctx *ctx;
  MarkerSet *ms;   /* the marker set whose device copy the context holds */
  int where;       /* ON_HOST: ms->markers is current; ON_DEVICE: the device copy is */
  int device;      /* -1: not chosen yet */
  int last_error;
} g = {NULL, NULL, ON_HOST, -1, 0};

/* a nodal field the glue uses as a staging slot for Vecs that are not NodalFields members (the
 * library computes the invariants there only in its own nodalStressStrain, which this build
 * leaves to the host) */
#define GLUE_SCRATCH_FIELD MIC_NF_SII

static int note(int e) {
  if (e) g.last_error = e;
  return e;
}

void micGlueSetDevice(int device) { g.device = device; }
mic_ctx *micGlueContext(void) { return g.ctx; }
int micGlueLastError(void) { return g.last_error; }

static int glue_device(void) {
  if (g.device < 0) {
    const char *s = getenv("FVMIC2D_GPU");
    g.device = s ? atoi(s) : 0;
  }
  return g.device;
}

static void set_options(const Options *opt) {
  mic_options o;
  o.etamin = opt->etamin;
  o.etamax = opt->etamax;
  o.fractionalEtamin = opt->fractionalEtamin;
  o.subgridStressDiffusivity = opt->subgridStressDiffusivity;
  o.subgridTemperatureDiffusivity = opt->subgridTemperatureDiffusivity;
  o.slabAngle = opt->slabAngle;
  o.decoupleThickness = opt->decoupleThickness;
  o.minDecoupleDepth = opt->minDecoupleDepth;
  o.maxDecoupleDepth = opt->maxDecoupleDepth;
  o.decoupleEtaScaler = opt->decoupleEtaScaler;
  note(mic_set_options(g.ctx, &o));
}

/* the context for this grid and marker set, created on first use with the set's capacity */
static int ensure_ctx(GridData *grid, MarkerSet *ms) {
  if (g.ctx) {
    if (g.ms != ms) return note(MIC_ERR_ARG); /* one marker set per process */
    return MIC_OK;
  }
  if (!grid || !ms) return note(MIC_ERR_ARG);
  /* x, y point at entry 0 of the grid's ghost-offset arrays (gridGenerator.c:127-130) */
  int e = mic_create(&g.ctx, glue_device(), NULL, grid->NX, grid->NY, grid->LX, grid->LY, grid->x, grid->y,
                     ms->maxMark);
  if (e) {
    g.ctx = NULL;
    return note(e);
  }
  g.ms = ms;
  g.where = ON_HOST;
#ifdef JAUMANN
  /* the application is built with the Jaumann stress rotation (markers.c:2147-2156) */
  if ((e = mic_set_stress_rotation(g.ctx, MIC_ROTATION_JAUMANN))) return note(e);
#endif
  return MIC_OK;
}

/* make the device copy current: upload the first n host records when the host array is */
static int to_device_n(MarkerSet *ms, PetscInt n) {
  if (!g.ctx) return note(MIC_ERR_ARG);
  if (g.where == ON_HOST) {
    int e = mic_markers_upload(g.ctx, (const mic_marker *)ms->markers, n);
    if (e) return note(e);
    g.where = ON_DEVICE;
  }
  return MIC_OK;
}
static int to_device(GridData *grid, MarkerSet *ms) {
  int e = ensure_ctx(grid, ms);
  return e ? e : to_device_n(ms, ms->nMark);
}

/* the device routines need a context; those without a grid argument need an existing one */
static int device_ready(MarkerSet *ms) {
  if (!g.ctx) return note(MIC_ERR_ARG);
  if (g.ms != ms) return note(MIC_ERR_ARG);
  return to_device_n(ms, ms->nMark);
}

PetscErrorCode micMarkersToHost(MarkerSet *ms) {
  if (!g.ctx || g.ms != ms || g.where == ON_HOST) return 0;
  int64_t n = 0;
  int e = mic_marker_count(g.ctx, &n);
  if (!e && n > ms->maxMark) e = MIC_ERR_CAPACITY;
  if (!e) e = mic_markers_download(g.ctx, (mic_marker *)ms->markers, n);
  if (e) return note(e);
  ms->nMark = (PetscInt)n;
  g.where = ON_HOST;
  return 0;
}

static int vec_up(Vec v, int field) {
  PetscScalar *a;
  VecGetArray(v, &a);
  int e = mic_nodal_upload(g.ctx, field, a);
  VecRestoreArray(v, &a);
  return note(e);
}
static int vec_down(Vec v, int field) {
  PetscScalar *a;
  VecGetArray(v, &a);
  int e = mic_nodal_download(g.ctx, field, a);
  VecRestoreArray(v, &a);
  return note(e);
}

/* byte offset of a marker field addressed as &markers[0].field */
static int field_offset(MarkerSet *ms, const PetscScalar *field) {
  return (int)((const char *)field - (const char *)ms->markers);
}

/* ---- lifecycle (markers.c:15-39, 332-400) ------------------------------------------------ */

PetscErrorCode allocateMarkers(PetscInt nMark, MarkerSet *ms, Options *opt) {
  const size_t bytes = (size_t)nMark * sizeof(Marker);
  PetscErrorCode ierr = PetscMalloc(bytes, &(ms->markers));
  CHKERRQ(ierr);
  /* zeroed: resetMarker leaves some fields (mu, cells, cpu, strain-rate residual) as they are,
   * which in the reference means uninitialised memory */
  memset(ms->markers, 0, bytes);
  ms->maxMark = nMark;
  ms->nOut = 0;
  if (g.ms == ms) g.where = ON_HOST; /* a fresh array for a set the context already knows */
  resetMarkers(ms, opt);
  return 0;
}

PetscErrorCode destroyMarkers(MarkerSet *ms, Options *opt) {
  (void)opt;
  if (g.ctx && g.ms == ms) {
    mic_destroy(g.ctx);
    g.ctx = NULL;
    g.ms = NULL;
    g.where = ON_HOST;
  }
  PetscErrorCode ierr = PetscFree(ms->markers);
  CHKERRQ(ierr);
  ms->markers = PETSC_NULL;
  ms->nMark = 0;
  ms->maxMark = 0;
  ms->nOut = 0;
  return 0;
}

/* resetMarker's values on every slot of the capacity, on whichever copy is current */
void resetMarkers(MarkerSet *ms, Options *opt) {
  (void)opt;
  if (g.ctx && g.ms == ms && g.where == ON_DEVICE)
    note(mic_reset_markers(g.ctx));
  else
    note(mic_markers_reset_host((mic_marker *)ms->markers, ms->maxMark));
}

/* NMX x NMY markers per cell on the domain-wide jittered lattice, drawn on the device; the host
 * array is current afterwards (main fills the initial conditions on it) */
PetscErrorCode distributeMarkersUniformInDomain(MarkerSet *ms, Options *opt, GridData *grid) {
  int e = ensure_ctx(grid, ms);
  if (e) return e;
  /* every slot of the capacity: distribution keeps the fields it does not place */
  if ((e = to_device_n(ms, ms->maxMark))) return e;
  int64_t n = 0;
  if ((e = mic_distribute_markers_uniform_in_domain(g.ctx, opt->NMX, opt->NMY, 0, &n))) return note(e);
  ms->nMark = (PetscInt)n;
  return micMarkersToHost(ms);
}

/* ---- cells, rheology, yield (markers.c:85-106, 1381-1505; viscosity.c:77-104) ------------- */

void findMarkerCells(MarkerSet *ms, GridData *grid) {
  if (to_device(grid, ms)) return;
  int64_t nout = 0;
  if (!note(mic_find_marker_cells(g.ctx, &nout))) ms->nOut = (PetscInt)nout;
}

PetscErrorCode checkPlasticYielding(GridData *grid, MarkerSet *ms, Materials *mat, PetscScalar dt,
                                    PetscInt *isYielding, Options *opt, PetscScalar t) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  int y = 0;
  e = note(mic_check_plastic_yielding(g.ctx, dt, &y, t));
  if (isYielding) *isYielding = (PetscInt)y;
  return e;
}

void updateViscosity(MarkerSet *ms, Options *opt, Materials *mat) {
  if (device_ready(ms)) return;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  note(mic_update_viscosity(g.ctx));
}

void limitViscosity(MarkerSet *ms, Options *opt, Materials *mat) {
  if (device_ready(ms)) return;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  note(mic_limit_viscosity(g.ctx));
}

/* ---- projections (markerProjection.c:11-269; markers.c:1507-1594, 1670-1706) -------------- */

PetscErrorCode projectMarkersNodesAll2(MarkerSet *ms, GridData *grid, NodalFields *nf, Materials *mat,
                                       Options *opt) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  if ((e = note(mic_project_markers_nodes_all2(g.ctx)))) return e;
  const struct {
    Vec v;
    int f;
  } out[] = {{nf->rho, MIC_NF_RHO},   {nf->rhodot, MIC_NF_RHODOT},     {nf->etaS, MIC_NF_ETAS},
             {nf->etaN, MIC_NF_ETAN}, {nf->muS, MIC_NF_MUS},           {nf->muN, MIC_NF_MUN},
             {nf->lastT, MIC_NF_LASTT}, {nf->kThermal, MIC_NF_KTHERMAL}, {nf->Cp, MIC_NF_CP},
             {nf->soxx, MIC_NF_SOXX}, {nf->soyy, MIC_NF_SOYY},         {nf->soxy, MIC_NF_SOXY}};
  for (size_t k = 0; k < sizeof(out) / sizeof(out[0]) && !e; ++k) e = vec_down(out[k].v, out[k].f);
  return e;
}

/* markerField is &markers[0].field (stride sizeof(Marker)); a non-NULL matProp takes its place
 * with a per-material constant (markerProjection.c:98-111) */
PetscErrorCode projectMarkerFieldToNodes(GridData *grid, MarkerSet *ms, PetscScalar *matProp, PetscScalar *markerField,
                                         Vec out, const PetscInt stagx, const PetscInt stagy,
                                         const PROJECTION_METHOD method) {
  int e = to_device(grid, ms);
  if (e) return e;
  const int off = (!matProp && markerField) ? field_offset(ms, markerField) : -1;
  if ((e = note(mic_project_marker_field_to_nodes(g.ctx, off, matProp, GLUE_SCRATCH_FIELD, (int)stagx, (int)stagy,
                                                  (int)method))))
    return e;
  return vec_down(out, GLUE_SCRATCH_FIELD);
}

/* scalar: one value per marker, in the marker array's order */
PetscErrorCode projectMarkersNodesFromScalar(MarkerSet *ms, GridData *grid, PetscScalar *scalar, Vec out) {
  int e = to_device(grid, ms);
  if (e) return e;
  if ((e = note(mic_project_markers_nodes_from_scalar(g.ctx, scalar, GLUE_SCRATCH_FIELD)))) return e;
  return vec_down(out, GLUE_SCRATCH_FIELD);
}

PetscErrorCode projectNodalFieldToMarkersS(NodalFields *nf, Vec field, MarkerSet *ms, PetscScalar *markerField,
                                           GridData *grid) {
  (void)nf;
  int e = to_device(grid, ms);
  if (e) return e;
  if ((e = vec_up(field, GLUE_SCRATCH_FIELD))) return e;
  return note(mic_project_nodal_field_to_markers(g.ctx, GLUE_SCRATCH_FIELD, field_offset(ms, markerField)));
}

/* ---- node -> marker updates (updateMarkerStrainPressure.c, subgridStressChanges.c,
 *      updateMarkerStress.c, subgridTemperatureChanges.c, residual.c) -------------------------- */

PetscErrorCode updateMarkerStrainPressure(GridData *grid, NodalFields *nf, MarkerSet *ms, Materials *mat,
                                          Options *opt, PetscScalar dt) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  const struct {
    Vec v;
    int f;
  } in[] = {{nf->p, MIC_NF_P},       {nf->edotxx, MIC_NF_EDOTXX}, {nf->edotyy, MIC_NF_EDOTYY},
            {nf->edotxy, MIC_NF_EDOTXY}, {nf->soxx, MIC_NF_SOXX},   {nf->soyy, MIC_NF_SOYY},
            {nf->soxy, MIC_NF_SOXY},   {nf->dsxx, MIC_NF_DSXX},     {nf->dsyy, MIC_NF_DSYY},
            {nf->dsxy, MIC_NF_DSXY},   {nf->wxy, MIC_NF_WXY}};
  for (size_t k = 0; k < sizeof(in) / sizeof(in[0]) && !e; ++k) e = vec_up(in[k].v, in[k].f);
  if (e) return e;
  return note(mic_update_marker_strain_pressure(g.ctx, dt));
}

PetscErrorCode updateGlobalStrainRateResidual(GridData *grid, MarkerSet *ms, PetscInt iter) {
  int e = to_device(grid, ms);
  if (e) return e;
  return note(mic_update_global_strain_rate_residual(g.ctx, (int)iter, NULL));
}

PetscScalar getGlobalStrainRateResidual(PetscInt iter) {
  double v = 0.0;
  if (g.ctx) note(mic_get_strain_rate_residual(g.ctx, (int)iter, &v));
  return v;
}

void setGlobalStrainRateResidual(PetscInt iter, PetscScalar value) {
  if (g.ctx) note(mic_set_strain_rate_residual(g.ctx, (int)iter, value));
}

PetscInt checkConvergence(PetscScalar atol, PetscScalar rtol, PetscInt iter) {
  int c = 0;
  if (g.ctx) note(mic_check_convergence(g.ctx, atol, rtol, (int)iter, &c));
  return (PetscInt)c;
}

PetscErrorCode subgridStressChanges(GridData *grid, NodalFields *nf, MarkerSet *ms, Materials *mat, PetscScalar dt,
                                    PetscScalar D) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  const struct {
    Vec v;
    int f;
  } in[] = {{nf->soxx, MIC_NF_SOXX}, {nf->soyy, MIC_NF_SOYY}, {nf->soxy, MIC_NF_SOXY},
            {nf->dsxx, MIC_NF_DSXX}, {nf->dsyy, MIC_NF_DSYY}, {nf->dsxy, MIC_NF_DSXY}};
  for (size_t k = 0; k < sizeof(in) / sizeof(in[0]) && !e; ++k) e = vec_up(in[k].v, in[k].f);
  if (e) return e;
  if ((e = note(mic_subgrid_stress_changes(g.ctx, dt, D)))) return e;
  /* the nodal stress changes lose their sub-grid part (subgridStressChanges.c:283-286) */
  if (!e) e = vec_down(nf->dsxx, MIC_NF_DSXX);
  if (!e) e = vec_down(nf->dsyy, MIC_NF_DSYY);
  if (!e) e = vec_down(nf->dsxy, MIC_NF_DSXY);
  return e;
}

PetscErrorCode updateMarkerStress(GridData *grid, NodalFields *nf, MarkerSet *ms, Materials *mat) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  if (!e) e = vec_up(nf->dsxx, MIC_NF_DSXX);
  if (!e) e = vec_up(nf->dsyy, MIC_NF_DSYY);
  if (!e) e = vec_up(nf->dsxy, MIC_NF_DSXY);
  if (e) return e;
  return note(mic_update_marker_stress(g.ctx));
}

PetscErrorCode subgridTemperatureChanges(Vec thisT, GridData *grid, NodalFields *nf, MarkerSet *ms, Materials *mat,
                                         PetscScalar dt, Options *opt) {
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  set_options(opt);
  const struct {
    Vec v;
    int f;
  } in[] = {{thisT, MIC_NF_THIST}, {nf->lastT, MIC_NF_LASTT}, {nf->rho, MIC_NF_RHO},
            {nf->Cp, MIC_NF_CP},   {nf->kThermal, MIC_NF_KTHERMAL}};
  for (size_t k = 0; k < sizeof(in) / sizeof(in[0]) && !e; ++k) e = vec_up(in[k].v, in[k].f);
  if (e) return e;
  return note(mic_subgrid_temperature_changes(g.ctx, dt));
}

/* ---- advection (markers.c:1865-2250) and density control (markers.c:455-781) -------------- */

PetscErrorCode advectMarkersRK(MarkerSet *ms, NodalFields *nf, GridData *grid, Options *opt, BoundaryValues *bv,
                               PetscScalar dt) {
  int e = to_device(grid, ms);
  if (e) return e;
  set_options(opt);
  if ((e = note(mic_set_bcs(g.ctx, (const mic_bcs *)bv)))) return e;
  if (!e) e = vec_up(nf->vx, MIC_NF_VX);
  if (!e) e = vec_up(nf->vy, MIC_NF_VY);
  if (!e) e = vec_up(nf->wxy, MIC_NF_WXY);
  if (e) return e;
  return note(mic_advect_markers_rk(g.ctx, dt));
}

/* The PETSc random object r is the one main() seeded (PETSCRAND48, seed 1, main_subduction.c:
 * 96-100): the library draws from that drand48 stream itself (state srand48(1) when the context
 * is created; mic_density_rng_state hands over another state).  Where the reference aborts on a
 * full marker array this returns MIC_ERR_CAPACITY. */
PetscErrorCode checkMarkerDensity(Problem *problem, MarkerSet *ms, GridData *grid, Options *opt, PetscRandom r) {
  (void)r;
  int e = to_device(grid, ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)&problem->materials));
  set_options(opt);
  mic_density_options d;
  d.NMX = opt->NMX;
  d.NMY = opt->NMY;
  d.minMarkers = opt->minMarkers;
  d.maxMarkers = opt->maxMarkers;
  d.slabAngle = opt->slabAngle;
  d.slabAge = opt->slabAge;
  d.overridingPlateThickness = opt->overridingPlateThickness;
  d.rootThickness = opt->rootThickness;
  d.rootCenter = opt->rootCenter;
  d.rootWidth = opt->rootWidth;
  int64_t added = 0, removed = 0, n = 0;
  if ((e = note(mic_check_marker_density(g.ctx, &d, &added, &removed)))) return e;
  if ((e = note(mic_marker_count(g.ctx, &n)))) return e;
  ms->nMark = (PetscInt)n;
  return 0;
}

/* ---- main_subduction.c's inline marker loops ------------------------------------------------ */

PetscErrorCode micUpdateMarkerRho(MarkerSet *ms, Materials *mat) {
  int e = device_ready(ms);
  if (e) return e;
  note(mic_set_materials(g.ctx, (const mic_materials *)mat));
  return note(mic_update_marker_rho(g.ctx));
}

PetscScalar micMaxMarkerT(MarkerSet *ms) {
  double v = 0.0;
  if (!device_ready(ms)) note(mic_max_marker_T(g.ctx, &v));
  return v;
}

PetscScalar micMaxAbsSxx(MarkerSet *ms) {
  double v = 0.0;
  if (!device_ready(ms)) note(mic_max_abs_sxx(g.ctx, &v));
  return v;
}
