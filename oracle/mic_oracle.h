/*
 * mic_oracle.h -- CPU restatement of fvmic2d's marker-in-cell transfer path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU kernels are compared
 * against (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline leg).  Each
 * function follows the reference function cited beside it, in the same marker
 * order and with the same floating-point expression order, so that on a given
 * host it reproduces the reference build (oracle/_ref) bit for bit
 * (tests/test_oracle_vs_ref.py) and the committed golden vectors
 * (tests/golden/).  Compile with -ffp-contract=off.
 *
 * Layout: markers are the 216-byte fvmic2d records (mic_marker); every nodal
 * field is an NX*NY array, x fastest; grid arrays x, y, xc, yc carry two ghost
 * entries on each side like GridData (gridGenerator.c:123-130).
 */
#ifndef MIC_ORACLE_H
#define MIC_ORACLE_H

#include <stdint.h>
#include "mic_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

enum {
  ORC_OK = 0,
  ORC_ERR_ARG = 1,
  ORC_ERR_CELL = 2,  /* impossible cell index (markers.c:74-77 aborts) */
  ORC_ERR_NAN = 3,   /* NaN strain-rate residual (updateMarkerStrainPressure.c:302-306 aborts) */
  ORC_ERR_LAW = 4,   /* unknown viscosity law (viscosity.c:60-62 aborts) */
  ORC_ERR_BC = 5,    /* boundary type whose ghost values the path would read */
};

orc_ctx *orc_create(int NX, int NY, double LX, double LY, const double *x, const double *y);
void orc_destroy(orc_ctx *c);
void orc_get_grid(const orc_ctx *c, double *xc, double *yc);
void orc_set_materials(orc_ctx *c, const mic_materials *m);
void orc_set_options(orc_ctx *c, const mic_options *o);
/* advectMarkersRK's stress rotation as the reference compiled with -DJAUMANN (markers.c:2147-2156) */
void orc_set_jaumann(orc_ctx *c, int on);
int orc_set_bcs(orc_ctx *c, const mic_bcs *b);
int orc_set_nodal(orc_ctx *c, int field, const double *v);
int orc_get_nodal(const orc_ctx *c, int field, double *v);

int64_t orc_find_marker_cells(orc_ctx *c, mic_marker *mk, int64_t n, int *err);
void orc_update_marker_rho(orc_ctx *c, mic_marker *mk, int64_t n);
double orc_max_marker_T(const orc_ctx *c, const mic_marker *mk, int64_t n);
double orc_max_abs_sxx(const orc_ctx *c, const mic_marker *mk, int64_t n);
int orc_project_marker_field(orc_ctx *c, const mic_marker *mk, int64_t n, int field_offset, const double *matprop,
                             int out_field, int stagx, int stagy, int method);
int orc_project_markers_nodes_all2(orc_ctx *c, const mic_marker *mk, int64_t n);
int orc_project_nodal_to_markers(orc_ctx *c, mic_marker *mk, int64_t n, int nodal_field, int field_offset);
int orc_check_plastic_yielding(orc_ctx *c, mic_marker *mk, int64_t n, double dt, int *is_yielding);
int orc_compute_rheology(const orc_ctx *c, const mic_marker *m, double *eta, double *mu);
void orc_limit_viscosity(orc_ctx *c, mic_marker *mk, int64_t n);
int orc_update_marker_strain_pressure(orc_ctx *c, mic_marker *mk, int64_t n, double dt);
double orc_update_global_strain_rate_residual(orc_ctx *c, const mic_marker *mk, int64_t n, int iter);
int orc_subgrid_stress_changes(orc_ctx *c, mic_marker *mk, int64_t n, double dt, double D);
int orc_update_marker_stress(orc_ctx *c, mic_marker *mk, int64_t n, int64_t *nan_count);
int orc_subgrid_temperature_changes(orc_ctx *c, mic_marker *mk, int64_t n, double dt);
int orc_advect_markers_rk(orc_ctx *c, mic_marker *mk, int64_t n, double dt);

/* One marker-path step in main_subduction.c order (main:243-448) with the host solves
 * replaced by the nodal inputs already stored in the context (vx, vy, p, edot*, wxy,
 * so*, ds*, thisT).  Writes the residual to *residual. */
int orc_step(orc_ctx *c, mic_marker *mk, int64_t n, double dt_disp, double dt_thermal, int do_subgrid_stress,
             double *residual);

/* Composite ice creep (Goldsby & Kohlstedt 2001) as written in viscosity.c:106-179:
 * returns the effective viscosity at stress s, temperature T, grain size d, pressure P. */
double orc_gk_viscosity(double s, double T, double d, double P);

int64_t orc_sizeof(int which);

/* Composite ice creep (material law 7, new): per-marker grain sizes, the strain rate of the
 * Goldsby-Kohlstedt law and the stress at which it equals a given strain rate. */
void orc_set_grain(orc_ctx *c, const double *d, int64_t n);
double orc_gk_strain_rate(double s, double T, double d, double P);
int orc_creep_stress(double edot, double T, double d, double P, double rtol, double *s_out, int *iters);
int orc_creep_stress_batch(const double *edot, const double *T, const double *d, const double *P, int64_t n,
                           double rtol, double *s_out, int *iters);

/* marker lifecycle: resetMarker (markers.c:255-330) and distributeMarkersUniformInDomain
 * (markers.c:342-400) with the stand-in's seeded erand48 stream */
void orc_reset_markers(mic_marker *mk, int64_t n);
int64_t orc_distribute_uniform(const orc_ctx *c, mic_marker *mk, int64_t cap, int NMX, int NMY, unsigned long seed);

/* checkMarkerDensity (markers.c:455-781) on an array of capacity cap; *state is the 48-bit
 * drand48 stream (orc_srand48_state(seed) = srand48(seed)) */
uint64_t orc_srand48_state(long seed);
/* grid routines between the solves: nodalStressStrain, limitDisplacementTimestep,
 * retrieveSolutions (S: [(j NX + i) 3 + {vx, vy, p}]) */
void orc_nodal_stress_strain(orc_ctx *c, double dt);
double orc_limit_displacement_timestep(const orc_ctx *c, double dt, double factor);
void orc_retrieve_solutions(orc_ctx *c, const double *S, double Kcont);
/* marker checkpoint in the reference's field-major binary format (io.c:299, restart.c:8) */
int orc_save_markers_binary(const char *path, const mic_marker *mk, int64_t n, double elapsed);
int64_t orc_restart_from_markers(orc_ctx *c, const char *path, mic_marker *mk, int64_t cap, double *elapsed);
int orc_project_from_scalar(orc_ctx *c, const mic_marker *mk, int64_t n, const double *v, int field);
int64_t orc_check_marker_density(orc_ctx *c, mic_marker *mk, int64_t n, int64_t cap, const mic_density_options *d,
                                 uint64_t *state, int64_t *n_added, int64_t *n_removed);

#ifdef __cplusplus
}
#endif

#endif
