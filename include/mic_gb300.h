/*
 * mic_gb300.h -- C ABI of the GB300 marker-in-cell transfer library (libmic_gb300.so).
 *
 * The library replaces fvmic2d's marker-side routines -- the work between and
 * around the host Stokes and thermal solves -- with CUDA kernels for sm_103a.
 * Every entry point takes plain pointers and sizes; markers use the reference's
 * 216-byte record (mic_marker == fdcode.h Marker), nodal fields the NX*NY
 * global-vector layout ([j][i] = j*NX + i).
 *
 * State model: a context owns one grid, the device copies of every nodal field
 * and up to `max_markers` markers kept on the device as columns.  Markers are
 * re-ordered by cell on the device after binning; mic_markers_download always
 * returns them in the caller's original order.  Calls on a context are
 * serialised on the context's stream; entry points that return host values
 * synchronise that stream.  All functions return 0 (MIC_OK) or an error code;
 * none aborts the process (the reference aborts, see the codes below).
 */
#ifndef MIC_GB300_H
#define MIC_GB300_H

#include <stdint.h>
#include "mic_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mic_ctx mic_ctx;

enum {
  MIC_OK = 0,
  MIC_ERR_ARG = 1,        /* invalid argument (bad field id, stagger, method, size) */
  MIC_ERR_CUDA = 2,       /* CUDA runtime error (context left usable where CUDA allows) */
  MIC_ERR_NOMEM = 3,      /* device or host allocation failed */
  MIC_ERR_CELL = 4,       /* impossible cell index; markers.c:74-77 aborts */
  MIC_ERR_NAN = 5,        /* NaN strain-rate residual; updateMarkerStrainPressure.c:302-306 aborts */
  MIC_ERR_LAW = 6,        /* undefined viscosity law; viscosity.c:60-62 aborts */
  MIC_ERR_BC = 7,         /* unsupported boundary type, or a routine outside the marker path on a grid
                             periodic in x */
  MIC_ERR_CAPACITY = 8,   /* more markers than the context was created for; markers.c:771-774 aborts */
  MIC_ERR_NO_DEVICE = 9,  /* no CUDA device: there is no CPU fallback */
  MIC_ERR_DENSITY = 10,   /* density control: a quarter cell would get a non-positive number of
                           * markers (markers.c:590-593 aborts), an overfull quarter cell with no
                           * marker inside its bounds, or more than 2048 markers in one */
  MIC_ERR_IO = 11,        /* checkpoint file could not be opened, read or written */
  MIC_ERR_SOLVE = 12      /* direct solve: zero pivot (singular matrix) or a band too wide */
};

typedef struct {
  uint64_t bad_cell;      /* markers with an impossible cell index in the last binning */
  uint64_t nan_residual;  /* markers with a NaN strain-rate residual */
  uint64_t nan_dsxy;      /* markers whose interpolated dsxy was NaN (the reference only prints) */
  uint64_t bad_law;       /* markers whose material has an undefined viscosity law */
  uint64_t n_out;         /* out-of-domain markers after the last binning */
  int32_t is_yielding;    /* any marker yielded in the last checkPlasticYielding */
} mic_status;

int mic_version(void);
const char *mic_error_string(int code);

/* ---- lifecycle: replaces GridData / NodalFields setup and allocateMarkers (markers.c:15-27) ---- */
/* x[NX], y[NY] are the basic gridlines; cell centres follow getCellCenters (gridSpacing.c:150-157).
 * stream: a cudaStream_t to run on, or NULL for a stream owned by the context. */
int mic_create(mic_ctx **out, int device, void *stream, int NX, int NY, double LX, double LY, const double *x,
               const double *y, int64_t max_markers);
/* destroyMarkers (markers.c:29-39) + nodal field / grid teardown */
int mic_destroy(mic_ctx *ctx);
int mic_set_materials(mic_ctx *ctx, const mic_materials *materials);
int mic_set_options(mic_ctx *ctx, const mic_options *options);
/* BoundaryValues read by advectMarkersRK (markers.c:1986-2023).  A left or right vx type 2 makes
 * the grid periodic in x, as the reference's grid generators and nodal DMDAs do
 * (gridGenerator.c:67-68, 97-110; nodalFields.c:11-19): x holds the first NX of NX + 1 uniform
 * lines from 0 to LX (NX cells in x; line NX = LX is line 0's image), the marker path wraps node
 * columns and marker positions across the seam (markers.c:2225-2231), and the routines outside
 * the marker path (density control, grid routines, systems, time step) return MIC_ERR_BC.  Top
 * vx type 0 or 1; on a non-periodic grid left vy type 0 or 1. */
int mic_set_bcs(mic_ctx *ctx, const mic_bcs *bcs);
int mic_get_bcs(mic_ctx *ctx, mic_bcs *bcs); /* the context's boundary conditions */
/* The stress rotation of advectMarkersRK, the reference's compile-time JAUMANN switch as a
 * context setting (new): MIC_ROTATION_EXACT (default) rotates the marker stresses through the
 * angle -wxy dt (markers.c:2158-2164, the reference built without JAUMANN); MIC_ROTATION_JAUMANN
 * adds the first-order Jaumann terms (markers.c:2147-2156, built with -DJAUMANN). */
enum { MIC_ROTATION_EXACT = 0, MIC_ROTATION_JAUMANN = 1 };
int mic_set_stress_rotation(mic_ctx *ctx, int rotation);
int mic_get_stress_rotation(mic_ctx *ctx, int *rotation);
int mic_get_grid_centres(mic_ctx *ctx, double *xc, double *yc); /* NX+1, NY+1 entries */

/* ---- markers: host AoS records <-> device columns ---- */
int mic_markers_upload(mic_ctx *ctx, const mic_marker *host, int64_t n);
int mic_markers_download(mic_ctx *ctx, mic_marker *host, int64_t n);
int mic_markers_count(mic_ctx *ctx, int64_t *n);

/* ---- nodal fields (MIC_NF_* ids) ---- */
int mic_nodal_upload(mic_ctx *ctx, int field, const double *host);
int mic_nodal_download(mic_ctx *ctx, int field, double *host);
/* Several nodal fields in one call (new): fields[k] to or from host[k], count <= 32, one
 * synchronization.  When every host buffer is pinned (mic_host_alloc, or registered) a single
 * kernel moves all of them through the device's view of host memory (coherent NVLink-C2C on
 * Grace-Blackwell); otherwise one copy per field. */
int mic_nodal_upload_many(mic_ctx *ctx, const int *fields, const double *const *host, int count);
int mic_nodal_download_many(mic_ctx *ctx, const int *fields, double *const *host, int count);
int mic_nodal_device_ptr(mic_ctx *ctx, int field, double **device_ptr);

/* ---- the marker path; each entry point replaces the reference function cited ---- */
/* findMarkerCells (markers.c:85-106; markers.h:15) plus the stable counting sort by cell
 * that orders the device columns; *n_out = markers outside the domain (MarkerSet.nOut). */
int mic_find_marker_cells(mic_ctx *ctx, int64_t *n_out);
/* density update inline in main_subduction.c:255-264 */
int mic_update_marker_rho(mic_ctx *ctx);
/* maximum marker temperature, main_subduction.c:271-289 */
int mic_max_marker_T(mic_ctx *ctx, double *max_T);
/* projectMarkersNodesAll2 (markerProjection.c:11-68; markerProjection.h:11) */
int mic_project_markers_nodes_all2(mic_ctx *ctx);
/* projectMarkerFieldToNodes (markerProjection.c:71-250; markerProjection.h:10).  The marker
 * field is named by its byte offset inside the record (the reference passes &markers[0].field
 * and strides by sizeof(Marker)); pass material_property (MIC_MAXMAT values) instead to
 * project a per-material constant, as with materialkThermal / materialCp. */
int mic_project_marker_field_to_nodes(mic_ctx *ctx, int marker_field_offset, const double *material_property,
                                      int out_field, int stagx, int stagy, int method);
/* projectNodalFieldToMarkersS (markers.c:1670-1706; markers.h:21) */
int mic_project_nodal_field_to_markers(mic_ctx *ctx, int nodal_field, int marker_field_offset);
/* checkPlasticYielding (markers.c:1381-1505; markers.h:14) with computeRheology
 * (viscosity.c:12-67) */
int mic_check_plastic_yielding(mic_ctx *ctx, double dt, int *is_yielding, double elapsed_time);
/* updateViscosity (viscosity.c:77-88; viscosity.h:2) */
int mic_update_viscosity(mic_ctx *ctx);
/* limitViscosity (viscosity.c:90-104; viscosity.h:3) */
int mic_limit_viscosity(mic_ctx *ctx);
/* updateMarkerStrainPressure (updateMarkerStrainPressure.c:9-399; updateMarkerStrainPressure.h:1) */
int mic_update_marker_strain_pressure(mic_ctx *ctx, double dt);
/* updateGlobalStrainRateResidual (residual.c:12-51; residual.h:4) */
int mic_update_global_strain_rate_residual(mic_ctx *ctx, int iter, double *residual);
/* checkConvergence (residual.c:53-69; residual.h:5) over the stored residuals */
int mic_check_convergence(mic_ctx *ctx, double atol, double rtol, int iter, int *converged);
/* getGlobalStrainRateResidual / setGlobalStrainRateResidual (residual.c; residual.h:2-3): the
 * stored residual of iteration iter (100 slots) */
int mic_get_strain_rate_residual(mic_ctx *ctx, int iter, double *value);
int mic_set_strain_rate_residual(mic_ctx *ctx, int iter, double value);
/* subgridStressChanges (subgridStressChanges.c:5-318; subgridStressChanges.h:1) */
int mic_subgrid_stress_changes(mic_ctx *ctx, double dt, double diffusivity);
/* updateMarkerStress (updateMarkerStress.c:5-163; updateMarkerStress.h:1) */
int mic_update_marker_stress(mic_ctx *ctx);
/* subgridTemperatureChanges (subgridTemperatureChanges.c:5-124; subgridTemperatureChanges.h:2);
 * the new temperature (the reference's thisT argument) is nodal field MIC_NF_THIST */
int mic_subgrid_temperature_changes(mic_ctx *ctx, double dt);
/* advectMarkersRK (markers.c:1865-2250; markers.h:20) */
int mic_advect_markers_rk(mic_ctx *ctx, double dt);
/* maximum |sxx| over in-domain markers, main_subduction.c:437-448 */
int mic_max_abs_sxx(mic_ctx *ctx, double *max_abs_sxx);

/* ---- one time step of the marker path, in main_subduction.c order (main:243-448) ----
 * pre_stokes:   findMarkerCells, density update, projectMarkersNodesAll2, max T,
 *               checkPlasticYielding, limitViscosity, projectMarkersNodesAll2
 * post_stokes:  updateMarkerStrainPressure, updateGlobalStrainRateResidual,
 *               subgridStressChanges (when subgrid_stress != 0), updateMarkerStress
 * post_thermal: subgridTemperatureChanges, advectMarkersRK, max |sxx|
 * mic_step runs all three with the nodal inputs already on the device. */
int mic_step_pre_stokes(mic_ctx *ctx, double dt_disp, int *is_yielding, double *max_T);
int mic_step_post_stokes(mic_ctx *ctx, double dt_disp, int subgrid_stress, double *residual);
int mic_step_post_thermal(mic_ctx *ctx, double dt_thermal, double *max_abs_sxx);
int mic_step(mic_ctx *ctx, double dt_disp, double dt_thermal, int subgrid_stress, double *residual);

/* ---- composite ice creep closure (material law 7; no reference counterpart) ----
 * fvmic2d evaluates the Goldsby-Kohlstedt law forwards only (goldsbyKohlstedt, viscosity.c:
 * 106-179, stress -> strain rate).  Law 7 inverts it per marker: the viscosity is s* / (2 edot_II)
 * where s* is the stress at which the law's strain rate equals the marker's strain-rate
 * invariant (grain size from mic_markers_set_grain_size, pressure and temperature from the
 * marker).  mode 0 solves exactly (FP64 Newton to |rate/edot - 1| <= tol).  Modes 1 and 2 start
 * from the trained surrogate, a 4 -> 64 -> 64 -> 1 MLP whose hidden-layer weights are BF16:
 * mode 1 on the CUDA cores in FP32; mode 2 with the hidden layer on the tensor cores, BF16
 * weights against the FP32 activations as two BF16 pieces, FP32 accumulation.  They take up to
 * polish_iters Halley steps and finish with the exact solve for markers still above polish_tol.
 * For polish_tol >= 1e-9 the polish runs in double-float arithmetic on the FP32 pipe, with the
 * law's terms to a relative 1e-11; below 1e-9 it runs in FP64.  With polish_tol = tol the
 * surrogate modes converge to the same root as mode 0. */
int mic_creep_configure(mic_ctx *ctx, int mode, double tol, int maxit, int polish_iters, double polish_tol);
int mic_markers_set_grain_size(mic_ctx *ctx, const double *grain_size, int64_t n); /* caller order */
int mic_creep_param_count(void);
/* the network's parameters (mic_creep_param_count floats); set_mlp rounds the hidden layer's
 * weights W2 to BF16 (round to nearest even), so get_mlp returns them rounded */
int mic_creep_set_mlp(mic_ctx *ctx, const float *params, int n);
int mic_creep_get_mlp(mic_ctx *ctx, float *params, int n);
/* train the surrogate on the GPU from nsamples exact solves (Adam, cosine decay, batch % 128 == 0);
 * quantization-aware: forward and backward passes use W2 rounded to BF16, the trained W2 is
 * rounded at the end */
int mic_creep_train(mic_ctx *ctx, int64_t nsamples, int batch, int steps, float lr, unsigned long long seed,
                    float *loss_history);
/* mean-squared-loss gradient of the training kernels at params over n samples (n % 128 == 0) */
int mic_creep_mlp_grad(mic_ctx *ctx, const float *params, const float *features, const float *targets, int n,
                       float *grad, float *loss);
/* batch solve from host arrays: mode 0 exact, 1 surrogate (CUDA-core inference), 2 surrogate
 * (tensor-core inference); outputs may be NULL except stress */
int mic_creep_solve_batch(mic_ctx *ctx, const double *edot, const double *T, const double *d, const double *P,
                          int64_t n, int mode, double *stress, int32_t *iterations, double *residual,
                          int32_t *fallback);
/* surrogate network outputs y[n] for normalised features feat[n][4] (host arrays) with the
 * context's parameters: mode 1 FP32 on the CUDA cores, mode 2 hidden layer on the tensor cores */
int mic_creep_mlp_infer(mic_ctx *ctx, const float *feat, int64_t n, int mode, float *y);
/* the same entry points under the names of the reference-side plan: exact Newton batch solve
 * (mic_creep_solve_batch, mode 0), surrogate training and inference */
int mic_creep_newton(mic_ctx *ctx, const double *edot, const double *T, const double *d, const double *P, int64_t n,
                     double *stress, int32_t *iterations, double *residual);
int mic_surrogate_train(mic_ctx *ctx, int64_t nsamples, int batch, int steps, float lr, unsigned long long seed,
                        float *loss_hist);
int mic_surrogate_infer(mic_ctx *ctx, const float *feat, int64_t n, int mode, float *y);
/* counters of the last law-7 pass (checkPlasticYielding or a batch solve): markers solved, Newton
 * iterations, exact fallbacks, largest final |rate/edot - 1|, tensor-core tiles whose completion
 * wait ran out (their markers took the exact solve) */
int mic_creep_stats(mic_ctx *ctx, int64_t *markers, int64_t *iterations, int64_t *fallbacks, double *max_residual,
                    int64_t *tc_timeouts);
/* the tensor-core inference's bounded completion wait: try_wait rounds per tile before a block
 * gives up on the tensor cores (default 2^20; 0 gives up at once, every marker then takes the
 * exact solve), and the last pass's counts of tiles that gave up and of blocks whose final
 * drain before freeing tensor memory ran out as well (nonzero only if the tensor pipe never
 * signalled) */
int mic_creep_set_tc_wait_limit(mic_ctx *ctx, int rounds);
int mic_creep_tc_stats(mic_ctx *ctx, int64_t *tile_timeouts, int64_t *drain_timeouts);

/* ---- plumbing ---- */
int mic_synchronize(mic_ctx *ctx);
int mic_get_stream(mic_ctx *ctx, void **stream);
int mic_get_status(mic_ctx *ctx, mic_status *status);
/* device order of the caller's marker indices and the per-cell start offsets
 * ((NX-1)*(NY-1)+2 entries; the last two bracket the out-of-domain markers) */
int mic_debug_sorted_ids(mic_ctx *ctx, int32_t *ids);
int mic_debug_cell_start(mic_ctx *ctx, int32_t *cell_start);
/* num[k] / den[k] (host arrays) computed the way the kernels divide by a grid spacing: the
 * correctly rounded reciprocal and one residual correction (the FMA-free build divides) */
int mic_debug_div_sp(mic_ctx *ctx, const double *num, const double *den, int64_t n, double *quot);
/* kernel launches issued by this context so far */
int mic_launch_count(mic_ctx *ctx, int64_t *launches);
/* per-launch CUDA-event timing on the context stream: enable with a record capacity (0 turns it
 * off); read aggregates by kernel name (names: max * 48 bytes) */
int mic_profile_enable(mic_ctx *ctx, int capacity);
int mic_profile_read(mic_ctx *ctx, int max, char *names, double *total_ms, int64_t *counts, int *nkernels);
/* Launch shapes (new; the reference has no counterpart).  The marker-parallel kernels of a step
 * each launch with one block size.  mic_autotune measures 128, 256 and 512 threads for each on
 * this context's workload: it saves the marker columns and nodal fields, runs for every candidate
 * one untimed and `steps` timed mic_step calls (dt_disp, dt_thermal, subgrid_stress as mic_step)
 * from the saved state, keeps per kernel the fastest size, and puts the saved state back, so the
 * simulation is where it was.  chosen (MIC_TUNE_COUNT ints, may be NULL) receives the sizes.
 * Results of a step do not depend on the sizes.  mic_get_tuning / mic_set_tuning read and set
 * them (0 = the default, 256), e.g. to reuse one tuning for many contexts of one workload. */
enum {
  MIC_TUNE_ADVECT = 0,
  MIC_TUNE_STRAIN,
  MIC_TUNE_YIELD,
  MIC_TUNE_SUBGRID_STRESS,
  MIC_TUNE_UPDATE_STRESS,
  MIC_TUNE_SUBGRID_T,
  MIC_TUNE_SUBGRID_T_APPLY,
  MIC_TUNE_REORDER,
  MIC_TUNE_FIND_CELLS,
  MIC_TUNE_UPDATE_RHO,
  MIC_TUNE_COUNT
};
int mic_autotune(mic_ctx *ctx, double dt_disp, double dt_thermal, int subgrid_stress, int steps, int *chosen);
int mic_get_tuning(mic_ctx *ctx, int *block, int count);
int mic_set_tuning(mic_ctx *ctx, const int *block, int count);
/* ---- marker lifecycle (markers.c:15-39, 255-400) ----
 * resetMarkers: every slot of the capacity gets resetMarker's values (X = Y = -1, Mat = -1, the
 * kinematic, thermal, stress, strain and density fields 0; mu, cellX, cellY, cpu and the
 * strain-rate residual untouched).  The marker count is unchanged. */
int mic_reset_markers(mic_ctx *ctx);
/* resetMarker's values on a host marker array (no device work): for host code that owns the array
 * before a context exists (allocateMarkers, markers.c:15-27) */
int mic_markers_reset_host(mic_marker *markers, int64_t n);
/* current number of markers (MarkerSet.nMark) */
int mic_marker_count(mic_ctx *ctx, int64_t *n);
/* distributeMarkersUniformInDomain on one rank: NMX x NMY markers per basic cell of the
 * domain-wide lattice (mdx = LX / (NMX (NX-1)), marker k*nyl + l at x0 + mdx (0.5 + k) plus a
 * U(-mdx/4, mdx/4) jitter, likewise in y), jitter drawn in marker order from the 48-bit stream
 * the reference's PETSc random object is seeded with (seed 0 reproduces the reference).  Sets
 * the marker count (*n_placed); other fields keep their values (call mic_reset_markers first). */
int mic_distribute_markers_uniform_in_domain(mic_ctx *ctx, int NMX, int NMY, unsigned long seed, int64_t *n_placed);
/* set one marker field, addressed as offsetof(mic_marker, field), to value for every marker
 * (integer fields take (int)value) -- the per-marker initial-condition loops of the host code */
int mic_markers_fill(mic_ctx *ctx, int field_offset, double value);

/* projectMarkersNodesFromScalar (markers.c:1507): a per-marker array (caller order, n values)
 * projected onto the basic nodes and divided by the weights, into nodal field out_field */
int mic_project_markers_nodes_from_scalar(mic_ctx *ctx, const double *values, int out_field);

/* ---- grid routines between the solves ----
 * nodalStressStrain (nodalStressStrain.c:6): from vx, vy (MIC_NF_VX/VY), etaN/S, muN/S and the
 * old stresses: deviatoric strain rates (edotxx, edotyy at cell centres, edotxy at basic nodes),
 * vorticity wxy, visco-elastic stress update (soxx, soyy, soxy) and stress changes (dsxx, dsyy,
 * dsxy), shear heating (MIC_NF_HEATING) and the invariants MIC_NF_EII / MIC_NF_SII at interior
 * basic nodes.  Walls from mic_set_bcs.  gy is the reference's unused gravity argument. */
int mic_nodal_stress_strain(mic_ctx *ctx, double dt, double gy);
/* limitDisplacementTimestep (limitTimestep.c:6): *dt = min(*dt, factor times the crossing time of
 * the smaller adjacent cell at every nodal vx, vy, 1% of rho / rhodot), then 0.01 / max |rhodot|
 * (factor = Options.displacementStepLimit) */
int mic_limit_displacement_timestep(mic_ctx *ctx, double factor, double *dt);
/* retrieveSolutions (retrieveSolutions.c:4): vx, vy, p from the solver's vector S
 * ([(j NX + i) 3 + {0 vx, 1 vy, 2 p}], host memory), p scaled by Kcont, minus the dx-weighted
 * mean of row 1 on every j, i >= 1.  The reference also scales the pressure entries of S in
 * place; here S is only read.  S = NULL takes the solution mic_linear_solve left on the device.
 * *foundnan = 0 (the reference checks only in its TEXTURE build). */
int mic_retrieve_solutions(mic_ctx *ctx, const double *S, double Kcont, int *foundnan);

/* ---- marker checkpoints (io.c:299-402, restart.c:8-125) ----
 * The reference's field-major binary format: int32 count of in-domain markers, float64 elapsed
 * time, then cpu, cellX, cellY (int32), X, Y, VX, VY (float64), Mat (int32), T, Tdot, eta, mu,
 * e11, e12, Eii, s11, s22, s12, p, rho, rhodot (float64), each over the markers with cellX != -1
 * in the caller's order.  The reference names the file output/Markers.<iMonte>.<iTime>; here the
 * caller passes the path.  Restart resets the marker set (as allocateMarkers does), fills the
 * file's markers in file order and bins them (findMarkerCells); MIC_ERR_CAPACITY when the file
 * holds more markers than the context. */
int mic_save_markers_binary(mic_ctx *ctx, const char *path, double elapsed_time);
int mic_restart_from_markers(mic_ctx *ctx, const char *path, double *elapsed_time);

/* ---- marker density control ----
 * checkMarkerDensity (markers.c:455-781): bins the markers if their positions changed (the
 * findMarkerCells the reference calls first, main:247), counts markers per basic quarter cell,
 * removes random markers (drand48) from quarter cells above maxMarkers, adds markers at random
 * positions (the reference's PETSCRAND48 object, which shares the drand48 stream) to quarter
 * cells below minMarkers, recycling out-of-domain slots last-in first-out before appending, and
 * gives each new marker its nearest neighbour's properties -- or, left of x[1] and right of
 * x[NX-2] below the overriding plate, those of a subduction inflow marker
 * (benchmarkInitialConditions.c:44-66; cpu and strainRateResidual, which the reference leaves
 * uninitialised there, are 0).  MIC_ERR_CAPACITY where the reference aborts on a full marker
 * array.  The marker count changes; *n_added / *n_removed report what was done. */
int mic_check_marker_density(mic_ctx *ctx, const mic_density_options *options, int64_t *n_added, int64_t *n_removed);
/* the drand48 stream density control draws from: srand48(seed) (the reference seeds 1, the
 * default), or read / replace the 48-bit state */
int mic_density_seed(mic_ctx *ctx, long seed);
int mic_density_rng_state(mic_ctx *ctx, uint64_t *get, const uint64_t *set);
/* rounds the last mic_check_marker_density took to settle which marker each new marker copies:
 * 0 nothing added; -1 a slot was recycled twice (the reference's over-asked removal), so the new
 * markers were filled one at a time in order; below -1 no fixed point within that many rounds,
 * filled in order too */
int mic_density_fill_rounds(mic_ctx *ctx, int *rounds);

/* ---- the linear systems of a time step ----
 * Assembly on the device from the context's nodal arrays, rows in the reference's ordering
 * (3 (j NX + i) + dof, dof 0 vx, 1 vy, 2 p, for Stokes; j NX + i for temperature), every entry
 * bit-identical to the reference's: the Stokes system (formVEPSystem, vep_system.c:12-726;
 * the caller's P matrix is not built: the reference's solve uses the system matrix itself),
 * the thermal boundary values of lastT (enforceThermalBCs1, enforceThermalBC.c:5-38) and the
 * thermal system, whose right-hand side starts as the heating field (MIC_NF_HEATING), as
 * main_subduction.c:381 copies nodal_heating into it (formThermalSystem,
 * formThermalSystem.c:6-249).  The slab / plate geometry is benchmarkInitialConditions.c's. */
int mic_form_vep_system(mic_ctx *ctx, const mic_subduction_options *options, double dt, double *Kbond,
                        double *Kcont);
int mic_enforce_thermal_bcs(mic_ctx *ctx, const mic_subduction_options *options);
int mic_form_thermal_system(mic_ctx *ctx, const mic_subduction_options *options, double dt, int doSteady);
/* which: 0 Stokes, 1 thermal.  Size, and a copy as CSR with ascending columns. */
int mic_system_size(mic_ctx *ctx, int which, int64_t *nrows, int64_t *nnz);
int mic_system_get(mic_ctx *ctx, int which, int32_t *rowptr, int32_t *cols, double *vals, double *rhs);
/* kspLinearSolve (kspLinearSolve.c:13) as the reference's option files run it (preonly + LU,
 * option_files/run_mumps.petscopt): a direct solve on the device, banded LU with partial
 * pivoting.  The Stokes solution stays on the device for mic_retrieve_solutions(ctx, NULL, ...);
 * the temperature goes to MIC_NF_THIST.  MIC_ERR_SOLVE for a zero pivot. */
int mic_linear_solve(mic_ctx *ctx, int which);
int mic_solution_get(mic_ctx *ctx, int which, double *out);
/* band widths (lower, upper) the last solve of a system factorised */
int mic_system_band(mic_ctx *ctx, int which, int *kl, int *ku);

/* One time step of main_subduction.c (227-460) without PETSc, everything on the device:
 * findMarkerCells, checkMarkerDensity (when options->densityControl), the marker density
 * anomaly, projection and melting check, then plasticity iterations (checkPlasticYielding,
 * limitViscosity, projection, the Stokes system and its direct solve, retrieveSolutions,
 * nodalStressStrain, updateMarkerStrainPressure, the strain-rate residual and convergence test,
 * limitDisplacementTimestep), subgridStressChanges (when the options' diffusivity is positive),
 * updateMarkerStress, the thermal system and its solve (again with a shorter step when the
 * largest nodal change exceeds maxTempChange), subgridTemperatureChanges and advectMarkersRK.
 * elapsed_time is the model time before the step (checkPlasticYielding's t); the caller adds
 * report->dt.  A step whose markers are above the reference's TBREAK (9999 K) stops after the
 * projection with report->stopped = 1, as main goes to the next Monte-Carlo run.  With
 * options->staticVelocity the Stokes system is assembled and solved once per context (the run's
 * first step, main:306-318) and its solution reused afterwards. */
int mic_subduction_timestep(mic_ctx *ctx, const mic_timestep_options *options, double elapsed_time,
                            mic_timestep_report *report);
/* adiabaticHeating (adiabaticHeating.c:7): every in-domain marker's alpha T VY rho gy projected to
 * the basic nodes (weights (1 - mdx)(1 - mdy), ..., divided by their sum), added to
 * MIC_NF_HEATING as main_subduction.c:377 adds it (VecAXPY(nodal_heating, 1.0, ha)) */
int mic_adiabatic_heating(mic_ctx *ctx, double gy);
/* main's per-step diagnostics (main_subduction.c:413-416): nusseltNumber (post.c:5) of the new
 * temperature MIC_NF_THIST with the boundary temperatures (thermalBCBottom.value[0],
 * thermalBCTop.value[0]), bit-identical; rmsVelocity (post.c:49) of the nodal vx, vy, summed by a
 * fixed tree instead of the reference's cell order (rounding differences only) */
int mic_nusselt_number(mic_ctx *ctx, double bottom_T, double top_T, double *Nu);
/* set-up of main (main_subduction.c:176-183): resetNodalFields (nodalFields.c:155) zeroes every
 * nodal field; initialConditionsVanKeken (benchmarkInitialConditions.c:8) gives every marker the
 * subduction benchmark's temperature (slab inflow profile, plate geotherm or mantle), material 0,
 * rho, rhodot = 0 and its viscosity, and sets the left (slab velocity) and top (no slip) boundary
 * conditions, as the reference sets them in its Options */
int mic_reset_nodal_fields(mic_ctx *ctx);
int mic_initial_conditions_van_keken(mic_ctx *ctx, const mic_subduction_options *options);
int mic_rms_velocity(mic_ctx *ctx, double *vrms);
/* No counterpart in the reference, whose main runs its Monte-Carlo realisations one after another
 * (iMonte): one mic_subduction_timestep on each of n independent contexts (each created with its
 * own stream), members on up to max_threads host threads at once (0: the host's core count), so
 * that their sequential parts overlap on the GPU.  options, elapsed_time (NULL: 0), reports and
 * codes (NULL allowed) have one entry per member; returns the first member's non-zero code.
 * Create every member before the call: mic_create's synchronous copies would disturb the
 * members' graph captures. */
int mic_subduction_timestep_many(mic_ctx *const *ctxs, int n, const mic_timestep_options *options,
                                 const double *elapsed_time, mic_timestep_report *reports, int *codes,
                                 int max_threads);

/* ---- ensembles ----
 * No counterpart in the reference (one problem per run; main_subduction.c:167-171 only reads an
 * iMonte option).  Independent problems, each a context with its own stream, stepped together:
 * one mic_ensemble_step is every member's mic_step (no residual read), with the same results as
 * each member stepped alone.  Batched (the default), each marker pass of the step is one kernel
 * over a work table of (member, tile) pairs for the members of a batch group, and the members'
 * other launches (binning, projections, node kernels) run on their own streams between the
 * passes; per-member, each member's whole step runs on its stream and small members overlap.  With
 * use_graph the whole ensemble step is captured as CUDA graphs on the first call and replayed as
 * one launch afterwards (re-captured when a member's settings, marker count or the time steps
 * change).  Asynchronous: mic_ensemble_synchronize waits; member streams are ordered after each
 * step.  Members stay owned by the caller and must outlive the ensemble. */
typedef struct mic_ensemble mic_ensemble;
int mic_ensemble_create(mic_ensemble **out, mic_ctx *const *members, int n_members);
int mic_ensemble_destroy(mic_ensemble *ens);
int mic_ensemble_step(mic_ensemble *ens, const double *dt_disp, const double *dt_thermal, int subgrid_stress,
                      int use_graph);
int mic_ensemble_synchronize(mic_ensemble *ens);
/* How a step runs its marker passes (new): groups 0 = each member's own kernels on its stream;
 * groups 1..8 = members dealt to that many batch groups by marker count (largest first, each to
 * the group with the fewest markers), one kernel per marker pass per group over the group's
 * (member, tile) table, the groups running beside one another.  Batched kernels cut each
 * member's markers into tiles of tile_mult (1..64) blocks' worth and run one block per tile
 * (persistent 0) or a persistent grid of SMs x resident blocks whose blocks take tiles
 * round-robin (chunked 0), one contiguous run each (1) or the next tile from a counter the grid
 * shares (2); tiles are ordered member by member in the issue order.  The surrogate yield passes
 * always take one-block tiles from a counter on a persistent grid (members whose networks are
 * equal read one copy).  Default: 4, 4, 1, 2. */
int mic_ensemble_set_schedule(mic_ensemble *ens, int groups, int tile_mult, int persistent, int chunked);
int mic_ensemble_get_schedule(mic_ensemble *ens, int *groups, int *tile_mult, int *persistent, int *chunked);
/* Launch shapes and member schedule measured on the ensemble (new): mic_autotune on every member,
 * then the fastest captured step among per-member steps in three issue orders (as given, largest
 * first, smallest first) and batched passes in 1, 2, 4 and 8 groups with three walks (tile_mult,
 * persistent, chunked = 1,0,0; 4,1,1; 4,1,2), each timed over 2 x steps graph replays from saved
 * member states.  The winner becomes the ensemble's schedule (mic_ensemble_get_schedule); every
 * member's state is restored; order_out (n_members ints, may be NULL) receives the member order. */
int mic_ensemble_autotune(mic_ensemble *ens, const double *dt_disp, const double *dt_thermal, int subgrid_stress,
                          int steps, int *order_out);
/* kernels issued through the ensemble so far, and kernels inside one captured step */
int mic_ensemble_launch_count(mic_ensemble *ens, int64_t *launches, int64_t *graph_kernels);
int mic_ensemble_get_stream(mic_ensemble *ens, void **stream);

/* ---- binning without allocation ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc -- a host that
 * forbids device allocation once it has started, or a plug-in whose application owns the
 * allocator -- this bins markers and returns their stable cell order without allocating
 * anything: the caller passes device pointers for every input and output, and the sort's
 * scratch lives in a fixed device array inside the library, reserved when the library is
 * loaded on a device and kept until the process exits.
 *   X, Y [n]          marker positions (device), any order
 *   x [NX], y [NY]    basic gridlines (device), increasing, x[0] >= 0, y[0] >= 0
 *   cellX, cellY [n]  out: findMarkerCells' cells (markers.c:41-106), -1 outside the domain
 *   perm [n]          out: perm[k] = index of the marker at sorted position k (stable by cell)
 *   cell_start [(NX-1)*(NY-1)+2]  out: first sorted position of each cell; the last two
 *                     entries bracket the out-of-domain markers
 *   stream            cudaStream_t to run on (NULL: the legacy default stream)
 *   n_out             optional host pointer: markers outside the domain (synchronises stream)
 * Limits: n <= MIC_NOALLOC_MAX_MARKERS and (NX-1)*(NY-1) <= MIC_NOALLOC_MAX_CELLS, else
 * MIC_ERR_CAPACITY.  The first call in a CUDA context (on each device, and again after a
 * cudaDeviceReset) looks up the array's device address, so make that first call before
 * capturing a stream.  All calls share the one array: calls that overlap on the GPU race and
 * must be ordered by the caller. */
#define MIC_NOALLOC_MAX_MARKERS 1048576
#define MIC_NOALLOC_MAX_CELLS 1048576
int mic_bin_sort_noalloc(const double *X, const double *Y, int64_t n, const double *x, const double *y, int NX,
                         int NY, double LX, double LY, int32_t *cellX, int32_t *cellY, int32_t *perm,
                         int32_t *cell_start, void *stream, int64_t *n_out);
/* pinned host memory for fast transfers */
int mic_host_alloc(void **ptr, int64_t bytes);
int mic_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif
