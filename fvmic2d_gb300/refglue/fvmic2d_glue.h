/*
 * fvmic2d_glue.h -- what fvmic2d's own main() needs beyond the replaced routines when the
 * marker path runs on the GPU through libmic_gb300 (fvmic2d_glue.c).
 *
 * The glue keeps one marker set on the device.  Either the host array MarkerSet.markers or the
 * device copy is current, never both at once:
 *   - the replaced routines (findMarkerCells, projectMarkersNodesAll2, ..., advectMarkersRK)
 *     work on the device copy, uploading the host array first when it is the current one;
 *   - distributeMarkersUniformInDomain leaves the host array current, because main() fills the
 *     initial conditions on it next (initialConditionsVanKeken, main_subduction.c:182);
 *   - any other host code that reads or writes markers inside the time loop (saveMarkersBinary,
 *     restart output, diagnostics) calls micMarkersToHost first; the host array is then the
 *     current copy, and the next replaced routine uploads whatever the host code left in it.
 */
#ifndef FVMIC2D_GLUE_H
#define FVMIC2D_GLUE_H

#include "mic_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* the device copy into markerset->markers (no-op when the host array is already current) */
PetscErrorCode micMarkersToHost(MarkerSet *markerset);
/* the library context of the marker set (NULL before the first routine that knows the grid) */
mic_ctx *micGlueContext(void);
/* the GPU the glue creates its context on (default: device 0, or FVMIC2D_GPU in the environment);
 * call before the first routine */
void micGlueSetDevice(int device);
/* the loops main_subduction.c runs inline on the markers, on the device copy:
 * density update (main:255-264), maximum temperature (main:271-289), maximum |sxx| (main:437-448) */
PetscErrorCode micUpdateMarkerRho(MarkerSet *markerset, Materials *materials);
PetscScalar micMaxMarkerT(MarkerSet *markerset);
PetscScalar micMaxAbsSxx(MarkerSet *markerset);
/* the last library error code seen by a replaced routine whose reference signature returns void */
int micGlueLastError(void);

#ifdef __cplusplus
}
#endif

#endif
