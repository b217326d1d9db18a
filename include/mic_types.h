/*
 * mic_types.h -- data model shared by the GB300 marker-in-cell library, its
 * host-side callers and the CPU oracle.
 *
 * The marker record, the material table and the boundary-value table are
 * byte-compatible with fvmic2d's `Marker`, `Materials` and `BoundaryValues`
 * (fdcode.h:97-129, 74-95, 141-152; PetscScalar = double, PetscInt = int32).
 * Keeping the layout identical is what lets a caller hand the reference's
 * host `MarkerSet.markers` array (216-byte records, cellX at offset 184) to
 * the library without repacking.
 */
#ifndef MIC_TYPES_H
#define MIC_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MIC_MAXMAT 8 /* fdcode.h:11 */

typedef struct {
  double T11, T22, T12; /* fdcode.h:27-29 Tensor33s */
} mic_tensor33s;

/* One marker; same field order, types and padding as fdcode.h:97-129 (TEXTURE off). */
typedef struct {
  double X, Y;
  double VX, VY;
  int32_t Mat;
  double T, Tdot;
  mic_tensor33s s; /* deviatoric stress */
  double eta;      /* effective viscosity */
  double mu;       /* elastic shear modulus */
  double rho;      /* density anomaly */
  double rhodot;
  double p;        /* pressure */
  mic_tensor33s e; /* strain rate */
  mic_tensor33s E; /* total strain */
  double Eii;      /* accumulated strain invariant */
  double wxy;      /* vorticity */
  int32_t cellX, cellY, cpu;
  double strainRateResidual;
  int32_t isYielding;
} mic_marker;

/* Marker density control settings (fdcode.h:158-159, 193-204 Options fields read by
 * checkMarkerDensity and by the inflow markers it creates, benchmarkInitialConditions.c). */
typedef struct {
  int32_t NMX, NMY;               /* markers per cell at set-up */
  int32_t minMarkers, maxMarkers; /* per basic quarter cell */
  double slabAngle;               /* radians */
  double slabAge;                 /* Myr */
  double overridingPlateThickness, rootThickness, rootCenter, rootWidth;
} mic_density_options;

/* Options fields read by the Stokes and thermal assemblies (vep_system.c:12-726,
 * formThermalSystem.c:6-249, enforceThermalBC.c:5-38; fdcode.h:155-211) and the slab / plate
 * geometry they share with the inflow markers (benchmarkInitialConditions.c:75-145). */
typedef struct {
  double gx, gy;                   /* gravity components */
  double slabVelocity;             /* imposed slab speed, m/s */
  double slabAngle;                /* radians */
  double slabAge;                  /* Myr */
  double overridingPlateThickness, rootThickness, rootCenter, rootWidth;
  int32_t thermalBCTopType;        /* thermalBCTop.type[0]: 0 fixed temperature, 1 fixed gradient */
  double thermalBCTopValue;        /* thermalBCTop.value[0] */
} mic_subduction_options;

/* One time step of main_subduction.c (227-460) on the device: the Options fields it reads
 * besides the marker path's (fdcode.h:155-211) and the two sets above. */
typedef struct {
  double dtMax;                  /* first time step tried (main:242) */
  double displacementStepLimit;  /* limitDisplacementTimestep's factor */
  double maxTempChange;          /* largest nodal temperature change before the step shrinks (main:392) */
  int32_t maxNumPlasticity;      /* plasticity iterations at most */
  int32_t shearHeating;          /* 0: the nodal heating is zeroed before the thermal solve (main:372) */
  int32_t firstStep;             /* iTime == 0: one plasticity iteration even when converged (main:294) */
  int32_t densityControl;        /* run checkMarkerDensity (main:250) with `density` */
  mic_density_options density;
  mic_subduction_options sub;
  int32_t adiabaticHeating;      /* add adiabatic heating to the nodal heating (main:374-378) */
  int32_t staticVelocity;        /* reuse the run's first Stokes solution (main:306-318) */
  double thermalBCBottomValue;   /* thermalBCBottom.value[0], for the Nusselt number (post.c:10) */
} mic_timestep_options;

/* What the step did. */
typedef struct {
  double dt;                /* time step taken (the thermal one, main:371 and 393) */
  double displacement_dt;   /* the last plasticity iteration's displacement time step */
  double Kbond, Kcont;      /* scalings of the last Stokes system */
  double max_T;             /* largest marker temperature before the step (main:271-289) */
  double residual;          /* last global strain-rate residual (residual.c) */
  double max_temp_change;   /* largest nodal change of the accepted thermal solve */
  double max_abs_sxx;       /* main:437-448 */
  int32_t plastic_iterations, is_yielding, converged, thermal_resolves;
  int32_t stopped;          /* 1: max_T above 9999 (TBREAK), nothing after the projection ran */
  int64_t markers_added, markers_removed;
  double nusselt, vrms;     /* main's diagnostics after the thermal solve (post.c) */
} mic_timestep_report;

/* Material table; same layout as fdcode.h:74-95. */
typedef struct {
  int32_t nMaterials;
  double materialEta[MIC_MAXMAT];
  double materialRho[MIC_MAXMAT];
  double materialkThermal[MIC_MAXMAT];
  double materialCp[MIC_MAXMAT];
  double materialAlpha[MIC_MAXMAT];
  double materialMu[MIC_MAXMAT];
  double materialFriction[MIC_MAXMAT];
  double materialCohesion[MIC_MAXMAT];
  int32_t hasPlasticity[MIC_MAXMAT];
  double gamma[MIC_MAXMAT][2];
  double C[MIC_MAXMAT][2];
  double F[MIC_MAXMAT][2];
  int32_t hasEtaT[MIC_MAXMAT];
  double QonR[MIC_MAXMAT];
  double Tref[MIC_MAXMAT];
} mic_materials;

/* fdcode.h:141-152: type 0 = prescribed velocity, 1 = free slip, 2 = periodic. */
typedef struct {
  int32_t type[3];
  double value[3];
} mic_bcinfo;

typedef struct {
  mic_bcinfo mechBCLeft, mechBCRight, mechBCTop, mechBCBottom;
} mic_bcs;

/* The subset of fvmic2d's Options (fdcode.h:155-211) read on the marker path. */
typedef struct {
  double etamin, etamax, fractionalEtamin;             /* markers.c:1383-1385, viscosity.c:99-103 */
  double subgridStressDiffusivity;                      /* main_subduction.c:365 */
  double subgridTemperatureDiffusivity;                 /* subgridTemperatureChanges.c:7 */
  double slabAngle, decoupleThickness;                  /* viscosity.c:43-47 (hasEtaT == 6) */
  double minDecoupleDepth, maxDecoupleDepth, decoupleEtaScaler;
} mic_options;

/* Nodal field identifiers.  Every field is an NX*NY array of doubles, x fastest
 * ([j][i] = j*NX + i), i.e. the global-vector layout of fvmic2d's DMDA. */
enum {
  MIC_NF_RHO = 0,
  MIC_NF_RHODOT,
  MIC_NF_ETAS,      /* viscosity at basic nodes */
  MIC_NF_ETAN,      /* viscosity at cell centres */
  MIC_NF_THIST,     /* new temperature from the host thermal solve */
  MIC_NF_LASTT,
  MIC_NF_KTHERMAL,
  MIC_NF_CP,
  MIC_NF_EDOTXX,
  MIC_NF_EDOTXY,
  MIC_NF_EDOTYY,
  MIC_NF_SOXX,
  MIC_NF_SOXY,
  MIC_NF_SOYY,
  MIC_NF_DSXX,
  MIC_NF_DSYY,
  MIC_NF_DSXY,
  MIC_NF_MUS,
  MIC_NF_MUN,
  MIC_NF_VX,
  MIC_NF_VY,
  MIC_NF_P,
  MIC_NF_WXY,
  MIC_NF_SRR,       /* strain-rate residual projected to cell centres (residual.c:20) */
  MIC_NF_EII,       /* strain-rate second invariant at basic nodes (nodalStressStrain.c) */
  MIC_NF_SII,       /* stress second invariant at basic nodes */
  MIC_NF_HEATING,   /* shear heating at basic nodes (the nodalHeating argument) */
  MIC_NF_COUNT
};

/* Projection methods; same numbering as markerProjection.h PROJECTION_METHOD. */
enum { MIC_ARITHMETIC = 0, MIC_ARITHMETIC_LOCAL = 1, MIC_HARMONIC = 2 };

#ifdef __cplusplus
}
#endif

#endif
