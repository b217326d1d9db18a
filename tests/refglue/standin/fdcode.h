/*
 * Stand-in for fvmic2d's fdcode.h, for building the reference-side binding
 * (fvmic2d_gb300/refglue/fvmic2d_glue.c) and its test driver where the fvmic2d tree is not
 * present (the GPU test host).  TEST INFRASTRUCTURE ONLY.
 *
 * The records must be the reference's byte for byte, because the binding reads them as fvmic2d
 * lays them out: the marker, material and boundary-value records come from the library's own
 * restatement (include/mic_types.h); the grid, nodal-field, marker-set, options and problem
 * records are restated below member for member in the reference's order (fdcode.h:13-24, 40-71,
 * 131-137, 155-239).  tests/test_refglue_build.py compares every member offset and size with the
 * reference's header wherever the reference tree exists.  PETSc's types are petsc_lite's.
 */
#ifndef FVMIC2D_STANDIN_FDCODE_H
#define FVMIC2D_STANDIN_FDCODE_H

#include <stdio.h>
#include <stdlib.h>

#include "petscdmda.h"
#include "petscksp.h"

#include "mic_types.h"

#define MAXMAT 8

typedef mic_tensor33s Tensor33s;
typedef mic_marker Marker;
typedef mic_materials Materials;
typedef mic_bcinfo BCInfo;
typedef mic_bcs BoundaryValues;

/* the grid: DMDAs, extents, node counts, decomposition, gridlines with ghosts, periodicity */
typedef struct {
  DM da, vda;
  PetscScalar LX, LY;
  PetscInt NX, NY;
  PetscInt mp, np;
  PetscScalar *x, *y, *xc, *yc;
  PetscInt xperiodic, yperiodic;
} GridData;

/* nodal fields: global Vecs of the temperature DMDA */
typedef struct {
  Vec rho, rhodot, etaS, etaN;
  Vec thisT, lastT, kThermal, Cp;
  PetscScalar boundaryT;
  Vec edotxx, edotxy;
  Vec edotyy, edotzz, edotxz, edotyz;
  Vec soxx, soxy;
  Vec soyy;
  Vec dsxx, dsyy, dsxy;
  Vec muS, muN;
  Vec vx, vy, p;
  Vec eii, sii, wxy;
  Vec ha;
  Vec nodalHeating;
  Vec VPTensorC;
  Vec VPTensorB;
  Vec strainRateResidual;
} NodalFields;

typedef struct {
  PetscInt nMark;
  PetscInt maxMark;
  PetscInt nOut;
  Marker *markers;
} MarkerSet;

typedef struct {
  PetscInt NX, NY;
  PetscScalar LX, LY;
  PetscInt NMX;
  PetscInt NMY;
  PetscScalar gridRatio;
  PetscInt nTime;
  PetscInt restartStep;
  PetscScalar totalTime;
  PetscInt maxNumPlasticity;
  PetscInt plasticDelay;
  PetscScalar Tperturb;
  PetscInt shearHeating, adiabaticHeating;
  PetscScalar gy;
  PetscScalar gx;
  PetscScalar gz;
  BCInfo mechBCLeft, mechBCRight, mechBCTop, mechBCBottom;
  BCInfo thermalBCLeft, thermalBCRight, thermalBCTop, thermalBCBottom;
  PetscScalar fractionalEtamin;
  PetscScalar etamin;
  PetscScalar etamax;
  PetscScalar dtMax;
  PetscScalar displacementStepLimit;
  PetscScalar maxTempChange;
  PetscInt saveInterval;
  PetscInt markerSaveInterval;
  PetscScalar subgridStressDiffusivity;
  PetscScalar subgridTemperatureDiffusivity;
  PetscScalar maxMarkFactor;
  PetscInt minMarkers, maxMarkers;
  PetscScalar grainSize;
  PetscScalar overridingPlateThickness;
  PetscScalar slabAge;
  PetscScalar slabAngle;
  PetscScalar slabVelocity;
  PetscScalar rootThickness;
  PetscScalar rootCenter;
  PetscScalar rootWidth;
  PetscInt staticVelocity;
  PetscScalar minDecoupleDepth;
  PetscScalar maxDecoupleDepth;
  PetscScalar decoupleThickness;
  PetscScalar decoupleEtaScaler;
} Options;

typedef struct {
  Mat lhs;
  Mat pc;
  Vec rhs;
  Vec solution;
  MatNullSpace ns;
  char label[80];
} LinearSystem;

typedef struct {
  Options options;
  Materials materials;
  GridData grid;
  NodalFields nodal_fields;
  MarkerSet markerset;
  LinearSystem mech_system;
  LinearSystem thermal_system;
  Vec nodal_heating;
} Problem;

#endif
