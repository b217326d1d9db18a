/* Prints the size of fvmic2d's records and the offset of each of their members, one per line.
 * Compiled once against the reference's fdcode.h and once against the stand-in
 * (tests/refglue/standin/fdcode.h); the two outputs must be equal.  TEST INFRASTRUCTURE ONLY. */
#include <stddef.h>
#include <stdio.h>

#include "fdcode.h"

#define SZ(T) printf(#T " %zu\n", sizeof(T))
#define OFF(T, m) printf(#T "." #m " %zu\n", offsetof(T, m))

int main(void) {
  SZ(GridData);
  OFF(GridData, da); OFF(GridData, vda); OFF(GridData, LX); OFF(GridData, LY); OFF(GridData, NX);
  OFF(GridData, NY); OFF(GridData, mp); OFF(GridData, np); OFF(GridData, x); OFF(GridData, y);
  OFF(GridData, xc); OFF(GridData, yc); OFF(GridData, xperiodic); OFF(GridData, yperiodic);
  SZ(NodalFields);
  OFF(NodalFields, rho); OFF(NodalFields, rhodot); OFF(NodalFields, etaS); OFF(NodalFields, etaN);
  OFF(NodalFields, thisT); OFF(NodalFields, lastT); OFF(NodalFields, kThermal); OFF(NodalFields, Cp);
  OFF(NodalFields, boundaryT); OFF(NodalFields, edotxx); OFF(NodalFields, edotxy); OFF(NodalFields, edotyy);
  OFF(NodalFields, edotzz); OFF(NodalFields, edotxz); OFF(NodalFields, edotyz); OFF(NodalFields, soxx);
  OFF(NodalFields, soxy); OFF(NodalFields, soyy); OFF(NodalFields, dsxx); OFF(NodalFields, dsyy);
  OFF(NodalFields, dsxy); OFF(NodalFields, muS); OFF(NodalFields, muN); OFF(NodalFields, vx);
  OFF(NodalFields, vy); OFF(NodalFields, p); OFF(NodalFields, eii); OFF(NodalFields, sii); OFF(NodalFields, wxy);
  OFF(NodalFields, ha); OFF(NodalFields, nodalHeating); OFF(NodalFields, VPTensorC); OFF(NodalFields, VPTensorB);
  OFF(NodalFields, strainRateResidual);
  SZ(Marker); OFF(Marker, Mat); OFF(Marker, T); OFF(Marker, s); OFF(Marker, e); OFF(Marker, E);
  OFF(Marker, cellX); OFF(Marker, strainRateResidual); OFF(Marker, isYielding);
  SZ(MarkerSet); OFF(MarkerSet, nMark); OFF(MarkerSet, maxMark); OFF(MarkerSet, nOut); OFF(MarkerSet, markers);
  SZ(Materials); OFF(Materials, hasPlasticity); OFF(Materials, gamma); OFF(Materials, hasEtaT); OFF(Materials, Tref);
  SZ(BCInfo); SZ(BoundaryValues); OFF(BoundaryValues, mechBCTop);
  SZ(Options);
  OFF(Options, NX); OFF(Options, NY); OFF(Options, LX); OFF(Options, LY); OFF(Options, NMX); OFF(Options, NMY);
  OFF(Options, gridRatio); OFF(Options, nTime); OFF(Options, restartStep); OFF(Options, totalTime);
  OFF(Options, maxNumPlasticity); OFF(Options, plasticDelay); OFF(Options, Tperturb); OFF(Options, shearHeating);
  OFF(Options, adiabaticHeating); OFF(Options, gy); OFF(Options, gx); OFF(Options, gz); OFF(Options, mechBCLeft);
  OFF(Options, mechBCRight); OFF(Options, mechBCTop); OFF(Options, mechBCBottom); OFF(Options, thermalBCLeft);
  OFF(Options, thermalBCRight); OFF(Options, thermalBCTop); OFF(Options, thermalBCBottom);
  OFF(Options, fractionalEtamin); OFF(Options, etamin); OFF(Options, etamax); OFF(Options, dtMax);
  OFF(Options, displacementStepLimit); OFF(Options, maxTempChange); OFF(Options, saveInterval);
  OFF(Options, markerSaveInterval); OFF(Options, subgridStressDiffusivity);
  OFF(Options, subgridTemperatureDiffusivity); OFF(Options, maxMarkFactor); OFF(Options, minMarkers);
  OFF(Options, maxMarkers); OFF(Options, grainSize); OFF(Options, overridingPlateThickness); OFF(Options, slabAge);
  OFF(Options, slabAngle); OFF(Options, slabVelocity); OFF(Options, rootThickness); OFF(Options, rootCenter);
  OFF(Options, rootWidth); OFF(Options, staticVelocity); OFF(Options, minDecoupleDepth);
  OFF(Options, maxDecoupleDepth); OFF(Options, decoupleThickness); OFF(Options, decoupleEtaScaler);
  SZ(LinearSystem); OFF(LinearSystem, ns); OFF(LinearSystem, label);
  SZ(Problem);
  OFF(Problem, options); OFF(Problem, materials); OFF(Problem, grid); OFF(Problem, nodal_fields);
  OFF(Problem, markerset); OFF(Problem, mech_system); OFF(Problem, thermal_system); OFF(Problem, nodal_heating);
  return 0;
}
