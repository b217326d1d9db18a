/* Stand-in for fvmic2d's updateMarkerStrainPressure.h.  TEST INFRASTRUCTURE ONLY. */
PetscErrorCode updateMarkerStrainPressure(GridData *, NodalFields *, MarkerSet *, Materials *, Options *, PetscScalar);
