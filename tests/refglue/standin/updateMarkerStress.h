/* Stand-in for fvmic2d's updateMarkerStress.h.  TEST INFRASTRUCTURE ONLY. */
PetscErrorCode updateMarkerStress(GridData *, NodalFields *, MarkerSet *, Materials *);
