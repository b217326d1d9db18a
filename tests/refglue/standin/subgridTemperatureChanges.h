/* Stand-in for fvmic2d's subgridTemperatureChanges.h.  TEST INFRASTRUCTURE ONLY. */
PetscErrorCode subgridTemperatureChanges(Vec, GridData *, NodalFields *, MarkerSet *, Materials *, PetscScalar,
                                         Options *);
