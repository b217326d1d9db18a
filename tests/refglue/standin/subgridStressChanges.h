/* Stand-in for fvmic2d's subgridStressChanges.h.  TEST INFRASTRUCTURE ONLY. */
PetscErrorCode subgridStressChanges(GridData *, NodalFields *, MarkerSet *, Materials *, PetscScalar, PetscScalar);
