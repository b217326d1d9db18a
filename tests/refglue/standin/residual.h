/* Stand-in for fvmic2d's residual.h.  TEST INFRASTRUCTURE ONLY. */
PetscScalar getGlobalStrainRateResidual(PetscInt);
void setGlobalStrainRateResidual(PetscInt, PetscScalar);
PetscErrorCode updateGlobalStrainRateResidual(GridData *, MarkerSet *, PetscInt);
PetscInt checkConvergence(PetscScalar, PetscScalar, PetscInt);
