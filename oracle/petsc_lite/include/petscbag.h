/* petscbag.h -- stand-in for PETSc's parameter bags (io.c writes the grid size and elapsed time
 * through one next to its nodal output).  TEST INFRASTRUCTURE ONLY: the stand-in bag holds
 * the registered storage and writes nothing. */
#ifndef PETSC_LITE_BAG_H
#define PETSC_LITE_BAG_H
#include "petsc_lite.h"
typedef struct _p_PetscBag *PetscBag;
PetscErrorCode PetscBagCreate(MPI_Comm, size_t, PetscBag *);
PetscErrorCode PetscBagGetData(PetscBag, void **);
PetscErrorCode PetscBagRegisterScalar(PetscBag, void *, PetscScalar, const char *, const char *);
PetscErrorCode PetscBagView(PetscBag, PetscViewer);
PetscErrorCode PetscBagDestroy(PetscBag *);
#endif
