/*
 * petsc_lite.h -- single-rank stand-in for the slice of the PETSc 3.x / MPI API
 * that fvmic2d's marker-transfer sources use.  TEST INFRASTRUCTURE ONLY: it lets
 * the reference's own hot-path C files (markers.c, markerProjection.c,
 * updateMarkerStrainPressure.c, subgridStressChanges.c, updateMarkerStress.c,
 * subgridTemperatureChanges.c, viscosity.c, residual.c, ...) be compiled
 * unmodified into oracle/_ref/ so that the project's own C restatement (the
 * oracle) and the GPU kernels can be pinned against the reference's arithmetic.
 *
 * Semantics fixed here (they decide the reference's results on one rank):
 *  - The DMDA: NX x NY nodes, dof 1 (dof 3 for the Stokes solution, values interleaved per
 *    node), stencil width 2, DMDA_STENCIL_BOX, boundary
 *    DM_BOUNDARY_GHOSTED in x and y (fvmic2d nodalFields.c:19-20), or in x
 *    DM_BOUNDARY_PERIODIC (nodalFields.c:11-19; plite_DMDASetPeriodicX).
 *  - Global vectors hold NX*NY values, x fastest ([j][i]); local vectors hold
 *    (NX+4)*(NY+4) values with ghost offset 2 on every side.
 *  - DMGlobalToLocal(INSERT_VALUES) copies the interior and leaves ghost
 *    entries untouched; DMLocalToGlobal(ADD_VALUES) adds the interior and drops
 *    the ghost entries (they have no owner on a ghosted, non-periodic DMDA).
 *    Periodic in x: DMGlobalToLocal also fills ghost columns -2, -1, NX, NX+1 of
 *    every row with columns NX-2, NX-1, 0, 1, and DMLocalToGlobal(ADD_VALUES)
 *    adds those ghost columns into their owners after the interior (in the
 *    order -2, -1, NX, NX+1); ghost rows are handled as before.
 *  - VecPointwiseDivide(w,x,y) gives w[i] = x[i]/y[i] when y[i] != 0 and 0
 *    otherwise (the zero-divisor guard of current PETSc releases).
 *  - Fresh vectors (DMCreate*Vector, DMGet*Vector, VecDuplicate) are zeroed.
 *  - VecMax / VecMin skip NaN entries (their comparisons are false).
 *  - MPI: one rank; MPI_Allreduce copies.
 */
#ifndef PETSC_LITE_H
#define PETSC_LITE_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef int PetscErrorCode;
typedef double PetscLogDouble;
typedef int PetscLogStage;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { INSERT_VALUES = 0, ADD_VALUES = 1 } InsertMode;
typedef enum { DM_BOUNDARY_NONE, DM_BOUNDARY_GHOSTED, DM_BOUNDARY_PERIODIC } DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR, DMDA_STENCIL_BOX } DMDAStencilType;
typedef const char *PetscRandomType;
#define PETSCRAND "rand"
#define PETSCRAND48 "rand48"

typedef struct _p_DM *DM;
typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_MatNullSpace *MatNullSpace;
typedef struct _p_PetscRandom *PetscRandom;
typedef struct _p_PetscViewer *PetscViewer;
typedef struct _p_KSP *KSP;

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_BYTE 3
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define PETSC_NULL NULL
#define PETSC_DECIDE (-1)
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define PETSC_ERR_MAX_VALUE 100

#define CHKERRQ(e) do { if (e) return (e); } while (0)
#define SETERRQ(c, n, s) return (n)
#define PetscFunctionBegin
#define PetscFunctionReturn(x) return (x)

#define PetscMalloc(sz, p) ((*(void **)(p) = malloc((size_t)(sz) ? (size_t)(sz) : 1)) == NULL)
#define PetscMalloc2(n1, p1, n2, p2) \
  (PetscMalloc((size_t)(n1) * sizeof(**(p1)), p1) || PetscMalloc((size_t)(n2) * sizeof(**(p2)), p2))
#define PetscFree(p) (free(p), (p) = NULL, 0)
#define PetscFree2(a, b) (PetscFree(a), PetscFree(b), 0)
#define PetscMemcpy(d, s, n) (memcpy((d), (s), (n)), 0)
#define PetscMemzero(d, n) (memset((d), 0, (n)), 0)

/* DMDA / Vec (single rank) */
PetscErrorCode plite_DMDACreate(PetscInt NX, PetscInt NY, DM *da);
PetscErrorCode plite_DMDACreateDOF(PetscInt NX, PetscInt NY, PetscInt dof, DM *da);
void plite_DMDASetPeriodicX(DM da, int periodic);
PetscErrorCode plite_DMDestroy(DM *da);
PetscErrorCode DMDAGetCorners(DM, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *);
PetscErrorCode DMCreateGlobalVector(DM, Vec *);
PetscErrorCode DMCreateLocalVector(DM, Vec *);
PetscErrorCode DMGetGlobalVector(DM, Vec *);
PetscErrorCode DMRestoreGlobalVector(DM, Vec *);
PetscErrorCode DMGetLocalVector(DM, Vec *);
PetscErrorCode DMRestoreLocalVector(DM, Vec *);
PetscErrorCode DMGlobalToLocalBegin(DM, Vec, InsertMode, Vec);
PetscErrorCode DMGlobalToLocalEnd(DM, Vec, InsertMode, Vec);
PetscErrorCode DMLocalToGlobalBegin(DM, Vec, InsertMode, Vec);
PetscErrorCode DMLocalToGlobalEnd(DM, Vec, InsertMode, Vec);
PetscErrorCode DMDAVecGetArray(DM, Vec, void *);
PetscErrorCode DMDAVecRestoreArray(DM, Vec, void *);
PetscErrorCode DMDAVecGetArrayDOF(DM, Vec, void *);
PetscErrorCode DMDAVecRestoreArrayDOF(DM, Vec, void *);
PetscErrorCode VecDuplicate(Vec, Vec *);
PetscErrorCode VecDestroy(Vec *);
PetscErrorCode VecZeroEntries(Vec);
PetscErrorCode VecSet(Vec, PetscScalar);
PetscErrorCode VecCopy(Vec, Vec);
PetscErrorCode VecAXPY(Vec, PetscScalar, Vec);
PetscErrorCode VecAXPBYPCZ(Vec, PetscScalar, PetscScalar, PetscScalar, Vec, Vec);
PetscErrorCode VecPointwiseDivide(Vec, Vec, Vec);
PetscErrorCode VecSum(Vec, PetscScalar *);
PetscErrorCode VecView(Vec, PetscViewer);
PetscErrorCode VecGetArray(Vec, PetscScalar **);
PetscErrorCode VecRestoreArray(Vec, PetscScalar **);
PetscErrorCode VecGetSize(Vec, PetscInt *);
PetscErrorCode VecScale(Vec, PetscScalar);
PetscErrorCode VecShift(Vec, PetscScalar);
PetscErrorCode VecPointwiseMult(Vec, Vec, Vec);
PetscErrorCode VecAYPX(Vec, PetscScalar, Vec);
PetscErrorCode VecMax(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecMin(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecStrideScale(Vec, PetscInt, PetscScalar);

/* logging: stages accumulate wall time per stage id (used for the CPU breakdown) */
PetscErrorCode PetscLogStageRegister(const char *, PetscLogStage *);
PetscErrorCode PetscLogStagePush(PetscLogStage);
PetscErrorCode PetscLogStagePop(void);
double plite_stage_seconds(int stage);
void plite_stage_reset(void);

PetscErrorCode PetscPrintf(MPI_Comm, const char *, ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm, const char *, ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm, ...);
void plite_set_quiet(int quiet);

/* random numbers (only reached by marker initialisation / density control) */
PetscErrorCode PetscRandomCreate(MPI_Comm, PetscRandom *);
PetscErrorCode PetscRandomSetType(PetscRandom, PetscRandomType);
PetscErrorCode PetscRandomSetSeed(PetscRandom, unsigned long);
PetscErrorCode PetscRandomSeed(PetscRandom);
PetscErrorCode PetscRandomSetInterval(PetscRandom, PetscScalar, PetscScalar);
PetscErrorCode PetscRandomGetValue(PetscRandom, PetscScalar *);
PetscErrorCode PetscRandomDestroy(PetscRandom *);

/* MPI, one rank */
int MPI_Comm_rank(MPI_Comm, int *);
int MPI_Comm_size(MPI_Comm, int *);
int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int,
                 MPI_Comm, MPI_Status *);
/* one rank: gathers copy, broadcasts do nothing, point-to-point is never reached */
int MPI_Allgather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm);
int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm);
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm);
int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *);
typedef int MPI_Info;
#define MPI_MODE_CREATE 1

/* Viewers, bags, object names and options: io.c's nodal-field and options writers use them;
 * the marker writer (saveMarkersBinary) does not.  These stand-ins do nothing and report an
 * error where output would be produced. */
typedef enum {
  PETSC_VIEWER_DEFAULT = 0, PETSC_VIEWER_ASCII_MATLAB, PETSC_VIEWER_BINARY_MATLAB, PETSC_VIEWER_ASCII_VTK,
  PETSC_VIEWER_VTK_VTS, PETSC_VIEWER_NATIVE
} PetscViewerFormat;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE = 1, FILE_MODE_APPEND = 2 } PetscFileMode;
typedef const char *PetscViewerType;
#define PETSCVIEWERBINARY "binary"
#define PETSCVIEWERASCII "ascii"
#define PETSCVIEWERVTK "vtk"
typedef void *PetscObject;
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm, const char *, PetscViewer *);
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm, const char *, PetscFileMode, PetscViewer *);
PetscErrorCode PetscViewerMatlabOpen(MPI_Comm, const char *, PetscFileMode, PetscViewer *);
PetscErrorCode PetscViewerCreate(MPI_Comm, PetscViewer *);
PetscErrorCode PetscViewerSetType(PetscViewer, PetscViewerType);
PetscErrorCode PetscViewerFileSetMode(PetscViewer, PetscFileMode);
PetscErrorCode PetscViewerFileSetName(PetscViewer, const char *);
PetscErrorCode PetscViewerSetFormat(PetscViewer, PetscViewerFormat);
PetscErrorCode PetscViewerMatlabPutArray(PetscViewer, int, int, const PetscScalar *, const char *);
PetscErrorCode PetscViewerDestroy(PetscViewer *);
PetscErrorCode PetscObjectSetName(PetscObject, const char *);
PetscErrorCode DMView(DM, PetscViewer);
PetscErrorCode DMGetCoordinates(DM, Vec *);
PetscErrorCode PetscOptionsGetBool(const char *, const char *, PetscBool *, PetscBool *);  /* PETSc 3.5 form */

/* Mat (one rank, AIJ semantics): rows of (column, value) entries.  MatSetValue(s) with
 * INSERT_VALUES replaces an existing entry and ADD_VALUES adds to it; rows or columns with a
 * negative index are skipped, which is how PETSc drops the ghost points of a ghosted DMDA
 * (their local-to-global index is -1).  Assembly does nothing.  VecSetValue(s) follow the same
 * rules on global vectors. */
typedef enum { MAT_FINAL_ASSEMBLY = 0, MAT_FLUSH_ASSEMBLY = 1 } MatAssemblyType;
typedef enum { DIFFERENT_NONZERO_PATTERN, SUBSET_NONZERO_PATTERN, SAME_NONZERO_PATTERN } MatStructure;
PetscErrorCode plite_MatCreate(PetscInt nrows, Mat *A);
PetscErrorCode MatDestroy(Mat *A);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt *rows, PetscInt n, const PetscInt *cols,
                            const PetscScalar *v, InsertMode mode);
PetscErrorCode MatSetValue(Mat A, PetscInt row, PetscInt col, PetscScalar v, InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatCopy(Mat A, Mat B, MatStructure s);
/* CSR copy, columns ascending within a row; the arrays are malloc'd; returns the entry count */
PetscInt plite_MatGetCSR(Mat A, PetscInt **rowptr, PetscInt **cols, PetscScalar **vals);
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *idx, const PetscScalar *y, InsertMode mode);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode mode);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
/* local-to-global map of the ghosted node layout ((NX+4) x (NY+4), offset 2): the node index
 * j NX + i inside the domain, -1 on the ghost points */
typedef struct _p_ISLocalToGlobalMapping *ISLocalToGlobalMapping;
PetscErrorCode DMGetLocalToGlobalMapping(DM da, ISLocalToGlobalMapping *map);
PetscErrorCode ISLocalToGlobalMappingGetIndices(ISLocalToGlobalMapping map, const PetscInt **idx);
PetscErrorCode ISLocalToGlobalMappingRestoreIndices(ISLocalToGlobalMapping map, const PetscInt **idx);
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                                   PetscInt *p);

#endif
