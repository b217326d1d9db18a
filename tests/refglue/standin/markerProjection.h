/* Stand-in for fvmic2d's markerProjection.h.  TEST INFRASTRUCTURE ONLY; see fdcode.h here. */
typedef enum { ARITHMETIC, ARITHMETIC_LOCAL, HARMONIC, GEOMETRIC } PROJECTION_METHOD;
PetscErrorCode projectMarkerFieldToNodes(GridData *, MarkerSet *, PetscScalar *, PetscScalar *, Vec, const PetscInt,
                                         const PetscInt, const PROJECTION_METHOD);
PetscErrorCode projectMarkersNodesAll2(MarkerSet *, GridData *, NodalFields *, Materials *, Options *);
