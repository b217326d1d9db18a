/* Stand-in for fvmic2d's markers.h (the prototypes of the marker routines the binding defines
 * or leaves to the host).  TEST INFRASTRUCTURE ONLY; see fdcode.h here. */
PetscErrorCode allocateMarkers(PetscInt, MarkerSet *, Options *);
PetscErrorCode destroyMarkers(MarkerSet *, Options *);
void resetMarkers(MarkerSet *, Options *);
PetscErrorCode distributeMarkersUniformInDomain(MarkerSet *, Options *, GridData *);
PetscErrorCode projectMarkersNodesFromScalar(MarkerSet *, GridData *, PetscScalar *, Vec);
PetscErrorCode checkPlasticYielding(GridData *, MarkerSet *, Materials *, PetscScalar, PetscInt *, Options *,
                                    PetscScalar);
void findMarkerCells(MarkerSet *, GridData *);
PetscErrorCode checkMarkerDensity(Problem *, MarkerSet *, GridData *, Options *, PetscRandom);
PetscErrorCode advectMarkersRK(MarkerSet *, NodalFields *, GridData *, Options *, BoundaryValues *, PetscScalar);
PetscErrorCode projectNodalFieldToMarkersS(NodalFields *, Vec, MarkerSet *, PetscScalar *, GridData *);
void resetMarker(Marker *);
