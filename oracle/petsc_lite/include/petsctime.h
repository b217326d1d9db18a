/* single-rank stand-in header; see petsc_lite.h */
#include "petsc_lite.h"
