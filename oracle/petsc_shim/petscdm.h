/* Single-rank PETSc API shim: every public PETSc header the reference includes maps to one declaration file. */
#include "petsc_shim.h"
