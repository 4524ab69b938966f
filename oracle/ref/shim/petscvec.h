/* Stand-in for petscvec.h (oracle/_ref only). */
#include "petsc_shim.h"
