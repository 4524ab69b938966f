/* Stand-in for petscmat.h (oracle/_ref only). */
#include "petsc_shim.h"
