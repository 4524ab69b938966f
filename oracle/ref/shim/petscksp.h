/* Stand-in for petscksp.h (oracle/_ref only). */
#include "petsc_shim.h"
