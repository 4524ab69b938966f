/* Stand-in for petscsys.h (oracle/_ref only). */
#include "petsc_shim.h"
