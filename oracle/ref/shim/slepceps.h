/* Stand-in for slepceps.h (oracle/_ref only). */
#include "petsc_shim.h"
