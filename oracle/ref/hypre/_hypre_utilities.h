/* Stand-in header, see HYPRE.h in this directory. */
#include "HYPRE.h"
