/* Stand-in for MATLAB's matrix.h: everything lives in the mex.h shim. Oracle only. */
#include "mex.h"
