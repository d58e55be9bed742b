/*
 * Stand-in for MATLAB's matrix.h: the mxArray API lives in the mex.h stand-in.
 * TEST INFRASTRUCTURE ONLY (see mex.h).
 */
#include "mex.h"
