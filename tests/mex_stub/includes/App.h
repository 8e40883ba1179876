/* The MEX gateway includes "./includes/App.h" (matlab/mex_includes.h); the
 * reference's build copies its headers there.  Here it is this library's
 * drop-in App header. */
#include "pfdtd/App.h"
