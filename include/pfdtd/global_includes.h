// Admittance/reflection conversions (ParallelFDTD src/global_includes.h:30-38).
#ifndef PFDTD_GLOBAL_INCLUDES_H
#define PFDTD_GLOBAL_INCLUDES_H

#include "logger.h"

// Y = (1 - R) / (1 + R), evaluated in single precision.
inline float reflection2Admitance(float coef) { return ((1.f - coef) / (1.f + coef)); }

// The same map is its own inverse.
inline float admitance2Reflection(float coef) { return reflection2Admitance(coef); }

#endif
