/*
 * TriDist.h -- PQP-interface restatement: triangle-triangle distance.
 * Called by C2A in its translation CA (C2A/src/InterpMotion.cpp:668, 708).
 * The shim implements it with the C2A library's own feature-annotated
 * TriDist (C2A/src/C2A.cpp:165-405), discarding the features.
 */
#ifndef C2A_SHIM_TRIDIST_H
#define C2A_SHIM_TRIDIST_H
#include "PQP_Compile.h"
PQP_REAL TriDist(PQP_REAL p[3], PQP_REAL q[3], const PQP_REAL s[3][3], const PQP_REAL t[3][3]);
#endif
