/* RectDist.h -- PQP-interface restatement; the C2A path uses its own C2ARectDist. */
#ifndef C2A_SHIM_RECTDIST_H
#define C2A_SHIM_RECTDIST_H
#include "PQP_Compile.h"
PQP_REAL RectDist(PQP_REAL Rab[3][3], PQP_REAL Tab[3], PQP_REAL a[2], PQP_REAL b[2]);
#endif
