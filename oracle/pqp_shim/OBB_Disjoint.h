/* OBB_Disjoint.h -- PQP-interface restatement: separating-axis test of two OBBs. */
#ifndef C2A_SHIM_OBB_DISJOINT_H
#define C2A_SHIM_OBB_DISJOINT_H
#include "PQP_Compile.h"
int obb_disjoint(PQP_REAL B[3][3], PQP_REAL T[3], PQP_REAL a[3], PQP_REAL b[3]);
#endif
