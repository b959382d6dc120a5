/* PQP-interface restatement: a triangle as C2A uses it (three vertices, id). */
#ifndef C2A_SHIM_TRI_H
#define C2A_SHIM_TRI_H
#include "PQP_Compile.h"
struct Tri
{
  PQP_REAL p1[3];
  PQP_REAL p2[3];
  PQP_REAL p3[3];
  int id;
};
#endif
