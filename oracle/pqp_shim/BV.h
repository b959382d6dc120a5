/*
 * PQP-interface restatement of the bounding-volume node.  C2A derives C2A_BV
 * from it (C2A/C2A_BV.h:33) and reads R, Tr, l, r, To, d and first_child.
 * Leaf():    first_child < 0 marks a leaf; the triangle is -first_child-1
 *            (C2A/src/C2A.cpp:1145).
 * GetSize(): RSS size measure used to pick the side to split
 *            (C2A/src/C2A.cpp:1192-1195): rectangle diagonal plus 2r.
 */
#ifndef C2A_SHIM_BV_H
#define C2A_SHIM_BV_H
#include <math.h>
#include "PQP_Compile.h"
#include "Tri.h"

struct BV
{
  PQP_REAL R[3][3];   // orientation of the RSS rectangle (parent-relative after build)
#if PQP_BV_TYPE & RSS_TYPE
  PQP_REAL Tr[3];     // rectangle corner (parent-relative after build)
  PQP_REAL l[2];      // rectangle side lengths
  PQP_REAL r;         // sphere radius swept over the rectangle
#endif
#if PQP_BV_TYPE & OBB_TYPE
  PQP_REAL To[3];     // OBB centre
  PQP_REAL d[3];      // OBB half extents
#endif
  int first_child;    // >= 0: index of first child node; < 0: -(triangle index)-1

  BV();
  ~BV();
  int Leaf() { return first_child < 0; }
  PQP_REAL GetSize();
  void FitToTris(PQP_REAL O[3][3], Tri *tris, int num_tris);
};

inline PQP_REAL BV::GetSize()
{
  return sqrt(l[0] * l[0] + l[1] * l[1]) + 2 * r;
}

int BV_Overlap(PQP_REAL R[3][3], PQP_REAL T[3], BV *b1, BV *b2);
#if PQP_BV_TYPE & RSS_TYPE
PQP_REAL BV_Distance(PQP_REAL R[3][3], PQP_REAL T[3], BV *b1, BV *b2);
#endif
#endif
