/*
 * PQP.h -- PQP-interface restatement: the model base class, the query result
 * records and the error codes that the C2A sources use.  Only used to compile
 * the C2A reference sources for the CPU oracle (genuine PQP is absent).
 */
#ifndef C2A_SHIM_PQP_H
#define C2A_SHIM_PQP_H

#include <string.h>
#include <stdlib.h>
#include "PQP_Compile.h"
#include "Tri.h"
#include "BV.h"

#define PQP_OK 0
#define PQP_Build_Error_Out_Of_Memory -1
#define PQP_ERR_MODEL_OUT_OF_MEMORY -1
#define PQP_ERR_OUT_OF_MEMORY -2
#define PQP_ERR_UNPROCESSED_MODEL -3
#define PQP_ERR_BUILD_OUT_OF_SEQUENCE -4
#define PQP_ERR_BUILD_EMPTY_MODEL -5

const int PQP_ALL_CONTACTS = 1;  // report every intersecting pair
const int PQP_FIRST_CONTACT = 2; // stop at the first one

// Model base: C2A_Model (C2A/C2A_Internal.h:32) derives from it and
// re-implements BeginModel/AddTri/EndModel itself.
class PQP_Model
{
public:
  int build_state;          // 0 empty, 1 begun, 2 processed (C2A/src/C2A_PQP.cpp:52-57)
  Tri *tris;
  int num_tris;
  int num_tris_alloced;
  BV *b;
  int num_bvs;
  int num_bvs_alloced;
  Tri *last_tri;            // seed triangle of the next distance query

  PQP_Model();
  ~PQP_Model();
  BV *child(int n) { return &b[n]; }
};

struct CollisionPair
{
  int id1;
  int id2;
};

struct PQP_CollideResult
{
  int num_bv_tests;
  int num_tri_tests;
  double query_time_secs;
  PQP_REAL R[3][3];
  PQP_REAL T[3];
  int num_pairs_alloced;
  int num_pairs;
  CollisionPair *pairs;

  void SizeTo(int n);
  void Add(int a, int b);

  PQP_CollideResult();
  ~PQP_CollideResult();
  int NumBVTests() { return num_bv_tests; }
  int NumTriTests() { return num_tri_tests; }
  double QueryTimeSecs() { return query_time_secs; }
  void FreePairsList();
  int Colliding() { return (num_pairs > 0); }
  int NumPairs() { return num_pairs; }
  int Id1(int k) { return pairs[k].id1; }
  int Id2(int k) { return pairs[k].id2; }
};

struct PQP_DistanceResult
{
  int num_bv_tests;
  int num_tri_tests;
  double query_time_secs;
  PQP_REAL R[3][3];
  PQP_REAL T[3];
  PQP_REAL rel_err;
  PQP_REAL abs_err;
  PQP_REAL distance;
  PQP_REAL p1[3];
  PQP_REAL p2[3];
  int qsize;

  int NumBVTests() { return num_bv_tests; }
  int NumTriTests() { return num_tri_tests; }
  double QueryTimeSecs() { return query_time_secs; }
  PQP_REAL Distance() { return distance; }
  const PQP_REAL *P1() { return p1; }
  const PQP_REAL *P2() { return p2; }
};

struct PQP_ToleranceResult
{
  int num_bv_tests;
  int num_tri_tests;
  double query_time_secs;
  PQP_REAL R[3][3];
  PQP_REAL T[3];
  int closer_than_tolerance;
  PQP_REAL tolerance;
  PQP_REAL distance;
  PQP_REAL p1[3];
  PQP_REAL p2[3];
  int qsize;

  int NumBVTests() { return num_bv_tests; }
  int NumTriTests() { return num_tri_tests; }
  double QueryTimeSecs() { return query_time_secs; }
  int CloserThanTolerance() { return closer_than_tolerance; }
  PQP_REAL Distance() { return distance; }
  const PQP_REAL *P1() { return p1; }
  const PQP_REAL *P2() { return p2; }
};

#endif
