/*
 * BVTQ.h -- PQP-interface restatement of the bounded priority queue of
 * bounding-volume tests used by the qsize > 2 distance/contact routines
 * (C2A/src/C2A.cpp:438-600, C2A/src/C2A_PQP.cpp:629-786).  Those routines are
 * off the CA path; the queue is a plain binary min-heap on d.
 */
#ifndef C2A_SHIM_BVTQ_H
#define C2A_SHIM_BVTQ_H
#include "PQP_Compile.h"

struct BVT
{
  PQP_REAL d;        // lower bound on the distance below this test
  int b1, b2;        // node pair
  PQP_REAL R[3][3];  // b2 relative to b1
  PQP_REAL T[3];
};

class BVTQ
{
  int size_;
  int num_;
  BVT *heap_;
public:
  explicit BVTQ(int sz);
  ~BVTQ();
  int Empty() { return num_ == 0; }
  int GetNumTests() { return num_; }
  int GetSize() { return size_; }
  PQP_REAL GetMinDist() { return heap_[0].d; }
  PQP_REAL MinTest() { return heap_[0].d; }
  BVT ExtractMinTest();
  void AddTest(BVT &t);
};
#endif
