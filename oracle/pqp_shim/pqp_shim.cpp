/*
 * pqp_shim.cpp -- PQP-interface restatement (implementations) for compiling
 * the C2A reference sources into the CPU oracle.  Genuine PQP (GammaUNC/PQP,
 * unpinned) is absent; everything here is written from the interface C2A
 * uses.  Test infrastructure only: the product never links it.
 */
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "PQP.h"
#include "MatVec.h"
#include "BVTQ.h"
#include "GetTime.h"
#include "TriDist.h"
#include "OBB_Disjoint.h"
#include "C2A/C2A.h"

BV::BV() { first_child = 0; }
BV::~BV() {}

PQP_Model::PQP_Model()
{
  build_state = 0;
  tris = 0; num_tris = 0; num_tris_alloced = 0;
  b = 0; num_bvs = 0; num_bvs_alloced = 0;
  last_tri = 0;
}

// C2A allocates b as C2A_BV[] and tris as C2A_Tri[] (C2A/src/C2A_PQP.cpp:98,
// 384); deleting them through the base-class pointers would be undefined, so
// the oracle keeps models for the life of the process.
PQP_Model::~PQP_Model() {}

PQP_CollideResult::PQP_CollideResult()
{
  num_bv_tests = num_tri_tests = 0; query_time_secs = 0;
  num_pairs_alloced = num_pairs = 0; pairs = 0;
}
PQP_CollideResult::~PQP_CollideResult() { free(pairs); }
void PQP_CollideResult::FreePairsList() { num_pairs = 0; }
void PQP_CollideResult::SizeTo(int n)
{
  if (n < num_pairs) return;
  CollisionPair *p = (CollisionPair *)realloc(pairs, sizeof(CollisionPair) * (size_t)n);
  if (!p) abort();
  pairs = p; num_pairs_alloced = n;
}
void PQP_CollideResult::Add(int a, int b)
{
  if (num_pairs >= num_pairs_alloced) SizeTo(num_pairs_alloced * 2 + 8);
  pairs[num_pairs].id1 = a; pairs[num_pairs].id2 = b; num_pairs++;
}

double GetTime()
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

// ---- bounded min-heap of BV tests -------------------------------------------
BVTQ::BVTQ(int sz) : size_(sz < 2 ? 2 : sz), num_(0) { heap_ = new BVT[size_]; }
BVTQ::~BVTQ() { delete[] heap_; }
void BVTQ::AddTest(BVT &t)
{
  int i = num_++;
  heap_[i] = t;
  while (i > 0) {
    int p = (i - 1) / 2;
    if (heap_[p].d <= heap_[i].d) break;
    BVT tmp = heap_[p]; heap_[p] = heap_[i]; heap_[i] = tmp; i = p;
  }
}
BVT BVTQ::ExtractMinTest()
{
  BVT top = heap_[0];
  heap_[0] = heap_[--num_];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < num_ && heap_[l].d < heap_[m].d) m = l;
    if (r < num_ && heap_[r].d < heap_[m].d) m = r;
    if (m == i) break;
    BVT tmp = heap_[m]; heap_[m] = heap_[i]; heap_[i] = tmp; i = m;
  }
  return top;
}

// ---- triangle distance --------------------------------------------------------
// C2A's own feature-annotated triangle distance (C2A/src/C2A.cpp:165).
PQP_REAL TriDist(PQP_REAL P[3], PQP_REAL Q[3], const PQP_REAL S[3][3], const PQP_REAL T[3][3],
                 C2A_ContactFeature &f1, C2A_ContactFeature &f2, bool &bCollided);

PQP_REAL TriDist(PQP_REAL p[3], PQP_REAL q[3], const PQP_REAL s[3][3], const PQP_REAL t[3][3])
{
  C2A_ContactFeature f1, f2;
  bool collided = false;
  return TriDist(p, q, s, t, f1, f2, collided);
}

// Distance between t1 and t2 after moving t2 by (R, T) into t1's frame; the
// signature C2A declares at C2A/src/C2A.cpp:41-43 ("Defined in PQP.cpp").
PQP_REAL TriDistance(PQP_REAL R[3][3], PQP_REAL T[3], Tri *t1, Tri *t2, PQP_REAL p[3], PQP_REAL q[3])
{
  PQP_REAL tri1[3][3], tri2[3][3];
  VcV(tri1[0], t1->p1);
  VcV(tri1[1], t1->p2);
  VcV(tri1[2], t1->p3);
  MxVpV(tri2[0], R, t2->p1, T);
  MxVpV(tri2[1], R, t2->p2, T);
  MxVpV(tri2[2], R, t2->p3, T);
  return TriDist(p, q, tri1, tri2);
}

// Triangle overlap (used only by the static collide query, off the CA path):
// the triangles touch when their exact distance is zero.
int TriContact(PQP_REAL *P1, PQP_REAL *P2, PQP_REAL *P3, PQP_REAL *Q1, PQP_REAL *Q2, PQP_REAL *Q3)
{
  PQP_REAL s[3][3], t[3][3], p[3], q[3];
  VcV(s[0], P1); VcV(s[1], P2); VcV(s[2], P3);
  VcV(t[0], Q1); VcV(t[1], Q2); VcV(t[2], Q3);
  return TriDist(p, q, s, t) == 0.0;
}

// ---- OBB separating-axis test (15 axes; B, T give box b in box a's frame) ------
int obb_disjoint(PQP_REAL B[3][3], PQP_REAL T[3], PQP_REAL a[3], PQP_REAL b[3])
{
  PQP_REAL Bf[3][3];
  const PQP_REAL eps = 1e-6;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Bf[i][j] = fabs(B[i][j]) + eps;
  // face axes of a
  for (int i = 0; i < 3; i++) {
    PQP_REAL s = b[0] * Bf[i][0] + b[1] * Bf[i][1] + b[2] * Bf[i][2];
    if (fabs(T[i]) > a[i] + s) return 1;
  }
  // face axes of b
  for (int j = 0; j < 3; j++) {
    PQP_REAL tproj = T[0] * B[0][j] + T[1] * B[1][j] + T[2] * B[2][j];
    PQP_REAL s = a[0] * Bf[0][j] + a[1] * Bf[1][j] + a[2] * Bf[2][j];
    if (fabs(tproj) > b[j] + s) return 1;
  }
  // edge-edge axes a_i x b_j
  for (int i = 0; i < 3; i++) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    for (int j = 0; j < 3; j++) {
      int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      PQP_REAL tproj = T[i2] * B[i1][j] - T[i1] * B[i2][j];
      PQP_REAL ra = a[i1] * Bf[i2][j] + a[i2] * Bf[i1][j];
      PQP_REAL rb = b[j1] * Bf[i][j2] + b[j2] * Bf[i][j1];
      if (fabs(tproj) > ra + rb) return 2;
    }
  }
  return 0;
}

int BV_Overlap(PQP_REAL R[3][3], PQP_REAL T[3], BV *b1, BV *b2)
{
  // centre of b2 relative to b1 in b1's frame: R^T-free form as in PQP (To are
  // parent-relative centres after the build)
  PQP_REAL Tc[3];
  VcV(Tc, T);
  return obb_disjoint(R, Tc, b1->d, b2->d) == 0;
}
