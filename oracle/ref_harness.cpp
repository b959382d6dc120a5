/*
 * ref_harness.cpp -- extern "C" driver around the C2A reference sources,
 * compiled with them (unmodified, from their own directory) into
 * oracle/_ref/libc2a_ref.so by oracle/Makefile.  Test infrastructure only:
 * it lets the tests run the reference's own classes and functions
 * (C2A_Model, CInterpMotion_Linear, C2A_QueryTimeOfContact,
 * C2A_QueryContact, C2A_Solve, C2ARectDist, TriDist) on the same inputs as
 * the CUDA path and the oracle port.
 */
#include <string.h>
#include <stdio.h>
#include <string>
#include <list>
#include <vector>
#include <algorithm>
#include <iostream>
#include "PQP.h"
#include "MatVec.h"
#include "C2A/C2A.h"
#include "C2A/C2A_Internal.h"
#include "C2A/InterpMotion.h"
#include "C2A/C2A_RectDist.h"

extern bool b_TanslationCCD; // C2A/src/C2A.cpp:33

PQP_REAL TriDist(PQP_REAL P[3], PQP_REAL Q[3], const PQP_REAL S[3][3], const PQP_REAL T[3][3],
                 C2A_ContactFeature &f1, C2A_ContactFeature &f2, bool &bCollided);

// defined in C2A/src/C2A.cpp:1778-1789, not declared in its headers
int C2A_TimeOfContactStep(CInterpMotion *objmotion1, CInterpMotion *objmotion2, C2A_TimeOfContactResult *res,
                          PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3], PQP_REAL T2[3],
                          C2A_Model *o2, PQP_REAL tolerance_t, PQP_REAL tolerance_d);

// defined in C2A/src/C2A_PQP.cpp (RSS builds) without a header declaration
int C2A_Tolerance(PQP_ToleranceResult *res, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                  PQP_REAL T2[3], C2A_Model *o2, PQP_REAL tolerance, int qsize);

extern "C" {

// Same layout as c2a_port_result / c2a_port_contact (oracle/c2a_port.h).
struct ref_result {
  int collisionfree, numCA, translation, num_contact;
  double toc, distance, mint;
  long long num_bv_tests, num_tri_tests;
  double R_toc[2][9];
  double T_toc[2][3];
  int seed_a, seed_b;
};
struct ref_contact {
  int type_a, type_b;
  int fid_a[3], fid_b[3];
  int tri_a, tri_b;
  double pa[3], pb[3];
  double distance;
};

// C2A_Model build through the reference's own AddTri/EndModel
// (C2A/src/C2A_PQP.cpp:82-417).  stdout chatter of EndModel is kept.
void *c2a_ref_model_build(int num_tris, const double *tv, const int *ids, const int *vidx)
{
  C2A_Model *m = new C2A_Model();
  m->BeginModel();
  for (int i = 0; i < num_tris; i++) {
    int id = ids ? ids[i] : i;
    int i1 = vidx ? vidx[3 * i] : -1, i2 = vidx ? vidx[3 * i + 1] : -1, i3 = vidx ? vidx[3 * i + 2] : -1;
    m->AddTri(tv + 9 * i, tv + 9 * i + 3, tv + 9 * i + 6, id, i1, i2, i3);
  }
  if (m->EndModel() != PQP_OK) return 0;
  return m;
}

int c2a_ref_model_num_nodes(void *h) { return ((C2A_Model *)h)->num_bvs; }
int c2a_ref_model_last_tri(void *h);
int c2a_ref_model_num_tris(void *h) { return ((C2A_Model *)h)->num_tris; }

// node fields the CA path reads: R(9) Tr(3) l(2) r angR Rloc(9) -> 25 doubles
// per node, first_child separately; triangles: 9 doubles + id + 3 vertex ids.
void c2a_ref_model_dump(void *h, double *node_f, int *first_child, double *tri_v, int *tri_id, int *tri_idx)
{
  C2A_Model *m = (C2A_Model *)h;
  for (int n = 0; n < m->num_bvs; n++) {
    C2A_BV *b = (C2A_BV *)m->child(n);
    double *o = node_f + 25 * n;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        o[3 * i + j] = b->R[i][j];
        o[16 + 3 * i + j] = b->R_loc[i][j];
      }
    o[9] = b->Tr[0]; o[10] = b->Tr[1]; o[11] = b->Tr[2];
    o[12] = b->l[0]; o[13] = b->l[1];
    o[14] = b->r;
    o[15] = b->angularRadius;
    first_child[n] = b->first_child;
  }
  for (int t = 0; t < m->num_tris; t++) {
    C2A_Tri *tr = m->GetTriangle(t);
    memcpy(tri_v + 9 * t, tr->p1, 3 * sizeof(double));
    memcpy(tri_v + 9 * t + 3, tr->p2, 3 * sizeof(double));
    memcpy(tri_v + 9 * t + 6, tr->p3, 3 * sizeof(double));
    tri_id[t] = tr->id;
    tri_idx[3 * t] = tr->Index()[0];
    tri_idx[3 * t + 1] = tr->Index()[1];
    tri_idx[3 * t + 2] = tr->Index()[2];
  }
}

static void m9(PQP_REAL R[3][3], const double *v)
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i][j] = v[3 * i + j];
}

static int tri_index(C2A_Model *m, Tri *t) { return (int)((C2A_Tri *)t - (C2A_Tri *)m->tris); }

// the model's last_tri (C2A.cpp:1175 and C2A_PQP.cpp:516 move it; the demo
// seeds each frame with it, CCDDemo/mainTorusknot.cpp:285-286)
int c2a_ref_model_last_tri(void *h)
{
  C2A_Model *m = (C2A_Model *)h;
  return tri_index(m, m->last_tri);
}

static int copy_contacts(const C2A_TimeOfContactResult &dres, ref_contact *out, int max_out)
{
  int n = 0;
  for (ContactFList::const_iterator it = dres.cont_l.begin(); it != dres.cont_l.end(); ++it, ++n) {
    if (!out || n >= max_out) continue;
    ref_contact &c = out[n];
    c.type_a = it->FeatureType_A;
    c.type_b = it->FeatureType_B;
    for (int k = 0; k < 3; k++) {
      // unused feature slots are uninitialised in the reference (C2A.cpp:1587-1588)
      c.fid_a[k] = (k < (c.type_a == 1 ? 1 : c.type_a == 2 ? 2 : 3)) ? it->FeatureID_A[k] : -1;
      c.fid_b[k] = (k < (c.type_b == 1 ? 1 : c.type_b == 2 ? 2 : 3)) ? it->FeatureID_B[k] : -1;
    }
    c.tri_a = it->TriangleID_A;
    c.tri_b = it->TriangleID_B;
    memcpy(c.pa, it->P_A, sizeof(c.pa));
    memcpy(c.pb, it->P_B, sizeof(c.pb));
    c.distance = it->Distance;
  }
  return n;
}

// Body of C2A_Solve (C2A/src/C2A.cpp:2315-2444) with tolerance_d, m_toc_delta
// and the contact threshold's absolute term taken from the caller (the
// shipped C2A_Solve ignores th_ca and hard-codes 1e-4), seeds set
// explicitly, and no per-call printf.
int c2a_ref_solve(void *ha, void *hb, const double *R0a, const double *T0a, const double *R1a, const double *T1a,
                  const double *R0b, const double *T0b, const double *R1b, const double *T1b, int seed_a,
                  int seed_b, double tol_d, double tol_t, double toc_delta, double contact_abs, int with_contacts,
                  int max_iters_unused, ref_result *out, ref_contact *contacts, int max_contacts)
{
  (void)max_iters_unused;
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  PQP_REAL R1[3][3], T1[3], R2[3][3], T2[3], R1e[3][3], T1e[3], R2e[3][3], T2e[3];
  m9(R1, R0a); VcV(T1, T0a); m9(R1e, R1a); VcV(T1e, T1a);
  m9(R2, R0b); VcV(T2, T0b); m9(R2e, R1b); VcV(T2e, T1b);
  CInterpMotion_Linear motion1(R1, T1, R1e, T1e);
  CInterpMotion_Linear motion2(R2, T2, R2e, T2e);
  motion1.m_toc_delta = toc_delta;
  motion2.m_toc_delta = toc_delta;
  b_TanslationCCD = (motion1.m_angVel < 1e-8 && motion2.m_angVel < 1e-8);
  C2A_TimeOfContactResult dres;
  dres.last_triA = A->GetTriangle(seed_a);
  dres.last_triB = B->GetTriangle(seed_b);
  dres.num_contact = 0;
  C2A_QueryTimeOfContact(&motion1, &motion2, &dres, A, B, tol_d, tol_t, 0);
  memset(out, 0, sizeof(*out));
  out->translation = b_TanslationCCD ? 1 : 0;
  out->collisionfree = dres.collisionfree ? 1 : 0;
  out->toc = dres.toc;
  out->numCA = dres.numCA;
  out->distance = dres.distance;
  out->mint = dres.mint;
  out->num_bv_tests = dres.num_bv_tests;
  out->num_tri_tests = dres.num_tri_tests;
  out->seed_a = tri_index(A, dres.last_triA);
  out->seed_b = tri_index(B, dres.last_triB);
  dres.cont_l.clear();
  if (!dres.collisionfree) {
    PQP_REAL qua[7], R[3][3], T[3];
    motion1.integrate(dres.toc, qua);
    motion1.transform.Rotation().Get_Value(R);
    motion1.transform.Translation().Get_Value(T);
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) out->R_toc[0][3 * i + j] = R[i][j];
      out->T_toc[0][i] = T[i];
    }
    motion2.integrate(dres.toc, qua);
    motion2.transform.Rotation().Get_Value(R);
    motion2.transform.Translation().Get_Value(T);
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) out->R_toc[1][3 * i + j] = R[i][j];
      out->T_toc[1][i] = T[i];
    }
    if (with_contacts) {
      double threshold = 2 * dres.distance + contact_abs;
      C2A_QueryContact(&motion1, &motion2, &dres, A, B, threshold);
      out->num_contact = dres.num_contact;
      copy_contacts(dres, contacts, max_contacts);
    }
  }
  return 0;
}

// CANONICAL composition of the reference's own functions: before every
// rotation step, C2A_Distance (rel_err = abs_err = 0, qsize 2; C2A_PQP.cpp:971)
// from the current seed pair finds the closest triangle pair, which then seeds
// C2A_TimeOfContactStep (res->last_triA/B).  The loop around the steps is a
// harness copy of C2A_QueryTimeOfContact's (C2A.cpp:1987-2146) so the
// distance query can run between steps; contacts are sorted by (tri_a, tri_b).
static void closest_seed(C2A_TimeOfContactResult &dres, C2A_Model *A, C2A_Model *B, PQP_REAL R1[3][3],
                         PQP_REAL T1[3], PQP_REAL R2[3][3], PQP_REAL T2[3])
{
  C2A_DistanceResult dd;
  A->last_tri = dres.last_triA;
  B->last_tri = dres.last_triB;
  C2A_Distance(&dd, R1, T1, A, R2, T2, B, 0.0, 0.0, 2);
  dres.last_triA = A->last_tri;
  dres.last_triB = B->last_tri;
}

// C2A_Tolerance (qsize 2); R/T place model B in model A's frame.  out:
// distance, p1[3], p2[3], num_bv_tests, num_tri_tests; returns closer_than_tolerance.
int c2a_ref_tolerance(void *ha, void *hb, const double *R9, const double *T3, double tolerance, double *out)
{
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  PQP_REAL I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, Z[3] = {0, 0, 0}, R[3][3], T[3];
  m9(R, R9);
  VcV(T, T3);
  PQP_ToleranceResult res;
  memset(&res, 0, sizeof(res));
  C2A_Tolerance(&res, I, Z, A, R, T, B, tolerance, 2);
  out[0] = res.distance;
  for (int i = 0; i < 3; i++) {
    out[1 + i] = res.p1[i];
    out[4 + i] = res.p2[i];
  }
  out[7] = res.num_bv_tests;
  out[8] = res.num_tri_tests;
  return res.closer_than_tolerance;
}

// C2A_Collide (the PQP_CollideResult form); R/T place model B in model A's
// frame.  Writes up to cap (id1, id2) pairs; counts[0..1]: BV and triangle
// tests; returns the number of pairs.
int c2a_ref_collide(void *ha, void *hb, const double *R9, const double *T3, int flag, int *pairs, int cap,
                    long long *counts)
{
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  PQP_REAL I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, Z[3] = {0, 0, 0}, R[3][3], T[3];
  m9(R, R9);
  VcV(T, T3);
  PQP_CollideResult res;
  C2A_Collide(&res, I, Z, A, R, T, B, flag);
  for (int k = 0; k < res.num_pairs && k < cap; k++) {
    pairs[2 * k] = res.Id1(k);
    pairs[2 * k + 1] = res.Id2(k);
  }
  counts[0] = res.num_bv_tests;
  counts[1] = res.num_tri_tests;
  return res.num_pairs;
}

// C2A_Distance (rel_err = abs_err = 0, qsize 2) from a seed pair; R/T place
// model B in model A's frame.  Returns the distance; *ta/*tb the closest pair.
double c2a_ref_distance(void *ha, void *hb, const double *R9, const double *T3, int seed_a, int seed_b, int *ta,
                        int *tb, long long *nbv, long long *ntri)
{
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  PQP_REAL I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, Z[3] = {0, 0, 0}, R[3][3], T[3];
  m9(R, R9);
  VcV(T, T3);
  C2A_DistanceResult dd;
  A->last_tri = A->GetTriangle(seed_a);
  B->last_tri = B->GetTriangle(seed_b);
  C2A_Distance(&dd, I, Z, A, R, T, B, 0.0, 0.0, 2);
  *ta = tri_index(A, A->last_tri);
  *tb = tri_index(B, B->last_tri);
  if (nbv) *nbv = dd.num_bv_tests;
  if (ntri) *ntri = dd.num_tri_tests;
  return dd.distance;
}

int c2a_ref_solve_canonical(void *ha, void *hb, const double *R0a, const double *T0a, const double *R1a,
                            const double *T1a, const double *R0b, const double *T0b, const double *R1b,
                            const double *T1b, int seed_a, int seed_b, double tol_d, double tol_t,
                            double toc_delta, double contact_abs, int with_contacts, int max_iters,
                            ref_result *out, ref_contact *contacts, int max_contacts)
{
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  PQP_REAL R1[3][3], T1[3], R2[3][3], T2[3], R1e[3][3], T1e[3], R2e[3][3], T2e[3];
  m9(R1, R0a); VcV(T1, T0a); m9(R1e, R1a); VcV(T1e, T1a);
  m9(R2, R0b); VcV(T2, T0b); m9(R2e, R1b); VcV(T2e, T1b);
  CInterpMotion_Linear motion1(R1, T1, R1e, T1e);
  CInterpMotion_Linear motion2(R2, T2, R2e, T2e);
  motion1.m_toc_delta = toc_delta;
  motion2.m_toc_delta = toc_delta;
  b_TanslationCCD = (motion1.m_angVel < 1e-8 && motion2.m_angVel < 1e-8);
  C2A_TimeOfContactResult dres;
  dres.last_triA = A->GetTriangle(seed_a);
  dres.last_triB = B->GetTriangle(seed_b);
  dres.num_contact = 0;
  dres.num_bv_tests = 0;
  dres.num_tri_tests = 0;
  dres.UpboundTOC = 1;
  dres.numCA = 0;
  motion1.transform.Rotation().Get_Value(R1);
  motion1.transform.Translation().Get_Value(T1);
  motion2.transform.Rotation().Get_Value(R2);
  motion2.transform.Translation().Get_Value(T2);
  PQP_REAL lamda = 0.0, lastLamda = 0, dlamda = 0.0, toc = 0;
  bool collisionfree = false, done = false;
  if (!b_TanslationCCD) closest_seed(dres, A, B, R1, T1, R2, T2);
  C2A_TimeOfContactStep(&motion1, &motion2, &dres, R1, T1, A, R2, T2, B, tol_t, tol_d);
  PQP_REAL dist = dres.distance, mint = dres.mint;
  if (b_TanslationCCD) {
    collisionfree = (mint >= 1.0);
    toc = mint;
    done = true;
  } else {
    dres.numCA = 1;
    lastLamda = mint;
    int nItrs = 0;
    while (dist > tol_d) {
      if (++nItrs > max_iters) break;
      if (mint >= 1.0) { collisionfree = true; toc = 0; done = true; break; }
      dlamda = mint;
      if (dlamda < tol_t) break;
      lamda += dlamda;
      if (lamda >= 1.0) { collisionfree = true; toc = 0; done = true; break; }
      lastLamda = lamda;
      dres.numCA++;
      ((CInterpMotion *)&motion1)->integrate(lamda, R1, T1); /* the base-class overload */
      ((CInterpMotion *)&motion2)->integrate(lamda, R2, T2);
      dres.UpboundTOC = 1.0 - lamda;
      closest_seed(dres, A, B, R1, T1, R2, T2);
      C2A_TimeOfContactStep(&motion1, &motion2, &dres, R1, T1, A, R2, T2, B, tol_t, tol_d);
      dist = dres.distance;
      mint = dres.mint;
    }
  }
  if (!done) {
    toc = (dist == 0 && mint < 0) ? lastLamda - dlamda : lastLamda;
    collisionfree = false;
    if (toc >= 1 - tol_t) toc = 0;
  }
  memset(out, 0, sizeof(*out));
  out->translation = b_TanslationCCD ? 1 : 0;
  out->collisionfree = collisionfree ? 1 : 0;
  out->toc = toc;
  out->numCA = dres.numCA;
  out->distance = dres.distance;
  out->mint = dres.mint;
  out->num_bv_tests = dres.num_bv_tests;
  out->num_tri_tests = dres.num_tri_tests;
  out->seed_a = tri_index(A, dres.last_triA);
  out->seed_b = tri_index(B, dres.last_triB);
  dres.cont_l.clear();
  if (!collisionfree) {
    PQP_REAL qua[7], R[3][3], T[3];
    motion1.integrate(toc, qua);
    motion1.transform.Rotation().Get_Value(R);
    motion1.transform.Translation().Get_Value(T);
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) out->R_toc[0][3 * i + j] = R[i][j];
      out->T_toc[0][i] = T[i];
    }
    motion2.integrate(toc, qua);
    motion2.transform.Rotation().Get_Value(R);
    motion2.transform.Translation().Get_Value(T);
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) out->R_toc[1][3 * i + j] = R[i][j];
      out->T_toc[1][i] = T[i];
    }
    if (with_contacts) {
      double threshold = 2 * dres.distance + contact_abs;
      C2A_QueryContact(&motion1, &motion2, &dres, A, B, threshold);
      out->num_contact = dres.num_contact;
      int kept = copy_contacts(dres, contacts, max_contacts);
      if (contacts) {
        if (kept > max_contacts) kept = max_contacts;
        std::vector<ref_contact> v(contacts, contacts + kept);
        std::sort(v.begin(), v.end(), [](const ref_contact &x, const ref_contact &y) {
          return x.tri_a != y.tri_a ? x.tri_a < y.tri_a : x.tri_b < y.tri_b;
        });
        std::copy(v.begin(), v.end(), contacts);
      }
    }
  }
  return 0;
}

// The shipped entry point itself (C2A/src/C2A.cpp:2315): th_ca is ignored,
// tolerance_d = m_toc_delta = t_delta = 1e-4, contacts within 2d + 0.001.
int c2a_ref_solve_shipped(void *ha, void *hb, const double *R0a, const double *T0a, const double *R1a,
                          const double *T1a, const double *R0b, const double *T0b, const double *R1b,
                          const double *T1b, int seed_a, int seed_b, ref_result *out, ref_contact *contacts,
                          int max_contacts)
{
  C2A_Model *A = (C2A_Model *)ha, *B = (C2A_Model *)hb;
  Transform t00, t01, t10, t11, tr0, tr1;
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) {
      t00.Rotation()[i][j] = R0a[3 * i + j];
      t01.Rotation()[i][j] = R1a[3 * i + j];
      t10.Rotation()[i][j] = R0b[3 * i + j];
      t11.Rotation()[i][j] = R1b[3 * i + j];
    }
    t00.Translation()[i] = T0a[i];
    t01.Translation()[i] = T1a[i];
    t10.Translation()[i] = T0b[i];
    t11.Translation()[i] = T1b[i];
  }
  C2A_TimeOfContactResult dres;
  dres.last_triA = A->GetTriangle(seed_a);
  dres.last_triB = B->GetTriangle(seed_b);
  dres.num_contact = 0;
  PQP_REAL toc = 0;
  int iters = 0, ncont = 0;
  C2A_Solve(&t00, &t01, A, &t10, &t11, B, tr0, tr1, toc, iters, ncont, 0.0, dres);
  memset(out, 0, sizeof(*out));
  out->translation = b_TanslationCCD ? 1 : 0;
  out->collisionfree = dres.collisionfree ? 1 : 0;
  out->toc = toc;
  out->numCA = iters;
  out->distance = dres.distance;
  out->mint = dres.mint;
  out->num_bv_tests = dres.num_bv_tests;
  out->num_tri_tests = dres.num_tri_tests;
  out->num_contact = dres.collisionfree ? 0 : ncont;
  out->seed_a = tri_index(A, dres.last_triA);
  out->seed_b = tri_index(B, dres.last_triB);
  if (!dres.collisionfree) {
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) {
        out->R_toc[0][3 * i + j] = tr0.Rotation()[i][j];
        out->R_toc[1][3 * i + j] = tr1.Rotation()[i][j];
      }
      out->T_toc[0][i] = tr0.Translation()[i];
      out->T_toc[1][i] = tr1.Translation()[i];
    }
    copy_contacts(dres, contacts, max_contacts);
  }
  return 0;
}

// C2ARectDist (C2A/C2A_RectDist.h:157) on raw inputs.
double c2a_ref_rectdist(const double *Rab9, const double *Tab, const double *a, const double *b, double *P,
                        double *Q, double *S)
{
  PQP_REAL Rab[3][3], T[3], aa[2] = {a[0], a[1]}, bb[2] = {b[0], b[1]};
  m9(Rab, Rab9);
  VcV(T, Tab);
  bool valid = false;
  return C2ARectDist(Rab, T, aa, bb, P, Q, valid, S);
}

// C2A's triangle distance with features (C2A/src/C2A.cpp:165).
double c2a_ref_tridist(double *P, double *Q, const double *S9, const double *T9, int *f1_type, int *f1_fid,
                       int *f2_type, int *f2_fid, int *collided)
{
  PQP_REAL S[3][3], T[3][3];
  m9(S, S9);
  m9(T, T9);
  C2A_ContactFeature f1, f2;
  bool col = false;
  double d = TriDist(P, Q, S, T, f1, f2, col);
  *f1_type = f1.type; *f1_fid = f1.fid[0];
  *f2_type = f2.type; *f2_fid = f2.fid[0];
  *collided = col ? 1 : 0;
  return d;
}

// CInterpMotion_Linear: velocity constants, then the pose at time t.
void c2a_ref_motion(const double *R0, const double *T0, const double *R1, const double *T1, double t,
                    double *axis_angvel_cv, double *R_t, double *T_t)
{
  PQP_REAL r0[3][3], t0[3], r1[3][3], t1[3], R[3][3], T[3];
  m9(r0, R0); VcV(t0, T0); m9(r1, R1); VcV(t1, T1);
  CInterpMotion_Linear m(r0, t0, r1, t1);
  m.m_axis.Get_Value(axis_angvel_cv);
  axis_angvel_cv[3] = m.m_angVel;
  m.cv.Get_Value(axis_angvel_cv + 4);
  CInterpMotion *base = &m; // integrate(t, R, T) lives in the base class
  base->integrate(t, R, T);
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) R_t[3 * i + j] = R[i][j];
    T_t[i] = T[i];
  }
}

} // extern "C"
