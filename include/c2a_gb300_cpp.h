/*
 * c2a_gb300_cpp.h -- C++ drop-in for the C2A conservative-advancement API.
 *
 * Same names, signatures and result fields as the reference's C2A/C2A.h,
 * C2A/C2A_Internal.h, C2A/InterpMotion.h and the Transform / Quaternion /
 * Coord3D / Matrix3x3 subset of C2A/LinearMath.h that the CA entry points
 * use, so a program written against the reference recompiles against this
 * header.  Every query runs on the GPU through the C ABI of c2a_gb300.h; the
 * classes here only hold inputs and results.
 *
 *   C2A_Solve               C2A/C2A.h:23-35           (C2A/src/C2A.cpp:2315-2444)
 *   C2A_QueryTimeOfContact  C2A/C2A.h:274-281         (C2A/src/C2A.cpp:1987-2146)
 *   C2A_TimeOfContactStep   C2A/src/C2A.cpp:1778-1789 (not in the reference's header)
 *   C2A_QueryContact        C2A/C2A.h:284-290         (C2A/src/C2A.cpp:1937-1966)
 *   C2A_QueryContactOnly    C2A/C2A.h:292-299         (C2A/src/C2A.cpp:1968-1983)
 *   C2A_Model               C2A/C2A_Internal.h:32-81  (C2A/src/C2A_PQP.cpp:61-438)
 *   CInterpMotion_Linear    C2A/InterpMotion.h:164-226
 *   C2A_Distance            C2A/C2A.h:256-260         (C2A/src/C2A_PQP.cpp:971-1056; rel_err = abs_err = 0)
 *   C2A_Tolerance           C2A/src/C2A_PQP.cpp:1762-1845 (not in the reference's header)
 *   C2A_Collide             C2A/C2A.h:249-253         (C2A/src/C2A_PQP.cpp:910-968)
 *   PQP_CollideResult, PQP_ToleranceResult, C2A_DistanceResult: the accessors
 *                           of the PQP result classes those queries fill
 *   C2A_SolveBatch          new: many independent C2A_Solve queries in one launch
 *
 * Differences a caller can see: C2A_Solve reads th_ca (the reference ignores
 * it and uses 1e-4, C2A.cpp:2326, 2384-2388; pass th_ca <= 0 to get exactly
 * the reference's behaviour), prints nothing, and is safe to call from
 * several threads (the reference keeps a global translation flag,
 * C2A.cpp:33).
 */
#ifndef C2A_GB300_CPP_H
#define C2A_GB300_CPP_H

#include <list>
#include <vector>

#include "c2a_gb300.h"

#ifndef PQP_REAL
#define PQP_REAL double
#endif
typedef double Real;

enum C2A_Result { OK, TOCFound, CollisionFound, CollisionFree, CollisionNotFound };

/* ---------------------------------------------------- LinearMath subset */
class Quaternion {
  public:
    Quaternion() : val{0.0, 0.0, 0.0, 1.0} {}
    Quaternion(Real x, Real y, Real z, Real w) : val{x, y, z, w} {}
    Real &X() { return val[0]; }
    Real &Y() { return val[1]; }
    Real &Z() { return val[2]; }
    Real &W() { return val[3]; }
    Real X() const { return val[0]; }
    Real Y() const { return val[1]; }
    Real Z() const { return val[2]; }
    Real W() const { return val[3]; }
    Real &operator[](int i) { return val[i & 3]; }
    Real operator[](int i) const { return val[i & 3]; }

  private:
    Real val[4];
};

class Coord3D {
  public:
    Coord3D() : val{0.0, 0.0, 0.0} {}
    Coord3D(Real x, Real y, Real z) : val{x, y, z} {}
    Real &X() { return val[0]; }
    Real &Y() { return val[1]; }
    Real &Z() { return val[2]; }
    Real X() const { return val[0]; }
    Real Y() const { return val[1]; }
    Real Z() const { return val[2]; }
    Real &operator[](int i) { return val[i % 3]; }
    Real operator[](int i) const { return val[i % 3]; }
    void Get_Value(Real v[]) const { v[0] = val[0], v[1] = val[1], v[2] = val[2]; }
    void Set_Value(const Real v[]) { val[0] = v[0], val[1] = v[1], val[2] = v[2]; }
    void Set_Value(Real x, Real y, Real z) { val[0] = x, val[1] = y, val[2] = z; }

  private:
    Real val[3];
};

class Matrix3x3 {
  public:
    Matrix3x3() : val{1, 0, 0, 0, 1, 0, 0, 0, 1} {}
    Real *operator[](int i) { return &val[(i % 3) * 3]; }
    const Real *operator[](int i) const { return &val[(i % 3) * 3]; }
    void Get_Value(Real v[3][3]) const;
    void Set_Value(const Real v[3][3]);
    void Set_Value(const Quaternion &q); /* LinearMath.h:809-829 */
    const Real *data() const { return val; }

  private:
    Real val[9];
};

class Transform {
  public:
    Transform() {}
    Matrix3x3 &Rotation() { return R; }
    const Matrix3x3 &Rotation() const { return R; }
    Coord3D &Translation() { return T; }
    const Coord3D &Translation() const { return T; }
    void Set_Rotation(const Matrix3x3 &r) { R = r; }
    void Set_Rotation(const Quaternion &q) { R.Set_Value(q); }
    void Set_Translation(const Coord3D &t) { T = t; }

  private:
    Matrix3x3 R;
    Coord3D T;
};

/* ---------------------------------------------------------------- model */
struct Tri {
    PQP_REAL p1[3];
    PQP_REAL p2[3];
    PQP_REAL p3[3];
    int id;
};

struct C2A_Tri : public Tri {
    int *Index() { return index_; }
    int index_[3];
};

/* Triangle soup with its RSS hierarchy.  EndModel builds the hierarchy on
 * the host exactly as the reference does and uploads it to the GPU of the
 * process-wide context (device 0 unless C2A_SetDevice was called). */
class C2A_Model {
  public:
    C2A_Model();
    ~C2A_Model();
    C2A_Model(const C2A_Model &) = delete;
    C2A_Model &operator=(const C2A_Model &) = delete;

    int BeginModel(int n = 8);
    int AddTri(const PQP_REAL *p1, const PQP_REAL *p2, const PQP_REAL *p3, int i, int i1, int i2, int i3);
    int AddTri(const PQP_REAL *p1, const PQP_REAL *p2, const PQP_REAL *p3, int id);
    int EndModel();
    C2A_Tri *GetTriangle(int idx) { return &tris[idx]; }

    int build_state;               /* 0 empty, 1 begun, 2 processed */
    int num_tris;
    std::vector<C2A_Tri> tris;     /* post-build order after EndModel */
    std::vector<C2A_Tri> trisConst;/* insertion order */
    C2A_Tri *last_tri;             /* default seed: tris[0] after EndModel */
    int num_bvs;
    int maxdeep;
    c2a_context *ctx;              /* GPU context holding the hierarchy */
    int32_t model_id;
};

/* ---------------------------------------------------------------- motion */
enum GMP_INTERP_MODE { GMP_IM_EULER = 0, GMP_IM_LINEAR = 1, GMP_IM_SCREW = 2, GMP_IM_SLERP = 3 };

class CInterpMotion {
  public:
    CInterpMotion();
    virtual ~CInterpMotion();
    virtual bool integrate(const double dt, PQP_REAL qua[7]) = 0;
    bool integrate(const double dt, PQP_REAL R[3][3], PQP_REAL T[3]);

    Real m_toc_delta;
    GMP_INTERP_MODE m_itpMode;
    Transform transform;   /* current pose */
    Transform transform_s; /* begin pose */
    Transform transform_t; /* end pose */
    Coord3D cv;            /* linear velocity */
    Coord3D m_axis;        /* rotation axis (body frame), unit */
    Real m_angVel;         /* rotation angle over t in [0, 1] */
    Real m_time;           /* time of `transform` (0: the begin pose as given) */
};

class CInterpMotion_Linear : public CInterpMotion {
  public:
    CInterpMotion_Linear(const PQP_REAL R0[3][3], const PQP_REAL T0[3], const PQP_REAL R1[3][3],
                         const PQP_REAL T1[3]);
    virtual ~CInterpMotion_Linear();
    virtual bool integrate(const double dt, PQP_REAL qua[7]);
    using CInterpMotion::integrate;
};

/* ---------------------------------------------------------------- results */
struct ContactF {
    ContactF(int FeatureType_A, int FeatureType_B, const int FeatureID_A[3], const int FeatureID_B[3],
             int TriangleID_A, int TriangleID_B, const PQP_REAL P_A[3], const PQP_REAL P_B[3], PQP_REAL Distance);
    int FeatureType_A, FeatureType_B;
    int FeatureID_A[3], FeatureID_B[3];
    int TriangleID_A, TriangleID_B;
    PQP_REAL P_A[3], P_B[3];
    PQP_REAL Distance;
};
typedef std::list<ContactF> ContactFList;

struct C2A_TimeOfContactResult {
    int num_bv_tests;
    int num_tri_tests;
    double query_time_secs;
    ContactFList cont_l;
    PQP_REAL R[3][3];
    PQP_REAL T[3];
    PQP_REAL rel_err;
    PQP_REAL abs_err;
    PQP_REAL UpboundTOC;
    PQP_REAL distance;
    PQP_REAL p1[3];
    PQP_REAL p2[3];
    int qsize;
    PQP_REAL mint;
    PQP_REAL toc;
    bool collisionfree;
    int numCA;
    PQP_REAL R_toc[3][3], T_toc[3];
    int num_contact;
    Tri *last_triA;
    Tri *last_triB;
    int status; /* C2A_QUERY_* flags of the GPU query */

    C2A_TimeOfContactResult();
    int NumBVTests() { return num_bv_tests; }
    int NumTriTests() { return num_tri_tests; }
    double QueryTimeSecs() { return query_time_secs; }
    PQP_REAL Distance() { return distance; }
    const PQP_REAL *P1() { return p1; }
    const PQP_REAL *P2() { return p2; }
};

/* ---------------------------------------------------------------- API */
/* selects the GPU of the process-wide context (before the first model) */
int C2A_SetDevice(int device);
c2a_context *C2A_DefaultContext();

C2A_Result C2A_Solve(Transform *trans00, Transform *trans01, C2A_Model *obj1_tested, Transform *trans10,
                     Transform *trans11, C2A_Model *obj2_tested, Transform &trans0, Transform &trans1,
                     PQP_REAL &time_of_contact, int &number_of_iteration, int &number_of_contact, PQP_REAL th_ca,
                     C2A_TimeOfContactResult &dres);

PQP_REAL C2A_QueryTimeOfContact(CInterpMotion *objmotion1, CInterpMotion *objmotion2, C2A_TimeOfContactResult *res,
                                C2A_Model *o1, C2A_Model *o2, PQP_REAL tolerance_d, PQP_REAL tolerance_t,
                                int qsize = 2);

int C2A_TimeOfContactStep(CInterpMotion *objmotion1, CInterpMotion *objmotion2, C2A_TimeOfContactResult *res,
                          PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3], PQP_REAL T2[3],
                          C2A_Model *o2, PQP_REAL tolerance_t, PQP_REAL tolerance_d);

PQP_REAL C2A_QueryContact(CInterpMotion *objmotion1, CInterpMotion *objmotion2, C2A_TimeOfContactResult *res,
                          C2A_Model *o1, C2A_Model *o2, double threshold);

PQP_REAL C2A_QueryContactOnly(C2A_TimeOfContactResult *res, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1,
                              PQP_REAL R2[3][3], PQP_REAL T2[3], C2A_Model *o2, double threshold);

/* ------------------------------------------------- static proximity queries */
const int C2A_ALL_CONTACTS = 1;  /* every contacting triangle pair */
const int C2A_FIRST_CONTACT = 2; /* the first one found */

struct CollisionPair {
    int id1, id2; /* caller triangle ids */
};

/* PQP_CollideResult's public face: counters and the contacting pairs in the
 * order the query found them */
class PQP_CollideResult {
  public:
    int num_bv_tests = 0, num_tri_tests = 0;
    double query_time_secs = 0;
    PQP_REAL R[3][3] = {}, T[3] = {}; /* model 2 in model 1's frame */
    std::vector<CollisionPair> pairs;
    int NumBVTests() { return num_bv_tests; }
    int NumTriTests() { return num_tri_tests; }
    double QueryTimeSecs() { return query_time_secs; }
    int Colliding() { return !pairs.empty(); }
    int NumPairs() { return (int)pairs.size(); }
    int Id1(int k) { return pairs[k].id1; }
    int Id2(int k) { return pairs[k].id2; }
    void FreePairsList() { pairs.clear(); }
};

/* PQP_ToleranceResult's public face */
class PQP_ToleranceResult {
  public:
    int num_bv_tests = 0, num_tri_tests = 0;
    double query_time_secs = 0;
    PQP_REAL R[3][3] = {}, T[3] = {};
    int closer_than_tolerance = 0;
    PQP_REAL tolerance = 0, distance = 0, p1[3] = {}, p2[3] = {};
    int NumBVTests() { return num_bv_tests; }
    int NumTriTests() { return num_tri_tests; }
    double QueryTimeSecs() { return query_time_secs; }
    int CloserThanTolerance() { return closer_than_tolerance; }
    PQP_REAL Distance() { return distance; }
    const PQP_REAL *P1() { return p1; }
    const PQP_REAL *P2() { return p2; }
};

/* C2A_DistanceResult's public face (the closest pair as triangles and ids) */
class C2A_DistanceResult {
  public:
    int num_bv_tests = 0, num_tri_tests = 0;
    double query_time_secs = 0;
    PQP_REAL R[3][3] = {}, T[3] = {};
    PQP_REAL rel_err = 0, abs_err = 0, distance = 0, p1[3] = {}, p2[3] = {};
    int qsize = 2;
    Tri *last_triA = nullptr, *last_triB = nullptr;
    int t1 = -1, t2 = -1; /* caller ids of the closest pair */
    int NumBVTests() { return num_bv_tests; }
    int NumTriTests() { return num_tri_tests; }
    double QueryTimeSecs() { return query_time_secs; }
    PQP_REAL Distance() { return distance; }
    const PQP_REAL *P1() { return p1; }
    const PQP_REAL *P2() { return p2; }
};

/* The exact distance (rel_err = abs_err = 0 only; other values return
 * C2A_ERR_INVALID_ARGUMENT), seeded with o1->last_tri / o2->last_tri; the
 * closest pair comes back in result->last_triA/B (the models are not
 * changed).  Returns 0 (PQP_OK) or a c2a_status. */
int C2A_Distance(C2A_DistanceResult *result, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                 PQP_REAL T2[3], C2A_Model *o2, PQP_REAL rel_err, PQP_REAL abs_err, int qsize = 2);

/* Is any triangle pair within `tolerance`? (qsize 2: the depth-first order
 * with the closer child first, stopping at the first such pair) */
int C2A_Tolerance(PQP_ToleranceResult *res, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                  PQP_REAL T2[3], C2A_Model *o2, PQP_REAL tolerance, int qsize = 2);

/* The contacting triangle pairs (all, or the first found) */
int C2A_Collide(PQP_CollideResult *result, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                PQP_REAL T2[3], C2A_Model *o2, int flag = C2A_ALL_CONTACTS);

/* One query of C2A_SolveBatch: the four poses of C2A_Solve and the seed pair
 * (dres.last_triA/B); seed < 0 means the model's last_tri. */
struct C2A_BatchQuery {
    Transform *trans00, *trans01; /* object 1 begin / end */
    C2A_Model *obj1;
    Transform *trans10, *trans11; /* object 2 begin / end */
    C2A_Model *obj2;
    int seed1, seed2;
};

/* n independent C2A_Solve queries in one GPU launch; th_ca as in C2A_Solve;
 * results[i] receives what dres receives in C2A_Solve.  Returns the number of
 * queries with a non-zero status (0 on success). */
int C2A_SolveBatch(const C2A_BatchQuery *queries, int n, PQP_REAL th_ca, C2A_TimeOfContactResult *results,
                   int contacts_per_query = 256);

#endif
