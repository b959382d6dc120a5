/*
 * c2a_port.h -- CPU oracle: a plain-C restatement of C2A's controlled
 * conservative advancement (CA) path; test infrastructure, used by the
 * tests, smoke() and the bench's CPU baseline to verify and time the CUDA
 * path.  Nothing in the product links it.
 *
 * It follows the reference function by function (file:line in each
 * definition): the RSS BVH build (C2A/src/C2A_Build.cpp, C2A/src/C2A_BV.cpp),
 * the linear motion (C2A/src/InterpMotion.cpp), the RSS and triangle
 * distances (C2A/C2A_RectDist.h, C2A/src/C2A.cpp:59-424), the BVTT CA step
 * and CA loop (C2A/src/C2A.cpp:1114-2146), contact enumeration
 * (C2A/src/C2A.cpp:1525-1775) and C2A_Solve (C2A/src/C2A.cpp:2315-2444).
 * Arithmetic is repeated operation for operation; build with
 * -ffp-contract=off.  sin/cos/acos come from c2a_detmath.h.
 */
#ifndef C2A_PORT_H
#define C2A_PORT_H

/* Operation-count attribution: oracle/flop_count.cpp compiles the port with a
 * counting double and defines this to open a scope whose arithmetic goes to
 * bucket k (1: a node-pair expansion, 2: a leaf triangle test, 3: contact
 * enumeration); empty everywhere else. */
#ifndef C2A_PORT_SCOPE
#define C2A_PORT_SCOPE(k)
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct c2a_port_node {
    double R[3][3];     /* RSS orientation, parent-relative */
    double Tr[3];       /* RSS rectangle corner, parent-relative */
    double l[2];        /* rectangle side lengths */
    double r;           /* swept-sphere radius */
    double angR;        /* max vertex distance from the model origin */
    double Rloc[3][3];  /* build-time orientation in the model frame */
    double To[3];       /* OBB centre, parent-relative (the static collide query) */
    double d[3];        /* OBB half extents */
    int first_child;    /* >= 0 child index; < 0: -(triangle)-1 */
    int pad;
} c2a_port_node;

typedef struct c2a_port_tri {
    double p1[3], p2[3], p3[3];
    int id;             /* caller's triangle id */
    int idx[3];         /* caller's vertex indices */
} c2a_port_tri;

typedef struct c2a_port_model {
    int num_tris;
    int num_nodes;
    c2a_port_tri *tris;   /* post-build order (the build permutes them) */
    c2a_port_node *nodes; /* 2n-1 nodes, root at 0 */
} c2a_port_model;

/* Builds the RSS hierarchy; tri_verts is num_tris x 9 doubles (p1,p2,p3),
 * ids and vidx (num_tris x 3) may be NULL (then id = i, vidx = -1). */
int c2a_port_model_build(c2a_port_model *m, int num_tris, const double *tri_verts,
                         const int *ids, const int *vidx);
void c2a_port_model_free(c2a_port_model *m);
/* Eigen-decomposition of a symmetric 3x3 matrix (cyclic Jacobi). */
void c2a_port_jacobi3(double vout[3][3], double dout[3], const double a[3][3]);

typedef struct c2a_port_params {
    double tol_d;        /* tolerance_d: contact distance (C2A.cpp:2384) */
    double tol_t;        /* tolerance_t: minimum step (C2A.cpp:2385) */
    double toc_delta;    /* CInterpMotion::m_toc_delta (C2A.cpp:2387-2388) */
    double contact_abs;  /* absolute term of the contact threshold (C2A.cpp:2433) */
    int with_contacts;   /* run the contact enumeration at the TOC */
    int max_iters;       /* CA iteration cap, 150 in the reference (C2A.cpp:2079) */
    int mode;            /* C2A_PORT_MODE_REFERENCE or C2A_PORT_MODE_CANONICAL */
    int reserved;
} c2a_port_params;

/* REFERENCE: every step starts from the caller's seed pair, as C2A_Solve does.
 * CANONICAL: every step first finds the closest triangle pair with the
 * reference's distance query (C2ADistanceRecurse, rel_err = abs_err = 0) and
 * seeds the step with it, so the step's running bound starts at the exact
 * minimum distance and its result no longer depends on the traversal order;
 * contacts are sorted by (tri_a, tri_b). */
enum { C2A_PORT_MODE_REFERENCE = 0, C2A_PORT_MODE_CANONICAL = 1 };

/* The reference's distance query from a seed pair (C2A_Distance with
 * rel_err = abs_err = 0, qsize <= 2; C2A/src/C2A_PQP.cpp:971-1056, 481-621):
 * R/T place model B in model A; returns the minimum distance and the
 * closest pair in *ta, *tb; counters in *nbv, *ntri (may be NULL). */
double c2a_port_distance(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                         int seed_a, int seed_b, int *ta, int *tb, long long *nbv, long long *ntri);

/* C2A_Tolerance (qsize 2) with B placed in A's frame by (R, T): returns
 * closer_than_tolerance; when set, the distance and closest points (p1 in
 * A's frame, p2 in B's) of the first pair found within the tolerance */
int c2a_port_tolerance(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                       double tolerance, double *distance, double p1[3], double p2[3], long long *nbv,
                       long long *ntri);

/* C2A_Collide (the PQP_CollideResult form, C2A_PQP.cpp:798-968) with B placed
 * in A's frame by (R, T); flag 1 all contacts, 2 the first only.  Writes up
 * to cap (id_a, id_b) caller-id pairs in the order found; returns the
 * number of pairs found. */
int c2a_port_collide(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                     int flag, int *pairs, int cap, long long *nbv, long long *ntri);

typedef struct c2a_port_contact {
    int type_a, type_b;  /* 1 vertex, 2 edge, 3 face (C2A.cpp:1584-1585) */
    int fid_a[3], fid_b[3]; /* vertex indices of the features, -1 unused */
    int tri_a, tri_b;    /* post-build triangle indices */
    double pa[3], pb[3]; /* closest points, each in its own model frame */
    double distance;
} c2a_port_contact;

typedef struct c2a_port_result {
    int collisionfree;
    int numCA;
    int translation;     /* both angular speeds < 1e-8: translation CA */
    int num_contact;
    double toc;
    double distance;     /* res->distance after the last CA step */
    double mint;         /* res->mint after the last CA step */
    long long num_bv_tests;
    long long num_tri_tests;
    double R_toc[2][9];  /* poses at the TOC when not collision free */
    double T_toc[2][3];
    int seed_a, seed_b;  /* seed pair after the query (changes only in translation CA) */
} c2a_port_result;

/* One full C2A_Solve-style query (harness form: tolerance_d and m_toc_delta
 * come from params).  Poses are row-major 3x3 + 3.  seed_a/seed_b are the
 * post-build triangle indices of the initial upper-bound pair.  contacts may
 * be NULL; at most max_contacts are written, num_contact counts all. */
int c2a_port_solve(const c2a_port_model *A, const c2a_port_model *B,
                   const double R0a[9], const double T0a[3], const double R1a[9], const double T1a[3],
                   const double R0b[9], const double T0b[3], const double R1b[9], const double T1b[3],
                   int seed_a, int seed_b, const c2a_port_params *prm,
                   c2a_port_result *res, c2a_port_contact *contacts, int max_contacts);

/* Independent queries over host threads.  qint is n x 4 (model_a, model_b,
 * seed_a, seed_b), poses n x 48 (R0a T0a R1a T1a R0b T0b R1b T1b, row-major);
 * query q writes res[q] and up to contacts_per_query contacts at
 * contacts + q * contacts_per_query.  Returns the number of rejected queries. */
int c2a_port_solve_batch(const c2a_port_model *models, int num_models, const int *qint, const double *poses, int n,
                         const c2a_port_params *prm, c2a_port_result *res, c2a_port_contact *contacts,
                         int contacts_per_query, int num_threads);

/* One CA step (C2A_TimeOfContactStep) of the query's motions at time lambda
 * (0: the begin poses as given), with the schedule inputs num_ca and
 * prev_mint; fills distance, mint, counters, translation and seeds. */
int c2a_port_step(const c2a_port_model *A, const c2a_port_model *B, const double pose48[48], int seed_a,
                  int seed_b, double lambda, int num_ca, double prev_mint, const c2a_port_params *prm,
                  c2a_port_result *res);

/* Contact enumeration alone (C2A_QueryContactOnly, C2A.cpp:1968-1983). */
int c2a_port_contact_only(const c2a_port_model *A, const c2a_port_model *B,
                          const double Ra[9], const double Ta[3], const double Rb[9], const double Tb[3],
                          double threshold, c2a_port_contact *contacts, int max_contacts);

/* Geometry kernels exposed for unit tests. */
double c2a_port_rectdist(const double Rab[9], const double Tab[3], const double a[2], const double b[2],
                         double P[3], double Q[3], double S[3]);
double c2a_port_tridist(double P[3], double Q[3], const double S[9], const double T[9],
                        int *f1_type, int *f1_fid, int *f2_type, int *f2_fid, int *collided);

/* Linear motion (CInterpMotion_Linear) exposed for unit tests. */
typedef struct c2a_port_motion {
    double R0[3][3], T0[3];  /* transform_s */
    double q0[4];            /* transform_s.Quaternion_(), (x, y, z, w) */
    double cv[3];            /* T1 - T0 */
    double axis[3];          /* m_axis */
    double angVel;           /* m_angVel */
    double toc_delta;
    double R[3][3], T[3];    /* current transform */
} c2a_port_motion;

void c2a_port_motion_init(c2a_port_motion *m, const double R0[9], const double T0[3],
                          const double R1[9], const double T1[3]);
void c2a_port_motion_integrate(c2a_port_motion *m, double dt, double R[9], double T[3], double qua[7]);

#ifdef __cplusplus
}
#endif
#endif
