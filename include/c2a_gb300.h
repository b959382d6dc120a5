/*
 * c2a_gb300.h -- C ABI of the GB300-native C2A conservative-advancement (CA)
 * library (libc2a_gb300.so).  Plain pointers and sizes only; every call
 * returns a c2a_status.  This is the boundary a host program, a ctypes/cgo
 * binding, or the C++ drop-in API (c2a_gb300_cpp.h) binds to.
 *
 * Reference interfaces replaced (paths within EwhaGlab/C2A):
 *   c2a_model_build          C2A_Model::BeginModel/AddTri/EndModel
 *                            (C2A/src/C2A_PQP.cpp:82-417) with the RSS
 *                            hierarchy build of C2A_BuildModel
 *                            (C2A/src/C2A_Build.cpp:546-574)
 *   c2a_model_build_many,    the same EndModel for many models at once, or
 *   c2a_model_build_async,   in two halves (the build on host threads, then
 *   c2a_model_wait           the upload)
 *   c2a_solve_batch          C2A_Solve (C2A/C2A.h:23-35, C2A/src/C2A.cpp:2315)
 *                            over many independent queries; each query is
 *                            C2A_QueryTimeOfContact (C2A/C2A.h:274-281)
 *                            followed, when not collision free, by
 *                            C2A_QueryContact (C2A/C2A.h:284-290)
 *   c2a_toc_step_batch       C2A_TimeOfContactStep (C2A/src/C2A.cpp:1778-1789)
 *   c2a_contact_only_batch   C2A_QueryContactOnly (C2A/C2A.h:292-299)
 *   c2a_motion_setup         CInterpMotion_Linear ctor/velocity
 *                            (C2A/src/InterpMotion.cpp:494-502, 228-270)
 *   c2a_motion_integrate     CInterpMotion_Linear::integrate
 *                            (C2A/src/InterpMotion.cpp:516-568)
 *
 * Semantics follow the reference exactly (FP64, same evaluation order; the
 * reference's C2A_Solve hard-codes tolerance_d = m_toc_delta = 1e-4 and
 * ignores th_ca, here they are parameters).  Results are bit-identical to the
 * reference on the same inputs.
 */
#ifndef C2A_GB300_H
#define C2A_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t c2a_status;
enum {
    C2A_OK = 0,
    C2A_ERR_INVALID_ARGUMENT = 1,
    C2A_ERR_NO_DEVICE = 2,
    C2A_ERR_CUDA = 3,
    C2A_ERR_OUT_OF_MEMORY = 4,
    C2A_ERR_EMPTY_MODEL = 5,      /* PQP_ERR_BUILD_EMPTY_MODEL (C2A_PQP.cpp:352-357) */
    C2A_ERR_BAD_MODEL = 6,        /* unknown or freed model id */
    C2A_ERR_TREE_TOO_DEEP = 7,    /* BVTT deeper than the traversal stack */
    C2A_ERR_QUERY_FAILED = 8,     /* at least one query has a non-zero status */
    C2A_ERR_NOALLOC_CAPACITY = 9  /* more models than c2a_solve_batch_noalloc's fixed table holds */
};

/* per-query status word (c2a_result.status), bit flags */
enum {
    C2A_QUERY_OK = 0,
    C2A_QUERY_BAD_INPUT = 1,        /* model id or seed triangle out of range */
    C2A_QUERY_STACK_OVERFLOW = 2,   /* traversal stack exhausted (never with checked models) */
    C2A_QUERY_CONTACT_OVERFLOW = 4, /* more contacts than contacts_per_query (num_contact is still exact) */
    C2A_QUERY_ITER_CAP = 8          /* hit max_iters; reported as contact at the last lambda, like the reference */
};

typedef struct c2a_context c2a_context;

/* Query: two models, the seed pair (C2A's dres.last_triA/B, post-build
 * triangle indices) and the four poses of C2A_Solve, each row-major R(9) then
 * T(3): A at t=0, A at t=1, B at t=0, B at t=1 (48 doubles). */
typedef struct c2a_query {
    int32_t model_a, model_b;
    int32_t seed_a, seed_b;
    double pose[48];
} c2a_query;

typedef struct c2a_params {
    double tol_d;        /* tolerance_d (C2A_Solve: 1e-4, C2A.cpp:2384) */
    double tol_t;        /* tolerance_t (C2A_Solve: 1e-4, C2A.cpp:2385) */
    double toc_delta;    /* CInterpMotion::m_toc_delta (C2A_Solve: 1e-4) */
    double contact_abs;  /* contact threshold = 2 d + contact_abs (C2A.cpp:2433: 0.001) */
    int32_t with_contacts;      /* enumerate contacts at the TOC */
    int32_t max_iters;          /* CA iteration cap (reference: 150) */
    int32_t qsize;              /* front capacity hint; never changes a result */
    int32_t contacts_per_query; /* contact slots per query in the output buffer */
    int32_t mode;               /* C2A_MODE_REFERENCE or C2A_MODE_CANONICAL */
    int32_t engine;             /* C2A_ENGINE_*; never changes a result */
    int32_t warps_per_sm;       /* launch shape: resident warps per SM of the solve kernel, 0 the most
                                   that fit (c2a_gb300.tune picks it); never changes a result */
    int32_t heavy_prefix;       /* ordered REFERENCE batches on the warp engine: the first heavy_prefix
                                   entries of the order (the costliest queries) each get an SM
                                   sub-partition of their own; 0: none.  Never changes a result */
} c2a_params;

/* C2A_MODE_REFERENCE: the reference's results bit for bit (its depth-first
 * order; every step starts from the caller's seed pair, as C2A_Solve does).
 * C2A_MODE_CANONICAL: before every rotation step, the reference's distance
 * query (C2A_Distance with rel_err = abs_err = 0, C2A/src/C2A_PQP.cpp:971)
 * finds the closest triangle pair and seeds the step with it, so each step's
 * result is independent of traversal order; one warp runs each query over a
 * parallel front.  Results equal that composition of the reference's own
 * functions; contacts come sorted by (tri_a, tri_b), seed_a/seed_b are the
 * last step's closest pair (ties: the smallest pair).  When a query has more
 * contacts than contacts_per_query, num_contact and C2A_QUERY_CONTACT_OVERFLOW
 * are exact but which of them fill the slots is unspecified in this mode. */
#define C2A_MODE_REFERENCE 0
#define C2A_MODE_CANONICAL 1

/* How a batch runs (never changes a result):
 * C2A_ENGINE_AUTO     one warp per query;
 * C2A_ENGINE_WARP     one warp per query: REFERENCE mode keeps the reference's
 *                     depth-first order and splits each node-pair test across the lanes
 *                     (the sixteen RectDist cases, the nine TriDist segment pairs);
 *                     CANONICAL mode walks a warp-shared front of node pairs;
 * C2A_ENGINE_BATCHED  CANONICAL only: every query in lockstep CA iterations, each phase
 *                     a series of waves over all queries' node pairs (the call
 *                     synchronises the stream between waves);
 * C2A_ENGINE_THREAD   REFERENCE only: one thread per query;
 * C2A_ENGINE_SPEC     REFERENCE only: one warp per query by speculative expansion
 *                     and ordered replay -- each round the warp tests up to sixteen
 *                     node pairs the reference's order is about to need (two lanes
 *                     each, certified FP32 with FP64 where undecided), then replays
 *                     the reference's decisions over them. */
#define C2A_ENGINE_AUTO 0
#define C2A_ENGINE_WARP 1
#define C2A_ENGINE_BATCHED 2
#define C2A_ENGINE_THREAD 3
#define C2A_ENGINE_SPEC 4

typedef struct c2a_result {
    int32_t collisionfree;
    int32_t numCA;
    int32_t translation;   /* both angular speeds < 1e-8: translation-only CA */
    int32_t num_contact;   /* all contacts found (may exceed contacts_per_query) */
    double toc;
    double distance;       /* res->distance after the last CA step */
    double mint;           /* res->mint after the last CA step */
    int64_t num_bv_tests;  /* reference counters (C2A.cpp:1180, 1279) */
    int64_t num_tri_tests;
    double R_toc[2][9];    /* poses at the TOC (when not collision free) */
    double T_toc[2][3];
    int32_t seed_a, seed_b; /* seed pair after the query */
    int32_t status;        /* C2A_QUERY_* flags */
    int32_t contact_offset; /* first of this query's contacts in the contact buffer */
} c2a_result;

/* One contact pair (ContactF, C2A/C2A.h:116-158), in the order the reference
 * visits them (its list is built with push_front, so reversed). */
typedef struct c2a_contact {
    int32_t type_a, type_b;         /* 1 vertex, 2 edge, 3 face */
    int32_t fid_a[3], fid_b[3];     /* caller vertex indices of the features, -1 unused */
    int32_t tri_a, tri_b;           /* post-build triangle indices */
    int32_t query, pad;             /* index of the query in its batch */
    double pa[3], pb[3];            /* closest points, each in its own model frame */
    double distance;
} c2a_contact;

/* Result of one distance query (C2A_Distance with rel_err = abs_err = 0,
 * C2A/src/C2A_PQP.cpp:970-1056): the exact minimum TriDist over all triangle
 * pairs.  distance is order-independent; ties between pairs go to the
 * smallest (tri_a, tri_b), where the reference keeps the first pair its
 * depth-first order meets. */
typedef struct c2a_distance_result {
    double distance;       /* res->distance */
    double p1[3];          /* closest point on model a, in model a's frame (res->p1) */
    double p2[3];          /* closest point on model b, in model b's frame (res->p2) */
    int32_t tri_a, tri_b;  /* the closest pair, post-build indices (the models' last_tri) */
    int32_t status;        /* C2A_QUERY_* flags */
    int32_t pad;
} c2a_distance_result;

/* C2A_Tolerance's outputs (PQP_ToleranceResult) for one pair of placed models */
typedef struct c2a_tolerance_result {
    int32_t closer;        /* a triangle pair lies within the tolerance (closer_than_tolerance) */
    int32_t status;        /* C2A_QUERY_* flags */
    double distance;       /* that pair's distance (when closer) */
    double p1[3];          /* its closest point on model a, model a's frame */
    double p2[3];          /* its closest point on model b, model b's frame */
    int64_t num_bv_tests;  /* reference counters */
    int64_t num_tri_tests;
} c2a_tolerance_result;

/* C2A_Collide's counts (PQP_CollideResult) for one pair of placed models; the
 * contacting triangle pairs (caller ids) go to a separate buffer */
typedef struct c2a_collide_result {
    int32_t num_pairs;     /* all contacting pairs found (may exceed the slots) */
    int32_t status;        /* C2A_QUERY_* flags (CONTACT_OVERFLOW: more pairs than slots) */
    int64_t num_bv_tests;
    int64_t num_tri_tests;
} c2a_collide_result;

/* ---- context --------------------------------------------------------- */
/* device >= 0: a CUDA device; device == -1: a host-only context that builds
 * and downloads models but runs no query (C2A_ERR_NO_DEVICE). */
c2a_status c2a_create(int device, c2a_context **ctx);
c2a_status c2a_destroy(c2a_context *ctx);
const char *c2a_status_str(c2a_status s);
/* number of kernel launches issued by this context so far */
c2a_status c2a_launch_count(c2a_context *ctx, int64_t *count);

/* ---- models ---------------------------------------------------------- */
/* Builds the RSS hierarchy of a triangle soup on the host (bit-identical to
 * the reference's EndModel) and uploads it.  tri_verts: num_tris x 9 doubles
 * (p1, p2, p3); ids and vidx (num_tris x 3) may be NULL.  Subtrees of 4,096
 * triangles or more build on parallel host threads (C2A_BUILD_THREADS, else
 * every hardware thread); the tree does not depend on the thread count. */
c2a_status c2a_model_build(c2a_context *ctx, int32_t num_tris, const double *tri_verts, const int32_t *ids,
                           const int32_t *vidx, int32_t *model_id);
/* c2a_model_build over count models at once (the reference builds each
 * C2A_Model on its own, C2A/src/C2A_PQP.cpp:332-417): the models build on
 * parallel host threads, largest first, and a model's subtrees split over
 * the threads the others leave free.  threads: host threads to use (at most
 * 256), 0 for C2A_BUILD_THREADS or else every hardware thread.  ids and vidx may be NULL,
 * or hold NULL entries.  model_ids[i] is model i's id, in the order given;
 * every tree is bit-identical to a c2a_model_build of the same model.  On an
 * error no model of the call is kept. */
c2a_status c2a_model_build_many(c2a_context *ctx, int32_t count, const int32_t *num_tris,
                                const double *const *tri_verts, const int32_t *const *ids,
                                const int32_t *const *vidx, int32_t threads, int32_t *model_ids);
/* c2a_model_build in two halves, so that a model builds on host threads
 * while the GPU works on queries of the models already uploaded:
 * c2a_model_build_async copies the arrays and returns at once with a handle;
 * c2a_model_wait finishes the build, uploads the model, returns its id (or
 * the build's error, -1 as the id) and frees the handle.  Every handle must
 * be waited for once, before the context is destroyed. */
typedef struct c2a_build_handle c2a_build_handle;
c2a_status c2a_model_build_async(c2a_context *ctx, int32_t num_tris, const double *tri_verts, const int32_t *ids,
                                 const int32_t *vidx, c2a_build_handle **handle);
c2a_status c2a_model_wait(c2a_build_handle *handle, int32_t *model_id);
c2a_status c2a_model_info(c2a_context *ctx, int32_t model_id, int32_t *num_tris, int32_t *num_nodes,
                          int32_t *depth);
/* Host copy of the built hierarchy: node_f num_nodes x 25 doubles (R 9, Tr 3,
 * l 2, r, angularRadius, R_loc 9), first_child, triangles in post-build
 * order (9 doubles, id, 3 vertex indices). */
c2a_status c2a_model_download(c2a_context *ctx, int32_t model_id, double *node_f, int32_t *first_child,
                              double *tri_verts, int32_t *tri_ids, int32_t *tri_vidx);
/* The OBB of every node (the collide query's bounding volumes, fitted in the
 * RSS frame as C2A/src/C2A_BV.cpp:144-170 does): 6 doubles per node, the
 * centre relative to the parent's frame (make_parent_relative,
 * C2A/src/C2A_Build.cpp:493-544) and the half extents. */
c2a_status c2a_model_download_obb(c2a_context *ctx, int32_t model_id, double *obb);
c2a_status c2a_model_free(c2a_context *ctx, int32_t model_id);

/* ---- queries (host buffers; synchronous) ------------------------------ */
/* Runs n queries.  contacts may be NULL; else it must hold n x
 * contacts_per_query records, of which only the first sum(min(num_contact,
 * contacts_per_query)) are written, densely: query q's contacts start at
 * results[q].contact_offset, in visiting order. */
c2a_status c2a_solve_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const c2a_params *params,
                           c2a_result *results, c2a_contact *contacts);

/* ---- queries (device buffers; asynchronous on stream) ----------------- */
/* Same as c2a_solve_batch with every buffer in device memory, except that
 * contacts stay in fixed slots: query q's at q * contacts_per_query.  stream
 * is a cudaStream_t (NULL: the legacy default stream). */
c2a_status c2a_solve_batch_device(c2a_context *ctx, const c2a_query *d_queries, int32_t n,
                                  const c2a_params *params, c2a_result *d_results, c2a_contact *d_contacts,
                                  void *stream);

/* ---- queries without any device allocation --------------------------- */
/* No counterpart in the reference.  For callers that may not allocate device
 * memory at query time: code running under another allocator's fixed device
 * budget (an engine or simulator that hands out its own buffers and forbids
 * cudaMalloc after start-up), and real-time loops where cudaMalloc/cudaFree
 * would stall on their implicit device synchronisation.  It gives the
 * results of c2a_solve_batch_device (contacts in fixed slots) with the
 * thread-per-query REFERENCE kernel, whatever params->engine says; its
 * scratch -- the work counter and the table of model pointers -- lives in
 * one file-scope device array of 8 KiB (room for C2A_NOALLOC_MAX_MODELS
 * models) that every GPU loading the library holds until the process exits.
 * No cudaMalloc, cudaFree or allocating library call is made.  The set-up
 * (the array's device address and the kernel's module) is done by
 * c2a_create, which allocates anyway.  The models must have been built with
 * c2a_model_build beforehand (that call allocates); the first call after the
 * context's model set changed copies the model table into the array and
 * waits for that copy, later calls only clear the counter and launch.  Calls
 * share the array and it keeps the last call's contents: two calls whose
 * kernels overlap on the GPU (different streams, or contexts on the same
 * device) race; serialise them.  More than C2A_NOALLOC_MAX_MODELS models in
 * the context is rejected with C2A_ERR_NOALLOC_CAPACITY, CANONICAL mode with
 * C2A_ERR_INVALID_ARGUMENT. */
#define C2A_NOALLOC_MAX_MODELS 120
c2a_status c2a_solve_batch_noalloc(c2a_context *ctx, const c2a_query *d_queries, int32_t n,
                                   const c2a_params *params, c2a_result *d_results, c2a_contact *d_contacts,
                                   void *stream);

/* One CA step per query (C2A_TimeOfContactStep) of the query's linear
 * motions at time lambda[q]: lambda 0 uses the begin poses as given (the
 * reference's first step), otherwise both motions are integrated to lambda.
 * num_ca is the reference's res->numCA and prev_mint its res->mint before the
 * step (the controlled error schedule reads both); the upper bound on the
 * step is 1 - lambda.  Writes distance, mint, translation and the counters. */
c2a_status c2a_toc_step_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *lambda,
                              const int32_t *num_ca, const double *prev_mint, const c2a_params *params,
                              c2a_result *results);

/* Contact enumeration alone at fixed poses (C2A_QueryContactOnly):
 * pose[0:12] = A, pose[24:36] = B; every triangle pair closer than
 * threshold[q]. */
c2a_status c2a_contact_only_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *threshold,
                                  int32_t contacts_per_query, c2a_result *results, c2a_contact *contacts);

/* ---- ordered, hinted and distance batches ---------------------------- */
/* c2a_solve_batch_device in C2A_MODE_REFERENCE (engine AUTO or WARP) taking
 * the queries in the caller's order: d_order (device int32) must hold a
 * permutation of [0, n).  Entries outside [0, n) are skipped; a duplicated
 * index makes two warps write the same result and contact slots and leaves
 * the left-out queries unwritten, so anything but a permutation gives
 * undefined results.  The order only
 * decides which warp takes which query when (a schedule that starts the
 * costliest queries first shortens the batch); every result equals the
 * unordered call's.  The learned cost model of c2a_gb300/learned.py
 * produces such orders. */
c2a_status c2a_solve_batch_ordered(c2a_context *ctx, const c2a_query *d_queries, int32_t n,
                                   const c2a_params *params, const int32_t *d_order, c2a_result *d_results,
                                   c2a_contact *d_contacts, void *stream);

/* c2a_solve_batch (host buffers in and out, dense contacts) taking the
 * queries in the order of d_order, a permutation of [0, n) in device memory
 * (it usually comes from a device-side cost model); REFERENCE mode, engine
 * AUTO or WARP.  Results equal c2a_solve_batch's. */
c2a_status c2a_solve_batch_ordered_host(c2a_context *ctx, const c2a_query *queries, int32_t n,
                                        const c2a_params *params, const int32_t *d_order, c2a_result *results,
                                        c2a_contact *contacts);

/* c2a_solve_batch_device in C2A_MODE_CANONICAL with hints: d_hints holds, per
 * query, hints_per_query (<= 16) pairs of hinted BVH nodes (model a's, then
 * model b's), each encoded as its path from the root in the low 16 bits (bit
 * k: the child taken at depth k, 0 first_child, 1 first_child + 1) and its
 * depth in the high 16 bits.  At the first CA step, a descent towards each
 * hinted pair gives an exact triangle-pair distance that may tighten the
 * closest-pair search's first bound.  Results are those of the unhinted
 * call, bit for bit (the search is exact); only its pruning changes.  The
 * learned seeding (c2a_gb300/learned.py) produces these hints. */
c2a_status c2a_solve_batch_hinted(c2a_context *ctx, const c2a_query *d_queries, int32_t n, const c2a_params *params,
                                  const uint32_t *d_hints, int32_t hints_per_query, c2a_result *d_results,
                                  c2a_contact *d_contacts, void *stream);

/* C2A_Distance(res, R1, T1, o1, R2, T2, o2, 0, 0, qsize) (C2A/src/C2A_PQP.cpp:970-1056)
 * for n pairs at once (host buffers; the call synchronises): query i places
 * model_a by pose[0..11] and model_b by pose[24..35] (the end poses are not
 * read); seed_a/seed_b give the first upper bound, as o1->last_tri and
 * o2->last_tri do.  One warp per pair walks a front of node pairs culled by
 * certified FP32 RSS bounds against the running minimum. */
c2a_status c2a_distance_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, c2a_distance_result *results);

/* C2A_Tolerance(res, R1, T1, o1, R2, T2, o2, tolerance, 2)
 * (C2A/src/C2A_PQP.cpp:1762-1845, C2AToleranceRecurse 1498-1603) for n
 * pairs at once (host buffers; the call synchronises): query i places
 * model_a by pose[0..11] and model_b by pose[24..35]; the search stops at the
 * first triangle pair within tolerance[i] in the reference's depth-first
 * order (closer child first).  One thread per pair, FP64. */
c2a_status c2a_tolerance_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *tolerance,
                               c2a_tolerance_result *results);

/* C2A_Collide(res, R1, T1, o1, R2, T2, o2, flag) (C2A/src/C2A_PQP.cpp:910-968,
 * CollideRecurse 798-909) for n pairs at once (host buffers; synchronous):
 * every triangle pair whose OBBs overlap all the way down and whose distance
 * is zero, in visiting order, as caller triangle ids (pairs: n x
 * pairs_per_query x 2 int32, may be NULL); flag 1 all contacts, 2 the first
 * only (C2A_FIRST_CONTACT). */
c2a_status c2a_collide_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, int32_t flag,
                             int32_t pairs_per_query, c2a_collide_result *results, int32_t *pairs);

/* ---- motion (host) --------------------------------------------------- */
/* CInterpMotion_Linear constants of one object: out[0:3] axis, out[3]
 * angular speed, out[4:7] linear velocity, out[7:11] begin quaternion
 * (x, y, z, w). */
c2a_status c2a_motion_setup(const double *R0, const double *T0, const double *R1, const double *T1, double *out);
/* Pose at time t (clamped to <= 1): R (9), T (3), qua (7: w, x, y, z, T). */
c2a_status c2a_motion_integrate(const double *R0, const double *T0, const double *R1, const double *T1,
                                double t, double *R, double *T, double *qua);

#ifdef __cplusplus
}
#endif
#endif
