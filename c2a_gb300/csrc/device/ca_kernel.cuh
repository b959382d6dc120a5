/*
 * ca_kernel.cuh -- the CA query on the GPU, in the reference's traversal order.
 *
 * One thread owns one query: the CA loop (C2A_QueryTimeOfContact,
 * C2A/src/C2A.cpp:1987-2146), each iteration's BVTT step
 * (C2A_TimeOfContactStep + TOCStepRecurse_Dis, C2A.cpp:1114-1354, 1778-1931),
 * the translation-only variant (C2A.cpp:1362-1521; InterpMotion.cpp:570-743)
 * and the contact enumeration at the TOC (C2A.cpp:1525-1775).  The recursion
 * is an explicit stack of pending second children, so node pairs are visited
 * -- and the running distance bound shrinks -- exactly as in the reference.
 *
 * GB300 executes FP64 on a narrow pipe (about 1/64 of FP32); a warp-wide FP64
 * instruction costs the same with one active lane as with 32, so per-thread
 * traversals that diverge serialise on it.  The traversal therefore keeps FP64
 * to one straight-line piece per visited node pair -- the exact transform of
 * that pair, computed at one program point so the lanes there issue it
 * together -- and runs the branchy geometry (RectDist, motion bounds, TriDist)
 * on the FP32 filter of geom.cuh, whose certified bounds decide every
 * comparison the reference makes.  Whatever a bound cannot decide (an order
 * of two distances, a descend decision, a candidate for the step's minimum
 * time, a leaf that may lower the running distance) is recomputed in FP64
 * with the reference's arithmetic, so every result stays bit-identical.
 */
#ifndef C2A_CA_KERNEL_CUH
#define C2A_CA_KERNEL_CUH

#include "../../../include/c2a_gb300.h"
#include "../host/bvh_build.h"
#include "geom.cuh"

namespace c2a {

/* the traversal is device code only (the geometry it calls is host+device) */
#define C2A_KDEV __device__ __forceinline__
#define C2A_KNOINL static __device__ __noinline__

/* traversal stack depth; models are checked at upload: 2 * depth + 2 <= this */
#ifndef C2A_STACK_DEPTH
#define C2A_STACK_DEPTH 96
#endif

/* event counters of a profiling build (-DC2A_STATS); compiled out otherwise */
#ifdef C2A_STATS
enum {
    ST_EXPAND, ST_BVE, ST_BVE_FAIL, ST_BVE_ZERO, ST_EX_DESCEND, ST_EX_CONTRIB, ST_EX_ORDER, ST_LEAF,
    ST_LEAF_SKIP, ST_LEAF_EXACT, ST_LEAF_IMPROVE, ST_NO_SHADOW, ST_EXACT, ST_STEP, ST_CLEAF, ST_CLEAF_EXACT,
    ST_D_ROUNDS, ST_D_POPS, ST_D_LEAF_EXACT, ST_D_KCYC, ST_T_ROUNDS, ST_T_POPS, ST_T_KCYC, ST_C_KCYC, ST_Q_KCYC,
    /* the warp kernel: events and clock64 cycles per phase (64-bit, per query in wst) */
    ST_W_EXPAND, ST_W_EFAIL, ST_W_MKEXACT, ST_W_LEAF, ST_W_LEAF_X, ST_W_CYC_XFORM, ST_W_CYC_TEST_E,
    ST_W_CYC_TEST_X, ST_W_CYC_STORE, ST_W_CYC_DECIDE, ST_W_CYC_LEAF, ST_W_CYC_DFS, ST_W_CYC_QUERY,
    ST_W_CYC_X_RECT, ST_W_CYC_X_BOUND, ST_W_CYC_E_RECT, ST_W_CYC_E_BOUND,
    /* the speculative engine: rounds, candidates, leaf candidates, lanes falling back to FP64,
     * replay-side exact recomputes, exact distances, exact leaves, deferred-mint evaluations,
     * pairs the replay decided; clock64 cycles per phase */
    ST_S_ROUNDS, ST_S_CANDS, ST_S_LEAFC, ST_S_LANEX, ST_S_MKEXACT, ST_S_DISTX, ST_S_LEAFX, ST_S_FLUSHX,
    ST_S_DECIDED, ST_S_CYC_REPLAY, ST_S_CYC_COLLECT, ST_S_CYC_EXPAND, ST_S_CYC_END,
    /* speculation queue pops: stale, already decided or tested, pruned; rounds that stopped on an
     * empty queue, on the pool */
    ST_S_Q_STALE, ST_S_Q_SEEN, ST_S_Q_PRUNED, ST_S_STOP_EMPTY, ST_S_STOP_POOL,
    /* per rotation step: the queue's and the pool's peak use, summed over steps, and the steps */
    ST_S_QPEAK, ST_S_RECPEAK, ST_S_STEPS,
    /* inside the test phase: the lane tests, the leaf tasks */
    ST_S_CYC_TEST, ST_S_CYC_LEAF,
    ST_COUNT
};
constexpr int ST_W_FIRST = ST_W_EXPAND;
static __device__ unsigned long long g_c2a_stats[ST_COUNT];
#define C2A_STAT(q, i) ((q).st[i]++)
#define C2A_WSTAT(q, i, x) ((q).wst[(i) - ST_W_FIRST] += (unsigned long long)(x))
#define C2A_WCLOCK(v) const long long v = clock64()
#else
#define C2A_STAT(q, i) ((void)0)
#define C2A_WSTAT(q, i, x) ((void)0)
#define C2A_WCLOCK(v) ((void)0)
#endif

struct DevModel {
    const NodeRec *nodes;
    const TriRec *tris;
    const NodeShadow *snodes;
    const TriShadow *stris;
    const ObbRec *obbs; /* OBB per node (the static collide query) */
    int32_t num_tris;
    int32_t num_nodes;
    int32_t depth;
    int32_t flags; /* bit 0: live; bit 1: FP32 shadows usable */
};
enum { C2A_MODEL_LIVE = 1, C2A_MODEL_SHADOW_OK = 2 };

/* ------------------------------------------------------------ loads */

C2A_KDEV M3 load_R(const NodeRec *n)
{
    const double2 *p = reinterpret_cast<const double2 *>(n);
    M3 r;
    double2 v[6];
#pragma unroll
    for (int i = 0; i < 6; i++) v[i] = __ldg(p + i); /* R (9) + Tr (3) */
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = reinterpret_cast<const double *>(v)[i];
    return r;
}
C2A_KDEV V3 load_Tr(const NodeRec *n) { return v3(__ldg(&n->Tr[0]), __ldg(&n->Tr[1]), __ldg(&n->Tr[2])); }

/* the FP64 fields of a node taking part in a BV test */
struct NodeX {
    M3 R, Rloc;
    V3 Tr;
    double l[2], r, angR;
};
C2A_KDEV void load_x(NodeX &c, const NodeRec *n)
{
    const double2 *p = reinterpret_cast<const double2 *>(n);
    double2 v[13];
#pragma unroll
    for (int i = 0; i < 13; i++) v[i] = __ldg(p + i);
    const double *f = reinterpret_cast<const double *>(v);
#pragma unroll
    for (int i = 0; i < 9; i++) c.R.m[i] = f[i];
    c.Tr = v3(f[9], f[10], f[11]);
    c.l[0] = f[12];
    c.l[1] = f[13];
    c.r = f[14];
    c.angR = f[15];
#pragma unroll
    for (int i = 0; i < 9; i++) c.Rloc.m[i] = f[16 + i];
}

/* the FP32 shadow of the same node (shadow_ok: every field inside FP32's normal range) */
struct NodeE {
    M3T<EF> R, Rloc;
    V3T<EF> Tr;
    EF l[2], r, angR;
};
C2A_KDEV void load_e(NodeE &c, const NodeShadow *n)
{
    const float4 *p = reinterpret_cast<const float4 *>(n);
    float4 v[7];
#pragma unroll
    for (int i = 0; i < 7; i++) v[i] = __ldg(p + i);
    const float *f = reinterpret_cast<const float *>(v);
#pragma unroll
    for (int i = 0; i < 9; i++) c.R.m[i] = ef_shadow(f[i]);
    c.Tr = v3t(ef_shadow(f[9]), ef_shadow(f[10]), ef_shadow(f[11]));
    c.l[0] = ef_shadow(f[12]);
    c.l[1] = ef_shadow(f[13]);
    c.r = ef_shadow(f[14]);
    c.angR = ef_shadow(f[15]);
#pragma unroll
    for (int i = 0; i < 9; i++) c.Rloc.m[i] = ef_shadow(f[16 + i]);
}

C2A_KDEV void load_tri(V3 t[3], const TriRec *tr)
{
    const double2 *p = reinterpret_cast<const double2 *>(tr);
    double2 v[5];
#pragma unroll
    for (int i = 0; i < 5; i++) v[i] = __ldg(p + i);
    const double *f = reinterpret_cast<const double *>(v);
    t[0] = v3(f[0], f[1], f[2]);
    t[1] = v3(f[3], f[4], f[5]);
    t[2] = v3(f[6], f[7], f[8]);
}
C2A_KDEV void load_tri_e(V3T<EF> t[3], const TriShadow *tr)
{
    const float4 *p = reinterpret_cast<const float4 *>(tr);
    float4 v[3];
#pragma unroll
    for (int i = 0; i < 3; i++) v[i] = __ldg(p + i);
    const float *f = reinterpret_cast<const float *>(v);
    t[0] = v3t(ef_shadow(f[0]), ef_shadow(f[1]), ef_shadow(f[2]));
    t[1] = v3t(ef_shadow(f[3]), ef_shadow(f[4]), ef_shadow(f[5]));
    t[2] = v3t(ef_shadow(f[6]), ef_shadow(f[7]), ef_shadow(f[8]));
}

C2A_KDEV M3T<EF> ef_m3(const M3 &R, EFCtx &c)
{
    M3T<EF> r;
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = in_d(R.m[i], c);
    return r;
}
C2A_KDEV V3T<EF> ef_v3(V3 v, EFCtx &c) { return v3t(in_d(v.x, c), in_d(v.y, c), in_d(v.z, c)); }

/* ------------------------------------------------------------ query state */

/* the reference's C2A_TimeOfContactResult of one query plus its two motions */
struct Query {
    const DevModel *A, *B;
    Motion m1, m2;
    MotionT<double> x1, x2; /* velocity constants, FP64 */
    MotionT<EF> e1, e2;     /* and their FP32 shadows */
    bool e_ok;              /* the shadows are usable */
    M3 r1;                  /* objmotion1->transform rotation */
    V3 t1;
    M3T<EF> r1e;
    M3 Rm;                  /* res->R: model 2 in model 1 */
    V3 Tm;                  /* res->T */
    M3T<EF> Rme;
    V3T<EF> Tme;
    double distance, mint, rel_err, abs_err, upbound;
    EF distance_e, bound_e, upbound_e, mint_e; /* shadows of distance, distance - abs_err, upbound, mint */
    EF rel1_e;                                 /* 1 + rel_err (1, 4 or 1.5: exact in FP32) */
    bool shadows_ok;
    bool want_mint;                            /* BV tests also bound the motion (not for contacts) */
    double *rt;                                /* the warp kernel's RectDist slots for this half-warp */
#ifdef C2A_STATS
    mutable unsigned int st[ST_COUNT];
    mutable unsigned long long wst[ST_COUNT - ST_W_FIRST];
#endif
    long long nbv, ntri;
    int numCA;
    int seed_a, seed_b;
    int status;
    double toc_delta;
};

C2A_KDEV void refresh_shadows(Query &q)
{
    EFCtx c{false};
    q.distance_e = in_d(q.distance, c);
    q.bound_e = in_d(q.distance - q.abs_err, c);
    q.upbound_e = in_d(q.upbound, c);
    q.mint_e = in_d(q.mint, c);
    q.rel1_e = in_d(1 + q.rel_err, c);
    q.shadows_ok = !c.bad && q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
}
C2A_KDEV void refresh_mint_shadow(Query &q)
{
    EFCtx c{false};
    q.mint_e = in_d(q.mint, c);
    q.shadows_ok = q.shadows_ok && !c.bad;
}

C2A_KDEV void set_motions(Query &q, const double *P)
{
    motion_setup(q.m1, P, P + 9, P + 12, P + 21);
    motion_setup(q.m2, P + 24, P + 33, P + 36, P + 45);
    ExactCtx xc{false};
    q.x1 = motion_t<double>(q.m1, xc);
    q.x2 = motion_t<double>(q.m2, xc);
    EFCtx c{false};
    q.e1 = motion_t<EF>(q.m1, c);
    q.e2 = motion_t<EF>(q.m2, c);
    q.e_ok = !c.bad;
}

/* objmotion1's current transform, with its FP32 shadow */
C2A_KDEV void set_pose1(Query &q, const M3 &R1, V3 T1)
{
    q.r1 = R1;
    q.t1 = T1;
    EFCtx c{false};
    q.r1e = ef_m3(R1, c);
    if (c.bad) q.e_ok = false;
}

/* model-level and root-level relative transforms (C2A.cpp:1793-1806) */
C2A_KDEV void relative_transforms(Query &q, const M3 &R1, V3 T1, const M3 &R2, V3 T2, M3 &Rr, V3 &Tr)
{
    q.Rm = tmmul(R1, R2);
    q.Tm = tmul(R1, T2 - T1);
    const NodeRec *a0 = q.A->nodes, *b0 = q.B->nodes;
    const M3 Ra = load_R(a0), Rb = load_R(b0);
    const M3 Rtemp = mmul(q.Rm, Rb);
    Rr = tmmul(Ra, Rtemp);
    V3 tt = mul_add(q.Rm, load_Tr(b0), q.Tm);
    tt = tt - load_Tr(a0);
    Tr = tmul(Ra, tt);
    EFCtx c{false};
    q.Rme = ef_m3(q.Rm, c);
    q.Tme = ef_v3(q.Tm, c);
    if (c.bad) q.e_ok = false;
}

/* ------------------------------------------------------------ exact pieces */

C2A_KDEV double tri_distance_x(const Query &q, int ia, int ib, V3 &p, V3 &qq, TriFeat &f, bool &col)
{
    V3 S[3], T[3], t[3];
    load_tri(S, q.A->tris + ia);
    load_tri(t, q.B->tris + ib);
    T[0] = mul_add(q.Rm, t[0], q.Tm);
    T[1] = mul_add(q.Rm, t[1], q.Tm);
    T[2] = mul_add(q.Rm, t[2], q.Tm);
    ExactCtx xc{false};
    return tri_dist(p, qq, S, T, f, col, xc);
}

/* exact transform of a child pair from its parent's (side 0: A's child, 1: B's child) */
C2A_KDEV void child_transform(const Query &q, int side, int b1, int b2, const M3 &PR, V3 PT, M3 &R, V3 &T)
{
    if (side == 0) {
        const NodeRec *n = q.A->nodes + b1;
        const M3 Rc = load_R(n);
        R = tmmul(Rc, PR);
        T = tmul(Rc, PT - load_Tr(n));
    } else {
        const NodeRec *n = q.B->nodes + b2;
        const M3 Rc = load_R(n);
        R = mmul(PR, Rc);
        T = mul_add(PR, load_Tr(n), PT);
    }
}

/* C2A_BV_Distance + both motion bounds of one child pair, exactly (C2A.cpp:1237-1274) */
C2A_KNOINL void bv_test_x(const Query &q, const M3 &R, V3 T, int x1, int x2, double &d, double &mint)
{
    ExactCtx xc{false};
    NodeX n1, n2;
    load_x(n1, q.A->nodes + x1);
    load_x(n2, q.B->nodes + x2);
    V3 S = v3(0, 0, 0);
    double z = rect_dist(R, T, n1.l, n2.l, S, xc);
    z -= (n1.r + n2.r);
    d = max0_c(z);
    if (d != 0.0 && q.want_mint) {
        V3 S1 = mul(q.r1, mul(n1.Rloc, S));
        V3 S2 = mul_s(S1, -1.0);
        const double mb1 = bound_rss(q.x1, n1.angR, S1, xc);
        const double mb2 = bound_rss(q.x2, n2.angR, S2, xc);
        mint = max0_c((d) / (mb1 + mb2));
    } else {
        mint = 0.0;
    }
}

/* the same with the FP32 filter from an FP64 parent transform; returns false
 * when the bounds cannot reproduce the FP64 branches */
C2A_KNOINL bool bv_test_e(const Query &q, int side, const M3T<EF> &PRe, V3T<EF> PTe, int x1, int x2, EF &d, EF &mint,
                       bool &d_zero)
{
    C2A_STAT(q, ST_BVE);
    if (!q.shadows_ok) {
        C2A_STAT(q, ST_NO_SHADOW);
        return false;
    }
    EFCtx c{false};
    NodeE n1, n2;
    load_e(n1, q.A->snodes + x1);
    load_e(n2, q.B->snodes + x2);
    M3T<EF> R;
    V3T<EF> T;
    if (side == 0) {
        R = tmmul(n1.R, PRe);
        T = tmul(n1.R, PTe - n1.Tr);
    } else {
        R = mmul(PRe, n2.R);
        T = mul_add(PRe, n2.Tr, PTe);
    }
    V3T<EF> S = v3t(ef_exact(0), ef_exact(0), ef_exact(0));
    const EF z = rect_dist(R, T, n1.l, n2.l, S, c) - (n1.r + n2.r);
    if (c.bad) return false;
    /* d = max(z, 0); the reference then branches on d != 0 */
    const int pos = ef_lt3(ef_exact(0), z);
    if (pos < 0) return false;
    if (pos == 0) {
        d_zero = true;
        d = ef_exact(0);
        mint = ef_exact(0);
        return true;
    }
    d_zero = false;
    d = z;
    if (!q.want_mint) {
        mint = ef_exact(0);
        return true;
    }
    V3T<EF> S1 = mul(q.r1e, mul(n1.Rloc, S));
    V3T<EF> S2 = mul_s(S1, ef_exact(-1));
    const EF mb1 = bound_rss(q.e1, n1.angR, S1, c);
    const EF mb2 = bound_rss(q.e2, n2.angR, S2, c);
    mint = max0_c(ef_div(d, mb1 + mb2, c));
    return !c.bad;
}

/* ------------------------------------------------------------ decisions */

/* a child pair waiting for its descend decision, or the pair being processed */
struct Pending {
    int32_t b1, b2;
    int32_t side;      /* 0: child of A's node, 1: child of B's node, -1: the root (PR/PT is its own) */
    int32_t exact;     /* d_x and m_x are valid */
    EF d, m;           /* FP32 shadows of d and mint (valid unless exact) */
    double d_x, m_x;
    M3 PR;             /* the parent's exact transform */
    V3 PT;
};

/* makes d and mint of a pending pair exact (their FP32 views follow) */
C2A_KNOINL void make_exact(const Query &q, Pending &p)
{
    if (p.exact) return;
    C2A_STAT(q, ST_EXACT);
    M3 R;
    V3 T;
    child_transform(q, p.side, p.b1, p.b2, p.PR, p.PT, R, T);
    bv_test_x(q, R, T, p.b1, p.b2, p.d_x, p.m_x);
    EFCtx c{false};
    p.d = in_d(p.d_x, c);
    p.m = in_d(p.m_x, c);
    if (c.bad) p.d = p.m = EF{0.0f, __int_as_float(0x7f800000)}; /* undecidable in FP32 */
    p.exact = 1;
}

/* Kleene AND / OR over {0, 1, -1 (undecided)} */
C2A_KDEV int and3(int a, int b) { return (a == 0 || b == 0) ? 0 : (a == 1 && b == 1) ? 1 : -1; }
C2A_KDEV int or3(int a, int b) { return (a == 1 || b == 1) ? 1 : (a == 0 && b == 0) ? 0 : -1; }

/* mint < UpboundTOC && (d < distance - abs_err || d * (1 + rel_err) < distance) (C2A.cpp:1281-1351) */
C2A_KDEV bool descend(const Query &q, Pending &p)
{
    if (!p.exact) {
        const int a = ef_lt3(p.m, q.upbound_e);
        const int b = ef_lt3(p.d, q.bound_e);
        const int c = ef_lt3(p.d * q.rel1_e, q.distance_e);
        const int r = and3(a, or3(b, c));
        if (r >= 0) return r == 1;
        C2A_STAT(q, ST_EX_DESCEND);
        make_exact(q, p);
    }
    return p.m_x < q.upbound && ((p.d_x < (q.distance - q.abs_err)) || (p.d_x * (1 + q.rel_err) < q.distance));
}

/* a pruned pair's mint lowers res->mint (C2A.cpp:1290-1311) */
C2A_KDEV void contribute(Query &q, Pending &p)
{
    if (!p.exact) {
        if (ef_lt3(p.m, q.mint_e) == 0) return; /* certainly >= the current minimum */
        C2A_STAT(q, ST_EX_CONTRIB);
        make_exact(q, p);
    }
    if (p.m_x < q.mint) {
        q.mint = p.m_x;
        refresh_mint_shadow(q);
    }
}

/* d2 < d1 (C2A.cpp:1281); the FP32 views of exact values decide too */
C2A_KDEV bool closer_second(const Query &q, Pending &a, Pending &c)
{
    const int r = ef_lt3(c.d, a.d);
    if (r >= 0) return r == 1;
    C2A_STAT(q, ST_EX_ORDER);
    make_exact(q, a);
    make_exact(q, c);
    return c.d_x < a.d_x;
}

/* a leaf pair of the rotation step (C2A.cpp:1141-1183) */
C2A_KNOINL void leaf_step(Query &q, int b1, int b2)
{
    const int ia = -q.A->nodes[b1].first_child - 1, ib = -q.B->nodes[b2].first_child - 1;
    q.ntri++;
    C2A_STAT(q, ST_LEAF);
    if (q.shadows_ok) {
        /* FP32 filter: most leaves cannot reach the running distance */
        EFCtx c{false};
        V3T<EF> S[3], T[3], t[3];
        load_tri_e(S, q.A->stris + ia);
        load_tri_e(t, q.B->stris + ib);
        T[0] = mul_add(q.Rme, t[0], q.Tme);
        T[1] = mul_add(q.Rme, t[1], q.Tme);
        T[2] = mul_add(q.Rme, t[2], q.Tme);
        V3T<EF> p, qq;
        TriFeat f;
        bool col = false;
        const EF dTri = tri_dist(p, qq, S, T, f, col, c);
        if (!c.bad && ef_le3(dTri, q.distance_e) == 0) {
            C2A_STAT(q, ST_LEAF_SKIP);
            return;
        }
    }
    C2A_STAT(q, ST_LEAF_EXACT);
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double dTri = tri_distance_x(q, ia, ib, p, qq, f, col);
    if (dTri <= q.distance) {
        C2A_STAT(q, ST_LEAF_IMPROVE);
        ExactCtx xc{false};
        q.distance = dTri;
        const V3 res1 = mul(q.r1, p) + q.t1;
        const V3 res2 = mul(q.r1, qq) + q.t1;
        V3 S1 = res2 - res1;
        V3 S2 = mul_s(S1, -1.0);
        const double mb1 = bound_leaf(q.x1, __ldg(&q.A->nodes[b1].angR), S1, xc);
        const double mb2 = bound_leaf(q.x2, __ldg(&q.B->nodes[b2].angR), S2, xc);
        double mint = (dTri) / (mb1 + mb2);
        if (mint < 0.0) mint = 0.0;
        if (mint <= q.mint) q.mint = mint;
        refresh_shadows(q);
    }
}

/* both children of an internal pair, tested; first = the closer one */
C2A_KNOINL void expand(Query &q, const Pending &cur, const M3 &R, V3 T, Pending &first, Pending &second)
{
    const NodeRec *n1 = q.A->nodes + cur.b1, *n2 = q.B->nodes + cur.b2;
    const int fc1 = n1->first_child, fc2 = n2->first_child;
    const bool l1 = fc1 < 0, l2 = fc2 < 0;
    Pending a, c;
    if (l2 || (!l1 && (n1->size > n2->size))) {
        a.b1 = fc1; c.b1 = fc1 + 1;
        a.b2 = c.b2 = cur.b2;
        a.side = c.side = 0;
    } else {
        a.b1 = c.b1 = cur.b1;
        a.b2 = fc2; c.b2 = fc2 + 1;
        a.side = c.side = 1;
    }
    a.PR = c.PR = R;
    a.PT = c.PT = T;
    a.exact = c.exact = 0;
    EFCtx ec{false};
    const M3T<EF> Re = ef_m3(R, ec);
    const V3T<EF> Te = ef_v3(T, ec);
    bool zero_a = false, zero_c = false;
    const bool ok_a = !ec.bad && bv_test_e(q, a.side, Re, Te, a.b1, a.b2, a.d, a.m, zero_a);
    const bool ok_c = !ec.bad && bv_test_e(q, c.side, Re, Te, c.b1, c.b2, c.d, c.m, zero_c);
    C2A_STAT(q, ST_EXPAND);
#ifdef C2A_STATS
    if (!ok_a) C2A_STAT(q, ST_BVE_FAIL);
    if (!ok_c) C2A_STAT(q, ST_BVE_FAIL);
    if (ok_a && zero_a) C2A_STAT(q, ST_BVE_ZERO);
    if (ok_c && zero_c) C2A_STAT(q, ST_BVE_ZERO);
#endif
    if (!ok_a) make_exact(q, a);
    else if (zero_a) { a.exact = 1; a.d_x = 0.0; a.m_x = 0.0; } /* d = max(z, 0) = 0, mint = 0 */
    if (!ok_c) make_exact(q, c);
    else if (zero_c) { c.exact = 1; c.d_x = 0.0; c.m_x = 0.0; }
    q.nbv += 2;
    if (closer_second(q, a, c)) { first = c; second = a; }
    else { first = a; second = c; }
}

/* TOCStepRecurse_Dis from the root pair, iteratively */
C2A_KNOINL void toc_dfs(Query &q, const M3 &Rroot, V3 Troot, Pending *stack)
{
    int sp = 0;
    Pending cur;
    cur.b1 = 0; cur.b2 = 0; cur.side = -1; cur.exact = 1;
    cur.PR = Rroot; cur.PT = Troot;
    for (;;) {
        const bool l1 = q.A->nodes[cur.b1].first_child < 0, l2 = q.B->nodes[cur.b2].first_child < 0;
        bool go = false;
        if (l1 && l2) {
            leaf_step(q, cur.b1, cur.b2);
        } else {
            M3 R;
            V3 T;
            if (cur.side < 0) { R = cur.PR; T = cur.PT; }
            else child_transform(q, cur.side, cur.b1, cur.b2, cur.PR, cur.PT, R, T);
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            Pending first;
            expand(q, cur, R, T, first, stack[sp]);
            sp++;
            if (descend(q, first)) {
                cur = first;
                go = true;
            } else {
                contribute(q, first);
            }
        }
        while (!go && sp > 0) {
            Pending &e = stack[--sp];
            if (descend(q, e)) {
                cur = e;
                go = true;
            } else {
                contribute(q, e);
            }
        }
        if (!go) return;
    }
}

/* ---------------------------------------------------- translation-only CA */

C2A_KDEV double conserv_d(const Query &q, double d) { return d - 0.1 * q.toc_delta; }

/* CAonNonAdjacentTriangles of motion 1 (InterpMotion.cpp:657-743) */
C2A_KNOINL bool ca_triangles(const Query &q, const V3 triA[3], const V3 triB[3], double &mint, double &distance)
{
    ExactCtx xc{false};
    const V3 Vel = tmul(q.r1, v3(q.m1.cv[0], q.m1.cv[1], q.m1.cv[2]));
    V3 p, qq;
    TriFeat f;
    bool col = false;
    double d = tri_dist(p, qq, triA, triB, f, col, xc);
    V3 n = normalized(qq - p, xc);
    double u = dot(Vel, n);
    if (u <= 0) u = 1e-30;
    if (d == 0) {
        mint = 0.0;
        distance = 0.0;
        return true;
    }
    const double dt = conserv_d(q, d) / u;
    int nIters = 1;
    if (dt >= mint) return false;
    double total_toc = dt;
    while ((d > q.toc_delta) && (total_toc <= mint) && (nIters < 50)) {
        V3 triA_t[3];
        for (int i = 0; i < 3; i++) triA_t[i] = add_mul(triA[i], Vel, total_toc);
        d = tri_dist(p, qq, triA_t, triB, f, col, xc);
        if (d == 0.0) break;
        n = normalized(qq - p, xc);
        u = dot(Vel, n);
        if (u <= 0) u = 1e-30;
        const double tofc = conserv_d(q, d) / u;
        nIters++;
        if (tofc < q.toc_delta) break;
        total_toc += tofc;
    }
    if (total_toc <= mint && total_toc >= 0.0) {
        mint = total_toc;
        const double cvl = sqrt(q.m1.cv[0] * q.m1.cv[0] + q.m1.cv[1] * q.m1.cv[1] + q.m1.cv[2] * q.m1.cv[2]);
        distance = (total_toc)*cvl + q.toc_delta;
        return true;
    }
    return false;
}

/* CAonRSS of motion 1 (InterpMotion.cpp:570-655).  The reference reads an
 * uninitialised S when the first rectangle distance leaves it unset
 * (C2A_RectDist.h:865-933); it starts at zero here. */
C2A_KNOINL bool ca_rss(const Query &q, const M3 &R, V3 T, int x1, int x2, double &mint, double &distance)
{
    ExactCtx xc{false};
    NodeX b1, b2;
    load_x(b1, q.A->nodes + x1);
    load_x(b2, q.B->nodes + x2);
    V3 S = v3(0, 0, 0);
    double d = max0_c(rect_dist(R, T, b1.l, b2.l, S, xc) - (b1.r + b2.r));
    S = mul(q.r1, mul(b1.Rloc, S));
    const V3 cvc = v3(q.m1.cv[0], q.m1.cv[1], q.m1.cv[2]);
    const V3 Vel = tmul(b1.Rloc, tmul(q.r1, cvc));
    double tocf = conserv_d(q, d) / bound_leaf(q.x1, b1.angR, S, xc);
    double total_toc = tocf;
    int nIters = 1;
    while ((d >= q.toc_delta) && (total_toc <= mint) && (nIters < 50)) {
        const V3 temp2 = add_mul(T, Vel, -total_toc);
        d = max0_c(rect_dist(R, temp2, b1.l, b2.l, S, xc) - (b1.r + b2.r));
        if (d == 0) break;
        S = mul(q.r1, mul(b1.Rloc, S));
        tocf = conserv_d(q, d) / bound_leaf(q.x1, b1.angR, S, xc);
        nIters++;
        if (tocf < q.toc_delta) break;
        total_toc += tocf;
    }
    if (total_toc < 1.0) {
        mint = total_toc;
        distance = (total_toc - q.toc_delta) * length(cvc);
        if (distance < 0) distance = 0;
        return true;
    }
    return false;
}

C2A_KDEV bool descend_translation(const Query &q, double mint, double d)
{
    return mint < q.mint && ((d < (q.distance - q.abs_err)) || (d * (1 + q.rel_err) < q.distance));
}

struct StackX {
    int32_t b1, b2;
    double d, mint;
    M3 R;
    V3 T;
};

/* TOCStepRecurse_Dis_Translation, iteratively, in FP64 (reached only when
 * both angular speeds are below 1e-8) */
C2A_KNOINL void translation_dfs(Query &q, const M3 &Rroot, V3 Troot, Pending *stack_mem)
{
    StackX *stack = reinterpret_cast<StackX *>(stack_mem); /* sizeof(StackX) <= sizeof(Pending) */
    int sp = 0;
    int b1 = 0, b2 = 0;
    M3 R = Rroot;
    V3 T = Troot;
    for (;;) {
        const NodeRec *n1 = q.A->nodes + b1, *n2 = q.B->nodes + b2;
        const bool l1 = n1->first_child < 0, l2 = n2->first_child < 0;
        bool go = false;
        if (l1 && l2) {
            const int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
            V3 triA[3], triB[3], t[3];
            load_tri(triA, q.A->tris + ia);
            load_tri(t, q.B->tris + ib);
            for (int k = 0; k < 3; k++) triB[k] = mul_add(q.Rm, t[k], q.Tm);
            if (ca_triangles(q, triA, triB, q.mint, q.distance)) {
                q.seed_a = ia;
                q.seed_b = ib;
            }
            q.ntri++;
        } else {
            int a1, a2, c1, c2, side;
            if (l2 || (!l1 && (n1->size > n2->size))) {
                a1 = n1->first_child; c1 = a1 + 1; a2 = c2 = b2; side = 0;
            } else {
                a1 = c1 = b1; a2 = n2->first_child; c2 = a2 + 1; side = 1;
            }
            M3 R1, R2;
            V3 T1, T2;
            child_transform(q, side, a1, a2, R, T, R1, T1);
            child_transform(q, side, c1, c2, R, T, R2, T2);
            double d1 = 1e+30, d2 = 1e+30, minta = q.mint, mintc = q.mint;
            ca_rss(q, R1, T1, a1, a2, minta, d1);
            ca_rss(q, R2, T2, c1, c2, mintc, d2);
            q.nbv += 2;
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            StackX &e = stack[sp++];
            if (d2 < d1) {
                e.b1 = a1; e.b2 = a2; e.d = d1; e.mint = minta; e.R = R1; e.T = T1;
                if (descend_translation(q, mintc, d2)) {
                    b1 = c1; b2 = c2; R = R2; T = T2;
                    go = true;
                }
            } else {
                e.b1 = c1; e.b2 = c2; e.d = d2; e.mint = mintc; e.R = R2; e.T = T2;
                if (descend_translation(q, minta, d1)) {
                    b1 = a1; b2 = a2; R = R1; T = T1;
                    go = true;
                }
            }
        }
        while (!go && sp > 0) {
            const StackX &e = stack[--sp];
            if (descend_translation(q, e.mint, e.d)) {
                b1 = e.b1; b2 = e.b2; R = e.R; T = e.T;
                go = true;
            }
        }
        if (!go) return;
    }
}

/* ---------------------------------------------------------- the CA step */

/* C2A_TimeOfContactStep (C2A.cpp:1778-1931).  R1/T1, R2/T2 are the current
 * poses (the translation branch moves them to the step's time, as the
 * reference does with its caller's arrays). */
C2A_KNOINL void toc_step(Query &q, M3 &R1, V3 &T1, M3 &R2, V3 &T2, bool translation, Pending *stack)
{
    M3 R;
    V3 T;
    C2A_STAT(q, ST_STEP);
    relative_transforms(q, R1, T1, R2, T2, R, T);
    if (translation) {
        V3 triA[3], triB[3], t[3];
        load_tri(triA, q.A->tris + q.seed_a);
        load_tri(t, q.B->tris + q.seed_b);
        for (int k = 0; k < 3; k++) triB[k] = mul_add(q.Rm, t[k], q.Tm);
        double mint = 1.0, dTri = 0;
        if (ca_triangles(q, triA, triB, mint, dTri)) {
            q.mint = mint;
            q.distance = dTri;
        } else {
            q.mint = 1.0;
            q.distance = 1e+30;
        }
        q.abs_err = 0;
        q.rel_err = 0;
        translation_dfs(q, R, T, stack);
        double orn[4];
        motion_integrate(q.m1, q.mint, R1.m, &T1.x, orn);
        motion_integrate(q.m2, q.mint, R2.m, &T2.x, orn);
        set_pose1(q, R1, T1);
        q.Rm = tmmul(R1, R2);
        q.Tm = tmul(R1, T2 - T1);
        V3 p, qq;
        TriFeat f;
        bool col = false;
        q.distance = tri_distance_x(q, q.seed_a, q.seed_b, p, qq, f, col);
        return;
    }
    {
        V3 p, qq;
        TriFeat f;
        bool col = false;
        q.distance = tri_distance_x(q, q.seed_a, q.seed_b, p, qq, f, col);
    }
    if (q.numCA == 0) q.mint = 1;
    /* controlled error schedule (C2A.cpp:1869-1891) */
    if (q.mint <= 0.005 || q.distance <= 0.5 || q.numCA > 5) {
        q.abs_err = 0;
        q.rel_err = 0;
    } else {
        q.abs_err = 1e+30;
        q.rel_err = (q.numCA <= 2) ? 3 : 0.5;
    }
    q.mint = 1;
    refresh_shadows(q);
    toc_dfs(q, R, T, stack);
}

/* --------------------------------------------------- contact enumeration */

/* a leaf pair of the contact enumeration: true when its triangles lie within
 * the threshold with valid features (C2A.cpp:1560-1630); fills c */
C2A_KNOINL bool contact_leaf_test(Query &q, int b1, int b2, double threshold, EF threshold_e, int query_index,
                                  c2a_contact &c)
{
    const int ia = -q.A->nodes[b1].first_child - 1, ib = -q.B->nodes[b2].first_child - 1;
    C2A_STAT(q, ST_CLEAF);
    if (q.shadows_ok) {
        EFCtx ec{false};
        V3T<EF> S[3], T[3], t[3];
        load_tri_e(S, q.A->stris + ia);
        load_tri_e(t, q.B->stris + ib);
        T[0] = mul_add(q.Rme, t[0], q.Tme);
        T[1] = mul_add(q.Rme, t[1], q.Tme);
        T[2] = mul_add(q.Rme, t[2], q.Tme);
        V3T<EF> p, qq;
        TriFeat f{-1, -1, -1, -1};
        bool col = false;
        const EF d = tri_dist(p, qq, S, T, f, col, ec);
        if (!ec.bad && f.type_a != -1 && f.type_b != -1 && ef_le3(d, threshold_e) == 0) return false;
    }
    C2A_STAT(q, ST_CLEAF_EXACT);
    V3 p, qq;
    TriFeat f{-1, -1, -1, -1};
    bool col = false;
    const double d = tri_distance_x(q, ia, ib, p, qq, f, col);
    if (f.type_a == -1 || f.type_b == -1 || !(d <= threshold)) return false;
    const TriRec *ta = q.A->tris + ia, *tb = q.B->tris + ib;
    c.type_a = f.type_a + 1;
    c.type_b = f.type_b + 1;
    for (int k = 0; k < 3; k++) c.fid_a[k] = c.fid_b[k] = -1;
    if (f.type_a == 0) c.fid_a[0] = ta->idx[f.fid_a];
    if (f.type_a == 1) { c.fid_a[0] = ta->idx[f.fid_a]; c.fid_a[1] = ta->idx[(f.fid_a + 1) % 3]; }
    if (f.type_a == 2) { c.fid_a[0] = ta->idx[0]; c.fid_a[1] = ta->idx[1]; c.fid_a[2] = ta->idx[2]; }
    if (f.type_b == 0) c.fid_b[0] = tb->idx[f.fid_b];
    if (f.type_b == 1) { c.fid_b[0] = tb->idx[f.fid_b]; c.fid_b[1] = tb->idx[(f.fid_b + 1) % 3]; }
    if (f.type_b == 2) { c.fid_b[0] = tb->idx[0]; c.fid_b[1] = tb->idx[1]; c.fid_b[2] = tb->idx[2]; }
    c.tri_a = ia;
    c.tri_b = ib;
    c.query = query_index;
    c.pad = 0;
    c.pa[0] = p.x; c.pa[1] = p.y; c.pa[2] = p.z;
    const V3 pb = tmul(q.Rm, qq - q.Tm);
    c.pb[0] = pb.x; c.pb[1] = pb.y; c.pb[2] = pb.z;
    c.distance = d;
    return true;
}

/* contacts of one leaf pair: written in visiting order; counted even when
 * the slots run out */
C2A_KDEV void contact_leaf(Query &q, int b1, int b2, double threshold, EF threshold_e, c2a_contact *out, int slots,
                           int query_index, int &count)
{
    c2a_contact c;
    if (!contact_leaf_test(q, b1, b2, threshold, threshold_e, query_index, c)) return;
    if (count < slots && out) out[count] = c;
    count++;
}

/* d < threshold for a pending pair (abs_err = rel_err = 0: both clauses are d < threshold) */
C2A_KDEV bool contact_descend(const Query &q, Pending &p, double threshold, EF threshold_e)
{
    if (!p.exact) {
        const int r = ef_lt3(p.d, threshold_e);
        if (r >= 0) return r == 1;
        make_exact(q, p);
    }
    return (p.d_x < (threshold - 0)) || (p.d_x * (1.0 + 0) < threshold);
}

/* TOCStepRecurse_Dis_contact with a fixed threshold (C2A.cpp:1525-1725) */
C2A_KNOINL int contact_dfs(Query &q, const M3 &Rroot, V3 Troot, double threshold, Pending *stack, c2a_contact *out,
                        int slots, int query_index)
{
    EFCtx tc{false};
    const EF threshold_e = in_d(threshold, tc);
    if (tc.bad) q.shadows_ok = false;
    int count = 0;
    int sp = 0;
    Pending cur;
    cur.b1 = 0; cur.b2 = 0; cur.side = -1; cur.exact = 1;
    cur.PR = Rroot; cur.PT = Troot;
    for (;;) {
        const bool l1 = q.A->nodes[cur.b1].first_child < 0, l2 = q.B->nodes[cur.b2].first_child < 0;
        bool go = false;
        if (l1 && l2) {
            contact_leaf(q, cur.b1, cur.b2, threshold, threshold_e, out, slots, query_index, count);
        } else {
            M3 R;
            V3 T;
            if (cur.side < 0) { R = cur.PR; T = cur.PT; }
            else child_transform(q, cur.side, cur.b1, cur.b2, cur.PR, cur.PT, R, T);
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return count;
            }
            Pending first;
            expand(q, cur, R, T, first, stack[sp]);
            q.nbv -= 2; /* the contact query is not counted in the CA counters */
            sp++;
            if (contact_descend(q, first, threshold, threshold_e)) {
                cur = first;
                go = true;
            }
        }
        while (!go && sp > 0) {
            Pending &e = stack[--sp];
            if (contact_descend(q, e, threshold, threshold_e)) {
                cur = e;
                go = true;
            }
        }
        if (!go) return count;
    }
}

/* ------------------------------------------------------------ one query */

C2A_KDEV M3 pose_R(const double *p)
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = p[i];
    return r;
}
C2A_KDEV V3 pose_T(const double *p) { return v3(p[9], p[10], p[11]); }

/* C2A_Solve body: C2A_QueryTimeOfContact then C2A_QueryContact at the TOC */
C2A_KDEV void solve_query(const c2a_query &in, const DevModel *models, int num_models, const c2a_params &prm,
                         c2a_result &out, c2a_contact *contacts, Pending *stack, int query_index)
{
    Query q;
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) q.st[i] = 0;
#endif
    out.status = C2A_QUERY_OK;
    out.contact_offset = query_index * prm.contacts_per_query;
    out.num_contact = 0;
    q.status = 0;
    if (in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 || in.model_b >= num_models ||
        !(models[in.model_a].flags & C2A_MODEL_LIVE) || !(models[in.model_b].flags & C2A_MODEL_LIVE)) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    q.want_mint = true;
    if (in.seed_a < 0 || in.seed_a >= q.A->num_tris || in.seed_b < 0 || in.seed_b >= q.B->num_tris) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    const double *P = in.pose;
    set_motions(q, P);
    q.toc_delta = prm.toc_delta;
    const bool translation = (q.m1.angVel < 1e-8 && q.m2.angVel < 1e-8);
    q.seed_a = in.seed_a;
    q.seed_b = in.seed_b;
    q.nbv = q.ntri = 0;
    q.upbound = 1;
    q.numCA = 0;
    q.mint = 1;
    q.distance = 0;
    q.abs_err = q.rel_err = 0;
    M3 R1 = pose_R(P), R2 = pose_R(P + 24);
    V3 T1 = pose_T(P), T2 = pose_T(P + 24);
    set_pose1(q, R1, T1);

    double toc = 0, lamda = 0.0, lastLamda = 0, dlamda = 0.0;
    bool collisionfree = false;
    toc_step(q, R1, T1, R2, T2, translation, stack);
    double dist = q.distance, mint = q.mint;
    if (translation) {
        collisionfree = (mint >= 1.0);
        toc = mint;
    } else {
        q.numCA = 1;
        lastLamda = mint;
        int nItrs = 0;
        bool done = false;
        while (dist > prm.tol_d && q.status == 0) {
            nItrs++;
            if (nItrs > prm.max_iters) {
                out.status |= C2A_QUERY_ITER_CAP;
                break;
            }
            if (mint >= 1.0) {
                collisionfree = true;
                done = true;
                break;
            }
            dlamda = mint;
            if (dlamda < prm.tol_t) break;
            lamda += dlamda;
            if (lamda >= 1.0) {
                collisionfree = true;
                done = true;
                break;
            }
            lastLamda = lamda;
            q.numCA++;
            double orn[4];
            motion_integrate(q.m1, lamda, R1.m, &T1.x, orn);
            motion_integrate(q.m2, lamda, R2.m, &T2.x, orn);
            set_pose1(q, R1, T1);
            q.upbound = 1.0 - lamda;
            toc_step(q, R1, T1, R2, T2, false, stack);
            dist = q.distance;
            mint = q.mint;
        }
        if (done) {
            toc = 0;
        } else {
            if (dist == 0 && mint < 0) toc = lastLamda - dlamda;
            else toc = lastLamda;
            collisionfree = false;
            if (toc >= 1 - prm.tol_t) toc = 0;
        }
    }
    out.collisionfree = collisionfree ? 1 : 0;
    out.toc = toc;
    out.numCA = q.numCA;
    out.translation = translation ? 1 : 0;
    out.distance = q.distance;
    out.mint = q.mint;
    out.num_bv_tests = q.nbv;
    out.num_tri_tests = q.ntri;
    out.seed_a = q.seed_a;
    out.seed_b = q.seed_b;
    for (int i = 0; i < 9; i++) out.R_toc[0][i] = out.R_toc[1][i] = 0.0;
    for (int i = 0; i < 3; i++) out.T_toc[0][i] = out.T_toc[1][i] = 0.0;
    if (!collisionfree && q.status == 0) {
        M3 Ra, Rb;
        V3 Ta, Tb;
        double orn[4];
        motion_integrate(q.m1, toc, Ra.m, &Ta.x, orn);
        motion_integrate(q.m2, toc, Rb.m, &Tb.x, orn);
        for (int i = 0; i < 9; i++) {
            out.R_toc[0][i] = Ra.m[i];
            out.R_toc[1][i] = Rb.m[i];
        }
        out.T_toc[0][0] = Ta.x; out.T_toc[0][1] = Ta.y; out.T_toc[0][2] = Ta.z;
        out.T_toc[1][0] = Tb.x; out.T_toc[1][1] = Tb.y; out.T_toc[1][2] = Tb.z;
        if (prm.with_contacts) {
            const double threshold = 2 * q.distance + prm.contact_abs;
            M3 R;
            V3 T;
            set_pose1(q, Ra, Ta);
            relative_transforms(q, Ra, Ta, Rb, Tb, R, T);
            q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
            q.want_mint = false; /* the contact recursion reads distances only */
            const int n = contact_dfs(q, R, T, threshold, stack, contacts, prm.contacts_per_query, query_index);
            out.num_contact = n;
            if (n > prm.contacts_per_query) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
        }
    }
    out.status |= q.status;
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) atomicAdd(&g_c2a_stats[i], (unsigned long long)q.st[i]);
#endif
}

} // namespace c2a
#endif
