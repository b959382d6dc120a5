/*
 * ca_kernel.cuh -- the CA query on the GPU, reference traversal order.
 *
 * One thread owns one query for its whole life: the CA loop
 * (C2A_QueryTimeOfContact, C2A/src/C2A.cpp:1987-2146), each iteration's BVTT
 * step (C2A_TimeOfContactStep + TOCStepRecurse_Dis, C2A.cpp:1114-1354,
 * 1778-1931), the translation-only variant (C2A.cpp:1362-1521;
 * InterpMotion.cpp:570-743) and the contact enumeration at the TOC
 * (C2A.cpp:1525-1775).  The recursion becomes an explicit stack of pending
 * second children, so the nodes are visited -- and the running distance bound
 * shrinks -- in exactly the reference's order; with the FP64 geometry of
 * geom64.cuh every result is bit-identical to the reference.
 *
 * Threads take queries from a device work counter (persistent grid), so
 * uneven CA iteration counts do not idle whole blocks.
 */
#ifndef C2A_CA_KERNEL_CUH
#define C2A_CA_KERNEL_CUH

#include "../../../include/c2a_gb300.h"
#include "../host/bvh_build.h"
#include "geom64.cuh"

namespace c2a {

/* traversal stack depth; models are checked at upload: depth(A) + depth(B) + 2 <= this */
#ifndef C2A_STACK_DEPTH
#define C2A_STACK_DEPTH 96
#endif

struct DevModel {
    const NodeRec *nodes;
    const TriRec *tris;
    int32_t num_tris;
    int32_t num_nodes;
    int32_t depth;
    int32_t live;
};

struct StackEntry {
    int32_t b1, b2;
    double d, mint;
    M3 R;
    V3 T;
};

/* node fields read when the node is a child in a BV test */
struct ChildNode {
    M3 R;
    V3 Tr;
    double l[2];
    double r, angR;
    M3 Rloc;
};

C2A_DEV void load_child(ChildNode &c, const NodeRec *n)
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

C2A_DEV M3 load_m3(const double *p)
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = p[i];
    return r;
}

C2A_DEV void load_tri(V3 t[3], const TriRec *tr)
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

/* state of one query across CA steps: the reference's C2A_TimeOfContactResult
 * plus the two motions and their current transforms */
struct Query {
    const DevModel *A, *B;
    Motion m1, m2;
    M3 r1;           /* objmotion1->transform rotation */
    V3 t1;           /* objmotion1->transform translation */
    M3 Rm;           /* res->R: model 2 in model 1 */
    V3 Tm;           /* res->T */
    double distance, mint, rel_err, abs_err, upbound;
    long long nbv, ntri;
    int numCA;
    int seed_a, seed_b;
    int status;
    double toc_delta;
};

/* model-level and root-level relative transforms (C2A.cpp:1793-1806) */
C2A_DEV void relative_transforms(Query &q, const M3 &R1, V3 T1, const M3 &R2, V3 T2, M3 &Rr, V3 &Tr)
{
    q.Rm = tmmul(R1, R2);
    q.Tm = tmul(R1, T2 - T1);
    const NodeRec *a0 = q.A->nodes, *b0 = q.B->nodes;
    const M3 Ra = load_m3(a0->R), Rb = load_m3(b0->R);
    const M3 Rtemp = mmul(q.Rm, Rb);
    Rr = tmmul(Ra, Rtemp);
    V3 tt = mul_add(q.Rm, v3(b0->Tr[0], b0->Tr[1], b0->Tr[2]), q.Tm);
    tt = tt - v3(a0->Tr[0], a0->Tr[1], a0->Tr[2]);
    Tr = tmul(Ra, tt);
}

/* triangle t2 of B moved into A's frame */
C2A_DEV void tri_in_a(V3 out[3], const Query &q, int ib)
{
    V3 t[3];
    load_tri(t, q.B->tris + ib);
    out[0] = mul_add(q.Rm, t[0], q.Tm);
    out[1] = mul_add(q.Rm, t[1], q.Tm);
    out[2] = mul_add(q.Rm, t[2], q.Tm);
}

C2A_DEV double tri_distance(const Query &q, int ia, int ib, V3 &p, V3 &qq, TriFeat &f, bool &col)
{
    V3 S[3], T[3];
    load_tri(S, q.A->tris + ia);
    tri_in_a(T, q, ib);
    return tri_dist(p, qq, S, T, f, col);
}

/* which tree to descend and the two child transforms (C2A.cpp:1192-1226) */
C2A_DEV void expand(const Query &q, int b1, int b2, bool l1, bool l2, const M3 &R, V3 T, int &a1, int &a2, int &c1,
                    int &c2, ChildNode &na1, ChildNode &na2, ChildNode &nc1, ChildNode &nc2, M3 &R1, V3 &T1, M3 &R2,
                    V3 &T2)
{
    const NodeRec *n1 = q.A->nodes + b1, *n2 = q.B->nodes + b2;
    const double sz1 = n1->size, sz2 = n2->size;
    if (l2 || (!l1 && (sz1 > sz2))) {
        a1 = n1->first_child;
        c1 = a1 + 1;
        a2 = c2 = b2;
        load_child(na1, q.A->nodes + a1);
        load_child(nc1, q.A->nodes + c1);
        load_child(na2, n2);
        nc2 = na2;
        R1 = tmmul(na1.R, R);
        T1 = tmul(na1.R, T - na1.Tr);
        R2 = tmmul(nc1.R, R);
        T2 = tmul(nc1.R, T - nc1.Tr);
    } else {
        a1 = c1 = b1;
        a2 = n2->first_child;
        c2 = a2 + 1;
        load_child(na1, n1);
        nc1 = na1;
        load_child(na2, q.B->nodes + a2);
        load_child(nc2, q.B->nodes + c2);
        R1 = mmul(R, na2.R);
        T1 = mul_add(R, na2.Tr, T);
        R2 = mmul(R, nc2.R);
        T2 = mul_add(R, nc2.Tr, T);
    }
}

C2A_DEV double bv_distance(const M3 &R, V3 T, const ChildNode &x1, const ChildNode &x2, V3 &S)
{
    double d = rect_dist(R, T, x1.l, x2.l, S);
    d -= (x1.r + x2.r);
    return (d < 0.0) ? 0.0 : d;
}

/* d / (bound1 + bound2) of one child pair, 0 when the RSSs touch (C2A.cpp:1237-1274) */
C2A_DEV double child_mint(const Query &q, const M3 &R, V3 T, const ChildNode &x1, const ChildNode &x2, double &d)
{
    V3 S = v3(0, 0, 0);
    d = bv_distance(R, T, x1, x2, S);
    if (d != 0.0) {
        V3 S1 = mul(q.r1, mul(x1.Rloc, S));
        V3 S2 = mul_s(S1, -1);
        const double mb1 = bound_rss(q.m1, x1.angR, S1);
        const double mb2 = bound_rss(q.m2, x2.angR, S2);
        double mint = (d) / (mb1 + mb2);
        if (mint <= 0) mint = 0.0;
        return mint;
    }
    return 0.0;
}

C2A_DEV bool descend_ok(const Query &q, double mint, double d)
{
    return mint < q.upbound && ((d < (q.distance - q.abs_err)) || (d * (1 + q.rel_err) < q.distance));
}

/* a leaf pair of the rotation step (C2A.cpp:1141-1183) */
C2A_DEV void leaf_step(Query &q, int b1, int b2)
{
    const NodeRec *n1 = q.A->nodes + b1, *n2 = q.B->nodes + b2;
    const int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double dTri = tri_distance(q, ia, ib, p, qq, f, col);
    if (dTri <= q.distance) {
        q.distance = dTri;
        const V3 res1 = mul(q.r1, p) + q.t1;
        const V3 res2 = mul(q.r1, qq) + q.t1;
        V3 S1 = res2 - res1;
        V3 S2 = mul_s(S1, -1);
        const double mb1 = bound_leaf(q.m1, n1->angR, S1);
        const double mb2 = bound_leaf(q.m2, n2->angR, S2);
        double mint = (dTri) / (mb1 + mb2);
        if (mint < 0.0) mint = 0.0;
        if (mint <= q.mint) q.mint = mint;
    }
    q.ntri++;
}

/* TOCStepRecurse_Dis from the root pair, iteratively */
C2A_DEV void toc_dfs(Query &q, const M3 &Rroot, V3 Troot, StackEntry *stack)
{
    int sp = 0;
    int b1 = 0, b2 = 0;
    M3 R = Rroot;
    V3 T = Troot;
    for (;;) {
        const bool l1 = q.A->nodes[b1].first_child < 0, l2 = q.B->nodes[b2].first_child < 0;
        bool go = false;
        if (l1 && l2) {
            leaf_step(q, b1, b2);
        } else {
            int a1, a2, c1, c2;
            ChildNode na1, na2, nc1, nc2;
            M3 R1, R2;
            V3 T1, T2;
            expand(q, b1, b2, l1, l2, R, T, a1, a2, c1, c2, na1, na2, nc1, nc2, R1, T1, R2, T2);
            double d1, d2;
            const double mintb = child_mint(q, R1, T1, na1, na2, d1);
            const double minta = child_mint(q, R2, T2, nc1, nc2, d2);
            q.nbv += 2;
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            StackEntry &e = stack[sp++];
            if (d2 < d1) { /* closer child c first; a waits */
                e.b1 = a1; e.b2 = a2; e.d = d1; e.mint = mintb; e.R = R1; e.T = T1;
                if (descend_ok(q, minta, d2)) {
                    b1 = c1; b2 = c2; R = R2; T = T2;
                    go = true;
                } else if (minta < q.mint) q.mint = minta;
            } else {
                e.b1 = c1; e.b2 = c2; e.d = d2; e.mint = minta; e.R = R2; e.T = T2;
                if (descend_ok(q, mintb, d1)) {
                    b1 = a1; b2 = a2; R = R1; T = T1;
                    go = true;
                } else if (mintb < q.mint) q.mint = mintb;
            }
        }
        while (!go && sp > 0) {
            const StackEntry &e = stack[--sp];
            if (descend_ok(q, e.mint, e.d)) {
                b1 = e.b1; b2 = e.b2; R = e.R; T = e.T;
                go = true;
            } else if (e.mint < q.mint) q.mint = e.mint;
        }
        if (!go) return;
    }
}

/* ---------------------------------------------------- translation-only CA */

C2A_DEV double conserv_d(const Query &q, double d) { return d - 0.1 * q.toc_delta; }

/* CAonNonAdjacentTriangles of motion 1 (InterpMotion.cpp:657-743) */
C2A_DEV bool ca_triangles(const Query &q, const V3 triA[3], const V3 triB[3], double &mint, double &distance)
{
    const V3 Vel = tmul(q.r1, v3(q.m1.cv[0], q.m1.cv[1], q.m1.cv[2]));
    V3 p, qq;
    TriFeat f;
    bool col = false;
    double d = tri_dist(p, qq, triA, triB, f, col);
    V3 n = normalized(qq - p);
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
        d = tri_dist(p, qq, triA_t, triB, f, col);
        if (d == 0.0) break;
        n = normalized(qq - p);
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
C2A_DEV bool ca_rss(const Query &q, const M3 &R, V3 T, const ChildNode &b1, const ChildNode &b2, double &mint,
                    double &distance)
{
    V3 S = v3(0, 0, 0);
    double d = bv_distance(R, T, b1, b2, S);
    S = mul(q.r1, mul(b1.Rloc, S));
    const V3 cvc = v3(q.m1.cv[0], q.m1.cv[1], q.m1.cv[2]);
    const V3 Vel = tmul(b1.Rloc, tmul(q.r1, cvc));
    double tocf = conserv_d(q, d) / bound_leaf(q.m1, b1.angR, S);
    double total_toc = tocf;
    int nIters = 1;
    while ((d >= q.toc_delta) && (total_toc <= mint) && (nIters < 50)) {
        const V3 temp2 = add_mul(T, Vel, -total_toc);
        d = bv_distance(R, temp2, b1, b2, S);
        if (d == 0) break;
        S = mul(q.r1, mul(b1.Rloc, S));
        tocf = conserv_d(q, d) / bound_leaf(q.m1, b1.angR, S);
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

C2A_DEV bool descend_translation(const Query &q, double mint, double d)
{
    return mint < q.mint && ((d < (q.distance - q.abs_err)) || (d * (1 + q.rel_err) < q.distance));
}

/* TOCStepRecurse_Dis_Translation, iteratively */
C2A_DEV void translation_dfs(Query &q, const M3 &Rroot, V3 Troot, StackEntry *stack)
{
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
            V3 triA[3], triB[3];
            load_tri(triA, q.A->tris + ia);
            tri_in_a(triB, q, ib);
            if (ca_triangles(q, triA, triB, q.mint, q.distance)) {
                q.seed_a = ia;
                q.seed_b = ib;
            }
            q.ntri++;
        } else {
            int a1, a2, c1, c2;
            ChildNode na1, na2, nc1, nc2;
            M3 R1, R2;
            V3 T1, T2;
            expand(q, b1, b2, l1, l2, R, T, a1, a2, c1, c2, na1, na2, nc1, nc2, R1, T1, R2, T2);
            double d1 = 1e+30, d2 = 1e+30, minta = q.mint, mintc = q.mint;
            ca_rss(q, R1, T1, na1, na2, minta, d1);
            ca_rss(q, R2, T2, nc1, nc2, mintc, d2);
            q.nbv += 2;
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            StackEntry &e = stack[sp++];
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
            const StackEntry &e = stack[--sp];
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
 * poses of both objects (the translation branch moves them to the step's
 * time, like the reference does with its caller's arrays). */
C2A_DEV void toc_step(Query &q, M3 &R1, V3 &T1, M3 &R2, V3 &T2, bool translation, StackEntry *stack)
{
    M3 R;
    V3 T;
    relative_transforms(q, R1, T1, R2, T2, R, T);
    if (translation) {
        V3 triA[3], triB[3];
        load_tri(triA, q.A->tris + q.seed_a);
        tri_in_a(triB, q, q.seed_b);
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
        q.r1 = R1;
        q.t1 = T1;
        q.Rm = tmmul(R1, R2);
        q.Tm = tmul(R1, T2 - T1);
        V3 p, qq;
        TriFeat f;
        bool col = false;
        q.distance = tri_distance(q, q.seed_a, q.seed_b, p, qq, f, col);
        return;
    }
    {
        V3 p, qq;
        TriFeat f;
        bool col = false;
        q.distance = tri_distance(q, q.seed_a, q.seed_b, p, qq, f, col);
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
    toc_dfs(q, R, T, stack);
}

/* --------------------------------------------------- contact enumeration */

/* TOCStepRecurse_Dis_contact with a fixed threshold (C2A.cpp:1525-1725):
 * contacts are written in visiting order; the count is exact even when the
 * slots run out */
C2A_DEV int contact_dfs(Query &q, const M3 &Rroot, V3 Troot, double threshold, StackEntry *stack,
                        c2a_contact *out, int slots, int query_index)
{
    int count = 0;
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
            V3 p, qq;
            TriFeat f{-1, -1, -1, -1};
            bool col = false;
            const double d = tri_distance(q, ia, ib, p, qq, f, col);
            if (f.type_a != -1 && f.type_b != -1 && d <= threshold) {
                if (count < slots && out) {
                    const TriRec *ta = q.A->tris + ia, *tb = q.B->tris + ib;
                    c2a_contact &c = out[count];
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
                }
                count++;
            }
        } else {
            int a1, a2, c1, c2;
            ChildNode na1, na2, nc1, nc2;
            M3 R1, R2;
            V3 T1, T2;
            expand(q, b1, b2, l1, l2, R, T, a1, a2, c1, c2, na1, na2, nc1, nc2, R1, T1, R2, T2);
            V3 S = v3(0, 0, 0);
            const double d1 = bv_distance(R1, T1, na1, na2, S);
            const double d2 = bv_distance(R2, T2, nc1, nc2, S);
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return count;
            }
            StackEntry &e = stack[sp++];
            if (d2 < d1) {
                e.b1 = a1; e.b2 = a2; e.d = d1; e.R = R1; e.T = T1;
                if ((d2 < (threshold - 0)) || (d2 * (1.0 + 0) < threshold)) {
                    b1 = c1; b2 = c2; R = R2; T = T2;
                    go = true;
                }
            } else {
                e.b1 = c1; e.b2 = c2; e.d = d2; e.R = R2; e.T = T2;
                if ((d1 < (threshold - 0)) || (d1 * (1.0 + 0) < threshold)) {
                    b1 = a1; b2 = a2; R = R1; T = T1;
                    go = true;
                }
            }
        }
        while (!go && sp > 0) {
            const StackEntry &e = stack[--sp];
            if ((e.d < (threshold - 0)) || (e.d * (1.0 + 0) < threshold)) {
                b1 = e.b1; b2 = e.b2; R = e.R; T = e.T;
                go = true;
            }
        }
        if (!go) return count;
    }
}

/* ------------------------------------------------------------ one query */

C2A_DEV M3 pose_R(const double *p)
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = p[i];
    return r;
}
C2A_DEV V3 pose_T(const double *p) { return v3(p[9], p[10], p[11]); }

/* C2A_Solve body: C2A_QueryTimeOfContact then C2A_QueryContact at the TOC */
C2A_DEV void solve_query(const c2a_query &in, const DevModel *models, int num_models, const c2a_params &prm,
                         c2a_result &out, c2a_contact *contacts, StackEntry *stack, int query_index)
{
    Query q;
    out.status = C2A_QUERY_OK;
    out.contact_offset = query_index * prm.contacts_per_query;
    out.num_contact = 0;
    q.status = 0;
    if (in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 || in.model_b >= num_models ||
        !models[in.model_a].live || !models[in.model_b].live) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    if (in.seed_a < 0 || in.seed_a >= q.A->num_tris || in.seed_b < 0 || in.seed_b >= q.B->num_tris) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    const double *P = in.pose;
    motion_setup(q.m1, P, P + 9, P + 12, P + 21);
    motion_setup(q.m2, P + 24, P + 33, P + 36, P + 45);
    q.toc_delta = prm.toc_delta;
    const bool translation = (q.m1.angVel < 1e-8 && q.m2.angVel < 1e-8);
    q.seed_a = in.seed_a;
    q.seed_b = in.seed_b;
    q.nbv = q.ntri = 0;
    q.upbound = 1;
    q.numCA = 0;
    q.mint = 1;
    q.distance = 0;
    M3 R1 = pose_R(P), R2 = pose_R(P + 24);
    V3 T1 = pose_T(P), T2 = pose_T(P + 24);
    q.r1 = R1;
    q.t1 = T1;

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
            q.r1 = R1;
            q.t1 = T1;
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
    out.num_contact = 0;
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
            q.r1 = Ra;
            q.t1 = Ta;
            relative_transforms(q, Ra, Ta, Rb, Tb, R, T);
            const int n = contact_dfs(q, R, T, threshold, stack, contacts, prm.contacts_per_query, query_index);
            out.num_contact = n;
            if (n > prm.contacts_per_query) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
        }
    }
    out.status |= q.status;
}

} // namespace c2a
#endif
