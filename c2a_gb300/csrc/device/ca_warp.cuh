/*
 * ca_warp.cuh -- the reference-order CA query on one warp: the depth-first
 * traversal stays sequential (the reference's order, its running bound, its
 * counters), while the work inside each step runs across the warp's lanes.
 *
 *   child pair tests  the two children of an expanded pair on the two
 *                     half-warps; lane j of a half evaluates C2ARectDist's
 *                     edge-pair case j (rect_cases.cuh), the first case that
 *                     holds wins (ballot), else the face-separation tail;
 *                     then d = max(dist - r1 - r2, 0) and the motion bounds
 *                     (C2A.cpp:1237-1274);
 *   TriDist           the nine segment pairs on nine lanes, then the
 *                     reference's in-order minimum/early-return logic replayed
 *                     over their results, and both vertex-over-face tests on
 *                     two lanes (C2A.cpp:165-405);
 *   control           descend decisions, the stack of pending second children
 *                     (shared memory, with their exact transforms) and the CA
 *                     loop run on every lane with identical values.
 *
 * Everything is the reference's FP64 arithmetic in its own order, so the
 * results are bit-identical to the thread-per-query kernel's (and the
 * reference's); only who computes which case changes.
 */
#ifndef C2A_CA_WARP_CUH
#define C2A_CA_WARP_CUH

#include "ca_kernel.cuh"
#include "rect_cases.cuh"

namespace c2a {

constexpr unsigned kWFull = 0xffffffffu;

/* a pending second child: the pair, its d and mint, its exact transform */
struct WStackEntry {
    int32_t b1, b2;
    double d, m;
    M3 R;
    V3 T;
};

/* per-warp shared state */
struct WarpShared {
    WStackEntry stack[C2A_STACK_DEPTH];
    WStackEntry child[2]; /* the children of the pair just expanded */
};

C2A_KDEV double shfl_d(double v, int src) { return __shfl_sync(kWFull, v, src); }
C2A_KDEV V3 shfl_v3(V3 v, int src) { return v3(shfl_d(v.x, src), shfl_d(v.y, src), shfl_d(v.z, src)); }

/* ------------------------------------------------------------- TriDist */

/* TriDist of S and Tt (same frame) with features, on the whole warp; the
 * results are identical on every lane */
C2A_KDEV double tri_dist_warp(const V3 S[3], const V3 Tt[3], V3 &P, V3 &Q, TriFeat &f, bool &collided, int lane)
{
    ExactCtx xc{false};
    V3 Sv[3], Tv[3];
    Sv[0] = S[1] - S[0];
    Sv[1] = S[2] - S[1];
    Sv[2] = S[0] - S[2];
    Tv[0] = Tt[1] - Tt[0];
    Tv[1] = Tt[2] - Tt[1];
    Tv[2] = Tt[0] - Tt[2];
    /* lanes 0..8: segment pair (i, j) = (lane / 3, lane % 3) */
    V3 VEC = v3(0, 0, 0), Pk = v3(0, 0, 0), Qk = v3(0, 0, 0);
    double dd = 0, ak = 0, bk = 0, pk = 0;
    if (lane < 9) {
        const int i = lane / 3, j = lane % 3;
        seg_pair(VEC, Pk, Qk, S[i], Sv[i], Tt[j], Tv[j], xc);
        const V3 V = Qk - Pk;
        dd = dot(V, V);
        ak = dot(S[(i + 2) % 3] - Pk, VEC);
        bk = dot(Tt[(j + 2) % 3] - Qk, VEC);
        pk = dot(V, VEC);
    }
    /* lanes 9 and 10: the two vertex-over-face tests */
    double tp = 0, nl = 0;
    V3 n = v3(0, 0, 0);
    bool disj = false;
    int point = -1;
    if (lane == 9) point = vertex_over_face(S, Sv, Tt, tp, nl, n, disj, xc);
    if (lane == 10) point = vertex_over_face(Tt, Tv, S, tp, nl, n, disj, xc);
    __syncwarp();
    /* the reference's loop over the nine pairs, in order */
    double mindd = dist2(S[0], Tt[0]) + 1.0;
    int mink = -1;
    bool shown_disjoint = false;
    for (int k = 0; k < 9; k++) {
        const double ddk = shfl_d(dd, k);
        const double ak_ = shfl_d(ak, k), bk_ = shfl_d(bk, k), pk_ = shfl_d(pk, k);
        if (ddk <= mindd) {
            mindd = ddk;
            mink = k;
            if (ak_ <= 0 && bk_ >= 0) { /* early return: the closest points of pair k */
                P = shfl_v3(Pk, k);
                Q = shfl_v3(Qk, k);
                f.type_a = 1;
                f.fid_a = k / 3;
                f.type_b = 1;
                f.fid_b = k % 3;
                collided = false;
                return sqrt(ddk);
            }
            const double a = max0_c(ak_), b = min0_c(bk_);
            if (pk_ - a + b > 0) shown_disjoint = true;
        }
    }
    const int p0 = __shfl_sync(kWFull, point, 9), p1 = __shfl_sync(kWFull, point, 10);
    const bool d0 = __shfl_sync(kWFull, (int)disj, 9) != 0, d1 = __shfl_sync(kWFull, (int)disj, 10) != 0;
    if (mink >= 0) {
        f.type_a = 1;
        f.fid_a = mink / 3;
        f.type_b = 1;
        f.fid_b = mink % 3;
    }
    const V3 minP = shfl_v3(Pk, mink < 0 ? 0 : mink), minQ = shfl_v3(Qk, mink < 0 ? 0 : mink);
    shown_disjoint = shown_disjoint || d0;
    if (p0 >= 0) {
        V3 Pw = v3(0, 0, 0), Qw = v3(0, 0, 0);
        double dw = 0;
        if (lane == 9) {
            Pw = add_mul(Tt[point], n, num_div(tp, nl, xc));
            Qw = Tt[point];
            dw = sqrt(dist2(Pw, Qw));
        }
        P = shfl_v3(Pw, 9);
        Q = shfl_v3(Qw, 9);
        f.type_a = 2;
        f.fid_a = -1;
        f.type_b = 0;
        f.fid_b = p0;
        collided = false;
        return shfl_d(dw, 9);
    }
    shown_disjoint = shown_disjoint || d1;
    if (p1 >= 0) {
        V3 Pw = v3(0, 0, 0), Qw = v3(0, 0, 0);
        double dw = 0;
        if (lane == 10) {
            Pw = S[point];
            Qw = add_mul(S[point], n, num_div(tp, nl, xc));
            dw = sqrt(dist2(Pw, Qw));
        }
        P = shfl_v3(Pw, 10);
        Q = shfl_v3(Qw, 10);
        f.type_a = 0;
        f.fid_a = p1;
        f.type_b = 2;
        f.fid_b = -1;
        collided = false;
        return shfl_d(dw, 10);
    }
    if (shown_disjoint) {
        P = minP;
        Q = minQ;
        collided = false;
        return sqrt(mindd);
    }
    /* collided: the points are those of the last pair tested, (2, 2) */
    P = shfl_v3(Pk, 8);
    Q = shfl_v3(Qk, 8);
    collided = true;
    return 0.0;
}

/* TriDist of leaf pair (ia, ib): B's triangle placed by (Rm, Tm) */
C2A_KDEV double tri_distance_warp(const Query &q, int ia, int ib, V3 &p, V3 &qq, TriFeat &f, bool &col, int lane)
{
    V3 S[3], T[3], t[3];
    load_tri(S, q.A->tris + ia);
    load_tri(t, q.B->tris + ib);
    T[0] = mul_add(q.Rm, t[0], q.Tm);
    T[1] = mul_add(q.Rm, t[1], q.Tm);
    T[2] = mul_add(q.Rm, t[2], q.Tm);
    return tri_dist_warp(S, T, p, qq, f, col, lane);
}

/* ------------------------------------------------------- child pair tests */

/* C2A_BV_Distance of this half-warp's child pair (x1, x2) placed by (R, T):
 * the rectangle distance with its S, on the half's sixteen lanes */
C2A_KDEV double rect_dist_half(const M3 &R, V3 T, const double a[2], const double b[2], V3 &S, int lane)
{
    ExactCtx xc{false};
    const int half = lane >> 4, j = lane & 15;
    V3 Sj = v3(0, 0, 0);
    bool hit = false;
    const double dj = rect_case(j, R, T, a, b, Sj, hit, xc);
    const unsigned m = (__ballot_sync(kWFull, hit) >> (16 * half)) & 0xffffu;
    const int win = m ? __ffs(m) - 1 : 0;
    const int src = 16 * half + win;
    const double dw = shfl_d(dj, src);
    const V3 Sw = shfl_v3(Sj, src);
    if (m) {
        S = Sw;
        return dw;
    }
    V3 St = S; /* the tail leaves S untouched when both separations are negative */
    const double dt = rect_tail(R, T, a, b, St, xc);
    S = St;
    return dt;
}

/* the two children of an expanded pair, tested like bv_test_x; each half
 * computes one child (transform, distance, motion bounds) and writes it to
 * sh.child[half]; nbv is counted by the caller */
C2A_KDEV void expand_warp(const Query &q, int b1, int b2, int fc1, int fc2, const M3 &PR, V3 PT, WarpShared &sh,
                          int lane)
{
    const int half = lane >> 4;
    int side, a1, a2, c1, c2;
    if (fc2 < 0 || (fc1 >= 0 && (__ldg(&q.A->nodes[b1].size) > __ldg(&q.B->nodes[b2].size)))) {
        side = 0;
        a1 = fc1; c1 = fc1 + 1;
        a2 = c2 = b2;
    } else {
        side = 1;
        a1 = c1 = b1;
        a2 = fc2; c2 = fc2 + 1;
    }
    const int x1 = half ? c1 : a1, x2 = half ? c2 : a2;
    M3 R;
    V3 T;
    child_transform(q, side, x1, x2, PR, PT, R, T);
    NodeX n1, n2;
    load_x(n1, q.A->nodes + x1);
    load_x(n2, q.B->nodes + x2);
    V3 S = v3(0, 0, 0);
    double z = rect_dist_half(R, T, n1.l, n2.l, S, lane);
    z -= (n1.r + n2.r);
    const double d = max0_c(z);
    double mint = 0.0;
    if (d != 0.0 && q.want_mint) {
        ExactCtx xc{false};
        V3 S1 = mul(q.r1, mul(n1.Rloc, S));
        V3 S2 = mul_s(S1, -1.0);
        const double mb1 = bound_rss(q.x1, n1.angR, S1, xc);
        const double mb2 = bound_rss(q.x2, n2.angR, S2, xc);
        mint = max0_c((d) / (mb1 + mb2));
    }
    if ((lane & 15) == 0) {
        WStackEntry &e = sh.child[half];
        e.b1 = x1;
        e.b2 = x2;
        e.d = d;
        e.m = mint;
        e.R = R;
        e.T = T;
    }
    __syncwarp();
}

/* ------------------------------------------------------------ the step */

C2A_KDEV bool descend_w(const Query &q, double m, double d)
{
    return m < q.upbound && ((d < (q.distance - q.abs_err)) || (d * (1 + q.rel_err) < q.distance));
}

/* a leaf pair of the rotation step (C2A.cpp:1141-1183) */
C2A_KDEV void leaf_step_warp(Query &q, int b1, int b2, int fc1, int fc2, int lane)
{
    const int ia = -fc1 - 1, ib = -fc2 - 1;
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double dTri = tri_distance_warp(q, ia, ib, p, qq, f, col, lane);
    if (dTri <= q.distance) {
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
    }
    q.ntri++;
}

/* TOCStepRecurse_Dis from the root pair, in the reference's order */
C2A_KDEV void toc_dfs_warp(Query &q, const M3 &Rroot, V3 Troot, WarpShared &sh, int lane)
{
    int sp = 0;
    int b1 = 0, b2 = 0;
    M3 R = Rroot;
    V3 T = Troot;
    for (;;) {
        const int fc1 = __ldg(&q.A->nodes[b1].first_child), fc2 = __ldg(&q.B->nodes[b2].first_child);
        bool go = false;
        if (fc1 < 0 && fc2 < 0) {
            leaf_step_warp(q, b1, b2, fc1, fc2, lane);
        } else {
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            expand_warp(q, b1, b2, fc1, fc2, R, T, sh, lane);
            q.nbv += 2;
            const WStackEntry &a = sh.child[0], &c = sh.child[1];
            const bool c_first = c.d < a.d; /* d2 < d1 (C2A.cpp:1281) */
            const WStackEntry &first = c_first ? c : a;
            if (lane == 0) sh.stack[sp] = c_first ? a : c;
            sp++;
            if (descend_w(q, first.m, first.d)) {
                b1 = first.b1;
                b2 = first.b2;
                R = first.R;
                T = first.T;
                go = true;
            } else if (first.m < q.mint) {
                q.mint = first.m;
            }
            __syncwarp();
        }
        while (!go && sp > 0) {
            const WStackEntry &e = sh.stack[--sp];
            if (descend_w(q, e.m, e.d)) {
                b1 = e.b1;
                b2 = e.b2;
                R = e.R;
                T = e.T;
                go = true;
            } else if (e.m < q.mint) {
                q.mint = e.m;
            }
        }
        __syncwarp();
        if (!go) return;
    }
}

/* C2A_TimeOfContactStep, rotation branch (C2A.cpp:1855-1931) */
C2A_KDEV void toc_step_warp(Query &q, M3 &R1, V3 &T1, M3 &R2, V3 &T2, WarpShared &sh, int lane)
{
    M3 R;
    V3 T;
    relative_transforms(q, R1, T1, R2, T2, R, T);
    {
        V3 p, qq;
        TriFeat f;
        bool col = false;
        q.distance = tri_distance_warp(q, q.seed_a, q.seed_b, p, qq, f, col, lane);
    }
    if (q.numCA == 0) q.mint = 1;
    if (q.mint <= 0.005 || q.distance <= 0.5 || q.numCA > 5) { /* C2A.cpp:1869-1891 */
        q.abs_err = 0;
        q.rel_err = 0;
    } else {
        q.abs_err = 1e+30;
        q.rel_err = (q.numCA <= 2) ? 3 : 0.5;
    }
    q.mint = 1;
    toc_dfs_warp(q, R, T, sh, lane);
}

/* --------------------------------------------------- contact enumeration */

/* a leaf pair of the contact enumeration (C2A.cpp:1560-1630) */
C2A_KDEV bool contact_leaf_warp(Query &q, int fc1, int fc2, double threshold, int query_index, c2a_contact &c,
                                int lane)
{
    const int ia = -fc1 - 1, ib = -fc2 - 1;
    V3 p, qq;
    TriFeat f{-1, -1, -1, -1};
    bool col = false;
    const double d = tri_distance_warp(q, ia, ib, p, qq, f, col, lane);
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

/* TOCStepRecurse_Dis_contact with a fixed threshold (C2A.cpp:1525-1725):
 * contacts in visiting order; returns how many were found */
C2A_KDEV int contact_dfs_warp(Query &q, const M3 &Rroot, V3 Troot, double threshold, WarpShared &sh,
                              c2a_contact *out, int slots, int query_index, int lane)
{
    int count = 0, sp = 0;
    int b1 = 0, b2 = 0;
    M3 R = Rroot;
    V3 T = Troot;
    for (;;) {
        const int fc1 = __ldg(&q.A->nodes[b1].first_child), fc2 = __ldg(&q.B->nodes[b2].first_child);
        bool go = false;
        if (fc1 < 0 && fc2 < 0) {
            c2a_contact c;
            if (contact_leaf_warp(q, fc1, fc2, threshold, query_index, c, lane)) {
                if (lane == 0 && count < slots && out) out[count] = c;
                count++;
            }
        } else {
            if (sp >= C2A_STACK_DEPTH) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return count;
            }
            expand_warp(q, b1, b2, fc1, fc2, R, T, sh, lane);
            const WStackEntry &a = sh.child[0], &c = sh.child[1];
            const bool c_first = c.d < a.d;
            const WStackEntry &first = c_first ? c : a;
            if (lane == 0) sh.stack[sp] = c_first ? a : c;
            sp++;
            if ((first.d < (threshold - 0)) || (first.d * (1.0 + 0) < threshold)) {
                b1 = first.b1;
                b2 = first.b2;
                R = first.R;
                T = first.T;
                go = true;
            }
            __syncwarp();
        }
        while (!go && sp > 0) {
            const WStackEntry &e = sh.stack[--sp];
            if ((e.d < (threshold - 0)) || (e.d * (1.0 + 0) < threshold)) {
                b1 = e.b1;
                b2 = e.b2;
                R = e.R;
                T = e.T;
                go = true;
            }
        }
        __syncwarp();
        if (!go) return count;
    }
}

/* ------------------------------------------------------------ one query */

/* C2A_Solve on one warp (reference order); lane 0 writes the result.  The
 * translation-only step runs the sequential code on every lane. */
C2A_KDEV void solve_query_warp(const c2a_query &in, const DevModel *models, int num_models, const c2a_params &prm,
                               c2a_result &out_g, c2a_contact *contacts, WarpShared &sh, Pending *tstack,
                               int query_index, int lane)
{
    c2a_result out;
    memset(&out, 0, sizeof(out));
    out.status = C2A_QUERY_OK;
    out.contact_offset = query_index * prm.contacts_per_query;
    const bool bad_models = in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 ||
                            in.model_b >= num_models || !(models[in.model_a].flags & C2A_MODEL_LIVE) ||
                            !(models[in.model_b].flags & C2A_MODEL_LIVE);
    if (bad_models || in.seed_a < 0 || in.seed_a >= models[in.model_a].num_tris || in.seed_b < 0 ||
        in.seed_b >= models[in.model_b].num_tris) {
        out.status = C2A_QUERY_BAD_INPUT;
        if (lane == 0) out_g = out;
        return;
    }
    Query q;
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) q.st[i] = 0;
#endif
    q.status = 0;
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    q.want_mint = true;
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
    if (translation) toc_step(q, R1, T1, R2, T2, true, tstack);
    else toc_step_warp(q, R1, T1, R2, T2, sh, lane);
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
            toc_step_warp(q, R1, T1, R2, T2, sh, lane);
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
            q.want_mint = false;
            const int n = contact_dfs_warp(q, R, T, threshold, sh, contacts, prm.contacts_per_query, query_index,
                                           lane);
            out.num_contact = n;
            if (n > prm.contacts_per_query) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
        }
    }
    out.status |= q.status;
    if (lane == 0) out_g = out;
}

} // namespace c2a
#endif
