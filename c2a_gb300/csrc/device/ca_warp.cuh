/*
 * ca_warp.cuh -- the reference-order CA query on one warp: the depth-first
 * traversal stays sequential (the reference's order, its running bound, its
 * counters), while the work inside each step runs across the warp's lanes.
 *
 *   child pair tests  the two children of an expanded pair on the two
 *                     half-warps: the child transform one output per lane;
 *                     C2ARectDist's shared sums a few per lane into
 *                     shared-memory slots, lane j then tests edge-pair case j
 *                     with operands read through tables (rect_table.cuh), the
 *                     first case that holds wins (ballot) and only its lane
 *                     evaluates the distance, else the face-separation tail;
 *                     then d = max(dist - r1 - r2, 0) and the motion bounds,
 *                     S one row per lane and the two bounds on alternate lanes
 *                     (C2A.cpp:1237-1274);
 *   TriDist           the nine segment pairs on nine lanes, then the
 *                     reference's in-order minimum/early-return logic replayed
 *                     over their results, and both vertex-over-face tests on
 *                     two lanes (C2A.cpp:165-405);
 *   control           descend decisions and the CA loop run on every lane with
 *                     identical values; the query state, the children just
 *                     tested and the stack of pending second children (with
 *                     their exact transforms) live in the warp's shared memory.
 *
 * Everything is the reference's FP64 arithmetic in its own order, so the
 * results are bit-identical to the thread-per-query kernel's (and the
 * reference's); only who computes which case changes.
 */
#ifndef C2A_CA_WARP_CUH
#define C2A_CA_WARP_CUH

#include "ca_kernel.cuh"
#include "rect_cases.cuh"
#include "rect_table.cuh"
#include "rect_table_ef.cuh"

namespace c2a {

constexpr unsigned kWFull = 0xffffffffu;

/* The warp-uniform state (the query, the speculative engine's bookkeeping)
 * is written by every lane with the same value.  The speculative engine's
 * shared writes go through C2A_WSET, which fences each write with warp
 * barriers, so no lane reads a location while another lane writes it even
 * where the lanes do not run converged; the warp kernel's query updates
 * rely on the warp executing that code converged.  A host emulation of the
 * warp replaces the query reference with a per-lane copy. */
#ifndef C2A_WARP_QUERY
#define C2A_WARP_QUERY(sh) ((sh).q)
#endif
#ifndef C2A_WSET
#define C2A_WSET(dst, v)                                                                                           \
    do {                                                                                                           \
        auto wset_v_ = (v);                                                                                        \
        __syncwarp();                                                                                              \
        (dst) = wset_v_;                                                                                           \
        __syncwarp();                                                                                              \
    } while (0)
#endif

/* 1: node-pair and leaf tests through the certified FP32 filter (FP64 only
 * where it cannot decide); 0: every test in FP64 */
#ifndef C2A_WARP_FILTER
#define C2A_WARP_FILTER 0
#endif

/* a child pair: its d and mint as certified FP32 values (d_e, m_e) or, once
 * exact, the reference's FP64 values (d, m); its exact transform */
struct WStackEntry {
    int32_t b1, b2;
    int32_t exact, pad;
    double d, m;
    EF d_e, m_e;
    M3 R;
    V3 T;
};

static_assert(sizeof(WStackEntry) % 8 == 0 && offsetof(WStackEntry, T) == offsetof(WStackEntry, R) + sizeof(M3),
              "a record is copied as 8-byte words and its transform written as 12 contiguous doubles");

/* per-warp shared state: the query (one copy per warp; every lane computes
 * the same values, so every lane may write them), the children of the pair
 * just expanded, each half's RectDist slots (rect_table.cuh), then the stack
 * of pending second children, `cap` entries (set at launch from the deepest
 * hierarchy in the context) */
struct WarpShared {
    Query q;
    WStackEntry child[2];
    double rt[2][64];
    int32_t cap, pad_[3];
    WStackEntry stack[1]; /* cap entries */
};

/* bytes of one warp's shared state with a stack of cap entries (16-byte multiple) */
__host__ __device__ constexpr size_t warp_shared_bytes(int cap)
{
    return ((offsetof(WarpShared, stack) + (size_t)cap * sizeof(WStackEntry)) + 15) / 16 * 16;
}

C2A_KDEV double shfl_d(double v, int src) { return __shfl_sync(kWFull, v, src); }
C2A_KDEV V3 shfl_v3(V3 v, int src) { return v3(shfl_d(v.x, src), shfl_d(v.y, src), shfl_d(v.z, src)); }
C2A_KDEV EF K_EF1() { return ef_exact(1.0f); }
C2A_KDEV EF shfl_e(EF v, int src) { return EF{__shfl_sync(kWFull, v.v, src), __shfl_sync(kWFull, v.e, src)}; }
C2A_KDEV V3T<EF> shfl_v3e(V3T<EF> v, int src) { return v3t(shfl_e(v.x, src), shfl_e(v.y, src), shfl_e(v.z, src)); }

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

/* the FP32 filter of TriDist on the warp: the distance with a certified
 * bound, or ok = false when a decision of the reference's TriDist cannot be
 * certified (the caller then computes it in FP64) */
C2A_KDEV EF tri_dist_warp_e(const V3T<EF> S[3], const V3T<EF> Tt[3], TriFeat &f, bool &ok, int lane)
{
    EFCtx ctx{false};
    const EF zero = ef_exact(0.0f);
    V3T<EF> Sv[3], Tv[3];
    Sv[0] = S[1] - S[0];
    Sv[1] = S[2] - S[1];
    Sv[2] = S[0] - S[2];
    Tv[0] = Tt[1] - Tt[0];
    Tv[1] = Tt[2] - Tt[1];
    Tv[2] = Tt[0] - Tt[2];
    V3T<EF> VEC = v3t(zero, zero, zero), Pk = VEC, Qk = VEC;
    EF dd = zero, ak = zero, bk = zero, pk = zero;
    bool lbad = false;
    if (lane < 9) {
        EFCtx lc{false};
        const int i = lane / 3, j = lane % 3;
        seg_pair(VEC, Pk, Qk, S[i], Sv[i], Tt[j], Tv[j], lc);
        const V3T<EF> V = Qk - Pk;
        dd = dot(V, V);
        ak = dot(S[(i + 2) % 3] - Pk, VEC);
        bk = dot(Tt[(j + 2) % 3] - Qk, VEC);
        pk = dot(V, VEC);
        lbad = lc.bad;
    }
    EF tp = zero, nl = zero;
    V3T<EF> n = v3t(zero, zero, zero);
    bool disj = false;
    int point = -1;
    if (lane == 9 || lane == 10) {
        EFCtx vc{false};
        point = lane == 9 ? vertex_over_face(S, Sv, Tt, tp, nl, n, disj, vc) : vertex_over_face(Tt, Tv, S, tp, nl, n, disj, vc);
        lbad = vc.bad;
    }
    __syncwarp();
    const unsigned badm = __ballot_sync(kWFull, lbad);
    EF mindd = dist2(S[0], Tt[0]) + K_EF1();
    int mink = -1;
    bool shown_disjoint = false;
    for (int k = 0; k < 9; k++) {
        const EF ddk = shfl_e(dd, k), ak_ = shfl_e(ak, k), bk_ = shfl_e(bk, k), pk_ = shfl_e(pk, k);
        if ((badm >> k) & 1u) ctx.bad = true;
        if (cmp_le(ddk, mindd, ctx, 0)) {
            mindd = ddk;
            mink = k;
            if (cmp_le(ak_, zero, ctx, 0) && cmp_le(zero, bk_, ctx, 0)) {
                f.type_a = 1;
                f.fid_a = k / 3;
                f.type_b = 1;
                f.fid_b = k % 3;
                ok = !ctx.bad;
                return num_sqrt(ddk);
            }
            const EF a = max0_c(ak_), b = min0_c(bk_);
            if (cmp_lt(zero, pk_ - a + b, ctx, 0)) shown_disjoint = true;
        }
    }
    if ((badm >> 9) & 1u) ctx.bad = true;
    const int p0 = __shfl_sync(kWFull, point, 9), p1 = __shfl_sync(kWFull, point, 10);
    const bool d0 = __shfl_sync(kWFull, (int)disj, 9) != 0, d1 = __shfl_sync(kWFull, (int)disj, 10) != 0;
    if (mink >= 0) {
        f.type_a = 1;
        f.fid_a = mink / 3;
        f.type_b = 1;
        f.fid_b = mink % 3;
    }
    shown_disjoint = shown_disjoint || d0;
    if (p0 >= 0) {
        EF dw = zero;
        bool wb = false;
        if (lane == 9) {
            EFCtx wc{false};
            const V3T<EF> Pw = add_mul(Tt[point], n, num_div(tp, nl, wc));
            dw = num_sqrt(dist2(Pw, Tt[point]));
            wb = wc.bad;
        }
        f.type_a = 2;
        f.fid_a = -1;
        f.type_b = 0;
        f.fid_b = p0;
        ok = !ctx.bad && !__shfl_sync(kWFull, (int)wb, 9);
        return shfl_e(dw, 9);
    }
    if ((badm >> 10) & 1u) ctx.bad = true;
    shown_disjoint = shown_disjoint || d1;
    if (p1 >= 0) {
        EF dw = zero;
        bool wb = false;
        if (lane == 10) {
            EFCtx wc{false};
            const V3T<EF> Qw = add_mul(S[point], n, num_div(tp, nl, wc));
            dw = num_sqrt(dist2(S[point], Qw));
            wb = wc.bad;
        }
        f.type_a = 0;
        f.fid_a = p1;
        f.type_b = 2;
        f.fid_b = -1;
        ok = !ctx.bad && !__shfl_sync(kWFull, (int)wb, 10);
        return shfl_e(dw, 10);
    }
    ok = !ctx.bad;
    if (shown_disjoint) return num_sqrt(mindd);
    f.type_a = f.type_b = -1; /* collided: left to the FP64 path */
    ok = false;
    return zero;
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

/* the FP32 filter of a leaf pair's TriDist (needs q.shadows_ok) */
C2A_KDEV EF tri_distance_warp_e(const Query &q, int ia, int ib, TriFeat &f, bool &ok, int lane)
{
    V3T<EF> S[3], T[3], t[3];
    load_tri_e(S, q.A->stris + ia);
    load_tri_e(t, q.B->stris + ib);
    T[0] = mul_add(q.Rme, t[0], q.Tme);
    T[1] = mul_add(q.Rme, t[1], q.Tme);
    T[2] = mul_add(q.Rme, t[2], q.Tme);
    return tri_dist_warp_e(S, T, f, ok, lane);
}

/* ------------------------------------------------------- child pair tests */

/* C2A_BV_Distance of this half-warp's child pair placed by (R, T): the
 * rectangle distance with its S, on the half's sixteen lanes.  The shared
 * sums are spread over the lanes (slots V in shared memory, rect_table.cuh),
 * lane j then tests edge-pair case j; the first case that holds wins and only
 * its lane evaluates the distance; no case: the face-separation tail. */
C2A_KDEV double rect_dist_half(const M3 &R, V3 T, const double a[2], const double b[2], V3 &S, double *V, int lane)
{
    const int half = lane >> 4, k = lane & 15;
    __syncwarp(); /* the previous call's reads of V are done */
    rt_inputs(R, T, a, b, V);
    __syncwarp();
    if (k < kRtStage1) V[kRtInputs + k] = rt_stage1(k, R, T, V);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const int i = k + 16 * r;
        if (i < kRtStage2) V[kRtStage2Base + i] = rt_stage2(i, V);
    }
    __syncwarp();
    const bool below = k < 8 && rt_compare(k, V);
    const unsigned mask = (__ballot_sync(kWFull, below) >> (16 * half)) & 0xffu;
    double L[4], Rr[4], s1[7], s2[7], e[5], qb;
    int px, py, qkind, cb, cu;
    rt_case_operands(k, mask, V, L, Rr, s1, s2, e, qb, px, py, qkind, cb, cu);
    const bool hit = rt_case_holds(L, Rr, s1, s2);
    const unsigned m = (__ballot_sync(kWFull, hit) >> (16 * half)) & 0xffffu;
    const int win = m ? __ffs(m) - 1 : 0;
    double dj = 0.0;
    V3 Sj = v3(0, 0, 0);
    if (m && k == win) dj = rt_case_value(e, qb, px, py, qkind, cb, cu, R, T, a, Sj);
    const int src = 16 * half + win;
    const double dw = shfl_d(dj, src);
    const V3 Sw = shfl_v3(Sj, src);
    if (m) {
        S = Sw;
        return dw;
    }
    ExactCtx xc{false};
    V3 St = S; /* the tail leaves S untouched when both separations are negative */
    const double dt = rect_tail(R, T, a, b, St, xc);
    S = St;
    return dt;
}

#if C2A_WARP_FILTER == 2
/* rect_dist_half in the certified FP32 filter (rect_table_ef.cuh): the same
 * slots, stages, comparison mask and operand tables with EF values; ok is
 * false when a sort comparison, a case condition before the winner, the
 * winner's own condition or its value could not be certified */
C2A_KDEV EF rect_dist_half_e(const M3T<EF> &R, V3T<EF> T, const EF a[2], const EF b[2], V3T<EF> &S, EF *V, bool &ok,
                             int lane)
{
    const int half = lane >> 4, k = lane & 15;
    __syncwarp(); /* the previous call's reads of V are done */
    rte_inputs(R, T, a, b, V);
    __syncwarp();
    if (k < kRtStage1) V[kRtInputs + k] = rte_stage1(k, R, T, V);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const int i = k + 16 * r;
        if (i < kRtStage2) V[kRtStage2Base + i] = rte_stage2(i, V);
    }
    __syncwarp();
    const int cmp = k < 8 ? rte_compare(k, V) : 0;
    const unsigned mask = (__ballot_sync(kWFull, cmp == 1) >> (16 * half)) & 0xffu;
    const bool sort_bad = ((__ballot_sync(kWFull, cmp < 0) >> (16 * half)) & 0xffu) != 0u;
    EF L[4], Rr[4], s1[7], s2[7], e[5], qb;
    int px, py, qkind, cb, cu;
    rte_case_operands(k, mask, V, L, Rr, s1, s2, e, qb, px, py, qkind, cb, cu);
    EFCtx hc{false};
    const bool holds = rte_case_holds(L, Rr, s1, s2, hc);
    const unsigned m = (__ballot_sync(kWFull, holds && !hc.bad) >> (16 * half)) & 0xffffu;
    const unsigned bad = (__ballot_sync(kWFull, hc.bad) >> (16 * half)) & 0xffffu;
    const int win = m ? __ffs(m) - 1 : 16;
    /* every case up to the winner (all sixteen when none holds) must be settled */
    const unsigned upto = win < 16 ? ((1u << (win + 1)) - 1u) : 0xffffu;
    ok = !sort_bad && (bad & upto) == 0u;
    EF dj = ef_exact(0.0f);
    V3T<EF> Sj = v3t(dj, dj, dj);
    int vbad = 0;
    if (m && k == win) {
        EFCtx vc{false};
        dj = rte_case_value(e, qb, px, py, qkind, cb, cu, R, T, a, Sj, vc);
        vbad = vc.bad ? 1 : 0;
    }
    const int src = 16 * half + (win < 16 ? win : 0);
    const EF dw = shfl_e(dj, src);
    const V3T<EF> Sw = shfl_v3e(Sj, src);
    const bool vb = __shfl_sync(kWFull, vbad, src) != 0;
    if (m) {
        S = Sw;
        ok = ok && !vb;
        return dw;
    }
    EFCtx tc{false};
    V3T<EF> St = S;
    const EF dt = rect_tail(R, T, a, b, St, tc);
    S = St;
    ok = ok && !tc.bad;
    return dt;
}
#endif

/* the children of an internal pair (C2A.cpp:1192-1226) */
C2A_KDEV void split_pair(const Query &q, int b1, int b2, int fc1, int fc2, int &side, int &a1, int &a2, int &c1,
                         int &c2)
{
    if (fc2 < 0 || (fc1 >= 0 && (__ldg(&q.A->nodes[b1].size) > __ldg(&q.B->nodes[b2].size)))) {
        side = 0;
        a1 = fc1; c1 = fc1 + 1;
        a2 = c2 = b2;
    } else {
        side = 1;
        a1 = c1 = b1;
        a2 = fc2; c2 = fc2 + 1;
    }
}

C2A_KDEV double pick3(double a, double b, double c, int i) { return i == 0 ? a : (i == 1 ? b : c); }

/* child_transform on one half-warp: lane k < 9 of the half computes R[k / 3][k % 3],
 * lanes 9..11 T[k - 9], with the expression trees of tmmul/tmul (side 0) or
 * mmul/mul_add (side 1); the half then shares the twelve values */
C2A_KDEV void child_transform_lanes(const Query &q, int side, int x1, int x2, const M3 &PR, V3 PT, M3 &R, V3 &T,
                                    double &own, int lane)
{
    const int half = lane >> 4, k = lane & 15;
    const NodeRec *n = side == 0 ? q.A->nodes + x1 : q.B->nodes + x2;
    const M3 Rc = load_R(n);
    const V3 Tr = load_Tr(n);
    const bool isT = k >= 9;
    const int i = isT ? (k - 9 < 3 ? k - 9 : 2) : k / 3, j = isT ? 0 : k % 3;
    double a0, a1, a2, b0, b1, b2, c = 0.0;
    if (side == 0) { /* R = Rc^T PR, T = Rc^T (PT - Tr) */
        a0 = pick3(Rc.m[0], Rc.m[1], Rc.m[2], i);
        a1 = pick3(Rc.m[3], Rc.m[4], Rc.m[5], i);
        a2 = pick3(Rc.m[6], Rc.m[7], Rc.m[8], i);
        const V3 v = PT - Tr;
        b0 = isT ? v.x : pick3(PR.m[0], PR.m[1], PR.m[2], j);
        b1 = isT ? v.y : pick3(PR.m[3], PR.m[4], PR.m[5], j);
        b2 = isT ? v.z : pick3(PR.m[6], PR.m[7], PR.m[8], j);
    } else { /* R = PR Rc, T = PR Tr + PT */
        a0 = pick3(PR.m[0], PR.m[3], PR.m[6], i);
        a1 = pick3(PR.m[1], PR.m[4], PR.m[7], i);
        a2 = pick3(PR.m[2], PR.m[5], PR.m[8], i);
        b0 = isT ? Tr.x : pick3(Rc.m[0], Rc.m[1], Rc.m[2], j);
        b1 = isT ? Tr.y : pick3(Rc.m[3], Rc.m[4], Rc.m[5], j);
        b2 = isT ? Tr.z : pick3(Rc.m[6], Rc.m[7], Rc.m[8], j);
        c = pick3(PT.x, PT.y, PT.z, i);
    }
    double v = a0 * b0 + a1 * b1 + a2 * b2;
    if (side == 1 && isT) v = v + c;
    own = v; /* lane k < 12 of the half: R.m[k], then T */
    const int base = 16 * half;
#pragma unroll
    for (int e = 0; e < 9; e++) R.m[e] = shfl_d(v, base + e);
    T = v3(shfl_d(v, base + 9), shfl_d(v, base + 10), shfl_d(v, base + 11));
}

/* bv_test_x of child pair (x1, x2) placed by (R, T), exactly, on one half-warp */
C2A_KDEV void child_test_x(const Query &q, int x1, int x2, const M3 &R, V3 T, double &d, double &mint, int lane)
{
    NodeX n1, n2;
    load_x(n1, q.A->nodes + x1);
    load_x(n2, q.B->nodes + x2);
    V3 S = v3(0, 0, 0);
    C2A_WCLOCK(xc0);
    double z = rect_dist_half(R, T, n1.l, n2.l, S, q.rt + 64 * (lane >> 4), lane);
    C2A_WCLOCK(xc1);
    C2A_WSTAT(q, ST_W_CYC_X_RECT, xc1 - xc0);
    z -= (n1.r + n2.r);
    d = max0_c(z);
    mint = 0.0;
    if (q.want_mint) { /* uniform over the warp; d differs between the halves */
        /* S1 = r1 (Rloc S) one row per lane, then the two motion bounds on
         * alternate lanes of the half, then shared; every lane computes (the
         * shuffles need the whole warp), the result is used where the reference
         * computes it (d != 0) */
        ExactCtx xc{false};
        const int base = 16 * (lane >> 4), row = (lane & 15) % 3;
        const double u = n1.Rloc.m[3 * row] * S.x + n1.Rloc.m[3 * row + 1] * S.y + n1.Rloc.m[3 * row + 2] * S.z;
        const V3 U = v3(shfl_d(u, base), shfl_d(u, base + 1), shfl_d(u, base + 2));
        const double w = q.r1.m[3 * row] * U.x + q.r1.m[3 * row + 1] * U.y + q.r1.m[3 * row + 2] * U.z;
        const V3 S1 = v3(shfl_d(w, base), shfl_d(w, base + 1), shfl_d(w, base + 2));
        const bool second = (lane & 1) != 0;
        V3 N = second ? mul_s(S1, -1.0) : S1;
        const MotionT<double> mm = second ? q.x2 : q.x1;
        const double mb = bound_rss(mm, second ? n2.angR : n1.angR, N, xc);
        const double mb1 = shfl_d(mb, base), mb2 = shfl_d(mb, base + 1);
        if (d != 0.0) mint = max0_c((d) / (mb1 + mb2));
        C2A_WCLOCK(xc2);
        C2A_WSTAT(q, ST_W_CYC_X_BOUND, xc2 - xc1);
    }
}

/* the same with the FP32 filter; false when a half cannot certify it */
C2A_KDEV bool child_test_e(const Query &q, int x1, int x2, const M3 &R, V3 T, EF &d, EF &mint, bool &d_zero,
                           int lane)
{
    const int half = lane >> 4, j = lane & 15;
    EFCtx pc{!q.shadows_ok};
    const M3T<EF> Re = ef_m3(R, pc);
    const V3T<EF> Te = ef_v3(T, pc);
    NodeE n1, n2;
    load_e(n1, q.A->snodes + x1);
    load_e(n2, q.B->snodes + x2);
    const EF zero = ef_exact(0.0f);
#if C2A_WARP_FILTER == 2
    C2A_WCLOCK(y0);
    bool ok;
    EF dist;
    V3T<EF> S = v3t(zero, zero, zero);
    {
        bool rok = true;
        dist = rect_dist_half_e(Re, Te, n1.l, n2.l, S, reinterpret_cast<EF *>(q.rt + 64 * half), rok, lane);
        ok = rok && !pc.bad;
        (void)j;
    }
#else
    V3T<EF> Sj = v3t(zero, zero, zero);
    int hit = 0;
    bool vbad = false;
    C2A_WCLOCK(y0);
    const EF dj = rect_case(j, Re, Te, n1.l, n2.l, Sj, hit, vbad, pc);
    const unsigned nz = (__ballot_sync(kWFull, hit != 0) >> (16 * half)) & 0xffffu;
    const int src = 16 * half + (nz ? __ffs(nz) - 1 : 0);
    const int hw = __shfl_sync(kWFull, hit, src);
    const bool vb = __shfl_sync(kWFull, (int)vbad, src) != 0;
    const EF dw = shfl_e(dj, src);
    const V3T<EF> Sw = shfl_v3e(Sj, src);
    bool ok;
    EF dist;
    V3T<EF> S;
    if (nz) {
        ok = hw == 1 && !vb;
        dist = dw;
        S = Sw;
    } else {
        EFCtx tc{pc.bad};
        V3T<EF> St = v3t(zero, zero, zero);
        dist = rect_tail(Re, Te, n1.l, n2.l, St, tc);
        S = St;
        ok = !tc.bad;
    }
#endif
    C2A_WCLOCK(y1);
    C2A_WSTAT(q, ST_W_CYC_E_RECT, y1 - y0);
    const EF z = dist - (n1.r + n2.r);
    const int pos = ef_lt3(zero, z);
    if (pos < 0) ok = false;
    d_zero = pos == 0;
    d = d_zero ? zero : z;
    mint = zero;
    if (ok && !d_zero && q.want_mint) {
        EFCtx bc{false};
        V3T<EF> S1 = mul(q.r1e, mul(n1.Rloc, S));
        V3T<EF> S2 = mul_s(S1, ef_exact(-1.0f));
        const EF mb1 = bound_rss(q.e1, n1.angR, S1, bc);
        const EF mb2 = bound_rss(q.e2, n2.angR, S2, bc);
        mint = max0_c(ef_div(d, mb1 + mb2, bc));
        ok = !bc.bad;
    }
    C2A_WCLOCK(y2);
    C2A_WSTAT(q, ST_W_CYC_E_BOUND, y2 - y1);
    return ok;
}

/* the two children of an expanded pair into sh.child[0] (a) and sh.child[1]
 * (c): each half tests one with the FP32 filter; if a half cannot certify
 * its child, both are tested in FP64 */
C2A_KDEV void expand_warp(const Query &q, int b1, int b2, int fc1, int fc2, const M3 &PR, V3 PT, WarpShared &sh,
                          int lane)
{
    const int half = lane >> 4;
    int side, a1, a2, c1, c2;
    split_pair(q, b1, b2, fc1, fc2, side, a1, a2, c1, c2);
    const int x1 = half ? c1 : a1, x2 = half ? c2 : a2;
    M3 R;
    V3 T;
    double own;
    C2A_WCLOCK(w0);
    child_transform_lanes(q, side, x1, x2, PR, PT, R, T, own, lane);
    C2A_WCLOCK(w1);
    EF d = ef_exact(0.0f), m = ef_exact(0.0f);
    bool d_zero = false;
    const bool ok = C2A_WARP_FILTER && child_test_e(q, x1, x2, R, T, d, m, d_zero, lane);
    C2A_WCLOCK(w2);
    double dx = 0.0, mx = 0.0;
    int exact = d_zero ? 1 : 0; /* d = max(z, 0) = 0 and mint = 0 exactly */
    if (!__all_sync(kWFull, ok)) {
        child_test_x(q, x1, x2, R, T, dx, mx, lane);
        exact = 1;
        C2A_WSTAT(q, ST_W_EFAIL, 1);
    }
    C2A_WCLOCK(w3);
    C2A_WSTAT(q, ST_W_EXPAND, 1);
    C2A_WSTAT(q, ST_W_CYC_XFORM, w1 - w0);
    C2A_WSTAT(q, ST_W_CYC_TEST_E, w2 - w1);
    C2A_WSTAT(q, ST_W_CYC_TEST_X, w3 - w2);
    WStackEntry &e = sh.child[half];
#if C2A_WARP_FILTER
    if ((lane & 15) == 0) {
        e.b1 = x1;
        e.b2 = x2;
        e.exact = exact;
        e.pad = 0;
        e.d = dx;
        e.m = mx;
        e.d_e = d;
        e.m_e = m;
        if (exact) { /* the FP32 views of exact values decide too */
            EFCtx cc{false};
            e.d_e = in_d(dx, cc);
            e.m_e = in_d(mx, cc);
            if (cc.bad) e.d_e = e.m_e = EF{0.0f, __int_as_float(0x7f800000)};
        }
        e.R = R;
        e.T = T;
    }
#else
    { /* the record written across the half: lane k < 12 its own transform entry */
        const int k = lane & 15;
        if (k < 12) reinterpret_cast<double *>(&e.R)[k] = own; /* R then T, contiguous */
        else if (k == 12) { e.b1 = x1; e.b2 = x2; }
        else if (k == 13) { e.exact = exact; e.pad = 0; }
        else if (k == 14) e.d = dx;
        else e.m = mx;
    }
#endif
    __syncwarp();
    C2A_WCLOCK(w4);
    C2A_WSTAT(q, ST_W_CYC_STORE, w4 - w3);
}

/* the exact d and mint of a child pair (both halves compute it; uniform) */
C2A_KDEV void make_exact_warp(const Query &q, WStackEntry &e, int lane)
{
    if (e.exact) return;
    C2A_WSTAT(q, ST_W_MKEXACT, 1);
    child_test_x(q, e.b1, e.b2, e.R, e.T, e.d, e.m, lane);
    EFCtx cc{false};
    e.d_e = in_d(e.d, cc);
    e.m_e = in_d(e.m, cc);
    if (cc.bad) e.d_e = e.m_e = EF{0.0f, __int_as_float(0x7f800000)};
    e.exact = 1;
}

/* ------------------------------------------------------------ the step */

/* mint < UpboundTOC && (d < distance - abs_err || d * (1 + rel_err) < distance) (C2A.cpp:1281-1351) */
C2A_KDEV bool descend_w(const Query &q, WStackEntry &e, int lane)
{
#if !C2A_WARP_FILTER /* every record is exact */
    return e.m < q.upbound && ((e.d < (q.distance - q.abs_err)) || (e.d * (1 + q.rel_err) < q.distance));
#endif
    if (q.shadows_ok) {
        const int a = ef_lt3(e.m_e, q.upbound_e);
        const int b = ef_lt3(e.d_e, q.bound_e);
        const int c = ef_lt3(e.d_e * q.rel1_e, q.distance_e);
        const int r = and3(a, or3(b, c));
        if (r >= 0) return r == 1;
    }
    make_exact_warp(q, e, lane);
    return e.m < q.upbound && ((e.d < (q.distance - q.abs_err)) || (e.d * (1 + q.rel_err) < q.distance));
}

/* a pruned pair's mint lowers res->mint (C2A.cpp:1290-1311) */
C2A_KDEV void contribute_w(Query &q, WStackEntry &e, int lane)
{
    if (C2A_WARP_FILTER && q.shadows_ok && ef_lt3(e.m_e, q.mint_e) == 0) return; /* certainly >= the current minimum */
    make_exact_warp(q, e, lane);
    if (e.m < q.mint) {
        q.mint = e.m;
        refresh_mint_shadow(q);
    }
}

/* d2 < d1 (C2A.cpp:1281) */
C2A_KDEV bool closer_second_w(const Query &q, WStackEntry &a, WStackEntry &c, int lane)
{
#if !C2A_WARP_FILTER /* every record is exact */
    return c.d < a.d;
#endif
    const int r = ef_lt3(c.d_e, a.d_e);
    if (r >= 0 && q.shadows_ok) return r == 1;
    make_exact_warp(q, a, lane);
    make_exact_warp(q, c, lane);
    return c.d < a.d;
}

/* a leaf pair of the rotation step (C2A.cpp:1141-1183) */
C2A_KDEV void leaf_step_warp(Query &q, int b1, int b2, int fc1, int fc2, int lane)
{
    const int ia = -fc1 - 1, ib = -fc2 - 1;
    q.ntri++;
    C2A_WSTAT(q, ST_W_LEAF, 1);
    if (C2A_WARP_FILTER && q.shadows_ok) { /* most leaves cannot reach the running distance */
        TriFeat fe;
        bool ok = false;
        const EF de = tri_distance_warp_e(q, ia, ib, fe, ok, lane);
        if (ok && ef_le3(de, q.distance_e) == 0) return;
    }
    V3 p, qq;
    TriFeat f;
    bool col = false;
    C2A_WSTAT(q, ST_W_LEAF_X, 1);
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
        refresh_shadows(q);
    }
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
            C2A_WCLOCK(l0);
            leaf_step_warp(q, b1, b2, fc1, fc2, lane);
            C2A_WCLOCK(l1);
            C2A_WSTAT(q, ST_W_CYC_LEAF, l1 - l0);
        } else {
            if (sp >= sh.cap) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return;
            }
            expand_warp(q, b1, b2, fc1, fc2, R, T, sh, lane);
            C2A_WCLOCK(k0);
            q.nbv += 2;
            WStackEntry &a = sh.child[0], &c = sh.child[1];
            const bool c_first = closer_second_w(q, a, c, lane);
            WStackEntry &first = c_first ? c : a;
            { /* the pending second child onto the stack, one 8-byte word per lane */
                const double *src = reinterpret_cast<const double *>(c_first ? &a : &c);
                if (lane < (int)(sizeof(WStackEntry) / 8)) reinterpret_cast<double *>(&sh.stack[sp])[lane] = src[lane];
            }
            sp++;
            if (descend_w(q, first, lane)) {
                b1 = first.b1;
                b2 = first.b2;
                R = first.R;
                T = first.T;
                go = true;
            } else {
                contribute_w(q, first, lane);
            }
            __syncwarp();
            C2A_WCLOCK(k1);
            C2A_WSTAT(q, ST_W_CYC_DECIDE, k1 - k0);
        }
        C2A_WCLOCK(p0);
        while (!go && sp > 0) {
            WStackEntry &e = sh.stack[--sp];
            if (descend_w(q, e, lane)) {
                b1 = e.b1;
                b2 = e.b2;
                R = e.R;
                T = e.T;
                go = true;
            } else {
                contribute_w(q, e, lane);
            }
        }
        __syncwarp();
        C2A_WCLOCK(p1);
        C2A_WSTAT(q, ST_W_CYC_DECIDE, p1 - p0);
        if (!go) return;
    }
}

/* the depth-first step traversal of the warp kernel */
struct WarpDfs {
    WarpShared &sh;
    C2A_KDEV void operator()(Query &q, const M3 &R, V3 T, int lane) const { toc_dfs_warp(q, R, T, sh, lane); }
};

/* C2A_TimeOfContactStep, rotation branch (C2A.cpp:1855-1931); dfs runs
 * TOCStepRecurse_Dis from the root pair */
template <class Dfs>
C2A_KDEV void toc_step_warp(Query &q, M3 &R1, V3 &T1, M3 &R2, V3 &T2, const Dfs &dfs, int lane)
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
    refresh_shadows(q);
    C2A_WCLOCK(d0);
    dfs(q, R, T, lane);
    C2A_WCLOCK(d1);
    C2A_WSTAT(q, ST_W_CYC_DFS, d1 - d0);
}

/* --------------------------------------------------- contact enumeration */

/* a leaf pair of the contact enumeration (C2A.cpp:1560-1630) */
C2A_KDEV bool contact_leaf_warp(Query &q, int fc1, int fc2, double threshold, int query_index, c2a_contact &c,
                                int lane)
{
    const int ia = -fc1 - 1, ib = -fc2 - 1;
    if (C2A_WARP_FILTER && q.shadows_ok) {
        EFCtx tc{false};
        const EF threshold_e = in_d(threshold, tc);
        TriFeat fe{-1, -1, -1, -1};
        bool ok = false;
        const EF de = tri_distance_warp_e(q, ia, ib, fe, ok, lane);
        if (ok && !tc.bad && fe.type_a != -1 && fe.type_b != -1 && ef_le3(de, threshold_e) == 0) return false;
    }
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

/* d < threshold (abs_err = rel_err = 0: both of the reference's clauses) */
C2A_KDEV bool contact_descend_w(const Query &q, WStackEntry &e, double threshold, int lane)
{
#if !C2A_WARP_FILTER /* every record is exact */
    return (e.d < (threshold - 0)) || (e.d * (1.0 + 0) < threshold);
#endif
    if (q.shadows_ok) {
        EFCtx tc{false};
        const EF te = in_d(threshold, tc);
        const int r = tc.bad ? -1 : ef_lt3(e.d_e, te);
        if (r >= 0) return r == 1;
    }
    make_exact_warp(q, e, lane);
    return (e.d < (threshold - 0)) || (e.d * (1.0 + 0) < threshold);
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
            if (sp >= sh.cap) {
                q.status |= C2A_QUERY_STACK_OVERFLOW;
                return count;
            }
            expand_warp(q, b1, b2, fc1, fc2, R, T, sh, lane);
            WStackEntry &a = sh.child[0], &c = sh.child[1];
            const bool c_first = closer_second_w(q, a, c, lane);
            WStackEntry &first = c_first ? c : a;
            { /* the pending second child onto the stack, one 8-byte word per lane */
                const double *src = reinterpret_cast<const double *>(c_first ? &a : &c);
                if (lane < (int)(sizeof(WStackEntry) / 8)) reinterpret_cast<double *>(&sh.stack[sp])[lane] = src[lane];
            }
            sp++;
            if (contact_descend_w(q, first, threshold, lane)) {
                b1 = first.b1;
                b2 = first.b2;
                R = first.R;
                T = first.T;
                go = true;
            }
            __syncwarp();
        }
        while (!go && sp > 0) {
            WStackEntry &e = sh.stack[--sp];
            if (contact_descend_w(q, e, threshold, lane)) {
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
 * translation-only step runs the sequential code on every lane; dfs runs
 * each rotation step's traversal. */
template <class Dfs>
C2A_KDEV void solve_query_warp(const c2a_query &in, const DevModel *models, int num_models, const c2a_params &prm,
                               c2a_result &out_g, c2a_contact *contacts, WarpShared &sh, Pending *tstack,
                               int query_index, int lane, const Dfs &dfs)
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
    Query &q = C2A_WARP_QUERY(sh); /* one copy per warp in shared memory, written with the same values by every lane */
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) q.st[i] = 0;
    for (int i = 0; i < ST_COUNT - ST_W_FIRST; i++) q.wst[i] = 0;
    C2A_WCLOCK(qc0);
#endif
    q.status = 0;
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    q.want_mint = true;
    q.rt = &sh.rt[0][0];
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
    else toc_step_warp(q, R1, T1, R2, T2, dfs, lane);
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
            toc_step_warp(q, R1, T1, R2, T2, dfs, lane);
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
            q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
            q.want_mint = false;
            const int n = contact_dfs_warp(q, R, T, threshold, sh, contacts, prm.contacts_per_query, query_index,
                                           lane);
            out.num_contact = n;
            if (n > prm.contacts_per_query) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
        }
    }
    out.status |= q.status;
    if (lane == 0) out_g = out;
#ifdef C2A_STATS
    C2A_WCLOCK(qc1);
    C2A_WSTAT(q, ST_W_CYC_QUERY, qc1 - qc0);
    if (lane == 0)
        for (int i = ST_W_FIRST; i < ST_COUNT; i++) atomicAdd(&g_c2a_stats[i], q.wst[i - ST_W_FIRST]);
#endif
}

} // namespace c2a
#endif
