/*
 * ca_front.cuh -- the CANONICAL CA query: one warp per query, node pairs in a
 * warp-shared front.
 *
 * In the reference, a CA step's result depends on the order of its depth-first
 * traversal: the running bound res->distance starts at the caller's seed pair
 * and shrinks as leaves are found (C2A.cpp:1141-1183), and pruned pairs add
 * their coarse mint (C2A.cpp:1290-1311).  The CANONICAL composition first
 * runs the reference's distance query (C2A_Distance with rel_err = abs_err = 0,
 * C2A/src/C2A_PQP.cpp:971-1056) from the seed and seeds the step with the
 * closest pair it returns.  The step's bound then starts at the exact minimum
 * distance d* and never moves (no leaf lies closer), so which pairs are
 * descended, the step's mint (a minimum) and its counters no longer depend
 * on the order the pairs are visited in.  That makes the step a parallel
 * front traversal:
 *
 *   distance phase  branch and bound for d* over a warp-shared stack: each
 *                   round the warp pops up to 32 pairs, prunes with certified
 *                   FP32 lower bounds of C2A_BV_Distance (plus a margin far
 *                   above FP64 rounding, so a pair that can hold the minimum
 *                   is never dropped), evaluates leaves exactly in FP64 when
 *                   their FP32 lower bound does not exclude them, and takes
 *                   the warp minimum (ties: the smallest triangle pair);
 *   step phase      TOCStepRecurse_Dis with res->distance = d* fixed: every
 *                   popped internal pair tests both children (FP32 filter,
 *                   FP64 where undecided), pushes the ones the reference
 *                   descends and folds the others' mint into a per-lane
 *                   minimum; leaves run the reference's leaf step;
 *   contacts        TOCStepRecurse_Dis_contact with its fixed threshold, the
 *                   found pairs compacted with ballot/popc, then sorted by
 *                   (tri_a, tri_b).
 *
 * Pushes of a round are compacted with a warp prefix sum; the stack lives in
 * a per-warp slice of global memory (cache-resident: a round touches the top
 * 32 entries).  The CA loop itself runs redundantly on all lanes with
 * identical values, so its FP64 work issues once per warp.
 */
#ifndef C2A_CA_FRONT_CUH
#define C2A_CA_FRONT_CUH

#include "ca_kernel.cuh"

namespace c2a {

constexpr unsigned kFullMask = 0xffffffffu;

/* entries of one warp's front; the translation-only step (run redundantly
 * with one private stack per lane) needs 32 * C2A_STACK_DEPTH of them */
#ifndef C2A_FRONT_CAP
#define C2A_FRONT_CAP 4096
#endif
static_assert(C2A_FRONT_CAP >= 32 * C2A_STACK_DEPTH, "front slice too small for the per-lane translation stacks");

C2A_KDEV double warp_min_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(kFullMask, v, o);
        v = (w < v) ? w : v;
    }
    return v;
}
C2A_KDEV long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    return v;
}
/* exclusive prefix sum of v over the warp; total receives the sum */
C2A_KDEV int warp_excl_scan(int v, int lane, int &total)
{
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(kFullMask, x, 31);
    return x - v;
}

/* certified FP32 lower bound of the FP64 C2A_BV_Distance of a child pair
 * (0 when the filter cannot certify one) */
C2A_KNOINL float bv_lower(const Query &q, int side, const M3T<EF> &PRe, V3T<EF> PTe, int x1, int x2)
{
    if (!q.shadows_ok) return 0.0f;
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
    if (c.bad) return 0.0f;
    const float lo = ef_rd_sub(z.v, z.e);
    return lo > 0.0f ? lo : 0.0f;
}

/* lower bound of a child pair's C2A_BV_Distance from its exact FP64 value
 * (when the FP32 filter is unusable for this query) */
C2A_KNOINL float bv_lower_exact(const Query &q, int side, const M3 &PR, V3 PT, int x1, int x2)
{
    M3 R;
    V3 T;
    child_transform(q, side, x1, x2, PR, PT, R, T);
    ExactCtx xc{false};
    NodeX n1, n2;
    load_x(n1, q.A->nodes + x1);
    load_x(n2, q.B->nodes + x2);
    V3 S = v3(0, 0, 0);
    double z = rect_dist(R, T, n1.l, n2.l, S, xc);
    z -= (n1.r + n2.r);
    const float lo = __double2float_rd(z);
    return lo > 0.0f ? lo : 0.0f;
}

/* certified FP32 lower bound of the FP64 TriDist of a leaf pair (0 when uncertified) */
C2A_KNOINL float tri_lower(const Query &q, int ia, int ib)
{
    if (!q.shadows_ok) return 0.0f;
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
    const EF d = tri_dist(p, qq, S, T, f, col, c);
    if (c.bad) return 0.0f;
    const float lo = ef_rd_sub(d.v, d.e);
    return lo > 0.0f ? lo : 0.0f;
}

/* the children of an internal pair (C2A.cpp:1192-1226): side 0 splits A's node */
C2A_KDEV void child_pairs(const Query &q, int b1, int b2, int fc1, int fc2, int &side, int &a1, int &a2, int &c1,
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

/* the pair's own exact transform */
C2A_KDEV void own_transform(const Query &q, const Pending &e, M3 &R, V3 &T)
{
    if (e.side < 0) {
        R = e.PR;
        T = e.PT;
    } else {
        child_transform(q, e.side, e.b1, e.b2, e.PR, e.PT, R, T);
    }
}

/* ------------------------------------------------------- seed descents */

/* a hinted node: its path from the root in the low 16 bits (bit k: which
 * child, 0 first_child, 1 first_child + 1, at depth k) and its depth above */
C2A_KDEV int hint_depth(uint32_t h) { return (int)(h >> 16); }

/* squared distance between the rectangle centres of a child pair, B's
 * rectangle placed by (R, T) in A's frame (a descent heuristic only) */
C2A_KDEV double rect_centre_dist2(const Query &q, const M3 &R, V3 T, int x1, int x2)
{
    const NodeRec *n1 = q.A->nodes + x1, *n2 = q.B->nodes + x2;
    const V3 ca = v3(0.5 * __ldg(&n1->l[0]), 0.5 * __ldg(&n1->l[1]), 0.0);
    const V3 cb = mul(R, v3(0.5 * __ldg(&n2->l[0]), 0.5 * __ldg(&n2->l[1]), 0.0)) + T;
    const V3 d = cb - ca;
    return dot(d, d);
}

/* one descent from the root pair (placed by R, T) to a leaf pair: while the
 * model being split is above its hinted node (ha for A, hb for B; depth 0:
 * no hint) it follows the hint's path, otherwise the child pair with the
 * smaller certified lower bound is taken (while both RSS pairs overlap, the
 * one with the closer rectangle centres).  Returns the leaf pair's exact
 * distance (C2A_TriDistance) and its triangles in ta, tb; an upper bound of
 * the closest-pair distance, so any descent may seed the search. */
C2A_KDEV double descend_to_leaf(const Query &q, const M3 &Rroot, V3 Troot, uint32_t ha, uint32_t hb, int &ta,
                                int &tb)
{
    int b1 = 0, b2 = 0, da = 0, db = 0;
    M3 Rc = Rroot;
    V3 Tc = Troot;
    for (int step = 0; step < 4 * C2A_STACK_DEPTH; step++) {
        const int fc1 = __ldg(&q.A->nodes[b1].first_child), fc2 = __ldg(&q.B->nodes[b2].first_child);
        if (fc1 < 0 && fc2 < 0) {
            ta = -fc1 - 1;
            tb = -fc2 - 1;
            V3 p, qq;
            TriFeat f;
            bool col = false;
            return tri_distance_x(q, ta, tb, p, qq, f, col);
        }
        int side, a1, a2, c1, c2;
        child_pairs(q, b1, b2, fc1, fc2, side, a1, a2, c1, c2);
        const int dpt = side == 0 ? da : db;
        const uint32_t h = side == 0 ? ha : hb;
        M3 Ra, Rcc;
        V3 Ta, Tcc;
        child_transform(q, side, a1, a2, Rc, Tc, Ra, Ta);
        child_transform(q, side, c1, c2, Rc, Tc, Rcc, Tcc);
        bool take_c;
        if (dpt < hint_depth(h)) {
            take_c = ((h >> dpt) & 1u) != 0;
        } else {
            float la, lc;
            EFCtx ec{false};
            const M3T<EF> Re = ef_m3(Rc, ec);
            const V3T<EF> Te = ef_v3(Tc, ec);
            if (q.shadows_ok && !ec.bad) {
                la = bv_lower(q, side, Re, Te, a1, a2);
                lc = bv_lower(q, side, Re, Te, c1, c2);
            } else {
                la = bv_lower_exact(q, side, Rc, Tc, a1, a2);
                lc = bv_lower_exact(q, side, Rc, Tc, c1, c2);
            }
            take_c = lc < la;
            if (lc == la) take_c = rect_centre_dist2(q, Rcc, Tcc, c1, c2) < rect_centre_dist2(q, Ra, Ta, a1, a2);
        }
        if (side == 0) da++;
        else db++;
        if (take_c) {
            b1 = c1;
            b2 = c2;
            Rc = Rcc;
            Tc = Tcc;
        } else {
            b1 = a1;
            b2 = a2;
            Rc = Ra;
            Tc = Ta;
        }
    }
    ta = tb = -1;
    return __longlong_as_double(0x7ff0000000000000LL);
}

/* the warp's smallest (d, a, b), exact ties to the smallest pair */
C2A_KDEV void warp_min_pair(double &d, int &a, int &b)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double d2 = __shfl_xor_sync(kFullMask, d, o);
        const int a2 = __shfl_xor_sync(kFullMask, a, o), b2 = __shfl_xor_sync(kFullMask, b, o);
        if (d2 < d || (d2 == d && (a2 < a || (a2 == a && b2 < b)))) {
            d = d2;
            a = a2;
            b = b2;
        }
    }
}

/* the seed of a closest-pair search: (best, ba, bb) becomes the smallest of
 * itself and the descents run on lanes 0..nd-1 (lane 0 greedy, lane l > 0
 * towards hinted pair l - 1), keeping distance and pair together */
C2A_KDEV void seed_descents(const Query &q, const M3 &R, V3 T, const uint32_t *hints, int nd, int lane,
                            double &best, int &ba, int &bb)
{
    double dl = __longlong_as_double(0x7ff0000000000000LL);
    int la = 0x7fffffff, lb = 0x7fffffff;
    if (lane < nd) {
        int ta = -1, tb = -1;
        const double d = descend_to_leaf(q, R, T, lane ? hints[2 * (lane - 1)] : 0u,
                                         lane ? hints[2 * (lane - 1) + 1] : 0u, ta, tb);
        if (ta >= 0) {
            dl = d;
            la = ta;
            lb = tb;
        }
    }
    warp_min_pair(dl, la, lb);
    if (dl < best || (dl == best && (la < ba || (la == ba && lb < bb)))) {
        best = dl;
        ba = la;
        bb = lb;
    }
}

C2A_KDEV Pending root_entry(const M3 &R, V3 T)
{
    Pending r;
    r.b1 = 0;
    r.b2 = 0;
    r.side = -1;
    r.exact = 1;
    r.d = ef_exact(0);
    r.m = ef_exact(0);
    r.d_x = r.m_x = 0.0;
    r.PR = R;
    r.PT = T;
    return r;
}

/* writes a round's pushes (0-2 per lane) above base; false when the slice is full */
C2A_KDEV bool push_round(Pending *stack, int cap, int base, int lane, int npush, const Pending &p0, const Pending &p1,
                         int &sp)
{
    int total;
    const int off = warp_excl_scan(npush, lane, total);
    if (base + total > cap) return false;
    if (npush > 0) stack[base + off] = p0;
    if (npush > 1) stack[base + off + 1] = p1;
    sp = base + total;
    __syncwarp();
    return true;
}

/* ---------------------------------------------------- distance phase */

/* closest triangle pair: best/ba/bb enter as the seed pair's exact distance
 * and indices and leave as the minimum over all pairs (ties: smallest pair) */
C2A_KDEV void warp_distance(Query &q, const M3 &Rroot, V3 Troot, Pending *stack, int cap, int lane, double &best,
                            int &ba, int &bb)
{
    const double margin = 1e-10 * (__ldg(&q.A->nodes[0].size) + __ldg(&q.B->nodes[0].size));
    if (lane == 0) stack[0] = root_entry(Rroot, Troot);
    __syncwarp();
#ifdef C2A_STATS
    const long long t0 = clock64();
#endif
    int sp = 1;
    while (sp > 0) {
        if (lane == 0) C2A_STAT(q, ST_D_ROUNDS);
        const int k = sp < 32 ? sp : 32;
        const int base = sp - k;
        Pending e;
        const bool have = lane < k;
        if (have) e = stack[base + lane];
        __syncwarp();
        double cand = __longlong_as_double(0x7ff0000000000000LL); /* +inf */
        int ca = 0x7fffffff, cb = 0x7fffffff;
        int npush = 0;
        Pending p0, p1;
        if (have && !((double)e.d.v > best + margin)) {
            C2A_STAT(q, ST_D_POPS);
            const int fc1 = __ldg(&q.A->nodes[e.b1].first_child), fc2 = __ldg(&q.B->nodes[e.b2].first_child);
            if (fc1 < 0 && fc2 < 0) {
                const int ia = -fc1 - 1, ib = -fc2 - 1;
                const float tl = tri_lower(q, ia, ib), ll = tl > e.d.v ? tl : e.d.v; /* or the leaf RSS bound */
                if ((double)ll <= best + margin) {
                    C2A_STAT(q, ST_D_LEAF_EXACT);
                    V3 p, qq;
                    TriFeat f;
                    bool col = false;
                    cand = tri_distance_x(q, ia, ib, p, qq, f, col);
                    ca = ia;
                    cb = ib;
                }
            } else {
                M3 R;
                V3 T;
                own_transform(q, e, R, T);
                int side, a1, a2, c1, c2;
                child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, c1, c2);
                EFCtx ec{false};
                const M3T<EF> Re = ef_m3(R, ec);
                const V3T<EF> Te = ef_v3(T, ec);
                float la, lc;
                if (q.shadows_ok && !ec.bad) {
                    la = bv_lower(q, side, Re, Te, a1, a2);
                    lc = bv_lower(q, side, Re, Te, c1, c2);
                } else {
                    la = bv_lower_exact(q, side, R, T, a1, a2);
                    lc = bv_lower_exact(q, side, R, T, c1, c2);
                }
                const bool pa = !((double)la > best + margin), pc = !((double)lc > best + margin);
                Pending a, c;
                a.b1 = a1; a.b2 = a2; c.b1 = c1; c.b2 = c2;
                a.side = c.side = side;
                a.exact = c.exact = 0;
                a.d = EF{la, 0.0f};
                c.d = EF{lc, 0.0f};
                a.PR = c.PR = R;
                a.PT = c.PT = T;
                /* the closer pair goes on top so that it is popped first */
                if (pa && pc) {
                    if (lc < la) { p0 = a; p1 = c; }
                    else { p0 = c; p1 = a; }
                    npush = 2;
                } else if (pa) {
                    p0 = a;
                    npush = 1;
                } else if (pc) {
                    p0 = c;
                    npush = 1;
                }
            }
        }
        if (!push_round(stack, cap, base, lane, npush, p0, p1, sp)) {
            q.status |= C2A_QUERY_STACK_OVERFLOW;
            return;
        }
        /* warp minimum of the round's candidates, ties to the smallest pair */
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double d2 = __shfl_xor_sync(kFullMask, cand, o);
            const int a2 = __shfl_xor_sync(kFullMask, ca, o), b2 = __shfl_xor_sync(kFullMask, cb, o);
            if (d2 < cand || (d2 == cand && (a2 < ca || (a2 == ca && b2 < cb)))) {
                cand = d2;
                ca = a2;
                cb = b2;
            }
        }
        if (cand < best || (cand == best && (ca < ba || (ca == ba && cb < bb)))) {
            best = cand;
            ba = ca;
            bb = cb;
        }
    }
#ifdef C2A_STATS
    if (lane == 0) q.st[ST_D_KCYC] += (unsigned)((clock64() - t0) >> 10);
#endif
}

/* -------------------------------------------------------- step phase */

/* TOCStepRecurse_Dis with res->distance fixed at d*: q.mint is a per-lane
 * minimum and the counters per-lane sums until the caller reduces them */
C2A_KDEV void warp_traverse(Query &q, const M3 &Rroot, V3 Troot, Pending *stack, int cap, int lane)
{
    if (lane == 0) stack[0] = root_entry(Rroot, Troot);
    __syncwarp();
#ifdef C2A_STATS
    const long long t0 = clock64();
#endif
    int sp = 1;
    while (sp > 0) {
        if (lane == 0) C2A_STAT(q, ST_T_ROUNDS);
        const int k = sp < 32 ? sp : 32;
        const int base = sp - k;
        Pending e;
        const bool have = lane < k;
        if (have) e = stack[base + lane];
        __syncwarp();
        int npush = 0;
        Pending p0, p1;
        if (have) {
            C2A_STAT(q, ST_T_POPS);
            const int fc1 = __ldg(&q.A->nodes[e.b1].first_child), fc2 = __ldg(&q.B->nodes[e.b2].first_child);
            if (fc1 < 0 && fc2 < 0) {
                leaf_step(q, e.b1, e.b2);
            } else {
                M3 R;
                V3 T;
                own_transform(q, e, R, T);
                int side, a1, a2, c1, c2;
                child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, c1, c2);
                Pending a, c;
                a.b1 = a1; a.b2 = a2; c.b1 = c1; c.b2 = c2;
                a.side = c.side = side;
                a.exact = c.exact = 0;
                a.PR = c.PR = R;
                a.PT = c.PT = T;
                EFCtx ec{false};
                const M3T<EF> Re = ef_m3(R, ec);
                const V3T<EF> Te = ef_v3(T, ec);
                bool zero_a = false, zero_c = false;
                const bool ok_a = !ec.bad && bv_test_e(q, side, Re, Te, a1, a2, a.d, a.m, zero_a);
                const bool ok_c = !ec.bad && bv_test_e(q, side, Re, Te, c1, c2, c.d, c.m, zero_c);
                if (!ok_a) make_exact(q, a);
                else if (zero_a) { a.exact = 1; a.d_x = 0.0; a.m_x = 0.0; }
                if (!ok_c) make_exact(q, c);
                else if (zero_c) { c.exact = 1; c.d_x = 0.0; c.m_x = 0.0; }
                q.nbv += 2;
                if (descend(q, a)) p0 = a, npush = 1;
                else contribute(q, a);
                if (descend(q, c)) {
                    if (npush) p1 = c;
                    else p0 = c;
                    npush++;
                } else {
                    contribute(q, c);
                }
            }
        }
        if (!push_round(stack, cap, base, lane, npush, p0, p1, sp)) {
            q.status |= C2A_QUERY_STACK_OVERFLOW;
            return;
        }
    }
#ifdef C2A_STATS
    if (lane == 0) q.st[ST_T_KCYC] += (unsigned)((clock64() - t0) >> 10);
#endif
}

/* ------------------------------------------------------------ one step */

/* C2A_Distance, then C2A_TimeOfContactStep seeded with the closest pair.
 * The search's first bound is the seed pair's distance, tightened by a
 * greedy descent (lane 0) and, at the first step, by descents towards the
 * hinted cluster pairs (lanes 1..nh); none of these changes the result. */
C2A_KDEV void canonical_step(Query &q, M3 &R1, V3 &T1, M3 &R2, V3 &T2, bool translation, Pending *stack, int cap,
                             int lane, const uint32_t *hints = nullptr, int nh = 0)
{
    if (translation) { /* the reference's translation step, one private stack per lane */
        toc_step(q, R1, T1, R2, T2, true, stack + lane * C2A_STACK_DEPTH);
        return;
    }
    M3 R;
    V3 T;
    relative_transforms(q, R1, T1, R2, T2, R, T);
    /* the distance phase's FP32 bounds need only the transforms and the node shadows */
    q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
    double best;
    {
        V3 p, qq;
        TriFeat f;
        bool col = false;
        best = tri_distance_x(q, q.seed_a, q.seed_b, p, qq, f, col);
    }
    int ba = q.seed_a, bb = q.seed_b;
    seed_descents(q, R, T, hints, 1 + ((q.numCA == 0 && hints) ? nh : 0), lane, best, ba, bb);
    warp_distance(q, R, T, stack, cap, lane, best, ba, bb);
    if (q.status) return;
    q.seed_a = ba;
    q.seed_b = bb;
    q.distance = best; /* C2A_TriDistance of the new seed pair */
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
    const long long nbv0 = q.nbv, ntri0 = q.ntri;
    warp_traverse(q, R, T, stack, cap, lane);
    q.mint = warp_min_d(q.mint);
    q.nbv = nbv0 + warp_sum_ll(q.nbv - nbv0);
    q.ntri = ntri0 + warp_sum_ll(q.ntri - ntri0);
    q.distance = best;
    q.status = __reduce_or_sync(kFullMask, (unsigned)q.status);
}

/* ----------------------------------------------------------- contacts */

/* TOCStepRecurse_Dis_contact with a fixed threshold; returns the number of
 * pairs found, stores the first slots of them, sorted by (tri_a, tri_b) */
C2A_KDEV int warp_contacts(Query &q, const M3 &Rroot, V3 Troot, double threshold, Pending *stack, int cap, int lane,
                           c2a_contact *out, int slots, int query_index)
{
    EFCtx tc{false};
    const EF threshold_e = in_d(threshold, tc);
    if (tc.bad) q.shadows_ok = false;
    if (lane == 0) stack[0] = root_entry(Rroot, Troot);
    __syncwarp();
    int sp = 1, count = 0;
    while (sp > 0) {
        const int k = sp < 32 ? sp : 32;
        const int base = sp - k;
        Pending e;
        const bool have = lane < k;
        if (have) e = stack[base + lane];
        __syncwarp();
        int npush = 0;
        Pending p0, p1;
        bool emit = false;
        c2a_contact ct;
        if (have) {
            const int fc1 = __ldg(&q.A->nodes[e.b1].first_child), fc2 = __ldg(&q.B->nodes[e.b2].first_child);
            if (fc1 < 0 && fc2 < 0) {
                emit = contact_leaf_test(q, e.b1, e.b2, threshold, threshold_e, query_index, ct);
            } else {
                M3 R;
                V3 T;
                own_transform(q, e, R, T);
                int side, a1, a2, c1, c2;
                child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, c1, c2);
                Pending a, c;
                a.b1 = a1; a.b2 = a2; c.b1 = c1; c.b2 = c2;
                a.side = c.side = side;
                a.exact = c.exact = 0;
                a.PR = c.PR = R;
                a.PT = c.PT = T;
                EFCtx ec{false};
                const M3T<EF> Re = ef_m3(R, ec);
                const V3T<EF> Te = ef_v3(T, ec);
                bool zero_a = false, zero_c = false;
                const bool ok_a = !ec.bad && bv_test_e(q, side, Re, Te, a1, a2, a.d, a.m, zero_a);
                const bool ok_c = !ec.bad && bv_test_e(q, side, Re, Te, c1, c2, c.d, c.m, zero_c);
                if (!ok_a) make_exact(q, a);
                else if (zero_a) { a.exact = 1; a.d_x = 0.0; a.m_x = 0.0; }
                if (!ok_c) make_exact(q, c);
                else if (zero_c) { c.exact = 1; c.d_x = 0.0; c.m_x = 0.0; }
                if (contact_descend(q, a, threshold, threshold_e)) p0 = a, npush = 1;
                if (contact_descend(q, c, threshold, threshold_e)) {
                    if (npush) p1 = c;
                    else p0 = c;
                    npush++;
                }
            }
        }
        const unsigned m = __ballot_sync(kFullMask, emit);
        const int slot = count + __popc(m & ((1u << lane) - 1u));
        if (emit && out && slot < slots) out[slot] = ct;
        count += __popc(m);
        if (!push_round(stack, cap, base, lane, npush, p0, p1, sp)) {
            q.status |= C2A_QUERY_STACK_OVERFLOW;
            break;
        }
    }
    /* canonical order: rank by (tri_a, tri_b) (unique per query), then
     * follow the permutation's cycles */
    const int n = count < slots ? count : slots;
    if (out && n > 1) {
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            const int ka = out[i].tri_a, kb = out[i].tri_b;
            int r = 0;
            for (int j = 0; j < n; j++) {
                const int ja = out[j].tri_a, jb = out[j].tri_b;
                r += (ja < ka || (ja == ka && jb < kb)) ? 1 : 0;
            }
            out[i].pad = r;
        }
        __syncwarp();
        if (lane == 0) {
            for (int i = 0; i < n; i++) {
                int guard = n;
                while (out[i].pad != i && guard-- > 0) {
                    const int j = out[i].pad;
                    const c2a_contact t = out[j];
                    out[j] = out[i];
                    out[i] = t;
                }
            }
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) out[i].pad = 0;
        __syncwarp();
    }
    return count;
}

/* ------------------------------------------------------------ one query */

/* the C2A_Solve body of the CANONICAL composition on one warp; lane 0 writes
 * the result */
/* C2A_Distance with rel_err = abs_err = 0 (C2A/src/C2A_PQP.cpp:970-1056) for one
 * pair: model a at pose[0..11], model b at pose[24..35], seeded with the
 * query's triangle pair */
C2A_KDEV void distance_query_warp(const c2a_query &in, const DevModel *models, int num_models,
                                  c2a_distance_result &out_g, Pending *stack, int cap, int lane)
{
    c2a_distance_result out;
    memset(&out, 0, sizeof(out));
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
    q.e_ok = true;
    q.nbv = q.ntri = 0;
    const double *P = in.pose;
    const M3 R1 = pose_R(P), R2 = pose_R(P + 24);
    const V3 T1 = pose_T(P), T2 = pose_T(P + 24);
    M3 R;
    V3 T;
    relative_transforms(q, R1, T1, R2, T2, R, T); /* res->R, res->T and the root pair (C2A_PQP.cpp:990-1033) */
    q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
    V3 p, qq;
    TriFeat f;
    bool col = false;
    double best = tri_distance_x(q, in.seed_a, in.seed_b, p, qq, f, col);
    int ba = in.seed_a, bb = in.seed_b;
    seed_descents(q, R, T, nullptr, 1, lane, best, ba, bb); /* a greedy descent may tighten the first bound */
    warp_distance(q, R, T, stack, cap, lane, best, ba, bb);
    tri_distance_x(q, ba, bb, p, qq, f, col); /* the closest pair's points, as its TriDistance left them */
    out.distance = best;
    out.p1[0] = p.x; out.p1[1] = p.y; out.p1[2] = p.z;
    const V3 u = qq - q.Tm; /* res->p2 back into model b's frame (C2A_PQP.cpp:1046-1048) */
    const V3 p2 = tmul(q.Rm, u);
    out.p2[0] = p2.x; out.p2[1] = p2.y; out.p2[2] = p2.z;
    out.tri_a = ba;
    out.tri_b = bb;
    out.status = q.status;
    if (lane == 0) out_g = out;
}

C2A_KDEV void solve_query_canonical(const c2a_query &in, const DevModel *models, int num_models,
                                    const c2a_params &prm, c2a_result &out_g, c2a_contact *contacts, Pending *stack,
                                    int cap, int lane, int query_index, const uint32_t *hints = nullptr,
                                    int nh = 0)
{
    c2a_result out;
    memset(&out, 0, sizeof(out));
#ifdef C2A_STATS
    const long long tq0 = clock64();
#endif
    out.status = C2A_QUERY_OK;
    out.contact_offset = query_index * prm.contacts_per_query;
    Query q;
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) q.st[i] = 0;
#endif
    q.status = 0;
    const bool bad_models = in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 ||
                            in.model_b >= num_models || !(models[in.model_a].flags & C2A_MODEL_LIVE) ||
                            !(models[in.model_b].flags & C2A_MODEL_LIVE);
    if (bad_models || in.seed_a < 0 || in.seed_a >= models[in.model_a].num_tris || in.seed_b < 0 ||
        in.seed_b >= models[in.model_b].num_tris) {
        out.status = C2A_QUERY_BAD_INPUT;
        if (lane == 0) out_g = out;
        return;
    }
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
    canonical_step(q, R1, T1, R2, T2, translation, stack, cap, lane, hints, nh);
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
            canonical_step(q, R1, T1, R2, T2, false, stack, cap, lane);
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
#ifdef C2A_STATS
            const long long tc0 = clock64();
#endif
            const int n = warp_contacts(q, R, T, threshold, stack, cap, lane, contacts, prm.contacts_per_query,
                                        query_index);
            out.num_contact = n;
            if (n > prm.contacts_per_query) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
#ifdef C2A_STATS
            if (lane == 0) q.st[ST_C_KCYC] += (unsigned)((clock64() - tc0) >> 10);
#endif
        }
    }
    out.status |= __reduce_or_sync(kFullMask, (unsigned)q.status);
#ifdef C2A_STATS
    if (lane == 0) q.st[ST_Q_KCYC] += (unsigned)((clock64() - tq0) >> 10);
#endif
#ifdef C2A_STATS
    for (int i = 0; i < ST_COUNT; i++) atomicAdd(&g_c2a_stats[i], (unsigned long long)q.st[i]);
#endif
    if (lane == 0) out_g = out;
}

} // namespace c2a
#endif
