/*
 * c2a_wave.cu -- the batched (wavefront) engine of the CANONICAL mode.
 *
 * Per CA iteration of every active query, in lockstep:
 *
 *   step_begin   relative transforms, the seed pair's exact distance and a
 *                greedy descent (the closer child pair by FP32 lower bound
 *                down to a leaf, whose exact distance tightens the bound);
 *   dwave*       the closest-pair search (C2A_Distance, rel_err = abs_err = 0)
 *                as breadth-first waves: an item is dropped when its
 *                certified lower bound exceeds the query's bound ub (plus a
 *                margin far above FP64 rounding), leaves shrink ub with their
 *                certified FP32 upper bounds and become candidates;
 *   dcand, dtie  candidates that can still be the minimum are evaluated
 *                exactly in FP64; the minimum and, among exact ties, the
 *                smallest triangle pair seed the step;
 *   tbegin       the controlled error schedule (C2A.cpp:1869-1891);
 *   twave*       TOCStepRecurse_Dis with res->distance fixed at d*: pairs the
 *                reference descends become the next wave's items, the mint of
 *                pruned pairs goes to an atomic minimum over exact FP64 values
 *                (deferred when the FP32 bounds cannot rule it out), leaves that
 *                may reach d* are deferred;
 *   tdefer/tleaf the deferred exact evaluations;
 *   ca           one iteration of C2A_QueryTimeOfContact's loop
 *                (C2A.cpp:2060-2146) and the compaction of the active list.
 *
 * After the last iteration, the contact enumeration at the TOC
 * (TOCStepRecurse_Dis_contact, fixed threshold) runs as waves over the
 * colliding queries, and each query's contacts are sorted by (tri_a, tri_b).
 * Translation-only queries (both |w| < 1e-8) run the reference's translation
 * CA in the init kernel, as the canonical composition does.
 *
 * Every kernel is one pass over a list; the host reads the next list's
 * length after each wave.  Buffer overflow sets a flag; the host then grows
 * the buffers and reruns the batch from the start.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "device/ca_front.cuh"
#include "wave_engine.h"

namespace c2a {

namespace {

constexpr int kWThreads = 128;

/* one (query, node pair) item; PR/PT: the exact transform of the pair's
 * parent (or of the pair itself for a root, side < 0) */
struct WItem {
    int32_t q, b1, b2, side;
    float lo;
    int32_t pad;
    M3 PR;
    V3 PT;
};
static_assert(sizeof(WItem) == 120, "wave item must stay 120 bytes");

struct WCand { /* a leaf pair that may hold the minimum distance */
    int32_t q, ia, ib;
    float lo;
    double d;
};
struct WDefer { /* a pruned child pair whose mint may be the minimum */
    int32_t q, b1, b2, side;
    float lo;
    int32_t parent; /* arena index of the expanded pair */
};
struct WLeaf { /* a leaf pair of the step that may reach d* */
    int32_t q, b1, b2, pad;
};

/* an entry of a warp's closest-pair search: the pair, its certified lower
 * bound and the FP32 shadow (with bounds) of its own transform */
struct DEntry {
    int32_t b1, b2;
    float lo;
    int32_t pad;
    M3T<EF> R;
    V3T<EF> T;
};
static_assert(sizeof(DEntry) == 112, "search entry must stay 112 bytes");
constexpr int kDCap = 4096; /* entries of one warp's search stack */
constexpr int kCCap = 8192; /* candidate leaves one search warp holds before filtering */
struct DCand {
    int32_t ia, ib;
    float lo;
    int32_t pad;
};

/* keeps the buffer's candidates whose lower bound does not exceed ub + margin
 * (warp-cooperative, order preserved); returns the new count */
C2A_KDEV int filter_cands(DCand *buf, int nc, float ub, double margin, int lane)
{
    int out = 0;
    for (int base = 0; base < nc; base += 32) {
        const int i = base + lane;
        DCand c;
        bool keep = false;
        if (i < nc) {
            c = buf[i];
            keep = !((double)c.lo > (double)ub + margin);
        }
        __syncwarp();
        const unsigned m = __ballot_sync(kFullMask, keep);
        if (keep) buf[out + __popc(m & ((1u << lane) - 1u))] = c;
        out += __popc(m);
        __syncwarp();
    }
    return out;
}

/* the CA loop of one query between iterations */
struct WLoop {
    M3 R1, R2;
    V3 T1, T2;
    double lamda, lastLamda, dlamda, toc, threshold;
    int32_t nItrs, first, collisionfree, contact; /* contact: enumerate at the TOC */
};

/* per-query accumulators of the current iteration */
struct WAcc {
    unsigned long long best_bits, pair_key, mint_bits, nbv, ntri;
    unsigned int ub_bits, U_bits;
    int32_t contacts, pad;
};

struct Lists {
    WItem *item[2];
    WItem *arena;
    WCand *cand;
    WDefer *defer;
    WLeaf *leaf;
    int32_t *active[2];
    DEntry *dstack; /* kDCap entries per search warp */
    DCand *dcand;   /* kCCap candidates per search warp */
    /* device counters: 0 next items, 1 arena end, 2 cand, 3 defer, 4 leaf, 5 next active, 6 overflow,
     * 7 search work counter */
    int32_t *cnt;
    int64_t cap_item, cap_arena, cap_cand, cap_defer, cap_leaf;
};

C2A_KDEV bool is_leaf_pair(const Query &q, int b1, int b2, int &fc1, int &fc2)
{
    fc1 = __ldg(&q.A->nodes[b1].first_child);
    fc2 = __ldg(&q.B->nodes[b2].first_child);
    return fc1 < 0 && fc2 < 0;
}

C2A_KDEV double dmargin(const Query &q)
{
    return 1e-10 * (__ldg(&q.A->nodes[0].size) + __ldg(&q.B->nodes[0].size));
}

C2A_KDEV float ru_float(double x) { return __double2float_ru(x); }

/* warp-aggregated append of n (0..2) entries to a list (any set of active
 * lanes); returns the first index, or -1 when the list is full (the overflow
 * flag is raised) */
C2A_KDEV int64_t append(int32_t *counter, int n, int64_t cap, int32_t *overflow, int which)
{
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned b1 = __ballot_sync(mask, n >= 1), b2 = __ballot_sync(mask, n >= 2);
    const int total = __popc(b1) + __popc(b2);
    const int prefix = __popc(b1 & lt) + __popc(b2 & lt);
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader && total > 0) base = atomicAdd(counter, total);
    base = __shfl_sync(mask, base, leader);
    const int64_t first = (int64_t)base + prefix;
    if (n > 0 && first + n > cap) {
        atomicOr(overflow, 1 << which);
        return -1;
    }
    return first;
}

/* ------------------------------------------------------------- kernels */

__global__ void __launch_bounds__(kWThreads) k_init(const c2a_query *__restrict__ queries, int n,
                                                    const DevModel *__restrict__ models, int num_models,
                                                    c2a_params prm, c2a_result *__restrict__ results,
                                                    c2a_contact *__restrict__ contacts, Query *__restrict__ qs,
                                                    WLoop *__restrict__ loops, Lists L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const c2a_query &in = queries[i];
    c2a_result &out = results[i];
    Query &q = qs[i];
    const bool bad_models = in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 ||
                            in.model_b >= num_models || !(models[in.model_a].flags & C2A_MODEL_LIVE) ||
                            !(models[in.model_b].flags & C2A_MODEL_LIVE);
    if (bad_models || in.seed_a < 0 || in.seed_a >= models[in.model_a].num_tris || in.seed_b < 0 ||
        in.seed_b >= models[in.model_b].num_tris) {
        memset(&out, 0, sizeof(out));
        out.status = C2A_QUERY_BAD_INPUT;
        out.contact_offset = i * prm.contacts_per_query;
        return;
    }
    const double *P = in.pose;
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    set_motions(q, P);
    if (q.m1.angVel < 1e-8 && q.m2.angVel < 1e-8) {
        /* translation-only CA: the reference's step, sequential */
        Pending stack[C2A_STACK_DEPTH];
        c2a_contact *cq = contacts ? contacts + (size_t)i * (size_t)prm.contacts_per_query : nullptr;
        solve_query(in, models, num_models, prm, out, cq, stack, i);
        /* canonical contact order: by triangle pair */
        const int m = cq ? (out.num_contact < prm.contacts_per_query ? out.num_contact : prm.contacts_per_query) : 0;
        for (int a = 1; a < m; a++) {
            const c2a_contact key = cq[a];
            int b = a - 1;
            while (b >= 0 && (cq[b].tri_a > key.tri_a || (cq[b].tri_a == key.tri_a && cq[b].tri_b > key.tri_b))) {
                cq[b + 1] = cq[b];
                b--;
            }
            cq[b + 1] = key;
        }
        return;
    }
#ifdef C2A_STATS
    for (int k = 0; k < ST_COUNT; k++) q.st[k] = 0;
#endif
    q.status = 0;
    q.want_mint = true;
    q.toc_delta = prm.toc_delta;
    q.seed_a = in.seed_a;
    q.seed_b = in.seed_b;
    q.nbv = q.ntri = 0;
    q.upbound = 1;
    q.numCA = 0;
    q.mint = 1;
    q.distance = 0;
    q.abs_err = q.rel_err = 0;
    WLoop &lp = loops[i];
    lp.R1 = pose_R(P);
    lp.R2 = pose_R(P + 24);
    lp.T1 = pose_T(P);
    lp.T2 = pose_T(P + 24);
    set_pose1(q, lp.R1, lp.T1);
    lp.lamda = lp.lastLamda = lp.dlamda = lp.toc = 0.0;
    lp.nItrs = 0;
    lp.first = 1;
    lp.collisionfree = 0;
    lp.contact = 0;
    const int64_t at = append(L.cnt + 5, 1, (int64_t)n, L.cnt + 6, 5);
    if (at >= 0) L.active[0][at] = i;
}

/* transforms, the seed's exact distance, a greedy descent, the root item */
__global__ void __launch_bounds__(kWThreads) k_step_begin(const int32_t *__restrict__ active, int na,
                                                          Query *__restrict__ qs, WLoop *__restrict__ loops,
                                                          WAcc *__restrict__ acc, Lists L, int out,
                                                          const uint32_t *__restrict__ hints, int nh)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int push = 0;
    int qi = -1;
    M3 R;
    V3 T;
    if (k < na) {
        qi = active[k];
        Query &q = qs[qi];
        WLoop &lp = loops[qi];
        relative_transforms(q, lp.R1, lp.T1, lp.R2, lp.T2, R, T);
        q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
        V3 p, qq;
        TriFeat f;
        bool col = false;
        double best = tri_distance_x(q, q.seed_a, q.seed_b, p, qq, f, col);
        /* a greedy descent and, at the first step, the hinted descents tighten the bound */
        const int use = (q.numCA == 0 && hints) ? nh : 0;
        for (int h = -1; h < use; h++) {
            int ta, tb;
            const double d = descend_to_leaf(q, R, T, h < 0 ? 0u : hints[(size_t)qi * nh * 2 + 2 * h],
                                             h < 0 ? 0u : hints[(size_t)qi * nh * 2 + 2 * h + 1], ta, tb);
            if (ta >= 0 && d < best) best = d;
        }
        WAcc &a = acc[qi];
        a.best_bits = (unsigned long long)__double_as_longlong(best);
        a.pair_key = ~0ull;
        a.ub_bits = __float_as_uint(ru_float(best));
        a.mint_bits = (unsigned long long)__double_as_longlong(1.0);
        a.U_bits = __float_as_uint(1.0f);
        a.nbv = a.ntri = 0;
        push = q.shadows_ok ? 0 : 1; /* with shadows, the warp search of k_dsearch */
    }
    const int64_t at = append(L.cnt + 0, push, L.cap_item, L.cnt + 6, 0);
    if (push && at >= 0) {
        WItem &it = L.item[out][at];
        it.q = qi;
        it.b1 = it.b2 = 0;
        it.side = -1;
        it.lo = 0.0f;
        it.pad = 0;
        it.PR = R;
        it.PT = T;
    }
}

/* a child pair's certified lower bound and FP32-shadowed transform, from
 * its parent's shadowed transform (the reference's child formulas) */
C2A_KDEV float child_lower_e(const Query &q, int side, const M3T<EF> &PR, V3T<EF> PT, int x1, int x2, M3T<EF> &R,
                             V3T<EF> &T)
{
    EFCtx c{false};
    NodeE n1, n2;
    load_e(n1, q.A->snodes + x1);
    load_e(n2, q.B->snodes + x2);
    if (side == 0) {
        R = tmmul(n1.R, PR);
        T = tmul(n1.R, PT - n1.Tr);
    } else {
        R = mmul(PR, n2.R);
        T = mul_add(PR, n2.Tr, PT);
    }
    V3T<EF> S = v3t(ef_exact(0), ef_exact(0), ef_exact(0));
    const EF z = rect_dist(R, T, n1.l, n2.l, S, c) - (n1.r + n2.r);
    if (c.bad) return 0.0f;
    const float lo = ef_rd_sub(z.v, z.e);
    return lo > 0.0f ? lo : 0.0f;
}

/* the closest-pair search of each active query on one warp: depth first,
 * 32 pairs a round, the closer child on top; no FP64 except in the
 * candidates' later exact evaluation.  Requires the FP32 shadows
 * (q.shadows_ok); other queries take the exact path of the wave kernel. */
__global__ void __launch_bounds__(kWThreads) k_dsearch(const int32_t *__restrict__ active, int na,
                                                       const Query *__restrict__ qs, WAcc *__restrict__ acc,
                                                       const WLoop *__restrict__ loops, Lists L)
{
    const int lane = threadIdx.x & 31;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    DEntry *stack = L.dstack + warp * (size_t)kDCap;
    DCand *cbuf = L.dcand + warp * (size_t)kCCap;
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(L.cnt + 7, 1);
        k = __shfl_sync(kFullMask, k, 0);
        if (k >= na) break;
        const int qi = active[k];
        const Query &q = qs[qi];
        if (!q.shadows_ok) continue; /* searched by the exact waves instead */
        const double margin = dmargin(q);
        float ub = __uint_as_float(acc[qi].ub_bits);
        if (lane == 0) {
            DEntry r;
            r.b1 = r.b2 = 0;
            r.lo = 0.0f;
            r.pad = 0;
            M3 R;
            V3 T;
            /* the root pair's transform (C2A.cpp:1799-1806 / C2A_PQP.cpp:1008-1019) */
            const NodeRec *a0 = q.A->nodes, *b0 = q.B->nodes;
            const M3 Ra = load_R(a0), Rb = load_R(b0);
            R = tmmul(Ra, mmul(q.Rm, Rb));
            T = tmul(Ra, mul_add(q.Rm, load_Tr(b0), q.Tm) - load_Tr(a0));
            EFCtx ec{false};
            r.R = ef_m3(R, ec);
            r.T = ef_v3(T, ec);
            stack[0] = r;
        }
        __syncwarp();
        int sp = 1, nc = 0;
        bool overflow = false;
        while (sp > 0) {
            const int kk = sp < 32 ? sp : 32;
            const int base = sp - kk;
            DEntry e;
            const bool have = lane < kk;
            if (have) e = stack[base + lane];
            __syncwarp();
            int npush = 0, ncand = 0;
            DEntry p0, p1;
            DCand cd;
            float hi_leaf = __int_as_float(0x7f800000);
            if (have && !((double)e.lo > (double)ub + margin)) {
                int fc1, fc2;
                if (is_leaf_pair(q, e.b1, e.b2, fc1, fc2)) {
                    const int ia = -fc1 - 1, ib = -fc2 - 1;
                    EFCtx c{false};
                    V3T<EF> S[3], Tt[3], t[3];
                    load_tri_e(S, q.A->stris + ia);
                    load_tri_e(t, q.B->stris + ib);
                    Tt[0] = mul_add(q.Rme, t[0], q.Tme);
                    Tt[1] = mul_add(q.Rme, t[1], q.Tme);
                    Tt[2] = mul_add(q.Rme, t[2], q.Tme);
                    V3T<EF> pp, qq;
                    TriFeat f;
                    bool col = false;
                    const EF d = tri_dist(pp, qq, S, Tt, f, col, c);
                    /* the leaf pair's RSS bound holds whatever the FP32 TriDist certifies */
                    float lo = e.lo;
                    if (!c.bad) {
                        const float l = ef_rd_sub(d.v, d.e);
                        if (l > lo) lo = l;
                        const float h = ef_ru_add(d.v, d.e);
                        if (h >= 0.0f) hi_leaf = h;
                    }
                    if (!((double)lo > (double)ub + margin)) {
                        ncand = 1;
                        cd.ia = ia;
                        cd.ib = ib;
                        cd.lo = lo;
                        cd.pad = 0;
                    }
                } else {
                    int side, a1, a2, c1, c2;
                    child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, c1, c2);
                    DEntry a, c;
                    a.b1 = a1; a.b2 = a2; c.b1 = c1; c.b2 = c2;
                    a.pad = c.pad = 0;
                    a.lo = child_lower_e(q, side, e.R, e.T, a1, a2, a.R, a.T);
                    c.lo = child_lower_e(q, side, e.R, e.T, c1, c2, c.R, c.T);
                    const bool pa = !((double)a.lo > (double)ub + margin);
                    const bool pc = !((double)c.lo > (double)ub + margin);
                    if (pa && pc) {
                        if (c.lo < a.lo) { p0 = a; p1 = c; }
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
            /* the bound: the smallest certified upper bound of a leaf */
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) hi_leaf = fminf(hi_leaf, __shfl_xor_sync(kFullMask, hi_leaf, o));
            if (hi_leaf < ub) ub = hi_leaf;
            /* candidates into the warp's buffer, filtered against ub when it fills */
            if (nc + 32 > kCCap) nc = filter_cands(cbuf, nc, ub, margin, lane);
            if (nc + 32 > kCCap) { /* still full: the survivors go to the global list now */
                for (int i = lane; i < nc; i += 32) {
                    const int64_t ac = append(L.cnt + 2, 1, L.cap_cand, L.cnt + 6, 2);
                    if (ac >= 0) L.cand[ac] = WCand{qi, cbuf[i].ia, cbuf[i].ib, cbuf[i].lo, 0.0};
                }
                __syncwarp();
                nc = 0;
            }
            {
                const unsigned m = __ballot_sync(kFullMask, ncand != 0);
                if (ncand) cbuf[nc + __popc(m & ((1u << lane) - 1u))] = cd;
                nc += __popc(m);
            }
            int total;
            const int off = warp_excl_scan(npush, lane, total);
            if (base + total > kDCap) {
                overflow = true;
                break;
            }
            if (npush > 0) stack[base + off] = p0;
            if (npush > 1) stack[base + off + 1] = p1;
            sp = base + total;
            __syncwarp();
        }
        __syncwarp();
        nc = filter_cands(cbuf, nc, ub, margin, lane);
        for (int base = 0; base < nc; base += 32) {
            const int i = base + lane;
            const int want = i < nc ? 1 : 0;
            const int64_t ac = append(L.cnt + 2, want, L.cap_cand, L.cnt + 6, 2);
            if (want && ac >= 0) L.cand[ac] = WCand{qi, cbuf[i].ia, cbuf[i].ib, cbuf[i].lo, 0.0};
        }
        if (lane == 0) {
            if (overflow) atomicOr(L.cnt + 6, 1 << 7);
            atomicMin(&acc[qi].ub_bits, __float_as_uint(ub));
        }
        __syncwarp();
    }
}

/* one wave of the closest-pair search */
__global__ void __launch_bounds__(kWThreads) k_dwave(const WItem *__restrict__ in, int n, WItem *__restrict__ out,
                                                     const Query *__restrict__ qs, WAcc *__restrict__ acc, Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int npush = 0, ncand = 0;
    WItem c0, c1;
    WCand cd;
    if (k < n) {
        const WItem &e = in[k];
        const Query &q = qs[e.q];
        const double margin = dmargin(q);
        const float ub = __uint_as_float(*(volatile unsigned int *)&acc[e.q].ub_bits);
        /* (only queries without usable FP32 shadows reach these waves) */
        if (!((double)e.lo > (double)ub + margin)) {
            int fc1, fc2;
            if (is_leaf_pair(q, e.b1, e.b2, fc1, fc2)) {
                const int ia = -fc1 - 1, ib = -fc2 - 1;
                float lo = e.lo; /* the leaf pair's RSS bound */
                if (q.shadows_ok) {
                    EFCtx c{false};
                    V3T<EF> S[3], Tt[3], t[3];
                    load_tri_e(S, q.A->stris + ia);
                    load_tri_e(t, q.B->stris + ib);
                    Tt[0] = mul_add(q.Rme, t[0], q.Tme);
                    Tt[1] = mul_add(q.Rme, t[1], q.Tme);
                    Tt[2] = mul_add(q.Rme, t[2], q.Tme);
                    V3T<EF> p, qq;
                    TriFeat f;
                    bool col = false;
                    const EF d = tri_dist(p, qq, S, Tt, f, col, c);
                    if (!c.bad) {
                        const float l = ef_rd_sub(d.v, d.e);
                        if (l > lo) lo = l;
                        const float hi = ef_ru_add(d.v, d.e);
                        if (hi >= 0.0f && hi < __int_as_float(0x7f800000))
                            atomicMin(&acc[e.q].ub_bits, __float_as_uint(hi));
                    }
                }
                const float ub2 = __uint_as_float(*(volatile unsigned int *)&acc[e.q].ub_bits);
                if (!((double)lo > (double)ub2 + margin)) {
                    ncand = 1;
                    cd.q = e.q;
                    cd.ia = ia;
                    cd.ib = ib;
                    cd.lo = lo;
                    cd.d = 0.0;
                }
            } else {
                M3 R;
                V3 T;
                if (e.side < 0) {
                    R = e.PR;
                    T = e.PT;
                } else {
                    child_transform(q, e.side, e.b1, e.b2, e.PR, e.PT, R, T);
                }
                int side, a1, a2, cc1, cc2;
                child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, cc1, cc2);
                EFCtx ec{false};
                const M3T<EF> Re = ef_m3(R, ec);
                const V3T<EF> Te = ef_v3(T, ec);
                float la, lc;
                if (q.shadows_ok && !ec.bad) {
                    la = bv_lower(q, side, Re, Te, a1, a2);
                    lc = bv_lower(q, side, Re, Te, cc1, cc2);
                } else {
                    la = bv_lower_exact(q, side, R, T, a1, a2);
                    lc = bv_lower_exact(q, side, R, T, cc1, cc2);
                }
                if (!((double)la > (double)ub + margin)) {
                    WItem &w = npush ? c1 : c0;
                    w.q = e.q; w.b1 = a1; w.b2 = a2; w.side = side; w.lo = la; w.pad = 0; w.PR = R; w.PT = T;
                    npush++;
                }
                if (!((double)lc > (double)ub + margin)) {
                    WItem &w = npush ? c1 : c0;
                    w.q = e.q; w.b1 = cc1; w.b2 = cc2; w.side = side; w.lo = lc; w.pad = 0; w.PR = R; w.PT = T;
                    npush++;
                }
            }
        }
    }
    const int64_t at = append(L.cnt + 0, npush, L.cap_item, L.cnt + 6, 0);
    if (npush > 0 && at >= 0) out[at] = c0;
    if (npush > 1 && at >= 0) out[at + 1] = c1;
    const int64_t ac = append(L.cnt + 2, ncand, L.cap_cand, L.cnt + 6, 2);
    if (ncand && ac >= 0) L.cand[ac] = cd;
}

/* exact distances of the candidates that can still be the minimum */
__global__ void __launch_bounds__(kWThreads) k_dcand(int n, const Query *__restrict__ qs, WAcc *__restrict__ acc,
                                                     Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    WCand &c = L.cand[k];
    const Query &q = qs[c.q];
    const float ub = __uint_as_float(acc[c.q].ub_bits);
    c.d = __longlong_as_double(0x7ff0000000000000LL);
    if ((double)c.lo > (double)ub + dmargin(q)) return;
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double d = tri_distance_x(q, c.ia, c.ib, p, qq, f, col);
    c.d = d;
    if (d >= 0.0) atomicMin(&acc[c.q].best_bits, (unsigned long long)__double_as_longlong(d));
}

/* among exactly tied minima, the smallest triangle pair */
__global__ void __launch_bounds__(kWThreads) k_dtie(int n, WAcc *__restrict__ acc, Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const WCand &c = L.cand[k];
    if (c.d == __longlong_as_double((long long)acc[c.q].best_bits))
        atomicMin(&acc[c.q].pair_key, ((unsigned long long)(unsigned)c.ia << 32) | (unsigned)c.ib);
}

/* the step's seed, error schedule and root item */
__global__ void __launch_bounds__(kWThreads) k_tbegin(const int32_t *__restrict__ active, int na,
                                                      Query *__restrict__ qs, WLoop *__restrict__ loops,
                                                      WAcc *__restrict__ acc, Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int push = 0, qi = -1;
    M3 R;
    V3 T;
    if (k < na) {
        qi = active[k];
        Query &q = qs[qi];
        WAcc &a = acc[qi];
        if (a.pair_key != ~0ull) {
            q.seed_a = (int)(a.pair_key >> 32);
            q.seed_b = (int)(a.pair_key & 0xffffffffu);
        }
        q.distance = __longlong_as_double((long long)a.best_bits);
        if (q.numCA == 0) q.mint = 1;
        if (q.mint <= 0.005 || q.distance <= 0.5 || q.numCA > 5) {
            q.abs_err = 0;
            q.rel_err = 0;
        } else {
            q.abs_err = 1e+30;
            q.rel_err = (q.numCA <= 2) ? 3 : 0.5;
        }
        q.mint = 1;
        refresh_shadows(q);
        /* the root transform again (relative_transforms is deterministic) */
        WLoop &lp = loops[qi];
        relative_transforms(q, lp.R1, lp.T1, lp.R2, lp.T2, R, T);
        q.shadows_ok = q.shadows_ok && q.e_ok;
        push = 1;
    }
    const int64_t at = append(L.cnt + 1, push, L.cap_arena, L.cnt + 6, 1);
    if (push && at >= 0) {
        WItem &it = L.arena[at];
        it.q = qi;
        it.b1 = it.b2 = 0;
        it.side = -1;
        it.lo = 0.0f;
        it.pad = 0;
        it.PR = R;
        it.PT = T;
    }
}

/* one wave of the fixed-bound step; items [b, e) of the arena */
__global__ void __launch_bounds__(kWThreads) k_twave(int64_t b, int64_t e_end, const Query *__restrict__ qs,
                                                     WAcc *__restrict__ acc, Lists L)
{
    const int64_t t = b + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int npush = 0, ndef = 0, nleaf = 0;
    WItem c0, c1;
    WDefer d0, d1;
    WLeaf lf;
    if (t < e_end) {
        const WItem e = L.arena[t];
        const Query &q = qs[e.q];
        WAcc &a = acc[e.q];
        int fc1, fc2;
        if (is_leaf_pair(q, e.b1, e.b2, fc1, fc2)) {
            atomicAdd(&a.ntri, 1ull);
            bool skip = false;
            if (q.shadows_ok) {
                const int ia = -fc1 - 1, ib = -fc2 - 1;
                EFCtx c{false};
                V3T<EF> S[3], Tt[3], tt[3];
                load_tri_e(S, q.A->stris + ia);
                load_tri_e(tt, q.B->stris + ib);
                Tt[0] = mul_add(q.Rme, tt[0], q.Tme);
                Tt[1] = mul_add(q.Rme, tt[1], q.Tme);
                Tt[2] = mul_add(q.Rme, tt[2], q.Tme);
                V3T<EF> p, qq;
                TriFeat f;
                bool col = false;
                const EF dTri = tri_dist(p, qq, S, Tt, f, col, c);
                skip = !c.bad && ef_le3(dTri, q.distance_e) == 0;
            }
            if (!skip) {
                nleaf = 1;
                lf.q = e.q;
                lf.b1 = e.b1;
                lf.b2 = e.b2;
                lf.pad = 0;
            }
        } else {
            M3 R;
            V3 T;
            if (e.side < 0) {
                R = e.PR;
                T = e.PT;
            } else {
                child_transform(q, e.side, e.b1, e.b2, e.PR, e.PT, R, T);
            }
            int side, a1, a2, cc1, cc2;
            child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, cc1, cc2);
            Pending pa, pc;
            pa.b1 = a1; pa.b2 = a2; pc.b1 = cc1; pc.b2 = cc2;
            pa.side = pc.side = side;
            pa.exact = pc.exact = 0;
            pa.PR = pc.PR = R;
            pa.PT = pc.PT = T;
            EFCtx ec{false};
            const M3T<EF> Re = ef_m3(R, ec);
            const V3T<EF> Te = ef_v3(T, ec);
            bool zero_a = false, zero_c = false;
            const bool ok_a = !ec.bad && bv_test_e(q, side, Re, Te, a1, a2, pa.d, pa.m, zero_a);
            const bool ok_c = !ec.bad && bv_test_e(q, side, Re, Te, cc1, cc2, pc.d, pc.m, zero_c);
            if (!ok_a) make_exact(q, pa);
            else if (zero_a) { pa.exact = 1; pa.d_x = 0.0; pa.m_x = 0.0; }
            if (!ok_c) make_exact(q, pc);
            else if (zero_c) { pc.exact = 1; pc.d_x = 0.0; pc.m_x = 0.0; }
            atomicAdd(&a.nbv, 2ull);
            Pending *ch[2] = {&pa, &pc};
            for (int j = 0; j < 2; j++) {
                Pending &p = *ch[j];
                if (descend(q, p)) {
                    WItem &w = npush ? c1 : c0;
                    w.q = e.q; w.b1 = p.b1; w.b2 = p.b2; w.side = side; w.lo = 0.0f; w.pad = 0; w.PR = R; w.PT = T;
                    npush++;
                } else if (p.exact) {
                    /* contribute: res->mint = min(res->mint, mint) (C2A.cpp:1290-1311) */
                    if (p.m_x >= 0.0) {
                        atomicMin(&a.mint_bits, (unsigned long long)__double_as_longlong(p.m_x));
                        atomicMin(&a.U_bits, __float_as_uint(ru_float(p.m_x)));
                    }
                } else {
                    const float hi = ef_ru_add(p.m.v, p.m.e), lo = ef_rd_sub(p.m.v, p.m.e);
                    if (hi >= 0.0f && hi < __int_as_float(0x7f800000)) atomicMin(&a.U_bits, __float_as_uint(hi));
                    const float U = __uint_as_float(*(volatile unsigned int *)&a.U_bits);
                    if (!(lo >= U)) {
                        WDefer &d = ndef ? d1 : d0;
                        d.q = e.q; d.b1 = p.b1; d.b2 = p.b2; d.side = side; d.lo = lo; d.parent = (int32_t)t;
                        ndef++;
                    }
                }
            }
        }
    }
    const int64_t at = append(L.cnt + 1, npush, L.cap_arena, L.cnt + 6, 1);
    if (npush > 0 && at >= 0) L.arena[at] = c0;
    if (npush > 1 && at >= 0) L.arena[at + 1] = c1;
    const int64_t ad = append(L.cnt + 3, ndef, L.cap_defer, L.cnt + 6, 3);
    if (ndef > 0 && ad >= 0) L.defer[ad] = d0;
    if (ndef > 1 && ad >= 0) L.defer[ad + 1] = d1;
    const int64_t al = append(L.cnt + 4, nleaf, L.cap_leaf, L.cnt + 6, 4);
    if (nleaf && al >= 0) L.leaf[al] = lf;
}

/* deferred mints of pruned pairs, exactly */
__global__ void __launch_bounds__(kWThreads) k_tdefer(int n, const Query *__restrict__ qs, WAcc *__restrict__ acc,
                                                      Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const WDefer d = L.defer[k];
    WAcc &a = acc[d.q];
    const float U = __uint_as_float(a.U_bits);
    if (d.lo >= U) return; /* certainly not below another contribution */
    const Query &q = qs[d.q];
    const WItem &par = L.arena[d.parent];
    M3 Rp, R;
    V3 Tp, T;
    if (par.side < 0) {
        Rp = par.PR;
        Tp = par.PT;
    } else {
        child_transform(q, par.side, par.b1, par.b2, par.PR, par.PT, Rp, Tp);
    }
    child_transform(q, d.side, d.b1, d.b2, Rp, Tp, R, T);
    double dd, m;
    bv_test_x(q, R, T, d.b1, d.b2, dd, m);
    if (m >= 0.0) atomicMin(&a.mint_bits, (unsigned long long)__double_as_longlong(m));
}

/* deferred leaves of the step (C2A.cpp:1141-1183 with res->distance = d*) */
__global__ void __launch_bounds__(kWThreads) k_tleaf(int n, const Query *__restrict__ qs, WAcc *__restrict__ acc,
                                                     Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const WLeaf l = L.leaf[k];
    const Query &q = qs[l.q];
    const int ia = -__ldg(&q.A->nodes[l.b1].first_child) - 1, ib = -__ldg(&q.B->nodes[l.b2].first_child) - 1;
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double dTri = tri_distance_x(q, ia, ib, p, qq, f, col);
    if (!(dTri <= q.distance)) return;
    ExactCtx xc{false};
    const V3 res1 = mul(q.r1, p) + q.t1;
    const V3 res2 = mul(q.r1, qq) + q.t1;
    V3 S1 = res2 - res1;
    V3 S2 = mul_s(S1, -1.0);
    const double mb1 = bound_leaf(q.x1, __ldg(&q.A->nodes[l.b1].angR), S1, xc);
    const double mb2 = bound_leaf(q.x2, __ldg(&q.B->nodes[l.b2].angR), S2, xc);
    double mint = (dTri) / (mb1 + mb2);
    if (mint < 0.0) mint = 0.0;
    if (mint >= 0.0) atomicMin(&acc[l.q].mint_bits, (unsigned long long)__double_as_longlong(mint));
}

/* one iteration of C2A_QueryTimeOfContact's loop (C2A.cpp:2029-2146) */
__global__ void __launch_bounds__(kWThreads) k_ca(const int32_t *__restrict__ active, int na, Query *__restrict__ qs,
                                                  WLoop *__restrict__ loops, WAcc *__restrict__ acc, c2a_params prm,
                                                  c2a_result *__restrict__ results, int32_t *__restrict__ next,
                                                  Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int keep = 0, qi = -1;
    if (k < na) {
        qi = active[k];
        Query &q = qs[qi];
        WLoop &lp = loops[qi];
        const WAcc &a = acc[qi];
        q.mint = __longlong_as_double((long long)a.mint_bits);
        q.nbv += (long long)a.nbv;
        q.ntri += (long long)a.ntri;
        const double dist = q.distance, mint = q.mint;
        bool exit_loop = false, done = false;
        if (lp.first) {
            lp.first = 0;
            q.numCA = 1;
            lp.lastLamda = mint;
        }
        if (!(dist > prm.tol_d) || q.status) {
            exit_loop = true;
        } else {
            lp.nItrs++;
            if (lp.nItrs > prm.max_iters) {
                q.status |= 0; /* the cap is reported on the result below */
                exit_loop = true;
                lp.contact = -1; /* marks the iteration cap */
            } else if (mint >= 1.0) {
                done = true;
            } else {
                lp.dlamda = mint;
                if (lp.dlamda < prm.tol_t) {
                    exit_loop = true;
                } else {
                    lp.lamda += lp.dlamda;
                    if (lp.lamda >= 1.0) {
                        done = true;
                    } else {
                        lp.lastLamda = lp.lamda;
                        q.numCA++;
                        double orn[4];
                        motion_integrate(q.m1, lp.lamda, lp.R1.m, &lp.T1.x, orn);
                        motion_integrate(q.m2, lp.lamda, lp.R2.m, &lp.T2.x, orn);
                        set_pose1(q, lp.R1, lp.T1);
                        q.upbound = 1.0 - lp.lamda;
                        keep = 1;
                    }
                }
            }
        }
        if (!keep) {
            const bool capped = lp.contact == -1;
            double toc;
            bool collisionfree;
            if (done) {
                toc = 0;
                collisionfree = true;
            } else {
                if (dist == 0 && mint < 0) toc = lp.lastLamda - lp.dlamda;
                else toc = lp.lastLamda;
                collisionfree = false;
                if (toc >= 1 - prm.tol_t) toc = 0;
            }
            c2a_result &out = results[qi];
            memset(&out, 0, sizeof(out));
            out.status = capped ? C2A_QUERY_ITER_CAP : 0;
            out.status |= q.status;
            out.contact_offset = qi * prm.contacts_per_query;
            out.collisionfree = collisionfree ? 1 : 0;
            out.toc = toc;
            out.numCA = q.numCA;
            out.translation = 0;
            out.distance = q.distance;
            out.mint = q.mint;
            out.num_bv_tests = q.nbv;
            out.num_tri_tests = q.ntri;
            out.seed_a = q.seed_a;
            out.seed_b = q.seed_b;
            lp.toc = toc;
            lp.collisionfree = collisionfree ? 1 : 0;
            lp.contact = 0;
            if (!collisionfree && q.status == 0) {
                M3 Ra, Rb;
                V3 Ta, Tb;
                double orn[4];
                motion_integrate(q.m1, toc, Ra.m, &Ta.x, orn);
                motion_integrate(q.m2, toc, Rb.m, &Tb.x, orn);
                for (int j = 0; j < 9; j++) {
                    out.R_toc[0][j] = Ra.m[j];
                    out.R_toc[1][j] = Rb.m[j];
                }
                out.T_toc[0][0] = Ta.x; out.T_toc[0][1] = Ta.y; out.T_toc[0][2] = Ta.z;
                out.T_toc[1][0] = Tb.x; out.T_toc[1][1] = Tb.y; out.T_toc[1][2] = Tb.z;
                if (prm.with_contacts) {
                    lp.contact = 1;
                    lp.R1 = Ra;
                    lp.T1 = Ta;
                    lp.R2 = Rb;
                    lp.T2 = Tb;
                    lp.threshold = 2 * q.distance + prm.contact_abs;
                }
            }
        }
    }
    const int64_t at = append(L.cnt + 5, keep, (int64_t)1 << 40, L.cnt + 6, 5);
    if (keep && at >= 0) next[at] = qi;
}

/* roots of the contact enumeration for the colliding queries */
__global__ void __launch_bounds__(kWThreads) k_cbegin(int n, Query *__restrict__ qs, WLoop *__restrict__ loops,
                                                      WAcc *__restrict__ acc, Lists L, int out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int push = 0;
    M3 R;
    V3 T;
    if (i < n && loops[i].contact == 1) {
        Query &q = qs[i];
        WLoop &lp = loops[i];
        set_pose1(q, lp.R1, lp.T1);
        relative_transforms(q, lp.R1, lp.T1, lp.R2, lp.T2, R, T);
        q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
        q.want_mint = false;
        acc[i].contacts = 0;
        push = 1;
    }
    const int64_t at = append(L.cnt + 0, push, L.cap_item, L.cnt + 6, 0);
    if (push && at >= 0) {
        WItem &it = L.item[out][at];
        it.q = i;
        it.b1 = it.b2 = 0;
        it.side = -1;
        it.lo = 0.0f;
        it.pad = 0;
        it.PR = R;
        it.PT = T;
    }
}

/* one wave of the contact enumeration */
__global__ void __launch_bounds__(kWThreads) k_cwave(const WItem *__restrict__ in, int n, WItem *__restrict__ out,
                                                     Query *__restrict__ qs, const WLoop *__restrict__ loops,
                                                     WAcc *__restrict__ acc, c2a_contact *__restrict__ contacts,
                                                     int slots, Lists L)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int npush = 0;
    WItem c0, c1;
    if (k < n) {
        const WItem e = in[k];
        Query &q = qs[e.q];
        const double threshold = loops[e.q].threshold;
        EFCtx tc{false};
        const EF threshold_e = in_d(threshold, tc);
        int fc1, fc2;
        if (is_leaf_pair(q, e.b1, e.b2, fc1, fc2)) {
            c2a_contact ct;
            const bool saved = q.shadows_ok;
            bool emit;
            if (tc.bad && saved) { /* an uncertifiable threshold: exact leaf test only */
                Query qc = q;
                qc.shadows_ok = false;
                emit = contact_leaf_test(qc, e.b1, e.b2, threshold, threshold_e, e.q, ct);
            } else {
                emit = contact_leaf_test(q, e.b1, e.b2, threshold, threshold_e, e.q, ct);
            }
            if (emit) {
                const int slot = atomicAdd(&acc[e.q].contacts, 1);
                if (contacts && slot < slots) contacts[(size_t)e.q * (size_t)slots + slot] = ct;
            }
        } else {
            M3 R;
            V3 T;
            if (e.side < 0) {
                R = e.PR;
                T = e.PT;
            } else {
                child_transform(q, e.side, e.b1, e.b2, e.PR, e.PT, R, T);
            }
            int side, a1, a2, cc1, cc2;
            child_pairs(q, e.b1, e.b2, fc1, fc2, side, a1, a2, cc1, cc2);
            Pending pa, pc;
            pa.b1 = a1; pa.b2 = a2; pc.b1 = cc1; pc.b2 = cc2;
            pa.side = pc.side = side;
            pa.exact = pc.exact = 0;
            pa.PR = pc.PR = R;
            pa.PT = pc.PT = T;
            EFCtx ec{false};
            const M3T<EF> Re = ef_m3(R, ec);
            const V3T<EF> Te = ef_v3(T, ec);
            bool zero_a = false, zero_c = false;
            const bool ok_a = !ec.bad && !tc.bad && bv_test_e(q, side, Re, Te, a1, a2, pa.d, pa.m, zero_a);
            const bool ok_c = !ec.bad && !tc.bad && bv_test_e(q, side, Re, Te, cc1, cc2, pc.d, pc.m, zero_c);
            if (!ok_a) make_exact(q, pa);
            else if (zero_a) { pa.exact = 1; pa.d_x = 0.0; pa.m_x = 0.0; }
            if (!ok_c) make_exact(q, pc);
            else if (zero_c) { pc.exact = 1; pc.d_x = 0.0; pc.m_x = 0.0; }
            if (contact_descend(q, pa, threshold, threshold_e)) {
                c0.q = e.q; c0.b1 = a1; c0.b2 = a2; c0.side = side; c0.lo = 0.0f; c0.pad = 0; c0.PR = R; c0.PT = T;
                npush = 1;
            }
            if (contact_descend(q, pc, threshold, threshold_e)) {
                WItem &w = npush ? c1 : c0;
                w.q = e.q; w.b1 = cc1; w.b2 = cc2; w.side = side; w.lo = 0.0f; w.pad = 0; w.PR = R; w.PT = T;
                npush++;
            }
        }
    }
    const int64_t at = append(L.cnt + 0, npush, L.cap_item, L.cnt + 6, 0);
    if (npush > 0 && at >= 0) out[at] = c0;
    if (npush > 1 && at >= 0) out[at + 1] = c1;
}

/* contacts of each query sorted by (tri_a, tri_b); the count into the result */
__global__ void __launch_bounds__(kWThreads) k_csort(int n, const WLoop *__restrict__ loops,
                                                     const WAcc *__restrict__ acc, c2a_contact *__restrict__ contacts,
                                                     int slots, c2a_result *__restrict__ results)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || loops[i].contact != 1) return;
    const int count = acc[i].contacts;
    results[i].num_contact = count;
    if (count > slots) results[i].status |= C2A_QUERY_CONTACT_OVERFLOW;
    if (!contacts) return;
    c2a_contact *c = contacts + (size_t)i * (size_t)slots;
    const int m = count < slots ? count : slots;
    for (int a = 1; a < m; a++) { /* insertion sort: the lists are short */
        const c2a_contact key = c[a];
        int b = a - 1;
        while (b >= 0 && (c[b].tri_a > key.tri_a || (c[b].tri_a == key.tri_a && c[b].tri_b > key.tri_b))) {
            c[b + 1] = c[b];
            b--;
        }
        c[b + 1] = key;
    }
}

} // namespace

/* ------------------------------------------------------------- host side */

struct WaveBuffers {
    int n_cap = 0;
    Query *qs = nullptr;
    WLoop *loops = nullptr;
    WAcc *acc = nullptr;
    Lists L{};
    int32_t *h_cnt = nullptr; /* pinned mirror of the counters */
    int64_t scale = 1;        /* list capacities grow after an overflow */
    int search_warps = 0;     /* warps of the k_dsearch grid (one stack each) */
};

namespace {

void free_lists(WaveBuffers *b)
{
    cudaFree(b->qs);
    cudaFree(b->loops);
    cudaFree(b->acc);
    cudaFree(b->L.item[0]);
    cudaFree(b->L.item[1]);
    cudaFree(b->L.arena);
    cudaFree(b->L.cand);
    cudaFree(b->L.defer);
    cudaFree(b->L.leaf);
    cudaFree(b->L.active[0]);
    cudaFree(b->L.active[1]);
    cudaFree(b->L.dstack);
    cudaFree(b->L.dcand);
    cudaFree(b->L.cnt);
    b->qs = nullptr;
    b->loops = nullptr;
    b->acc = nullptr;
    b->L = Lists{};
    b->n_cap = 0;
}

c2a_status alloc_lists(WaveBuffers *b, int n)
{
    free_lists(b);
    const int64_t nn = n > 1024 ? n : 1024;
    Lists &L = b->L;
    L.cap_item = nn * 512 * b->scale;
    L.cap_arena = nn * 1024 * b->scale;
    L.cap_cand = nn * 1024 * b->scale;
    L.cap_defer = nn * 1024 * b->scale;
    L.cap_leaf = nn * 256 * b->scale;
    cudaError_t e = cudaMalloc(&b->qs, sizeof(Query) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&b->loops, sizeof(WLoop) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&b->acc, sizeof(WAcc) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&L.item[0], sizeof(WItem) * L.cap_item);
    if (e == cudaSuccess) e = cudaMalloc(&L.item[1], sizeof(WItem) * L.cap_item);
    if (e == cudaSuccess) e = cudaMalloc(&L.arena, sizeof(WItem) * L.cap_arena);
    if (e == cudaSuccess) e = cudaMalloc(&L.cand, sizeof(WCand) * L.cap_cand);
    if (e == cudaSuccess) e = cudaMalloc(&L.defer, sizeof(WDefer) * L.cap_defer);
    if (e == cudaSuccess) e = cudaMalloc(&L.leaf, sizeof(WLeaf) * L.cap_leaf);
    if (e == cudaSuccess) e = cudaMalloc(&L.active[0], sizeof(int32_t) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&L.active[1], sizeof(int32_t) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&L.dstack, sizeof(DEntry) * (size_t)kDCap * (size_t)b->search_warps);
    if (e == cudaSuccess) e = cudaMalloc(&L.dcand, sizeof(DCand) * (size_t)kCCap * (size_t)b->search_warps);
    if (e == cudaSuccess) e = cudaMalloc(&L.cnt, sizeof(int32_t) * 8);
    if (e != cudaSuccess) {
        fprintf(stderr, "c2a_gb300: wave engine buffers (%lld queries): %s\n", (long long)nn, cudaGetErrorString(e));
        free_lists(b);
        return e == cudaErrorMemoryAllocation ? C2A_ERR_OUT_OF_MEMORY : C2A_ERR_CUDA;
    }
    b->n_cap = (int)nn;
    return C2A_OK;
}

unsigned grid1(int64_t n) { return (unsigned)((n + kWThreads - 1) / kWThreads); }

/* C2A_WAVE_TRACE=2 prints the wall time per kernel kind at the end of a batch */
bool times_on()
{
    static const bool on = getenv("C2A_WAVE_TRACE") && getenv("C2A_WAVE_TRACE")[0] == '2';
    return on;
}
struct PhaseClock {
    double t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::chrono::steady_clock::time_point last = std::chrono::steady_clock::now();
    void lap(int k)
    {
        const auto now = std::chrono::steady_clock::now();
        t[k] += std::chrono::duration<double, std::milli>(now - last).count();
        last = now;
    }
};

/* C2A_WAVE_TRACE=1 prints every wave's list lengths to stderr */
bool trace_on()
{
    static const bool on = getenv("C2A_WAVE_TRACE") && getenv("C2A_WAVE_TRACE")[0] == '1';
    return on;
}

} // namespace

#define C2A_WCUDA(call)                                                                                            \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            fprintf(stderr, "c2a_gb300: %s failed: %s\n", #call, cudaGetErrorString(e_));                          \
            return e_ == cudaErrorMemoryAllocation ? C2A_ERR_OUT_OF_MEMORY : C2A_ERR_CUDA;                          \
        }                                                                                                          \
    } while (0)

void wave_free(WaveBuffers *b)
{
    if (!b) return;
    free_lists(b);
    if (b->h_cnt) cudaFreeHost(b->h_cnt);
    delete b;
}

namespace {

/* reads the counters (after the stream's work so far) */
c2a_status read_counters(WaveBuffers *b, cudaStream_t s)
{
    C2A_WCUDA(cudaMemcpyAsync(b->h_cnt, b->L.cnt, sizeof(int32_t) * 8, cudaMemcpyDeviceToHost, s));
    C2A_WCUDA(cudaStreamSynchronize(s));
    return C2A_OK;
}

c2a_status set_counter(WaveBuffers *b, cudaStream_t s, int which, int32_t v)
{
    b->h_cnt[which] = v;
    C2A_WCUDA(cudaMemcpyAsync(b->L.cnt + which, b->h_cnt + which, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    return C2A_OK;
}

/* one full batch; returns C2A_OK, an error, or (overflow) C2A_ERR_OUT_OF_MEMORY with *overflow set */
c2a_status run_batch(WaveBuffers *b, cudaStream_t s, const c2a_query *d_queries, int n, const DevModel *d_models,
                     int num_models, const c2a_params &prm, c2a_result *d_results, c2a_contact *d_contacts,
                     int64_t *launches, bool *overflow, const uint32_t *hints, int nh)
{
    Lists &L = b->L;
    *overflow = false;
    PhaseClock clk; /* 0 init, 1 step begin + search, 2 exact waves of the search, 3 candidates, 4 step waves,
                       5 deferred, 6 CA loop, 7 contacts */
    C2A_WCUDA(cudaMemsetAsync(L.cnt, 0, sizeof(int32_t) * 8, s));
    C2A_WCUDA(cudaMemsetAsync(b->loops, 0, sizeof(WLoop) * (size_t)n, s));
    k_init<<<grid1(n), kWThreads, 0, s>>>(d_queries, n, d_models, num_models, prm, d_results, d_contacts, b->qs,
                                          b->loops, L);
    (*launches)++;
    C2A_WCUDA(cudaGetLastError());
    c2a_status st = read_counters(b, s);
    if (st) return st;
    clk.lap(0);
    int na = b->h_cnt[5];
    int cur_active = 0;
    while (na > 0) {
        /* closest-pair search */
        for (int w : {0, 2, 3, 4}) {
            st = set_counter(b, s, w, 0);
            if (st) return st;
        }
        st = set_counter(b, s, 1, 0);
        if (st) return st;
        int cur = 0;
        if (trace_on()) fprintf(stderr, "step: %d active\n", na);
        k_step_begin<<<grid1(na), kWThreads, 0, s>>>(L.active[cur_active], na, b->qs, b->loops, b->acc, L, cur,
                                                     hints, nh);
        st = set_counter(b, s, 7, 0);
        if (st) return st;
        k_dsearch<<<b->search_warps / (kWThreads / 32), kWThreads, 0, s>>>(L.active[cur_active], na, b->qs, b->acc,
                                                                          b->loops, L);
        *launches += 2;
        st = read_counters(b, s);
        if (st) return st;
        if (trace_on()) fprintf(stderr, "dsearch: %d candidates\n", b->h_cnt[2]);
        clk.lap(1);
        if (b->h_cnt[6]) {
            fprintf(stderr, "c2a_gb300: wave list overflow (mask %d)\n", b->h_cnt[6]);
            *overflow = true;
            return C2A_ERR_OUT_OF_MEMORY;
        }
        int items = b->h_cnt[0];
        while (items > 0) {
            st = set_counter(b, s, 0, 0);
            if (st) return st;
            k_dwave<<<grid1(items), kWThreads, 0, s>>>(L.item[cur], items, L.item[1 - cur], b->qs, b->acc, L);
            (*launches)++;
            st = read_counters(b, s);
            if (st) return st;
            if (trace_on())
                fprintf(stderr, "dwave in %d out %d cand %d\n", items, b->h_cnt[0], b->h_cnt[2]);
            if (b->h_cnt[6]) {
                fprintf(stderr, "c2a_gb300: wave list overflow (mask %d)\n", b->h_cnt[6]);
                *overflow = true;
                return C2A_ERR_OUT_OF_MEMORY;
            }
            cur = 1 - cur;
            items = b->h_cnt[0];
        }
        clk.lap(2);
        const int ncand = b->h_cnt[2];
        if (ncand > 0) {
            k_dcand<<<grid1(ncand), kWThreads, 0, s>>>(ncand, b->qs, b->acc, L);
            k_dtie<<<grid1(ncand), kWThreads, 0, s>>>(ncand, b->acc, L);
            *launches += 2;
            if (times_on()) cudaStreamSynchronize(s);
        }
        clk.lap(3);
        /* the fixed-bound step */
        k_tbegin<<<grid1(na), kWThreads, 0, s>>>(L.active[cur_active], na, b->qs, b->loops, b->acc, L);
        (*launches)++;
        st = read_counters(b, s);
        if (st) return st;
        int64_t begin = 0, end = b->h_cnt[1];
        while (end > begin) {
            k_twave<<<grid1(end - begin), kWThreads, 0, s>>>(begin, end, b->qs, b->acc, L);
            (*launches)++;
            st = read_counters(b, s);
            if (st) return st;
            if (trace_on())
                fprintf(stderr, "twave [%lld, %lld) out %d defer %d leaf %d\n", (long long)begin, (long long)end,
                        b->h_cnt[1], b->h_cnt[3], b->h_cnt[4]);
            if (b->h_cnt[6]) {
                fprintf(stderr, "c2a_gb300: wave list overflow (mask %d)\n", b->h_cnt[6]);
                *overflow = true;
                return C2A_ERR_OUT_OF_MEMORY;
            }
            begin = end;
            end = b->h_cnt[1];
        }
        clk.lap(4);
        const int ndef = b->h_cnt[3], nleaf = b->h_cnt[4];
        if (ndef > 0) {
            k_tdefer<<<grid1(ndef), kWThreads, 0, s>>>(ndef, b->qs, b->acc, L);
            (*launches)++;
        }
        if (nleaf > 0) {
            k_tleaf<<<grid1(nleaf), kWThreads, 0, s>>>(nleaf, b->qs, b->acc, L);
            (*launches)++;
        }
        if (times_on()) cudaStreamSynchronize(s);
        clk.lap(5);
        /* the CA loop */
        st = set_counter(b, s, 5, 0);
        if (st) return st;
        k_ca<<<grid1(na), kWThreads, 0, s>>>(L.active[cur_active], na, b->qs, b->loops, b->acc, prm, d_results,
                                             L.active[1 - cur_active], L);
        (*launches)++;
        st = read_counters(b, s);
        if (st) return st;
        if (b->h_cnt[6]) {
            *overflow = true;
            return C2A_ERR_OUT_OF_MEMORY;
        }
        cur_active = 1 - cur_active;
        na = b->h_cnt[5];
        clk.lap(6);
    }
    if (prm.with_contacts) {
        st = set_counter(b, s, 0, 0);
        if (st) return st;
        int cur = 0;
        k_cbegin<<<grid1(n), kWThreads, 0, s>>>(n, b->qs, b->loops, b->acc, L, cur);
        (*launches)++;
        st = read_counters(b, s);
        if (st) return st;
        int items = b->h_cnt[0];
        while (items > 0) {
            st = set_counter(b, s, 0, 0);
            if (st) return st;
            k_cwave<<<grid1(items), kWThreads, 0, s>>>(L.item[cur], items, L.item[1 - cur], b->qs, b->loops, b->acc,
                                                       d_contacts, prm.contacts_per_query, L);
            (*launches)++;
            st = read_counters(b, s);
            if (st) return st;
            if (b->h_cnt[6]) {
                *overflow = true;
                return C2A_ERR_OUT_OF_MEMORY;
            }
            cur = 1 - cur;
            items = b->h_cnt[0];
        }
        k_csort<<<grid1(n), kWThreads, 0, s>>>(n, b->loops, b->acc, d_contacts, prm.contacts_per_query, d_results);
        (*launches)++;
        if (times_on()) cudaStreamSynchronize(s);
        clk.lap(7);
    }
    if (times_on())
        fprintf(stderr, "wave engine ms: init %.1f search %.1f search-waves %.1f candidates %.1f step-waves %.1f "
                        "deferred %.1f ca %.1f contacts %.1f\n",
                clk.t[0], clk.t[1], clk.t[2], clk.t[3], clk.t[4], clk.t[5], clk.t[6], clk.t[7]);
    C2A_WCUDA(cudaGetLastError());
    return C2A_OK;
}

} // namespace

c2a_status wave_solve(WaveBuffers **bufs, int sm_count, cudaStream_t s, const c2a_query *d_queries, int n,
                      const DevModel *d_models, int num_models, const c2a_params &prm, c2a_result *d_results,
                      c2a_contact *d_contacts, int64_t *launches, const uint32_t *hints, int nh)
{
    if (!*bufs) {
        WaveBuffers *b = new (std::nothrow) WaveBuffers();
        if (!b) return C2A_ERR_OUT_OF_MEMORY;
        if (cudaMallocHost(&b->h_cnt, sizeof(int32_t) * 8) != cudaSuccess) {
            delete b;
            return C2A_ERR_OUT_OF_MEMORY;
        }
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_dsearch, kWThreads, 0);
        b->search_warps = (sm_count > 0 ? sm_count : 1) * (occ > 0 ? occ : 1) * (kWThreads / 32);
        *bufs = b;
    }
    WaveBuffers *b = *bufs;
    for (int attempt = 0; attempt < 4; attempt++) {
        if (b->n_cap < n) {
            C2A_WCUDA(cudaStreamSynchronize(s));
            const c2a_status st = alloc_lists(b, n);
            if (st) return st;
        }
        bool overflow = false;
        const c2a_status st = run_batch(b, s, d_queries, n, d_models, num_models, prm, d_results, d_contacts,
                                        launches, &overflow, hints, nh);
        if (!overflow) return st;
        /* a list ran out of room: grow every list and solve the batch again */
        C2A_WCUDA(cudaStreamSynchronize(s));
        b->scale *= 2;
        b->n_cap = 0;
        fprintf(stderr, "c2a_gb300: wave lists overflowed; retrying with %lldx capacity\n", (long long)b->scale);
    }
    return C2A_ERR_OUT_OF_MEMORY;
}

} // namespace c2a
