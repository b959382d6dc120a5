/*
 * ca_spec.cuh -- the reference-order CA step (TOCStepRecurse_Dis,
 * C2A/src/C2A.cpp:1114-1354) on one warp by speculative expansion and
 * ordered replay.
 *
 * The reference's depth-first traversal decides, pair by pair, with a
 * running distance that only shrinks (leaves lower it, C2A.cpp:1150-1174).
 * A node pair's test (its two children's RSS distances and motion-bounded
 * step sizes, C2A.cpp:1192-1279) does not depend on that running state; only
 * the decisions do.  So the warp runs in rounds:
 *
 *   replay    all lanes walk the reference's depth-first order over pairs
 *             already tested, with the reference's decisions and running
 *             distance, until the order reaches a pair whose test is not
 *             there yet (the due pair);
 *   speculate the due pair plus the next pairs, in depth-first order, that
 *             the current running distance would descend into (a superset of
 *             what the replay will ask for, since the distance only
 *             shrinks) make up to 16 candidates;
 *   test      lanes 2i and 2i+1 expand candidate i: the pair's exact FP64
 *             transform (six outputs per lane), then one child's RSS test per
 *             lane through the certified FP32 filter (FP64 where the filter
 *             cannot decide); a leaf pair's triangle distance runs on one lane.
 *
 * Tested pairs live in records: the pair's exact transform (global scratch)
 * and its two children in the reference's visiting order with their
 * certified d and mint (shared memory).  Records the replay will not reach
 * (pruned ancestors) are freed with their subtree; a generation count per
 * record tells the speculation queue which of its entries went stale.
 *
 * Exact FP64 values are produced only where a decision needs them: an
 * undecided comparison, the step's final distance, and the step's minimum
 * mint, which is evaluated at the end of the step over the few contributions
 * whose certified interval can still be the minimum (the reference's mint is
 * a plain minimum and no decision reads it, C2A.cpp:1290-1311).  The
 * counters, the order and every decision are the reference's, so the results
 * are bit-identical to the sequential kernels'.
 */
#ifndef C2A_CA_SPEC_CUH
#define C2A_CA_SPEC_CUH

#include "ca_warp.cuh"

namespace c2a {

constexpr int kSpecSlots = 16; /* candidates per round: two lanes each */
#ifndef C2A_SPEC_QUEUE
#define C2A_SPEC_QUEUE 128
#endif
constexpr int kSpecQueue = C2A_SPEC_QUEUE; /* speculation queue (ring of entry references) */
constexpr int kSpecMinCand = 8;            /* deferred minimum-mint candidates */
constexpr uint32_t kSpecRoot = 0xfffffffeu;
constexpr uint32_t kSpecNone = 0xffffffffu;

enum : uint16_t {
    SF_EXACT = 1,  /* the exact d and mint are in the record's global part */
    SF_LEAF = 2,   /* both nodes are leaves: the pair's task is a triangle distance */
    SF_DONE = 4,   /* leaf: tri and lm hold its certified distance and mint */
    SF_LBAD = 8,   /* leaf: the filter could not certify the triangle distance */
    SF_MBAD = 16,  /* leaf: ... nor its mint */
    SF_USED = 32,   /* the replay has decided this pair */
    SF_FLIGHT = 64, /* a candidate of the current round */
    SF_LEXACT = 128 /* leaf: the exact triangle distance and leaf mint are in the record's global part */
};

/* a child pair of a record (shared memory, 48 bytes) */
struct SpecEnt {
    int32_t b1, b2;
    EF d, m;     /* certified views of the pair's d and mint (tight views once exact) */
    EF tri, lm;  /* leaf pairs: certified triangle distance and leaf mint */
    int16_t exp; /* record of this pair's own expansion, -1: not expanded */
    uint16_t flags;
    int32_t pad;
};

/* the tested children of one expanded pair (shared memory) */
struct SpecRec {
    int32_t gen;  /* bumped at every allocation and free */
    int32_t side; /* 0: the children split A's node, 1: B's */
    int32_t b1, b2;
    SpecEnt ent[2]; /* [0] visited first (the closer), [1] second */
};

/* the same record's FP64 part (global scratch) */
struct SpecRecG {
    double R[9], T[3];   /* the expanded pair's exact transform */
    double dx[2], mx[2]; /* the children's exact d and mint (SF_EXACT) */
    double tx[2], tm[2]; /* leaf children: exact triangle distance and leaf mint (SF_LEXACT) */
};

/* a contribution to the step's mint that may be the minimum (global scratch) */
struct SpecMinCand {
    int32_t kind; /* 0: a child pair placed from (R, T) by side; 1: a leaf pair */
    int32_t b1, b2, side;
    float lo, pad;
    double R[9], T[3];
};

/* per-warp shared state; the records, the free list, the kill stack and the
 * replay stack follow it (spec_shared_bytes) */
struct SpecShared {
    int32_t nrec, nfree, qhead, qcount;
    int32_t bad, pad_[3]; /* a checked build's first failed index check (site code), else 0 */
    uint32_t qref[kSpecQueue];
    uint32_t qgen[kSpecQueue];
    uint32_t cref[kSpecSlots];
    int32_t cnew[kSpecSlots];
};

__host__ __device__ constexpr size_t spec_align16(size_t x) { return (x + 15) / 16 * 16; }
/* bytes of one warp's speculation state with nrec records */
__host__ __device__ constexpr size_t spec_shared_bytes(int nrec)
{
    return spec_align16(sizeof(SpecShared)) + spec_align16(sizeof(SpecRec) * (size_t)nrec) +
           spec_align16(sizeof(int16_t) * (size_t)nrec) * 2 + spec_align16(sizeof(uint32_t) * (size_t)nrec);
}
/* global scratch of one warp */
__host__ __device__ constexpr size_t spec_global_bytes(int nrec)
{
    return sizeof(SpecRecG) * (size_t)nrec + sizeof(SpecMinCand) * kSpecMinCand;
}

/* the warp's view of its speculation state; the replay's registers */
struct SpecCtx {
    SpecShared *sh;
    SpecRec *rec;
    int16_t *freel, *kill;
    uint32_t *rstack;
    SpecRecG *g;
    SpecMinCand *mc;
    int nrec; /* records in the pool */
#ifdef C2A_STATS
    const Query *qs; /* the query whose counters the bookkeeping adds to */
    int qpeak, recpeak;
#endif
    /* replay state (identical on every lane) */
    uint32_t cur;     /* the pair the replay descends into next (kSpecRoot, kSpecNone or a reference) */
    int rsp;          /* replay stack depth */
    int root_rec;     /* the root pair's record once expanded */
    int pending_free; /* record whose second child the replay entered before its test was there */
    /* the running distance: certified view, exact value when known, and the pair that set it */
    EF dist_e;
    double dist_x;
    bool dist_exact;
    int dist_b1, dist_b2; /* -1: the step's seed pair */
    /* the step's mint: exact minimum so far, the certified upper bound of
     * the deferred ones, and how many are deferred */
    double mint_x;
    float mint_hi;
    int nmc;
    int overflow; /* 0, or why the step gave up (a code for the status word) */
};

/* Checked builds (C2A_SPEC_CHECK) verify every record reference and node or
 * triangle index before use; a failure records a site code, the access goes
 * to index 0 instead and the step ends with a status. */
#ifdef C2A_SPEC_CHECK
#define C2A_SPEC_OK(c, cond, site) ((cond) ? true : ((c).sh->bad == 0 ? ((c).sh->bad = (site)) : 0, false))
#else
#define C2A_SPEC_OK(c, cond, site) true
#endif

C2A_KDEV SpecEnt &spec_ent(const SpecCtx &c, uint32_t ref)
{
    if (!C2A_SPEC_OK(c, (int)(ref >> 1) < c.nrec, 10)) ref = 0;
    return c.rec[ref >> 1].ent[ref & 1];
}
C2A_KDEV bool spec_pair_ok(const SpecCtx &c, const Query &q, int b1, int b2, int site)
{
    return C2A_SPEC_OK(c, b1 >= 0 && b1 < q.A->num_nodes && b2 >= 0 && b2 < q.B->num_nodes, site);
}

C2A_KDEV void spec_layout(SpecCtx &c, unsigned char *smem, unsigned char *gmem, int nrec)
{
    c.sh = reinterpret_cast<SpecShared *>(smem);
    size_t o = spec_align16(sizeof(SpecShared));
    c.rec = reinterpret_cast<SpecRec *>(smem + o);
    o += spec_align16(sizeof(SpecRec) * (size_t)nrec);
    c.freel = reinterpret_cast<int16_t *>(smem + o);
    o += spec_align16(sizeof(int16_t) * (size_t)nrec);
    c.kill = reinterpret_cast<int16_t *>(smem + o);
    o += spec_align16(sizeof(int16_t) * (size_t)nrec);
    c.rstack = reinterpret_cast<uint32_t *>(smem + o);
    c.g = reinterpret_cast<SpecRecG *>(gmem);
    c.mc = reinterpret_cast<SpecMinCand *>(gmem + sizeof(SpecRecG) * (size_t)nrec);
    c.nrec = nrec;
}

/* every record free, queue empty (start of a step); generations carry on */
C2A_KDEV void spec_reset(SpecCtx &c, int nrec, int lane)
{
    __syncwarp();
    for (int i = lane; i < nrec; i += 32) c.freel[i] = (int16_t)(nrec - 1 - i);
    if (lane == 0) {
        c.sh->nrec = nrec;
        c.sh->nfree = nrec;
        c.sh->qhead = 0;
        c.sh->qcount = 0;
        c.sh->bad = 0;
    }
    __syncwarp();
}

/* ---- records (every lane runs these with the same values) */

C2A_KDEV int spec_alloc(SpecCtx &c)
{
    const int n = c.sh->nfree;
    if (n <= 0) return -1;
    const int r = c.freel[n - 1];
    SpecRec &x = c.rec[r];
    C2A_WSET(c.sh->nfree, n - 1);
    C2A_WSET(x.gen, x.gen + 1);
    return r;
}

C2A_KDEV void spec_free(SpecCtx &c, int r)
{
    const int n = c.sh->nfree;
    const int g = c.rec[r].gen;
    if (n >= c.nrec) { /* never with a consistent pool: refuse rather than write past the list */
        c.overflow = 4;
        return;
    }
    C2A_WSET(c.rec[r].gen, g + 1);
    C2A_WSET(c.freel[n], (int16_t)r);
    C2A_WSET(c.sh->nfree, n + 1);
}

/* frees record r and every record below it (speculation the replay will not use) */
C2A_KDEV void spec_free_subtree(SpecCtx &c, int r)
{
    const int cap = c.nrec;
    int ks = 0, guard = 0;
    C2A_WSET(c.kill[ks], (int16_t)r);
    ks++;
    while (ks > 0) {
        if (++guard > cap) { /* more records than the pool holds: a cycle, never with a consistent pool */
            c.overflow = 5;
            return;
        }
        const int x = c.kill[--ks];
        const int e0 = c.rec[x].ent[0].exp, e1 = c.rec[x].ent[1].exp;
        if (e0 >= 0 && ks < cap) {
            C2A_WSET(c.kill[ks], (int16_t)e0);
            ks++;
        }
        if (e1 >= 0 && ks < cap) {
            C2A_WSET(c.kill[ks], (int16_t)e1);
            ks++;
        }
        spec_free(c, x);
    }
}

/* ---- speculation queue */

C2A_KDEV void spec_q_push_front(SpecCtx &c, uint32_t ref, uint32_t gen)
{
    int h = c.sh->qhead, n = c.sh->qcount;
    h = (h + kSpecQueue - 1) % kSpecQueue;
    if (n < kSpecQueue) n++; /* full: the entry furthest in the order falls off the back */
    C2A_WSET(c.sh->qref[h], ref);
    C2A_WSET(c.sh->qgen[h], gen);
    C2A_WSET(c.sh->qhead, h);
    C2A_WSET(c.sh->qcount, n);
}

/* ------------------------------------------------------- exact pieces */

/* makes entry ref's d and mint exact (FP64 on the warp, from its record's transform) */
C2A_KDEV void spec_make_exact(const Query &q, SpecCtx &c, uint32_t ref, int lane)
{
    SpecEnt &e = spec_ent(c, ref);
    if (e.flags & SF_EXACT) return;
    C2A_WSTAT(q, ST_S_MKEXACT, 1);
    const int r = (int)(ref >> 1), s = (int)(ref & 1);
    M3 PR, R;
    V3 PT, T;
#pragma unroll
    for (int i = 0; i < 9; i++) PR.m[i] = c.g[r].R[i];
    PT = v3(c.g[r].T[0], c.g[r].T[1], c.g[r].T[2]);
    int b1 = e.b1, b2 = e.b2;
    if (!spec_pair_ok(c, q, b1, b2, 11)) b1 = b2 = 0;
    child_transform(q, c.rec[r].side, b1, b2, PR, PT, R, T);
    double d, m;
    child_test_x(q, b1, b2, R, T, d, m, lane);
    EFCtx cc{false};
    EF de = in_d(d, cc), me = in_d(m, cc);
    if (cc.bad) de = me = EF{0.0f, __int_as_float(0x7f800000)};
    __syncwarp();
    if (lane == 0) {
        c.g[r].dx[s] = d;
        c.g[r].mx[s] = m;
    }
    C2A_WSET(e.d, de);
    C2A_WSET(e.m, me);
    C2A_WSET(e.flags, (uint16_t)(e.flags | SF_EXACT));
}

/* the running distance's exact value (the triangle pair that set it, in FP64) */
C2A_KDEV void spec_exact_distance(Query &q, SpecCtx &c, int lane)
{
    if (c.dist_exact) return;
    C2A_WSTAT(q, ST_S_DISTX, 1);
    if (!spec_pair_ok(c, q, c.dist_b1, c.dist_b2, 12)) c.dist_b1 = c.dist_b2 = 0;
    const int fc1 = __ldg(&q.A->nodes[c.dist_b1].first_child), fc2 = __ldg(&q.B->nodes[c.dist_b2].first_child);
    V3 p, qq;
    TriFeat f;
    bool col = false;
    c.dist_x = tri_distance_warp(q, -fc1 - 1, -fc2 - 1, p, qq, f, col, lane);
    c.dist_exact = true;
    q.distance = c.dist_x;
    refresh_shadows(q);
    c.dist_e = q.distance_e;
}

/* the exact mint of a leaf pair whose triangle distance is dTri with closest points p, qq (C2A.cpp:1152-1170) */
C2A_KDEV double spec_leaf_mint_x(const Query &q, int b1, int b2, double dTri, V3 p, V3 qq)
{
    ExactCtx xc{false};
    const V3 res1 = mul(q.r1, p) + q.t1;
    const V3 res2 = mul(q.r1, qq) + q.t1;
    V3 S1 = res2 - res1;
    V3 S2 = mul_s(S1, -1.0);
    const double mb1 = bound_leaf(q.x1, __ldg(&q.A->nodes[b1].angR), S1, xc);
    const double mb2 = bound_leaf(q.x2, __ldg(&q.B->nodes[b2].angR), S2, xc);
    double mint = (dTri) / (mb1 + mb2);
    if (mint < 0.0) mint = 0.0;
    return mint;
}

/* exact value of a deferred minimum candidate */
C2A_KDEV double spec_min_cand_x(Query &q, const SpecMinCand &k, int lane)
{
    if (k.kind == 1) {
        const int fc1 = __ldg(&q.A->nodes[k.b1].first_child), fc2 = __ldg(&q.B->nodes[k.b2].first_child);
        V3 p, qq;
        TriFeat f;
        bool col = false;
        const double dTri = tri_distance_warp(q, -fc1 - 1, -fc2 - 1, p, qq, f, col, lane);
        return spec_leaf_mint_x(q, k.b1, k.b2, dTri, p, qq);
    }
    M3 PR, R;
    V3 PT, T;
#pragma unroll
    for (int i = 0; i < 9; i++) PR.m[i] = k.R[i];
    PT = v3(k.T[0], k.T[1], k.T[2]);
    child_transform(q, k.side, k.b1, k.b2, PR, PT, R, T);
    double d, m;
    child_test_x(q, k.b1, k.b2, R, T, d, m, lane);
    return m;
}

/* every deferred candidate that can still be the minimum, exactly: one
 * whose lower bound is not below the exact minimum so far, or not below
 * another candidate's upper bound (that one is evaluated), cannot lower it */
C2A_KDEV void spec_flush_mint(Query &q, SpecCtx &c, int lane)
{
    for (int i = 0; i < c.nmc; i++) {
        const float lo = c.mc[i].lo;
        if (!((double)lo < c.mint_x && lo < c.mint_hi)) continue;
        C2A_WSTAT(q, ST_S_FLUSHX, 1);
        const double v = spec_min_cand_x(q, c.mc[i], lane);
        if (v < c.mint_x) c.mint_x = v;
    }
    c.nmc = 0;
    c.mint_hi = __int_as_float(0x7f800000);
}

/* a contribution of certified value m (not exact) from child (b1, b2) of the
 * pair placed by record r's transform, or from a leaf pair (kind 1) */
C2A_KDEV void spec_defer(Query &q, SpecCtx &c, int kind, int r, int b1, int b2, EF m, int lane)
{
    const float lo = efr_sub_rd(m.v, m.e), hi = efr_add_ru(m.v, m.e);
    if (!((double)lo < c.mint_x && lo < c.mint_hi)) return; /* cannot lower the minimum */
    if (c.nmc >= kSpecMinCand) spec_flush_mint(q, c, lane);
    SpecMinCand &k = c.mc[c.nmc];
    __syncwarp();
    if (lane == 0) {
        k.kind = kind;
        k.b1 = b1;
        k.b2 = b2;
        k.side = kind == 0 ? c.rec[r].side : 0;
        k.lo = lo;
    }
    if (kind == 0 && lane < 12) {
        if (lane < 9) k.R[lane] = c.g[r].R[lane];
        else k.T[lane - 9] = c.g[r].T[lane - 9];
    }
    __syncwarp();
    c.nmc++;
    if (hi < c.mint_hi) c.mint_hi = hi;
}

/* ------------------------------------------------------------- replay */

/* mint < UpboundTOC && (d < distance - abs_err || d * (1 + rel_err) < distance) (C2A.cpp:1281-1351) */
C2A_KDEV bool spec_descend(Query &q, SpecCtx &c, uint32_t ref, int lane)
{
    {
        const SpecEnt &e = spec_ent(c, ref);
        const int a = ef_lt3(e.m, q.upbound_e);
        const int b = ef_lt3(e.d, q.bound_e);
        const int d = ef_lt3(e.d * q.rel1_e, c.dist_e);
        const int r = and3(a, or3(b, d));
        if (r >= 0) return r == 1;
    }
    spec_make_exact(q, c, ref, lane);
    spec_exact_distance(q, c, lane);
    const int r = (int)(ref >> 1), s = (int)(ref & 1);
    const double dx = c.g[r].dx[s], mx = c.g[r].mx[s];
    return mx < q.upbound && ((dx < (q.distance - q.abs_err)) || (dx * (1 + q.rel_err) < q.distance));
}

/* a pruned pair's mint lowers res->mint (C2A.cpp:1290-1311) */
C2A_KDEV void spec_contribute(Query &q, SpecCtx &c, uint32_t ref, int lane)
{
    const SpecEnt &e = spec_ent(c, ref);
    const int r = (int)(ref >> 1), s = (int)(ref & 1);
    if (e.flags & SF_EXACT) {
        const double mx = c.g[r].mx[s];
        if (mx < c.mint_x) c.mint_x = mx;
        return;
    }
    spec_defer(q, c, 0, r, e.b1, e.b2, e.m, lane);
}

/* a leaf pair of the step (C2A.cpp:1141-1183) whose certified distance is known */
C2A_KDEV void spec_leaf(Query &q, SpecCtx &c, uint32_t ref, int lane)
{
    q.ntri++;
    const SpecEnt &e = spec_ent(c, ref);
    int b1 = e.b1, b2 = e.b2;
    if (!spec_pair_ok(c, q, b1, b2, 13)) b1 = b2 = 0;
    const uint16_t fl = e.flags;
    if (fl & SF_LEXACT) { /* the lane computed it in FP64: the reference's comparison directly */
        const double dTri = c.g[ref >> 1].tx[ref & 1], mint = c.g[ref >> 1].tm[ref & 1];
        spec_exact_distance(q, c, lane);
        if (dTri <= q.distance) {
            q.distance = dTri;
            c.dist_x = dTri;
            c.dist_exact = true;
            c.dist_b1 = b1;
            c.dist_b2 = b2;
            if (mint <= c.mint_x) c.mint_x = mint;
            refresh_shadows(q);
            c.dist_e = q.distance_e;
        }
        return;
    }
    const EF tri = e.tri, lm = e.lm;
    const int le = (fl & SF_LBAD) ? -1 : ef_le3(tri, c.dist_e);
    if (le == 0) return;
    if (le == 1 && !(fl & SF_MBAD)) { /* certainly dTri <= distance: the distance is this pair's now */
        c.dist_e = tri;
        c.dist_exact = false;
        c.dist_b1 = b1;
        c.dist_b2 = b2;
        q.distance_e = tri;
        EFCtx bc{false};
        q.bound_e = tri - in_d(q.abs_err, bc); /* distance - abs_err, certified like every other bound */
        spec_defer(q, c, 1, 0, b1, b2, lm, lane);
        return;
    }
    /* undecided: the reference's comparison in FP64 */
    C2A_WSTAT(q, ST_S_LEAFX, 1);
    const int fc1 = __ldg(&q.A->nodes[b1].first_child), fc2 = __ldg(&q.B->nodes[b2].first_child);
    V3 p, qq;
    TriFeat f;
    bool col = false;
    const double dTri = tri_distance_warp(q, -fc1 - 1, -fc2 - 1, p, qq, f, col, lane);
    spec_exact_distance(q, c, lane);
    if (dTri <= q.distance) {
        q.distance = dTri;
        c.dist_x = dTri;
        c.dist_exact = true;
        c.dist_b1 = b1;
        c.dist_b2 = b2;
        const double mint = spec_leaf_mint_x(q, b1, b2, dTri, p, qq);
        if (mint <= c.mint_x) c.mint_x = mint;
        refresh_shadows(q);
        c.dist_e = q.distance_e;
    }
}

/* pushes a record's children onto the speculation queue (first ends up in front) */
C2A_KDEV void spec_q_children(SpecCtx &c, int r)
{
    const uint32_t g = (uint32_t)c.rec[r].gen;
    spec_q_push_front(c, ((uint32_t)r << 1) | 1u, g);
    spec_q_push_front(c, ((uint32_t)r << 1), g);
}

/* marks a decided entry; a pruned one's speculative subtree is freed */
C2A_KDEV void spec_mark_used(SpecCtx &c, uint32_t ref, bool pruned)
{
#ifdef C2A_STATS
    C2A_WSTAT(*c.qs, ST_S_DECIDED, 1);
#endif
    SpecEnt &e = spec_ent(c, ref);
    const int x = e.exp;
    C2A_WSET(e.flags, (uint16_t)(e.flags | SF_USED));
    if (pruned && x >= 0) {
        C2A_WSET(e.exp, (int16_t)-1);
        spec_free_subtree(c, x);
    }
}

/* frees the record kept for a descended second child once that child's own
 * task has been read */
C2A_KDEV void spec_release_pending(SpecCtx &c)
{
    if (c.pending_free >= 0) {
        spec_free(c, c.pending_free);
        c.pending_free = -1;
    }
}

/* walks the reference's order until a pair's test is missing; returns the
 * due pair (kSpecNone when the step is complete).  c.cur is the pair to
 * descend into next (already decided) or kSpecNone. */
C2A_KDEV uint32_t spec_replay(Query &q, SpecCtx &c, int lane)
{
    for (;;) {
        if (c.cur != kSpecNone) {
            int x;
            if (c.cur == kSpecRoot) {
                if (c.root_rec < 0) return kSpecRoot;
                x = c.root_rec;
            } else {
                const SpecEnt &e = spec_ent(c, c.cur);
                const uint16_t fl = e.flags;
                if (fl & SF_LEAF) {
                    if (!(fl & SF_DONE)) return c.cur;
                    spec_leaf(q, c, c.cur, lane);
                    spec_release_pending(c);
                    c.cur = kSpecNone;
                    x = -1;
                } else {
                    x = e.exp;
                    if (x < 0) return c.cur;
                    spec_release_pending(c);
                }
            }
            if (x >= 0) {
                /* enter x: its children were tested (C2A.cpp:1237-1279) */
                q.nbv += 2;
                if (c.rsp >= c.nrec) {
                    c.overflow = 1;
                    return kSpecNone;
                }
                C2A_WSET(c.rstack[c.rsp], ((uint32_t)x << 1) | 1u);
                c.rsp++;
                const uint32_t f = (uint32_t)x << 1;
                if (spec_descend(q, c, f, lane)) {
                    spec_mark_used(c, f, false);
                    c.cur = f;
                    continue;
                }
                spec_contribute(q, c, f, lane);
                spec_mark_used(c, f, true);
                c.cur = kSpecNone;
            }
        }
        /* pop pending second children */
        while (c.cur == kSpecNone && c.rsp > 0) {
            const uint32_t s = c.rstack[--c.rsp];
            const int r = (int)(s >> 1);
            if (spec_descend(q, c, s, lane)) {
                spec_mark_used(c, s, false);
                c.cur = s;
                c.pending_free = r; /* freed once s's own task has been read */
            } else {
                spec_contribute(q, c, s, lane);
                spec_mark_used(c, s, true);
                spec_free(c, r);
            }
        }
        if (c.cur == kSpecNone) return kSpecNone;
    }
}

/* frees every speculative record (those below the replay's pending second
 * children): makes room for the due pair when speculation filled the pool */
C2A_KDEV void spec_evict(SpecCtx &c)
{
    for (int i = 0; i < c.rsp; i++) {
        SpecEnt &e = spec_ent(c, c.rstack[i]);
        const int x = e.exp;
        if (x >= 0) {
            C2A_WSET(e.exp, (int16_t)-1);
            spec_free_subtree(c, x);
        }
    }
}

/* ------------------------------------------------------------ speculate */

/* the due pair and up to kSpecSlots - 1 more pairs the current distance
 * would descend into, in the reference's order; returns how many */
C2A_KDEV int spec_collect(Query &q, SpecCtx &c, uint32_t due)
{
    SpecShared &sh = *c.sh;
    int n = 0;
    /* one record stays free for the next round's due pair */
    auto take = [&](uint32_t ref, bool leaf) -> bool {
        int nr = -1;
        if (!leaf) {
            const bool is_due = ref == due;
            if (is_due && sh.nfree < 1) spec_evict(c);
            if (sh.nfree < (is_due ? 1 : 2)) return false;
            nr = spec_alloc(c);
        }
        C2A_WSET(sh.cref[n], ref);
        C2A_WSET(sh.cnew[n], nr);
        if (ref != kSpecRoot) {
            SpecEnt &e = spec_ent(c, ref);
            C2A_WSET(e.flags, (uint16_t)(e.flags | SF_FLIGHT));
        }
        n++;
        return true;
    };
    if (due == kSpecRoot) {
        if (!take(due, false)) return 0;
    } else if (!take(due, (spec_ent(c, due).flags & SF_LEAF) != 0)) {
        return 0;
    }
    while (n < kSpecSlots && sh.qcount > 0) {
        const int h = sh.qhead;
        const uint32_t ref = sh.qref[h], gen = sh.qgen[h];
        const SpecRec &r = c.rec[ref >> 1];
        const SpecEnt &e = r.ent[ref & 1];
        const bool stale = (uint32_t)r.gen != gen;
        const uint16_t fl = e.flags;
        bool skip = stale || (fl & (SF_USED | SF_FLIGHT | SF_DONE)) || e.exp >= 0;
#ifdef C2A_STATS
        if (stale) C2A_WSTAT(q, ST_S_Q_STALE, 1);
        else if (skip) C2A_WSTAT(q, ST_S_Q_SEEN, 1);
#endif
        if (!skip) { /* the current distance decides; undecided counts as descend */
            const int a = ef_lt3(e.m, q.upbound_e);
            const int b = ef_lt3(e.d, q.bound_e);
            const int d = ef_lt3(e.d * q.rel1_e, c.dist_e);
            skip = and3(a, or3(b, d)) == 0;
            if (skip) C2A_WSTAT(q, ST_S_Q_PRUNED, 1);
        }
        if (!skip && !(fl & SF_LEAF) && sh.nfree < 2) { /* no record to spare: stop here */
            C2A_WSTAT(q, ST_S_STOP_POOL, 1);
            break;
        }
        C2A_WSET(sh.qhead, (h + 1) % kSpecQueue);
        C2A_WSET(sh.qcount, sh.qcount - 1);
        if (!skip) take(ref, (fl & SF_LEAF) != 0);
    }
    if (n < kSpecSlots && sh.qcount == 0) C2A_WSTAT(q, ST_S_STOP_EMPTY, 1);
    return n;
}

/* ----------------------------------------------------------------- test */

/* the leaf task of one lane: certified triangle distance and leaf mint
 * (C2A_SPEC_FP64: the exact ones) */
C2A_KDEV void spec_leaf_task(const Query &q, SpecCtx &sc, uint32_t ref)
{
    SpecEnt &e = spec_ent(sc, ref);
    int b1 = e.b1, b2 = e.b2;
    if (!spec_pair_ok(sc, q, b1, b2, 14)) b1 = b2 = 0;
    int ia = -__ldg(&q.A->nodes[b1].first_child) - 1, ib = -__ldg(&q.B->nodes[b2].first_child) - 1;
    if (!C2A_SPEC_OK(sc, ia >= 0 && ia < q.A->num_tris && ib >= 0 && ib < q.B->num_tris, 15)) ia = ib = 0;
#ifdef C2A_SPEC_FP64
    {
        V3 p, qq;
        TriFeat f;
        bool col = false;
        const double dTri = tri_distance_x(q, ia, ib, p, qq, f, col);
        const int r = (int)(ref >> 1), s = (int)(ref & 1);
        sc.g[r].tx[s] = dTri;
        sc.g[r].tm[s] = spec_leaf_mint_x(q, b1, b2, dTri, p, qq);
        e.flags = (uint16_t)((e.flags & ~SF_FLIGHT) | SF_DONE | SF_LEXACT);
        return;
    }
#endif
    EFCtx c{!q.shadows_ok};
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
    uint16_t fl = SF_DONE;
    EF lm = ef_exact(0.0f);
    if (c.bad || col) {
        fl |= SF_LBAD | SF_MBAD;
    } else {
        EFCtx mc{false};
        const V3T<EF> t1e = ef_v3(q.t1, mc);
        const V3T<EF> res1 = mul(q.r1e, p) + t1e;
        const V3T<EF> res2 = mul(q.r1e, qq) + t1e;
        V3T<EF> S1 = res2 - res1;
        V3T<EF> S2 = mul_s(S1, ef_exact(-1.0f));
        const EF ar1 = ef_shadow(__ldg(&q.A->snodes[b1].angR)), ar2 = ef_shadow(__ldg(&q.B->snodes[b2].angR));
        const EF mb1 = bound_leaf(q.e1, ar1, S1, mc);
        const EF mb2 = bound_leaf(q.e2, ar2, S2, mc);
        lm = max0_c(ef_div(dTri, mb1 + mb2, mc));
        if (mc.bad) fl |= SF_MBAD;
    }
    e.tri = dTri;
    e.lm = lm;
    e.flags = (uint16_t)((e.flags & ~SF_FLIGHT) | fl);
}

/* C2A_BV_Distance and both motion bounds of child pair (x1, x2) of a pair
 * placed by (PRe, PTe) (C2A.cpp:1195-1274), through the certified FP32
 * filter on one lane: the child transform, RectDist with the cases through
 * one code path (rect_dist_lane), d = max(z, 0) and mint.  Returns false
 * when a decision cannot be certified (the caller recomputes in FP64). */
C2A_KDEV bool spec_bv_test_e(const Query &q, int side, const M3T<EF> &PRe, V3T<EF> PTe, int x1, int x2, EF &d,
                             EF &mint, bool &d_zero)
{
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
    const EF z = rect_dist_lane(R, T, n1.l, n2.l, S, c) - (n1.r + n2.r);
    if (c.bad) return false;
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
    V3T<EF> S1 = mul(q.r1e, mul(n1.Rloc, S));
    V3T<EF> S2 = mul_s(S1, ef_exact(-1));
    const EF mb1 = bound_rss(q.e1, n1.angR, S1, c);
    const EF mb2 = bound_rss(q.e2, n2.angR, S2, c);
    mint = max0_c(ef_div(d, mb1 + mb2, c));
    return !c.bad;
}

/* one output of a child transform (the expression trees of tmmul/tmul for
 * side 0, mmul/mul_add for side 1): k < 9 R.m[k], else T[k - 9] */
C2A_KDEV double spec_xform_out(int side, int k, const M3 &Rc, V3 Tr, const M3 &PR, V3 PT)
{
    const bool isT = k >= 9;
    const int i = isT ? k - 9 : k / 3, j = isT ? 0 : k % 3;
    double a0, a1, a2, b0, b1, b2, cc = 0.0;
    if (side == 0) { /* R = Rc^T PR, T = Rc^T (PT - Tr) */
        a0 = Rc.m[i];
        a1 = Rc.m[3 + i];
        a2 = Rc.m[6 + i];
        const V3 v = PT - Tr;
        b0 = isT ? v.x : PR.m[j];
        b1 = isT ? v.y : PR.m[3 + j];
        b2 = isT ? v.z : PR.m[6 + j];
    } else { /* R = PR Rc, T = PR Tr + PT */
        a0 = PR.m[3 * i];
        a1 = PR.m[3 * i + 1];
        a2 = PR.m[3 * i + 2];
        b0 = isT ? Tr.x : Rc.m[j];
        b1 = isT ? Tr.y : Rc.m[3 + j];
        b2 = isT ? Tr.z : Rc.m[6 + j];
        cc = i == 0 ? PT.x : (i == 1 ? PT.y : PT.z);
    }
    double v = a0 * b0 + a1 * b1 + a2 * b2;
    if (side == 1 && isT) v = v + cc;
    return v;
}

/* lanes 2i, 2i+1 expand candidate i; a leaf candidate's triangle distance
 * runs on lane 2i afterwards.  Every lane takes part in every shuffle: lanes
 * without an expansion (beyond the candidates, or holding a leaf) expand the
 * root pair as a stand-in and write nothing. */
C2A_KDEV void spec_expand(const Query &q, SpecCtx &c, int ncand, const M3 &Rroot, V3 Troot, int lane)
{
    const int slot = lane >> 1, sub = lane & 1;
    const bool live = slot < ncand;
    const int ci = live ? slot : 0;
    const uint32_t ref = c.sh->cref[ci];
    const int nr = c.sh->cnew[ci];
    const bool is_leaf = live && nr < 0;
    const bool do_exp = live && nr >= 0;
    const bool stand_in = !do_exp || ref == kSpecRoot;
    /* the pair's exact transform: six outputs per lane, then shared */
    int b1 = 0, b2 = 0;
    double o[6];
    if (stand_in) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const int j = 6 * sub + k;
            o[k] = j < 9 ? Rroot.m[j] : (j == 9 ? Troot.x : (j == 10 ? Troot.y : Troot.z));
        }
    } else {
        const SpecEnt &e = spec_ent(c, ref);
        b1 = e.b1;
        b2 = e.b2;
        if (!spec_pair_ok(c, q, b1, b2, 16)) b1 = b2 = 0;
        const int pr = (int)(ref >> 1) < c.nrec ? (int)(ref >> 1) : 0, side = c.rec[pr].side;
        M3 PR;
#pragma unroll
        for (int i = 0; i < 9; i++) PR.m[i] = c.g[pr].R[i];
        const V3 PT = v3(c.g[pr].T[0], c.g[pr].T[1], c.g[pr].T[2]);
        const NodeRec *n = side == 0 ? q.A->nodes + b1 : q.B->nodes + b2;
        const M3 Rc = load_R(n);
        const V3 Tr = load_Tr(n);
#pragma unroll
        for (int k = 0; k < 6; k++) o[k] = spec_xform_out(side, 6 * sub + k, Rc, Tr, PR, PT);
    }
    double w[6];
#pragma unroll
    for (int k = 0; k < 6; k++) w[k] = __shfl_xor_sync(kWFull, o[k], 1);
    M3 R;
    V3 T;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        R.m[k] = sub == 0 ? o[k] : w[k];
        const double hi = sub == 0 ? w[k] : o[k];
        if (k < 3) R.m[6 + k] = hi;
        else if (k == 3) T.x = hi;
        else if (k == 4) T.y = hi;
        else T.z = hi;
    }
    if (do_exp) {
        if (sub == 0) {
#pragma unroll
            for (int k = 0; k < 6; k++) c.g[nr].R[k] = R.m[k];
        } else {
            c.g[nr].R[6] = R.m[6];
            c.g[nr].R[7] = R.m[7];
            c.g[nr].R[8] = R.m[8];
            c.g[nr].T[0] = T.x;
            c.g[nr].T[1] = T.y;
            c.g[nr].T[2] = T.z;
        }
    }
    /* the children (C2A.cpp:1192-1226); this lane tests child `sub` */
    const int fc1 = __ldg(&q.A->nodes[b1].first_child), fc2 = __ldg(&q.B->nodes[b2].first_child);
    int side, a1, a2, c1, c2;
    split_pair(q, b1, b2, fc1, fc2, side, a1, a2, c1, c2);
    int x1 = sub ? c1 : a1, x2 = sub ? c2 : a2;
    if (!spec_pair_ok(c, q, x1, x2, 17)) x1 = x2 = 0;
    EFCtx ec{!q.shadows_ok};
    const M3T<EF> Re = ef_m3(R, ec);
    const V3T<EF> Te = ef_v3(T, ec);
    EF d = ef_exact(0.0f), m = ef_exact(0.0f);
    bool dz = false;
#ifdef C2A_STATS
    __syncwarp();
    C2A_WCLOCK(x1c);
#endif
#ifdef C2A_SPEC_FP64
    const bool ok = false; /* every lane test in FP64 */
    (void)Re;
    (void)Te;
#else
    const bool ok = !ec.bad && spec_bv_test_e(q, side, Re, Te, x1, x2, d, m, dz);
#endif
#ifdef C2A_STATS
    {
        const int nx = __popc(__ballot_sync(kWFull, do_exp && !ok));
        C2A_WSTAT(q, ST_S_LANEX, nx);
    }
#endif
    bool exact = false;
    double dx = 0.0, mx = 0.0;
    if (!ok) {
        M3 Rx;
        V3 Tx;
        child_transform(q, side, x1, x2, R, T, Rx, Tx);
        bv_test_x(q, Rx, Tx, x1, x2, dx, mx);
        exact = true;
    } else if (dz) {
        exact = true; /* d = max(z, 0) = 0 and mint = 0 exactly */
    }
    if (exact) {
        EFCtx cc{false};
        d = in_d(dx, cc);
        m = in_d(mx, cc);
        if (cc.bad) d = m = EF{0.0f, __int_as_float(0x7f800000)};
    }
#ifdef C2A_STATS
    __syncwarp();
    C2A_WCLOCK(x2c);
    C2A_WSTAT(q, ST_S_CYC_TEST, x2c - x1c);
#endif
    /* d2 < d1: child c (lane sub 1) first? (C2A.cpp:1281) */
    const EF dp = EF{__shfl_xor_sync(kWFull, d.v, 1), __shfl_xor_sync(kWFull, d.e, 1)};
    const EF da = sub ? dp : d, dc = sub ? d : dp;
    int cfirst = ef_lt3(dc, da);
    const bool need_x = __shfl_xor_sync(kWFull, (int)(cfirst < 0), 1) != 0 || cfirst < 0;
    if (need_x && !exact) { /* undecided order: both children exactly */
        M3 Rx;
        V3 Tx;
        child_transform(q, side, x1, x2, R, T, Rx, Tx);
        bv_test_x(q, Rx, Tx, x1, x2, dx, mx);
        exact = true;
        EFCtx cc{false};
        d = in_d(dx, cc);
        m = in_d(mx, cc);
        if (cc.bad) d = m = EF{0.0f, __int_as_float(0x7f800000)};
    }
    const double dxp = __shfl_xor_sync(kWFull, dx, 1);
    if (need_x) cfirst = (sub ? dx : dxp) < (sub ? dxp : dx) ? 1 : 0;
    if (do_exp) {
        const int pos = (cfirst == 1) ? (sub ? 0 : 1) : sub;
        const bool lleaf = __ldg(&q.A->nodes[x1].first_child) < 0 && __ldg(&q.B->nodes[x2].first_child) < 0;
        SpecEnt &o2 = c.rec[nr].ent[pos];
        o2.b1 = x1;
        o2.b2 = x2;
        o2.d = d;
        o2.m = m;
        o2.tri = ef_exact(0.0f);
        o2.lm = ef_exact(0.0f);
        o2.exp = -1;
        o2.flags = (uint16_t)((exact ? SF_EXACT : 0) | (lleaf ? SF_LEAF : 0));
        o2.pad = 0;
        if (exact) {
            c.g[nr].dx[pos] = dx;
            c.g[nr].mx[pos] = mx;
        }
        if (sub == 0) {
            c.rec[nr].side = side;
            c.rec[nr].b1 = b1;
            c.rec[nr].b2 = b2;
            if (ref != kSpecRoot) {
                SpecEnt &e = spec_ent(c, ref);
                e.exp = (int16_t)nr;
                e.flags = (uint16_t)(e.flags & ~SF_FLIGHT);
            }
        }
    }
    /* leaf candidates: the triangle distance on the slot's first lane */
#ifdef C2A_STATS
    __syncwarp();
    C2A_WCLOCK(x3c);
#endif
    if (is_leaf && sub == 0) spec_leaf_task(q, c, ref);
#ifdef C2A_STATS
    __syncwarp();
    C2A_WCLOCK(x4c);
    C2A_WSTAT(q, ST_S_CYC_LEAF, x4c - x3c);
#endif
}

/* ------------------------------------------------------------- the step */

/* TOCStepRecurse_Dis from the root pair (q.distance: the seed pair's exact
 * distance, q.mint = 1, schedule set): speculative rounds until the replay
 * completes; leaves q.distance and q.mint exact */
C2A_KDEV void spec_dfs(Query &q, const M3 &Rroot, V3 Troot, SpecCtx &c, int lane)
{
    spec_reset(c, c.nrec, lane);
    c.cur = kSpecRoot;
    c.rsp = 0;
    c.root_rec = -1;
    c.pending_free = -1;
    c.dist_e = q.distance_e;
    c.dist_x = q.distance;
    c.dist_exact = true;
    c.dist_b1 = c.dist_b2 = -1;
    c.mint_x = 1.0;
    c.mint_hi = __int_as_float(0x7f800000);
    c.nmc = 0;
    c.overflow = 0;
    /* a root pair of two leaves: one triangle each */
    if (__ldg(&q.A->nodes[0].first_child) < 0 && __ldg(&q.B->nodes[0].first_child) < 0) {
        leaf_step_warp(q, 0, 0, __ldg(&q.A->nodes[0].first_child), __ldg(&q.B->nodes[0].first_child), lane);
        return;
    }
#ifdef C2A_STATS
    c.qs = &q;
    c.qpeak = c.recpeak = 0;
#endif
    for (int round = 0;; round++) {
        C2A_WCLOCK(t0);
        const uint32_t due = spec_replay(q, c, lane);
        if (c.sh->bad) {
            c.overflow = 16 + c.sh->bad;
            break;
        }
        C2A_WCLOCK(t1);
        C2A_WSTAT(q, ST_S_CYC_REPLAY, t1 - t0);
        if (due == kSpecNone || c.overflow) break;
        if (round >= (1 << 24)) { /* far beyond any hierarchy's node pairs: give up with a status */
            c.overflow = 6;
            break;
        }
        const int n = spec_collect(q, c, due);
        if (c.overflow || n < 1) {
            c.overflow = 2;
            break;
        }
        C2A_WCLOCK(t2);
        C2A_WSTAT(q, ST_S_CYC_COLLECT, t2 - t1);
        C2A_WSTAT(q, ST_S_ROUNDS, 1);
        C2A_WSTAT(q, ST_S_CANDS, n);
#ifdef C2A_STATS
        if (c.sh->qcount > c.qpeak) c.qpeak = c.sh->qcount;
        if (c.nrec - c.sh->nfree > c.recpeak) c.recpeak = c.nrec - c.sh->nfree;
        for (int i = 0; i < n; i++)
            if (c.sh->cnew[i] < 0) C2A_WSTAT(q, ST_S_LEAFC, 1);
#endif
        __syncwarp();
        spec_expand(q, c, n, Rroot, Troot, lane);
        __syncwarp();
        C2A_WCLOCK(t3);
        C2A_WSTAT(q, ST_S_CYC_EXPAND, t3 - t2);
        if (c.sh->bad) { /* a checked build found an index out of range */
            c.overflow = 16 + c.sh->bad;
            break;
        }
        /* the due pair's task must be there now, or the replay would ask again */
        if (due != kSpecRoot) {
            const SpecEnt &e = spec_ent(c, due);
            if (e.exp < 0 && !(e.flags & SF_DONE)) {
                c.overflow = 3;
                break;
            }
        }
        /* the new records' children join the queue, in the order of the candidates */
        for (int i = n - 1; i >= 0; i--) {
            const int nr = c.sh->cnew[i];
            if (nr >= 0) spec_q_children(c, nr);
        }
        if (due == kSpecRoot) c.root_rec = c.sh->cnew[0];
    }
    if (c.overflow) {
        q.status |= C2A_QUERY_STACK_OVERFLOW | (c.overflow << 8);
        return;
    }
#ifdef C2A_STATS
    C2A_WSTAT(q, ST_S_QPEAK, c.qpeak);
    C2A_WSTAT(q, ST_S_RECPEAK, c.recpeak);
    C2A_WSTAT(q, ST_S_STEPS, 1);
#endif
    C2A_WCLOCK(e0);
    spec_flush_mint(q, c, lane);
    spec_exact_distance(q, c, lane);
    C2A_WCLOCK(e1);
    C2A_WSTAT(q, ST_S_CYC_END, e1 - e0);
    q.distance = c.dist_x;
    q.mint = c.mint_x;
    refresh_shadows(q);
}

/* the rotation step's traversal of the speculative engine; the sequential
 * warp traversal where the FP32 shadows are unusable */
struct SpecDfs {
    WarpShared &sh;
    SpecCtx &c;
    C2A_KDEV void operator()(Query &q, const M3 &R, V3 T, int lane) const
    {
        if (!q.shadows_ok) {
            toc_dfs_warp(q, R, T, sh, lane);
            return;
        }
        spec_dfs(q, R, T, c, lane);
    }
};

} // namespace c2a
#endif
