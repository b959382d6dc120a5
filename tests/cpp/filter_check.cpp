/*
 * filter_check.cpp -- host build of the kernels' FP32 filter next to their
 * FP64 path, for the CPU soundness test (tests/test_filter.py).
 *
 * Each entry evaluates one piece of the CA step twice from the same inputs:
 * in FP64 with the reference's arithmetic (the values the GPU reproduces bit
 * for bit) and in the FP32 filter (value v, bound e).  The test checks
 * |v - x64| <= e whenever the filter reports its result as certified, and
 * collects how often -- and at which source line -- it gives up.
 */
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../c2a_gb300/csrc/device/geom.cuh"
#include "../../c2a_gb300/csrc/device/rect_cases.cuh"
#include "../../c2a_gb300/csrc/device/rect_table.cuh"

using namespace c2a;

namespace {

struct NodeIn {
    M3 R, Rloc;
    V3 Tr;
    double l[2], r, angR;
};
NodeIn node_in(const double *f)
{
    NodeIn n;
    for (int i = 0; i < 9; i++) {
        n.R.m[i] = f[i];
        n.Rloc.m[i] = f[16 + i];
    }
    n.Tr = v3(f[9], f[10], f[11]);
    n.l[0] = f[12];
    n.l[1] = f[13];
    n.r = f[14];
    n.angR = f[15];
    return n;
}
/* the FP32 shadow of a node as the host build stores it (round to nearest) */
struct NodeEF {
    M3T<EF> R, Rloc;
    V3T<EF> Tr;
    EF l[2], r, angR;
};
NodeEF node_ef(const double *f)
{
    NodeEF n;
    for (int i = 0; i < 9; i++) {
        n.R.m[i] = ef_shadow((float)f[i]);
        n.Rloc.m[i] = ef_shadow((float)f[16 + i]);
    }
    n.Tr = v3t(ef_shadow((float)f[9]), ef_shadow((float)f[10]), ef_shadow((float)f[11]));
    n.l[0] = ef_shadow((float)f[12]);
    n.l[1] = ef_shadow((float)f[13]);
    n.r = ef_shadow((float)f[14]);
    n.angR = ef_shadow((float)f[15]);
    return n;
}
M3 m3_of(const double *p)
{
    M3 r;
    for (int i = 0; i < 9; i++) r.m[i] = p[i];
    return r;
}

} // namespace

extern "C" {

/*
 * One child BV test of the rotation step: the child pair's transform from its
 * parent's exact (PR, PT), C2A_BV_Distance and both motion bounds.
 * out: d64, mint64, d.v, d.e, mint.v, mint.e, certified (1/0), failing line,
 * d-is-zero flag of the filter.
 */
int c2a_fc_bv(const double *PR, const double *PT, const double *f1, const double *f2, int side,
              const double *pose, const double *r1, double *out)
{
    Motion m1, m2;
    motion_setup(m1, pose, pose + 9, pose + 12, pose + 21);
    motion_setup(m2, pose + 24, pose + 33, pose + 36, pose + 45);
    /* FP64 */
    ExactCtx xc{false};
    const MotionT<double> x1 = motion_t<double>(m1, xc), x2 = motion_t<double>(m2, xc);
    const NodeIn a = node_in(f1), b = node_in(f2);
    const M3 R0 = m3_of(PR), Rq = m3_of(r1);
    const V3 T0 = v3(PT[0], PT[1], PT[2]);
    M3 R;
    V3 T;
    if (side == 0) {
        R = tmmul(a.R, R0);
        T = tmul(a.R, T0 - a.Tr);
    } else {
        R = mmul(R0, b.R);
        T = mul_add(R0, b.Tr, T0);
    }
    V3 S = v3(0, 0, 0);
    double z = rect_dist(R, T, a.l, b.l, S, xc);
    z -= (a.r + b.r);
    const double d = max0_c(z);
    double mint = 0.0;
    if (d != 0.0) {
        V3 S1 = mul(Rq, mul(a.Rloc, S));
        V3 S2 = mul_s(S1, -1.0);
        const double mb1 = bound_rss(x1, a.angR, S1, xc);
        const double mb2 = bound_rss(x2, b.angR, S2, xc);
        mint = max0_c((d) / (mb1 + mb2));
    }
    out[0] = d;
    out[1] = mint;
    /* FP32 filter */
    EFCtx c{false};
    const MotionT<EF> e1 = motion_t<EF>(m1, c), e2 = motion_t<EF>(m2, c);
    M3T<EF> PRe, Rqe;
    for (int i = 0; i < 9; i++) {
        PRe.m[i] = in_d(PR[i], c);
        Rqe.m[i] = in_d(r1[i], c);
    }
    const V3T<EF> PTe = v3t(in_d(PT[0], c), in_d(PT[1], c), in_d(PT[2], c));
    const NodeEF ea = node_ef(f1), eb = node_ef(f2);
    M3T<EF> Re;
    V3T<EF> Te;
    if (side == 0) {
        Re = tmmul(ea.R, PRe);
        Te = tmul(ea.R, PTe - ea.Tr);
    } else {
        Re = mmul(PRe, eb.R);
        Te = mul_add(PRe, eb.Tr, PTe);
    }
    V3T<EF> Se = v3t(ef_exact(0), ef_exact(0), ef_exact(0));
    const EF ze = rect_dist(Re, Te, ea.l, eb.l, Se, c) - (ea.r + eb.r);
    EF de = ef_exact(0), me = ef_exact(0);
    int zero = 0;
    if (!c.bad) {
        const int pos = ef_lt3(ef_exact(0), ze);
        if (pos < 0) {
            C2A_EF_FAIL(c, 100000);
        } else if (pos == 0) {
            zero = 1;
        } else {
            de = ze;
            V3T<EF> S1 = mul(Rqe, mul(ea.Rloc, Se));
            V3T<EF> S2 = mul_s(S1, ef_exact(-1));
            const EF mb1 = bound_rss(e1, ea.angR, S1, c);
            const EF mb2 = bound_rss(e2, eb.angR, S2, c);
            me = max0_c(ef_div(de, mb1 + mb2, c));
        }
    }
    out[2] = de.v;
    out[3] = de.e;
    out[4] = me.v;
    out[5] = me.e;
    out[6] = c.bad ? 0.0 : 1.0;
    out[7] = c.where;
    out[8] = zero;
    /* the one-lane form of the speculative engine (rect_dist_lane): d.v, d.e, certified, zero flag */
    EFCtx cl{false};
    V3T<EF> Sl = v3t(ef_exact(0), ef_exact(0), ef_exact(0));
    const EF zl = rect_dist_lane(Re, Te, ea.l, eb.l, Sl, cl) - (ea.r + eb.r);
    EF dl = ef_exact(0);
    int zl0 = 0;
    if (!cl.bad) {
        const int pos = ef_lt3(ef_exact(0), zl);
        if (pos < 0) C2A_EF_FAIL(cl, 100001);
        else if (pos == 0) zl0 = 1;
        else dl = zl;
    }
    out[9] = dl.v;
    out[10] = dl.e;
    out[11] = cl.bad ? 0.0 : 1.0;
    out[12] = zl0;
    return 0;
}

/*
 * TriDist of two triangles given in their models' frames, B placed by (Rm, Tm)
 * as the leaf test does.  out: d64, d.v, d.e, certified, failing line,
 * feature types a/b of FP64 and of the filter.
 */
int c2a_fc_tri(const double *ta, const double *tb, const double *Rm, const double *Tm, double *out)
{
    const M3 R = m3_of(Rm);
    const V3 T0 = v3(Tm[0], Tm[1], Tm[2]);
    V3 S[3], Tt[3];
    for (int k = 0; k < 3; k++) {
        S[k] = v3(ta[3 * k], ta[3 * k + 1], ta[3 * k + 2]);
        Tt[k] = mul_add(R, v3(tb[3 * k], tb[3 * k + 1], tb[3 * k + 2]), T0);
    }
    ExactCtx xc{false};
    V3 p, q;
    TriFeat f{-1, -1, -1, -1};
    bool col = false;
    out[0] = tri_dist(p, q, S, Tt, f, col, xc);
    EFCtx c{false};
    M3T<EF> Re;
    for (int i = 0; i < 9; i++) Re.m[i] = in_d(Rm[i], c);
    const V3T<EF> Te = v3t(in_d(Tm[0], c), in_d(Tm[1], c), in_d(Tm[2], c));
    V3T<EF> Se[3], Tte[3];
    for (int k = 0; k < 3; k++) {
        Se[k] = v3t(ef_shadow((float)ta[3 * k]), ef_shadow((float)ta[3 * k + 1]), ef_shadow((float)ta[3 * k + 2]));
        const V3T<EF> t = v3t(ef_shadow((float)tb[3 * k]), ef_shadow((float)tb[3 * k + 1]),
                              ef_shadow((float)tb[3 * k + 2]));
        Tte[k] = mul_add(Re, t, Te);
    }
    V3T<EF> pe, qe;
    TriFeat fe{-1, -1, -1, -1};
    bool cole = false;
    const EF de = tri_dist(pe, qe, Se, Tte, fe, cole, c);
    out[1] = de.v;
    out[2] = de.e;
    out[3] = c.bad ? 0.0 : 1.0;
    out[4] = c.where;
    out[5] = f.type_a;
    out[6] = f.type_b;
    out[7] = fe.type_a;
    out[8] = fe.type_b;
    return 0;
}

/*
 * C2ARectDist two ways in FP64: the sequential rect_dist and the lane-parallel
 * case form (cases 0..15 evaluated independently, the first that holds wins,
 * else the face-separation tail).  out: d_seq, S_seq[3], d_lanes, S_lanes[3],
 * winning case (-1: tail).
 */
int c2a_fc_rect_lanes(const double *Rab9, const double *Tab3, const double *a, const double *b, double *out)
{
    const M3 R = m3_of(Rab9);
    const V3 T = v3(Tab3[0], Tab3[1], Tab3[2]);
    ExactCtx xc{false};
    V3 S = v3(0, 0, 0);
    out[0] = rect_dist(R, T, a, b, S, xc);
    out[1] = S.x; out[2] = S.y; out[3] = S.z;
    int win = -1;
    double d = 0.0;
    V3 Sw = v3(0, 0, 0);
    for (int j = 0; j < 16; j++) {
        V3 Sj;
        int hit = 0;
        bool vbad = false;
        const double dj = rect_case(j, R, T, a, b, Sj, hit, vbad, xc);
        if (hit == 1) {
            win = j;
            d = dj;
            Sw = Sj;
            break;
        }
    }
    if (win < 0) d = rect_tail(R, T, a, b, Sw, xc);
    out[4] = d;
    out[5] = Sw.x; out[6] = Sw.y; out[7] = Sw.z;
    out[8] = win;
    return 0;
}

/*
 * C2ARectDist on one lane (rect_dist_lane: the cases through one code path in
 * order) next to the sequential rect_dist, FP64.  out: d_seq, S_seq[3], d_lane,
 * S_lane[3].
 */
int c2a_fc_rect_one_lane(const double *Rab9, const double *Tab3, const double *a, const double *b, double *out)
{
    const M3 R = m3_of(Rab9);
    const V3 T = v3(Tab3[0], Tab3[1], Tab3[2]);
    ExactCtx xc{false};
    V3 S = v3(0, 0, 0), Sl = v3(0, 0, 0);
    out[0] = rect_dist(R, T, a, b, S, xc);
    out[1] = S.x; out[2] = S.y; out[3] = S.z;
    out[4] = rect_dist_lane(R, T, a, b, Sl, xc);
    out[5] = Sl.x; out[6] = Sl.y; out[7] = Sl.z;
    return 0;
}

/*
 * rect_table.cuh (the half-warp form: slots computed a few per lane, the
 * eight sort comparisons as a mask, operands through the table), emulated
 * lane by lane.  out: d, S[3], winning case (-1: tail).
 */
int c2a_fc_rect_table(const double *Rab9, const double *Tab3, const double *a, const double *b, double *out)
{
    const M3 R = m3_of(Rab9);
    const V3 T = v3(Tab3[0], Tab3[1], Tab3[2]);
    double V[64];
    rt_inputs(R, T, a, b, V);
    for (int k = 0; k < kRtStage1; k++) V[kRtInputs + k] = rt_stage1(k, R, T, V);
    for (int i = 0; i < kRtStage2; i++) V[kRtStage2Base + i] = rt_stage2(i, V);
    unsigned mask = 0;
    for (int g = 0; g < 8; g++)
        if (rt_compare(g, V)) mask |= 1u << g;
    int win = -1;
    double d = 0.0;
    V3 S = v3(0, 0, 0);
    for (int j = 0; j < 16 && win < 0; j++) {
        double L[4], Rr[4], s1[7], s2[7], e[5], qb;
        int px, py, qkind, cb, cu;
        rt_case_operands(j, mask, V, L, Rr, s1, s2, e, qb, px, py, qkind, cb, cu);
        if (rt_case_holds(L, Rr, s1, s2)) {
            win = j;
            d = rt_case_value(e, qb, px, py, qkind, cb, cu, R, T, a, S);
        }
    }
    if (win < 0) {
        ExactCtx xc{false};
        d = rect_tail(R, T, a, b, S, xc);
    }
    out[0] = d;
    out[1] = S.x; out[2] = S.y; out[3] = S.z;
    out[4] = win;
    return 0;
}

} // extern "C"
