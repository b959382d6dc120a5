/*
 * c2a_port_ca.c -- oracle port of the C2A conservative-advancement path:
 * linear motion, the per-iteration BVTT step with its controlled error
 * schedule, the CA loop, the contact enumeration at the TOC, the
 * translation-only CA and the C2A_Solve body.  Test infrastructure only.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "c2a_port.h"
#include "c2a_port_matvec.h"
#include "../c2a_gb300/csrc/common/c2a_detmath.h"

/* ------------------------------------------------------------------ motion */

/* Matrix3x3::Quaternion_, C2A/LinearMath.h:759-794; q = (x, y, z, w) */
static void mat_to_quat(double q[4], const double m[3][3])
{
    const double *v = &m[0][0];
    double trace = v[0] + v[4] + v[8];
    if (trace > 0.0) {
        double s = sqrt(trace + 1.0);
        q[3] = s * 0.5;
        s = 0.5 / s;
        q[0] = (v[7] - v[5]) * s;
        q[1] = (v[2] - v[6]) * s;
        q[2] = (v[3] - v[1]) * s;
    } else {
        int i = v[0] < v[4] ? (v[4] < v[8] ? 2 : 1) : (v[0] < v[8] ? 2 : 0);
        int j = (i + 1) % 3, k = (i + 2) % 3;
        double s = sqrt(v[i * 3 + i] - v[j * 3 + j] - v[k * 3 + k] + 1.0);
        q[i] = s * 0.5;
        s = 0.5 / s;
        q[3] = (v[k * 3 + j] - v[j * 3 + k]) * s;
        q[j] = (v[j * 3 + i] + v[i * 3 + j]) * s;
        q[k] = (v[k * 3 + i] + v[i * 3 + k]) * s;
    }
}

/* quaternion product, C2A/LinearMath.h:1018-1025 */
static void quat_mul(double r[4], const double a[4], const double b[4])
{
    double x = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    double y = a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2];
    double z = a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0];
    double w = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
    r[0] = x; r[1] = y; r[2] = z; r[3] = w;
}

/* Matrix3x3::Set_Value(Quaternion), C2A/LinearMath.h:809-829 */
static void quat_to_mat(double m[3][3], const double q[4])
{
    double d = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    double s = 2.0 / d;
    double xs = q[0] * s, ys = q[1] * s, zs = q[2] * s;
    double wx = q[3] * xs, wy = q[3] * ys, wz = q[3] * zs;
    double xx = q[0] * xs, xy = q[0] * ys, xz = q[0] * zs;
    double yy = q[1] * ys, yz = q[1] * zs, zz = q[2] * zs;
    m[0][0] = 1.0 - (yy + zz); m[0][1] = xy - wz; m[0][2] = xz + wy;
    m[1][0] = xy + wz; m[1][1] = 1.0 - (xx + zz); m[1][2] = yz - wx;
    m[2][0] = xz - wy; m[2][1] = yz + wx; m[2][2] = 1.0 - (xx + yy);
}

/* CInterpMotion ctor + CInterpMotion_Linear::velocity + LinearAngularVelocity,
 * C2A/src/InterpMotion.cpp:148-168, 228-270, 486-502 */
void c2a_port_motion_init(c2a_port_motion *m, const double R0[9], const double T0[3], const double R1[9],
                          const double T1[3])
{
    double Rt[3][3], qs[4], qt[4], sq0[4], st[4], s, sign, a, tang[3], len;
    memset(m, 0, sizeof(*m));
    pm_from9(m->R0, R0);
    pv_copy(m->T0, T0);
    pm_from9(Rt, R1);
    pm_copy(m->R, (const double(*)[3])m->R0);
    pv_copy(m->T, T0);
    pv_sub(m->cv, T1, T0);
    mat_to_quat(qs, (const double(*)[3])m->R0);
    mat_to_quat(qt, (const double(*)[3])Rt);
    sq0[0] = -qs[0]; sq0[1] = -qs[1]; sq0[2] = -qs[2]; sq0[3] = qs[3];
    quat_mul(st, sq0, qt);
    s = 1 < st[3] ? 1 : st[3];
    sign = s < 0 ? -1 : 1;
    a = (fabs(s - 1) <= 1e-40 || fabs(s + 1) <= 1e-40) ? (2 * sign)
                                                      : (sign * c2a_det_acos(2 * s * s - 1) / sqrt(1 - s * s));
    tang[0] = a * st[0];
    tang[1] = a * st[1];
    tang[2] = a * st[2];
    pv_copy(m->axis, tang);
    m->angVel = pv_len(tang);
    len = m->axis[0] * m->axis[0] + m->axis[1] * m->axis[1] + m->axis[2] * m->axis[2];
    if (len < (double)0.00000001f) {
        m->axis[0] = 1.0; m->axis[1] = 0.0; m->axis[2] = 0.0;
    } else {
        double inv = 1.0 / sqrt(len);
        m->axis[0] *= inv; m->axis[1] *= inv; m->axis[2] *= inv;
    }
    mat_to_quat(m->q0, (const double(*)[3])m->R0);
}

/* CInterpMotion_Linear::integrate + DeltaRt/AbsoluteRt, InterpMotion.cpp:273-287, 516-568 */
void c2a_port_motion_integrate(c2a_port_motion *m, double dt, double R[9], double T[3], double qua[7])
{
    double ang, sa, drt[4], orn[4], cvdt[3];
    if (dt > 1) dt = 1;
    cvdt[0] = dt * m->cv[0]; cvdt[1] = dt * m->cv[1]; cvdt[2] = dt * m->cv[2];
    pv_add(m->T, m->T0, cvdt);
    ang = 0.5 * m->angVel * dt;
    sa = c2a_det_sin(ang);
    drt[0] = sa * m->axis[0];
    drt[1] = sa * m->axis[1];
    drt[2] = sa * m->axis[2];
    drt[3] = c2a_det_cos(ang);
    quat_mul(orn, m->q0, drt);
    quat_to_mat(m->R, orn);
    if (R) pm_to9(R, (const double(*)[3])m->R);
    if (T) pv_copy(T, m->T);
    if (qua) {
        qua[0] = orn[3]; qua[1] = orn[0]; qua[2] = orn[1]; qua[3] = orn[2];
        qua[4] = m->T[0]; qua[5] = m->T[1]; qua[6] = m->T[2];
    }
}

/* CInterpMotion_Linear::computeTOC(d, r1, S): directional bound at a leaf,
 * InterpMotion.cpp:746-828 (normalises S in place) */
static double motion_bound_leaf(const c2a_port_motion *m, double r1, double S[3])
{
    double w_max, v_max, path_max;
    pv_normalize(S);
    if (m->angVel == 0) {
        w_max = 0;
        v_max = pv_dot(m->cv, S);
        if (v_max < 0) v_max = 0;
    } else {
        double cwc[3], cross[3];
        cwc[0] = m->axis[0]; cwc[1] = m->axis[1]; cwc[2] = m->axis[2];
        cwc[0] *= m->angVel; cwc[1] *= m->angVel; cwc[2] *= m->angVel;
        pv_cross(cross, cwc, S);
        w_max = r1 * pv_len(cross);
        v_max = pv_dot(m->cv, S);
        if (v_max < 0) v_max = 0;
    }
    path_max = w_max + v_max;
    if (path_max == 0) path_max = 1e-30;
    return path_max;
}

/* CInterpMotion_Linear::computeTOC_MotionBound, InterpMotion.cpp:831-881 */
static double motion_bound_rss(const c2a_port_motion *m, double angR, double N[3])
{
    double cross[3], w_max, v_max, path_max;
    pv_normalize(N);
    pv_cross(cross, m->axis, N);
    w_max = angR * pv_len(cross) * m->angVel;
    v_max = pv_dot(m->cv, N);
    if (v_max < 0) v_max = 0;
    path_max = v_max + w_max;
    if (path_max <= 0) path_max = 1e-30;
    return path_max;
}

/* ConservD, InterpMotion.cpp:289-298 */
static double conserv_d(const c2a_port_motion *m, double d) { return d - 0.1 * m->toc_delta; }

/* -------------------------------------------------------------- BV / tris */

static double node_size(const c2a_port_node *b) { return sqrt(b->l[0] * b->l[0] + b->l[1] * b->l[1]) + 2 * b->r; }

/* C2A_BV_Distance, C2A/src/C2A_BV.cpp:666-675 */
static double bv_distance(const double R[3][3], const double T[3], const c2a_port_node *b1,
                          const c2a_port_node *b2, double S[3])
{
    double P[3], Q[3], R9[9], dist;
    pm_to9(R9, R);
    dist = c2a_port_rectdist(R9, T, b1->l, b2->l, P, Q, S);
    dist -= (b1->r + b2->r);
    return (dist < 0.0) ? 0.0 : dist;
}

/* PQP TriDistance (t2 moved by R, T into t1's frame) and C2A_TriDistance
 * (C2A.cpp:408-424) */
static double tri_distance(const double R[3][3], const double T[3], const c2a_port_tri *t1, const c2a_port_tri *t2,
                           double p[3], double q[3], int *ft1, int *fid1, int *ft2, int *fid2, int *collided)
{
    double s[9], t[9];
    memcpy(s, t1->p1, 3 * sizeof(double));
    memcpy(s + 3, t1->p2, 3 * sizeof(double));
    memcpy(s + 6, t1->p3, 3 * sizeof(double));
    pm_mul_v_add(t, R, t2->p1, T);
    pm_mul_v_add(t + 3, R, t2->p2, T);
    pm_mul_v_add(t + 6, R, t2->p3, T);
    return c2a_port_tridist(p, q, s, t, ft1, fid1, ft2, fid2, collided);
}

static double tri_distance_plain(const double R[3][3], const double T[3], const c2a_port_tri *t1,
                                 const c2a_port_tri *t2, double p[3], double q[3])
{
    int a = -1, b = -1, fa[3], fb[3], c = 0;
    return tri_distance(R, T, t1, t2, p, q, &a, fa, &b, fb, &c);
}

/* ----------------------------------------------------------- step state */

typedef struct step_state {
    const c2a_port_model *o1, *o2;
    c2a_port_motion *m1, *m2;
    double R[3][3], T[3]; /* model 2 relative to model 1 */
    double distance, mint, rel_err, abs_err, UpboundTOC;
    double p1[3], p2[3];
    long long num_bv_tests, num_tri_tests;
    int seed_a, seed_b;
    int numCA;
    int canonical;        /* seed every rotation step with the closest pair */
    /* contact enumeration output */
    c2a_port_contact *contacts;
    int max_contacts, num_contact;
} step_state;

/* child pair of (b1, b2): split the larger unless b2 is a leaf
 * (C2A.cpp:1192-1226); writes the two child transforms */
static void children(const step_state *st, int b1, int b2, const double R[3][3], const double T[3], int *a1,
                     int *a2, int *c1, int *c2, double R1[3][3], double T1[3], double R2[3][3], double T2[3])
{
    const c2a_port_node *n1 = &st->o1->nodes[b1], *n2 = &st->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    double sz1 = node_size(n1), sz2 = node_size(n2), Ttemp[3];
    if (l2 || (!l1 && (sz1 > sz2))) {
        const c2a_port_node *na, *nc;
        *a1 = n1->first_child; *a2 = b2;
        *c1 = n1->first_child + 1; *c2 = b2;
        na = &st->o1->nodes[*a1];
        nc = &st->o1->nodes[*c1];
        pm_tmul(R1, (const double(*)[3])na->R, R);
        pv_sub(Ttemp, T, na->Tr);
        pm_tmul_v(T1, (const double(*)[3])na->R, Ttemp);
        pm_tmul(R2, (const double(*)[3])nc->R, R);
        pv_sub(Ttemp, T, nc->Tr);
        pm_tmul_v(T2, (const double(*)[3])nc->R, Ttemp);
    } else {
        const c2a_port_node *na, *nc;
        *a1 = b1; *a2 = n2->first_child;
        *c1 = b1; *c2 = n2->first_child + 1;
        na = &st->o2->nodes[*a2];
        nc = &st->o2->nodes[*c2];
        pm_mul(R1, R, (const double(*)[3])na->R);
        pm_mul_v_add(T1, R, na->Tr, T);
        pm_mul(R2, R, (const double(*)[3])nc->R);
        pm_mul_v_add(T2, R, nc->Tr, T);
    }
}

/* mint of one child pair: d / (motion bound 1 + motion bound 2), 0 if the
 * RSSs touch (C2A.cpp:1237-1274) */
static double child_mint(step_state *st, const double R[3][3], const double T[3], int x1, int x2, double *d_out)
{
    const c2a_port_node *n1 = &st->o1->nodes[x1], *n2 = &st->o2->nodes[x2];
    double S1[3], S2[3], temp[3], d, mint;
    d = bv_distance(R, T, n1, n2, S1);
    if (d != 0.0) {
        double mb1, mb2;
        pm_mul_v(temp, (const double(*)[3])n1->Rloc, S1);
        pm_mul_v(S1, (const double(*)[3])st->m1->R, temp);
        pv_scale(S2, S1, -1);
        mb1 = motion_bound_rss(st->m1, n1->angR, S1);
        mb2 = motion_bound_rss(st->m2, n2->angR, S2);
        mint = (d) / (mb1 + mb2);
        if (mint <= 0) mint = 0.0;
    } else {
        mint = 0.0;
    }
    *d_out = d;
    return mint;
}

static int descend_ok(const step_state *st, double mint, double d)
{
    return mint < st->UpboundTOC && ((d < (st->distance - st->abs_err)) || (d * (1 + st->rel_err) < st->distance));
}

/* TOCStepRecurse_Dis, C2A/src/C2A.cpp:1114-1354 */
static void toc_recurse(step_state *st, const double R[3][3], const double T[3], int b1, int b2)
{
    const c2a_port_node *n1 = &st->o1->nodes[b1], *n2 = &st->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    if (l1 && l2) {
        double p[3], q[3], dTri;
        C2A_PORT_SCOPE(2);
        const c2a_port_tri *t1 = &st->o1->tris[-n1->first_child - 1];
        const c2a_port_tri *t2 = &st->o2->tris[-n2->first_child - 1];
        dTri = tri_distance_plain((const double(*)[3])st->R, st->T, t1, t2, p, q);
        if (dTri <= st->distance) {
            double temp1[3], temp2[3], res1[3], res2[3], S1[3], S2[3], mb1, mb2, mint;
            st->distance = dTri;
            pm_mul_v(temp1, (const double(*)[3])st->m1->R, p);
            pv_add(res1, temp1, st->m1->T);
            pm_mul_v(temp2, (const double(*)[3])st->m1->R, q);
            pv_add(res2, temp2, st->m1->T);
            pv_sub(S1, res2, res1);
            pv_scale(S2, S1, -1);
            pv_copy(st->p1, p);
            pv_copy(st->p2, q);
            mb1 = motion_bound_leaf(st->m1, n1->angR, S1);
            mb2 = motion_bound_leaf(st->m2, n2->angR, S2);
            mint = (dTri) / (mb1 + mb2);
            if (mint < 0.0) mint = 0.0;
            if (mint <= st->mint) st->mint = mint;
            st->distance = dTri;
        }
        st->num_tri_tests++;
        return;
    }
    {
        int a1, a2, c1, c2;
        double R1[3][3], T1[3], R2[3][3], T2[3], d1, d2, mintb, minta;
        C2A_PORT_SCOPE(1);
        children(st, b1, b2, R, T, &a1, &a2, &c1, &c2, R1, T1, R2, T2);
        mintb = child_mint(st, (const double(*)[3])R1, T1, a1, a2, &d1);
        minta = child_mint(st, (const double(*)[3])R2, T2, c1, c2, &d2);
        st->num_bv_tests += 2;
        if (d2 < d1) {
            if (descend_ok(st, minta, d2)) toc_recurse(st, (const double(*)[3])R2, T2, c1, c2);
            else if (minta < st->mint) st->mint = minta;
            if (descend_ok(st, mintb, d1)) toc_recurse(st, (const double(*)[3])R1, T1, a1, a2);
            else if (mintb < st->mint) st->mint = mintb;
        } else {
            if (descend_ok(st, mintb, d1)) toc_recurse(st, (const double(*)[3])R1, T1, a1, a2);
            else if (mintb < st->mint) st->mint = mintb;
            if (descend_ok(st, minta, d2)) toc_recurse(st, (const double(*)[3])R2, T2, c1, c2);
            else if (minta < st->mint) st->mint = minta;
        }
    }
}

/* ------------------------------------------------------- distance query */

typedef struct dist_state {
    const c2a_port_model *o1, *o2;
    double R[3][3], T[3]; /* model 2 relative to model 1 */
    double distance;
    int t1, t2;
    long long num_bv_tests, num_tri_tests;
} dist_state;

/* C2ADistanceRecurse, C2A/src/C2A_PQP.cpp:481-621, with rel_err = abs_err = 0 */
static void dist_recurse(dist_state *ds, const double R[3][3], const double T[3], int b1, int b2)
{
    const c2a_port_node *n1 = &ds->o1->nodes[b1], *n2 = &ds->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    if (l1 && l2) {
        double p[3], q[3], d;
        int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
        ds->num_tri_tests++;
        d = tri_distance_plain((const double(*)[3])ds->R, ds->T, &ds->o1->tris[ia], &ds->o2->tris[ib], p, q);
        if (d < ds->distance) {
            ds->distance = d;
            ds->t1 = ia;
            ds->t2 = ib;
        }
        return;
    }
    {
        int a1, a2, c1, c2;
        double R1[3][3], T1[3], R2[3][3], T2[3], S[3], d1, d2;
        step_state cs;
        cs.o1 = ds->o1;
        cs.o2 = ds->o2;
        children(&cs, b1, b2, R, T, &a1, &a2, &c1, &c2, R1, T1, R2, T2);
        ds->num_bv_tests += 2;
        d1 = bv_distance((const double(*)[3])R1, T1, &ds->o1->nodes[a1], &ds->o2->nodes[a2], S);
        d2 = bv_distance((const double(*)[3])R2, T2, &ds->o1->nodes[c1], &ds->o2->nodes[c2], S);
        if (d2 < d1) {
            if ((d2 < (ds->distance - 0)) || (d2 * (1 + 0) < ds->distance))
                dist_recurse(ds, (const double(*)[3])R2, T2, c1, c2);
            if ((d1 < (ds->distance - 0)) || (d1 * (1 + 0) < ds->distance))
                dist_recurse(ds, (const double(*)[3])R1, T1, a1, a2);
        } else {
            if ((d1 < (ds->distance - 0)) || (d1 * (1 + 0) < ds->distance))
                dist_recurse(ds, (const double(*)[3])R1, T1, a1, a2);
            if ((d2 < (ds->distance - 0)) || (d2 * (1 + 0) < ds->distance))
                dist_recurse(ds, (const double(*)[3])R2, T2, c1, c2);
        }
    }
}

/* C2A_Distance (C2A_PQP.cpp:971-1056): initial bound from the seed pair, then
 * the recursion from the two root nodes */
static double distance_query(const c2a_port_model *A, const c2a_port_model *B, const double Rm[3][3],
                             const double Tm[3], int seed_a, int seed_b, int *ta, int *tb, long long *nbv,
                             long long *ntri)
{
    dist_state ds;
    double p[3], q[3], Rtemp[3][3], R[3][3], Ttemp[3], T[3];
    const c2a_port_node *r1 = &A->nodes[0], *r2 = &B->nodes[0];
    ds.o1 = A;
    ds.o2 = B;
    pm_copy(ds.R, Rm);
    pv_copy(ds.T, Tm);
    ds.distance = tri_distance_plain(Rm, Tm, &A->tris[seed_a], &B->tris[seed_b], p, q);
    ds.t1 = seed_a;
    ds.t2 = seed_b;
    ds.num_bv_tests = 0;
    ds.num_tri_tests = 0;
    pm_mul(Rtemp, Rm, (const double(*)[3])r2->R);
    pm_tmul(R, (const double(*)[3])r1->R, (const double(*)[3])Rtemp);
    pm_mul_v_add(Ttemp, Rm, r2->Tr, Tm);
    pv_sub(Ttemp, Ttemp, r1->Tr);
    pm_tmul_v(T, (const double(*)[3])r1->R, Ttemp);
    dist_recurse(&ds, (const double(*)[3])R, T, 0, 0);
    *ta = ds.t1;
    *tb = ds.t2;
    if (nbv) *nbv = ds.num_bv_tests;
    if (ntri) *ntri = ds.num_tri_tests;
    return ds.distance;
}

double c2a_port_distance(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                         int seed_a, int seed_b, int *ta, int *tb, long long *nbv, long long *ntri)
{
    double Rm[3][3];
    pm_from9(Rm, R);
    return distance_query(A, B, (const double(*)[3])Rm, T, seed_a, seed_b, ta, tb, nbv, ntri);
}

/* ------------------------------------------------------- tolerance query */

typedef struct tol_state {
    const c2a_port_model *o1, *o2;
    double R[3][3], T[3]; /* model 2 relative to model 1 */
    double tolerance, distance, p1[3], p2[3];
    int closer;
    long long num_bv_tests, num_tri_tests;
} tol_state;

/* C2AToleranceRecurse, C2A/src/C2A_PQP.cpp:1498-1603: depth first, the pair
 * with the smaller RSS distance first, stopping at the first triangle pair
 * within the tolerance */
static void tol_recurse(tol_state *ts, const double R[3][3], const double T[3], int b1, int b2)
{
    const c2a_port_node *n1 = &ts->o1->nodes[b1], *n2 = &ts->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    if (l1 && l2) {
        double p[3], q[3], d;
        int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
        ts->num_tri_tests++;
        d = tri_distance_plain((const double(*)[3])ts->R, ts->T, &ts->o1->tris[ia], &ts->o2->tris[ib], p, q);
        if (d <= ts->tolerance) {
            ts->closer = 1;
            ts->distance = d;
            pv_copy(ts->p1, p);
            pv_copy(ts->p2, q);
        }
        return;
    }
    {
        int a1, a2, c1, c2;
        double R1[3][3], T1[3], R2[3][3], T2[3], S[3], d1, d2;
        step_state cs;
        cs.o1 = ts->o1;
        cs.o2 = ts->o2;
        children(&cs, b1, b2, R, T, &a1, &a2, &c1, &c2, R1, T1, R2, T2);
        ts->num_bv_tests += 2;
        d1 = bv_distance((const double(*)[3])R1, T1, &ts->o1->nodes[a1], &ts->o2->nodes[a2], S);
        d2 = bv_distance((const double(*)[3])R2, T2, &ts->o1->nodes[c1], &ts->o2->nodes[c2], S);
        if (d2 < d1) {
            if (d2 <= ts->tolerance) tol_recurse(ts, (const double(*)[3])R2, T2, c1, c2);
            if (ts->closer) return;
            if (d1 <= ts->tolerance) tol_recurse(ts, (const double(*)[3])R1, T1, a1, a2);
        } else {
            if (d1 <= ts->tolerance) tol_recurse(ts, (const double(*)[3])R1, T1, a1, a2);
            if (ts->closer) return;
            if (d2 <= ts->tolerance) tol_recurse(ts, (const double(*)[3])R2, T2, c1, c2);
        }
    }
}

/* C2A_Tolerance with qsize 2 (C2A_PQP.cpp:1762-1845): the root RSS distance
 * as a trivial reject, then the recursion; p2 back into model 2's frame */
int c2a_port_tolerance(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                       double tolerance, double *distance, double p1[3], double p2[3], long long *nbv,
                       long long *ntri)
{
    tol_state ts;
    double Rm[3][3], Rtemp[3][3], Rr[3][3], Ttemp[3], Tr[3], S[3], u[3], d;
    const c2a_port_node *r1 = &A->nodes[0], *r2 = &B->nodes[0];
    pm_from9(Rm, R);
    ts.o1 = A;
    ts.o2 = B;
    pm_copy(ts.R, (const double(*)[3])Rm);
    pv_copy(ts.T, T);
    if (tolerance < 0.0) tolerance = 0.0;
    ts.tolerance = tolerance;
    ts.num_bv_tests = ts.num_tri_tests = 0;
    ts.closer = 0;
    ts.distance = 0.0;
    ts.p1[0] = ts.p1[1] = ts.p1[2] = 0.0;
    ts.p2[0] = ts.p2[1] = ts.p2[2] = 0.0;
    pm_mul(Rtemp, (const double(*)[3])Rm, (const double(*)[3])r2->R);
    pm_tmul(Rr, (const double(*)[3])r1->R, (const double(*)[3])Rtemp);
    pm_mul_v_add(Ttemp, (const double(*)[3])Rm, r2->Tr, T);
    pv_sub(Ttemp, Ttemp, r1->Tr);
    pm_tmul_v(Tr, (const double(*)[3])r1->R, Ttemp);
    d = bv_distance((const double(*)[3])Rr, Tr, r1, r2, S);
    if (d <= ts.tolerance) tol_recurse(&ts, (const double(*)[3])Rr, Tr, 0, 0);
    if (ts.closer) {
        pv_sub(u, ts.p2, T);
        pm_tmul_v(p2, (const double(*)[3])Rm, u);
        pv_copy(p1, ts.p1);
        *distance = ts.distance;
    }
    if (nbv) *nbv = ts.num_bv_tests;
    if (ntri) *ntri = ts.num_tri_tests;
    return ts.closer;
}

/* --------------------------------------------------------- collide query */

/* the OBB separating-axis test of the PQP interface as the oracle's shim
 * states it (oracle/pqp_shim/pqp_shim.cpp): box b placed by (B, T) in box a's
 * frame, the 15 axes with |B| inflated by 1e-6; 0 when no axis separates */
static int obb_disjoint(const double B[3][3], const double T[3], const double a[3], const double b[3])
{
    double Bf[3][3], s, tproj, ra, rb;
    int i, j;
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) Bf[i][j] = fabs(B[i][j]) + 1e-6;
    for (i = 0; i < 3; i++) {
        s = b[0] * Bf[i][0] + b[1] * Bf[i][1] + b[2] * Bf[i][2];
        if (fabs(T[i]) > a[i] + s) return 1;
    }
    for (j = 0; j < 3; j++) {
        tproj = T[0] * B[0][j] + T[1] * B[1][j] + T[2] * B[2][j];
        s = a[0] * Bf[0][j] + a[1] * Bf[1][j] + a[2] * Bf[2][j];
        if (fabs(tproj) > b[j] + s) return 1;
    }
    for (i = 0; i < 3; i++) {
        int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        for (j = 0; j < 3; j++) {
            int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            tproj = T[i2] * B[i1][j] - T[i1] * B[i2][j];
            ra = a[i1] * Bf[i2][j] + a[i2] * Bf[i1][j];
            rb = b[j1] * Bf[i][j2] + b[j2] * Bf[i][j1];
            if (fabs(tproj) > ra + rb) return 2;
        }
    }
    return 0;
}

typedef struct coll_state {
    const c2a_port_model *o1, *o2;
    double R[3][3], T[3]; /* model 2 relative to model 1 */
    int flag, num_pairs, cap;
    int *pairs;
    long long num_bv_tests, num_tri_tests;
} coll_state;

/* CollideRecurse, C2A/src/C2A_PQP.cpp:798-909: overlapping OBB pairs only,
 * the first child before the second; triangles touch when their distance is
 * zero (the shim's TriContact) */
static void coll_recurse(coll_state *cs, const double R[3][3], const double T[3], int b1, int b2)
{
    const c2a_port_node *n1 = &cs->o1->nodes[b1], *n2 = &cs->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    double Rc[3][3], Tc[3], Ttemp[3];
    cs->num_bv_tests++;
    if (obb_disjoint(R, T, n1->d, n2->d) != 0) return;
    if (l1 && l2) {
        const c2a_port_tri *t1 = &cs->o1->tris[-n1->first_child - 1], *t2 = &cs->o2->tris[-n2->first_child - 1];
        double p[3], q[3];
        cs->num_tri_tests++;
        if (tri_distance_plain((const double(*)[3])cs->R, cs->T, t1, t2, p, q) == 0.0) {
            if (cs->pairs && cs->num_pairs < cs->cap) {
                cs->pairs[2 * cs->num_pairs] = t1->id;
                cs->pairs[2 * cs->num_pairs + 1] = t2->id;
            }
            cs->num_pairs++;
        }
        return;
    }
    if (l2 || (!l1 && (node_size(n1) > node_size(n2)))) {
        int c1 = n1->first_child, c2 = c1 + 1;
        const c2a_port_node *m1 = &cs->o1->nodes[c1], *m2 = &cs->o1->nodes[c2];
        pm_tmul(Rc, (const double(*)[3])m1->R, R);
        pv_sub(Ttemp, T, m1->To);
        pm_tmul_v(Tc, (const double(*)[3])m1->R, Ttemp);
        coll_recurse(cs, (const double(*)[3])Rc, Tc, c1, b2);
        if (cs->flag == 2 && cs->num_pairs > 0) return;
        pm_tmul(Rc, (const double(*)[3])m2->R, R);
        pv_sub(Ttemp, T, m2->To);
        pm_tmul_v(Tc, (const double(*)[3])m2->R, Ttemp);
        coll_recurse(cs, (const double(*)[3])Rc, Tc, c2, b2);
    } else {
        int c1 = n2->first_child, c2 = c1 + 1;
        const c2a_port_node *m1 = &cs->o2->nodes[c1], *m2 = &cs->o2->nodes[c2];
        pm_mul(Rc, R, (const double(*)[3])m1->R);
        pm_mul_v_add(Tc, R, m1->To, T);
        coll_recurse(cs, (const double(*)[3])Rc, Tc, b1, c1);
        if (cs->flag == 2 && cs->num_pairs > 0) return;
        pm_mul(Rc, R, (const double(*)[3])m2->R);
        pm_mul_v_add(Tc, R, m2->To, T);
        coll_recurse(cs, (const double(*)[3])Rc, Tc, b1, c2);
    }
}

/* C2A_Collide (C2A_PQP.cpp:910-968): the root OBB pair's transform, then the recursion */
int c2a_port_collide(const c2a_port_model *A, const c2a_port_model *B, const double R[9], const double T[3],
                     int flag, int *pairs, int cap, long long *nbv, long long *ntri)
{
    coll_state cs;
    double Rm[3][3], Rtemp[3][3], Rr[3][3], Ttemp[3], Tr[3];
    const c2a_port_node *r1 = &A->nodes[0], *r2 = &B->nodes[0];
    pm_from9(Rm, R);
    cs.o1 = A;
    cs.o2 = B;
    pm_copy(cs.R, (const double(*)[3])Rm);
    pv_copy(cs.T, T);
    cs.flag = flag;
    cs.num_pairs = 0;
    cs.cap = cap;
    cs.pairs = pairs;
    cs.num_bv_tests = cs.num_tri_tests = 0;
    pm_mul(Rtemp, (const double(*)[3])Rm, (const double(*)[3])r2->R);
    pm_tmul(Rr, (const double(*)[3])r1->R, (const double(*)[3])Rtemp);
    pm_mul_v_add(Ttemp, (const double(*)[3])Rm, r2->To, T);
    pv_sub(Ttemp, Ttemp, r1->To);
    pm_tmul_v(Tr, (const double(*)[3])r1->R, Ttemp);
    coll_recurse(&cs, (const double(*)[3])Rr, Tr, 0, 0);
    if (nbv) *nbv = cs.num_bv_tests;
    if (ntri) *ntri = cs.num_tri_tests;
    return cs.num_pairs;
}

/* -------------------------------------------------- translation-only CA */

/* CInterpMotion_Linear::CAonNonAdjacentTriangles, InterpMotion.cpp:657-743 */
static int ca_triangles(const c2a_port_motion *m, const double R[3][3], const double triA[3][3],
                        const double triB[3][3], double *mint, double *distance)
{
    double p[3], q[3], Vel[3], n[3], d, u, dt, total_toc, triA_t[3][3], s9[9], t9[9];
    int nIters, i, fa, fb, fia[3], fib[3], col = 0;
    pm_tmul_v(Vel, R, m->cv);
    pm_to9(s9, triA);
    pm_to9(t9, triB);
    d = c2a_port_tridist(p, q, s9, t9, &fa, fia, &fb, fib, &col);
    pv_sub(n, q, p);
    pv_normalize(n);
    u = pv_dot(Vel, n);
    if (u <= 0) u = 1e-30;
    if (d == 0) {
        mint[0] = 0.0;
        distance[0] = 0.0;
        return 1;
    }
    dt = conserv_d(m, d) / u;
    nIters = 1;
    if (dt >= mint[0]) return 0;
    total_toc = dt;
    while ((d > m->toc_delta) && (total_toc <= mint[0]) && (nIters < 50)) {
        double tofc;
        for (i = 0; i < 3; i++) pv_add_scaled(triA_t[i], triA[i], Vel, total_toc);
        pm_to9(s9, (const double(*)[3])triA_t);
        d = c2a_port_tridist(p, q, s9, t9, &fa, fia, &fb, fib, &col);
        if (d == 0.0) break;
        pv_sub(n, q, p);
        pv_normalize(n);
        u = pv_dot(Vel, n);
        if (u <= 0) u = 1e-30;
        tofc = conserv_d(m, d) / u;
        nIters++;
        if (tofc < m->toc_delta) break;
        total_toc += tofc;
    }
    if (total_toc <= mint[0] && total_toc >= 0.0) {
        mint[0] = total_toc;
        distance[0] = (total_toc)*pv_len(m->cv) + m->toc_delta;
        return 1;
    }
    return 0;
}

/* CInterpMotion_Linear::CAonRSS, InterpMotion.cpp:570-655.  The reference
 * reads an uninitialised S when the first rectangle distance falls through
 * to a negative face separation (C2A_RectDist.h:865-933 then leaves S
 * unset); S starts at zero here. */
static int ca_rss(const c2a_port_motion *m, const double r1[3][3], const double R[3][3], const double T[3],
                  const c2a_port_node *b1, const c2a_port_node *b2, double *mint, double *distance)
{
    double S[3] = {0.0, 0.0, 0.0}, temp1[3], temp2[3], Vel[3], d, tocf, total_toc;
    int nIters;
    d = bv_distance(R, T, b1, b2, S);
    pm_mul_v(temp1, (const double(*)[3])b1->Rloc, S);
    pm_mul_v(S, r1, temp1);
    pm_tmul_v(temp1, r1, m->cv);
    pm_tmul_v(Vel, (const double(*)[3])b1->Rloc, temp1);
    tocf = conserv_d(m, d) / motion_bound_leaf(m, b1->angR, S);
    total_toc = tocf;
    nIters = 1;
    while ((d >= m->toc_delta) && (total_toc <= mint[0]) && (nIters < 50)) {
        pv_add_scaled(temp2, T, Vel, -total_toc);
        d = bv_distance(R, temp2, b1, b2, S);
        if (d == 0) break;
        pm_mul_v(temp1, (const double(*)[3])b1->Rloc, S);
        pm_mul_v(S, r1, temp1);
        tocf = conserv_d(m, d) / motion_bound_leaf(m, b1->angR, S);
        nIters++;
        if (tocf < m->toc_delta) break;
        total_toc += tocf;
    }
    if (total_toc < 1.0) {
        mint[0] = total_toc;
        distance[0] = (total_toc - m->toc_delta) * pv_len(m->cv);
        if (distance[0] < 0) distance[0] = 0;
        return 1;
    }
    return 0;
}

/* TOCStepRecurse_Dis_Translation, C2A/src/C2A.cpp:1362-1521 */
static void toc_recurse_translation(step_state *st, const double R[3][3], const double T[3], int b1, int b2)
{
    const c2a_port_node *n1 = &st->o1->nodes[b1], *n2 = &st->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    if (l1 && l2) {
        double tri1[3][3], tri2[3][3];
        C2A_PORT_SCOPE(2);
        int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
        const c2a_port_tri *t1 = &st->o1->tris[ia], *t2 = &st->o2->tris[ib];
        pv_copy(tri1[0], t1->p1);
        pv_copy(tri1[1], t1->p2);
        pv_copy(tri1[2], t1->p3);
        pm_mul_v_add(tri2[0], (const double(*)[3])st->R, t2->p1, st->T);
        pm_mul_v_add(tri2[1], (const double(*)[3])st->R, t2->p2, st->T);
        pm_mul_v_add(tri2[2], (const double(*)[3])st->R, t2->p3, st->T);
        if (ca_triangles(st->m1, (const double(*)[3])st->m1->R, (const double(*)[3])tri1,
                         (const double(*)[3])tri2, &st->mint, &st->distance)) {
            st->seed_a = ia;
            st->seed_b = ib;
        }
        st->num_tri_tests++;
        return;
    }
    {
        int a1, a2, c1, c2;
        double R1[3][3], T1[3], R2[3][3], T2[3], d1, d2, minta, mintc;
        C2A_PORT_SCOPE(1);
        children(st, b1, b2, R, T, &a1, &a2, &c1, &c2, R1, T1, R2, T2);
        d1 = d2 = 1e+30;
        minta = mintc = st->mint;
        ca_rss(st->m1, (const double(*)[3])st->m1->R, (const double(*)[3])R1, T1, &st->o1->nodes[a1],
               &st->o2->nodes[a2], &minta, &d1);
        ca_rss(st->m1, (const double(*)[3])st->m1->R, (const double(*)[3])R2, T2, &st->o1->nodes[c1],
               &st->o2->nodes[c2], &mintc, &d2);
        st->num_bv_tests += 2;
        if (d2 < d1) {
            if (mintc < st->mint && ((d2 < (st->distance - st->abs_err)) || (d2 * (1 + st->rel_err) < st->distance)))
                toc_recurse_translation(st, (const double(*)[3])R2, T2, c1, c2);
            if (minta < st->mint && ((d1 < (st->distance - st->abs_err)) || (d1 * (1 + st->rel_err) < st->distance)))
                toc_recurse_translation(st, (const double(*)[3])R1, T1, a1, a2);
        } else {
            if (minta < st->mint && ((d1 < (st->distance - st->abs_err)) || (d1 * (1 + st->rel_err) < st->distance)))
                toc_recurse_translation(st, (const double(*)[3])R1, T1, a1, a2);
            if (mintc < st->mint && ((d2 < (st->distance - st->abs_err)) || (d2 * (1 + st->rel_err) < st->distance)))
                toc_recurse_translation(st, (const double(*)[3])R2, T2, c1, c2);
        }
    }
}

/* ------------------------------------------------------------ the CA step */

/* relative transform of model 2 in model 1 and of root 2 in root 1
 * (C2A.cpp:1793-1806) */
static void relative_transforms(step_state *st, const double R1[3][3], const double T1[3], const double R2[3][3],
                                const double T2[3], double R[3][3], double T[3])
{
    double Ttemp[3], Rtemp[3][3];
    const c2a_port_node *r1 = &st->o1->nodes[0], *r2 = &st->o2->nodes[0];
    pm_tmul(st->R, R1, R2);
    pv_sub(Ttemp, T2, T1);
    pm_tmul_v(st->T, R1, Ttemp);
    pm_mul(Rtemp, (const double(*)[3])st->R, (const double(*)[3])r2->R);
    pm_tmul(R, (const double(*)[3])r1->R, (const double(*)[3])Rtemp);
    pm_mul_v_add(Ttemp, (const double(*)[3])st->R, r2->Tr, st->T);
    pv_sub(Ttemp, Ttemp, r1->Tr);
    pm_tmul_v(T, (const double(*)[3])r1->R, Ttemp);
}

/* C2A_TimeOfContactStep, C2A/src/C2A.cpp:1778-1931 */
static void toc_step(step_state *st, double R1[3][3], double T1[3], double R2[3][3], double T2[3], int translation)
{
    double R[3][3], T[3], p[3], q[3];
    relative_transforms(st, (const double(*)[3])R1, T1, (const double(*)[3])R2, T2, R, T);
    if (translation) {
        double tri1[3][3], tri2[3][3], dTri = 0, mint = 1.0;
        const c2a_port_tri *t1 = &st->o1->tris[st->seed_a], *t2 = &st->o2->tris[st->seed_b];
        pv_copy(tri1[0], t1->p1);
        pv_copy(tri1[1], t1->p2);
        pv_copy(tri1[2], t1->p3);
        pm_mul_v_add(tri2[0], (const double(*)[3])st->R, t2->p1, st->T);
        pm_mul_v_add(tri2[1], (const double(*)[3])st->R, t2->p2, st->T);
        pm_mul_v_add(tri2[2], (const double(*)[3])st->R, t2->p3, st->T);
        if (ca_triangles(st->m1, (const double(*)[3])st->m1->R, (const double(*)[3])tri1, (const double(*)[3])tri2,
                         &mint, &dTri)) {
            st->mint = mint;
            st->distance = dTri;
        } else {
            st->mint = 1.0;
            st->distance = 1e+30;
        }
        st->abs_err = 0;
        st->rel_err = 0;
        toc_recurse_translation(st, (const double(*)[3])R, T, 0, 0);
        {
            double R19[9], R29[9], Ttemp[3];
            c2a_port_motion_integrate(st->m1, st->mint, R19, T1, NULL);
            c2a_port_motion_integrate(st->m2, st->mint, R29, T2, NULL);
            pm_from9(R1, R19);
            pm_from9(R2, R29);
            pm_tmul(st->R, (const double(*)[3])R1, (const double(*)[3])R2);
            pv_sub(Ttemp, T2, T1);
            pm_tmul_v(st->T, (const double(*)[3])R1, Ttemp);
            st->distance = tri_distance_plain((const double(*)[3])st->R, st->T, &st->o1->tris[st->seed_a],
                                              &st->o2->tris[st->seed_b], p, q);
        }
        return;
    }
    if (st->canonical) {
        /* the closest pair becomes the step's seed (C2A_Distance, then
         * res->last_triA/B := that pair, then C2A_TimeOfContactStep) */
        int ta, tb;
        distance_query(st->o1, st->o2, (const double(*)[3])st->R, st->T, st->seed_a, st->seed_b, &ta, &tb, NULL,
                       NULL);
        st->seed_a = ta;
        st->seed_b = tb;
    }
    st->distance = tri_distance_plain((const double(*)[3])st->R, st->T, &st->o1->tris[st->seed_a],
                                      &st->o2->tris[st->seed_b], p, q);
    if (st->numCA == 0) st->mint = 1;
    /* controlled error schedule (C2A.cpp:1869-1891) */
    if (st->mint <= 0.005 || st->distance <= 0.5 || st->numCA > 5) {
        st->abs_err = 0;
        st->rel_err = 0;
    } else {
        st->abs_err = 1e+30;
        st->rel_err = (st->numCA <= 2) ? 3 : 0.5;
    }
    st->mint = 1;
    toc_recurse(st, (const double(*)[3])R, T, 0, 0);
}

/* ------------------------------------------------------ contact at the TOC */

/* TOCStepRecurse_Dis_contact, C2A/src/C2A.cpp:1525-1725 (threshold fixed,
 * rel_err = abs_err = 0); contacts are appended in visiting order (the
 * reference pushes each at the front of its list) */
static void contact_recurse(step_state *st, const double R[3][3], const double T[3], int b1, int b2)
{
    C2A_PORT_SCOPE(3);
    const c2a_port_node *n1 = &st->o1->nodes[b1], *n2 = &st->o2->nodes[b2];
    int l1 = n1->first_child < 0, l2 = n2->first_child < 0;
    if (l1 && l2) {
        double p[3], q[3], d;
        int ia = -n1->first_child - 1, ib = -n2->first_child - 1;
        const c2a_port_tri *t1 = &st->o1->tris[ia], *t2 = &st->o2->tris[ib];
        int ft1 = -1, ft2 = -1, fid1[3] = {-1, -1, -1}, fid2[3] = {-1, -1, -1}, col = 0;
        d = tri_distance((const double(*)[3])st->R, st->T, t1, t2, p, q, &ft1, fid1, &ft2, fid2, &col);
        if (ft1 == -1 || ft2 == -1) return;
        if (d <= st->distance) {
            if (st->contacts && st->num_contact < st->max_contacts) {
                c2a_port_contact *c = &st->contacts[st->num_contact];
                double temp[3];
                int k;
                c->type_a = ft1 + 1;
                c->type_b = ft2 + 1;
                for (k = 0; k < 3; k++) c->fid_a[k] = c->fid_b[k] = -1;
                if (ft1 == 0) c->fid_a[0] = t1->idx[fid1[0]];
                if (ft1 == 1) { c->fid_a[0] = t1->idx[fid1[0]]; c->fid_a[1] = t1->idx[(fid1[0] + 1) % 3]; }
                if (ft1 == 2) { c->fid_a[0] = t1->idx[0]; c->fid_a[1] = t1->idx[1]; c->fid_a[2] = t1->idx[2]; }
                if (ft2 == 0) c->fid_b[0] = t2->idx[fid2[0]];
                if (ft2 == 1) { c->fid_b[0] = t2->idx[fid2[0]]; c->fid_b[1] = t2->idx[(fid2[0] + 1) % 3]; }
                if (ft2 == 2) { c->fid_b[0] = t2->idx[0]; c->fid_b[1] = t2->idx[1]; c->fid_b[2] = t2->idx[2]; }
                c->tri_a = ia;
                c->tri_b = ib;
                pv_copy(c->pa, p);
                pv_sub(temp, q, st->T);
                pm_tmul_v(c->pb, (const double(*)[3])st->R, temp);
                c->distance = d;
            }
            st->num_contact++;
        }
        return;
    }
    {
        int a1, a2, c1, c2;
        double R1[3][3], T1[3], R2[3][3], T2[3], S[3], d1, d2;
        children(st, b1, b2, R, T, &a1, &a2, &c1, &c2, R1, T1, R2, T2);
        d1 = bv_distance((const double(*)[3])R1, T1, &st->o1->nodes[a1], &st->o2->nodes[a2], S);
        d2 = bv_distance((const double(*)[3])R2, T2, &st->o1->nodes[c1], &st->o2->nodes[c2], S);
        if (d2 < d1) {
            if ((d2 < (st->distance - st->abs_err)) || (d2 * (1.0 + st->rel_err) < st->distance))
                contact_recurse(st, (const double(*)[3])R2, T2, c1, c2);
            if ((d1 < (st->distance - st->abs_err)) || (d1 * (1.0 + st->rel_err) < st->distance))
                contact_recurse(st, (const double(*)[3])R1, T1, a1, a2);
        } else {
            if ((d1 < (st->distance - st->abs_err)) || (d1 * (1.0 + st->rel_err) < st->distance))
                contact_recurse(st, (const double(*)[3])R1, T1, a1, a2);
            if ((d2 < (st->distance - st->abs_err)) || (d2 * (1.0 + st->rel_err) < st->distance))
                contact_recurse(st, (const double(*)[3])R2, T2, c1, c2);
        }
    }
}

/* canonical contact order: by post-build triangle pair */
static int contact_cmp(const void *a, const void *b)
{
    const c2a_port_contact *x = (const c2a_port_contact *)a, *y = (const c2a_port_contact *)b;
    if (x->tri_a != y->tri_a) return x->tri_a < y->tri_a ? -1 : 1;
    if (x->tri_b != y->tri_b) return x->tri_b < y->tri_b ? -1 : 1;
    return 0;
}

/* C2A_TimeOfContactStep_Contact, C2A.cpp:1727-1775 */
static void contact_step(step_state *st, const double R1[3][3], const double T1[3], const double R2[3][3],
                         const double T2[3], double threshold)
{
    double R[3][3], T[3], dTri;
    relative_transforms(st, R1, T1, R2, T2, R, T);
    dTri = st->distance;
    st->distance = threshold;
    st->rel_err = 0;
    st->abs_err = 0;
    st->mint = 1;
    contact_recurse(st, (const double(*)[3])R, T, 0, 0);
    st->distance = dTri;
}

/* ---------------------------------------------------------- the CA query */

/* C2A_QueryTimeOfContact, C2A/src/C2A.cpp:1987-2146; returns the TOC and
 * fills collisionfree / numCA */
static double query_toc(step_state *st, const c2a_port_params *prm, int translation, int *collisionfree)
{
    double R1[3][3], T1[3], R2[3][3], T2[3];
    double lamda = 0.0, lastLamda = 0, dlamda = 0.0, dist, mint, toc = 0;
    int nItrs;
    st->num_bv_tests = 0;
    st->num_tri_tests = 0;
    st->UpboundTOC = 1;
    st->numCA = 0;
    pm_copy(R1, (const double(*)[3])st->m1->R);
    pv_copy(T1, st->m1->T);
    pm_copy(R2, (const double(*)[3])st->m2->R);
    pv_copy(T2, st->m2->T);
    toc_step(st, R1, T1, R2, T2, translation);
    dist = st->distance;
    mint = st->mint;
    if (translation) {
        *collisionfree = (mint >= 1.0);
        return mint;
    }
    st->numCA = 1;
    lastLamda = mint;
    nItrs = 0;
    while (dist > prm->tol_d) {
        nItrs++;
        if (nItrs > prm->max_iters) break;
        if (mint >= 1.0) {
            *collisionfree = 1;
            return 0;
        }
        dlamda = mint;
        if (dlamda < prm->tol_t) break;
        lamda += dlamda;
        if (lamda >= 1.0) {
            *collisionfree = 1;
            return 0;
        }
        lastLamda = lamda;
        st->numCA++;
        {
            double R19[9], R29[9];
            c2a_port_motion_integrate(st->m1, lamda, R19, T1, NULL);
            c2a_port_motion_integrate(st->m2, lamda, R29, T2, NULL);
            pm_from9(R1, R19);
            pm_from9(R2, R29);
        }
        st->UpboundTOC = 1.0 - lamda;
        toc_step(st, R1, T1, R2, T2, 0);
        dist = st->distance;
        mint = st->mint;
    }
    if (dist == 0 && mint < 0) toc = lastLamda - dlamda;
    else toc = lastLamda;
    *collisionfree = 0;
    if (toc >= 1 - prm->tol_t) toc = 0;
    return toc;
}

int c2a_port_solve(const c2a_port_model *A, const c2a_port_model *B, const double R0a[9], const double T0a[3],
                   const double R1a[9], const double T1a[3], const double R0b[9], const double T0b[3],
                   const double R1b[9], const double T1b[3], int seed_a, int seed_b, const c2a_port_params *prm,
                   c2a_port_result *res, c2a_port_contact *contacts, int max_contacts)
{
    c2a_port_motion m1, m2;
    step_state st;
    int translation, cf = 0;
    double toc;
    memset(res, 0, sizeof(*res));
    if (seed_a < 0 || seed_a >= A->num_tris || seed_b < 0 || seed_b >= B->num_tris) return -1;
    memset(&st, 0, sizeof(st));
    c2a_port_motion_init(&m1, R0a, T0a, R1a, T1a);
    c2a_port_motion_init(&m2, R0b, T0b, R1b, T1b);
    m1.toc_delta = prm->toc_delta;
    m2.toc_delta = prm->toc_delta;
    translation = (m1.angVel < 1e-8 && m2.angVel < 1e-8);
    st.o1 = A;
    st.o2 = B;
    st.m1 = &m1;
    st.m2 = &m2;
    st.seed_a = seed_a;
    st.seed_b = seed_b;
    st.canonical = (prm->mode == C2A_PORT_MODE_CANONICAL);
    toc = query_toc(&st, prm, translation, &cf);
    res->translation = translation;
    res->collisionfree = cf;
    res->toc = toc;
    res->numCA = st.numCA;
    res->distance = st.distance;
    res->mint = st.mint;
    res->num_bv_tests = st.num_bv_tests;
    res->num_tri_tests = st.num_tri_tests;
    res->seed_a = st.seed_a;
    res->seed_b = st.seed_b;
    if (!cf) {
        /* poses at the TOC, then every pair within 2 d + contact_abs (C2A.cpp:2411-2435) */
        double Ra[9], Ta[3], Rb[9], Tb[3], Ram[3][3], Rbm[3][3];
        c2a_port_motion_integrate(&m1, toc, Ra, Ta, NULL);
        c2a_port_motion_integrate(&m2, toc, Rb, Tb, NULL);
        memcpy(res->R_toc[0], Ra, sizeof(Ra));
        memcpy(res->T_toc[0], Ta, sizeof(Ta));
        memcpy(res->R_toc[1], Rb, sizeof(Rb));
        memcpy(res->T_toc[1], Tb, sizeof(Tb));
        if (prm->with_contacts) {
            double threshold = 2 * st.distance + prm->contact_abs;
            pm_from9(Ram, Ra);
            pm_from9(Rbm, Rb);
            st.contacts = contacts;
            st.max_contacts = contacts ? max_contacts : 0;
            st.num_contact = 0;
            st.UpboundTOC = 1;
            contact_step(&st, (const double(*)[3])Ram, Ta, (const double(*)[3])Rbm, Tb, threshold);
            res->num_contact = st.num_contact;
            if (st.canonical && contacts) {
                const int kept = st.num_contact < st.max_contacts ? st.num_contact : st.max_contacts;
                qsort(contacts, (size_t)kept, sizeof(c2a_port_contact), contact_cmp);
            }
        }
    }
    return 0;
}

int c2a_port_contact_only(const c2a_port_model *A, const c2a_port_model *B, const double Ra[9], const double Ta[3],
                          const double Rb[9], const double Tb[3], double threshold, c2a_port_contact *contacts,
                          int max_contacts)
{
    step_state st;
    double Ram[3][3], Rbm[3][3];
    memset(&st, 0, sizeof(st));
    st.o1 = A;
    st.o2 = B;
    st.contacts = contacts;
    st.max_contacts = contacts ? max_contacts : 0;
    pm_from9(Ram, Ra);
    pm_from9(Rbm, Rb);
    contact_step(&st, (const double(*)[3])Ram, Ta, (const double(*)[3])Rbm, Tb, threshold);
    return st.num_contact;
}

int c2a_port_step(const c2a_port_model *A, const c2a_port_model *B, const double P[48], int seed_a, int seed_b,
                  double lambda, int num_ca, double prev_mint, const c2a_port_params *prm, c2a_port_result *res)
{
    c2a_port_motion m1, m2;
    step_state st;
    double R1[3][3], T1[3], R2[3][3], T2[3];
    int translation;
    memset(res, 0, sizeof(*res));
    if (seed_a < 0 || seed_a >= A->num_tris || seed_b < 0 || seed_b >= B->num_tris) return -1;
    memset(&st, 0, sizeof(st));
    c2a_port_motion_init(&m1, P, P + 9, P + 12, P + 21);
    c2a_port_motion_init(&m2, P + 24, P + 33, P + 36, P + 45);
    m1.toc_delta = prm->toc_delta;
    m2.toc_delta = prm->toc_delta;
    translation = (m1.angVel < 1e-8 && m2.angVel < 1e-8);
    if (lambda != 0.0) {
        double R19[9], R29[9];
        c2a_port_motion_integrate(&m1, lambda, R19, T1, NULL);
        c2a_port_motion_integrate(&m2, lambda, R29, T2, NULL);
        pm_from9(R1, R19);
        pm_from9(R2, R29);
    } else {
        pm_copy(R1, (const double(*)[3])m1.R);
        pv_copy(T1, m1.T);
        pm_copy(R2, (const double(*)[3])m2.R);
        pv_copy(T2, m2.T);
    }
    st.o1 = A;
    st.o2 = B;
    st.m1 = &m1;
    st.m2 = &m2;
    st.seed_a = seed_a;
    st.seed_b = seed_b;
    st.numCA = num_ca;
    st.mint = prev_mint;
    st.UpboundTOC = 1.0 - lambda;
    st.canonical = (prm->mode == C2A_PORT_MODE_CANONICAL);
    toc_step(&st, R1, T1, R2, T2, translation);
    res->translation = translation;
    res->numCA = num_ca;
    res->toc = lambda;
    res->distance = st.distance;
    res->mint = st.mint;
    res->num_bv_tests = st.num_bv_tests;
    res->num_tri_tests = st.num_tri_tests;
    res->seed_a = st.seed_a;
    res->seed_b = st.seed_b;
    return 0;
}
