/*
 * c2a_port_build.c -- oracle port of the C2A RSS hierarchy build.
 *
 * Restates C2A_Model::EndModel (C2A/src/C2A_PQP.cpp:332-417), C2A_BuildModel /
 * build_recurse / split_tris / make_parent_relative (C2A/src/C2A_Build.cpp:
 * 279-574) and C2A_BV::FitToTris_Corner / ComputeAngularRadius
 * (C2A/src/C2A_BV.cpp:71-111, 354-635), keeping only the fields the CA path
 * reads (R, Tr, l, r, angularRadius, R_loc, first_child).  The eigen-solver
 * stands in for PQP's Meigen (absent third-party code): cyclic Jacobi
 * rotations, Golub and Van Loan, "Matrix Computations", sec. 8.5.
 * Test infrastructure only.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "c2a_port.h"
#include "c2a_port_matvec.h"

void c2a_port_jacobi3(double v[3][3], double d[3], const double a_in[3][3])
{
    double a[3][3];
    int i, j, sweep, p, q;
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) {
            a[i][j] = a_in[i][j];
            v[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (sweep = 0; sweep < 50; sweep++) {
        double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (off == 0.0) break;
        for (p = 0; p < 2; p++) {
            for (q = p + 1; q < 3; q++) {
                double apq = a[p][q], app = a[p][p], aqq = a[q][q];
                int r = 3 - p - q, k;
                double theta, t, c, s, arp, arq;
                if (apq == 0.0) continue;
                /* entry already below the precision of both diagonal terms */
                if (sweep > 3 && fabs(app) + 100.0 * fabs(apq) == fabs(app) &&
                    fabs(aqq) + 100.0 * fabs(apq) == fabs(aqq)) {
                    a[p][q] = a[q][p] = 0.0;
                    continue;
                }
                theta = (aqq - app) / (2.0 * apq);
                t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
                if (theta < 0.0) t = -t;
                c = 1.0 / sqrt(t * t + 1.0);
                s = t * c;
                a[p][p] = app - t * apq;
                a[q][q] = aqq + t * apq;
                a[p][q] = a[q][p] = 0.0;
                arp = a[r][p];
                arq = a[r][q];
                a[r][p] = a[p][r] = c * arp - s * arq;
                a[r][q] = a[q][r] = s * arp + c * arq;
                for (k = 0; k < 3; k++) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
        }
    }
    d[0] = a[0][0];
    d[1] = a[1][1];
    d[2] = a[2][2];
}

/* C2A_Build.cpp:279-335 get_covariance_triverts */
static void covariance_triverts(double M[3][3], const c2a_port_tri *tris, int n)
{
    double S1[3] = {0.0, 0.0, 0.0};
    double S2[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    int i;
    double nn;
    for (i = 0; i < n; i++) {
        const double *p1 = tris[i].p1, *p2 = tris[i].p2, *p3 = tris[i].p3;
        S1[0] += p1[0] + p2[0] + p3[0];
        S1[1] += p1[1] + p2[1] + p3[1];
        S1[2] += p1[2] + p2[2] + p3[2];
        S2[0][0] += (p1[0] * p1[0] + p2[0] * p2[0] + p3[0] * p3[0]);
        S2[1][1] += (p1[1] * p1[1] + p2[1] * p2[1] + p3[1] * p3[1]);
        S2[2][2] += (p1[2] * p1[2] + p2[2] * p2[2] + p3[2] * p3[2]);
        S2[0][1] += (p1[0] * p1[1] + p2[0] * p2[1] + p3[0] * p3[1]);
        S2[0][2] += (p1[0] * p1[2] + p2[0] * p2[2] + p3[0] * p3[2]);
        S2[1][2] += (p1[1] * p1[2] + p2[1] * p2[2] + p3[1] * p3[2]);
    }
    nn = (double)(3 * n);
    M[0][0] = S2[0][0] - S1[0] * S1[0] / nn;
    M[1][1] = S2[1][1] - S1[1] * S1[1] / nn;
    M[2][2] = S2[2][2] - S1[2] * S1[2] / nn;
    M[0][1] = S2[0][1] - S1[0] * S1[1] / nn;
    M[1][2] = S2[1][2] - S1[1] * S1[2] / nn;
    M[0][2] = S2[0][2] - S1[0] * S1[2] / nn;
    M[1][0] = M[0][1];
    M[2][0] = M[0][2];
    M[2][1] = M[1][2];
}

/* C2A_Build.cpp:252-275 get_centroid_triverts */
static void centroid_triverts(double c[3], const c2a_port_tri *tris, int n)
{
    int i;
    double nn;
    c[0] = c[1] = c[2] = 0.0;
    for (i = 0; i < n; i++) {
        const double *p1 = tris[i].p1, *p2 = tris[i].p2, *p3 = tris[i].p3;
        c[0] += p1[0] + p2[0] + p3[0];
        c[1] += p1[1] + p2[1] + p3[1];
        c[2] += p1[2] + p2[2] + p3[2];
    }
    nn = (double)(3 * n);
    c[0] /= nn;
    c[1] /= nn;
    c[2] /= nn;
}

/* C2A_Build.cpp:344-385 split_tris: in-place partition by projected centroid */
static int split_tris(c2a_port_tri *tris, int n, const double a[3], double c)
{
    int i, c1 = 0;
    for (i = 0; i < n; i++) {
        double p[3], x;
        pv_copy(p, tris[i].p1);
        pv_add(p, p, tris[i].p2);
        pv_add(p, p, tris[i].p3);
        x = pv_dot(p, a);
        x /= 3.0;
        if (x <= c) {
            c2a_port_tri tmp = tris[i];
            tris[i] = tris[c1];
            tris[c1] = tmp;
            c1++;
        }
    }
    if (c1 == 0 || c1 == n) c1 = n / 2;
    return c1;
}

static double max_of_two(double a, double b) { return a > b ? a : b; }

/* C2A_BV.cpp:71-111 ComputeAngularRadius + 354-635 FitToTris_Corner (RSS part) */
static void fit_rss(c2a_port_node *b, const double O[3][3], const c2a_port_tri *tris, int n, double *P)
{
    int i, np = 3 * n, minindex, maxindex;
    double minx, maxx, miny, maxy, minz, maxz, cz, radsqr, x, y, dz, c[3];
    double dx, dy, u, t, a;

    /* distance of the farthest vertex from the model origin */
    b->angR = 0.0;
    for (i = 0; i < n; i++) {
        double d;
        d = pv_len(tris[i].p1);
        if (d > b->angR) b->angR = d;
        d = pv_len(tris[i].p2);
        if (d > b->angR) b->angR = d;
        d = pv_len(tris[i].p3);
        if (d > b->angR) b->angR = d;
    }

    pm_copy(b->R, O);
    for (i = 0; i < n; i++) {
        pm_tmul_v(&P[9 * i + 0], b->R, tris[i].p1);
        pm_tmul_v(&P[9 * i + 3], b->R, tris[i].p2);
        pm_tmul_v(&P[9 * i + 6], b->R, tris[i].p3);
    }
#define PX(k) P[3 * (k) + 0]
#define PY(k) P[3 * (k) + 1]
#define PZ(k) P[3 * (k) + 2]
    /* the OBB in the same frame (C2A/src/C2A_BV.cpp:144-170): the projected
     * extents, centre back in the model frame */
    minx = maxx = PX(0);
    miny = maxy = PY(0);
    minz = maxz = PZ(0);
    for (i = 1; i < np; i++) {
        if (PX(i) < minx) minx = PX(i);
        else if (PX(i) > maxx) maxx = PX(i);
        if (PY(i) < miny) miny = PY(i);
        else if (PY(i) > maxy) maxy = PY(i);
        if (PZ(i) < minz) minz = PZ(i);
        else if (PZ(i) > maxz) maxz = PZ(i);
    }
    c[0] = 0.5 * (maxx + minx);
    c[1] = 0.5 * (maxy + miny);
    c[2] = 0.5 * (maxz + minz);
    pm_mul_v(b->To, (const double(*)[3])b->R, c);
    b->d[0] = 0.5 * (maxx - minx);
    b->d[1] = 0.5 * (maxy - miny);
    b->d[2] = 0.5 * (maxz - minz);
    /* thickness -> radius and rectangle height */
    minz = maxz = PZ(0);
    for (i = 1; i < np; i++) {
        if (PZ(i) < minz) minz = PZ(i);
        else if (PZ(i) > maxz) maxz = PZ(i);
    }
    b->r = 0.5 * (maxz - minz);
    radsqr = b->r * b->r;
    cz = 0.5 * (maxz + minz);

    /* x extent, shrunk by the sphere cap at the extreme points, then grown */
    minindex = maxindex = 0;
    for (i = 1; i < np; i++) {
        if (PX(i) < PX(minindex)) minindex = i;
        else if (PX(i) > PX(maxindex)) maxindex = i;
    }
    dz = PZ(minindex) - cz;
    minx = PX(minindex) + sqrt(max_of_two(radsqr - dz * dz, 0));
    dz = PZ(maxindex) - cz;
    maxx = PX(maxindex) - sqrt(max_of_two(radsqr - dz * dz, 0));
    for (i = 0; i < np; i++) {
        if (PX(i) < minx) {
            dz = PZ(i) - cz;
            x = PX(i) + sqrt(max_of_two(radsqr - dz * dz, 0));
            if (x < minx) minx = x;
        }
    }
    for (i = 0; i < np; i++) {
        if (PX(i) > maxx) {
            dz = PZ(i) - cz;
            x = PX(i) - sqrt(max_of_two(radsqr - dz * dz, 0));
            if (x > maxx) maxx = x;
        }
    }
    /* same for y */
    minindex = maxindex = 0;
    for (i = 1; i < np; i++) {
        if (PY(i) < PY(minindex)) minindex = i;
        else if (PY(i) > PY(maxindex)) maxindex = i;
    }
    dz = PZ(minindex) - cz;
    miny = PY(minindex) + sqrt(max_of_two(radsqr - dz * dz, 0));
    dz = PZ(maxindex) - cz;
    maxy = PY(maxindex) - sqrt(max_of_two(radsqr - dz * dz, 0));
    for (i = 0; i < np; i++) {
        if (PY(i) < miny) {
            dz = PZ(i) - cz;
            y = PY(i) + sqrt(max_of_two(radsqr - dz * dz, 0));
            if (y < miny) miny = y;
        }
    }
    for (i = 0; i < np; i++) {
        if (PY(i) > maxy) {
            dz = PZ(i) - cz;
            y = PY(i) - sqrt(max_of_two(radsqr - dz * dz, 0));
            if (y > maxy) maxy = y;
        }
    }
    /* grow the rectangle diagonally where a corner leaves points uncovered */
    a = sqrt(0.5);
    for (i = 0; i < np; i++) {
        if (PX(i) > maxx) {
            if (PY(i) > maxy) {
                dx = PX(i) - maxx;
                dy = PY(i) - maxy;
                u = dx * a + dy * a;
                t = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - PZ(i)) * (cz - PZ(i));
                u = u - sqrt(max_of_two(radsqr - t, 0));
                if (u > 0) {
                    maxx += u * a;
                    maxy += u * a;
                }
            } else if (PY(i) < miny) {
                dx = PX(i) - maxx;
                dy = PY(i) - miny;
                u = dx * a - dy * a;
                t = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - PZ(i)) * (cz - PZ(i));
                u = u - sqrt(max_of_two(radsqr - t, 0));
                if (u > 0) {
                    maxx += u * a;
                    miny -= u * a;
                }
            }
        } else if (PX(i) < minx) {
            if (PY(i) > maxy) {
                dx = PX(i) - minx;
                dy = PY(i) - maxy;
                u = dy * a - dx * a;
                t = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - PZ(i)) * (cz - PZ(i));
                u = u - sqrt(max_of_two(radsqr - t, 0));
                if (u > 0) {
                    minx -= u * a;
                    maxy += u * a;
                }
            } else if (PY(i) < miny) {
                dx = PX(i) - minx;
                dy = PY(i) - miny;
                u = -dx * a - dy * a;
                t = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - PZ(i)) * (cz - PZ(i));
                u = u - sqrt(max_of_two(radsqr - t, 0));
                if (u > 0) {
                    minx -= u * a;
                    miny -= u * a;
                }
            }
        }
    }
#undef PX
#undef PY
#undef PZ
    c[0] = minx;
    c[1] = miny;
    c[2] = cz;
    pm_mul_v(b->Tr, b->R, c); /* rectangle corner (minx, miny, cz) back in the model frame */
    b->l[0] = maxx - minx;
    if (b->l[0] < 0) b->l[0] = 0;
    b->l[1] = maxy - miny;
    if (b->l[1] < 0) b->l[1] = 0;
}

typedef struct build_ctx {
    c2a_port_model *m;
    int num_nodes;
    double *P; /* scratch: projected vertices */
} build_ctx;

/* C2A_Build.cpp:394-488 build_recurse */
static void build_recurse(build_ctx *ctx, int bn, int first_tri, int n)
{
    c2a_port_model *m = ctx->m;
    c2a_port_node *b = &m->nodes[bn];
    double C[3][3], E[3][3], R[3][3], s[3], axis[3], mean[3], coord;
    int mn, mid, mx;

    covariance_triverts(C, &m->tris[first_tri], n);
    c2a_port_jacobi3(E, s, (const double(*)[3])C);
    /* axes in order of decreasing eigenvalue */
    if (s[0] > s[1]) { mx = 0; mn = 1; }
    else { mn = 0; mx = 1; }
    if (s[2] < s[mn]) { mid = mn; mn = 2; }
    else if (s[2] > s[mx]) { mid = mx; mx = 2; }
    else { mid = 2; }
    R[0][0] = E[0][mx]; R[1][0] = E[1][mx]; R[2][0] = E[2][mx];
    R[0][1] = E[0][mid]; R[1][1] = E[1][mid]; R[2][1] = E[2][mid];
    R[0][2] = E[1][mx] * E[2][mid] - E[1][mid] * E[2][mx];
    R[1][2] = E[0][mid] * E[2][mx] - E[0][mx] * E[2][mid];
    R[2][2] = E[0][mx] * E[1][mid] - E[0][mid] * E[1][mx];

    fit_rss(b, (const double(*)[3])R, &m->tris[first_tri], n, ctx->P);
    pm_copy(b->Rloc, b->R);

    if (n == 1) {
        b->first_child = -(first_tri + 1);
    } else {
        int nfirst, fc;
        b->first_child = ctx->num_nodes;
        ctx->num_nodes += 2;
        axis[0] = R[0][0]; axis[1] = R[1][0]; axis[2] = R[2][0];
        centroid_triverts(mean, &m->tris[first_tri], n);
        coord = pv_dot(axis, mean);
        nfirst = split_tris(&m->tris[first_tri], n, axis, coord);
        fc = b->first_child;
        build_recurse(ctx, fc, first_tri, nfirst);
        build_recurse(ctx, fc + 1, first_tri + nfirst, n - nfirst);
    }
}

/* C2A_Build.cpp:493-544 make_parent_relative (children first, then self) */
static void make_parent_relative(c2a_port_model *m, int bn, const double pR[3][3], const double pTr[3],
                                 const double pTo[3])
{
    c2a_port_node *b = &m->nodes[bn];
    double Rpc[3][3], Tpc[3];
    if (b->first_child >= 0) {
        make_parent_relative(m, b->first_child, (const double(*)[3])b->R, b->Tr, b->To);
        make_parent_relative(m, b->first_child + 1, (const double(*)[3])b->R, b->Tr, b->To);
    }
    pm_tmul(Rpc, pR, (const double(*)[3])b->R);
    pm_copy(b->R, (const double(*)[3])Rpc);
    pv_sub(Tpc, b->Tr, pTr);
    pm_tmul_v(b->Tr, pR, Tpc);
    pv_sub(Tpc, b->To, pTo);
    pm_tmul_v(b->To, pR, Tpc);
}

int c2a_port_model_build(c2a_port_model *m, int num_tris, const double *tv, const int *ids, const int *vidx)
{
    int i;
    build_ctx ctx;
    double I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double Z[3] = {0, 0, 0};
    memset(m, 0, sizeof(*m));
    if (num_tris <= 0) return -5; /* PQP_ERR_BUILD_EMPTY_MODEL (C2A_PQP.cpp:352-357) */
    m->num_tris = num_tris;
    m->num_nodes = 2 * num_tris - 1;
    m->tris = (c2a_port_tri *)calloc((size_t)num_tris, sizeof(c2a_port_tri));
    m->nodes = (c2a_port_node *)calloc((size_t)m->num_nodes, sizeof(c2a_port_node));
    ctx.P = (double *)malloc(sizeof(double) * 9 * (size_t)num_tris);
    if (!m->tris || !m->nodes || !ctx.P) {
        free(ctx.P);
        c2a_port_model_free(m);
        return -1;
    }
    for (i = 0; i < num_tris; i++) {
        c2a_port_tri *t = &m->tris[i];
        memcpy(t->p1, tv + 9 * i, 3 * sizeof(double));
        memcpy(t->p2, tv + 9 * i + 3, 3 * sizeof(double));
        memcpy(t->p3, tv + 9 * i + 6, 3 * sizeof(double));
        t->id = ids ? ids[i] : i;
        t->idx[0] = vidx ? vidx[3 * i] : -1;
        t->idx[1] = vidx ? vidx[3 * i + 1] : -1;
        t->idx[2] = vidx ? vidx[3 * i + 2] : -1;
    }
    ctx.m = m;
    ctx.num_nodes = 1;
    build_recurse(&ctx, 0, 0, num_tris);
    make_parent_relative(m, 0, (const double(*)[3])I, Z, Z);
    free(ctx.P);
    return 0;
}

void c2a_port_model_free(c2a_port_model *m)
{
    free(m->tris);
    free(m->nodes);
    m->tris = 0;
    m->nodes = 0;
    m->num_tris = m->num_nodes = 0;
}
