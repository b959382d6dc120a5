/*
 * c2a_port_geom.c -- oracle port of the two distance kernels of the CA path.
 *
 *  - RSS rectangle distance with closest-point direction S:
 *    C2ARectDist, C2A/C2A_RectDist.h:44-934 (Larsen's edge-pair Voronoi
 *    tests, then the face-normal separation fallback).
 *  - Triangle distance with contact features:
 *    ClosestPoints / TriDist, C2A/src/C2A.cpp:59-405.
 *
 * Every expression keeps the reference's left-to-right evaluation so the
 * results are bit-identical under -ffp-contract=off.  Test infrastructure.
 */
#include <math.h>
#include "c2a_port.h"
#include "c2a_port_matvec.h"

/* ---------------------------------------------------------------- RectDist */

static void clampd(double *v, double lo, double hi)
{
    if (*v < lo) *v = lo;
    else if (*v > hi) *v = hi;
}

/* segment parameters of the closest points of two edges (C2A_RectDist.h:81-111) */
static void seg_closest(double *t, double *u, double a, double b, double AdB, double AdT, double BdT)
{
    double denom = 1 - (AdB) * (AdB);
    if (denom == 0) *t = 0;
    else {
        *t = (AdT - BdT * AdB) / denom;
        clampd(t, 0, a);
    }
    *u = *t * AdB - BdT;
    if (*u < 0) {
        *u = 0;
        *t = AdT;
        clampd(t, 0, a);
    } else if (*u > b) {
        *u = b;
        *t = *u * AdB + AdT;
        clampd(t, 0, a);
    }
}

/* is the edge-pair closest point inside the edge's Voronoi slab (C2A_RectDist.h:123-154) */
static int voronoi_ok(double a, double b, double AnB, double AnT, double AdB, double AdT, double BdT)
{
    double t, u, v;
    if ((AnB < 0 ? -AnB : AnB) < 1e-7) return 0;
    u = -AnT / AnB;
    clampd(&u, 0, b);
    t = u * AdB + AdT;
    clampd(&t, 0, a);
    v = t * AdB - BdT;
    if (AnB > 0) return v > (u + 1e-7);
    return v < (u - 1e-7);
}

/* d = |Q - P| for an accepted edge pair; S = Q - P */
static double finish(double P[3], double Q[3], double S[3])
{
    S[0] = Q[0] - P[0];
    S[1] = Q[1] - P[1];
    S[2] = Q[2] - P[2];
    return sqrt(pv_dot(S, S));
}

double c2a_port_rectdist(const double Rab9[9], const double Tab[3], const double a[2], const double b[2],
                         double P[3], double Q[3], double S[3])
{
    double Rab[3][3];
    double A0B0, A0B1, A1B0, A1B1;
    double aA0B0, aA0B1, aA1B0, aA1B1, bA0B0, bA0B1, bA1B0, bA1B1;
    double Tba[3], t, u;
    double ALLx, ALUx, AULx, AUUx, BLLx, BLUx, BULx, BUUx;
    double LA1lx, LA1ux, UA1lx, UA1ux, LB1lx, LB1ux, UB1lx, UB1ux;
    double ALLy, ALUy, AULy, AUUy, LA1ly, LA1uy, UA1ly, UA1uy, LB0lx, LB0ux, UB0lx, UB0ux;
    double BLLy, BLUy, BULy, BUUy, LA0lx, LA0ux, UA0lx, UA0ux, LB1ly, LB1uy, UB1ly, UB1uy;
    double LA0ly, LA0uy, UA0ly, UA0uy, LB0ly, LB0uy, UB0ly, UB0uy;
    double sep1, sep2, sep;

    pm_from9(Rab, Rab9);
    A0B0 = Rab[0][0]; A0B1 = Rab[0][1]; A1B0 = Rab[1][0]; A1B1 = Rab[1][1];
    aA0B0 = a[0] * A0B0; aA0B1 = a[0] * A0B1; aA1B0 = a[1] * A1B0; aA1B1 = a[1] * A1B1;
    bA0B0 = b[0] * A0B0; bA1B0 = b[0] * A1B0; bA0B1 = b[1] * A0B1; bA1B1 = b[1] * A1B1;
    pm_tmul_v(Tba, (const double(*)[3])Rab, Tab);

    /* x-extents of A's edges along B0, and of B's edges along A0 */
    ALLx = -Tba[0];
    ALUx = ALLx + aA1B0;
    AULx = ALLx + aA0B0;
    AUUx = ALUx + aA0B0;
    if (ALLx < ALUx) { LA1lx = ALLx; LA1ux = ALUx; UA1lx = AULx; UA1ux = AUUx; }
    else { LA1lx = ALUx; LA1ux = ALLx; UA1lx = AUUx; UA1ux = AULx; }
    BLLx = Tab[0];
    BLUx = BLLx + bA0B1;
    BULx = BLLx + bA0B0;
    BUUx = BLUx + bA0B0;
    if (BLLx < BLUx) { LB1lx = BLLx; LB1ux = BLUx; UB1lx = BULx; UB1ux = BUUx; }
    else { LB1lx = BLUx; LB1ux = BLLx; UB1lx = BUUx; UB1ux = BULx; }

    /* edge pairs (A edge along A1) x (B edge along B1) */
    if ((UA1ux > b[0]) && (UB1ux > a[0])) {
        if (((UA1lx > b[0]) ||
             voronoi_ok(b[1], a[1], A1B0, aA0B0 - b[0] - Tba[0], A1B1, aA0B1 - Tba[1], -Tab[1] - bA1B0)) &&
            ((UB1lx > a[0]) ||
             voronoi_ok(a[1], b[1], A0B1, Tab[0] + bA0B0 - a[0], A1B1, Tab[1] + bA1B0, Tba[1] - aA0B1))) {
            seg_closest(&t, &u, a[1], b[1], A1B1, Tab[1] + bA1B0, Tba[1] - aA0B1);
            P[0] = a[0]; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * b[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][0] * b[0] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][0] * b[0] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((UA1lx < 0) && (LB1ux > a[0])) {
        if (((UA1ux < 0) ||
             voronoi_ok(b[1], a[1], -A1B0, Tba[0] - aA0B0, A1B1, aA0B1 - Tba[1], -Tab[1])) &&
            ((LB1lx > a[0]) ||
             voronoi_ok(a[1], b[1], A0B1, Tab[0] - a[0], A1B1, Tab[1], Tba[1] - aA0B1))) {
            seg_closest(&t, &u, a[1], b[1], A1B1, Tab[1], Tba[1] - aA0B1);
            P[0] = a[0]; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA1ux > b[0]) && (UB1lx < 0)) {
        if (((LA1lx > b[0]) ||
             voronoi_ok(b[1], a[1], A1B0, -Tba[0] - b[0], A1B1, -Tba[1], -Tab[1] - bA1B0)) &&
            ((UB1ux < 0) ||
             voronoi_ok(a[1], b[1], -A0B1, -Tab[0] - bA0B0, A1B1, Tab[1] + bA1B0, Tba[1]))) {
            seg_closest(&t, &u, a[1], b[1], A1B1, Tab[1] + bA1B0, Tba[1]);
            P[0] = 0; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * b[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][0] * b[0] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][0] * b[0] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA1lx < 0) && (LB1lx < 0)) {
        if (((LA1ux < 0) ||
             voronoi_ok(b[1], a[1], -A1B0, Tba[0], A1B1, -Tba[1], -Tab[1])) &&
            ((LB1ux < 0) ||
             voronoi_ok(a[1], b[1], -A0B1, -Tab[0], A1B1, Tab[1], Tba[1]))) {
            seg_closest(&t, &u, a[1], b[1], A1B1, Tab[1], Tba[1]);
            P[0] = 0; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }

    /* y-extents of A's edges along B1, and B's edges (along B0) along A0 */
    ALLy = -Tba[1];
    ALUy = ALLy + aA1B1;
    AULy = ALLy + aA0B1;
    AUUy = ALUy + aA0B1;
    if (ALLy < ALUy) { LA1ly = ALLy; LA1uy = ALUy; UA1ly = AULy; UA1uy = AUUy; }
    else { LA1ly = ALUy; LA1uy = ALLy; UA1ly = AUUy; UA1uy = AULy; }
    if (BLLx < BULx) { LB0lx = BLLx; LB0ux = BULx; UB0lx = BLUx; UB0ux = BUUx; }
    else { LB0lx = BULx; LB0ux = BLLx; UB0lx = BUUx; UB0ux = BLUx; }

    /* (A edge along A1) x (B edge along B0) */
    if ((UA1uy > b[1]) && (UB0ux > a[0])) {
        if (((UA1ly > b[1]) ||
             voronoi_ok(b[0], a[1], A1B1, aA0B1 - Tba[1] - b[1], A1B0, aA0B0 - Tba[0], -Tab[1] - bA1B1)) &&
            ((UB0lx > a[0]) ||
             voronoi_ok(a[1], b[0], A0B0, Tab[0] - a[0] + bA0B1, A1B0, Tab[1] + bA1B1, Tba[0] - aA0B0))) {
            seg_closest(&t, &u, a[1], b[0], A1B0, Tab[1] + bA1B1, Tba[0] - aA0B0);
            P[0] = a[0]; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * b[1] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][1] * b[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][1] * b[1] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((UA1ly < 0) && (LB0ux > a[0])) {
        if (((UA1uy < 0) ||
             voronoi_ok(b[0], a[1], -A1B1, Tba[1] - aA0B1, A1B0, aA0B0 - Tba[0], -Tab[1])) &&
            ((LB0lx > a[0]) ||
             voronoi_ok(a[1], b[0], A0B0, Tab[0] - a[0], A1B0, Tab[1], Tba[0] - aA0B0))) {
            seg_closest(&t, &u, a[1], b[0], A1B0, Tab[1], Tba[0] - aA0B0);
            P[0] = a[0]; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA1uy > b[1]) && (UB0lx < 0)) {
        if (((LA1ly > b[1]) ||
             voronoi_ok(b[0], a[1], A1B1, -Tba[1] - b[1], A1B0, -Tba[0], -Tab[1] - bA1B1)) &&
            ((UB0ux < 0) ||
             voronoi_ok(a[1], b[0], -A0B0, -Tab[0] - bA0B1, A1B0, Tab[1] + bA1B1, Tba[0]))) {
            seg_closest(&t, &u, a[1], b[0], A1B0, Tab[1] + bA1B1, Tba[0]);
            P[0] = 0; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * b[1] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][1] * b[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][1] * b[1] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA1ly < 0) && (LB0lx < 0)) {
        if (((LA1uy < 0) ||
             voronoi_ok(b[0], a[1], -A1B1, Tba[1], A1B0, -Tba[0], -Tab[1])) &&
            ((LB0ux < 0) ||
             voronoi_ok(a[1], b[0], -A0B0, -Tab[0], A1B0, Tab[1], Tba[0]))) {
            seg_closest(&t, &u, a[1], b[0], A1B0, Tab[1], Tba[0]);
            P[0] = 0; P[1] = t; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }

    /* y-extents of B's edges; x-extents of A's edges along A0 */
    BLLy = Tab[1];
    BLUy = BLLy + bA1B1;
    BULy = BLLy + bA1B0;
    BUUy = BLUy + bA1B0;
    if (ALLx < AULx) { LA0lx = ALLx; LA0ux = AULx; UA0lx = ALUx; UA0ux = AUUx; }
    else { LA0lx = AULx; LA0ux = ALLx; UA0lx = AUUx; UA0ux = ALUx; }
    if (BLLy < BLUy) { LB1ly = BLLy; LB1uy = BLUy; UB1ly = BULy; UB1uy = BUUy; }
    else { LB1ly = BLUy; LB1uy = BLLy; UB1ly = BUUy; UB1uy = BULy; }

    /* (A edge along A0) x (B edge along B1) */
    if ((UA0ux > b[0]) && (UB1uy > a[1])) {
        if (((UA0lx > b[0]) ||
             voronoi_ok(b[1], a[0], A0B0, aA1B0 - Tba[0] - b[0], A0B1, aA1B1 - Tba[1], -Tab[0] - bA0B0)) &&
            ((UB1ly > a[1]) ||
             voronoi_ok(a[0], b[1], A1B1, Tab[1] - a[1] + bA1B0, A0B1, Tab[0] + bA0B0, Tba[1] - aA1B1))) {
            seg_closest(&t, &u, a[0], b[1], A0B1, Tab[0] + bA0B0, Tba[1] - aA1B1);
            P[0] = t; P[1] = a[1]; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * b[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][0] * b[0] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][0] * b[0] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((UA0lx < 0) && (LB1uy > a[1])) {
        if (((UA0ux < 0) ||
             voronoi_ok(b[1], a[0], -A0B0, Tba[0] - aA1B0, A0B1, aA1B1 - Tba[1], -Tab[0])) &&
            ((LB1ly > a[1]) ||
             voronoi_ok(a[0], b[1], A1B1, Tab[1] - a[1], A0B1, Tab[0], Tba[1] - aA1B1))) {
            seg_closest(&t, &u, a[0], b[1], A0B1, Tab[0], Tba[1] - aA1B1);
            P[0] = t; P[1] = a[1]; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA0ux > b[0]) && (UB1ly < 0)) {
        if (((LA0lx > b[0]) ||
             voronoi_ok(b[1], a[0], A0B0, -b[0] - Tba[0], A0B1, -Tba[1], -bA0B0 - Tab[0])) &&
            ((UB1uy < 0) ||
             voronoi_ok(a[0], b[1], -A1B1, -Tab[1] - bA1B0, A0B1, Tab[0] + bA0B0, Tba[1]))) {
            seg_closest(&t, &u, a[0], b[1], A0B1, Tab[0] + bA0B0, Tba[1]);
            P[0] = t; P[1] = 0; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * b[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][0] * b[0] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][0] * b[0] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA0lx < 0) && (LB1ly < 0)) {
        if (((LA0ux < 0) ||
             voronoi_ok(b[1], a[0], -A0B0, Tba[0], A0B1, -Tba[1], -Tab[0])) &&
            ((LB1uy < 0) ||
             voronoi_ok(a[0], b[1], -A1B1, -Tab[1], A0B1, Tab[0], Tba[1]))) {
            seg_closest(&t, &u, a[0], b[1], A0B1, Tab[0], Tba[1]);
            P[0] = t; P[1] = 0; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * u;
            Q[1] = Tab[1] + Rab[1][1] * u;
            Q[2] = Tab[2] + Rab[2][1] * u;
            return finish(P, Q, S);
        }
    }

    /* y-extents along A1 of A's edges along A0, and of B's edges along B0 */
    if (ALLy < AULy) { LA0ly = ALLy; LA0uy = AULy; UA0ly = ALUy; UA0uy = AUUy; }
    else { LA0ly = AULy; LA0uy = ALLy; UA0ly = AUUy; UA0uy = ALUy; }
    if (BLLy < BULy) { LB0ly = BLLy; LB0uy = BULy; UB0ly = BLUy; UB0uy = BUUy; }
    else { LB0ly = BULy; LB0uy = BLLy; UB0ly = BUUy; UB0uy = BLUy; }

    /* (A edge along A0) x (B edge along B0) */
    if ((UA0uy > b[1]) && (UB0uy > a[1])) {
        if (((UA0ly > b[1]) ||
             voronoi_ok(b[0], a[0], A0B1, aA1B1 - Tba[1] - b[1], A0B0, aA1B0 - Tba[0], -Tab[0] - bA0B1)) &&
            ((UB0ly > a[1]) ||
             voronoi_ok(a[0], b[0], A1B0, Tab[1] - a[1] + bA1B1, A0B0, Tab[0] + bA0B1, Tba[0] - aA1B0))) {
            seg_closest(&t, &u, a[0], b[0], A0B0, Tab[0] + bA0B1, Tba[0] - aA1B0);
            P[0] = t; P[1] = a[1]; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * b[1] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][1] * b[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][1] * b[1] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((UA0ly < 0) && (LB0uy > a[1])) {
        if (((UA0uy < 0) ||
             voronoi_ok(b[0], a[0], -A0B1, Tba[1] - aA1B1, A0B0, aA1B0 - Tba[0], -Tab[0])) &&
            ((LB0ly > a[1]) ||
             voronoi_ok(a[0], b[0], A1B0, Tab[1] - a[1], A0B0, Tab[0], Tba[0] - aA1B0))) {
            seg_closest(&t, &u, a[0], b[0], A0B0, Tab[0], Tba[0] - aA1B0);
            P[0] = t; P[1] = a[1]; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA0uy > b[1]) && (UB0ly < 0)) {
        if (((LA0ly > b[1]) ||
             voronoi_ok(b[0], a[0], A0B1, -Tba[1] - b[1], A0B0, -Tba[0], -Tab[0] - bA0B1)) &&
            ((UB0uy < 0) ||
             voronoi_ok(a[0], b[0], -A1B0, -Tab[1] - bA1B1, A0B0, Tab[0] + bA0B1, Tba[0]))) {
            seg_closest(&t, &u, a[0], b[0], A0B0, Tab[0] + bA0B1, Tba[0]);
            P[0] = t; P[1] = 0; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][1] * b[1] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][1] * b[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][1] * b[1] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }
    if ((LA0ly < 0) && (LB0ly < 0)) {
        if (((LA0uy < 0) ||
             voronoi_ok(b[0], a[0], -A0B1, Tba[1], A0B0, -Tba[0], -Tab[0])) &&
            ((LB0uy < 0) ||
             voronoi_ok(a[0], b[0], -A1B0, -Tab[1], A0B0, Tab[0], Tba[0]))) {
            seg_closest(&t, &u, a[0], b[0], A0B0, Tab[0], Tba[0]);
            P[0] = t; P[1] = 0; P[2] = 0;
            Q[0] = Tab[0] + Rab[0][0] * u;
            Q[1] = Tab[1] + Rab[1][0] * u;
            Q[2] = Tab[2] + Rab[2][0] * u;
            return finish(P, Q, S);
        }
    }

    /* no edge pair holds the closest points: separation along the face normals */
    if (Tab[2] > 0.0) {
        sep1 = Tab[2];
        if (Rab[2][0] < 0.0) sep1 += b[0] * Rab[2][0];
        if (Rab[2][1] < 0.0) sep1 += b[1] * Rab[2][1];
    } else {
        sep1 = -Tab[2];
        if (Rab[2][0] > 0.0) sep1 -= b[0] * Rab[2][0];
        if (Rab[2][1] > 0.0) sep1 -= b[1] * Rab[2][1];
    }
    if (Tba[2] < 0) {
        sep2 = -Tba[2];
        if (Rab[0][2] < 0.0) sep2 += a[0] * Rab[0][2];
        if (Rab[1][2] < 0.0) sep2 += a[1] * Rab[1][2];
    } else {
        sep2 = Tba[2];
        if (Rab[0][2] > 0.0) sep2 -= a[0] * Rab[0][2];
        if (Rab[1][2] > 0.0) sep2 -= a[1] * Rab[1][2];
    }
    if (sep1 >= sep2 && sep1 >= 0) {
        P[0] = 0.0; P[1] = 0.0; P[2] = 0.0;
        Q[0] = 0.0; Q[1] = 0.0;
        Q[2] = (Tab[2] > 0.0) ? sep1 : -sep1;
        S[0] = Q[0] - P[0]; S[1] = Q[1] - P[1]; S[2] = Q[2] - P[2];
    }
    if (sep2 >= sep1 && sep2 >= 0) {
        Q[0] = Tab[0]; Q[1] = Tab[1]; Q[2] = Tab[2];
        if (Tba[2] < 0) {
            P[0] = Rab[0][2] * sep2 + Tab[0];
            P[1] = Rab[1][2] * sep2 + Tab[1];
            P[2] = Rab[2][2] * sep2 + Tab[2];
        } else {
            P[0] = -Rab[0][2] * sep2 + Tab[0];
            P[1] = -Rab[1][2] * sep2 + Tab[1];
            P[2] = -Rab[2][2] * sep2 + Tab[2];
        }
        S[0] = Q[0] - P[0]; S[1] = Q[1] - P[1]; S[2] = Q[2] - P[2];
    }
    sep = (sep1 > sep2 ? sep1 : sep2);
    return (sep > 0 ? sep : 0);
}

/* -------------------------------------------------------------- TriDist */

/* closest points X, Y of segments P+A*[0,1], Q+B*[0,1] and a separating
 * direction VEC (C2A.cpp:59-163) */
static void seg_seg(double VEC[3], double X[3], double Y[3], const double P[3], const double A[3],
                    const double Q[3], const double B[3])
{
    double T[3], AA, BB, AB, AT, BT, TMP[3], t, u, denom;
    pv_sub(T, Q, P);
    AA = pv_dot(A, A);
    BB = pv_dot(B, B);
    AB = pv_dot(A, B);
    AT = pv_dot(A, T);
    BT = pv_dot(B, T);
    denom = AA * BB - AB * AB;
    t = (AT * BB - BT * AB) / denom;
    if ((t < 0) || isnan(t)) t = 0;
    else if (t > 1) t = 1;
    u = (t * AB - BT) / BB;
    if ((u <= 0) || isnan(u)) {
        pv_copy(Y, Q);
        t = AT / AA;
        if ((t <= 0) || isnan(t)) {
            pv_copy(X, P);
            pv_sub(VEC, Q, P);
        } else if (t >= 1) {
            pv_add(X, P, A);
            pv_sub(VEC, Q, X);
        } else {
            pv_add_scaled(X, P, A, t);
            pv_cross(TMP, T, A);
            pv_cross(VEC, A, TMP);
        }
    } else if (u >= 1) {
        pv_add(Y, Q, B);
        t = (AB + AT) / AA;
        if ((t <= 0) || isnan(t)) {
            pv_copy(X, P);
            pv_sub(VEC, Y, P);
        } else if (t >= 1) {
            pv_add(X, P, A);
            pv_sub(VEC, Y, X);
        } else {
            pv_add_scaled(X, P, A, t);
            pv_sub(T, Y, P);
            pv_cross(TMP, T, A);
            pv_cross(VEC, A, TMP);
        }
    } else {
        pv_add_scaled(Y, Q, B, u);
        if ((t <= 0) || isnan(t)) {
            pv_copy(X, P);
            pv_cross(TMP, T, B);
            pv_cross(VEC, B, TMP);
        } else if (t >= 1) {
            pv_add(X, P, A);
            pv_sub(T, Q, X);
            pv_cross(TMP, T, B);
            pv_cross(VEC, B, TMP);
        } else {
            pv_add_scaled(X, P, A, t);
            pv_cross(VEC, A, B);
            if (pv_dot(VEC, T) < 0) pv_scale(VEC, VEC, -1);
        }
    }
}

/* vertex-face test of one triangle's face against the other's vertices
 * (C2A.cpp:268-332 and 335-386, the two mirrored halves).  Returns the vertex
 * index found inside the face, or -1; *disjoint set when the face normal
 * separates. */
static int vertex_face(const double S[3][3], const double Sv[3][3], const double T[3][3],
                       double *Tp_out, double *Snl_out, double Sn_out[3], int *disjoint)
{
    double Sn[3], Snl, Tp[3], V[3], Z[3];
    int point = -1;
    pv_cross(Sn, Sv[0], Sv[1]);
    Snl = pv_dot(Sn, Sn);
    if (!(Snl > 1e-15)) return -1;
    pv_sub(V, S[0], T[0]);
    Tp[0] = pv_dot(V, Sn);
    pv_sub(V, S[0], T[1]);
    Tp[1] = pv_dot(V, Sn);
    pv_sub(V, S[0], T[2]);
    Tp[2] = pv_dot(V, Sn);
    if ((Tp[0] > 0) && (Tp[1] > 0) && (Tp[2] > 0)) {
        if (Tp[0] < Tp[1]) point = 0; else point = 1;
        if (Tp[2] < Tp[point]) point = 2;
    } else if ((Tp[0] < 0) && (Tp[1] < 0) && (Tp[2] < 0)) {
        if (Tp[0] > Tp[1]) point = 0; else point = 1;
        if (Tp[2] > Tp[point]) point = 2;
    }
    if (point < 0) return -1;
    *disjoint = 1;
    pv_sub(V, T[point], S[0]);
    pv_cross(Z, Sn, Sv[0]);
    if (!(pv_dot(V, Z) > 0)) return -1;
    pv_sub(V, T[point], S[1]);
    pv_cross(Z, Sn, Sv[1]);
    if (!(pv_dot(V, Z) > 0)) return -1;
    pv_sub(V, T[point], S[2]);
    pv_cross(Z, Sn, Sv[2]);
    if (!(pv_dot(V, Z) > 0)) return -1;
    *Tp_out = Tp[point];
    *Snl_out = Snl;
    pv_copy(Sn_out, Sn);
    return point;
}

double c2a_port_tridist(double P[3], double Q[3], const double S9[9], const double T9[9], int *f1_type,
                        int *f1_fid, int *f2_type, int *f2_fid, int *collided)
{
    double S[3][3], T[3][3], Sv[3][3], Tv[3][3], VEC[3], V[3], Z[3], mindd;
    double minP[3] = {0.0, 0.0, 0.0}, minQ[3] = {0.0, 0.0, 0.0}; /* set by the first edge pair unless inputs are NaN */
    int shown_disjoint = 0, i, j, point;
    double tp, nl, n[3];

    pm_from9(S, S9);
    pm_from9(T, T9);
    pv_sub(Sv[0], S[1], S[0]);
    pv_sub(Sv[1], S[2], S[1]);
    pv_sub(Sv[2], S[0], S[2]);
    pv_sub(Tv[0], T[1], T[0]);
    pv_sub(Tv[1], T[2], T[1]);
    pv_sub(Tv[2], T[0], T[2]);

    /* the 9 edge pairs; a pair whose slab holds both off-edge vertices wins */
    mindd = pv_dist2(S[0], T[0]) + 1;
    for (i = 0; i < 3; i++) {
        for (j = 0; j < 3; j++) {
            double dd, a, b, p;
            seg_seg(VEC, P, Q, S[i], Sv[i], T[j], Tv[j]);
            pv_sub(V, Q, P);
            dd = pv_dot(V, V);
            if (dd <= mindd) {
                pv_copy(minP, P);
                pv_copy(minQ, Q);
                mindd = dd;
                *f1_type = 1; f1_fid[0] = i;
                *f2_type = 1; f2_fid[0] = j;
                pv_sub(Z, S[(i + 2) % 3], P);
                a = pv_dot(Z, VEC);
                pv_sub(Z, T[(j + 2) % 3], Q);
                b = pv_dot(Z, VEC);
                if ((a <= 0) && (b >= 0)) return sqrt(dd);
                p = pv_dot(V, VEC);
                if (a < 0) a = 0;
                if (b > 0) b = 0;
                if ((p - a + b) > 0) shown_disjoint = 1;
            }
        }
    }

    /* a vertex of T over the face of S */
    point = vertex_face((const double(*)[3])S, (const double(*)[3])Sv, (const double(*)[3])T, &tp, &nl, n,
                        &shown_disjoint);
    if (point >= 0) {
        *f1_type = 2; f1_fid[0] = -1;
        *f2_type = 0; f2_fid[0] = point;
        pv_add_scaled(P, T[point], n, tp / nl);
        pv_copy(Q, T[point]);
        return sqrt(pv_dist2(P, Q));
    }
    /* a vertex of S over the face of T */
    point = vertex_face((const double(*)[3])T, (const double(*)[3])Tv, (const double(*)[3])S, &tp, &nl, n,
                        &shown_disjoint);
    if (point >= 0) {
        *f1_type = 0; f1_fid[0] = point;
        *f2_type = 2; f2_fid[0] = -1;
        pv_copy(P, S[point]);
        pv_add_scaled(Q, S[point], n, tp / nl);
        return sqrt(pv_dist2(P, Q));
    }

    if (shown_disjoint) {
        pv_copy(P, minP);
        pv_copy(Q, minQ);
        return sqrt(mindd);
    }
    *collided = 1;
    return 0;
}
