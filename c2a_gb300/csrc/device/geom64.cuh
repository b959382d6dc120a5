/*
 * geom64.cuh -- FP64 device geometry of the CA step.
 *
 *   rect_dist      C2ARectDist (C2A/C2A_RectDist.h:157-934): distance of two
 *                  RSS rectangles and the direction S between the closest
 *                  points, in the first rectangle's frame
 *   bv_distance    C2A_BV_Distance (C2A/src/C2A_BV.cpp:666-675): minus r1+r2, >= 0
 *   tri_dist       TriDist with contact features (C2A/src/C2A.cpp:59-405)
 *   bound_leaf     CInterpMotion_Linear::computeTOC(d, r, S)
 *                  (C2A/src/InterpMotion.cpp:746-828)
 *   bound_rss      CInterpMotion_Linear::computeTOC_MotionBound
 *                  (InterpMotion.cpp:831-881)
 *
 * Compiled with --fmad=false so that every product and sum rounds on its own,
 * in the reference's left-to-right order: results are bit-identical to the
 * reference's double-precision code.
 */
#ifndef C2A_GEOM64_CUH
#define C2A_GEOM64_CUH

#include "../common/c2a_motion.h"

namespace c2a {

#define C2A_DEV __device__ __forceinline__

struct V3 {
    double x, y, z;
};

C2A_DEV V3 v3(double x, double y, double z) { return V3{x, y, z}; }
C2A_DEV V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
C2A_DEV V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
C2A_DEV V3 mul_s(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); } /* a * s, per component */
C2A_DEV V3 add_mul(V3 a, V3 b, double s) { return v3(a.x + b.x * s, a.y + b.y * s, a.z + b.z * s); }
C2A_DEV double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
C2A_DEV V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
C2A_DEV double dist2(V3 a, V3 b)
{
    return (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z);
}
C2A_DEV V3 normalized(V3 a)
{
    double d = 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return v3(a.x * d, a.y * d, a.z * d);
}
C2A_DEV double length(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

/* row-major 3x3 */
struct M3 {
    double m[9];
};
C2A_DEV V3 mul(const M3 &R, V3 p) /* R p */
{
    return v3(R.m[0] * p.x + R.m[1] * p.y + R.m[2] * p.z, R.m[3] * p.x + R.m[4] * p.y + R.m[5] * p.z,
              R.m[6] * p.x + R.m[7] * p.y + R.m[8] * p.z);
}
C2A_DEV V3 mul_add(const M3 &R, V3 p, V3 t) /* R p + t */
{
    return v3(R.m[0] * p.x + R.m[1] * p.y + R.m[2] * p.z + t.x, R.m[3] * p.x + R.m[4] * p.y + R.m[5] * p.z + t.y,
              R.m[6] * p.x + R.m[7] * p.y + R.m[8] * p.z + t.z);
}
C2A_DEV V3 tmul(const M3 &R, V3 p) /* R^T p */
{
    return v3(R.m[0] * p.x + R.m[3] * p.y + R.m[6] * p.z, R.m[1] * p.x + R.m[4] * p.y + R.m[7] * p.z,
              R.m[2] * p.x + R.m[5] * p.y + R.m[8] * p.z);
}
C2A_DEV M3 mmul(const M3 &A, const M3 &B) /* A B */
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = A.m[3 * i] * B.m[j] + A.m[3 * i + 1] * B.m[3 + j] + A.m[3 * i + 2] * B.m[6 + j];
    return r;
}
C2A_DEV M3 tmmul(const M3 &A, const M3 &B) /* A^T B */
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = A.m[i] * B.m[j] + A.m[3 + i] * B.m[3 + j] + A.m[6 + i] * B.m[6 + j];
    return r;
}

/* ------------------------------------------------------------- RectDist */

C2A_DEV double clamp_ab(double v, double lo, double hi)
{
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}

/* parameters of the closest points of two rectangle edges (RectDist.h:81-111) */
C2A_DEV void edge_params(double &t, double &u, double a, double b, double AdB, double AdT, double BdT)
{
    double denom = 1 - (AdB) * (AdB);
    if (denom == 0) t = 0;
    else t = clamp_ab((AdT - BdT * AdB) / denom, 0, a);
    u = t * AdB - BdT;
    if (u < 0) {
        u = 0;
        t = clamp_ab(AdT, 0, a);
    } else if (u > b) {
        u = b;
        t = clamp_ab(u * AdB + AdT, 0, a);
    }
}

/* closest point of edge B inside edge A's Voronoi slab (RectDist.h:123-154) */
C2A_DEV bool in_slab(double a, double b, double AnB, double AnT, double AdB, double AdT, double BdT)
{
    if ((AnB < 0 ? -AnB : AnB) < 1e-7) return false;
    double u = clamp_ab(-AnT / AnB, 0, b);
    double t = clamp_ab(u * AdB + AdT, 0, a);
    double v = t * AdB - BdT;
    if (AnB > 0) return v > (u + 1e-7);
    return v < (u - 1e-7);
}

/* Q = Tab + Rab[:,cb] * qb + Rab[:,cu] * u, evaluated as (Tab + Rq) + Ru */
C2A_DEV V3 rect_point2(const M3 &R, V3 T, int cb, double qb, int cu, double u)
{
    return v3(T.x + R.m[cb] * qb + R.m[cu] * u, T.y + R.m[3 + cb] * qb + R.m[3 + cu] * u,
              T.z + R.m[6 + cb] * qb + R.m[6 + cu] * u);
}
C2A_DEV V3 rect_point1(const M3 &R, V3 T, int cu, double u)
{
    return v3(T.x + R.m[cu] * u, T.y + R.m[3 + cu] * u, T.z + R.m[6 + cu] * u);
}

/*
 * Distance between rectangle A = [0,a0]x[0,a1] and B = Tab + Rab [0,b0]x[0,b1]
 * (B in A's frame).  S receives Q - P of the closest points; it is left
 * untouched only when the result is 0 through the face-separation fallback,
 * exactly like the reference.
 */
C2A_DEV double rect_dist(const M3 &Rab, V3 Tab, const double a[2], const double b[2], V3 &S)
{
    const double A0B0 = Rab.m[0], A0B1 = Rab.m[1], A1B0 = Rab.m[3], A1B1 = Rab.m[4];
    const double aA0B0 = a[0] * A0B0, aA0B1 = a[0] * A0B1, aA1B0 = a[1] * A1B0, aA1B1 = a[1] * A1B1;
    const double bA0B0 = b[0] * A0B0, bA1B0 = b[0] * A1B0, bA0B1 = b[1] * A0B1, bA1B1 = b[1] * A1B1;
    const V3 Tba = tmul(Rab, Tab);
    double t, u;
    V3 P, Q;

    const double ALLx = -Tba.x, ALUx = ALLx + aA1B0, AULx = ALLx + aA0B0, AUUx = ALUx + aA0B0;
    double LA1lx, LA1ux, UA1lx, UA1ux, LB1lx, LB1ux, UB1lx, UB1ux;
    if (ALLx < ALUx) { LA1lx = ALLx; LA1ux = ALUx; UA1lx = AULx; UA1ux = AUUx; }
    else { LA1lx = ALUx; LA1ux = ALLx; UA1lx = AUUx; UA1ux = AULx; }
    const double BLLx = Tab.x, BLUx = BLLx + bA0B1, BULx = BLLx + bA0B0, BUUx = BLUx + bA0B0;
    if (BLLx < BLUx) { LB1lx = BLLx; LB1ux = BLUx; UB1lx = BULx; UB1ux = BUUx; }
    else { LB1lx = BLUx; LB1ux = BLLx; UB1lx = BUUx; UB1ux = BULx; }

#define C2A_EDGE_HIT(PX, PY, QEXPR)                                                                                \
    do {                                                                                                           \
        P = v3((PX), (PY), 0);                                                                                     \
        Q = (QEXPR);                                                                                               \
        S = v3(Q.x - P.x, Q.y - P.y, Q.z - P.z);                                                                   \
        return sqrt(dot(S, S));                                                                                    \
    } while (0)

    /* A edges along A1 against B edges along B1 */
    if ((UA1ux > b[0]) && (UB1ux > a[0]) &&
        ((UA1lx > b[0]) || in_slab(b[1], a[1], A1B0, aA0B0 - b[0] - Tba.x, A1B1, aA0B1 - Tba.y, -Tab.y - bA1B0)) &&
        ((UB1lx > a[0]) || in_slab(a[1], b[1], A0B1, Tab.x + bA0B0 - a[0], A1B1, Tab.y + bA1B0, Tba.y - aA0B1))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y + bA1B0, Tba.y - aA0B1);
        C2A_EDGE_HIT(a[0], t, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if ((UA1lx < 0) && (LB1ux > a[0]) &&
        ((UA1ux < 0) || in_slab(b[1], a[1], -A1B0, Tba.x - aA0B0, A1B1, aA0B1 - Tba.y, -Tab.y)) &&
        ((LB1lx > a[0]) || in_slab(a[1], b[1], A0B1, Tab.x - a[0], A1B1, Tab.y, Tba.y - aA0B1))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y, Tba.y - aA0B1);
        C2A_EDGE_HIT(a[0], t, rect_point1(Rab, Tab, 1, u));
    }
    if ((LA1ux > b[0]) && (UB1lx < 0) &&
        ((LA1lx > b[0]) || in_slab(b[1], a[1], A1B0, -Tba.x - b[0], A1B1, -Tba.y, -Tab.y - bA1B0)) &&
        ((UB1ux < 0) || in_slab(a[1], b[1], -A0B1, -Tab.x - bA0B0, A1B1, Tab.y + bA1B0, Tba.y))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y + bA1B0, Tba.y);
        C2A_EDGE_HIT(0, t, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if ((LA1lx < 0) && (LB1lx < 0) &&
        ((LA1ux < 0) || in_slab(b[1], a[1], -A1B0, Tba.x, A1B1, -Tba.y, -Tab.y)) &&
        ((LB1ux < 0) || in_slab(a[1], b[1], -A0B1, -Tab.x, A1B1, Tab.y, Tba.y))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y, Tba.y);
        C2A_EDGE_HIT(0, t, rect_point1(Rab, Tab, 1, u));
    }

    const double ALLy = -Tba.y, ALUy = ALLy + aA1B1, AULy = ALLy + aA0B1, AUUy = ALUy + aA0B1;
    double LA1ly, LA1uy, UA1ly, UA1uy, LB0lx, LB0ux, UB0lx, UB0ux;
    if (ALLy < ALUy) { LA1ly = ALLy; LA1uy = ALUy; UA1ly = AULy; UA1uy = AUUy; }
    else { LA1ly = ALUy; LA1uy = ALLy; UA1ly = AUUy; UA1uy = AULy; }
    if (BLLx < BULx) { LB0lx = BLLx; LB0ux = BULx; UB0lx = BLUx; UB0ux = BUUx; }
    else { LB0lx = BULx; LB0ux = BLLx; UB0lx = BUUx; UB0ux = BLUx; }

    /* A edges along A1 against B edges along B0 */
    if ((UA1uy > b[1]) && (UB0ux > a[0]) &&
        ((UA1ly > b[1]) || in_slab(b[0], a[1], A1B1, aA0B1 - Tba.y - b[1], A1B0, aA0B0 - Tba.x, -Tab.y - bA1B1)) &&
        ((UB0lx > a[0]) || in_slab(a[1], b[0], A0B0, Tab.x - a[0] + bA0B1, A1B0, Tab.y + bA1B1, Tba.x - aA0B0))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y + bA1B1, Tba.x - aA0B0);
        C2A_EDGE_HIT(a[0], t, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if ((UA1ly < 0) && (LB0ux > a[0]) &&
        ((UA1uy < 0) || in_slab(b[0], a[1], -A1B1, Tba.y - aA0B1, A1B0, aA0B0 - Tba.x, -Tab.y)) &&
        ((LB0lx > a[0]) || in_slab(a[1], b[0], A0B0, Tab.x - a[0], A1B0, Tab.y, Tba.x - aA0B0))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y, Tba.x - aA0B0);
        C2A_EDGE_HIT(a[0], t, rect_point1(Rab, Tab, 0, u));
    }
    if ((LA1uy > b[1]) && (UB0lx < 0) &&
        ((LA1ly > b[1]) || in_slab(b[0], a[1], A1B1, -Tba.y - b[1], A1B0, -Tba.x, -Tab.y - bA1B1)) &&
        ((UB0ux < 0) || in_slab(a[1], b[0], -A0B0, -Tab.x - bA0B1, A1B0, Tab.y + bA1B1, Tba.x))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y + bA1B1, Tba.x);
        C2A_EDGE_HIT(0, t, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if ((LA1ly < 0) && (LB0lx < 0) &&
        ((LA1uy < 0) || in_slab(b[0], a[1], -A1B1, Tba.y, A1B0, -Tba.x, -Tab.y)) &&
        ((LB0ux < 0) || in_slab(a[1], b[0], -A0B0, -Tab.x, A1B0, Tab.y, Tba.x))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y, Tba.x);
        C2A_EDGE_HIT(0, t, rect_point1(Rab, Tab, 0, u));
    }

    const double BLLy = Tab.y, BLUy = BLLy + bA1B1, BULy = BLLy + bA1B0, BUUy = BLUy + bA1B0;
    double LA0lx, LA0ux, UA0lx, UA0ux, LB1ly, LB1uy, UB1ly, UB1uy;
    if (ALLx < AULx) { LA0lx = ALLx; LA0ux = AULx; UA0lx = ALUx; UA0ux = AUUx; }
    else { LA0lx = AULx; LA0ux = ALLx; UA0lx = AUUx; UA0ux = ALUx; }
    if (BLLy < BLUy) { LB1ly = BLLy; LB1uy = BLUy; UB1ly = BULy; UB1uy = BUUy; }
    else { LB1ly = BLUy; LB1uy = BLLy; UB1ly = BUUy; UB1uy = BULy; }

    /* A edges along A0 against B edges along B1 */
    if ((UA0ux > b[0]) && (UB1uy > a[1]) &&
        ((UA0lx > b[0]) || in_slab(b[1], a[0], A0B0, aA1B0 - Tba.x - b[0], A0B1, aA1B1 - Tba.y, -Tab.x - bA0B0)) &&
        ((UB1ly > a[1]) || in_slab(a[0], b[1], A1B1, Tab.y - a[1] + bA1B0, A0B1, Tab.x + bA0B0, Tba.y - aA1B1))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x + bA0B0, Tba.y - aA1B1);
        C2A_EDGE_HIT(t, a[1], rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if ((UA0lx < 0) && (LB1uy > a[1]) &&
        ((UA0ux < 0) || in_slab(b[1], a[0], -A0B0, Tba.x - aA1B0, A0B1, aA1B1 - Tba.y, -Tab.x)) &&
        ((LB1ly > a[1]) || in_slab(a[0], b[1], A1B1, Tab.y - a[1], A0B1, Tab.x, Tba.y - aA1B1))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x, Tba.y - aA1B1);
        C2A_EDGE_HIT(t, a[1], rect_point1(Rab, Tab, 1, u));
    }
    if ((LA0ux > b[0]) && (UB1ly < 0) &&
        ((LA0lx > b[0]) || in_slab(b[1], a[0], A0B0, -b[0] - Tba.x, A0B1, -Tba.y, -bA0B0 - Tab.x)) &&
        ((UB1uy < 0) || in_slab(a[0], b[1], -A1B1, -Tab.y - bA1B0, A0B1, Tab.x + bA0B0, Tba.y))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x + bA0B0, Tba.y);
        C2A_EDGE_HIT(t, 0, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if ((LA0lx < 0) && (LB1ly < 0) &&
        ((LA0ux < 0) || in_slab(b[1], a[0], -A0B0, Tba.x, A0B1, -Tba.y, -Tab.x)) &&
        ((LB1uy < 0) || in_slab(a[0], b[1], -A1B1, -Tab.y, A0B1, Tab.x, Tba.y))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x, Tba.y);
        C2A_EDGE_HIT(t, 0, rect_point1(Rab, Tab, 1, u));
    }

    double LA0ly, LA0uy, UA0ly, UA0uy, LB0ly, LB0uy, UB0ly, UB0uy;
    if (ALLy < AULy) { LA0ly = ALLy; LA0uy = AULy; UA0ly = ALUy; UA0uy = AUUy; }
    else { LA0ly = AULy; LA0uy = ALLy; UA0ly = AUUy; UA0uy = ALUy; }
    if (BLLy < BULy) { LB0ly = BLLy; LB0uy = BULy; UB0ly = BLUy; UB0uy = BUUy; }
    else { LB0ly = BULy; LB0uy = BLLy; UB0ly = BUUy; UB0uy = BLUy; }

    /* A edges along A0 against B edges along B0 */
    if ((UA0uy > b[1]) && (UB0uy > a[1]) &&
        ((UA0ly > b[1]) || in_slab(b[0], a[0], A0B1, aA1B1 - Tba.y - b[1], A0B0, aA1B0 - Tba.x, -Tab.x - bA0B1)) &&
        ((UB0ly > a[1]) || in_slab(a[0], b[0], A1B0, Tab.y - a[1] + bA1B1, A0B0, Tab.x + bA0B1, Tba.x - aA1B0))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x + bA0B1, Tba.x - aA1B0);
        C2A_EDGE_HIT(t, a[1], rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if ((UA0ly < 0) && (LB0uy > a[1]) &&
        ((UA0uy < 0) || in_slab(b[0], a[0], -A0B1, Tba.y - aA1B1, A0B0, aA1B0 - Tba.x, -Tab.x)) &&
        ((LB0ly > a[1]) || in_slab(a[0], b[0], A1B0, Tab.y - a[1], A0B0, Tab.x, Tba.x - aA1B0))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x, Tba.x - aA1B0);
        C2A_EDGE_HIT(t, a[1], rect_point1(Rab, Tab, 0, u));
    }
    if ((LA0uy > b[1]) && (UB0ly < 0) &&
        ((LA0ly > b[1]) || in_slab(b[0], a[0], A0B1, -Tba.y - b[1], A0B0, -Tba.x, -Tab.x - bA0B1)) &&
        ((UB0uy < 0) || in_slab(a[0], b[0], -A1B0, -Tab.y - bA1B1, A0B0, Tab.x + bA0B1, Tba.x))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x + bA0B1, Tba.x);
        C2A_EDGE_HIT(t, 0, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if ((LA0ly < 0) && (LB0ly < 0) &&
        ((LA0uy < 0) || in_slab(b[0], a[0], -A0B1, Tba.y, A0B0, -Tba.x, -Tab.x)) &&
        ((LB0uy < 0) || in_slab(a[0], b[0], -A1B0, -Tab.y, A0B0, Tab.x, Tba.x))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x, Tba.x);
        C2A_EDGE_HIT(t, 0, rect_point1(Rab, Tab, 0, u));
    }
#undef C2A_EDGE_HIT

    /* no edge pair: largest separation along the two face normals */
    double sep1, sep2;
    if (Tab.z > 0.0) {
        sep1 = Tab.z;
        if (Rab.m[6] < 0.0) sep1 += b[0] * Rab.m[6];
        if (Rab.m[7] < 0.0) sep1 += b[1] * Rab.m[7];
    } else {
        sep1 = -Tab.z;
        if (Rab.m[6] > 0.0) sep1 -= b[0] * Rab.m[6];
        if (Rab.m[7] > 0.0) sep1 -= b[1] * Rab.m[7];
    }
    if (Tba.z < 0) {
        sep2 = -Tba.z;
        if (Rab.m[2] < 0.0) sep2 += a[0] * Rab.m[2];
        if (Rab.m[5] < 0.0) sep2 += a[1] * Rab.m[5];
    } else {
        sep2 = Tba.z;
        if (Rab.m[2] > 0.0) sep2 -= a[0] * Rab.m[2];
        if (Rab.m[5] > 0.0) sep2 -= a[1] * Rab.m[5];
    }
    if (sep1 >= sep2 && sep1 >= 0) {
        const double qz = (Tab.z > 0.0) ? sep1 : -sep1;
        S = v3(0.0 - 0.0, 0.0 - 0.0, qz - 0.0);
    }
    if (sep2 >= sep1 && sep2 >= 0) {
        V3 Pp;
        if (Tba.z < 0) Pp = v3(Rab.m[2] * sep2 + Tab.x, Rab.m[5] * sep2 + Tab.y, Rab.m[8] * sep2 + Tab.z);
        else Pp = v3(-Rab.m[2] * sep2 + Tab.x, -Rab.m[5] * sep2 + Tab.y, -Rab.m[8] * sep2 + Tab.z);
        S = v3(Tab.x - Pp.x, Tab.y - Pp.y, Tab.z - Pp.z);
    }
    const double sep = (sep1 > sep2 ? sep1 : sep2);
    return (sep > 0 ? sep : 0);
}

/* ------------------------------------------------------------- TriDist */

/* closest points X, Y of segments P + A[0,1] and Q + B[0,1] and a direction
 * VEC separating them (C2A.cpp:59-163) */
C2A_DEV void seg_pair(V3 &VEC, V3 &X, V3 &Y, V3 P, V3 A, V3 Q, V3 B)
{
    V3 T = Q - P;
    const double AA = dot(A, A), BB = dot(B, B), AB = dot(A, B), AT = dot(A, T), BT = dot(B, T);
    const double denom = AA * BB - AB * AB;
    double t = (AT * BB - BT * AB) / denom;
    if ((t < 0) || isnan(t)) t = 0;
    else if (t > 1) t = 1;
    double u = (t * AB - BT) / BB;
    if ((u <= 0) || isnan(u)) {
        Y = Q;
        t = AT / AA;
        if ((t <= 0) || isnan(t)) {
            X = P;
            VEC = Q - P;
        } else if (t >= 1) {
            X = P + A;
            VEC = Q - X;
        } else {
            X = add_mul(P, A, t);
            VEC = cross(A, cross(T, A));
        }
    } else if (u >= 1) {
        Y = Q + B;
        t = (AB + AT) / AA;
        if ((t <= 0) || isnan(t)) {
            X = P;
            VEC = Y - P;
        } else if (t >= 1) {
            X = P + A;
            VEC = Y - X;
        } else {
            X = add_mul(P, A, t);
            T = Y - P;
            VEC = cross(A, cross(T, A));
        }
    } else {
        Y = add_mul(Q, B, u);
        if ((t <= 0) || isnan(t)) {
            X = P;
            VEC = cross(B, cross(T, B));
        } else if (t >= 1) {
            X = P + A;
            T = Q - X;
            VEC = cross(B, cross(T, B));
        } else {
            X = add_mul(P, A, t);
            VEC = cross(A, B);
            if (dot(VEC, T) < 0) VEC = mul_s(VEC, -1);
        }
    }
}

struct TriFeat {
    int type_a, fid_a, type_b, fid_b;
};

/*
 * Vertex of triangle T over the face of S?  Returns the vertex index (with
 * its projection Tp and the squared normal length) or -1; sets *disjoint when
 * S's normal separates (C2A.cpp:268-332; the mirrored half swaps S and T).
 */
C2A_DEV int vertex_over_face(const V3 S[3], const V3 Sv[3], const V3 T[3], double &tp, double &nl, V3 &n,
                             bool &disjoint)
{
    const V3 Sn = cross(Sv[0], Sv[1]);
    const double Snl = dot(Sn, Sn);
    if (!(Snl > 1e-15)) return -1;
    double Tp[3];
    Tp[0] = dot(S[0] - T[0], Sn);
    Tp[1] = dot(S[0] - T[1], Sn);
    Tp[2] = dot(S[0] - T[2], Sn);
    int point = -1;
    if ((Tp[0] > 0) && (Tp[1] > 0) && (Tp[2] > 0)) {
        point = (Tp[0] < Tp[1]) ? 0 : 1;
        if (Tp[2] < Tp[point]) point = 2;
    } else if ((Tp[0] < 0) && (Tp[1] < 0) && (Tp[2] < 0)) {
        point = (Tp[0] > Tp[1]) ? 0 : 1;
        if (Tp[2] > Tp[point]) point = 2;
    }
    if (point < 0) return -1;
    disjoint = true;
#pragma unroll
    for (int e = 0; e < 3; e++)
        if (!(dot(T[point] - S[e], cross(Sn, Sv[e])) > 0)) return -1;
    tp = Tp[point];
    nl = Snl;
    n = Sn;
    return point;
}

/* distance between triangles S and T (same frame), closest points P, Q,
 * features; collided set on overlap (C2A.cpp:165-405) */
C2A_DEV double tri_dist(V3 &P, V3 &Q, const V3 S[3], const V3 T[3], TriFeat &f, bool &collided)
{
    V3 Sv[3], Tv[3];
    Sv[0] = S[1] - S[0];
    Sv[1] = S[2] - S[1];
    Sv[2] = S[0] - S[2];
    Tv[0] = T[1] - T[0];
    Tv[1] = T[2] - T[1];
    Tv[2] = T[0] - T[2];
    V3 minP = v3(0, 0, 0), minQ = v3(0, 0, 0), VEC;
    double mindd = dist2(S[0], T[0]) + 1;
    bool shown_disjoint = false;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            seg_pair(VEC, P, Q, S[i], Sv[i], T[j], Tv[j]);
            const V3 V = Q - P;
            const double dd = dot(V, V);
            if (dd <= mindd) {
                minP = P;
                minQ = Q;
                mindd = dd;
                f.type_a = 1;
                f.fid_a = i;
                f.type_b = 1;
                f.fid_b = j;
                double a = dot(S[(i + 2) % 3] - P, VEC);
                double b = dot(T[(j + 2) % 3] - Q, VEC);
                if ((a <= 0) && (b >= 0)) return sqrt(dd);
                const double p = dot(V, VEC);
                if (a < 0) a = 0;
                if (b > 0) b = 0;
                if ((p - a + b) > 0) shown_disjoint = true;
            }
        }
    }
    double tp, nl;
    V3 n;
    int point = vertex_over_face(S, Sv, T, tp, nl, n, shown_disjoint);
    if (point >= 0) {
        f.type_a = 2;
        f.fid_a = -1;
        f.type_b = 0;
        f.fid_b = point;
        P = add_mul(T[point], n, tp / nl);
        Q = T[point];
        return sqrt(dist2(P, Q));
    }
    point = vertex_over_face(T, Tv, S, tp, nl, n, shown_disjoint);
    if (point >= 0) {
        f.type_a = 0;
        f.fid_a = point;
        f.type_b = 2;
        f.fid_b = -1;
        P = S[point];
        Q = add_mul(S[point], n, tp / nl);
        return sqrt(dist2(P, Q));
    }
    if (shown_disjoint) {
        P = minP;
        Q = minQ;
        return sqrt(mindd);
    }
    collided = true;
    return 0;
}

/* --------------------------------------------------------- motion bounds */

/* computeTOC(d, r1, S) at a leaf; S is normalised in place */
C2A_DEV double bound_leaf(const Motion &m, double r1, V3 &S)
{
    S = normalized(S);
    double w_max, v_max;
    if (m.angVel == 0) {
        w_max = 0;
        v_max = m.cv[0] * S.x + m.cv[1] * S.y + m.cv[2] * S.z;
        if (v_max < 0) v_max = 0;
    } else {
        const V3 cwc = v3(m.axis[0] * m.angVel, m.axis[1] * m.angVel, m.axis[2] * m.angVel);
        w_max = r1 * length(cross(cwc, S));
        v_max = m.cv[0] * S.x + m.cv[1] * S.y + m.cv[2] * S.z;
        if (v_max < 0) v_max = 0;
    }
    double path_max = w_max + v_max;
    if (path_max == 0) path_max = 1e-30;
    return path_max;
}

/* computeTOC_MotionBound for an RSS of angular radius angR; N normalised in place */
C2A_DEV double bound_rss(const Motion &m, double angR, V3 &N)
{
    N = normalized(N);
    const V3 c = cross(v3(m.axis[0], m.axis[1], m.axis[2]), N);
    const double w_max = angR * length(c) * m.angVel;
    double v_max = m.cv[0] * N.x + m.cv[1] * N.y + m.cv[2] * N.z;
    if (v_max < 0) v_max = 0;
    double path_max = v_max + w_max;
    if (path_max <= 0) path_max = 1e-30;
    return path_max;
}

} // namespace c2a
#endif
