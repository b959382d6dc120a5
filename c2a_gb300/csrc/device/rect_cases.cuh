/* generated by gen_rect_cases.py from rect_dist in geom.cuh; do not edit */
#ifndef C2A_RECT_CASES_CUH
#define C2A_RECT_CASES_CUH

#include "geom.cuh"

namespace c2a {

/* Kleene AND / OR over {1, 0, -1 (undecided)} */
C2A_DEV int rc_and3(int a, int b) { return (a == 0 || b == 0) ? 0 : (a == 1 && b == 1) ? 1 : -1; }
C2A_DEV int rc_or3(int a, int b) { return (a == 1 || b == 1) ? 1 : (a == 0 && b == 0) ? 0 : -1; }

/* case j (0..15) of C2ARectDist.  hit: 1 its condition holds, 0 it does not,
 * -1 undecided (the FP32 filter only; each part keeps its own context, so a
 * part the sequential form would not evaluate decides nothing); vbad: the
 * distance and S are not certified; ctx: the shared preamble's decisions.
 * The caller takes the first case that holds. */
template <class T, class C>
C2A_DEV T rect_case(int j, const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, int &hit,
                    bool &vbad, C &ctx)
{
    const T zero = K(0.0);
    const T A0B0 = Rab.m[0], A0B1 = Rab.m[1], A1B0 = Rab.m[3], A1B1 = Rab.m[4];
    const T aA0B0 = a[0] * A0B0, aA0B1 = a[0] * A0B1, aA1B0 = a[1] * A1B0, aA1B1 = a[1] * A1B1;
    const T bA0B0 = b[0] * A0B0, bA1B0 = b[0] * A1B0, bA0B1 = b[1] * A0B1, bA1B1 = b[1] * A1B1;
    const V3T<T> Tba = tmul(Rab, Tab);

    const T ALLx = -Tba.x, ALUx = ALLx + aA1B0, AULx = ALLx + aA0B0, AUUx = ALUx + aA0B0;
    T LA1lx, LA1ux, UA1lx, UA1ux, LB1lx, LB1ux, UB1lx, UB1ux;
    if (LT(ALLx, ALUx)) { LA1lx = ALLx; LA1ux = ALUx; UA1lx = AULx; UA1ux = AUUx; }
    else { LA1lx = ALUx; LA1ux = ALLx; UA1lx = AUUx; UA1ux = AULx; }
    const T BLLx = Tab.x, BLUx = BLLx + bA0B1, BULx = BLLx + bA0B0, BUUx = BLUx + bA0B0;
    if (LT(BLLx, BLUx)) { LB1lx = BLLx; LB1ux = BLUx; UB1lx = BULx; UB1ux = BUUx; }
    else { LB1lx = BLUx; LB1ux = BLLx; UB1lx = BUUx; UB1ux = BULx; }

    const T ALLy = -Tba.y, ALUy = ALLy + aA1B1, AULy = ALLy + aA0B1, AUUy = ALUy + aA0B1;
    T LA1ly, LA1uy, UA1ly, UA1uy, LB0lx, LB0ux, UB0lx, UB0ux;
    if (LT(ALLy, ALUy)) { LA1ly = ALLy; LA1uy = ALUy; UA1ly = AULy; UA1uy = AUUy; }
    else { LA1ly = ALUy; LA1uy = ALLy; UA1ly = AUUy; UA1uy = AULy; }
    if (LT(BLLx, BULx)) { LB0lx = BLLx; LB0ux = BULx; UB0lx = BLUx; UB0ux = BUUx; }
    else { LB0lx = BULx; LB0ux = BLLx; UB0lx = BUUx; UB0ux = BLUx; }

    const T BLLy = Tab.y, BLUy = BLLy + bA1B1, BULy = BLLy + bA1B0, BUUy = BLUy + bA1B0;
    T LA0lx, LA0ux, UA0lx, UA0ux, LB1ly, LB1uy, UB1ly, UB1uy;
    if (LT(ALLx, AULx)) { LA0lx = ALLx; LA0ux = AULx; UA0lx = ALUx; UA0ux = AUUx; }
    else { LA0lx = AULx; LA0ux = ALLx; UA0lx = AUUx; UA0ux = ALUx; }
    if (LT(BLLy, BLUy)) { LB1ly = BLLy; LB1uy = BLUy; UB1ly = BULy; UB1uy = BUUy; }
    else { LB1ly = BLUy; LB1uy = BLLy; UB1ly = BUUy; UB1uy = BULy; }

    T LA0ly, LA0uy, UA0ly, UA0uy, LB0ly, LB0uy, UB0ly, UB0uy;
    if (LT(ALLy, AULy)) { LA0ly = ALLy; LA0uy = AULy; UA0ly = ALUy; UA0uy = AUUy; }
    else { LA0ly = AULy; LA0uy = ALLy; UA0ly = AUUy; UA0uy = ALUy; }
    if (LT(BLLy, BULy)) { LB0ly = BLLy; LB0uy = BULy; UB0ly = BLUy; UB0uy = BUUy; }
    else { LB0ly = BULy; LB0uy = BLLy; UB0ly = BUUy; UB0uy = BLUy; }

    
    const T x0 = aA0B0 - b[0] - Tba.x;
    const T x1 = aA0B1 - Tba.y;
    const T x2 = -Tab.y - bA1B0;
    const T x3 = Tab.x + bA0B0 - a[0];
    const T x4 = Tab.y + bA1B0;
    const T x5 = Tba.y - aA0B1;
    const T x6 = -A1B0;
    const T x7 = Tba.x - aA0B0;
    const T x8 = -Tab.y;
    const T x9 = Tab.x - a[0];
    const T x10 = -Tba.x - b[0];
    const T x11 = -Tba.y;
    const T x12 = -A0B1;
    const T x13 = -Tab.x - bA0B0;
    const T x14 = -Tab.x;
    const T x15 = aA0B1 - Tba.y - b[1];
    const T x16 = aA0B0 - Tba.x;
    const T x17 = -Tab.y - bA1B1;
    const T x18 = Tab.x - a[0] + bA0B1;
    const T x19 = Tab.y + bA1B1;
    const T x20 = -A1B1;
    const T x21 = -Tba.y - b[1];
    const T x22 = -Tba.x;
    const T x23 = -A0B0;
    const T x24 = -Tab.x - bA0B1;
    const T x25 = aA1B0 - Tba.x - b[0];
    const T x26 = aA1B1 - Tba.y;
    const T x27 = Tab.y - a[1] + bA1B0;
    const T x28 = Tab.x + bA0B0;
    const T x29 = Tba.y - aA1B1;
    const T x30 = Tba.x - aA1B0;
    const T x31 = Tab.y - a[1];
    const T x32 = -b[0] - Tba.x;
    const T x33 = -bA0B0 - Tab.x;
    const T x34 = aA1B1 - Tba.y - b[1];
    const T x35 = aA1B0 - Tba.x;
    const T x36 = Tab.y - a[1] + bA1B1;
    const T x37 = Tab.x + bA0B1;
    T L[4], R[4], s1[7], s2[7], e[5], qb = zero;
    int px = 0, py = 0, qkind = 1, cb = 0, cu = 0;
    switch (j) {
    case 0:
        L[0] = b[0]; R[0] = UA1ux;
        L[1] = a[0]; R[1] = UB1ux;
        L[2] = b[0]; R[2] = UA1lx;
        L[3] = a[0]; R[3] = UB1lx;
        s1[0] = b[1]; s1[1] = a[1]; s1[2] = A1B0; s1[3] = x0; s1[4] = A1B1; s1[5] = x1; s1[6] = x2;
        s2[0] = a[1]; s2[1] = b[1]; s2[2] = A0B1; s2[3] = x3; s2[4] = A1B1; s2[5] = x4; s2[6] = x5;
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = x4; e[4] = x5;
        px = 0; py = 4; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 1:
        L[0] = UA1lx; R[0] = zero;
        L[1] = a[0]; R[1] = LB1ux;
        L[2] = UA1ux; R[2] = zero;
        L[3] = a[0]; R[3] = LB1lx;
        s1[0] = b[1]; s1[1] = a[1]; s1[2] = x6; s1[3] = x7; s1[4] = A1B1; s1[5] = x1; s1[6] = x8;
        s2[0] = a[1]; s2[1] = b[1]; s2[2] = A0B1; s2[3] = x9; s2[4] = A1B1; s2[5] = Tab.y; s2[6] = x5;
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = Tab.y; e[4] = x5;
        px = 0; py = 4; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 2:
        L[0] = b[0]; R[0] = LA1ux;
        L[1] = UB1lx; R[1] = zero;
        L[2] = b[0]; R[2] = LA1lx;
        L[3] = UB1ux; R[3] = zero;
        s1[0] = b[1]; s1[1] = a[1]; s1[2] = A1B0; s1[3] = x10; s1[4] = A1B1; s1[5] = x11; s1[6] = x2;
        s2[0] = a[1]; s2[1] = b[1]; s2[2] = x12; s2[3] = x13; s2[4] = A1B1; s2[5] = x4; s2[6] = Tba.y;
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = x4; e[4] = Tba.y;
        px = 2; py = 4; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 3:
        L[0] = LA1lx; R[0] = zero;
        L[1] = LB1lx; R[1] = zero;
        L[2] = LA1ux; R[2] = zero;
        L[3] = LB1ux; R[3] = zero;
        s1[0] = b[1]; s1[1] = a[1]; s1[2] = x6; s1[3] = Tba.x; s1[4] = A1B1; s1[5] = x11; s1[6] = x8;
        s2[0] = a[1]; s2[1] = b[1]; s2[2] = x12; s2[3] = x14; s2[4] = A1B1; s2[5] = Tab.y; s2[6] = Tba.y;
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = Tab.y; e[4] = Tba.y;
        px = 2; py = 4; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 4:
        L[0] = b[1]; R[0] = UA1uy;
        L[1] = a[0]; R[1] = UB0ux;
        L[2] = b[1]; R[2] = UA1ly;
        L[3] = a[0]; R[3] = UB0lx;
        s1[0] = b[0]; s1[1] = a[1]; s1[2] = A1B1; s1[3] = x15; s1[4] = A1B0; s1[5] = x16; s1[6] = x17;
        s2[0] = a[1]; s2[1] = b[0]; s2[2] = A0B0; s2[3] = x18; s2[4] = A1B0; s2[5] = x19; s2[6] = x7;
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = x19; e[4] = x7;
        px = 0; py = 4; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 5:
        L[0] = UA1ly; R[0] = zero;
        L[1] = a[0]; R[1] = LB0ux;
        L[2] = UA1uy; R[2] = zero;
        L[3] = a[0]; R[3] = LB0lx;
        s1[0] = b[0]; s1[1] = a[1]; s1[2] = x20; s1[3] = x5; s1[4] = A1B0; s1[5] = x16; s1[6] = x8;
        s2[0] = a[1]; s2[1] = b[0]; s2[2] = A0B0; s2[3] = x9; s2[4] = A1B0; s2[5] = Tab.y; s2[6] = x7;
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = Tab.y; e[4] = x7;
        px = 0; py = 4; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 6:
        L[0] = b[1]; R[0] = LA1uy;
        L[1] = UB0lx; R[1] = zero;
        L[2] = b[1]; R[2] = LA1ly;
        L[3] = UB0ux; R[3] = zero;
        s1[0] = b[0]; s1[1] = a[1]; s1[2] = A1B1; s1[3] = x21; s1[4] = A1B0; s1[5] = x22; s1[6] = x17;
        s2[0] = a[1]; s2[1] = b[0]; s2[2] = x23; s2[3] = x24; s2[4] = A1B0; s2[5] = x19; s2[6] = Tba.x;
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = x19; e[4] = Tba.x;
        px = 2; py = 4; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 7:
        L[0] = LA1ly; R[0] = zero;
        L[1] = LB0lx; R[1] = zero;
        L[2] = LA1uy; R[2] = zero;
        L[3] = LB0ux; R[3] = zero;
        s1[0] = b[0]; s1[1] = a[1]; s1[2] = x20; s1[3] = Tba.y; s1[4] = A1B0; s1[5] = x22; s1[6] = x8;
        s2[0] = a[1]; s2[1] = b[0]; s2[2] = x23; s2[3] = x14; s2[4] = A1B0; s2[5] = Tab.y; s2[6] = Tba.x;
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = Tab.y; e[4] = Tba.x;
        px = 2; py = 4; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 8:
        L[0] = b[0]; R[0] = UA0ux;
        L[1] = a[1]; R[1] = UB1uy;
        L[2] = b[0]; R[2] = UA0lx;
        L[3] = a[1]; R[3] = UB1ly;
        s1[0] = b[1]; s1[1] = a[0]; s1[2] = A0B0; s1[3] = x25; s1[4] = A0B1; s1[5] = x26; s1[6] = x13;
        s2[0] = a[0]; s2[1] = b[1]; s2[2] = A1B1; s2[3] = x27; s2[4] = A0B1; s2[5] = x28; s2[6] = x29;
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = x28; e[4] = x29;
        px = 4; py = 1; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 9:
        L[0] = UA0lx; R[0] = zero;
        L[1] = a[1]; R[1] = LB1uy;
        L[2] = UA0ux; R[2] = zero;
        L[3] = a[1]; R[3] = LB1ly;
        s1[0] = b[1]; s1[1] = a[0]; s1[2] = x23; s1[3] = x30; s1[4] = A0B1; s1[5] = x26; s1[6] = x14;
        s2[0] = a[0]; s2[1] = b[1]; s2[2] = A1B1; s2[3] = x31; s2[4] = A0B1; s2[5] = Tab.x; s2[6] = x29;
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = Tab.x; e[4] = x29;
        px = 4; py = 1; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 10:
        L[0] = b[0]; R[0] = LA0ux;
        L[1] = UB1ly; R[1] = zero;
        L[2] = b[0]; R[2] = LA0lx;
        L[3] = UB1uy; R[3] = zero;
        s1[0] = b[1]; s1[1] = a[0]; s1[2] = A0B0; s1[3] = x32; s1[4] = A0B1; s1[5] = x11; s1[6] = x33;
        s2[0] = a[0]; s2[1] = b[1]; s2[2] = x20; s2[3] = x2; s2[4] = A0B1; s2[5] = x28; s2[6] = Tba.y;
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = x28; e[4] = Tba.y;
        px = 4; py = 2; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 11:
        L[0] = LA0lx; R[0] = zero;
        L[1] = LB1ly; R[1] = zero;
        L[2] = LA0ux; R[2] = zero;
        L[3] = LB1uy; R[3] = zero;
        s1[0] = b[1]; s1[1] = a[0]; s1[2] = x23; s1[3] = Tba.x; s1[4] = A0B1; s1[5] = x11; s1[6] = x14;
        s2[0] = a[0]; s2[1] = b[1]; s2[2] = x20; s2[3] = x8; s2[4] = A0B1; s2[5] = Tab.x; s2[6] = Tba.y;
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = Tab.x; e[4] = Tba.y;
        px = 4; py = 2; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 12:
        L[0] = b[1]; R[0] = UA0uy;
        L[1] = a[1]; R[1] = UB0uy;
        L[2] = b[1]; R[2] = UA0ly;
        L[3] = a[1]; R[3] = UB0ly;
        s1[0] = b[0]; s1[1] = a[0]; s1[2] = A0B1; s1[3] = x34; s1[4] = A0B0; s1[5] = x35; s1[6] = x24;
        s2[0] = a[0]; s2[1] = b[0]; s2[2] = A1B0; s2[3] = x36; s2[4] = A0B0; s2[5] = x37; s2[6] = x30;
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = x37; e[4] = x30;
        px = 4; py = 1; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 13:
        L[0] = UA0ly; R[0] = zero;
        L[1] = a[1]; R[1] = LB0uy;
        L[2] = UA0uy; R[2] = zero;
        L[3] = a[1]; R[3] = LB0ly;
        s1[0] = b[0]; s1[1] = a[0]; s1[2] = x12; s1[3] = x29; s1[4] = A0B0; s1[5] = x35; s1[6] = x14;
        s2[0] = a[0]; s2[1] = b[0]; s2[2] = A1B0; s2[3] = x31; s2[4] = A0B0; s2[5] = Tab.x; s2[6] = x30;
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = Tab.x; e[4] = x30;
        px = 4; py = 1; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 14:
        L[0] = b[1]; R[0] = LA0uy;
        L[1] = UB0ly; R[1] = zero;
        L[2] = b[1]; R[2] = LA0ly;
        L[3] = UB0uy; R[3] = zero;
        s1[0] = b[0]; s1[1] = a[0]; s1[2] = A0B1; s1[3] = x21; s1[4] = A0B0; s1[5] = x22; s1[6] = x24;
        s2[0] = a[0]; s2[1] = b[0]; s2[2] = x6; s2[3] = x17; s2[4] = A0B0; s2[5] = x37; s2[6] = Tba.x;
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = x37; e[4] = Tba.x;
        px = 4; py = 2; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 15:
        L[0] = LA0ly; R[0] = zero;
        L[1] = LB0ly; R[1] = zero;
        L[2] = LA0uy; R[2] = zero;
        L[3] = LB0uy; R[3] = zero;
        s1[0] = b[0]; s1[1] = a[0]; s1[2] = x12; s1[3] = Tba.y; s1[4] = A0B0; s1[5] = x22; s1[6] = x14;
        s2[0] = a[0]; s2[1] = b[0]; s2[2] = x6; s2[3] = x8; s2[4] = A0B0; s2[5] = Tab.x; s2[6] = Tba.x;
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = Tab.x; e[4] = Tba.x;
        px = 4; py = 2; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    default:
        break;
    }
    /* every part evaluated on every lane (all are pure), each with its own context */
    C c0 = ctx, c1 = ctx, c2 = ctx, c3 = ctx, ci1 = ctx, ci2 = ctx, ce = ctx;
    const bool k0 = cmp_lt(L[0], R[0], c0, 0), k1 = cmp_lt(L[1], R[1], c1, 0);
    const bool k2 = cmp_lt(L[2], R[2], c2, 0), k3 = cmp_lt(L[3], R[3], c3, 0);
    const bool i1 = in_slab(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], ci1);
    const bool i2 = in_slab(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], ci2);
    const int t0 = c0.bad ? -1 : k0, t1 = c1.bad ? -1 : k1, t2 = c2.bad ? -1 : k2, t3 = c3.bad ? -1 : k3;
    const int u1 = ci1.bad ? -1 : i1, u2 = ci2.bad ? -1 : i2;
    hit = (j < 16 && !ctx.bad) ? rc_and3(rc_and3(t0, t1), rc_and3(rc_or3(t2, u1), rc_or3(t3, u2))) : (ctx.bad ? -1 : 0);
    T t, u;
    edge_params(t, u, e[0], e[1], e[2], e[3], e[4], ce);
    const T Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : zero;
    const T Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : zero;
    const V3T<T> P = v3t<T>(Px, Py, zero);
    /* rect_point2 / rect_point1 with the column picks as selects (cb, cu in {0, 1}) */
    const T rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];
    const T rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];
    const V3T<T> Q2 = v3t(Tab.x + rbx * qb + rux * u, Tab.y + rby * qb + ruy * u, Tab.z + rbz * qb + ruz * u);
    const V3T<T> Q1 = v3t(Tab.x + rux * u, Tab.y + ruy * u, Tab.z + ruz * u);
    const V3T<T> Q = qkind == 2 ? Q2 : Q1;
    S = v3t(Q.x - P.x, Q.y - P.y, Q.z - P.z);
    vbad = ce.bad;
    return num_sqrt(dot(S, S));
}

/* the face-separation tail of C2ARectDist (no edge pair holds) */
template <class T, class C>
C2A_DEV T rect_tail(const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, C &ctx)
{
    const T zero = K(0.0);
    const V3T<T> Tba = tmul(Rab, Tab);
/* no edge pair: largest separation along the two face normals */
    T sep1, sep2;
    if (GT(Tab.z, zero)) {
        sep1 = Tab.z;
        if (LT(Rab.m[6], zero)) sep1 = sep1 + b[0] * Rab.m[6];
        if (LT(Rab.m[7], zero)) sep1 = sep1 + b[1] * Rab.m[7];
    } else {
        sep1 = -Tab.z;
        if (GT(Rab.m[6], zero)) sep1 = sep1 - b[0] * Rab.m[6];
        if (GT(Rab.m[7], zero)) sep1 = sep1 - b[1] * Rab.m[7];
    }
    if (LT(Tba.z, zero)) {
        sep2 = -Tba.z;
        if (LT(Rab.m[2], zero)) sep2 = sep2 + a[0] * Rab.m[2];
        if (LT(Rab.m[5], zero)) sep2 = sep2 + a[1] * Rab.m[5];
    } else {
        sep2 = Tba.z;
        if (GT(Rab.m[2], zero)) sep2 = sep2 - a[0] * Rab.m[2];
        if (GT(Rab.m[5], zero)) sep2 = sep2 - a[1] * Rab.m[5];
    }
    if (GE(sep1, sep2) && GE(sep1, zero)) {
        const T qz = GT(Tab.z, zero) ? sep1 : -sep1;
        S = v3t(zero - zero, zero - zero, qz - zero);
    }
    if (GE(sep2, sep1) && GE(sep2, zero)) {
        V3T<T> Pp;
        if (LT(Tba.z, zero)) Pp = v3t(Rab.m[2] * sep2 + Tab.x, Rab.m[5] * sep2 + Tab.y, Rab.m[8] * sep2 + Tab.z);
        else Pp = v3t(-Rab.m[2] * sep2 + Tab.x, -Rab.m[5] * sep2 + Tab.y, -Rab.m[8] * sep2 + Tab.z);
        S = v3t(Tab.x - Pp.x, Tab.y - Pp.y, Tab.z - Pp.z);
    }
    /* sep1 > sep2 ? sep1 : sep2, then > 0 ? sep : 0: both continuous */
    return pos_or0_c(max_c(sep1, sep2));
}

/* C2ARectDist on one lane without diverging across the cases: the preamble
 * once, then the sixteen cases in the reference's order, each through the
 * same code path with its operands picked by a switch, until one holds; its
 * edge-pair distance, or the face-separation tail when none does.  Same
 * expression trees and the same first-hit rule as rect_dist; with the FP32
 * filter an undecided case sets ctx.bad (the caller recomputes in FP64). */
template <class T, class C>
C2A_DEV T rect_dist_lane(const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, C &ctx)
{
    const T zero = K(0.0);
    const T A0B0 = Rab.m[0], A0B1 = Rab.m[1], A1B0 = Rab.m[3], A1B1 = Rab.m[4];
    const T aA0B0 = a[0] * A0B0, aA0B1 = a[0] * A0B1, aA1B0 = a[1] * A1B0, aA1B1 = a[1] * A1B1;
    const T bA0B0 = b[0] * A0B0, bA1B0 = b[0] * A1B0, bA0B1 = b[1] * A0B1, bA1B1 = b[1] * A1B1;
    const V3T<T> Tba = tmul(Rab, Tab);

    const T ALLx = -Tba.x, ALUx = ALLx + aA1B0, AULx = ALLx + aA0B0, AUUx = ALUx + aA0B0;
    T LA1lx, LA1ux, UA1lx, UA1ux, LB1lx, LB1ux, UB1lx, UB1ux;
    if (LT(ALLx, ALUx)) { LA1lx = ALLx; LA1ux = ALUx; UA1lx = AULx; UA1ux = AUUx; }
    else { LA1lx = ALUx; LA1ux = ALLx; UA1lx = AUUx; UA1ux = AULx; }
    const T BLLx = Tab.x, BLUx = BLLx + bA0B1, BULx = BLLx + bA0B0, BUUx = BLUx + bA0B0;
    if (LT(BLLx, BLUx)) { LB1lx = BLLx; LB1ux = BLUx; UB1lx = BULx; UB1ux = BUUx; }
    else { LB1lx = BLUx; LB1ux = BLLx; UB1lx = BUUx; UB1ux = BULx; }

    const T ALLy = -Tba.y, ALUy = ALLy + aA1B1, AULy = ALLy + aA0B1, AUUy = ALUy + aA0B1;
    T LA1ly, LA1uy, UA1ly, UA1uy, LB0lx, LB0ux, UB0lx, UB0ux;
    if (LT(ALLy, ALUy)) { LA1ly = ALLy; LA1uy = ALUy; UA1ly = AULy; UA1uy = AUUy; }
    else { LA1ly = ALUy; LA1uy = ALLy; UA1ly = AUUy; UA1uy = AULy; }
    if (LT(BLLx, BULx)) { LB0lx = BLLx; LB0ux = BULx; UB0lx = BLUx; UB0ux = BUUx; }
    else { LB0lx = BULx; LB0ux = BLLx; UB0lx = BUUx; UB0ux = BLUx; }

    const T BLLy = Tab.y, BLUy = BLLy + bA1B1, BULy = BLLy + bA1B0, BUUy = BLUy + bA1B0;
    T LA0lx, LA0ux, UA0lx, UA0ux, LB1ly, LB1uy, UB1ly, UB1uy;
    if (LT(ALLx, AULx)) { LA0lx = ALLx; LA0ux = AULx; UA0lx = ALUx; UA0ux = AUUx; }
    else { LA0lx = AULx; LA0ux = ALLx; UA0lx = AUUx; UA0ux = ALUx; }
    if (LT(BLLy, BLUy)) { LB1ly = BLLy; LB1uy = BLUy; UB1ly = BULy; UB1uy = BUUy; }
    else { LB1ly = BLUy; LB1uy = BLLy; UB1ly = BUUy; UB1uy = BULy; }

    T LA0ly, LA0uy, UA0ly, UA0uy, LB0ly, LB0uy, UB0ly, UB0uy;
    if (LT(ALLy, AULy)) { LA0ly = ALLy; LA0uy = AULy; UA0ly = ALUy; UA0uy = AUUy; }
    else { LA0ly = AULy; LA0uy = ALLy; UA0ly = AUUy; UA0uy = ALUy; }
    if (LT(BLLy, BULy)) { LB0ly = BLLy; LB0uy = BULy; UB0ly = BLUy; UB0uy = BUUy; }
    else { LB0ly = BULy; LB0uy = BLLy; UB0ly = BUUy; UB0uy = BLUy; }

    
    const T x0 = aA0B0 - b[0] - Tba.x;
    const T x1 = aA0B1 - Tba.y;
    const T x2 = -Tab.y - bA1B0;
    const T x3 = Tab.x + bA0B0 - a[0];
    const T x4 = Tab.y + bA1B0;
    const T x5 = Tba.y - aA0B1;
    const T x6 = -A1B0;
    const T x7 = Tba.x - aA0B0;
    const T x8 = -Tab.y;
    const T x9 = Tab.x - a[0];
    const T x10 = -Tba.x - b[0];
    const T x11 = -Tba.y;
    const T x12 = -A0B1;
    const T x13 = -Tab.x - bA0B0;
    const T x14 = -Tab.x;
    const T x15 = aA0B1 - Tba.y - b[1];
    const T x16 = aA0B0 - Tba.x;
    const T x17 = -Tab.y - bA1B1;
    const T x18 = Tab.x - a[0] + bA0B1;
    const T x19 = Tab.y + bA1B1;
    const T x20 = -A1B1;
    const T x21 = -Tba.y - b[1];
    const T x22 = -Tba.x;
    const T x23 = -A0B0;
    const T x24 = -Tab.x - bA0B1;
    const T x25 = aA1B0 - Tba.x - b[0];
    const T x26 = aA1B1 - Tba.y;
    const T x27 = Tab.y - a[1] + bA1B0;
    const T x28 = Tab.x + bA0B0;
    const T x29 = Tba.y - aA1B1;
    const T x30 = Tba.x - aA1B0;
    const T x31 = Tab.y - a[1];
    const T x32 = -b[0] - Tba.x;
    const T x33 = -bA0B0 - Tab.x;
    const T x34 = aA1B1 - Tba.y - b[1];
    const T x35 = aA1B0 - Tba.x;
    const T x36 = Tab.y - a[1] + bA1B1;
    const T x37 = Tab.x + bA0B1;
    int win = -1;
#pragma unroll 1
    for (int j = 0; j < 16 && !ctx.bad; j++) {
        T L[4], R[4], s1[7], s2[7];
        switch (j) {
        case 0:
            L[0] = b[0]; R[0] = UA1ux;
            L[1] = a[0]; R[1] = UB1ux;
            L[2] = b[0]; R[2] = UA1lx;
            L[3] = a[0]; R[3] = UB1lx;
            s1[0] = b[1]; s1[1] = a[1]; s1[2] = A1B0; s1[3] = x0; s1[4] = A1B1; s1[5] = x1; s1[6] = x2;
            s2[0] = a[1]; s2[1] = b[1]; s2[2] = A0B1; s2[3] = x3; s2[4] = A1B1; s2[5] = x4; s2[6] = x5;
            break;
        case 1:
            L[0] = UA1lx; R[0] = zero;
            L[1] = a[0]; R[1] = LB1ux;
            L[2] = UA1ux; R[2] = zero;
            L[3] = a[0]; R[3] = LB1lx;
            s1[0] = b[1]; s1[1] = a[1]; s1[2] = x6; s1[3] = x7; s1[4] = A1B1; s1[5] = x1; s1[6] = x8;
            s2[0] = a[1]; s2[1] = b[1]; s2[2] = A0B1; s2[3] = x9; s2[4] = A1B1; s2[5] = Tab.y; s2[6] = x5;
            break;
        case 2:
            L[0] = b[0]; R[0] = LA1ux;
            L[1] = UB1lx; R[1] = zero;
            L[2] = b[0]; R[2] = LA1lx;
            L[3] = UB1ux; R[3] = zero;
            s1[0] = b[1]; s1[1] = a[1]; s1[2] = A1B0; s1[3] = x10; s1[4] = A1B1; s1[5] = x11; s1[6] = x2;
            s2[0] = a[1]; s2[1] = b[1]; s2[2] = x12; s2[3] = x13; s2[4] = A1B1; s2[5] = x4; s2[6] = Tba.y;
            break;
        case 3:
            L[0] = LA1lx; R[0] = zero;
            L[1] = LB1lx; R[1] = zero;
            L[2] = LA1ux; R[2] = zero;
            L[3] = LB1ux; R[3] = zero;
            s1[0] = b[1]; s1[1] = a[1]; s1[2] = x6; s1[3] = Tba.x; s1[4] = A1B1; s1[5] = x11; s1[6] = x8;
            s2[0] = a[1]; s2[1] = b[1]; s2[2] = x12; s2[3] = x14; s2[4] = A1B1; s2[5] = Tab.y; s2[6] = Tba.y;
            break;
        case 4:
            L[0] = b[1]; R[0] = UA1uy;
            L[1] = a[0]; R[1] = UB0ux;
            L[2] = b[1]; R[2] = UA1ly;
            L[3] = a[0]; R[3] = UB0lx;
            s1[0] = b[0]; s1[1] = a[1]; s1[2] = A1B1; s1[3] = x15; s1[4] = A1B0; s1[5] = x16; s1[6] = x17;
            s2[0] = a[1]; s2[1] = b[0]; s2[2] = A0B0; s2[3] = x18; s2[4] = A1B0; s2[5] = x19; s2[6] = x7;
            break;
        case 5:
            L[0] = UA1ly; R[0] = zero;
            L[1] = a[0]; R[1] = LB0ux;
            L[2] = UA1uy; R[2] = zero;
            L[3] = a[0]; R[3] = LB0lx;
            s1[0] = b[0]; s1[1] = a[1]; s1[2] = x20; s1[3] = x5; s1[4] = A1B0; s1[5] = x16; s1[6] = x8;
            s2[0] = a[1]; s2[1] = b[0]; s2[2] = A0B0; s2[3] = x9; s2[4] = A1B0; s2[5] = Tab.y; s2[6] = x7;
            break;
        case 6:
            L[0] = b[1]; R[0] = LA1uy;
            L[1] = UB0lx; R[1] = zero;
            L[2] = b[1]; R[2] = LA1ly;
            L[3] = UB0ux; R[3] = zero;
            s1[0] = b[0]; s1[1] = a[1]; s1[2] = A1B1; s1[3] = x21; s1[4] = A1B0; s1[5] = x22; s1[6] = x17;
            s2[0] = a[1]; s2[1] = b[0]; s2[2] = x23; s2[3] = x24; s2[4] = A1B0; s2[5] = x19; s2[6] = Tba.x;
            break;
        case 7:
            L[0] = LA1ly; R[0] = zero;
            L[1] = LB0lx; R[1] = zero;
            L[2] = LA1uy; R[2] = zero;
            L[3] = LB0ux; R[3] = zero;
            s1[0] = b[0]; s1[1] = a[1]; s1[2] = x20; s1[3] = Tba.y; s1[4] = A1B0; s1[5] = x22; s1[6] = x8;
            s2[0] = a[1]; s2[1] = b[0]; s2[2] = x23; s2[3] = x14; s2[4] = A1B0; s2[5] = Tab.y; s2[6] = Tba.x;
            break;
        case 8:
            L[0] = b[0]; R[0] = UA0ux;
            L[1] = a[1]; R[1] = UB1uy;
            L[2] = b[0]; R[2] = UA0lx;
            L[3] = a[1]; R[3] = UB1ly;
            s1[0] = b[1]; s1[1] = a[0]; s1[2] = A0B0; s1[3] = x25; s1[4] = A0B1; s1[5] = x26; s1[6] = x13;
            s2[0] = a[0]; s2[1] = b[1]; s2[2] = A1B1; s2[3] = x27; s2[4] = A0B1; s2[5] = x28; s2[6] = x29;
            break;
        case 9:
            L[0] = UA0lx; R[0] = zero;
            L[1] = a[1]; R[1] = LB1uy;
            L[2] = UA0ux; R[2] = zero;
            L[3] = a[1]; R[3] = LB1ly;
            s1[0] = b[1]; s1[1] = a[0]; s1[2] = x23; s1[3] = x30; s1[4] = A0B1; s1[5] = x26; s1[6] = x14;
            s2[0] = a[0]; s2[1] = b[1]; s2[2] = A1B1; s2[3] = x31; s2[4] = A0B1; s2[5] = Tab.x; s2[6] = x29;
            break;
        case 10:
            L[0] = b[0]; R[0] = LA0ux;
            L[1] = UB1ly; R[1] = zero;
            L[2] = b[0]; R[2] = LA0lx;
            L[3] = UB1uy; R[3] = zero;
            s1[0] = b[1]; s1[1] = a[0]; s1[2] = A0B0; s1[3] = x32; s1[4] = A0B1; s1[5] = x11; s1[6] = x33;
            s2[0] = a[0]; s2[1] = b[1]; s2[2] = x20; s2[3] = x2; s2[4] = A0B1; s2[5] = x28; s2[6] = Tba.y;
            break;
        case 11:
            L[0] = LA0lx; R[0] = zero;
            L[1] = LB1ly; R[1] = zero;
            L[2] = LA0ux; R[2] = zero;
            L[3] = LB1uy; R[3] = zero;
            s1[0] = b[1]; s1[1] = a[0]; s1[2] = x23; s1[3] = Tba.x; s1[4] = A0B1; s1[5] = x11; s1[6] = x14;
            s2[0] = a[0]; s2[1] = b[1]; s2[2] = x20; s2[3] = x8; s2[4] = A0B1; s2[5] = Tab.x; s2[6] = Tba.y;
            break;
        case 12:
            L[0] = b[1]; R[0] = UA0uy;
            L[1] = a[1]; R[1] = UB0uy;
            L[2] = b[1]; R[2] = UA0ly;
            L[3] = a[1]; R[3] = UB0ly;
            s1[0] = b[0]; s1[1] = a[0]; s1[2] = A0B1; s1[3] = x34; s1[4] = A0B0; s1[5] = x35; s1[6] = x24;
            s2[0] = a[0]; s2[1] = b[0]; s2[2] = A1B0; s2[3] = x36; s2[4] = A0B0; s2[5] = x37; s2[6] = x30;
            break;
        case 13:
            L[0] = UA0ly; R[0] = zero;
            L[1] = a[1]; R[1] = LB0uy;
            L[2] = UA0uy; R[2] = zero;
            L[3] = a[1]; R[3] = LB0ly;
            s1[0] = b[0]; s1[1] = a[0]; s1[2] = x12; s1[3] = x29; s1[4] = A0B0; s1[5] = x35; s1[6] = x14;
            s2[0] = a[0]; s2[1] = b[0]; s2[2] = A1B0; s2[3] = x31; s2[4] = A0B0; s2[5] = Tab.x; s2[6] = x30;
            break;
        case 14:
            L[0] = b[1]; R[0] = LA0uy;
            L[1] = UB0ly; R[1] = zero;
            L[2] = b[1]; R[2] = LA0ly;
            L[3] = UB0uy; R[3] = zero;
            s1[0] = b[0]; s1[1] = a[0]; s1[2] = A0B1; s1[3] = x21; s1[4] = A0B0; s1[5] = x22; s1[6] = x24;
            s2[0] = a[0]; s2[1] = b[0]; s2[2] = x6; s2[3] = x17; s2[4] = A0B0; s2[5] = x37; s2[6] = Tba.x;
            break;
        case 15:
            L[0] = LA0ly; R[0] = zero;
            L[1] = LB0ly; R[1] = zero;
            L[2] = LA0uy; R[2] = zero;
            L[3] = LB0uy; R[3] = zero;
            s1[0] = b[0]; s1[1] = a[0]; s1[2] = x12; s1[3] = Tba.y; s1[4] = A0B0; s1[5] = x22; s1[6] = x14;
            s2[0] = a[0]; s2[1] = b[0]; s2[2] = x6; s2[3] = x8; s2[4] = A0B0; s2[5] = Tab.x; s2[6] = Tba.x;
            break;
        default:
            break;
        }
        C c0 = ctx, c1 = ctx, c2 = ctx, c3 = ctx, ci1 = ctx, ci2 = ctx;
        const bool k0 = cmp_lt(L[0], R[0], c0, 0), k1 = cmp_lt(L[1], R[1], c1, 0);
        const int t0 = c0.bad ? -1 : k0, t1 = c1.bad ? -1 : k1;
        if (rc_and3(t0, t1) == 0) continue; /* the usual outcome: no in_slab needed */
        const bool k2 = cmp_lt(L[2], R[2], c2, 0), k3 = cmp_lt(L[3], R[3], c3, 0);
        const int t2 = c2.bad ? -1 : k2, t3 = c3.bad ? -1 : k3;
        int u1 = 1, u2 = 1;
        if (t2 != 1) {
            const bool i1 = in_slab_inl(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], ci1);
            u1 = ci1.bad ? -1 : i1;
        }
        if (t3 != 1) {
            const bool i2 = in_slab_inl(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], ci2);
            u2 = ci2.bad ? -1 : i2;
        }
        const int hit = rc_and3(rc_and3(t0, t1), rc_and3(rc_or3(t2, u1), rc_or3(t3, u2)));
        if (hit < 0) ctx.bad = true;
        else if (hit == 1) {
            win = j;
            break;
        }
    }
    if (ctx.bad) return zero;
    if (win < 0) return rect_tail(Rab, Tab, a, b, S, ctx);
    T e[5], qb = zero;
    int px = 0, py = 0, qkind = 1, cb = 0, cu = 0;
    switch (win) {
    case 0:
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = x4; e[4] = x5;
        px = 0; py = 4; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 1:
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = Tab.y; e[4] = x5;
        px = 0; py = 4; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 2:
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = x4; e[4] = Tba.y;
        px = 2; py = 4; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 3:
        e[0] = a[1]; e[1] = b[1]; e[2] = A1B1; e[3] = Tab.y; e[4] = Tba.y;
        px = 2; py = 4; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 4:
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = x19; e[4] = x7;
        px = 0; py = 4; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 5:
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = Tab.y; e[4] = x7;
        px = 0; py = 4; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 6:
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = x19; e[4] = Tba.x;
        px = 2; py = 4; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 7:
        e[0] = a[1]; e[1] = b[0]; e[2] = A1B0; e[3] = Tab.y; e[4] = Tba.x;
        px = 2; py = 4; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 8:
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = x28; e[4] = x29;
        px = 4; py = 1; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 9:
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = Tab.x; e[4] = x29;
        px = 4; py = 1; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 10:
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = x28; e[4] = Tba.y;
        px = 4; py = 2; qkind = 2; cb = 0; qb = b[0]; cu = 1;
        break;
    case 11:
        e[0] = a[0]; e[1] = b[1]; e[2] = A0B1; e[3] = Tab.x; e[4] = Tba.y;
        px = 4; py = 2; qkind = 1; cb = 0; qb = zero; cu = 1;
        break;
    case 12:
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = x37; e[4] = x30;
        px = 4; py = 1; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 13:
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = Tab.x; e[4] = x30;
        px = 4; py = 1; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    case 14:
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = x37; e[4] = Tba.x;
        px = 4; py = 2; qkind = 2; cb = 1; qb = b[1]; cu = 0;
        break;
    case 15:
        e[0] = a[0]; e[1] = b[0]; e[2] = A0B0; e[3] = Tab.x; e[4] = Tba.x;
        px = 4; py = 2; qkind = 1; cb = 0; qb = zero; cu = 0;
        break;
    default:
        break;
    }
    T t, u;
    edge_params_inl(t, u, e[0], e[1], e[2], e[3], e[4], ctx);
    const T Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : zero;
    const T Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : zero;
    const V3T<T> P = v3t<T>(Px, Py, zero);
    const T rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];
    const T rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];
    const V3T<T> Q2 = v3t(Tab.x + rbx * qb + rux * u, Tab.y + rby * qb + ruy * u, Tab.z + rbz * qb + ruz * u);
    const V3T<T> Q1 = v3t(Tab.x + rux * u, Tab.y + ruy * u, Tab.z + ruz * u);
    const V3T<T> Q = qkind == 2 ? Q2 : Q1;
    S = v3t(Q.x - P.x, Q.y - P.y, Q.z - P.z);
    return num_sqrt(dot(S, S));
}

} // namespace c2a
#endif
