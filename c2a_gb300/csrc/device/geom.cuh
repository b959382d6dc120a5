/*
 * geom.cuh -- device geometry of the CA step, written once for two number
 * types:
 *
 *   double  the exact path: every product and sum rounds on its own
 *           (--fmad=false) in the reference's left-to-right order, so the
 *           results are bit-identical to the reference;
 *   EF      the FP32 filter (ef.cuh): the same expression trees in FP32 with
 *           a certified bound to the FP64 result; a branch the bound cannot
 *           decide marks the context bad and the caller recomputes in FP64.
 *
 *   rect_dist   C2ARectDist (C2A/C2A_RectDist.h:157-934)
 *   tri_dist    TriDist with contact features (C2A/src/C2A.cpp:59-405)
 *   bound_leaf  CInterpMotion_Linear::computeTOC(d, r, S) (C2A/src/InterpMotion.cpp:746-828)
 *   bound_rss   CInterpMotion_Linear::computeTOC_MotionBound (InterpMotion.cpp:831-881)
 *
 * Decisions go through the cmp_* helpers (plain comparisons for double);
 * clamps, max(., 0) and |x| go through the *_c helpers, which are continuous
 * and need no decision in FP32.
 */
#ifndef C2A_GEOM_CUH
#define C2A_GEOM_CUH

#include "../common/c2a_motion.h"
#include "ef.cuh"

namespace c2a {

#if !defined(__CUDACC__)
using std::isnan;
using std::sqrt;
#endif

#if defined(__CUDACC__)
#define C2A_DEV __host__ __device__ __forceinline__
/* the large pieces stay out of line: one copy each, reached from every call site */
#define C2A_NOINL __host__ __device__ __noinline__
#else /* host build of the CPU soundness test */
#define C2A_DEV inline
#define C2A_NOINL inline
#endif

struct ExactCtx {
    bool bad; /* never set */
};

/* ---------------------------------------------------- number-type glue */
C2A_DEV double num_div(double a, double b, ExactCtx &) { return a / b; }
C2A_DEV EF num_div(EF a, EF b, EFCtx &c) { return ef_div(a, b, c); }
C2A_DEV double num_sqrt(double a) { return sqrt(a); }
C2A_DEV EF num_sqrt(EF a) { return ef_sqrt(a); }
C2A_DEV double abs_c(double a) { return a < 0 ? -a : a; }
C2A_DEV EF abs_c(EF a) { return ef_abs(a); }
C2A_DEV double max0_c(double a) { return a < 0 ? 0 : a; }  /* if (a < 0) a = 0 */
C2A_DEV EF max0_c(EF a) { return ef_max0(a); }
C2A_DEV double min0_c(double a) { return a > 0 ? 0 : a; }  /* if (a > 0) a = 0 */
C2A_DEV EF min0_c(EF a) { return EF{a.v > 0.0f ? 0.0f : a.v, a.e}; }
C2A_DEV double pos_or0_c(double a) { return a > 0 ? a : 0; } /* a > 0 ? a : 0 */
C2A_DEV EF pos_or0_c(EF a) { return ef_max0(a); }
C2A_DEV double max_c(double a, double b) { return a > b ? a : b; }
C2A_DEV EF max_c(EF a, EF b) { return EF{a.v > b.v ? a.v : b.v, ef_emax(a.e, b.e)}; }
/* if ((t < 0) || isnan(t)) t = 0; else if (t > 1) t = 1 */
C2A_DEV double nan_to_zero_clamp01(double t)
{
    if ((t < 0) || isnan(t)) return 0;
    if (t > 1) return 1;
    return t;
}
C2A_DEV EF nan_to_zero_clamp01(EF t) { return ef_clamp(t, EF{0.0f, 0.0f}, EF{1.0f, 0.0f}); }
/* Clamp (RectDist.h:44-50): val < lo ? lo : val > hi ? hi : val, with lo <= hi */
C2A_DEV double clamp_c(double v, double lo, double hi)
{
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}
C2A_DEV EF clamp_c(EF v, EF lo, EF hi) { return ef_clamp(v, lo, hi); }
C2A_DEV bool is_nan(double a) { return isnan(a); }
C2A_DEV bool is_nan(EF a) { return isnan(a.v); }

template <class T> C2A_DEV T cst(double c);
template <> C2A_DEV double cst<double>(double c) { return c; }
/* a constant of the reference's source: its FP32 rounding and that rounding's size */
template <> C2A_DEV EF cst<EF>(double c)
{
    const float v = (float)c;
    const double err = (double)v - c;
    return EF{v, (float)((err < 0 ? -err : err) * 1.001)};
}
/* an FP64 input (a transform entry, a motion constant, a running distance) */
C2A_DEV double in_d(double x, ExactCtx &) { return x; }
C2A_DEV EF in_d(double x, EFCtx &c)
{
    long long b;
    memcpy(&b, &x, sizeof(b));
    const int ex = (int)((b >> 52) & 0x7ff);
    if ((ex < 897 && (b & 0x7fffffffffffffffLL) != 0) || ex > 1150) C2A_EF_FAIL(c, __LINE__); /* outside FP32's normal range */
    return ef_of(x);
}

C2A_DEV bool cmp_eq0(double a, ExactCtx &, int) { return a == 0; }
C2A_DEV bool cmp_eq0(EF a, EFCtx &c, int line)
{
    if (a.v == 0.0f && a.e == 0.0f) return true;
    if (ef_rd_sub(fabsf(a.v), a.e) > 0.0f) return false;
    C2A_EF_FAIL(c, line);
    return false;
}
C2A_DEV bool cmp_lt(double a, double b, ExactCtx &, int) { return a < b; }
C2A_DEV bool cmp_le(double a, double b, ExactCtx &, int) { return a <= b; }
C2A_DEV bool cmp_lt(EF a, EF b, EFCtx &c, int line)
{
    const int r = ef_lt3(a, b);
    if (r < 0) C2A_EF_FAIL(c, line);
    return r == 1;
}
C2A_DEV bool cmp_le(EF a, EF b, EFCtx &c, int line)
{
    const int r = ef_le3(a, b);
    if (r < 0) C2A_EF_FAIL(c, line);
    return r == 1;
}
#define LT(a, b) cmp_lt((a), (b), ctx, __LINE__)
#define GT(a, b) cmp_lt((b), (a), ctx, __LINE__)
#define LE(a, b) cmp_le((a), (b), ctx, __LINE__)
#define GE(a, b) cmp_le((b), (a), ctx, __LINE__)
#define EQ0(a) cmp_eq0((a), ctx, __LINE__)
#define K(c) cst<T>(c)

/* ---------------------------------------------------------- 3-vectors */
template <class T> struct V3T {
    T x, y, z;
};
template <class T> C2A_DEV V3T<T> v3t(T x, T y, T z) { return V3T<T>{x, y, z}; }
template <class T> C2A_DEV V3T<T> operator-(V3T<T> a, V3T<T> b) { return v3t(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> C2A_DEV V3T<T> operator+(V3T<T> a, V3T<T> b) { return v3t(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> C2A_DEV V3T<T> mul_s(V3T<T> a, T s) { return v3t(a.x * s, a.y * s, a.z * s); }
template <class T> C2A_DEV V3T<T> add_mul(V3T<T> a, V3T<T> b, T s)
{
    return v3t(a.x + b.x * s, a.y + b.y * s, a.z + b.z * s);
}
template <class T> C2A_DEV T dot(V3T<T> a, V3T<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> C2A_DEV V3T<T> cross(V3T<T> a, V3T<T> b)
{
    return v3t(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> C2A_DEV T dist2(V3T<T> a, V3T<T> b)
{
    return (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z);
}
template <class T, class C> C2A_DEV V3T<T> normalized(V3T<T> a, C &ctx)
{
    T d = num_div(K(1.0), num_sqrt(a.x * a.x + a.y * a.y + a.z * a.z), ctx);
    return v3t(a.x * d, a.y * d, a.z * d);
}
template <class T> C2A_DEV T length(V3T<T> a) { return num_sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

/* row-major 3x3 */
template <class T> struct M3T {
    T m[9];
};
template <class T> C2A_DEV V3T<T> mul(const M3T<T> &R, V3T<T> p)
{
    return v3t(R.m[0] * p.x + R.m[1] * p.y + R.m[2] * p.z, R.m[3] * p.x + R.m[4] * p.y + R.m[5] * p.z,
               R.m[6] * p.x + R.m[7] * p.y + R.m[8] * p.z);
}
template <class T> C2A_DEV V3T<T> mul_add(const M3T<T> &R, V3T<T> p, V3T<T> t)
{
    return v3t(R.m[0] * p.x + R.m[1] * p.y + R.m[2] * p.z + t.x, R.m[3] * p.x + R.m[4] * p.y + R.m[5] * p.z + t.y,
               R.m[6] * p.x + R.m[7] * p.y + R.m[8] * p.z + t.z);
}
template <class T> C2A_DEV V3T<T> tmul(const M3T<T> &R, V3T<T> p)
{
    return v3t(R.m[0] * p.x + R.m[3] * p.y + R.m[6] * p.z, R.m[1] * p.x + R.m[4] * p.y + R.m[7] * p.z,
               R.m[2] * p.x + R.m[5] * p.y + R.m[8] * p.z);
}
template <class T> C2A_DEV M3T<T> mmul(const M3T<T> &A, const M3T<T> &B)
{
    M3T<T> r;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = A.m[3 * i] * B.m[j] + A.m[3 * i + 1] * B.m[3 + j] + A.m[3 * i + 2] * B.m[6 + j];
    return r;
}
template <class T> C2A_DEV M3T<T> tmmul(const M3T<T> &A, const M3T<T> &B)
{
    M3T<T> r;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = A.m[i] * B.m[j] + A.m[3 + i] * B.m[3 + j] + A.m[6 + i] * B.m[6 + j];
    return r;
}

typedef V3T<double> V3;
typedef M3T<double> M3;
C2A_DEV V3 v3(double x, double y, double z) { return V3{x, y, z}; }

/* ------------------------------------------------------------- RectDist */

template <class T, class C>
C2A_DEV void edge_params_inl(T &t, T &u, T a, T b, T AdB, T AdT, T BdT, C &ctx)
{
    const T zero = K(0.0);
    T denom = K(1.0) - (AdB) * (AdB);
    if (EQ0(denom)) t = zero;
    else t = clamp_c(num_div(AdT - BdT * AdB, denom, ctx), zero, a);
    u = t * AdB - BdT;
    if (LT(u, zero)) {
        u = zero;
        t = clamp_c(AdT, zero, a);
    } else if (GT(u, b)) {
        u = b;
        t = clamp_c(u * AdB + AdT, zero, a);
    }
}

template <class T, class C>
C2A_DEV bool in_slab_inl(T a, T b, T AnB, T AnT, T AdB, T AdT, T BdT, C &ctx)
{
    const T zero = K(0.0);
    if (LT(abs_c(AnB), K(1e-7))) return false;
    T u = clamp_c(num_div(-AnT, AnB, ctx), zero, b);
    T t = clamp_c(u * AdB + AdT, zero, a);
    T v = t * AdB - BdT;
    if (GT(AnB, zero)) return GT(v, (u + K(1e-7)));
    return LT(v, (u - K(1e-7)));
}

/* the out-of-line forms the sequential rect_dist calls from its sixteen cases */
template <class T, class C>
C2A_NOINL void edge_params(T &t, T &u, T a, T b, T AdB, T AdT, T BdT, C &ctx)
{
    edge_params_inl(t, u, a, b, AdB, AdT, BdT, ctx);
}
template <class T, class C>
C2A_NOINL bool in_slab(T a, T b, T AnB, T AnT, T AdB, T AdT, T BdT, C &ctx)
{
    return in_slab_inl(a, b, AnB, AnT, AdB, AdT, BdT, ctx);
}

/* Q = Tab + Rab[:,cb] qb + Rab[:,cu] u, evaluated as (Tab + R qb) + R u */
template <class T> C2A_DEV V3T<T> rect_point2(const M3T<T> &R, V3T<T> T0, int cb, T qb, int cu, T u)
{
    return v3t(T0.x + R.m[cb] * qb + R.m[cu] * u, T0.y + R.m[3 + cb] * qb + R.m[3 + cu] * u,
               T0.z + R.m[6 + cb] * qb + R.m[6 + cu] * u);
}
template <class T> C2A_DEV V3T<T> rect_point1(const M3T<T> &R, V3T<T> T0, int cu, T u)
{
    return v3t(T0.x + R.m[cu] * u, T0.y + R.m[3 + cu] * u, T0.z + R.m[6 + cu] * u);
}

/*
 * Distance between rectangle A = [0,a0]x[0,a1] and B = Tab + Rab [0,b0]x[0,b1]
 * (B in A's frame).  S receives Q - P of the closest points; it is left
 * untouched only when the result is 0 through the face-separation fallback,
 * exactly like the reference.
 */
template <class T, class C>
C2A_NOINL T rect_dist(const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, C &ctx)
{
    const T zero = K(0.0);
    const T A0B0 = Rab.m[0], A0B1 = Rab.m[1], A1B0 = Rab.m[3], A1B1 = Rab.m[4];
    const T aA0B0 = a[0] * A0B0, aA0B1 = a[0] * A0B1, aA1B0 = a[1] * A1B0, aA1B1 = a[1] * A1B1;
    const T bA0B0 = b[0] * A0B0, bA1B0 = b[0] * A1B0, bA0B1 = b[1] * A0B1, bA1B1 = b[1] * A1B1;
    const V3T<T> Tba = tmul(Rab, Tab);
    T t, u;
    V3T<T> P, Q;

    const T ALLx = -Tba.x, ALUx = ALLx + aA1B0, AULx = ALLx + aA0B0, AUUx = ALUx + aA0B0;
    T LA1lx, LA1ux, UA1lx, UA1ux, LB1lx, LB1ux, UB1lx, UB1ux;
    if (LT(ALLx, ALUx)) { LA1lx = ALLx; LA1ux = ALUx; UA1lx = AULx; UA1ux = AUUx; }
    else { LA1lx = ALUx; LA1ux = ALLx; UA1lx = AUUx; UA1ux = AULx; }
    const T BLLx = Tab.x, BLUx = BLLx + bA0B1, BULx = BLLx + bA0B0, BUUx = BLUx + bA0B0;
    if (LT(BLLx, BLUx)) { LB1lx = BLLx; LB1ux = BLUx; UB1lx = BULx; UB1ux = BUUx; }
    else { LB1lx = BLUx; LB1ux = BLLx; UB1lx = BUUx; UB1ux = BULx; }
    if (ctx.bad) return zero;

#define C2A_EDGE_HIT(PX, PY, QEXPR)                                                                                \
    do {                                                                                                           \
        P = v3t<T>((PX), (PY), zero);                                                                              \
        Q = (QEXPR);                                                                                               \
        S = v3t(Q.x - P.x, Q.y - P.y, Q.z - P.z);                                                                  \
        return num_sqrt(dot(S, S));                                                                                \
    } while (0)

    /* A edges along A1 against B edges along B1 */
    if (GT(UA1ux, b[0]) && GT(UB1ux, a[0]) &&
        (GT(UA1lx, b[0]) || in_slab(b[1], a[1], A1B0, aA0B0 - b[0] - Tba.x, A1B1, aA0B1 - Tba.y, -Tab.y - bA1B0, ctx)) &&
        (GT(UB1lx, a[0]) || in_slab(a[1], b[1], A0B1, Tab.x + bA0B0 - a[0], A1B1, Tab.y + bA1B0, Tba.y - aA0B1, ctx))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y + bA1B0, Tba.y - aA0B1, ctx);
        C2A_EDGE_HIT(a[0], t, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if (LT(UA1lx, zero) && GT(LB1ux, a[0]) &&
        (LT(UA1ux, zero) || in_slab(b[1], a[1], -A1B0, Tba.x - aA0B0, A1B1, aA0B1 - Tba.y, -Tab.y, ctx)) &&
        (GT(LB1lx, a[0]) || in_slab(a[1], b[1], A0B1, Tab.x - a[0], A1B1, Tab.y, Tba.y - aA0B1, ctx))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y, Tba.y - aA0B1, ctx);
        C2A_EDGE_HIT(a[0], t, rect_point1(Rab, Tab, 1, u));
    }
    if (GT(LA1ux, b[0]) && LT(UB1lx, zero) &&
        (GT(LA1lx, b[0]) || in_slab(b[1], a[1], A1B0, -Tba.x - b[0], A1B1, -Tba.y, -Tab.y - bA1B0, ctx)) &&
        (LT(UB1ux, zero) || in_slab(a[1], b[1], -A0B1, -Tab.x - bA0B0, A1B1, Tab.y + bA1B0, Tba.y, ctx))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y + bA1B0, Tba.y, ctx);
        C2A_EDGE_HIT(zero, t, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if (LT(LA1lx, zero) && LT(LB1lx, zero) &&
        (LT(LA1ux, zero) || in_slab(b[1], a[1], -A1B0, Tba.x, A1B1, -Tba.y, -Tab.y, ctx)) &&
        (LT(LB1ux, zero) || in_slab(a[1], b[1], -A0B1, -Tab.x, A1B1, Tab.y, Tba.y, ctx))) {
        edge_params(t, u, a[1], b[1], A1B1, Tab.y, Tba.y, ctx);
        C2A_EDGE_HIT(zero, t, rect_point1(Rab, Tab, 1, u));
    }
    if (ctx.bad) return zero;

    const T ALLy = -Tba.y, ALUy = ALLy + aA1B1, AULy = ALLy + aA0B1, AUUy = ALUy + aA0B1;
    T LA1ly, LA1uy, UA1ly, UA1uy, LB0lx, LB0ux, UB0lx, UB0ux;
    if (LT(ALLy, ALUy)) { LA1ly = ALLy; LA1uy = ALUy; UA1ly = AULy; UA1uy = AUUy; }
    else { LA1ly = ALUy; LA1uy = ALLy; UA1ly = AUUy; UA1uy = AULy; }
    if (LT(BLLx, BULx)) { LB0lx = BLLx; LB0ux = BULx; UB0lx = BLUx; UB0ux = BUUx; }
    else { LB0lx = BULx; LB0ux = BLLx; UB0lx = BUUx; UB0ux = BLUx; }

    /* A edges along A1 against B edges along B0 */
    if (GT(UA1uy, b[1]) && GT(UB0ux, a[0]) &&
        (GT(UA1ly, b[1]) || in_slab(b[0], a[1], A1B1, aA0B1 - Tba.y - b[1], A1B0, aA0B0 - Tba.x, -Tab.y - bA1B1, ctx)) &&
        (GT(UB0lx, a[0]) || in_slab(a[1], b[0], A0B0, Tab.x - a[0] + bA0B1, A1B0, Tab.y + bA1B1, Tba.x - aA0B0, ctx))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y + bA1B1, Tba.x - aA0B0, ctx);
        C2A_EDGE_HIT(a[0], t, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if (LT(UA1ly, zero) && GT(LB0ux, a[0]) &&
        (LT(UA1uy, zero) || in_slab(b[0], a[1], -A1B1, Tba.y - aA0B1, A1B0, aA0B0 - Tba.x, -Tab.y, ctx)) &&
        (GT(LB0lx, a[0]) || in_slab(a[1], b[0], A0B0, Tab.x - a[0], A1B0, Tab.y, Tba.x - aA0B0, ctx))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y, Tba.x - aA0B0, ctx);
        C2A_EDGE_HIT(a[0], t, rect_point1(Rab, Tab, 0, u));
    }
    if (GT(LA1uy, b[1]) && LT(UB0lx, zero) &&
        (GT(LA1ly, b[1]) || in_slab(b[0], a[1], A1B1, -Tba.y - b[1], A1B0, -Tba.x, -Tab.y - bA1B1, ctx)) &&
        (LT(UB0ux, zero) || in_slab(a[1], b[0], -A0B0, -Tab.x - bA0B1, A1B0, Tab.y + bA1B1, Tba.x, ctx))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y + bA1B1, Tba.x, ctx);
        C2A_EDGE_HIT(zero, t, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if (LT(LA1ly, zero) && LT(LB0lx, zero) &&
        (LT(LA1uy, zero) || in_slab(b[0], a[1], -A1B1, Tba.y, A1B0, -Tba.x, -Tab.y, ctx)) &&
        (LT(LB0ux, zero) || in_slab(a[1], b[0], -A0B0, -Tab.x, A1B0, Tab.y, Tba.x, ctx))) {
        edge_params(t, u, a[1], b[0], A1B0, Tab.y, Tba.x, ctx);
        C2A_EDGE_HIT(zero, t, rect_point1(Rab, Tab, 0, u));
    }
    if (ctx.bad) return zero;

    const T BLLy = Tab.y, BLUy = BLLy + bA1B1, BULy = BLLy + bA1B0, BUUy = BLUy + bA1B0;
    T LA0lx, LA0ux, UA0lx, UA0ux, LB1ly, LB1uy, UB1ly, UB1uy;
    if (LT(ALLx, AULx)) { LA0lx = ALLx; LA0ux = AULx; UA0lx = ALUx; UA0ux = AUUx; }
    else { LA0lx = AULx; LA0ux = ALLx; UA0lx = AUUx; UA0ux = ALUx; }
    if (LT(BLLy, BLUy)) { LB1ly = BLLy; LB1uy = BLUy; UB1ly = BULy; UB1uy = BUUy; }
    else { LB1ly = BLUy; LB1uy = BLLy; UB1ly = BUUy; UB1uy = BULy; }

    /* A edges along A0 against B edges along B1 */
    if (GT(UA0ux, b[0]) && GT(UB1uy, a[1]) &&
        (GT(UA0lx, b[0]) || in_slab(b[1], a[0], A0B0, aA1B0 - Tba.x - b[0], A0B1, aA1B1 - Tba.y, -Tab.x - bA0B0, ctx)) &&
        (GT(UB1ly, a[1]) || in_slab(a[0], b[1], A1B1, Tab.y - a[1] + bA1B0, A0B1, Tab.x + bA0B0, Tba.y - aA1B1, ctx))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x + bA0B0, Tba.y - aA1B1, ctx);
        C2A_EDGE_HIT(t, a[1], rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if (LT(UA0lx, zero) && GT(LB1uy, a[1]) &&
        (LT(UA0ux, zero) || in_slab(b[1], a[0], -A0B0, Tba.x - aA1B0, A0B1, aA1B1 - Tba.y, -Tab.x, ctx)) &&
        (GT(LB1ly, a[1]) || in_slab(a[0], b[1], A1B1, Tab.y - a[1], A0B1, Tab.x, Tba.y - aA1B1, ctx))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x, Tba.y - aA1B1, ctx);
        C2A_EDGE_HIT(t, a[1], rect_point1(Rab, Tab, 1, u));
    }
    if (GT(LA0ux, b[0]) && LT(UB1ly, zero) &&
        (GT(LA0lx, b[0]) || in_slab(b[1], a[0], A0B0, -b[0] - Tba.x, A0B1, -Tba.y, -bA0B0 - Tab.x, ctx)) &&
        (LT(UB1uy, zero) || in_slab(a[0], b[1], -A1B1, -Tab.y - bA1B0, A0B1, Tab.x + bA0B0, Tba.y, ctx))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x + bA0B0, Tba.y, ctx);
        C2A_EDGE_HIT(t, zero, rect_point2(Rab, Tab, 0, b[0], 1, u));
    }
    if (LT(LA0lx, zero) && LT(LB1ly, zero) &&
        (LT(LA0ux, zero) || in_slab(b[1], a[0], -A0B0, Tba.x, A0B1, -Tba.y, -Tab.x, ctx)) &&
        (LT(LB1uy, zero) || in_slab(a[0], b[1], -A1B1, -Tab.y, A0B1, Tab.x, Tba.y, ctx))) {
        edge_params(t, u, a[0], b[1], A0B1, Tab.x, Tba.y, ctx);
        C2A_EDGE_HIT(t, zero, rect_point1(Rab, Tab, 1, u));
    }
    if (ctx.bad) return zero;

    T LA0ly, LA0uy, UA0ly, UA0uy, LB0ly, LB0uy, UB0ly, UB0uy;
    if (LT(ALLy, AULy)) { LA0ly = ALLy; LA0uy = AULy; UA0ly = ALUy; UA0uy = AUUy; }
    else { LA0ly = AULy; LA0uy = ALLy; UA0ly = AUUy; UA0uy = ALUy; }
    if (LT(BLLy, BULy)) { LB0ly = BLLy; LB0uy = BULy; UB0ly = BLUy; UB0uy = BUUy; }
    else { LB0ly = BULy; LB0uy = BLLy; UB0ly = BUUy; UB0uy = BLUy; }

    /* A edges along A0 against B edges along B0 */
    if (GT(UA0uy, b[1]) && GT(UB0uy, a[1]) &&
        (GT(UA0ly, b[1]) || in_slab(b[0], a[0], A0B1, aA1B1 - Tba.y - b[1], A0B0, aA1B0 - Tba.x, -Tab.x - bA0B1, ctx)) &&
        (GT(UB0ly, a[1]) || in_slab(a[0], b[0], A1B0, Tab.y - a[1] + bA1B1, A0B0, Tab.x + bA0B1, Tba.x - aA1B0, ctx))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x + bA0B1, Tba.x - aA1B0, ctx);
        C2A_EDGE_HIT(t, a[1], rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if (LT(UA0ly, zero) && GT(LB0uy, a[1]) &&
        (LT(UA0uy, zero) || in_slab(b[0], a[0], -A0B1, Tba.y - aA1B1, A0B0, aA1B0 - Tba.x, -Tab.x, ctx)) &&
        (GT(LB0ly, a[1]) || in_slab(a[0], b[0], A1B0, Tab.y - a[1], A0B0, Tab.x, Tba.x - aA1B0, ctx))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x, Tba.x - aA1B0, ctx);
        C2A_EDGE_HIT(t, a[1], rect_point1(Rab, Tab, 0, u));
    }
    if (GT(LA0uy, b[1]) && LT(UB0ly, zero) &&
        (GT(LA0ly, b[1]) || in_slab(b[0], a[0], A0B1, -Tba.y - b[1], A0B0, -Tba.x, -Tab.x - bA0B1, ctx)) &&
        (LT(UB0uy, zero) || in_slab(a[0], b[0], -A1B0, -Tab.y - bA1B1, A0B0, Tab.x + bA0B1, Tba.x, ctx))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x + bA0B1, Tba.x, ctx);
        C2A_EDGE_HIT(t, zero, rect_point2(Rab, Tab, 1, b[1], 0, u));
    }
    if (LT(LA0ly, zero) && LT(LB0ly, zero) &&
        (LT(LA0uy, zero) || in_slab(b[0], a[0], -A0B1, Tba.y, A0B0, -Tba.x, -Tab.x, ctx)) &&
        (LT(LB0uy, zero) || in_slab(a[0], b[0], -A1B0, -Tab.y, A0B0, Tab.x, Tba.x, ctx))) {
        edge_params(t, u, a[0], b[0], A0B0, Tab.x, Tba.x, ctx);
        C2A_EDGE_HIT(t, zero, rect_point1(Rab, Tab, 0, u));
    }
#undef C2A_EDGE_HIT
    if (ctx.bad) return zero;

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

/* ------------------------------------------------------------- TriDist */

/* closest points X, Y of segments P + A[0,1] and Q + B[0,1] and a direction
 * VEC separating them (C2A.cpp:59-163) */
template <class T, class C>
C2A_NOINL void seg_pair(V3T<T> &VEC, V3T<T> &X, V3T<T> &Y, V3T<T> P, V3T<T> A, V3T<T> Q, V3T<T> B, C &ctx)
{
    const T zero = K(0.0), one = K(1.0);
    V3T<T> T_ = Q - P;
    const T AA = dot(A, A), BB = dot(B, B), AB = dot(A, B), AT = dot(A, T_), BT = dot(B, T_);
    const T denom = AA * BB - AB * AB;
    T t = nan_to_zero_clamp01(num_div(AT * BB - BT * AB, denom, ctx));
    T u = num_div(t * AB - BT, BB, ctx);
    if (LE(u, zero) || is_nan(u)) {
        Y = Q;
        t = num_div(AT, AA, ctx);
        if (LE(t, zero) || is_nan(t)) {
            X = P;
            VEC = Q - P;
        } else if (GE(t, one)) {
            X = P + A;
            VEC = Q - X;
        } else {
            X = add_mul(P, A, t);
            VEC = cross(A, cross(T_, A));
        }
    } else if (GE(u, one)) {
        Y = Q + B;
        t = num_div(AB + AT, AA, ctx);
        if (LE(t, zero) || is_nan(t)) {
            X = P;
            VEC = Y - P;
        } else if (GE(t, one)) {
            X = P + A;
            VEC = Y - X;
        } else {
            X = add_mul(P, A, t);
            T_ = Y - P;
            VEC = cross(A, cross(T_, A));
        }
    } else {
        Y = add_mul(Q, B, u);
        if (LE(t, zero) || is_nan(t)) {
            X = P;
            VEC = cross(B, cross(T_, B));
        } else if (GE(t, one)) {
            X = P + A;
            T_ = Q - X;
            VEC = cross(B, cross(T_, B));
        } else {
            X = add_mul(P, A, t);
            VEC = cross(A, B);
            if (LT(dot(VEC, T_), zero)) VEC = mul_s(VEC, K(-1.0));
        }
    }
}

struct TriFeat {
    int type_a, fid_a, type_b, fid_b;
};

/*
 * Vertex of triangle T over the face of S?  Returns the vertex index (with
 * its projection Tp and the squared normal length) or -1; sets disjoint when
 * S's normal separates (C2A.cpp:268-332; the mirrored half swaps S and T).
 */
template <class T, class C>
C2A_DEV int vertex_over_face(const V3T<T> S[3], const V3T<T> Sv[3], const V3T<T> Tt[3], T &tp, T &nl, V3T<T> &n,
                             bool &disjoint, C &ctx)
{
    const T zero = K(0.0);
    const V3T<T> Sn = cross(Sv[0], Sv[1]);
    const T Snl = dot(Sn, Sn);
    if (!GT(Snl, K(1e-15))) return -1;
    T Tp[3];
    Tp[0] = dot(S[0] - Tt[0], Sn);
    Tp[1] = dot(S[0] - Tt[1], Sn);
    Tp[2] = dot(S[0] - Tt[2], Sn);
    int point = -1;
    if (GT(Tp[0], zero) && GT(Tp[1], zero) && GT(Tp[2], zero)) {
        point = LT(Tp[0], Tp[1]) ? 0 : 1;
        if (LT(Tp[2], Tp[point])) point = 2;
    } else if (LT(Tp[0], zero) && LT(Tp[1], zero) && LT(Tp[2], zero)) {
        point = GT(Tp[0], Tp[1]) ? 0 : 1;
        if (GT(Tp[2], Tp[point])) point = 2;
    }
    if (point < 0) return -1;
    disjoint = true;
#pragma unroll
    for (int e = 0; e < 3; e++)
        if (!GT(dot(Tt[point] - S[e], cross(Sn, Sv[e])), zero)) return -1;
    tp = Tp[point];
    nl = Snl;
    n = Sn;
    return point;
}

/* distance between triangles S and T (same frame), closest points P, Q,
 * features; collided set on overlap (C2A.cpp:165-405) */
template <class T, class C>
C2A_NOINL T tri_dist(V3T<T> &P, V3T<T> &Q, const V3T<T> S[3], const V3T<T> Tt[3], TriFeat &f, bool &collided, C &ctx)
{
    const T zero = K(0.0);
    V3T<T> Sv[3], Tv[3];
    Sv[0] = S[1] - S[0];
    Sv[1] = S[2] - S[1];
    Sv[2] = S[0] - S[2];
    Tv[0] = Tt[1] - Tt[0];
    Tv[1] = Tt[2] - Tt[1];
    Tv[2] = Tt[0] - Tt[2];
    V3T<T> minP = v3t(zero, zero, zero), minQ = minP, VEC;
    T mindd = dist2(S[0], Tt[0]) + K(1.0);
    bool shown_disjoint = false;
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
#pragma unroll 1
        for (int j = 0; j < 3; j++) {
            seg_pair(VEC, P, Q, S[i], Sv[i], Tt[j], Tv[j], ctx);
            if (ctx.bad) return zero;
            const V3T<T> V = Q - P;
            const T dd = dot(V, V);
            if (LE(dd, mindd)) {
                minP = P;
                minQ = Q;
                mindd = dd;
                f.type_a = 1;
                f.fid_a = i;
                f.type_b = 1;
                f.fid_b = j;
                T a = dot(S[(i + 2) % 3] - P, VEC);
                T b = dot(Tt[(j + 2) % 3] - Q, VEC);
                if (LE(a, zero) && GE(b, zero)) return num_sqrt(dd);
                const T p = dot(V, VEC);
                a = max0_c(a);
                b = min0_c(b);
                if (GT(p - a + b, zero)) shown_disjoint = true;
            }
        }
    }
    if (ctx.bad) return zero;
    T tp, nl;
    V3T<T> n;
    int point = vertex_over_face(S, Sv, Tt, tp, nl, n, shown_disjoint, ctx);
    if (point >= 0) {
        f.type_a = 2;
        f.fid_a = -1;
        f.type_b = 0;
        f.fid_b = point;
        P = add_mul(Tt[point], n, num_div(tp, nl, ctx));
        Q = Tt[point];
        return num_sqrt(dist2(P, Q));
    }
    point = vertex_over_face(Tt, Tv, S, tp, nl, n, shown_disjoint, ctx);
    if (point >= 0) {
        f.type_a = 0;
        f.fid_a = point;
        f.type_b = 2;
        f.fid_b = -1;
        P = S[point];
        Q = add_mul(S[point], n, num_div(tp, nl, ctx));
        return num_sqrt(dist2(P, Q));
    }
    if (shown_disjoint) {
        P = minP;
        Q = minQ;
        return num_sqrt(mindd);
    }
    collided = true;
    return zero;
}

/* --------------------------------------------------------- motion bounds */

/* the velocity constants of one linear motion in number type T */
template <class T> struct MotionT {
    T cv[3], axis[3], w;
    bool w_zero; /* m_angVel == 0 exactly */
};
template <class T, class C> C2A_DEV MotionT<T> motion_t(const Motion &m, C &ctx)
{
    MotionT<T> r;
    for (int i = 0; i < 3; i++) {
        r.cv[i] = in_d(m.cv[i], ctx);
        r.axis[i] = in_d(m.axis[i], ctx);
    }
    r.w = in_d(m.angVel, ctx);
    r.w_zero = (m.angVel == 0);
    return r;
}

/* computeTOC(d, r1, S) at a leaf; S is normalised in place */
template <class T, class C> C2A_DEV T bound_leaf(const MotionT<T> &m, T r1, V3T<T> &S, C &ctx)
{
    const T zero = K(0.0);
    S = normalized(S, ctx);
    T w_max, v_max;
    if (m.w_zero) {
        w_max = zero;
        v_max = max0_c(m.cv[0] * S.x + m.cv[1] * S.y + m.cv[2] * S.z);
    } else {
        const V3T<T> cwc = v3t(m.axis[0] * m.w, m.axis[1] * m.w, m.axis[2] * m.w);
        w_max = r1 * length(cross(cwc, S));
        v_max = max0_c(m.cv[0] * S.x + m.cv[1] * S.y + m.cv[2] * S.z);
    }
    T path_max = w_max + v_max;
    if (EQ0(path_max)) path_max = K(1e-30);
    return path_max;
}

/* computeTOC_MotionBound for an RSS of angular radius angR; N normalised in place */
template <class T, class C> C2A_DEV T bound_rss(const MotionT<T> &m, T angR, V3T<T> &N, C &ctx)
{
    const T zero = K(0.0);
    N = normalized(N, ctx);
    const V3T<T> c = cross(v3t(m.axis[0], m.axis[1], m.axis[2]), N);
    const T w_max = angR * length(c) * m.w;
    const T v_max = max0_c(m.cv[0] * N.x + m.cv[1] * N.y + m.cv[2] * N.z);
    T path_max = v_max + w_max;
    if (LE(path_max, zero)) path_max = K(1e-30);
    return path_max;
}

} // namespace c2a
#endif
