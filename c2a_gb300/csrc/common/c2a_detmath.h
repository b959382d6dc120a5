/*
 * c2a_detmath.h -- deterministic sin, cos and acos for the CA motion model.
 *
 * The linear motion of C2A evaluates sin/cos on every CA iteration
 * (C2A/src/InterpMotion.cpp:273-279, DeltaRt) and acos once per query
 * (InterpMotion.cpp:251, LinearAngularVelocity).  The platform libm differs
 * between x86-64 glibc (FMA ifunc variants), aarch64 glibc and CUDA, so the
 * same query could take different ulp-level poses on each of them.  Every
 * implementation in this project (CUDA kernels, host library, CPU oracle)
 * calls these functions instead, so poses agree bit for bit everywhere.
 *
 * Method: double-double arithmetic (Dekker 1971 splitting and product,
 * Knuth TwoSum), Taylor series of sin/cos around 0 after folding the argument
 * into [-pi/4, pi/4] with a double-double pi/2, and Newton iteration on
 * cos(y) = x for acos.  The double-double result carries ~100 bits, so its
 * rounding to double is the correctly rounded value except for arguments
 * within ~1e-30 of a rounding midpoint.  Only IEEE add/sub/mul/div/sqrt are
 * used; build with FP contraction off (-ffp-contract=off, nvcc --fmad=false).
 *
 * Header-only; compiles as C99, C++ and CUDA (host and device).
 */
#ifndef C2A_DETMATH_H
#define C2A_DETMATH_H

#include <math.h>

#if defined(__CUDACC__)
#define C2A_DM_FN static __host__ __device__ __forceinline__
#else
#define C2A_DM_FN static inline
#endif

typedef struct { double hi, lo; } c2a_dd;

/* Knuth's TwoSum: s + e == a + b exactly. */
C2A_DM_FN c2a_dd c2a_dd_two_sum(double a, double b)
{
    c2a_dd r;
    double s = a + b;
    double bb = s - a;
    r.hi = s;
    r.lo = (a - (s - bb)) + (b - bb);
    return r;
}

/* Fast TwoSum, requires |a| >= |b| or a == 0. */
C2A_DM_FN c2a_dd c2a_dd_fast_sum(double a, double b)
{
    c2a_dd r;
    double s = a + b;
    r.hi = s;
    r.lo = b - (s - a);
    return r;
}

/* Dekker's product: p + e == a * b exactly (no FMA needed). */
C2A_DM_FN c2a_dd c2a_dd_two_prod(double a, double b)
{
    const double split = 134217729.0; /* 2^27 + 1 */
    double p = a * b;
    double ta = split * a, tb = split * b;
    double ah = ta - (ta - a), al = a - ah;
    double bh = tb - (tb - b), bl = b - bh;
    c2a_dd r;
    r.hi = p;
    r.lo = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
    return r;
}

C2A_DM_FN c2a_dd c2a_dd_make(double hi, double lo)
{
    return c2a_dd_fast_sum(hi, lo);
}

C2A_DM_FN c2a_dd c2a_dd_add(c2a_dd x, c2a_dd y)
{
    c2a_dd s = c2a_dd_two_sum(x.hi, y.hi);
    c2a_dd t = c2a_dd_two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = c2a_dd_fast_sum(s.hi, s.lo);
    s.lo += t.lo;
    return c2a_dd_fast_sum(s.hi, s.lo);
}

C2A_DM_FN c2a_dd c2a_dd_neg(c2a_dd x)
{
    c2a_dd r;
    r.hi = -x.hi;
    r.lo = -x.lo;
    return r;
}

C2A_DM_FN c2a_dd c2a_dd_sub(c2a_dd x, c2a_dd y)
{
    return c2a_dd_add(x, c2a_dd_neg(y));
}

C2A_DM_FN c2a_dd c2a_dd_mul(c2a_dd x, c2a_dd y)
{
    c2a_dd p = c2a_dd_two_prod(x.hi, y.hi);
    p.lo += x.hi * y.lo + x.lo * y.hi;
    return c2a_dd_fast_sum(p.hi, p.lo);
}

/* x / d for a double d (long division, one correction step). */
C2A_DM_FN c2a_dd c2a_dd_div_d(c2a_dd x, double d)
{
    double q1 = x.hi / d;
    c2a_dd p = c2a_dd_two_prod(q1, d);
    c2a_dd r = c2a_dd_two_sum(x.hi, -p.hi);
    r.lo -= p.lo;
    r.lo += x.lo;
    double q2 = (r.hi + r.lo) / d;
    return c2a_dd_fast_sum(q1, q2);
}

C2A_DM_FN c2a_dd c2a_dd_div(c2a_dd x, c2a_dd y)
{
    double q1 = x.hi / y.hi;
    c2a_dd r = c2a_dd_sub(x, c2a_dd_mul(y, c2a_dd_make(q1, 0.0)));
    double q2 = r.hi / y.hi;
    r = c2a_dd_sub(r, c2a_dd_mul(y, c2a_dd_make(q2, 0.0)));
    double q3 = r.hi / y.hi;
    c2a_dd q = c2a_dd_fast_sum(q1, q2);
    return c2a_dd_add(q, c2a_dd_make(q3, 0.0));
}

/* pi/2 and pi/4 as double-double (hi = nearest double, lo = remainder). */
#define C2A_DD_PIO2_HI 1.5707963267948966192e+00
#define C2A_DD_PIO2_LO 6.1232339957367658e-17
#define C2A_DD_PIO4_HI 7.8539816339744830962e-01
#define C2A_DD_PIO4_LO 3.0616169978683829e-17

/*
 * Taylor sums for |y| <= pi/4 (+ a little):
 *   sin y = y * (1 - y^2/(2*3) * (1 - y^2/(4*5) * (1 - ...)))
 *   cos y = 1 - y^2/(1*2) * (1 - y^2/(3*4) * (1 - ...))
 * 15 nested factors: the last neglected term is below 1e-33 relative.
 */
C2A_DM_FN c2a_dd c2a_dd_sin_taylor(c2a_dd y)
{
    c2a_dd y2 = c2a_dd_mul(y, y);
    c2a_dd acc = c2a_dd_make(1.0, 0.0);
    int k;
    for (k = 15; k >= 1; --k) {
        double den = (double)(2 * k) * (double)(2 * k + 1);
        c2a_dd t = c2a_dd_div_d(c2a_dd_mul(y2, acc), den);
        acc = c2a_dd_sub(c2a_dd_make(1.0, 0.0), t);
    }
    return c2a_dd_mul(y, acc);
}

C2A_DM_FN c2a_dd c2a_dd_cos_taylor(c2a_dd y)
{
    c2a_dd y2 = c2a_dd_mul(y, y);
    c2a_dd acc = c2a_dd_make(1.0, 0.0);
    int k;
    for (k = 15; k >= 1; --k) {
        double den = (double)(2 * k - 1) * (double)(2 * k);
        c2a_dd t = c2a_dd_div_d(c2a_dd_mul(y2, acc), den);
        acc = c2a_dd_sub(c2a_dd_make(1.0, 0.0), t);
    }
    return acc;
}

/*
 * sin and cos of a double-double argument with |x| <= 4*pi (the CA motion
 * only needs [0, pi/2]).  Quadrant reduction by a double-double pi/2, then a
 * fold at pi/4.
 */
C2A_DM_FN void c2a_dd_sincos(c2a_dd x, c2a_dd *s, c2a_dd *c)
{
    const c2a_dd pio2 = {C2A_DD_PIO2_HI, C2A_DD_PIO2_LO};
    const c2a_dd pio4 = {C2A_DD_PIO4_HI, C2A_DD_PIO4_LO};
    double kq = floor(x.hi / C2A_DD_PIO2_HI + 0.5);
    int q = (int)kq;
    c2a_dd r = c2a_dd_sub(x, c2a_dd_mul(pio2, c2a_dd_make(kq, 0.0)));
    c2a_dd sr, cr;
    /* r in about [-pi/4, pi/4]; fold the rare overshoot */
    if (r.hi > pio4.hi) {
        c2a_dd u = c2a_dd_sub(pio2, r);
        sr = c2a_dd_cos_taylor(u);
        cr = c2a_dd_sin_taylor(u);
    } else if (r.hi < -pio4.hi) {
        c2a_dd u = c2a_dd_add(pio2, r);
        sr = c2a_dd_neg(c2a_dd_cos_taylor(u));
        cr = c2a_dd_sin_taylor(u);
    } else {
        sr = c2a_dd_sin_taylor(r);
        cr = c2a_dd_cos_taylor(r);
    }
    switch (((q % 4) + 4) % 4) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = c2a_dd_neg(sr); break;
    case 2: *s = c2a_dd_neg(sr); *c = c2a_dd_neg(cr); break;
    default: *s = c2a_dd_neg(cr); *c = sr; break;
    }
}

C2A_DM_FN double c2a_det_sin(double x)
{
    if (x != x) return x;
    if (x == 0.0) return x; /* keeps the sign of zero */
    if (!(fabs(x) <= 12.566370614359172)) return (x - x) / (x - x); /* outside the supported range */
    c2a_dd s, c;
    c2a_dd_sincos(c2a_dd_make(x, 0.0), &s, &c);
    return s.hi + s.lo;
}

C2A_DM_FN double c2a_det_cos(double x)
{
    if (x != x) return x;
    if (!(fabs(x) <= 12.566370614359172)) return (x - x) / (x - x);
    c2a_dd s, c;
    c2a_dd_sincos(c2a_dd_make(x, 0.0), &s, &c);
    return c.hi + c.lo;
}

/*
 * acos(x) for x in [-1, 1]: NaN outside (as libm), exact endpoints, otherwise
 * Newton iteration y <- y + (cos y - x) / sin y in double-double, started from
 * atan2(sqrt(1 - x^2), x).  Three steps take any start within 1e-8 to the
 * double-double fixed point, so the answer does not depend on the host's atan2.
 */
C2A_DM_FN double c2a_det_acos(double x)
{
    if (x != x) return x;
    if (x > 1.0 || x < -1.0) return (x - x) / (x - x);
    if (x == 1.0) return 0.0;
    if (x == -1.0) return 2.0 * C2A_DD_PIO2_HI;
    c2a_dd y = c2a_dd_make(atan2(sqrt((1.0 - x) * (1.0 + x)), x), 0.0);
    int it;
    for (it = 0; it < 3; ++it) {
        c2a_dd s, c;
        c2a_dd_sincos(y, &s, &c);
        c2a_dd f = c2a_dd_sub(c, c2a_dd_make(x, 0.0));
        if (s.hi == 0.0) break;
        y = c2a_dd_add(y, c2a_dd_div(f, s));
    }
    return y.hi + y.lo;
}

#endif /* C2A_DETMATH_H */
