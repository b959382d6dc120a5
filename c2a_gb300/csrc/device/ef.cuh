/*
 * ef.cuh -- FP32 values with a certified bound on their distance to the FP64
 * result of the same expression.
 *
 * An EF {v, e} stands for a quantity x64 that the FP64 code computes with
 * the same expression tree (same operands, same association): |v - x64| <= e.
 * Each operation rounds its value to nearest in FP32 and propagates e with
 * directed (upward) rounding:
 *
 *   x +- y:  e = s + U (|v| + s),            s = ex + ey
 *   x * y:   e = s + U (|v| + s),            s = |vx| ey + |vy| ex + ex ey
 *   x / y:   e = s + U (|v| + s),            s = (ex + |v|(1+2^-22) ey) / (|vy| - ey),  needs |vy| > ey
 *   sqrt x:  e = s + U (|v| + s),            s = ex / (sqrt(vx) + sqrt(vx - ex)), or sqrt(vx + ex) when vx <= ex
 *
 * with U = 2^-24 (1 + 2^-20): it covers the FP32 rounding of v, the FP64
 * rounding of x64 (2^-53 relative) and the FP32 slack of the bound itself.
 * A product or quotient whose FP32 value lies below 2^-126 adds 2^-149 for
 * gradual underflow (it may be off by up to 2^-150 absolutely; sums that
 * underflow are exact) -- unless an operand is an exact zero, whose product
 * is an exact zero in both precisions.  A bound that overflows becomes inf or NaN, and every comparison
 * with such a bound is undecided.
 * Comparisons are three-valued: a decision the bounds cannot settle is
 * reported, and the caller then recomputes exactly in FP64.  Clamps, max and
 * |x| are 1-Lipschitz, so they carry e through without a decision.
 */
#ifndef C2A_EF_CUH
#define C2A_EF_CUH

#include <cmath>
#include <cstdint>
#include <cstring>

/* Device code uses the hardware's directed roundings.  The host build (for
 * the CPU soundness test of the filter) derives the same directed roundings
 * from double arithmetic and an exactness check. */
#if defined(__CUDACC__)
#define C2A_EFI __host__ __device__ __forceinline__
#else
#define C2A_EFI inline
#endif

namespace c2a {

#if defined(__CUDA_ARCH__)
C2A_EFI float efr_add_ru(float a, float b) { return __fadd_ru(a, b); }
C2A_EFI float efr_add_rd(float a, float b) { return __fadd_rd(a, b); }
C2A_EFI float efr_sub_rd(float a, float b) { return __fsub_rd(a, b); }
C2A_EFI float efr_mul_ru(float a, float b) { return __fmul_ru(a, b); }
C2A_EFI float efr_div_ru(float a, float b) { return __fdiv_ru(a, b); }
C2A_EFI float efr_fma_ru(float a, float b, float c) { return __fmaf_ru(a, b, c); }
C2A_EFI float efr_sqrt_rd(float a) { return __fsqrt_rd(a); }
C2A_EFI float efr_sqrt_ru(float a) { return __fsqrt_ru(a); }
C2A_EFI float efr_d2f(double x) { return __double2float_rn(x); }
#else
/* host: directed roundings of exact float results, from round-to-nearest
 * double arithmetic and an exactness check of each double result */
inline float efr_up_from(double x, double err) /* exact value = x + err */
{
    float f = (float)x;
    if ((double)f < x || ((double)f == x && err > 0)) f = std::nextafter(f, INFINITY);
    return f;
}
inline float efr_dn_from(double x, double err)
{
    float f = (float)x;
    if ((double)f > x || ((double)f == x && err < 0)) f = std::nextafter(f, -INFINITY);
    return f;
}
inline double efr_two_sum(double a, double b, double &err) /* Knuth's TwoSum */
{
    const double s = a + b, bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}
inline float efr_add_ru(float a, float b) { double e; const double s = efr_two_sum(a, b, e); return efr_up_from(s, e); }
inline float efr_add_rd(float a, float b) { double e; const double s = efr_two_sum(a, b, e); return efr_dn_from(s, e); }
inline float efr_sub_rd(float a, float b) { return efr_add_rd(a, -b); }
inline float efr_mul_ru(float a, float b) { return efr_up_from((double)a * (double)b, 0.0); } /* exact in double */
inline float efr_fma_ru(float a, float b, float c)
{
    double e;
    const double s = efr_two_sum((double)a * (double)b, c, e);
    return efr_up_from(s, e);
}
inline float efr_div_ru(float a, float b)
{
    const double q = (double)a / (double)b;
    const double r = std::fma(-q, (double)b, (double)a); /* a - q b, exact */
    return efr_up_from(q, b > 0 ? r : -r);
}
inline float efr_sqrt_ru(float a)
{
    const double s = std::sqrt((double)a);
    return efr_up_from(s, (double)a - s * s > 0 ? 1.0 : (s * s > (double)a ? -1.0 : 0.0));
}
inline float efr_sqrt_rd(float a)
{
    const double s = std::sqrt((double)a);
    return efr_dn_from(s, (double)a - s * s > 0 ? 1.0 : (s * s > (double)a ? -1.0 : 0.0));
}
inline float efr_d2f(double x) { return (float)x; }
#endif

struct EF {
    float v, e;
};

#define C2A_EF_U 5.9604710e-08f /* >= 2^-24 (1 + 2^-20) */

C2A_EFI float ef_ru_add(float a, float b) { return efr_add_ru(a, b); }
C2A_EFI float ef_ru_mul(float a, float b) { return efr_mul_ru(a, b); }
C2A_EFI float ef_rd_sub(float a, float b) { return efr_sub_rd(a, b); }

#define C2A_EF_TINY 1.40129846e-45f   /* 2^-149 */
#define C2A_EF_NORMAL 1.17549435e-38f /* 2^-126, FP32's smallest normal */

/* total bound after a fresh rounding of v, given the propagated input bound s:
 * s + U (|v| + s), one upward-rounded fused multiply-add */
C2A_EFI float ef_round_err(float v, float s)
{
    return efr_fma_ru(C2A_EF_U, ef_ru_add(fabsf(v), s), s);
}

/* max of two bounds that keeps a NaN (fmaxf would drop it) */
C2A_EFI float ef_emax(float a, float b)
{
    return (a != a || b != b) ? a + b : fmaxf(a, b);
}

/* an FP64 value rounded to FP32: |v - x| <= 2^-24 |v| for normal v, exact 0 stays exact */
C2A_EFI EF ef_of(double x)
{
    const float v = efr_d2f(x);
    return EF{v, ef_ru_mul(fabsf(v), C2A_EF_U)};
}
/* a value already held in FP32 from an FP64 source (node/triangle shadows) */
C2A_EFI EF ef_shadow(float v) { return EF{v, ef_ru_mul(fabsf(v), C2A_EF_U)}; }
/* a value exactly representable in FP32 */
C2A_EFI EF ef_exact(float v) { return EF{v, 0.0f}; }

C2A_EFI EF operator+(EF a, EF b)
{
    const float v = a.v + b.v;
    return EF{v, ef_round_err(v, ef_ru_add(a.e, b.e))};
}
C2A_EFI EF operator-(EF a, EF b)
{
    const float v = a.v - b.v;
    return EF{v, ef_round_err(v, ef_ru_add(a.e, b.e))};
}
C2A_EFI EF operator-(EF a) { return EF{-a.v, a.e}; }
C2A_EFI bool ef_is_exact_zero(EF a) { return a.v == 0.0f && a.e == 0.0f; }
C2A_EFI EF operator*(EF a, EF b)
{
    const float v = a.v * b.v;
    float s = ef_ru_add(ef_ru_add(ef_ru_mul(fabsf(a.v), b.e), ef_ru_mul(fabsf(b.v), a.e)), ef_ru_mul(a.e, b.e));
    if (fabsf(v) < C2A_EF_NORMAL && !ef_is_exact_zero(a) && !ef_is_exact_zero(b)) s = ef_ru_add(s, C2A_EF_TINY);
    return EF{v, ef_round_err(v, s)};
}

/* set when a division or a decision could not be certified; the host test
 * build also records the source line of the first failure */
struct EFCtx {
    bool bad;
#ifdef C2A_EF_WHERE
    int where = 0;
#endif
};
#ifdef C2A_EF_WHERE
#define C2A_EF_FAIL(c, line) ((c).bad = true, (c).where = (c).where ? (c).where : (line))
#else
#define C2A_EF_FAIL(c, line) ((c).bad = true)
#endif

/* Device fast paths of the quotient and the square root.  They use CUDA's
 * approximate intrinsics within their documented accuracy: __fdividef(x, y)
 * is within 2 ulp of x / y for 2^-126 <= |y| <= 2^126, rsqrtf(x) within 2
 * ulp of 1 / sqrt(x).  Each approximation error enters e with a margin
 * (2^-21 relative, i.e. 4 ulp), and the propagated part is rounded upwards
 * through an inflation by 1 + 2^-20; outside the guarded ranges the exact
 * directed-rounding forms below are used. */
#if defined(__CUDA_ARCH__) && !defined(C2A_EF_PRECISE)
#define C2A_EF_FAST 1
#define C2A_EF_ULP4 4.76837158e-07f  /* 2^-21 */
#define C2A_EF_INFL 1.00000095f      /* 1 + 2^-20 */
#define C2A_EF_DEFL 0.99999905f      /* 1 - 2^-20 */
C2A_EFI bool ef_fast_range(float x) { return fabsf(x) >= 1.0e-30f && fabsf(x) <= 1.0e30f; }
#endif

C2A_EFI EF ef_div(EF a, EF b, EFCtx &c)
{
    const float den = ef_rd_sub(fabsf(b.v), b.e);
    if (!(den > 0.0f)) {
        C2A_EF_FAIL(c, __LINE__);
        return EF{0.0f, 0.0f};
    }
#ifdef C2A_EF_FAST
    if (ef_fast_range(b.v) && ef_fast_range(den) && fabsf(a.v) <= 1.0e30f && a.e <= 1.0e30f) {
        const float v = __fdividef(a.v, b.v);
        if (a.v == 0.0f || ef_fast_range(v)) {
            /* |a.v / b.v| <= |v| (1 + 2^-21) */
            const float num = ef_ru_add(a.e, ef_ru_mul(ef_ru_mul(fabsf(v), 1.00000048f), b.e));
            float s = __fmul_ru(__fdividef(num, den), C2A_EF_INFL);
            s = ef_ru_add(s, ef_ru_mul(fabsf(v), C2A_EF_ULP4));
            if (s == s && s <= 1.0e30f) return EF{v, ef_round_err(v, s)};
        }
    }
#endif
    const float v = a.v / b.v;
    const float num = ef_ru_add(a.e, ef_ru_mul(ef_ru_mul(fabsf(v), 1.00000024f), b.e));
    float s = efr_div_ru(num, den);
    if (fabsf(v) < C2A_EF_NORMAL && !ef_is_exact_zero(a)) s = ef_ru_add(s, C2A_EF_TINY);
    return EF{v, ef_round_err(v, s)};
}

C2A_EFI EF ef_sqrt(EF a)
{
    const float x = a.v > 0.0f ? a.v : 0.0f;
#ifdef C2A_EF_FAST
    if ((x == 0.0f || ef_fast_range(x)) && a.e <= 1.0e30f) {
        const float v = x == 0.0f ? 0.0f : x * rsqrtf(x); /* within 2.5 ulp of sqrt(x) */
        const float lo = ef_rd_sub(a.v, a.e);
        float s;
        if (lo > 0.0f && ef_fast_range(lo)) { /* e / (sqrt(x) + sqrt(lo)) */
            const float den = __fmul_rd(efr_add_rd(v, lo * rsqrtf(lo)), 0.9999981f);
            s = __fmul_ru(__fdividef(a.e, den), C2A_EF_INFL);
        } else { /* sqrt(x + e) */
            const float t = ef_ru_add(x, a.e);
            s = t == 0.0f ? 0.0f : __fmul_ru(t * rsqrtf(t), 1.0000019f);
        }
        s = ef_ru_add(s, ef_ru_mul(v, C2A_EF_ULP4));
        if (s == s && s <= 1.0e30f) return EF{v, ef_round_err(v, s)};
    }
#endif
    const float v = sqrtf(x);
    const float lo = ef_rd_sub(a.v, a.e);
    float s;
    if (lo > 0.0f) s = efr_div_ru(a.e, efr_add_rd(efr_sqrt_rd(x), efr_sqrt_rd(lo)));
    else s = efr_sqrt_ru(ef_ru_add(x, a.e));
    return EF{v, ef_round_err(v, s)};
}

C2A_EFI EF ef_abs(EF a) { return EF{fabsf(a.v), a.e}; }
C2A_EFI EF ef_max0(EF a) { return EF{a.v > 0.0f ? a.v : 0.0f, a.e}; }
/* if (x < lo) x = lo; else if (x > hi) x = hi.  Where the FP64 comparisons
 * are certain, the FP64 result is exactly that bound or x, so the result
 * carries that operand's own error (an exact bound stays exact, and later
 * comparisons against it decide); otherwise every operand's error. */
C2A_EFI EF ef_clamp(EF x, EF lo, EF hi)
{
    const float xl = ef_rd_sub(x.v, x.e), xh = ef_ru_add(x.v, x.e);
    if (xh < ef_rd_sub(lo.v, lo.e)) return lo;                                 /* x < lo certainly */
    if (xl >= ef_ru_add(lo.v, lo.e) && xl > ef_ru_add(hi.v, hi.e)) return hi; /* not below lo, above hi */
    float v = x.v < lo.v ? lo.v : x.v;
    v = v > hi.v ? hi.v : v;
    return EF{v, ef_emax(x.e, ef_emax(lo.e, hi.e))};
}

/* three-valued comparisons: 1 true, 0 false, -1 undecided */
C2A_EFI int ef_lt3(EF a, EF b)
{
    if (ef_ru_add(a.v, a.e) < ef_rd_sub(b.v, b.e)) return 1;
    if (ef_rd_sub(a.v, a.e) >= ef_ru_add(b.v, b.e)) return 0;
    return -1;
}
C2A_EFI int ef_le3(EF a, EF b)
{
    if (ef_ru_add(a.v, a.e) <= ef_rd_sub(b.v, b.e)) return 1;
    if (ef_rd_sub(a.v, a.e) > ef_ru_add(b.v, b.e)) return 0;
    return -1;
}

} // namespace c2a
#endif
