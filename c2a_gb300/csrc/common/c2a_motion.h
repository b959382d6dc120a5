/*
 * c2a_motion.h -- C2A's linear interpolating motion (CInterpMotion_Linear),
 * compiled for both the host library and the CUDA kernels.
 *
 *   setup:     cv = T1 - T0; body-frame axis/angle of q0^-1 q1
 *              (C2A/src/InterpMotion.cpp:148-168, 228-270, 486-502)
 *   integrate: T(t) = T0 + cv t; R(t) = R0 * dR(t) via quaternions
 *              (InterpMotion.cpp:273-287, 516-568)
 *   quaternion <-> matrix and product: C2A/LinearMath.h:759-829, 1018-1025
 *
 * Every expression keeps the reference's evaluation order; sin/cos/acos are
 * the deterministic ones of c2a_detmath.h.  Build without FP contraction.
 */
#ifndef C2A_MOTION_H
#define C2A_MOTION_H

#include "c2a_detmath.h"

#if defined(__CUDACC__)
#define C2A_HD __host__ __device__ __forceinline__
#else
#define C2A_HD inline
#endif

namespace c2a {

/* Linear motion of one object.  q0 is (x, y, z, w). */
struct Motion {
    double R0[9], T0[3];
    double q0[4];
    double cv[3];
    double axis[3];
    double angVel;
};

/* Matrix3x3::Quaternion_ (LinearMath.h:759-794), m row-major */
C2A_HD void mat_to_quat(double q[4], const double *v)
{
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
        double qq[3];
        qq[i] = s * 0.5;
        s = 0.5 / s;
        q[3] = (v[k * 3 + j] - v[j * 3 + k]) * s;
        qq[j] = (v[j * 3 + i] + v[i * 3 + j]) * s;
        qq[k] = (v[k * 3 + i] + v[i * 3 + k]) * s;
        q[0] = qq[0];
        q[1] = qq[1];
        q[2] = qq[2];
    }
}

/* quaternion product a % b (LinearMath.h:1018-1025) */
C2A_HD void quat_mul(double r[4], const double a[4], const double b[4])
{
    double x = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    double y = a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2];
    double z = a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0];
    double w = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
    r[0] = x;
    r[1] = y;
    r[2] = z;
    r[3] = w;
}

/* Matrix3x3::Set_Value(Quaternion) (LinearMath.h:809-829), m row-major */
C2A_HD void quat_to_mat(double m[9], const double q[4])
{
    double d = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    double s = 2.0 / d;
    double xs = q[0] * s, ys = q[1] * s, zs = q[2] * s;
    double wx = q[3] * xs, wy = q[3] * ys, wz = q[3] * zs;
    double xx = q[0] * xs, xy = q[0] * ys, xz = q[0] * zs;
    double yy = q[1] * ys, yz = q[1] * zs, zz = q[2] * zs;
    m[0] = 1.0 - (yy + zz);
    m[1] = xy - wz;
    m[2] = xz + wy;
    m[3] = xy + wz;
    m[4] = 1.0 - (xx + zz);
    m[5] = yz - wx;
    m[6] = xz - wy;
    m[7] = yz + wx;
    m[8] = 1.0 - (xx + yy);
}

/* CInterpMotion_Linear(R0, T0, R1, T1): velocity() with LinearAngularVelocity */
C2A_HD void motion_setup(Motion &m, const double *R0, const double *T0, const double *R1, const double *T1)
{
    double qs[4], qt[4], sq0[4], st[4];
    for (int i = 0; i < 9; i++) m.R0[i] = R0[i];
    for (int i = 0; i < 3; i++) {
        m.T0[i] = T0[i];
        m.cv[i] = T1[i] - T0[i];
    }
    mat_to_quat(qs, R0);
    mat_to_quat(qt, R1);
    sq0[0] = -qs[0];
    sq0[1] = -qs[1];
    sq0[2] = -qs[2];
    sq0[3] = qs[3];
    quat_mul(st, sq0, qt);
    double s = 1 < st[3] ? 1 : st[3];
    double sign = s < 0 ? -1 : 1;
    double a = (fabs(s - 1) <= 1e-40 || fabs(s + 1) <= 1e-40) ? (2 * sign)
                                                             : (sign * c2a_det_acos(2 * s * s - 1) / sqrt(1 - s * s));
    double t0 = a * st[0], t1 = a * st[1], t2 = a * st[2];
    m.axis[0] = t0;
    m.axis[1] = t1;
    m.axis[2] = t2;
    m.angVel = sqrt(t0 * t0 + t1 * t1 + t2 * t2);
    double len = m.axis[0] * m.axis[0] + m.axis[1] * m.axis[1] + m.axis[2] * m.axis[2];
    if (len < (double)0.00000001f) {
        m.axis[0] = 1.0;
        m.axis[1] = 0.0;
        m.axis[2] = 0.0;
    } else {
        double inv = 1.0 / sqrt(len);
        m.axis[0] *= inv;
        m.axis[1] *= inv;
        m.axis[2] *= inv;
    }
    mat_to_quat(m.q0, R0);
}

/* integrate(dt): R (row-major), T; orn = the quaternion (x, y, z, w) */
C2A_HD void motion_integrate(const Motion &m, double dt, double R[9], double T[3], double orn[4])
{
    if (dt > 1) dt = 1;
    T[0] = m.T0[0] + dt * m.cv[0];
    T[1] = m.T0[1] + dt * m.cv[1];
    T[2] = m.T0[2] + dt * m.cv[2];
    double ang = 0.5 * m.angVel * dt;
    double sa = c2a_det_sin(ang);
    double drt[4];
    drt[0] = sa * m.axis[0];
    drt[1] = sa * m.axis[1];
    drt[2] = sa * m.axis[2];
    drt[3] = c2a_det_cos(ang);
    quat_mul(orn, m.q0, drt);
    quat_to_mat(R, orn);
}

} // namespace c2a
#endif
