/*
 * c2a_port_matvec.h -- 3-vector / 3x3 helpers of the oracle port.  Each one
 * evaluates left to right in the order the PQP-interface helpers use
 * (oracle/pqp_shim/MatVec.h), e.g. MxVpV row i = ((m0*v0 + m1*v1) + m2*v2) + w.
 * Test infrastructure only.
 */
#ifndef C2A_PORT_MATVEC_H
#define C2A_PORT_MATVEC_H
#include <math.h>

typedef double pm3[3][3];

static inline void pv_copy(double r[3], const double v[3]) { r[0] = v[0]; r[1] = v[1]; r[2] = v[2]; }
static inline void pm_copy(double r[3][3], const double m[3][3])
{
    int i, j;
    for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) r[i][j] = m[i][j];
}
static inline void pv_sub(double r[3], const double a[3], const double b[3])
{
    r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
}
static inline void pv_add(double r[3], const double a[3], const double b[3])
{
    r[0] = a[0] + b[0]; r[1] = a[1] + b[1]; r[2] = a[2] + b[2];
}
/* r = a + b * s */
static inline void pv_add_scaled(double r[3], const double a[3], const double b[3], double s)
{
    r[0] = a[0] + b[0] * s; r[1] = a[1] + b[1] * s; r[2] = a[2] + b[2] * s;
}
static inline void pv_scale(double r[3], const double v[3], double s)
{
    r[0] = v[0] * s; r[1] = v[1] * s; r[2] = v[2] * s;
}
static inline double pv_dot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void pv_cross(double r[3], const double a[3], const double b[3])
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double pv_len(const double v[3]) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static inline void pv_normalize(double v[3])
{
    double d = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= d; v[1] *= d; v[2] *= d;
}
static inline double pv_dist2(const double a[3], const double b[3])
{
    return (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
}
/* r = M v */
static inline void pm_mul_v(double r[3], const double m[3][3], const double v[3])
{
    r[0] = m[0][0] * v[0] + m[0][1] * v[1] + m[0][2] * v[2];
    r[1] = m[1][0] * v[0] + m[1][1] * v[1] + m[1][2] * v[2];
    r[2] = m[2][0] * v[0] + m[2][1] * v[1] + m[2][2] * v[2];
}
/* r = M v + w */
static inline void pm_mul_v_add(double r[3], const double m[3][3], const double v[3], const double w[3])
{
    r[0] = m[0][0] * v[0] + m[0][1] * v[1] + m[0][2] * v[2] + w[0];
    r[1] = m[1][0] * v[0] + m[1][1] * v[1] + m[1][2] * v[2] + w[1];
    r[2] = m[2][0] * v[0] + m[2][1] * v[1] + m[2][2] * v[2] + w[2];
}
/* r = M^T v */
static inline void pm_tmul_v(double r[3], const double m[3][3], const double v[3])
{
    r[0] = m[0][0] * v[0] + m[1][0] * v[1] + m[2][0] * v[2];
    r[1] = m[0][1] * v[0] + m[1][1] * v[1] + m[2][1] * v[2];
    r[2] = m[0][2] * v[0] + m[1][2] * v[1] + m[2][2] * v[2];
}
/* r = A B */
static inline void pm_mul(double r[3][3], const double a[3][3], const double b[3][3])
{
    int i, j;
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) r[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}
/* r = A^T B */
static inline void pm_tmul(double r[3][3], const double a[3][3], const double b[3][3])
{
    int i, j;
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) r[i][j] = a[0][i] * b[0][j] + a[1][i] * b[1][j] + a[2][i] * b[2][j];
}
static inline void pm_from9(double r[3][3], const double *v)
{
    int i, j;
    for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) r[i][j] = v[3 * i + j];
}
static inline void pm_to9(double *r, const double m[3][3])
{
    int i, j;
    for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) r[3 * i + j] = m[i][j];
}
#endif
