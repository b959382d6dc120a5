/*
 * MatVec.h -- PQP-interface restatement of the small 3-vector / 3x3-matrix
 * helpers the C2A sources call (VmV, MxVpV, MTxM, Vnormalize, ...), and the
 * symmetric 3x3 eigen-solver Meigen used by the BVH build
 * (C2A/src/C2A_Build.cpp:416).  Used only to compile the reference sources
 * for the CPU oracle.
 *
 * Every helper spells out its evaluation order, left to right, so that the
 * CUDA kernels and the plain-C oracle port can repeat it operation for
 * operation (the project builds all of them without FP contraction).
 * Matrices are row-major PQP_REAL[3][3].
 */
#ifndef C2A_SHIM_MATVEC_H
#define C2A_SHIM_MATVEC_H

#include <math.h>
#include "PQP_Compile.h"

inline void Midentity(PQP_REAL M[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) M[i][j] = (i == j) ? 1.0 : 0.0;
}

inline void Videntity(PQP_REAL T[3]) { T[0] = T[1] = T[2] = 0.0; }

inline void McM(PQP_REAL Mr[3][3], const PQP_REAL M[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Mr[i][j] = M[i][j];
}

inline void MTcM(PQP_REAL Mr[3][3], const PQP_REAL M[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Mr[i][j] = M[j][i];
}

inline void VcV(PQP_REAL Vr[3], const PQP_REAL V[3])
{
  Vr[0] = V[0]; Vr[1] = V[1]; Vr[2] = V[2];
}

// column c of M into V
inline void McolcV(PQP_REAL V[3], const PQP_REAL M[3][3], int c)
{
  V[0] = M[0][c]; V[1] = M[1][c]; V[2] = M[2][c];
}

// column cr of Mr := column c of M
inline void McolcMcol(PQP_REAL Mr[3][3], int cr, const PQP_REAL M[3][3], int c)
{
  Mr[0][cr] = M[0][c]; Mr[1][cr] = M[1][c]; Mr[2][cr] = M[2][c];
}

// Mr = M1 * M2, entry (i,j) = (M1[i][0]*M2[0][j] + M1[i][1]*M2[1][j]) + M1[i][2]*M2[2][j]
inline void MxM(PQP_REAL Mr[3][3], const PQP_REAL M1[3][3], const PQP_REAL M2[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Mr[i][j] = M1[i][0] * M2[0][j] + M1[i][1] * M2[1][j] + M1[i][2] * M2[2][j];
}

// Mr = M1^T * M2
inline void MTxM(PQP_REAL Mr[3][3], const PQP_REAL M1[3][3], const PQP_REAL M2[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Mr[i][j] = M1[0][i] * M2[0][j] + M1[1][i] * M2[1][j] + M1[2][i] * M2[2][j];
}

// Mr = M1 * M2^T
inline void MxMT(PQP_REAL Mr[3][3], const PQP_REAL M1[3][3], const PQP_REAL M2[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Mr[i][j] = M1[i][0] * M2[j][0] + M1[i][1] * M2[j][1] + M1[i][2] * M2[j][2];
}

inline void MxV(PQP_REAL Vr[3], const PQP_REAL M1[3][3], const PQP_REAL V1[3])
{
  Vr[0] = M1[0][0] * V1[0] + M1[0][1] * V1[1] + M1[0][2] * V1[2];
  Vr[1] = M1[1][0] * V1[0] + M1[1][1] * V1[1] + M1[1][2] * V1[2];
  Vr[2] = M1[2][0] * V1[0] + M1[2][1] * V1[1] + M1[2][2] * V1[2];
}

// Vr = M1 * V1 + V2, each row ((a + b) + c) + V2
inline void MxVpV(PQP_REAL Vr[3], const PQP_REAL M1[3][3], const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  Vr[0] = M1[0][0] * V1[0] + M1[0][1] * V1[1] + M1[0][2] * V1[2] + V2[0];
  Vr[1] = M1[1][0] * V1[0] + M1[1][1] * V1[1] + M1[1][2] * V1[2] + V2[1];
  Vr[2] = M1[2][0] * V1[0] + M1[2][1] * V1[1] + M1[2][2] * V1[2] + V2[2];
}

// Vr = s * (M1 * V1) + V2
inline void sMxVpV(PQP_REAL Vr[3], PQP_REAL s1, const PQP_REAL M1[3][3], const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  Vr[0] = s1 * (M1[0][0] * V1[0] + M1[0][1] * V1[1] + M1[0][2] * V1[2]) + V2[0];
  Vr[1] = s1 * (M1[1][0] * V1[0] + M1[1][1] * V1[1] + M1[1][2] * V1[2]) + V2[1];
  Vr[2] = s1 * (M1[2][0] * V1[0] + M1[2][1] * V1[1] + M1[2][2] * V1[2]) + V2[2];
}

// Vr = M1^T * V1
inline void MTxV(PQP_REAL Vr[3], const PQP_REAL M1[3][3], const PQP_REAL V1[3])
{
  Vr[0] = M1[0][0] * V1[0] + M1[1][0] * V1[1] + M1[2][0] * V1[2];
  Vr[1] = M1[0][1] * V1[0] + M1[1][1] * V1[1] + M1[2][1] * V1[2];
  Vr[2] = M1[0][2] * V1[0] + M1[1][2] * V1[1] + M1[2][2] * V1[2];
}

inline void sMTxV(PQP_REAL Vr[3], PQP_REAL s1, const PQP_REAL M1[3][3], const PQP_REAL V1[3])
{
  Vr[0] = s1 * (M1[0][0] * V1[0] + M1[1][0] * V1[1] + M1[2][0] * V1[2]);
  Vr[1] = s1 * (M1[0][1] * V1[0] + M1[1][1] * V1[1] + M1[2][1] * V1[2]);
  Vr[2] = s1 * (M1[0][2] * V1[0] + M1[1][2] * V1[1] + M1[2][2] * V1[2]);
}

inline void VmV(PQP_REAL Vr[3], const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  Vr[0] = V1[0] - V2[0]; Vr[1] = V1[1] - V2[1]; Vr[2] = V1[2] - V2[2];
}

inline void VpV(PQP_REAL Vr[3], const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  Vr[0] = V1[0] + V2[0]; Vr[1] = V1[1] + V2[1]; Vr[2] = V1[2] + V2[2];
}

// Vr = V1 + V2 * s
inline void VpVxS(PQP_REAL Vr[3], const PQP_REAL V1[3], const PQP_REAL V2[3], PQP_REAL s)
{
  Vr[0] = V1[0] + V2[0] * s; Vr[1] = V1[1] + V2[1] * s; Vr[2] = V1[2] + V2[2] * s;
}

inline void VcrossV(PQP_REAL Vr[3], const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  Vr[0] = V1[1] * V2[2] - V1[2] * V2[1];
  Vr[1] = V1[2] * V2[0] - V1[0] * V2[2];
  Vr[2] = V1[0] * V2[1] - V1[1] * V2[0];
}

inline PQP_REAL Vlength(const PQP_REAL V[3])
{
  return sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
}

// V *= 1/|V|  (the reciprocal is formed first)
inline void Vnormalize(PQP_REAL V[3])
{
  PQP_REAL d = (PQP_REAL)1.0 / sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
  V[0] *= d; V[1] *= d; V[2] *= d;
}

inline PQP_REAL VdotV(const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  return V1[0] * V2[0] + V1[1] * V2[1] + V1[2] * V2[2];
}

inline PQP_REAL VdistV2(const PQP_REAL V1[3], const PQP_REAL V2[3])
{
  return (V1[0] - V2[0]) * (V1[0] - V2[0]) + (V1[1] - V2[1]) * (V1[1] - V2[1]) +
         (V1[2] - V2[2]) * (V1[2] - V2[2]);
}

// Vr = V * s
inline void VxS(PQP_REAL Vr[3], const PQP_REAL V[3], PQP_REAL s)
{
  Vr[0] = V[0] * s; Vr[1] = V[1] * s; Vr[2] = V[2] * s;
}

/*
 * Meigen: eigen-decomposition of the symmetric matrix a.  Columns of vout are
 * the eigenvectors, dout the eigenvalues.  Cyclic Jacobi rotations (Golub and
 * Van Loan, "Matrix Computations", sec. 8.5); implemented in
 * oracle/c2a_port_build.c (c2a_port_jacobi3) so the oracle port and this
 * PQP-interface restatement run the identical arithmetic.
 */
#ifdef __cplusplus
extern "C" {
#endif
void c2a_port_jacobi3(double vout[3][3], double dout[3], const double a[3][3]);
#ifdef __cplusplus
}
#endif

inline void Meigen(PQP_REAL vout[3][3], PQP_REAL dout[3], PQP_REAL a[3][3])
{
  c2a_port_jacobi3(vout, dout, a);
}

#endif
