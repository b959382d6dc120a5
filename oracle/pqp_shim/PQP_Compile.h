/*
 * PQP_Compile.h -- PQP-interface restatement used only to compile the C2A
 * reference sources for the CPU oracle.  Genuine PQP (GammaUNC/PQP, version
 * not pinned by C2A, README.md:9-19) is absent; this file restates the
 * compile-time configuration the C2A sources rely on.
 */
#ifndef C2A_SHIM_PQP_COMPILE_H
#define C2A_SHIM_PQP_COMPILE_H

#define PQP_REAL double

#define RSS_TYPE 1
#define OBB_TYPE 2
/* C2A_PQP.cpp:296-324 only compiles with OBB enabled; the CA path uses RSS. */
#define PQP_BV_TYPE (RSS_TYPE | OBB_TYPE)

inline PQP_REAL myfabs(PQP_REAL x) { return x < 0 ? -x : x; }

#endif
