/* Build.h -- PQP-interface restatement; C2A uses its own build (C2A/src/C2A_Build.cpp). */
#ifndef C2A_SHIM_BUILD_H
#define C2A_SHIM_BUILD_H
#endif
