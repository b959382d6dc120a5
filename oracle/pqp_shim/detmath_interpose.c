/*
 * detmath_interpose.c -- links the deterministic sin/cos/acos into the
 * reference oracle library in place of the platform libm, so the reference
 * code (C2A/src/InterpMotion.cpp:251, 275-278) computes the same correctly
 * rounded poses on x86-64 and aarch64 hosts as the CUDA kernels and the
 * oracle port.  Hidden visibility binds the reference's calls to these
 * definitions inside the library without exporting them to the process.
 */
#include "../../c2a_gb300/csrc/common/c2a_detmath.h"

__attribute__((visibility("hidden"))) double sin(double x) { return c2a_det_sin(x); }
__attribute__((visibility("hidden"))) double cos(double x) { return c2a_det_cos(x); }
__attribute__((visibility("hidden"))) double acos(double x) { return c2a_det_acos(x); }
