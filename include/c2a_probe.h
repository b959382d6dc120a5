/*
 * c2a_probe.h -- the FP64 pipe's measured peak, the ceiling of the CA
 * kernels' roofline.  The node-pair and triangle tests are chains of FP64
 * adds, multiplies, divisions and square roots; this probe measures what the
 * GPU's FP64 units deliver to such code, on every SM at once.
 */
#ifndef C2A_PROBE_H
#define C2A_PROBE_H

#include "c2a_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs two FP64 throughput kernels on `device` (every SM, eight independent
 * dependency chains per thread) and returns the best of `repeats` timed
 * launches of each: fma_flops, FP64 flop/s of fused multiply-adds (two flops
 * each: the conventional peak); add_flops, flop/s of plain additions (one
 * flop per instruction: the ceiling of code compiled without contraction, as
 * the reference's is).  Synchronous; allocates 4 KiB of device memory. */
c2a_status c2a_probe_fp64_peak(int device, int repeats, double *fma_flops, double *add_flops);

#ifdef __cplusplus
}
#endif
#endif
