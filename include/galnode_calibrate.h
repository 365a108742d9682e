/*
 * galnode_calibrate.h -- measurement helpers of the GB300 node evolver.
 *
 * These entry points have no counterpart in the reference; they exist so
 * that benchmark drivers can express kernel throughput as a fraction of the
 * device's measured FP64 rate (the pipe that bounds the node integrator).
 */
#ifndef GALNODE_CALIBRATE_H
#define GALNODE_CALIBRATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Measure the sustained FP64 fused-multiply-add rate of the current device
 * with a register-resident DFMA loop on every SM.  Writes FLOP/s (2 per
 * DFMA) to *flops and the kernel time in ms to *ms.  Returns 0 on success. */
int gal_calibrate_fp64(double* flops, double* ms);

#ifdef __cplusplus
}
#endif

#endif
