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

/* Self-test of the integrator's short FP64 functions against the CUDA library
 * over 4M arguments: reciprocal, quotient, reciprocal square root and square
 * root on 1e-29..1e29 (relative error), log on 1e-29..1e29 (error relative
 * to max(1, |ln x|)), exp on -120..5 (relative error) and the controller's inverse fifth
 * and sixth roots on 3e-5..1900 (relative error), then the FP32-rate
 * controller's 0.9 x^(-1/5) and 0.9 x^(-1/6) from a seed ratio off by up to
 * 3e-6 (relative error; [10] counts the arguments that needed the Newton
 * fallback), and the integer-pipe comparisons and conversions of doubles
 * and floats against the IEEE comparisons and the conversion instructions,
 * on signed zeros, subnormals, infinities, NaNs and bit patterns spread
 * over every exponent ([11] counts the disagreements).  Writes twelve values to maxRelErr[0..11]: the worst
 * errors, and in [10] and [11] the largest per-thread counts.  Returns 0 on
 * success. */
int gal_selftest_fastmath(double* maxRelErr);

#ifdef __cplusplus
}
#endif

#endif
