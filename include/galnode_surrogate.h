/*
 * galnode_surrogate.h -- the learned cooling-function surrogate of the GB300
 * node evolver.
 *
 * The reference evaluates its cooling function by bilinear interpolation in
 * a tabulated CIE file (cieFileCoolingFunction,
 * source/cooling/cooling_function/CIE_file.F90:238-317).  These entry
 * points have no counterpart in the reference: they train a 3-64-64-64-1
 * SiLU network, log10 Lambda(log10 T, log10 Z/Zsun, log10 n_H), on samples
 * of that interpolation, with the project's own FP32 forward/backward and
 * Adam kernels, and install it in an evolution context, where the integrator
 * evaluates it on the tensor cores (BF16 x BF16 -> FP32) in place of the
 * table.  The table stays the fallback outside the training domain and in
 * the cells of an error map where the network misses it by more than a set
 * tolerance.
 *
 * Parameter layout (FP32): W1[64][3], b1[64], W2[64][64], b2[64],
 * W3[64][64], b3[64], W4[64], b4 (gal_surrogate_param_count() values).
 * Inputs are normalised as (x - in_mean)/in_scale.  The cooling function
 * scales exactly as n_H^2 (CIE_file.F90:514-533), so that dependence is a
 * fixed term: log10 Lambda = y_n y_scale + y_mean + 2 log10 n_H, where y_n
 * is the network output.
 */
#ifndef GALNODE_SURROGATE_H
#define GALNODE_SURROGATE_H

#include <stdint.h>
#include "galnode.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gal_surrogate_train_config {
  int64_t batch_size;   /* multiple of 64 */
  int32_t epochs;
  int32_t seed;         /* shuffling seed */
  float learning_rate;  /* Adam */
  float beta1, beta2, epsilon;
  float learning_rate_final; /* cosine decay from learning_rate to this over the run;
                                <= 0 or equal to learning_rate: constant rate */
} gal_surrogate_train_config;

typedef struct gal_surrogate {
  const float* params;         /* trained network, FP32 */
  float in_mean[3], in_scale[3];
  float y_mean, y_scale;
  float lo[3], hi[3];          /* training domain of (log10 T, log10 Z/Zsun, log10 n_H) */
  int32_t map_t, map_z;        /* error-map cells along log10 T and log10 Z/Zsun */
  float map_lo_t, map_lo_z, map_dt, map_dz;
  const uint8_t* use_table;    /* [map_t][map_z]; 1 = the table is used in that cell */
} gal_surrogate;

/* Number of network parameters (8641). */
int gal_surrogate_param_count(void);

/* Train the network with mini-batch Adam on the mean squared error of the
 * normalised targets.  x_* are [n][3] normalised inputs, y_* normalised
 * targets (host arrays); params holds the initial weights on entry and the
 * trained weights on return; history[2*epoch] and history[2*epoch+1]
 * receive the epoch's mean training loss and the validation loss. */
int gal_surrogate_train(const gal_surrogate_train_config* cfg, const float* x_train, const float* y_train,
                        int64_t n_train, const float* x_val, const float* y_val, int64_t n_val, float* params,
                        float* history);

/* Mean squared error over n samples and its gradient with respect to the
 * parameters, from the training kernels (for gradient checks). */
int gal_surrogate_gradient(const float* params, const float* x, const float* y, int64_t n, float* grad, float* loss);

/* Normalised network output for n normalised inputs: FP32 throughout
 * (tensor_cores = 0) or the integrator's BF16 tensor-core path (1). */
int gal_surrogate_predict(const float* params, const float* x, int64_t n, float* y, int32_t tensor_cores);

/* Install (s != NULL) or remove (s == NULL) the surrogate in a context.
 * While installed, gal_gpu_evolve_batch* evaluate the cooling function with
 * it (512 threads per block is not available then). */
int gal_gpu_set_surrogate(gal_ctx* ctx, const gal_surrogate* s);

/* How a batch is launched while a surrogate is installed: split = 1
 * (default) sorts the nodes by whether the network may serve them at their
 * starting state and runs those with the network kernel and the others
 * with the kernel of the same rates without it, at once on two streams;
 * split = 0 runs one network kernel over all nodes.  Results are the same
 * except that in the split launch a node whose starting cell the error map
 * gives to the table uses the table throughout the call.  No counterpart in
 * the reference. */
int gal_gpu_set_surrogate_split(gal_ctx* ctx, int32_t split);

/* Cooling-function evaluations by the surrogate and by the table fallback
 * since the surrogate was installed (one per node and right-hand side). */
int gal_gpu_surrogate_stats(const gal_ctx* ctx, uint64_t* network, uint64_t* table);

#ifdef __cplusplus
}
#endif

#endif
