/*
 * disco_gpu_mlp.h -- a learned starting point for the GRMHD module's Newton
 * cons2prim.
 *
 * The reference starts its Noble et al. 2D Newton iteration from the
 * previous primitives (Hydro/grmhd.c:885-893) and iterates to a relative
 * change of 1e-12 plus 10 more iterations (:910-957).  Here a small MLP
 * corrects that start: from 10 features -- the Noble invariants of the new
 * conserved state, the rest mass, the lapse, r, and log(W^2 - 1) and
 * log(P / rho) of the previous primitives -- it predicts how much those two
 * logarithms change (two hidden layers of 64, tanh).  It is trained on the
 * GPU, on pairs the method harvests from its own solves during torus runs,
 * by hand-written BF16 tensor-core forward and backward kernels with FP32
 * accumulation and FP32 Adam.  The
 * Newton solve is unchanged and still runs to the same tolerance; the
 * previous primitives stay the starting point wherever they leave the
 * smaller residual of the two Noble equations, so the converged primitives
 * are the same and only the iteration count changes.
 *
 * No reference counterpart beyond the warm start it replaces.
 */
#ifndef DISCO_GPU_MLP_H
#define DISCO_GPU_MLP_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct disco_mlp disco_mlp;

#define DISCO_MLP_FEATURES 10
#define DISCO_MLP_OUTPUTS 2
/* FP32 parameters, flat: W1[64][16] (inputs 10..15 zero), b1[64],
 * W2[64][64], b2[64], W3[8][64] (rows 2..7 zero), b3[8] */
#define DISCO_MLP_PARAMS 5768
/* standardisation: feature means[10], feature scales[10], target means[2],
 * target scales[2] */
#define DISCO_MLP_NORM 24

/* A model with Xavier-uniform weights drawn from splitmix64(seed), zero
 * biases, identity standardisation, and room for `capacity` training pairs
 * on the current device. */
int disco_mlp_create(unsigned long long seed, long capacity, disco_mlp **out);
void disco_mlp_free(disco_mlp *m);

/* Advances g by `steps` timesteps (getmindt + timestep) with the
 * reference's start, recording a training pair for every stride-th real
 * cell at every cons2prim: its features and the change of log(W^2 - 1) and
 * log(P / rho) from the previous primitives to the converged solution.
 * *count = pairs held (at most the capacity).  GRMHD instances only. */
int disco_mlp_harvest(disco_mlp *m, disco_gpu *g, int stride, int steps, long *count);

/* Copies held pairs [first, first + n) to the host (either array may be
 * NULL): X [n][10] features, Y [n][2] targets. */
int disco_mlp_pairs(disco_mlp *m, long first, long n, float *X, float *Y);

/* Sets the standardisation from the mean and standard deviation of the held
 * pairs. */
int disco_mlp_fit_norm(disco_mlp *m);

/* steps of Adam (lr, beta 0.9 / 0.999) on batches of `batch` pairs drawn by
 * splitmix64 from the held ones; loss_first / loss_last (may be NULL): the
 * mean squared error of the standardised outputs on the first / last
 * batch. */
int disco_mlp_train(disco_mlp *m, int steps, int batch, float lr, unsigned long long seed,
                    float *loss_first, float *loss_last);

/* One forward and backward pass over n given pairs (raw X [n][10], Y [n][2])
 * without an update: *loss = the summed squared error of the standardised
 * outputs, grad[DISCO_MLP_PARAMS] = the gradient of loss / n. */
int disco_mlp_grad(disco_mlp *m, const float *X, const float *Y, int n, float *loss, float *grad);

/* The network's raw outputs Y [n][2] for raw features X [n][10]. */
int disco_mlp_predict(disco_mlp *m, const float *X, long n, float *Y);

/* Reads (get != NULL) and/or replaces (set != NULL) the FP32 parameters
 * (DISCO_MLP_PARAMS floats) and the standardisation (DISCO_MLP_NORM). */
int disco_mlp_params(disco_mlp *m, float *get, const float *set, float *norm_get, const float *norm_set);

/* When cons2prim takes the model's start.  With r_w the residual of the two
 * Noble equations (each relative to the term it balances) at the previous
 * primitives and r_g at the model's start, the model's start is taken where
 * r_w > floor and r_g < ratio r_w (defaults 0 and 1; 0 < ratio <= 1).
 * Takes effect at the next disco_gpu_attach_guess. */
int disco_mlp_set_gate(disco_mlp *m, double floor, double ratio);

/* Makes g's cons2prim start from the model's guess (m NULL: from the
 * previous primitives only, the reference's start).  The instance keeps the
 * model's device pointers and its current standardisation: train or change
 * the parameters as much as wished afterwards, but attach again after
 * disco_mlp_fit_norm.  GRMHD instances only. */
int disco_gpu_attach_guess(disco_gpu *g, disco_mlp *m);

/* Newton cons2prim counters of g since the last reset: out[0] calls,
 * out[1] summed iteration at first convergence (k_converge), out[2] summed
 * iterations, out[3] calls that started from the model's guess.  reset != 0
 * zeroes them after reading. */
int disco_gpu_c2p_stats(disco_gpu *g, long long out[4], int reset);

#ifdef __cplusplus
}
#endif
#endif
