/*
 * disco_gpu_debug.h -- stage dumps of the constrained-transport chain, for
 * tests that compare the device path with the CPU oracle kernel by kernel.
 * Not part of the reference-facing interface.
 */
#ifndef DISCO_GPU_DEBUG_H
#define DISCO_GPU_DEBUG_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs getmindt and the first RK substep of a timestep up to `stage` of the
 * constrained-transport chain, then copies per-cell arrays (SoA, Ncell
 * each; NULL to skip):
 *   stage 1: after the flux sweeps and edge gathers  -> E[8], B[8], Ephi[4]
 *   stage 2: + avg_Efields and advective subtraction -> E[8] slots 0,1,4,5
 *   stage 3: + update_B_fluxes circulation           -> Phi[5]
 *   stage 4: + make_edge_adjust                       -> Phi[5]
 * The instance is left mid-step and must not be stepped afterwards. */
int disco_gpu_debug_ct(disco_gpu *g, int stage, double *E, double *B,
                       double *Ephi, double *Phi);

#ifdef __cplusplus
}
#endif
#endif
