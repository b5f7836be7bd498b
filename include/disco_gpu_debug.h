/*
 * disco_gpu_debug.h -- test access to intermediate device state: the stages
 * of the constrained-transport chain, the sheared-face tables, the PLM
 * gradients, and the FP64 <-> FP32 conversions of the mixed path, for tests
 * that compare the device with the reference's fixtures and the CPU oracle
 * stage by stage.  Not part of the reference-facing interface.
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

/* The sheared-face tables of dimension dim (1 = r, 2 = z) as the device
 * holds them, in the reference's layout (faces_alt.c:80-179, misc.c:522):
 * fIndex[npair + 1] is the first face of each ring pair (the reference's
 * fIndex_r / fIndex_z, pairs ordered j + (Nr-1)*k for r, j + Nr*k for z),
 * and per face L, R (global cell ids: ring_off[jk] + i), LRtype, the phi of
 * the face centroid (cm[1]) and the area dA (widened on the mixed path).
 * *npair and *nface receive the sizes; any array may be NULL (call once
 * with all NULL to size the buffers). */
int disco_gpu_debug_faces(disco_gpu *g, int dim, int *npair, long *nface,
                          int *fIndex, int *L, int *R, int *LRtype,
                          double *phic, double *dA);

/* plm_phi and plm_trans (onestep.c:104-130, plm.c:6-232) on the current
 * state with the current faces; copies gradp, gradr, gradz
 * [num_q*Ncell] (NULL to skip), widened to FP64 on the mixed path.  The
 * state is left unchanged, so stepping may continue. */
int disco_gpu_debug_grad(disco_gpu *g, double *gradp, double *gradr, double *gradz);

/* The mixed path's azimuthal sweep: on = 1 selects the staged single-pass
 * kernel (k_phi_sweep, the default where it applies), 0 the separate
 * plm_phi and phi-flux kernels, for tests that compare the two; 2 the
 * staged kernel with its tensor copies withheld, so that its bounded
 * waits (about a second each) run out: every block then counts a timeout
 * in disco_gpu_status's async_timeouts and returns without its fluxes
 * (the state of that step is not meaningful).  Returns the setting in
 * force (0 where the staged sweep does not apply: the plain FP64 path,
 * explicit viscosity). */
int disco_gpu_debug_sweep(disco_gpu *g, int on);

/* Applies the library's integer-pipe FP64 -> FP32 and FP32 -> FP64
 * conversions and the hardware's (cvt.rn.f32.f64, cvt.f64.f32) to n values
 * on the current device: f_int/f_hw[i] from in[i], d_int/d_hw[i] from
 * fin[i].  Host arrays of n elements each. */
int disco_gpu_debug_convert(const double *in, const float *fin, long n,
                            float *f_int, float *f_hw, double *d_int, double *d_hw);

#ifdef __cplusplus
}
#endif
#endif
