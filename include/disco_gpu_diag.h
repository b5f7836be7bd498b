/*
 * disco_gpu_diag.h -- the time-averaged ring diagnostics that the
 * reference's timestep() accumulates at every step (add_diagnostics,
 * analysis.c:52-108, called at timestep.c:51) with the Diagnostics/ plugin
 * that Makefile_opt.in's ANALYSIS names.
 *
 * Layout as the reference's struct diagnostic_avg (paul.h): Qrz[jk*n + q]
 * for ring jk = k*Nr + j (ghost rings included), q < n = num_diagnostics(),
 * plus t_avg, the time summed over since the last zero.  Each step adds
 * (sum over the ring of Q_q dV) * dt / (ring volume) to Qrz and dt to t_avg;
 * the device does so inside disco_gpu_timestep / disco_gpu_run.
 *
 * The reference's output step (h5out.c:389, :610) divides Qrz by t_avg
 * (avg_diagnostics), writes it and zeroes both (zero_diagnostics); the
 * restart reads them back (h5in.c:329).  A host replacing those calls uses
 * download / zero / upload below.
 */
#ifndef DISCO_GPU_DIAG_H
#define DISCO_GPU_DIAG_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* num_diagnostics() of the configured plugin: 8 (diag_euler), 5
 * (diag_disk2d), 6 (diag_cb), 5 (diag_bl), 18 (diag_mhdmri), 48
 * (diag_grmhdmri, GRMHD only), 0 when
 * Makefile_opt.in names no ANALYSIS.  Negative DISCO_E_* on error. */
int disco_gpu_diag_count(disco_gpu *g);

/* Copies Nr*Nz*n accumulators to Qrz (len >= Nr*Nz*n; Qrz may be NULL to
 * read t_avg alone) and t_avg (may be NULL).  Returns n, or DISCO_E_*. */
int disco_gpu_diag_download(disco_gpu *g, double *Qrz, long long len, double *t_avg);

/* Replaces the accumulators (restart): len must be Nr*Nz*n.  Qrz NULL
 * zeroes them and t_avg (zero_diagnostics, analysis.c:9-27).  Returns n. */
int disco_gpu_diag_upload(disco_gpu *g, const double *Qrz, long long len, double t_avg);

/* Divergence of B as constrained transport holds it: per cell, the net
 * outward flux through its faces, from the face fluxes Phi (the sum of
 * Python/discopy/geom.py:370-520, calcDivB, which the reference applies to
 * its checkpoints).  div[c] is that sum and scale[c] the sum of the
 * absolute face fluxes of cell c, so |div| / scale is the divergence
 * relative to the flux through the cell; cells without a neighbour ring on
 * every side get div 0 and scale -1.  Arrays of Ncell (either may be NULL).
 * Constrained-transport instances only (DISCO_E_STATE otherwise). */
int disco_gpu_divb(disco_gpu *g, double *div, double *scale);

#ifdef __cplusplus
}
#endif
#endif
