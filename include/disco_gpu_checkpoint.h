/*
 * disco_gpu_checkpoint.h -- checkpoint output and restart in the layout of
 * the reference's Output/h5out.c (output, :366-620) and Restart/h5in.c
 * (restart, :100-354), serial case.
 *
 * File layout (HDF5; groups and datasets by the reference's names):
 *   /GIT_VERSION                       variable-length string
 *   /Grid/T [1]                        t
 *   /Grid/r_jph [Nr+1], z_kph [Nz+1]   ring and layer edges, ghosts included
 *   /Grid/Index, Np, Id_phi0 [Nz][Nr]  int32: first cell of each ring, its
 *                                      cell count, the cell nearest phi = 0
 *   /Data/Cells [Ncell][NUM_Q + NUM_FACES + 1]
 *                                      per cell: prim, the CT face fluxes
 *                                      Phi (0, 3 or 5), piph
 *   /Data/Planets [Npl][7]             M, vr, omega, r, phi, eps, type
 *   /Data/Diagnostics [Nz][Nr][n]      the ring diagnostics averaged over
 *                                      their accumulation time
 *   /Opts/...                          module names (strings) and NUM_C,
 *                                      NUM_N, CT_MODE
 *   /Pars/...                          the in.par values, one [1] dataset each
 * Rings are in the order jk = j + Nr*k, every ring written (the serial
 * reference writes ghosts too).
 *
 * The file is written by the library's own HDF5 writer (superblock version
 * 2, compact groups, contiguous datasets; no HDF5 library involved), which
 * any HDF5 1.8+ reader accepts.  disco_host_restart reads files in that
 * subset; a file written by the HDF5 library itself (superblock 0 with
 * symbol-table groups) is reported as unsupported.
 */
#ifndef DISCO_GPU_CHECKPOINT_H
#define DISCO_GPU_CHECKPOINT_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* output() for a checkpoint: downloads the device state of g (created from
 * dom, or from a domain with the same grid) and writes `path`.  As
 * h5out.c:389 and :610 do, the ring diagnostics are divided by their
 * accumulation time for the file and then zeroed on the device.  Returns
 * 0 or a negative DISCO_E_* code. */
int disco_gpu_checkpoint(disco_gpu *g, const disco_host_domain *dom, const char *path);

/* The same file from a host domain alone (the initial state of
 * disco_host_setup, or a restarted one): Phi from dom->Phi (zero if NULL),
 * no diagnostics (n = 0). */
int disco_host_checkpoint(const disco_host_domain *dom, const char *path);

/* restart() plus setupCells (domain.c:139-238) for Restart = 1: the grid
 * (Num_R, Num_Z from the file's Index shape, r_jph, z_kph, Np), the cells'
 * primitives, face fluxes and phases, t and the planets (type point mass,
 * h5in.c:303-318) from `path`, the noise of Noise_Type drawn as the
 * reference draws it after its in.par grid's ring phases, dphi from the
 * phases (calc_dp).  par and mod come from in.par and Makefile_opt.in as
 * for disco_host_setup.  disco_gpu_create on the result uses the file's
 * face fluxes (out->Phi) instead of the initial field's. */
int disco_host_restart(const disco_params *par, const disco_modules *mod,
                       const char *path, disco_host_domain **out);

#ifdef __cplusplus
}
#endif
#endif
