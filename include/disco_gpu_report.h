/*
 * disco_gpu_report.h -- the domain diagnostics of the reference's report()
 * (report.c:4-329) computed on the device.
 *
 * The reference writes one line of report.dat at every report: the time,
 * the mass ratio, per-planet sink accumulators, then the gas mass and the
 * gravitational torques of the gas on the first two bodies, in total and
 * outside five cut radii (n + 1) * Sink_Par3, n = 0..4, around the second
 * body.  This entry point returns those sums from the device state, summed
 * in a fixed order (equal to the reference's serial sums to rounding).  The
 * per-planet sink accumulators are zero in this build (sinks are not
 * built) and are not returned.
 */
#ifndef DISCO_GPU_REPORT_H
#define DISCO_GPU_REPORT_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Number of values disco_gpu_report returns:
 *   [0] t, [1] q = M_1 / M_0 (0 with one body), [2] Mass,
 *   [3] Torque, [4] Torque2,
 *   [5 + 2n] Torque1_cut[n], [6 + 2n] Torque2_cut[n], n = 0..4. */
#define DISCO_REPORT_NVALUES 15

/* Writes min(nout, DISCO_REPORT_NVALUES) values to out and returns that
 * count, or a negative DISCO_E_* code.  The first call allocates a small
 * device buffer for the block partials (about 100 bytes per 256 cells). */
int disco_gpu_report(disco_gpu *g, double *out, int nout);

#ifdef __cplusplus
}
#endif
#endif
