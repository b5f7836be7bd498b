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
 * per-planet sink accumulators come from disco_gpu_sink_accum.
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

/* The sink bodies' accumulators that report.c prints after the mass ratio
 * (report.c:81-88, sink.c:189-245), accumulated by every substep's
 * sink_src since the last reset with the RK blend of the planets'
 * auxiliary fields (planet.c:261-270).  For sink body b (the first
 * Sink_Number bodies, or all) out[8 b + k] holds, k = 0..7: gravL, dM,
 * accL, Ls, kin, therm, linXmom, linYmom.  reset != 0 then zeroes them and
 * their RK copy, as report() does after printing (report.c:91-108).
 * Returns the number of bodies written (0 without sinks), at most
 * max_bodies, or a negative DISCO_E_* code. */
#define DISCO_SINK_NACC 8
int disco_gpu_sink_accum(disco_gpu *g, double *out, int max_bodies, int reset);

#ifdef __cplusplus
}
#endif
#endif
