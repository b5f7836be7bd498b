/*
 * disco_gpu_noalloc.h -- the CFL timestep of a device instance computed
 * without any device memory allocation.
 *
 * No reference counterpart: the reference's getmindt (misc.c:39) is a serial
 * CPU loop with nothing to allocate.  This entry point exists for callers
 * that may not allocate device memory at the moment they need dt:
 *   - a host loop running beside a caching allocator that already holds
 *     almost all device memory, where a new cudaMalloc can fail or force the
 *     allocator to release its cache;
 *   - a stepping loop with a fixed device-memory budget set at start-up;
 *   - a latency-sensitive loop that must not take the device-wide
 *     synchronisation that cudaFree implies.
 * disco_gpu_getmindt itself allocates nothing per call either (its
 * accumulator is part of the instance, allocated once by disco_gpu_create);
 * this variant also leaves the instance untouched: its scratch is a
 * statically sized __device__ array of the library.
 */
#ifndef DISCO_GPU_NOALLOC_H
#define DISCO_GPU_NOALLOC_H

#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Largest instance (cells including ghosts) the static scratch serves: one
 * partial minimum per block of 256 cells, 131072 blocks. */
#define DISCO_NOALLOC_MAX_CELLS (131072L * 256L)

/* Same result as disco_gpu_getmindt (bit for bit): CFL * min over real cells
 * of the module's mindt, capped by maxDT.  Reads the instance's state and
 * writes nothing in it; per-block partial minima go to the static scratch
 * array, located with cudaGetSymbolAddress once per device.  Nothing in the
 * scratch has to start at zero: every slot is written before it is read
 * within the call.  Returns DISCO_E_ARG (nothing launched) when the instance
 * has more than DISCO_NOALLOC_MAX_CELLS cells.
 *
 * The call runs on the instance's device (the device that was current when
 * disco_gpu_create made it): the caller's current device is switched to it
 * for the call and restored before returning.  The scratch address is
 * looked up for that device on its first call there.
 *
 * The scratch array is shared by all instances of the same hydro module and
 * precision on a device: concurrent calls from several host threads or
 * streams race on it and must be serialised by the caller. */
int disco_gpu_getmindt_noalloc(disco_gpu *g, double *dt);

#ifdef __cplusplus
}
#endif
#endif
