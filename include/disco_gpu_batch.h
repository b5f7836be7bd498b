/*
 * disco_gpu_batch.h -- many independent device instances advanced together.
 *
 * No reference counterpart: the reference advances one domain per process
 * (main.c:69-74).  A batch stands for N independent runs of that loop (for
 * example a parameter survey of disks with different resolutions and planet
 * masses): every step of the batch is one CUDA-graph launch whose branches
 * are the members' full steps (getmindt + RK2 timestep, each member with its
 * own dt), so the small kernels of different members run concurrently.
 */
#ifndef DISCO_GPU_BATCH_H
#define DISCO_GPU_BATCH_H

#include <stddef.h>
#include "disco_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct disco_batch disco_batch;

/* Groups n existing instances (created by disco_gpu_create, any hydro module
 * and precision, all on the current device).  The batch borrows them: they
 * stay usable on their own between batch calls (download, status, ...) and
 * must outlive the batch. */
int disco_batch_create(disco_gpu *const *members, int n, disco_batch **out);

/* nsteps steps of every member (dt computed per member on the device). */
int disco_batch_run(disco_batch *b, int nsteps);

/* As disco_batch_run, each step bracketed by CUDA events on the batch's
 * stream; flush_bytes > 0 overwrites a scratch buffer before each step,
 * outside the timed interval.  *ms_total = summed device time. */
int disco_batch_run_timed(disco_batch *b, int nsteps, size_t flush_bytes, double *ms_total);

/* Frees the batch's graphs and streams, not its members. */
void disco_batch_free(disco_batch *b);

#ifdef __cplusplus
}
#endif
#endif
