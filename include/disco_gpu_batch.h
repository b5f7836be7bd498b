/*
 * disco_gpu_batch.h -- many independent device instances advanced together.
 *
 * No reference counterpart: the reference advances one domain per process
 * (main.c:69-74).  A batch stands for N independent runs of that loop (for
 * example a parameter survey of disks with different resolutions and planet
 * masses): every step of the batch is one CUDA-graph launch of the members'
 * full steps (getmindt + RK2/RK3 timestep, each member with its own dt).
 *
 * Members of one hydro module and precision whose steps launch the same
 * kernel sequence form a group.  A group is split into sub-groups, each
 * advanced by persistent multi-instance stage kernels: each stage of the
 * step is ONE launch whose blocks walk the work items (member, tile) of
 * every member of the sub-group, so a sub-group of 64 small disks launches
 * as many kernels per step as one disk does.  Sub-groups are branches of
 * the step's graph, so the stages of different sub-groups overlap.  Members
 * with constrained transport, a boundary plugin, the staged phi sweep, a
 * learned cons2prim start or sinks, and groups of one, run their own launch
 * sequence as a branch of the graph.  A member ends where it ends alone:
 * bit for bit on the FP64 path; to FP32 rounding on the mixed path, whose
 * units contract multiply-adds per kernel.
 *
 * The split -- sub-groups per group, from {1, 2, 4, 8, 16}, or 0: every
 * member on its own launch sequence -- is chosen by timing each candidate
 * on two of the batch's first twelve steps (real steps of every member),
 * unless disco_batch_set_split fixed it.
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

/* As disco_batch_create; flags DISCO_BATCH_NO_GROUPS gives every member its
 * own launch sequence (one graph branch each), forming no groups. */
#define DISCO_BATCH_NO_GROUPS 1
int disco_batch_create_flags(disco_gpu *const *members, int n, int flags, disco_batch **out);

/* nsteps steps of every member (dt computed per member on the device). */
int disco_batch_run(disco_batch *b, int nsteps);

/* As disco_batch_run, each step bracketed by CUDA events on the batch's
 * stream; flush_bytes > 0 overwrites a scratch buffer before each step,
 * outside the timed interval.  *ms_total = summed device time. */
int disco_batch_run_timed(disco_batch *b, int nsteps, size_t flush_bytes, double *ms_total);

/* The stage kernels' grid: at most ctas_per_sm blocks per SM (1..64,
 * default 8), and never more than are resident at once. */
int disco_batch_set_grid(disco_batch *b, int ctas_per_sm);

/* Fixes the split (0, 1, 2, 4, 8 or 16), or -1: choose it by timing over
 * the next twelve steps. */
int disco_batch_set_split(disco_batch *b, int split);

/* Groups formed, members in them, the split in force (-1: still timing),
 * the grid, and the best step time (ms) of each split candidate in the
 * order {1, 2, 4, 8, 16, 0} (-1: not timed); any pointer may be NULL. */
#define DISCO_BATCH_NSPLIT 6
int disco_batch_info(const disco_batch *b, int *groups, int *grouped_members, int *split, int *ctas_per_sm,
                     double *tune_ms);

/* nsteps steps of every member without the graph: each stage kernel of
 * every sub-group launched by itself and bracketed by CUDA events (at the
 * split in force, or 1 while it is still being chosen); members on their
 * own sequences take their steps untimed.  Per stage name: launches and
 * summed milliseconds over the sub-groups (at most max_out entries). */
int disco_batch_profile(disco_batch *b, int nsteps, disco_kernel_time *out, int max_out, int *n_out);

/* Frees the batch's graphs and streams, not its members. */
void disco_batch_free(disco_batch *b);

#ifdef __cplusplus
}
#endif
#endif
