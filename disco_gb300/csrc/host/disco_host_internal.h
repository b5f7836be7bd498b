/* Internal declarations shared by the host C set-up and the CUDA driver. */
#ifndef DISCO_HOST_INTERNAL_H
#define DISCO_HOST_INTERNAL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct disco_rand_state {
   uint32_t r[34];
   int pos;
} disco_rand_state;

void disco_rand_seed(disco_rand_state *st, unsigned int seed);
int disco_rand_next(disco_rand_state *st);
void disco_set_error(const char *msg);

/* Exposed for tests of the glibc-rand restatement. */
int disco_rand_sequence(unsigned int seed, int n, int *out);

/* The ring whose cells a periodic ghost ring (j, k) holds for dimension
 * dim (1: r, 2: z), or -1 when (j, k) is not a periodic ghost of dim. */
int disco_periodic_source(const disco_host_domain *d, int dim, int j, int k);

/* The two halves of disco_host_setup: the grid, ring phases and planets
 * (leaving *rs where setupCells draws its noise), then the real cells'
 * primitives (initial() when from_ic, else the ones already in d) with the
 * noise, and the periodic ghosts' first exchange. */
int disco_host_grid(const disco_params *par, const disco_modules *mod,
                    disco_host_domain **out, disco_rand_state *rs);
void disco_host_cells(disco_host_domain *d, disco_rand_state *rs, int from_ic);

#ifdef __cplusplus
}
#endif
#endif
