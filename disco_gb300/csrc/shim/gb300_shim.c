/*
 * gb300_shim.c -- the reference-side binding of libdisco_gb300: the file a
 * Disco maintainer adds to the reference build so that its main loop
 * (main.c:69-74) runs the hot path on the GPU.
 *
 * It defines the two symbols the main loop calls, getmindt (misc.c:39) and
 * timestep (timestep.c:7), on top of include/disco_gpu.h, and keeps the
 * reference's struct domain for everything else (output, report, restart):
 *
 *   gb300_init(theDomain)          after setupCells (main.c:47): creates the
 *                                  device instance from in.par and
 *                                  Makefile_opt.in (the same grid, phases and
 *                                  initial state as the reference's set-up)
 *   gb300_sync_to_host(theDomain)  before possiblyOutput()/report(): copies
 *                                  positions, primitives, conserved state,
 *                                  face fluxes (CT), the point masses and the
 *                                  ring diagnostics into theDomain
 *   gb300_zero_diagnostics()       after the output step's zero_diagnostics
 *   gb300_output(theDomain, name)  in place of output() (h5out.c:366) when
 *                                  the build has no HDF5 library: writes
 *                                  <name>.h5 in output()'s layout from the
 *                                  device state
 *   gb300_free()                   before freeDomain
 *
 * With Restart = 1 in in.par, gb300_init builds the device instance from
 * input.h5 (the file restart() reads, h5in.c:116) as the library's
 * checkpoint reader understands it.
 *
 * The build compiles the reference's misc.c and timestep.c with their own
 * definitions renamed out of the way (-Dgetmindt=... for misc.c,
 * -Dtimestep=... for timestep.c; oracle/ref/Makefile, target gb300) and
 * links -ldisco_gb300.  GB300_PRECISION (0 plain FP64, 1 mixed; default 0)
 * selects the device path.
 */
#include <stdio.h>
#include <stdlib.h>

#include "paul.h"
#include "disco_gpu.h"
#include "disco_gpu_diag.h"
#include "disco_gpu_checkpoint.h"

#ifndef GB300_PRECISION
#define GB300_PRECISION 0
#endif

static disco_gpu *G = NULL;
static disco_host_domain *H = NULL;

/* the library returns 0 or a count on success, a negative code on error */
static void gb300_check(int rc, const char *what)
{
   if(rc < 0) {
      fprintf(stderr, "gb300: %s failed (%d): %s\n", what, rc, disco_last_error());
      exit(1);
   }
}

void gb300_init(struct domain *theDomain)
{
   disco_params p;
   disco_modules m;
   gb300_check(disco_params_read("in.par", &p), "disco_params_read");
   gb300_check(disco_modules_read("Makefile_opt.in", &m), "disco_modules_read");
   if(p.restart_flag) {
      gb300_check(disco_host_restart(&p, &m, "input.h5", &H), "disco_host_restart");
      /* what restart() sets in theDomain (h5in.c:135-160, :303-318); the
       * cells follow at the first gb300_sync_to_host */
      theDomain->t = H->t;
      for(int q = 0; q < H->Npl && q < theDomain->Npl; ++q) {
         struct planet *P = &theDomain->thePlanets[q];
         P->r = H->planets[q].r; P->phi = H->planets[q].phi; P->M = H->planets[q].M;
         P->omega = H->planets[q].omega; P->vr = H->planets[q].vr; P->eps = H->planets[q].eps;
      }
   } else {
      gb300_check(disco_host_setup(&p, &m, &H), "disco_host_setup");
   }
   if(H->Nr != theDomain->Nr || H->Nz != theDomain->Nz) {
      fprintf(stderr, "gb300: grid differs from the reference's set-up\n");
      exit(1);
   }
   gb300_check(disco_gpu_create(H, GB300_PRECISION, &G), "disco_gpu_create");
}

double getmindt(struct domain *theDomain)
{
   double dt;
   (void)theDomain;
   gb300_check(disco_gpu_getmindt(G, &dt), "disco_gpu_getmindt");
   return dt;
}

void timestep(struct domain *theDomain, double dt)
{
   gb300_check(disco_gpu_timestep(G, dt), "disco_gpu_timestep");
   theDomain->t += dt;                      /* timestep.c:32-47 */
   theDomain->count_steps += 1;             /* timestep.c:52 */
}

void gb300_sync_to_host(struct domain *theDomain)
{
   long N = disco_gpu_num_cells(G);
   int nq = H->num_q, nf = H->num_faces;
   disco_state_view v = {0};
   v.piph = malloc(N*sizeof(double));
   v.dphi = malloc(N*sizeof(double));
   v.wiph = malloc(N*sizeof(double));
   v.prim = malloc((size_t)nq*N*sizeof(double));
   v.cons = malloc((size_t)nq*N*sizeof(double));
   v.Phi = nf > 0 ? calloc((size_t)nf*N, sizeof(double)) : NULL;
   gb300_check(disco_gpu_download(G, &v), "disco_gpu_download");
   for(int jk = 0; jk < theDomain->Nr*theDomain->Nz; ++jk)
      for(int i = 0; i < theDomain->Np[jk]; ++i) {
         long c = H->ring_off[jk] + i;
         struct cell *cl = &theDomain->theCells[jk][i];
         cl->piph = v.piph[c];
         cl->dphi = v.dphi[c];
         cl->wiph = v.wiph[c];
         for(int q = 0; q < nq; ++q) {
            cl->prim[q] = v.prim[(size_t)q*N + c];
            cl->cons[q] = v.cons[(size_t)q*N + c];
         }
         for(int f = 0; f < nf && f < NUM_FACES; ++f)   /* h5out.c:77-85 writes Phi */
            cl->Phi[f] = v.Phi[(size_t)f*N + c];
      }
   free(v.piph); free(v.dphi); free(v.wiph); free(v.prim); free(v.cons); free(v.Phi);
   /* the point masses (report.c, h5out.c read theDomain->thePlanets) */
   disco_planet pl[DISCO_MAX_PLANETS];
   int npl = 0;
   gb300_check(disco_gpu_planets(G, pl, DISCO_MAX_PLANETS, &npl), "disco_gpu_planets");
   for(int p = 0; p < npl && p < theDomain->Npl && p < DISCO_MAX_PLANETS; ++p) {
      struct planet *P = &theDomain->thePlanets[p];
      P->r = pl[p].r; P->phi = pl[p].phi; P->M = pl[p].M;
      P->omega = pl[p].omega; P->vr = pl[p].vr; P->eps = pl[p].eps;
   }
   /* the ring diagnostics timestep() accumulated, for avg_diagnostics */
   int nd = disco_gpu_diag_count(G);
   if(nd > 0)
      gb300_check(disco_gpu_diag_download(G, theDomain->theTools.Qrz,
                                          (long long)theDomain->Nr*theDomain->Nz*nd,
                                          &theDomain->theTools.t_avg), "disco_gpu_diag_download");
}

void gb300_output(struct domain *theDomain, const char *filestart)
{
   char fname[512];
   (void)theDomain;
   snprintf(fname, sizeof fname, "%s.h5", filestart);   /* h5out.c:392 */
   gb300_check(disco_gpu_checkpoint(G, H, fname), "disco_gpu_checkpoint");
}

void gb300_zero_diagnostics(void)
{
   gb300_check(disco_gpu_diag_upload(G, NULL, 0, 0.0), "disco_gpu_diag_upload");
}

void gb300_free(void)
{
   disco_gpu_free(G);
   disco_host_free(H);
   G = NULL;
   H = NULL;
}
