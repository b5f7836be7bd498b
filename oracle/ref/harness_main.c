/*
 * CHECKER INFRASTRUCTURE (oracle).  Not product code.
 *
 * Replacement main() linked against the reference's own objects (built from
 * the reference sources, out of tree, by oracle/ref/Makefile).  It performs
 * the same initialisation as the reference main (main.c:27-61) and then
 * either dumps state, dumps the reconstruction/face tables of the initial
 * state, or advances exactly N timesteps with the reference hot loop
 * (main.c:68-74: getmindt -> timestep; check_dt/possiblyOutput are skipped so
 * that exactly N steps run) and dumps the result.
 *
 * Usage (in a directory holding in.par):
 *    disco_ref init  OUT.bin
 *    disco_ref grad  OUT.bin          (plm_phi + faces + plm_trans, then dump)
 *    disco_ref run N OUT.bin          (N full RK steps, then dump, then the
 *                                      reference's report() into report.dat)
 *    disco_ref time N [W]             (W untimed warm-up steps, then N timed
 *                                      steps; prints zone-updates/s only)
 *
 * Dump format: little-endian raw, see write_state() / write_faces();
 * tests/golden/dumpio.py reads it.
 */
#include "paul.h"
#include <time.h>

#ifdef GB300
/* the reference-side binding of libdisco_gb300 (gb300_shim.c): getmindt
 * and timestep run on the GPU; these hooks create the device instance and
 * copy its state back before anything reads theDomain */
void gb300_init(struct domain *);
void gb300_sync_to_host(struct domain *);
void gb300_output(struct domain *, const char *);
void gb300_free(void);
#define GB300_INIT(d) gb300_init(d)
#define GB300_SYNC(d) gb300_sync_to_host(d)
#define GB300_OUTPUT(d, name) gb300_output(d, name)
#else
#define GB300_INIT(d) ((void)0)
#define GB300_SYNC(d) ((void)0)
#define GB300_OUTPUT(d, name) ((void)0)
#endif

int mpiSetup(struct domain *, int, char *[]);
void setupGrid(struct domain *);
void timestep(struct domain *, double);
void setupCells(struct domain *);
void boundary_trans(struct domain *, int);
void exchangeData(struct domain *, int);
double getmindt(struct domain *);
int read_par_file(struct domain *);
void setupDomain(struct domain *);
void freeDomain(struct domain *);
void plm_phi(struct domain *);
void setup_faces(struct domain *, int);
void plm_trans(struct domain *, struct face *, int, int);
void report(struct domain *);

#define DUMP_MAGIC 0x4f435344  /* "DSCO" */

static void wi(FILE *f, int v) { fwrite(&v, sizeof(int), 1, f); }
static void wd(FILE *f, double v) { fwrite(&v, sizeof(double), 1, f); }

static long total_cells(struct domain *d)
{
   long n = 0;
   int jk;
   for(jk = 0; jk < d->Nr*d->Nz; jk++) n += d->Np[jk];
   return n;
}

/* Header + grid + per-cell SoA arrays. */
static void write_state(struct domain *d, FILE *f, int with_grad)
{
   int Nr = d->Nr, Nz = d->Nz, jk, i, q;
   long N = total_cells(d);
   wi(f, DUMP_MAGIC); wi(f, 1);
   wi(f, Nr); wi(f, Nz); wi(f, d->NgRa); wi(f, d->NgRb); wi(f, d->NgZa);
   wi(f, d->NgZb); wi(f, NUM_Q); wi(f, NUM_FACES); wi(f, (int)N);
   wi(f, with_grad);
   wd(f, d->t); wd(f, d->phi_max);
   for(jk = 0; jk < Nr*Nz; jk++) wi(f, d->Np[jk]);
   for(i = -1; i < Nr; i++) wd(f, d->r_jph[i]);
   for(i = -1; i < Nz; i++) wd(f, d->z_kph[i]);
#define PER_CELL(EXPR) \
   for(jk = 0; jk < Nr*Nz; jk++) for(i = 0; i < d->Np[jk]; i++) { \
      struct cell *c = &d->theCells[jk][i]; (void)c; EXPR; }
   PER_CELL(wd(f, c->piph));
   PER_CELL(wd(f, c->dphi));
   PER_CELL(wd(f, c->wiph));
   PER_CELL(wi(f, c->real));
   for(q = 0; q < NUM_Q; q++) PER_CELL(wd(f, c->prim[q]));
   for(q = 0; q < NUM_Q; q++) PER_CELL(wd(f, c->cons[q]));
   for(q = 0; q < NUM_FACES; q++) PER_CELL(wd(f, c->Phi[q]));
   if(with_grad) {
      for(q = 0; q < NUM_Q; q++) PER_CELL(wd(f, c->gradp[q]));
      for(q = 0; q < NUM_Q; q++) PER_CELL(wd(f, c->gradr[q]));
      for(q = 0; q < NUM_Q; q++) PER_CELL(wd(f, c->gradz[q]));
   }
#undef PER_CELL
}

/* Locate a cell pointer as (jk, i). */
static void locate(struct domain *d, struct cell *c, int *jk_out, int *i_out)
{
   int jk;
   for(jk = 0; jk < d->Nr*d->Nz; jk++) {
      struct cell *b = d->theCells[jk];
      if(c >= b && c < b + d->Np[jk]) { *jk_out = jk; *i_out = (int)(c - b); return; }
   }
   *jk_out = -1; *i_out = -1;
}

static void write_faces(struct domain *d, FILE *f, int dim)
{
   int NN = dim == 1 ? d->N_ftracks_r : d->N_ftracks_z;
   int *fI = dim == 1 ? d->fIndex_r : d->fIndex_z;
   struct face *F = dim == 1 ? d->theFaces_1 : d->theFaces_2;
   int n, k;
   wi(f, dim); wi(f, NN);
   for(k = 0; k <= NN; k++) wi(f, fI[k]);
   int Nf = fI[NN];
   for(n = 0; n < Nf; n++) {
      int a, b, c2, e;
      locate(d, F[n].L, &a, &b);
      locate(d, F[n].R, &c2, &e);
      wi(f, a); wi(f, b); wi(f, c2); wi(f, e); wi(f, F[n].LRtype);
   }
   for(n = 0; n < Nf; n++) {
      wd(f, F[n].cm[0]); wd(f, F[n].cm[1]); wd(f, F[n].cm[2]);
      wd(f, F[n].dphi); wd(f, F[n].dA); wd(f, F[n].dl);
      wd(f, F[n].dxL); wd(f, F[n].dxR);
   }
}

static void init_domain(struct domain *d, int argc, char **argv)
{
   read_par_file(d);
   mpiSetup(d, argc, argv);
   setupGrid(d);
   setupDomain(d);
   setupCells(d);
   if(d->Nr > 1) {
      exchangeData(d, 0);
      if(!d->theParList.R_Periodic) boundary_trans(d, 1);
   }
   if(d->Nz > 1) {
      exchangeData(d, 1);
      if(!d->theParList.Z_Periodic) boundary_trans(d, 2);
   }
}

static double now_s(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return ts.tv_sec + 1e-9*ts.tv_nsec;
}

int main(int argc, char **argv)
{
   if(argc < 3) {
      fprintf(stderr, "usage: %s init|grad OUT | run N OUT | time N\n", argv[0]);
      return 2;
   }
   struct domain theDomain = {0};
   struct domain *d = &theDomain;
   init_domain(d, 1, argv);
   GB300_INIT(d);

   const char *mode = argv[1];
   if(strcmp(mode, "init") == 0) {
      FILE *f = fopen(argv[2], "wb");
      write_state(d, f, 0);
      fclose(f);
   } else if(strcmp(mode, "grad") == 0) {
      plm_phi(d);
      if(d->Nr > 1) {
         setup_faces(d, 1);
         plm_trans(d, d->theFaces_1, d->fIndex_r[d->N_ftracks_r], 1);
      }
      if(d->Nz > 1) {
         setup_faces(d, 2);
         plm_trans(d, d->theFaces_2, d->fIndex_z[d->N_ftracks_z], 2);
      }
      FILE *f = fopen(argv[2], "wb");
      write_state(d, f, 1);
      if(d->Nr > 1) write_faces(d, f, 1); else { wi(f, 0); }
      if(d->Nz > 1) write_faces(d, f, 2); else { wi(f, 0); }
      fclose(f);
   } else if(strcmp(mode, "run") == 0 || strcmp(mode, "time") == 0) {
      int nsteps = atoi(argv[2]);
      long ncells = 0;
      int j, k, s;
      for(k = d->NgZa; k < d->Nz - d->NgZb; k++)
         for(j = d->NgRa; j < d->Nr - d->NgRb; j++) ncells += d->Np[j + d->Nr*k];
      if(strcmp(mode, "time") == 0 && argc > 3) {
         int nwarm = atoi(argv[3]);
         for(s = 0; s < nwarm; s++) {
            double dt = getmindt(d);
            timestep(d, dt);
         }
      }
      double t0 = now_s();
      for(s = 0; s < nsteps; s++) {
         double dt = getmindt(d);
         timestep(d, dt);
      }
      double t1 = now_s();
      fprintf(stderr, "{\"cells\": %ld, \"steps\": %d, \"seconds\": %.6f, "
              "\"zone_updates_per_s\": %.6e}\n", ncells, nsteps, t1 - t0,
              (double)ncells*nsteps/(t1 - t0));
      GB300_SYNC(d);
      if(strcmp(mode, "run") == 0) {
         FILE *f = fopen(argv[3], "wb");
         write_state(d, f, 0);
         fclose(f);
         /* the bodies and their sink accumulators, before report() prints
          * and zeroes them: int32 Npl, then per body r, phi, M, omega, vr,
          * eps, gravL, dM, accL, Ls, kin, therm, linXmom, linYmom */
         FILE *pf = fopen("planets.bin", "wb");
         int npl = d->Npl, p;
         fwrite(&npl, sizeof npl, 1, pf);
         for(p = 0; p < npl; p++) {
            struct planet *b = d->thePlanets + p;
            double v[14] = {b->r, b->phi, b->M, b->omega, b->vr, b->eps, b->gravL, b->dM, b->accL,
                            b->Ls, b->kin, b->therm, b->linXmom, b->linYmom};
            fwrite(v, sizeof(double), 14, pf);
         }
         fclose(pf);
         /* the reference's own diagnostics of the final state: one line
          * appended to report.dat in the working directory */
         report(d);
         /* the ring diagnostics timestep() accumulated (analysis.c):
          * int32 num_tools, int32 Nr*Nz, double t_avg, double Qrz[] */
         FILE *g = fopen("diag.bin", "wb");
         int nq = d->num_tools, nring = d->Nr * d->Nz;
         fwrite(&nq, sizeof nq, 1, g);
         fwrite(&nring, sizeof nring, 1, g);
         fwrite(&d->theTools.t_avg, sizeof(double), 1, g);
         fwrite(d->theTools.Qrz, sizeof(double), (size_t)nq * nring, g);
         fclose(g);
         /* with the binding: the checkpoint of output() written by the
          * library from the device state (checkpoint_gb300.h5) */
         GB300_OUTPUT(d, "checkpoint_gb300");
      }
   } else {
      fprintf(stderr, "unknown mode %s\n", mode);
      return 2;
   }
   return 0;
}
