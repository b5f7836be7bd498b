/*
 * Checkpoint output and restart in the layout of the reference's
 * Output/h5out.c (output, :366-620; writeOpts :98-166; writePars :168-364)
 * and Restart/h5in.c (restart, :100-354), serial case, on the HDF5 subset
 * of h5lite.c.
 */
#include "disco_gpu.h"
#include "disco_gpu_checkpoint.h"
#include "disco_gpu_diag.h"
#include "disco_host_internal.h"
#include "h5lite.h"

#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The state a checkpoint holds, as host arrays (structure of arrays). */
typedef struct {
   const disco_host_domain *dom;     /* grid, parameters, modules */
   const double *prim, *Phi, *piph, *dphi;
   double t;
   const disco_planet *pl;
   int npl;
   const double *Qrz;                /* [Nr*Nz*ntools], already averaged */
   int ntools;
} ck_state;

/* writePars (h5out.c:168-364): in.par name, type, field. */
typedef struct { const char *name; int type; size_t off; } par_entry;
#define PI_(N, F) { N, H5L_I32, offsetof(disco_params, F) }
#define PD_(N, F) { N, H5L_F64, offsetof(disco_params, F) }
static const par_entry kPars[] = {
   PI_("Num_R", Num_R), PI_("Num_Z", Num_Z), PD_("aspect", aspect),
   PI_("Num_Reports", NumRepts), PI_("Num_Snapshots", NumSnaps), PI_("Num_Checkpoints", NumChecks),
   PD_("T_Start", t_min), PD_("T_End", t_max),
   PD_("R_Min", rmin), PD_("R_Max", rmax), PD_("Z_Min", zmin), PD_("Z_Max", zmax),
   PD_("Phi_Max", phimax),
   PI_("Use_Logtime", Out_LogTime), PI_("Log_Zoning", LogZoning),
   PI_("R_Periodic", R_Periodic), PI_("Z_Periodic", Z_Periodic),
   PI_("NoBC_Rmin", NoBC_Rmin), PI_("NoBC_Rmax", NoBC_Rmax),
   PI_("NoBC_Zmin", NoBC_Zmin), PI_("NoBC_Zmax", NoBC_Zmax),
   PD_("Log_Radius", LogRadius), PD_("Max_Aspect_Short", MaxShort), PD_("Max_Aspect_Long", MaxLong),
   PD_("CFL", CFL), PD_("PLM", PLM), PD_("Max_DT", maxDT),
   PD_("Adiabatic_Index", Adiabatic_Index), PI_("Isothermal", isothermal_flag),
   PI_("Cs2_Profile", Cs2_Profile), PD_("Cs2_Par", Cs2_Par),
   PD_("Density_Floor", Density_Floor), PD_("Pressure_Floor", Pressure_Floor),
   PI_("Mesh_Motion", Mesh_Motion), PI_("Riemann_Solver", Riemann_Solver),
   PI_("Initial_Regrid", Initial_Regrid), PI_("Restart", restart_flag),
   PI_("Exact_Mesh_Omega", Exact_Mesh_Omega), PD_("Exact_Mesh_Omega_Par", Exact_Mesh_Omega_Par),
   PI_("Energy_Omega", Energy_Omega), PD_("Energy_Omega_Par", Energy_Omega_Par),
   PI_("RotFrame", RotFrame), PD_("RotOmega", RotOmega), PD_("RotD", RotD),
   PI_("Use_Viscosity", visc_flag), PD_("Viscosity", viscosity), PI_("Use_As_Alpha", alpha_flag),
   PI_("Include_Atmos", include_atmos), PD_("Mach_Number", Disk_Mach), PD_("Mass_Ratio", Mass_Ratio),
   PD_("Eccentricity", Eccentricity), PD_("Drift_Rate", Drift_Rate), PD_("Drift_Exp", Drift_Exp),
   PI_("Constrained_Transport", CT),
   PI_("Metric_Par0", metricPar0), PD_("Metric_Par1", metricPar1), PD_("Metric_Par2", metricPar2),
   PD_("Metric_Par3", metricPar3), PD_("Metric_Par4", metricPar4),
   PI_("Init_Par0", initPar0), PD_("Init_Par1", initPar1), PD_("Init_Par2", initPar2),
   PD_("Init_Par3", initPar3), PD_("Init_Par4", initPar4), PD_("Init_Par5", initPar5),
   PD_("Init_Par6", initPar6), PD_("Init_Par7", initPar7), PD_("Init_Par8", initPar8),
   PI_("Noise_Type", noiseType), PD_("Noise_Abs", noiseAbs), PD_("Noise_Rel", noiseRel),
   PI_("Sink_Type", sinkType), PD_("Sink_Par1", sinkPar1), PD_("Sink_Par2", sinkPar2),
   PD_("Sink_Par3", sinkPar3), PD_("Sink_Par4", sinkPar4), PD_("Sink_Par5", sinkPar5),
   PI_("Nozzle_Type", nozzleType), PD_("Nozzle_Par1", nozzlePar1), PD_("Nozzle_Par2", nozzlePar2),
   PD_("Nozzle_Par3", nozzlePar3), PD_("Nozzle_Par4", nozzlePar4),
   PI_("Cool_Type", coolType), PD_("Cool_Par1", coolPar1), PD_("Cool_Par2", coolPar2),
   PD_("Cool_Par3", coolPar3), PD_("Cool_Par4", coolPar4),
   PD_("Softening", grav_eps),
};
#undef PI_
#undef PD_

#define NPDAT 7   /* planet columns, h5out.c:385 */

static int ck_write(const ck_state *s, const char *path)
{
   const disco_host_domain *d = s->dom;
   const long N = d->Ncell;
   const int Nr = d->Nr, Nz = d->Nz, nq = d->num_q, nf = d->num_faces, nd = nq + nf + 1;
   const int nring = Nr*Nz;
   int rc = DISCO_OK;
   double *cells = (double *)malloc(sizeof(double)*(size_t)(N > 0 ? N : 1)*(size_t)nd);
   int *index = (int *)malloc(sizeof(int)*(size_t)nring);
   int *np = (int *)malloc(sizeof(int)*(size_t)nring);
   int *id0 = (int *)malloc(sizeof(int)*(size_t)nring);
   double *pdat = (double *)malloc(sizeof(double)*(size_t)(s->npl > 0 ? s->npl : 1)*NPDAT);
   h5w *w = h5w_create();
   if(!cells || !index || !np || !id0 || !pdat || !w) { rc = DISCO_E_NOMEM; goto done; }
   if(N > 0x7fffffffL) { disco_set_error("checkpoint: more cells than an int32 Index holds"); rc = DISCO_E_ARG; goto done; }

   /* Cell2Doub (h5out.c:79-88) and the ring tables (h5out.c:529-549) */
   for(long c = 0; c < N; c++) {
      double *row = cells + (size_t)c*(size_t)nd;
      for(int q = 0; q < nq; q++) row[q] = s->prim[(size_t)q*(size_t)N + (size_t)c];
      for(int f = 0; f < nf; f++) row[nq + f] = s->Phi ? s->Phi[(size_t)f*(size_t)N + (size_t)c] : 0.0;
      row[nq + nf] = s->piph[c];
   }
   for(int jk = 0; jk < nring; jk++) {
      const long c0 = d->ring_off[jk];
      index[jk] = (int)c0;
      np[jk] = d->Np[jk];
      double phi0 = M_PI;
      int id = 0;
      for(int i = 0; i < d->Np[jk]; i++) {
         const double phi = s->piph[c0 + i] - .5*s->dphi[c0 + i];
         if(cos(phi0) < cos(phi)) { phi0 = phi; id = (int)(c0 + i); }
      }
      id0[jk] = id;
   }
   for(int p = 0; p < s->npl; p++) {   /* h5out.c:461-472 */
      double *row = pdat + (size_t)p*NPDAT;
      row[0] = s->pl[p].M; row[1] = s->pl[p].vr; row[2] = s->pl[p].omega;
      row[3] = s->pl[p].r; row[4] = s->pl[p].phi; row[5] = s->pl[p].eps;
      row[6] = (double)s->pl[p].type;
   }

   int g_grid = h5w_group(w, "Grid"), g_data = h5w_group(w, "Data");
   int g_opts = h5w_group(w, "Opts"), g_pars = h5w_group(w, "Pars");
   if(g_grid < 0 || g_data < 0 || g_opts < 0 || g_pars < 0) { rc = DISCO_E_NOMEM; goto done; }
   uint64_t one = 1, dr = (uint64_t)Nr + 1, dz = (uint64_t)Nz + 1;
   uint64_t d2[2] = {(uint64_t)Nz, (uint64_t)Nr};
   uint64_t dc[2] = {(uint64_t)N, (uint64_t)nd};
   uint64_t dp[2] = {(uint64_t)s->npl, NPDAT};
   uint64_t d3[3] = {(uint64_t)Nz, (uint64_t)Nr, (uint64_t)s->ntools};
   int e = 0;
   e |= h5w_dataset(w, g_grid, "T", H5L_F64, 1, &one, &s->t);
   e |= h5w_dataset(w, g_grid, "r_jph", H5L_F64, 1, &dr, d->r_jph);
   e |= h5w_dataset(w, g_grid, "z_kph", H5L_F64, 1, &dz, d->z_kph);
   e |= h5w_dataset(w, g_grid, "Index", H5L_I32, 2, d2, index);
   e |= h5w_dataset(w, g_grid, "Np", H5L_I32, 2, d2, np);
   e |= h5w_dataset(w, g_grid, "Id_phi0", H5L_I32, 2, d2, id0);
   e |= h5w_dataset(w, g_data, "Cells", H5L_F64, 2, dc, cells);
   e |= h5w_dataset(w, g_data, "Planets", H5L_F64, 2, dp, pdat);
   e |= h5w_dataset(w, g_data, "Diagnostics", H5L_F64, 3, d3, s->Qrz);

   /* writeOpts (h5out.c:98-166) */
   const disco_modules *m = &d->mod;
   static const char *git = "disco_gb300";
   const char *opt_names[] = {"INITIAL", "HYDRO", "GEOMETRY", "BOUNDARY", "OUTPUT", "RESTART",
                              "PLANETS", "HLLD", "ANALYSIS", "METRIC", "FRAME"};
   const char *opt_vals[11] = {m->initial_name, m->hydro_name, m->geometry_name, m->boundary_name,
                               m->output_name, m->restart_name, m->planets_name, m->hlld_name,
                               m->analysis_name, m->metric_name, m->frame_name};
   e |= h5w_dataset(w, 0, "GIT_VERSION", H5L_VSTR, 1, &one, &git);
   for(int i = 0; i < 11; i++) e |= h5w_dataset(w, g_opts, opt_names[i], H5L_VSTR, 1, &one, &opt_vals[i]);
   e |= h5w_dataset(w, g_opts, "NUM_C", H5L_I32, 1, &one, &m->num_c);
   e |= h5w_dataset(w, g_opts, "NUM_N", H5L_I32, 1, &one, &m->num_n);
   e |= h5w_dataset(w, g_opts, "CT_MODE", H5L_I32, 1, &one, &m->ct_mode);
   for(size_t i = 0; i < sizeof kPars/sizeof kPars[0]; i++)
      e |= h5w_dataset(w, g_pars, kPars[i].name, kPars[i].type, 1, &one,
                       (const char *)&d->par + kPars[i].off);
   if(e) { disco_set_error("checkpoint: dataset declaration failed"); rc = DISCO_E_ARG; goto done; }
   {
      int wr = h5w_close(w, path);
      w = NULL;
      if(wr) {
         char msg[300];
         snprintf(msg, sizeof msg, "checkpoint: cannot write %s (%d)", path, wr);
         disco_set_error(msg);
         rc = DISCO_E_PARFILE;
      }
   }
done:
   h5w_abort(w);
   free(cells); free(index); free(np); free(id0); free(pdat);
   return rc;
}

int disco_host_checkpoint(const disco_host_domain *dom, const char *path)
{
   if(!dom || !path) { disco_set_error("disco_host_checkpoint: null argument"); return DISCO_E_ARG; }
   ck_state s = {dom, dom->prim, dom->Phi, dom->piph, dom->dphi, dom->t, dom->planets, dom->Npl, NULL, 0};
   if(dom->num_faces && !dom->Phi) {   /* no field yet: zero face fluxes */
      double *z = (double *)calloc((size_t)dom->num_faces*(size_t)(dom->Ncell > 0 ? dom->Ncell : 1), sizeof(double));
      if(!z) return DISCO_E_NOMEM;
      s.Phi = z;
      int rc = ck_write(&s, path);
      free(z);
      return rc;
   }
   return ck_write(&s, path);
}

int disco_gpu_checkpoint(disco_gpu *g, const disco_host_domain *dom, const char *path)
{
   if(!g || !dom || !path) { disco_set_error("disco_gpu_checkpoint: null argument"); return DISCO_E_ARG; }
   const long N = disco_gpu_num_cells(g);
   if(N != dom->Ncell) { disco_set_error("disco_gpu_checkpoint: the domain's grid is not the instance's"); return DISCO_E_ARG; }
   const int nq = dom->num_q, nf = dom->num_faces, nring = dom->Nr*dom->Nz;
   int rc = DISCO_OK;
   double *prim = (double *)malloc(sizeof(double)*(size_t)nq*(size_t)N);
   double *piph = (double *)malloc(sizeof(double)*(size_t)N);
   double *dphi = (double *)malloc(sizeof(double)*(size_t)N);
   double *Phi = nf ? (double *)malloc(sizeof(double)*(size_t)nf*(size_t)N) : NULL;
   double *Qrz = NULL;
   disco_planet pl[DISCO_MAX_PLANETS];
   int npl = 0;
   if(!prim || !piph || !dphi || (nf && !Phi)) { rc = DISCO_E_NOMEM; goto done; }
   disco_state_view v;
   memset(&v, 0, sizeof v);
   v.prim = prim; v.piph = piph; v.dphi = dphi; v.Phi = Phi;
   if((rc = disco_gpu_download(g, &v)) != 0) goto done;
   if((rc = disco_gpu_planets(g, pl, DISCO_MAX_PLANETS, &npl)) != 0) goto done;
   if(npl > DISCO_MAX_PLANETS) npl = DISCO_MAX_PLANETS;
   int nt = disco_gpu_diag_count(g);
   if(nt < 0) { rc = nt; goto done; }
   double t_avg = 0.0;
   if(nt > 0) {
      const long long len = (long long)nring*nt;
      Qrz = (double *)malloc(sizeof(double)*(size_t)len);
      if(!Qrz) { rc = DISCO_E_NOMEM; goto done; }
      if((rc = disco_gpu_diag_download(g, Qrz, len, &t_avg)) < 0) goto done;
      for(long long i = 0; i < len; i++) Qrz[i] /= t_avg;   /* avg_diagnostics, analysis.c:29-49 */
   }
   {
      ck_state s = {dom, prim, Phi, piph, dphi, v.t, pl, npl, Qrz, nt};
      if((rc = ck_write(&s, path)) != 0) goto done;
   }
   if(nt > 0) {   /* zero_diagnostics (h5out.c:610) */
      int u = disco_gpu_diag_upload(g, NULL, (long long)nring*nt, 0.0);
      rc = u < 0 ? u : DISCO_OK;
   }
done:
   free(prim); free(piph); free(dphi); free(Phi); free(Qrz);
   return rc;
}

static int rs_fail(h5r *r, disco_host_domain *d, disco_host_domain *g0, const char *path, const char *what)
{
   char msg[400];
   snprintf(msg, sizeof msg, "disco_host_restart: %s: %s", path, what);
   disco_set_error(msg);
   h5r_close(r);
   disco_host_free(d);
   disco_host_free(g0);
   return DISCO_E_PARFILE;
}

int disco_host_restart(const disco_params *par, const disco_modules *mod,
                       const char *path, disco_host_domain **out)
{
   if(!par || !mod || !path || !out) { disco_set_error("disco_host_restart: null argument"); return DISCO_E_ARG; }
   /* setupGrid + setupDomain on in.par's grid come first in the reference
    * (main.c:43-44), so the noise of setupCells draws after their phases */
   disco_rand_state rs;
   disco_host_domain *g0 = NULL, *d = NULL;
   int rc = disco_host_grid(par, mod, &g0, &rs);
   if(rc) return rc;
   char err[300];
   h5r *r = h5r_open(path, err, sizeof err);
   if(!r) { disco_set_error(err); disco_host_free(g0); return DISCO_E_PARFILE; }
   uint64_t dims[3];
   int ty;
   double T;
   if(h5r_read(r, "Grid/T", H5L_F64, 0, -1, &T) != 1) return rs_fail(r, d, g0, path, "no Grid/T");
   if(h5r_dims(r, "Grid/Index", dims, 2, &ty) != 2) return rs_fail(r, d, g0, path, "no Grid/Index");
   const int Ng = DISCO_NUM_G;
   const int Nz_tot = (int)dims[0], Nr_tot = (int)dims[1];
   /* h5in.c:150-157 */
   int NUM_R = Nr_tot, NUM_Z = Nz_tot;
   if(!par->NoBC_Rmin) NUM_R -= Ng;
   if(!par->NoBC_Rmax) NUM_R -= Ng;
   if(Nz_tot > 1 && !par->NoBC_Zmin) NUM_Z -= Ng;
   if(Nz_tot > 1 && !par->NoBC_Zmax) NUM_Z -= Ng;
   if(NUM_R < 1 || NUM_Z < 1) return rs_fail(r, d, g0, path, "grid too small for its ghost rings");

   d = (disco_host_domain *)calloc(1, sizeof(*d));
   if(!d) return rs_fail(r, d, g0, path, "out of memory");
   d->par = *par;
   d->par.Num_R = NUM_R;
   d->par.Num_Z = NUM_Z;
   d->mod = *mod;
   d->num_q = g0->num_q;
   d->num_faces = g0->num_faces;
   d->NgRa = par->NoBC_Rmin ? 0 : Ng;
   d->NgRb = par->NoBC_Rmax ? 0 : Ng;
   d->NgZa = (NUM_Z == 1 || par->NoBC_Zmin) ? 0 : Ng;
   d->NgZb = (NUM_Z == 1 || par->NoBC_Zmax) ? 0 : Ng;
   d->Nr = NUM_R + d->NgRa + d->NgRb;
   d->Nz = NUM_Z + d->NgZa + d->NgZb;
   if(d->Nr != Nr_tot || d->Nz != Nz_tot) return rs_fail(r, d, g0, path, "ring counts inconsistent with NoBC_*");
   const int Nr = d->Nr, Nz = d->Nz, nring = Nr*Nz;
   d->Np = (int *)malloc(sizeof(int)*(size_t)nring);
   d->ring_off = (long *)malloc(sizeof(long)*(size_t)(nring + 1));
   d->r_jph = (double *)malloc(sizeof(double)*(size_t)(Nr + 1));
   d->z_kph = (double *)malloc(sizeof(double)*(size_t)(Nz + 1));
   int *index = (int *)malloc(sizeof(int)*(size_t)nring);
   if(!d->Np || !d->ring_off || !d->r_jph || !d->z_kph || !index) {
      free(index);
      return rs_fail(r, d, g0, path, "out of memory");
   }
   if(h5r_dims(r, "Grid/r_jph", dims, 1, &ty) != 1 || dims[0] != (uint64_t)Nr + 1 ||
      h5r_read(r, "Grid/r_jph", H5L_F64, 0, -1, d->r_jph) != Nr + 1 ||
      h5r_dims(r, "Grid/z_kph", dims, 1, &ty) != 1 || dims[0] != (uint64_t)Nz + 1 ||
      h5r_read(r, "Grid/z_kph", H5L_F64, 0, -1, d->z_kph) != Nz + 1 ||
      h5r_read(r, "Grid/Np", H5L_I32, 0, -1, d->Np) != nring ||
      h5r_read(r, "Grid/Index", H5L_I32, 0, -1, index) != nring) {
      free(index);
      return rs_fail(r, d, g0, path, "bad Grid datasets");
   }
   long off = 0;
   for(int jk = 0; jk < nring; jk++) {
      if(d->Np[jk] < 1) { free(index); return rs_fail(r, d, g0, path, "a ring without cells"); }
      d->ring_off[jk] = off;
      off += d->Np[jk];
   }
   d->ring_off[nring] = off;
   d->Ncell = off;
   const int nq = d->num_q, nf = d->num_faces, nd = nq + nf + 1;
   if(h5r_dims(r, "Data/Cells", dims, 2, &ty) != 2) { free(index); return rs_fail(r, d, g0, path, "no Data/Cells"); }
   if(dims[1] != (uint64_t)nd) {   /* h5in.c:322 */
      free(index);
      return rs_fail(r, d, g0, path, "Data/Cells columns differ from NUM_Q + NUM_FACES + 1");
   }
   const uint64_t nc = dims[0];
   const long N = d->Ncell;
   d->piph = (double *)malloc(sizeof(double)*(size_t)N);
   d->dphi = (double *)malloc(sizeof(double)*(size_t)N);
   d->prim = (double *)malloc(sizeof(double)*(size_t)nq*(size_t)N);
   d->Phi = nf ? (double *)malloc(sizeof(double)*(size_t)nf*(size_t)N) : NULL;
   int maxnp = 0;
   for(int jk = 0; jk < nring; jk++) if(d->Np[jk] > maxnp) maxnp = d->Np[jk];
   double *track = (double *)malloc(sizeof(double)*(size_t)maxnp*(size_t)nd);
   if(!d->piph || !d->dphi || !d->prim || (nf && !d->Phi) || !track) {
      free(index); free(track);
      return rs_fail(r, d, g0, path, "out of memory");
   }
   /* one ring at a time from its Index row (h5in.c:262-284) */
   for(int jk = 0; jk < nring; jk++) {
      const int np = d->Np[jk];
      if(index[jk] < 0 || (uint64_t)index[jk] + (uint64_t)np > nc ||
         h5r_read(r, "Data/Cells", H5L_F64, index[jk], np, track) != (long)np*nd) {
         free(index); free(track);
         return rs_fail(r, d, g0, path, "bad Data/Cells rows");
      }
      const long c0 = d->ring_off[jk];
      for(int i = 0; i < np; i++) {
         const double *row = track + (size_t)i*(size_t)nd;
         for(int q = 0; q < nq; q++) d->prim[(size_t)q*(size_t)N + (size_t)(c0 + i)] = row[q];
         for(int f = 0; f < nf; f++) d->Phi[(size_t)f*(size_t)N + (size_t)(c0 + i)] = row[nq + f];
         d->piph[c0 + i] = row[nq + nf];
      }
   }
   free(index);
   free(track);
   /* calc_dp (misc.c:281-298) */
   d->phi_max = par->phimax;
   for(int jk = 0; jk < nring; jk++) {
      const long c0 = d->ring_off[jk];
      const int np = d->Np[jk];
      for(int i = 0; i < np; i++) {
         const int im = i == 0 ? np - 1 : i - 1;
         double dp = d->piph[c0 + i] - d->piph[c0 + im];
         while(dp > d->phi_max) dp -= d->phi_max;
         while(dp < 0.0) dp += d->phi_max;
         d->dphi[c0 + i] = dp;
      }
   }
   d->t = T;
   /* setPlanetParams + initializePlanets, then the file's values
    * (h5in.c:286-318) */
   d->Npl = g0->Npl;
   memcpy(d->planets, g0->planets, sizeof d->planets);
   memcpy(d->ic_aux, g0->ic_aux, sizeof d->ic_aux);
   if(d->Npl > 0) {
      double pdat[DISCO_MAX_PLANETS*16];
      if(h5r_dims(r, "Data/Planets", dims, 2, &ty) != 2 || dims[0] < (uint64_t)d->Npl || dims[1] < 6 ||
         dims[1] > 16 || h5r_read(r, "Data/Planets", H5L_F64, 0, d->Npl, pdat) != (long)d->Npl*(long)dims[1])
         return rs_fail(r, d, g0, path, "bad Data/Planets");
      for(int p = 0; p < d->Npl; p++) {
         const double *row = pdat + (size_t)p*dims[1];
         d->planets[p].M = row[0]; d->planets[p].vr = row[1]; d->planets[p].omega = row[2];
         d->planets[p].r = row[3]; d->planets[p].phi = row[4]; d->planets[p].eps = row[5];
         d->planets[p].type = 0;   /* PLPOINTMASS */
      }
   }
   h5r_close(r);
   disco_host_free(g0);
   /* setupCells with restart_flag: the noise on the real cells, then the
    * first exchange of periodic ghosts */
   disco_host_cells(d, &rs, 0);
   *out = d;
   return DISCO_OK;
}
