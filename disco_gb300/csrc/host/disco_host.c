/*
 * Host-side set-up of the Disco domain in C: parameter reader, module
 * selection, grid, ring phases and initial primitives.  This is the part of
 * the reference's start-up (main.c:34-47) that runs before the hot path; its
 * output is handed to the device by disco_gpu_create().
 *
 * Integer and FP64 results are bit-identical to the reference's serial build:
 * same formulas in the same order, and the reference's glibc rand() sequence
 * is restated (disco_glibc_rand) so ring phases do not depend on the C
 * library the host links.
 */
#include "disco_gpu.h"
#include "disco_host_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../plugins/ic_vortex_gauss.h"
#include "../plugins/ic_disks.h"
#include "../plugins/ic_fm_torus.h"

/* ------------------------------------------------------------------------
 * Error string shared by the whole library.
 * ---------------------------------------------------------------------- */
static char g_err[512];

void disco_set_error(const char *msg)
{
   strncpy(g_err, msg, sizeof(g_err) - 1);
   g_err[sizeof(g_err) - 1] = 0;
}

const char *disco_last_error(void) { return g_err; }
int disco_abi_version(void) { return DISCO_ABI_VERSION; }

/* ------------------------------------------------------------------------
 * glibc random() TYPE_3 generator (additive feedback, r[i] = r[i-3] +
 * r[i-31] mod 2^32, output r >> 1, first 310 outputs discarded; seeded by a
 * Lehmer sequence 16807*r mod (2^31-1)).  This is the published algorithm
 * behind the rand() the reference calls after srand(314159)
 * (domain.c:172-173, noise.c:372).
 * ---------------------------------------------------------------------- */
void disco_rand_seed(disco_rand_state *st, unsigned int seed)
{
   int32_t r[34];
   int i;
   if(seed == 0) seed = 1;
   r[0] = (int32_t)seed;
   for(i = 1; i < 31; i++) {
      long long v = (16807LL*r[i-1]) % 2147483647LL;
      if(v < 0) v += 2147483647LL;
      r[i] = (int32_t)v;
   }
   for(i = 31; i < 34; i++) r[i] = r[i-31];
   for(i = 0; i < 34; i++) st->r[i] = (uint32_t)r[i];
   st->pos = 0;   /* st->r[pos] is the oldest of the last 34 values */
   for(i = 34; i < 344; i++) (void)disco_rand_next(st);
}

int disco_rand_next(disco_rand_state *st)
{
   /* ring buffer of the last 34 values; new = r[i-31] + r[i-3] */
   int p = st->pos;
   uint32_t v = st->r[(p + 3) % 34] + st->r[(p + 31) % 34];
   st->r[p] = v;
   st->pos = (p + 1) % 34;
   return (int)(v >> 1);
}

#define DISCO_RAND_MAX 2147483647

/* ------------------------------------------------------------------------
 * in.par reader: readvar() semantics of readpar.c:6-42.  The first line
 * whose first whitespace-separated token equals the key wins; the value
 * follows after any of "\t :=>_".  Absent keys leave the field at 0 and
 * count in read_errors.
 * ---------------------------------------------------------------------- */
enum { VAR_INT, VAR_DOUB };

static int readvar(const char *buf, const char *key, int type, void *ptr)
{
   const char *line = buf;
   while(*line) {
      const char *eol = strchr(line, '\n');
      size_t len = eol ? (size_t)(eol - line) : strlen(line);
      char s[512];
      if(len > 510) len = 510;
      memcpy(s, line, len);
      s[len] = 0;
      char nm[512] = "";
      if(sscanf(s, "%511s", nm) == 1 && strcmp(nm, key) == 0) {
         const char *s2 = s + strlen(nm);
         s2 += strspn(s2, "\t :=>_");
         double temp = 0.0;
         if(sscanf(s2, "%lf", &temp) != 1) temp = 0.0;
         if(type == VAR_INT) *(int *)ptr = (int)temp;
         else *(double *)ptr = temp;
         return 0;
      }
      if(!eol) break;
      line = eol + 1;
   }
   return 1;
}

static char *slurp(const char *path)
{
   FILE *f = fopen(path, "rb");
   if(!f) return NULL;
   fseek(f, 0, SEEK_END);
   long n = ftell(f);
   fseek(f, 0, SEEK_SET);
   char *b = (char *)malloc((size_t)n + 1);
   if(!b) { fclose(f); return NULL; }
   size_t got = fread(b, 1, (size_t)n, f);
   b[got] = 0;
   fclose(f);
   return b;
}

int disco_params_read(const char *path, disco_params *p)
{
   if(!path || !p) { disco_set_error("disco_params_read: null argument"); return DISCO_E_ARG; }
   char *b = slurp(path);
   if(!b) { disco_set_error("disco_params_read: cannot open in.par"); return DISCO_E_PARFILE; }
   memset(p, 0, sizeof(*p));
   int err = 0, tTimes_2pi = 0, pTimes_2pi = 0, zTimes_pi = 0;
#define RI(K, F) err += readvar(b, K, VAR_INT, &(p->F))
#define RD(K, F) err += readvar(b, K, VAR_DOUB, &(p->F))
   RI("Num_R", Num_R); RI("Num_Z", Num_Z); RD("aspect", aspect);
   RD("T_Start", t_min); RD("T_End", t_max);
   RD("R_Min", rmin); RD("R_Max", rmax); RD("Z_Min", zmin); RD("Z_Max", zmax);
   RD("Phi_Max", phimax);
   RI("Log_Zoning", LogZoning); RI("R_Periodic", R_Periodic); RI("Z_Periodic", Z_Periodic);
   RI("NoBC_Rmin", NoBC_Rmin); RI("NoBC_Rmax", NoBC_Rmax);
   RI("NoBC_Zmin", NoBC_Zmin); RI("NoBC_Zmax", NoBC_Zmax);
   RD("Log_Radius", LogRadius);
   RI("Timestep", Timestep); RD("CFL", CFL); RD("Max_DT", maxDT); RD("PLM", PLM);
   RD("Adiabatic_Index", Adiabatic_Index); RI("Isothermal", isothermal_flag);
   RI("Cs2_Profile", Cs2_Profile); RD("Cs2_Par", Cs2_Par);
   RD("Density_Floor", Density_Floor); RD("Pressure_Floor", Pressure_Floor);
   RI("Mesh_Motion", Mesh_Motion);
   RI("Exact_Mesh_Omega", Exact_Mesh_Omega); RD("Exact_Mesh_Omega_Par", Exact_Mesh_Omega_Par);
   RI("Energy_Omega", Energy_Omega); RD("Energy_Omega_Par", Energy_Omega_Par);
   RI("RotFrame", RotFrame); RD("RotOmega", RotOmega); RD("RotD", RotD);
   RI("Riemann_Solver", Riemann_Solver);
   RI("Use_Viscosity", visc_flag); RD("Viscosity", viscosity); RI("Use_As_Alpha", alpha_flag);
   err += readvar(b, "T_Times_2pi", VAR_INT, &tTimes_2pi);
   err += readvar(b, "P_Times_2pi", VAR_INT, &pTimes_2pi);
   err += readvar(b, "Z_Times_pi", VAR_INT, &zTimes_pi);
   RD("Mach_Number", Disk_Mach); RD("Mass_Ratio", Mass_Ratio); RI("Grav2D", grav2D);
   RI("Constrained_Transport", CT);
   RI("Metric_Par0", metricPar0); RD("Metric_Par1", metricPar1); RD("Metric_Par2", metricPar2);
   RD("Metric_Par3", metricPar3); RD("Metric_Par4", metricPar4);
   RI("Init_Par0", initPar0); RD("Init_Par1", initPar1); RD("Init_Par2", initPar2);
   RD("Init_Par3", initPar3); RD("Init_Par4", initPar4); RD("Init_Par5", initPar5);
   RD("Init_Par6", initPar6); RD("Init_Par7", initPar7); RD("Init_Par8", initPar8);
   RI("Noise_Type", noiseType); RD("Noise_Abs", noiseAbs); RD("Noise_Rel", noiseRel);
   RI("Sink_Type", sinkType); RI("Nozzle_Type", nozzleType); RI("Cool_Type", coolType);
   RI("DampInner_Type", dampInnerType); RI("DampOuter_Type", dampOuterType);
   RI("DampUpper_Type", dampUpperType); RI("DampLower_Type", dampLowerType);
   RD("Cool_Par1", coolPar1); RD("Cool_Par2", coolPar2); RD("Cool_Par3", coolPar3); RD("Cool_Par4", coolPar4);
   RD("DampInner_Time", dampTimeInner); RD("DampInner_Len", dampLenInner);
   RD("DampOuter_Time", dampTimeOuter); RD("DampOuter_Len", dampLenOuter);
   RD("DampUpper_Time", dampTimeUpper); RD("DampUpper_Len", dampLenUpper);
   RD("DampLower_Time", dampTimeLower); RD("DampLower_Len", dampLenLower);
   RD("Softening", grav_eps);
   RI("Sink_Number", sinkNumber);
   RD("Sink_Par1", sinkPar1); RD("Sink_Par2", sinkPar2); RD("Sink_Par3", sinkPar3);
   RD("Sink_Par4", sinkPar4); RD("Sink_Par5", sinkPar5);
   RD("Nozzle_Par1", nozzlePar1); RD("Nozzle_Par2", nozzlePar2);
   RD("Nozzle_Par3", nozzlePar3); RD("Nozzle_Par4", nozzlePar4);
   RI("Num_Reports", NumRepts); RI("Num_Snapshots", NumSnaps); RI("Num_Checkpoints", NumChecks);
   RI("Use_Logtime", Out_LogTime); RD("Max_Aspect_Short", MaxShort); RD("Max_Aspect_Long", MaxLong);
   RI("Initial_Regrid", Initial_Regrid); RI("Restart", restart_flag); RI("Include_Atmos", include_atmos);
   RD("Eccentricity", Eccentricity); RD("Drift_Rate", Drift_Rate); RD("Drift_Exp", Drift_Exp);
   /* not a reference key: an upper bound on cells per ring (0 = none) */
   { int e0 = err; RI("Max_Np", maxNp); err = e0; }
#undef RI
#undef RD
   free(b);
   /* readpar.c:185-196 */
   if(tTimes_2pi) { p->t_min *= 2.*M_PI; p->t_max *= 2.*M_PI; }
   if(pTimes_2pi) p->phimax *= 2.*M_PI;
   if(zTimes_pi) { p->zmin *= M_PI; p->zmax *= M_PI; }
   p->read_errors = err;
   return DISCO_OK;
}

/* ------------------------------------------------------------------------
 * Makefile_opt.in: "KEY = value  # comment" lines.
 * ---------------------------------------------------------------------- */
static int mk_value(const char *buf, const char *key, char *val, size_t n)
{
   const char *line = buf;
   while(*line) {
      const char *eol = strchr(line, '\n');
      size_t len = eol ? (size_t)(eol - line) : strlen(line);
      char s[512];
      if(len > 510) len = 510;
      memcpy(s, line, len);
      s[len] = 0;
      char *hash = strchr(s, '#');
      if(hash) *hash = 0;
      char k[128] = "", v[128] = "";
      char *eq = strchr(s, '=');
      if(eq) {
         *eq = 0;
         if(sscanf(s, "%127s", k) == 1 && strcmp(k, key) == 0 &&
            sscanf(eq + 1, "%127s", v) == 1) {
            strncpy(val, v, n - 1);
            val[n - 1] = 0;
            return 0;
         }
      }
      if(!eol) break;
      line = eol + 1;
   }
   return 1;
}

int disco_modules_read(const char *path, disco_modules *m)
{
   if(!path || !m) { disco_set_error("disco_modules_read: null argument"); return DISCO_E_ARG; }
   char *b = slurp(path);
   if(!b) { disco_set_error("disco_modules_read: cannot open Makefile_opt.in"); return DISCO_E_PARFILE; }
   memset(m, 0, sizeof(*m));
   char v[128];
   int bad = 0;
   if(mk_value(b, "HYDRO", m->hydro_name, sizeof m->hydro_name)) bad = 1;
   if(mk_value(b, "INITIAL", m->initial_name, sizeof m->initial_name)) bad = 1;
   if(mk_value(b, "BOUNDARY", m->boundary_name, sizeof m->boundary_name)) bad = 1;
   if(mk_value(b, "PLANETS", m->planets_name, sizeof m->planets_name)) bad = 1;
   if(!mk_value(b, "NUM_C", v, sizeof v)) m->num_c = atoi(v); else bad = 1;
   if(!mk_value(b, "NUM_N", v, sizeof v)) m->num_n = atoi(v); else bad = 1;
   if(!mk_value(b, "CT_MODE", v, sizeof v)) m->ct_mode = atoi(v); else bad = 1;
   /* METRIC and FRAME matter to GRMHD only; absent keys read as "" */
   if(mk_value(b, "METRIC", m->metric_name, sizeof m->metric_name)) m->metric_name[0] = 0;
   if(mk_value(b, "FRAME", m->frame_name, sizeof m->frame_name)) m->frame_name[0] = 0;
   if(mk_value(b, "ANALYSIS", m->analysis_name, sizeof m->analysis_name)) m->analysis_name[0] = 0;
   if(mk_value(b, "GEOMETRY", m->geometry_name, sizeof m->geometry_name)) m->geometry_name[0] = 0;
   if(mk_value(b, "OUTPUT", m->output_name, sizeof m->output_name)) m->output_name[0] = 0;
   if(mk_value(b, "RESTART", m->restart_name, sizeof m->restart_name)) m->restart_name[0] = 0;
   if(mk_value(b, "HLLD", m->hlld_name, sizeof m->hlld_name)) m->hlld_name[0] = 0;
   if(!mk_value(b, "GEOMETRY", v, sizeof v) && strcmp(v, "cylindrical") != 0) {
      free(b);
      disco_set_error("GEOMETRY: only cylindrical is built");
      return DISCO_E_MODULE;
   }
   free(b);
   if(bad) { disco_set_error("Makefile_opt.in: missing module key"); return DISCO_E_PARFILE; }

   static const char *hyd[] = {"euler", "mhd", "grmhd"};
   static const char *ini[] = {"vortex_gauss", "disk_mhd", "disk_planet", "disk_cbd", "gr_disk",
                               "fm_torus"};
   static const char *bnd[] = {"fixed", "fixed3d", "outflow3d", "zerograd", "zerograd_omk",
                               "zerograd_omIN", "accrete3d", "fixRrefZ", "polar3d", "fixed_gap",
                               "tube", "surfaceGravBox", "flowthrough", "polar", "horizon3d",
                               "horizon", "horizon_bin"};
   static const char *pla[] = {"none", "sun", "circular", "cm"};
   static const char *ana[] = {"diag_euler", "diag_disk2d", "diag_cb", "diag_bl", "diag_mhdmri",
                               "diag_grmhdmri"};
   int i;
   m->hydro = m->initial = m->boundary = m->planets = -1;
   for(i = 0; i < 3; i++) if(!strcmp(m->hydro_name, hyd[i])) m->hydro = i;
   for(i = 0; i < 6; i++) if(!strcmp(m->initial_name, ini[i])) m->initial = i;
   m->metric = !strcmp(m->metric_name, "schw_ks_rpz") ? DISCO_METRIC_SCHW_KS_RPZ
             : !strcmp(m->metric_name, "kerr_ks_rpz") ? DISCO_METRIC_KERR_KS_RPZ : DISCO_METRIC_NONE;
   m->frame = !strcmp(m->frame_name, "normal") ? DISCO_FRAME_NORMAL : DISCO_FRAME_NONE;
   for(i = 0; i < DISCO_BC_COUNT; i++) if(!strcmp(m->boundary_name, bnd[i])) m->boundary = i;
   for(i = 0; i < 4; i++) if(!strcmp(m->planets_name, pla[i])) m->planets = i;
   m->analysis = DISCO_DIAG_NONE;
   for(i = 0; i < 6; i++) if(!strcmp(m->analysis_name, ana[i])) m->analysis = i;
   char msg[256];
   if(m->analysis_name[0] && m->analysis < 0) { snprintf(msg, sizeof msg, "ANALYSIS=%s not built", m->analysis_name); disco_set_error(msg); return DISCO_E_MODULE; }
   if(m->hydro < 0) { snprintf(msg, sizeof msg, "HYDRO=%s not built", m->hydro_name); disco_set_error(msg); return DISCO_E_MODULE; }
   if(m->initial < 0) { snprintf(msg, sizeof msg, "INITIAL=%s not built", m->initial_name); disco_set_error(msg); return DISCO_E_MODULE; }
   if(m->boundary < 0) { snprintf(msg, sizeof msg, "BOUNDARY=%s not built", m->boundary_name); disco_set_error(msg); return DISCO_E_MODULE; }
   if(m->planets < 0) { snprintf(msg, sizeof msg, "PLANETS=%s not built", m->planets_name); disco_set_error(msg); return DISCO_E_MODULE; }
   if(m->hydro == DISCO_HYDRO_EULER && (m->num_c != 5 || m->ct_mode != 0)) {
      disco_set_error("euler needs NUM_C=5, CT_MODE=0"); return DISCO_E_MODULE;
   }
   if(m->hydro == DISCO_HYDRO_MHD && m->num_c != 8) {
      disco_set_error("mhd needs NUM_C=8"); return DISCO_E_MODULE;
   }
   if(m->hydro == DISCO_HYDRO_GRMHD) {
      if(m->num_c != 8 || m->ct_mode != 0) {
         disco_set_error("grmhd is built with NUM_C=8 and CT_MODE=0 (cell-centred B)");
         return DISCO_E_MODULE;
      }
      if(m->metric == DISCO_METRIC_NONE || m->frame != DISCO_FRAME_NORMAL) {
         snprintf(msg, sizeof msg, "grmhd: METRIC=%s FRAME=%s not built (schw_ks_rpz or kerr_ks_rpz, "
                  "normal are)", m->metric_name, m->frame_name);
         disco_set_error(msg); return DISCO_E_MODULE;
      }
   }
   if(m->num_n < 0 || m->num_n > 1) { disco_set_error("NUM_N must be 0 or 1"); return DISCO_E_MODULE; }
   return DISCO_OK;
}

/* ------------------------------------------------------------------------
 * Planets plugins: setPlanetParams + initializePlanets (Planets/none.c,
 * Planets/sun.c, Planets/circular.c).
 * ---------------------------------------------------------------------- */
static void setup_planets(disco_host_domain *d)
{
   const disco_params *p = &d->par;
   memset(d->planets, 0, sizeof d->planets);
   switch(d->mod.planets) {
   case DISCO_PL_NONE:       /* Planets/none.c:3-22 */
      d->Npl = 1;
      d->planets[0].eps = 1.0;
      break;
   case DISCO_PL_SUN:        /* Planets/sun.c:5-24 */
      d->Npl = 1;
      d->planets[0].M = 1.0;
      d->planets[0].omega = 1.0;
      d->planets[0].eps = p->grav_eps;
      break;
   case DISCO_PL_CIRCULAR:   /* Planets/circular.c:6-40 */
      d->Npl = 2;
      d->planets[0].M = 1.0;
      d->planets[1].M = p->Mass_Ratio;
      d->planets[1].omega = 1.0;
      d->planets[1].r = 1.0;
      d->planets[1].eps = 0.5/p->Disk_Mach;
      break;
   case DISCO_PL_CM: {       /* Planets/cm.c:7-50: binary about its centre of mass */
      double a = 1.0, q = p->Mass_Ratio, mu = q/(1. + q), om = pow(a, -1.5);
      double smooth = 0.5/p->Disk_Mach;
      d->Npl = 2;
      d->planets[0].M = 1. - mu; d->planets[0].omega = om; d->planets[0].r = a*mu;
      d->planets[0].phi = M_PI; d->planets[0].eps = smooth;
      d->planets[1].M = mu; d->planets[1].omega = om; d->planets[1].r = a*(1. - mu);
      d->planets[1].phi = 0.0; d->planets[1].eps = smooth;
      break;
   }
   }
}

/* ------------------------------------------------------------------------
 * Grid: gridsetup.c:15-142 (serial: dim_rank = 0, dim_size = 1).
 * ---------------------------------------------------------------------- */
static double centroid_r(double xp, double xm)
{
   return 2.0*(xp*xp + xp*xm + xm*xm)/(3.0*(xp + xm));   /* cylindrical.c:24 */
}

static double get_dp(double phip, double phim, double phi_max)
{
   double dp = phip - phim;                                /* cylindrical.c:10 */
   while(dp < 0.0) dp += phi_max;
   while(dp > phi_max) dp -= phi_max;
   return dp;
}

/* fm_torus: the parameters from in.par and the derived constants of
 * disco_ic_fm_setup (kept in ic_aux: ell, F_in, h_pk - 1, field scale) */
static void fm_params(const disco_params *p, const double *aux, struct disco_ic_fm *P)
{
   P->gam = p->Adiabatic_Index; P->M = p->metricPar2; P->a = p->metricPar3;
   P->rin = p->initPar1; P->rpk = p->initPar2; P->beta = p->initPar3; P->acut = p->initPar4;
   P->rho_atm = p->Density_Floor; P->cs2_atm = p->Pressure_Floor;
   P->ell = aux[0]; P->F_in = aux[1]; P->hpk1 = aux[2]; P->bscale = aux[3];
}

static void ic_eval(const disco_host_domain *d, double *prim, const double *x)
{
   const disco_params *p = &d->par;
   int nc = d->mod.num_c, nq = d->num_q;
   switch(d->mod.initial) {
   case DISCO_IC_VORTEX_GAUSS: {
      struct disco_ic_vortex_gauss P = { p->initPar1, p->initPar2, p->initPar3,
                                         p->initPar4, p->initPar5, p->Adiabatic_Index };
      disco_ic_vortex_gauss_eval(&P, prim, x, nc, nq);
      break; }
   case DISCO_IC_DISK_MHD: {
      struct disco_ic_disk P;
      disco_ic_disk_from_params(&P, p->Adiabatic_Index, p->Disk_Mach, p->initPar1,
                                p->initPar2, p->initPar3, p->initPar4, p->initPar5,
                                p->initPar6);
      disco_ic_disk_mhd_eval(&P, prim, x, nc, nq);
      break; }
   case DISCO_IC_DISK_PLANET: {
      struct disco_ic_disk P;
      disco_ic_disk_from_params(&P, p->Adiabatic_Index, p->Disk_Mach, p->initPar1,
                                p->initPar2, p->initPar3, p->initPar4, p->initPar5,
                                p->initPar6);
      disco_ic_disk_planet_eval(&P, prim, x, nc, nq);
      break;
   }
   case DISCO_IC_DISK_CBD: {
      struct disco_ic_disk P;
      disco_ic_disk_from_params(&P, p->Adiabatic_Index, p->Disk_Mach, p->initPar1,
                                p->initPar2, p->initPar3, p->initPar4, p->initPar5,
                                p->initPar6);
      disco_ic_disk_cbd_eval(&P, prim, x, nc, nq);
      break; }
   case DISCO_IC_GR_DISK: {
      struct disco_ic_gr_disk P = { p->Adiabatic_Index, p->metricPar2, p->initPar1,
                                    p->initPar2, p->initPar3, p->initPar4 };
      disco_ic_gr_disk_eval(&P, prim, x, nc, nq);
      break; }
   case DISCO_IC_FM_TORUS: {
      struct disco_ic_fm P;
      fm_params(p, d->ic_aux, &P);
      disco_ic_fm_eval(&P, prim, x, nc, nq);
      break; }
   }
   if(p->RotFrame) prim[3] -= p->RotOmega;   /* subtract_omega, rotframe.c:15 */
}

/* addNoise (noise.c:15-47) drawing from the shared rand() stream. */
static void add_noise(const disco_params *p, disco_rand_state *rs, double *prim,
                      const double *x)
{
   double relMag = p->noiseRel, absMag = p->noiseAbs;
   const double RM = (double)DISCO_RAND_MAX;
   if(p->noiseType == 1) {
      double x1 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x2 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x3 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x4 = 2*((double)disco_rand_next(rs)/RM) - 1;
      prim[2] = (1.0 + x1*relMag)*prim[2] + x2*absMag;
      prim[3] = (1.0 + x3*relMag)*prim[3] + x4*absMag;
   } else if(p->noiseType == 2) {
      double x1 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x2 = 2*((double)disco_rand_next(rs)/RM) - 1;
      prim[1] = (1.0 + x1*relMag)*prim[1] + x2*absMag;
   } else if(p->noiseType == 3) {
      double x1 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x2 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x3 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double x4 = 2*((double)disco_rand_next(rs)/RM) - 1;
      double vc1 = prim[3]*x[0];   /* get_vec_covariant: v^phi * r */
      prim[2] = x1*relMag*vc1 + x2*absMag;
      prim[4] = x3*relMag*vc1 + x4*absMag;
   }
}

/* The grid of main.c:34-47 up to the ring phases: gridsetup.c (r_jph,
 * z_kph, Np), setupDomain's phases from rand() after srand(314159)
 * (domain.c:172-233), the planets, and calc_dp.  *rs is left where the
 * reference's rand() stream stands when setupCells begins. */
int disco_host_grid(const disco_params *par, const disco_modules *mod,
                    disco_host_domain **out, disco_rand_state *rs_out)
{
   if(!par || !mod || !out || !rs_out) { disco_set_error("disco_host_setup: null argument"); return DISCO_E_ARG; }
   if(par->Num_R < 1 || par->Num_Z < 1 || par->aspect <= 0.0 || par->phimax <= 0.0) {
      disco_set_error("disco_host_setup: Num_R, Num_Z, aspect, Phi_Max must be positive");
      return DISCO_E_ARG;
   }
   if(par->LogZoning != 0) {
      disco_set_error("disco_host_setup: only Log_Zoning 0 is built"); return DISCO_E_MODULE;
   }
   if((mod->boundary == DISCO_BC_POLAR || mod->boundary == DISCO_BC_HORIZON ||
       mod->boundary == DISCO_BC_HORIZON_BIN) && par->RotFrame) {
      /* Boundary/polar.c, horizon.c and horizon_bin.c fill their cells
       * without subtract_omega; the fill here is written for the
       * non-rotating frame */
      char msg[96];
      snprintf(msg, sizeof msg, "BOUNDARY=%s with RotFrame is not built", mod->boundary_name);
      disco_set_error(msg);
      return DISCO_E_MODULE;
   }
   disco_host_domain *d = (disco_host_domain *)calloc(1, sizeof(*d));
   if(!d) return DISCO_E_NOMEM;
   d->par = *par;
   d->mod = *mod;
   d->num_q = mod->num_c + mod->num_n;
   d->num_faces = mod->ct_mode == 2 ? 5 : (mod->ct_mode == 1 ? 3 : 0);

   const int Ng = DISCO_NUM_G;
   int Num_R = par->Num_R, Num_Z = par->Num_Z;
   int NgRa = par->NoBC_Rmin ? 0 : Ng;
   int NgRb = par->NoBC_Rmax ? 0 : Ng;
   int N0r = 0 - NgRa, N1r = Num_R + NgRb;
   int Nr = N1r - N0r;
   int NgZa = (Num_Z == 1 || par->NoBC_Zmin) ? 0 : Ng;
   int NgZb = (Num_Z == 1 || par->NoBC_Zmax) ? 0 : Ng;
   int N0z = 0 - NgZa, N1z = Num_Z + NgZb;
   int Nz = N1z - N0z;
   int Nr_glob = Num_R, N0r_glob = 0;
   if(!par->NoBC_Rmin) { Nr_glob += Ng; N0r_glob -= Ng; }
   if(!par->NoBC_Rmax) Nr_glob += Ng;
   int N0z_glob = 0;
   if(!par->NoBC_Zmin) N0z_glob -= Ng;
   d->Nr = Nr; d->Nz = Nz; d->NgRa = NgRa; d->NgRb = NgRb; d->NgZa = NgZa; d->NgZb = NgZb;

   d->Np = (int *)malloc(sizeof(int)*Nr*Nz);
   d->ring_off = (long *)malloc(sizeof(long)*(Nr*Nz + 1));
   d->r_jph = (double *)malloc(sizeof(double)*(Nr + 1));
   d->z_kph = (double *)malloc(sizeof(double)*(Nz + 1));
   if(!d->Np || !d->ring_off || !d->r_jph || !d->z_kph) { disco_host_free(d); return DISCO_E_NOMEM; }

   /* gridsetup.c:99-114; index shifted by one (our [0] is their [-1]) */
   int j, k;
   for(j = -1; j < Nr; j++) {
      double x = (N0r + j + 1)/(double)Num_R;
      d->r_jph[j + 1] = par->rmin + x*(par->rmax - par->rmin);
   }
   double dz = (par->zmax - par->zmin)/(double)Num_Z;
   double z0 = par->zmin + (double)N0z*dz;
   for(k = -1; k < Nz; k++) d->z_kph[k + 1] = z0 + ((double)k + 1.)*dz;
   d->phi_max = par->phimax;
   double Pmax = d->phi_max;

   /* gridsetup.c:119-141: Np from the OUTER edge radius (scale factor at xp) */
   long off = 0;
   for(k = 0; k < Nz; k++) {
      for(j = 0; j < Nr; j++) {
         int jk = j + Nr*k;
         double rp = d->r_jph[j + 1], rm = d->r_jph[j];
         double dr = rp - rm;
         double hp = rp;
         double dp = par->aspect*dr/hp;
         int Np = (int)(Pmax/dp);
         if(Np < 4) Np = 4;
         if(par->maxNp > 0 && Np > par->maxNp) Np = par->maxNp;
         d->Np[jk] = Np;
      }
   }
   /* periodic dimensions: a ghost ring holds the cells of its source ring,
    * Np included (exchange.c:123-171 sends Np with the cells) */
   for(k = 0; k < Nz; k++)
      for(j = 0; j < Nr; j++) {
         int src = disco_periodic_source(d, 1, j, k);
         if(src >= 0) d->Np[j + Nr*k] = d->Np[src];
      }
   for(k = 0; k < Nz; k++)
      for(j = 0; j < Nr; j++) {
         int src = disco_periodic_source(d, 2, j, k);
         if(src >= 0) d->Np[j + Nr*k] = d->Np[src];
      }
   for(k = 0; k < Nr*Nz; k++) { d->ring_off[k] = off; off += d->Np[k]; }
   d->ring_off[Nr*Nz] = off;
   d->Ncell = off;

   d->piph = (double *)malloc(sizeof(double)*off);
   d->dphi = (double *)malloc(sizeof(double)*off);
   d->prim = (double *)calloc((size_t)d->num_q*off, sizeof(double));
   if(!d->piph || !d->dphi || !d->prim) { disco_host_free(d); return DISCO_E_NOMEM; }

   /* domain.c:172-233: one rand() per global ring, layout-independent */
   disco_rand_state rs;
   disco_rand_seed(&rs, 314159u);
   (void)disco_rand_next(&rs);
   for(k = N0z_glob; k < N0z; k++)
      for(j = 0; j < Nr_glob; j++) (void)disco_rand_next(&rs);
   for(k = 0; k < Nz; k++) {
      for(j = N0r_glob; j < N0r; j++) (void)disco_rand_next(&rs);
      for(j = 0; j < Nr; j++) {
         int jk = k*Nr + j;
         double p0 = Pmax*(double)disco_rand_next(&rs)/(double)DISCO_RAND_MAX;
         double dp = Pmax/(double)d->Np[jk];
         long c0 = d->ring_off[jk];
         int i;
         for(i = 0; i < d->Np[jk]; i++) {
            double phi = p0 + dp*(double)i;
            if(phi > Pmax) phi -= Pmax;
            d->piph[c0 + i] = phi;
            d->dphi[c0 + i] = dp;
         }
      }
      for(j = N0r + Nr; j < N0r_glob + Nr_glob; j++) (void)disco_rand_next(&rs);
   }
   d->t = par->t_min;
   setup_planets(d);
   memset(d->ic_aux, 0, sizeof d->ic_aux);
   if(d->mod.initial == DISCO_IC_FM_TORUS) {
      struct disco_ic_fm P;
      fm_params(par, d->ic_aux, &P);
      disco_ic_fm_setup(&P);
      d->ic_aux[0] = P.ell; d->ic_aux[1] = P.F_in; d->ic_aux[2] = P.hpk1; d->ic_aux[3] = P.bscale;
   }

   /* setupCells (domain.c:283-353) begins with calc_dp */
   int jk;
   for(jk = 0; jk < Nr*Nz; jk++) {
      long c0 = d->ring_off[jk];
      int Np = d->Np[jk], i;
      for(i = 0; i < Np; i++) {
         int im = i == 0 ? Np - 1 : i - 1;
         d->dphi[c0 + i] = get_dp(d->piph[c0 + i], d->piph[c0 + im], Pmax);
      }
   }
   *rs_out = rs;
   *out = d;
   return DISCO_OK;
}

/* The rest of setupCells (domain.c:319-353) on the real cells in (k, j, i)
 * order: initial() when from_ic (a restart keeps the primitives it read),
 * then the noise, drawn from *rs; prim2cons/cons2prim run on the device.
 * Then the first exchange of a periodic run (main.c:53-61): r ghost rings,
 * then whole z ghost layers, take their source rings' cells. */
void disco_host_cells(disco_host_domain *d, disco_rand_state *rs, int from_ic)
{
   const disco_params *par = &d->par;
   const int Nr = d->Nr, Nz = d->Nz, NgRa = d->NgRa, NgRb = d->NgRb, NgZa = d->NgZa, NgZb = d->NgZb;
   long N = d->Ncell;
   int nq = d->num_q, j, k;
   for(k = NgZa; k < Nz - NgZb; k++) {
      double z = 0.5*(d->z_kph[k + 1] + d->z_kph[k]);
      for(j = NgRa; j < Nr - NgRb; j++) {
         double r = centroid_r(d->r_jph[j + 1], d->r_jph[j]);
         int jk2 = j + Nr*k;
         long c0 = d->ring_off[jk2];
         int i, q;
         for(i = 0; i < d->Np[jk2]; i++) {
            long c = c0 + i;
            double phi = d->piph[c] - .5*d->dphi[c];
            double x[3] = {r, phi, z};
            double prim[16];
            if(from_ic) ic_eval(d, prim, x);
            else for(q = 0; q < nq; q++) prim[q] = d->prim[(size_t)q*N + c];
            if(par->noiseType != 0) add_noise(par, rs, prim, x);
            for(q = 0; q < nq; q++) d->prim[(size_t)q*N + c] = prim[q];
         }
      }
   }
   for(int dim = 1; dim <= 2; dim++)
      for(k = 0; k < Nz; k++)
         for(j = 0; j < Nr; j++) {
            int src = disco_periodic_source(d, dim, j, k);
            if(src < 0) continue;
            long c0 = d->ring_off[j + Nr*k], s0 = d->ring_off[src];
            int i, q;
            for(i = 0; i < d->Np[src]; i++) {
               d->piph[c0 + i] = d->piph[s0 + i];
               d->dphi[c0 + i] = d->dphi[s0 + i];
               for(q = 0; q < nq; q++) d->prim[(size_t)q*N + c0 + i] = d->prim[(size_t)q*N + s0 + i];
               for(q = 0; d->Phi && q < d->num_faces; q++)
                  d->Phi[(size_t)q*N + c0 + i] = d->Phi[(size_t)q*N + s0 + i];
            }
         }
}

int disco_host_setup(const disco_params *par, const disco_modules *mod,
                     disco_host_domain **out)
{
   disco_rand_state rs;
   disco_host_domain *d = NULL;
   int rc = disco_host_grid(par, mod, &d, &rs);
   if(rc) return rc;
   disco_host_cells(d, &rs, 1);
   *out = d;
   return DISCO_OK;
}

/* The ring whose cells a periodic ghost ring holds, or -1: with R_Periodic
 * (dim 1) ghost ring j < NgRa takes real ring j + Nr_real and ring
 * j >= Nr - NgRb takes j - Nr_real, in every layer; with Z_Periodic (dim 2)
 * likewise in k, for every j.  With one rank, the cartesian communicator's
 * wrap-around makes exchangeData (exchange.c:173-279) exactly this copy. */
int disco_periodic_source(const disco_host_domain *d, int dim, int j, int k)
{
   int Nr = d->Nr, Nz = d->Nz;
   if(dim == 1) {
      if(!d->par.R_Periodic || Nr <= 1) return -1;
      int nreal = Nr - d->NgRa - d->NgRb;
      if(j < d->NgRa) return (j + nreal) + Nr*k;
      if(j >= Nr - d->NgRb) return (j - nreal) + Nr*k;
      return -1;
   }
   if(!d->par.Z_Periodic || Nz <= 1) return -1;
   int nreal = Nz - d->NgZa - d->NgZb;
   if(k < d->NgZa) return j + Nr*(k + nreal);
   if(k >= Nz - d->NgZb) return j + Nr*(k - nreal);
   return -1;
}

void disco_host_free(disco_host_domain *d)
{
   if(!d) return;
   free(d->Np); free(d->ring_off); free(d->r_jph); free(d->z_kph);
   free(d->piph); free(d->dphi); free(d->prim); free(d->Phi);
   free(d);
}

int disco_rand_sequence(unsigned int seed, int n, int *out)
{
   disco_rand_state st;
   int i;
   disco_rand_seed(&st, seed);
   for(i = 0; i < n; i++) out[i] = disco_rand_next(&st);
   return DISCO_OK;
}
