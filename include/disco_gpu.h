/*
 * disco_gpu.h -- C ABI of the GB300 (sm_103a) implementation of Disco's
 * moving-mesh RK substep cycle.
 *
 * The reference enters its hot path through two link-time C symbols called
 * from its main loop (main.c:70,73):
 *
 *     double getmindt(struct domain *);          misc.c:39
 *     void   timestep(struct domain *, double);  timestep.c:7
 *
 * and is configured by in.par (readpar.c:44-210) plus the module names of
 * Makefile_opt.in (Makefile:1-26).  This ABI replaces that pair.  Everything
 * crosses as plain pointers, sizes and POD structs; no C++ or torch types.
 *
 * Conventions (all functions):
 *   return 0 on success; a negative DISCO_E_* code on a usage or CUDA error
 *   (message available from disco_last_error()); kernels never trap.
 *   Physics warnings (NaN counts, floors hit) are reported by
 *   disco_gpu_status(), not by return codes.
 *
 * Layout of cell arrays exchanged with the caller: cells are ordered ring
 * by ring, ring jk = j + Nr*k (j radial, k vertical, ghosts included, same as
 * the reference's theCells[jk]), cell i inside ring jk (reference
 * theCells[jk][i]).  Per-component arrays are structure-of-arrays:
 * prim[q*Ncell + c].
 */
#ifndef DISCO_GPU_H
#define DISCO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DISCO_ABI_VERSION 1

enum disco_status_code {
   DISCO_OK = 0,
   DISCO_E_ARG = -1,       /* bad argument / inconsistent sizes */
   DISCO_E_PARFILE = -2,   /* in.par or Makefile_opt.in unreadable */
   DISCO_E_MODULE = -3,    /* module named in Makefile_opt.in not built */
   DISCO_E_CUDA = -4,      /* CUDA runtime error */
   DISCO_E_NOMEM = -5,     /* host or device allocation failed */
   DISCO_E_NODEV = -6,     /* no CUDA device / extension built without GPU */
   DISCO_E_STATE = -7      /* call out of order (e.g. step before create) */
};

/* Module ids selected by name from Makefile_opt.in (Makefile:12-26). */
enum disco_hydro_id   { DISCO_HYDRO_EULER = 0, DISCO_HYDRO_MHD = 1, DISCO_HYDRO_GRMHD = 2 };
enum disco_initial_id { DISCO_IC_VORTEX_GAUSS = 0, DISCO_IC_DISK_MHD = 1,
                        DISCO_IC_DISK_PLANET = 2, DISCO_IC_DISK_CBD = 3,
                        DISCO_IC_GR_DISK = 4, DISCO_IC_FM_TORUS = 5 };
/* GRMHD only: METRIC and FRAME of Makefile_opt.in (Hydro/Metric, Hydro/Frame);
 * kerr_ks_rpz is the Kerr metric (spin Metric_Par3) in the same Kerr-Schild
 * cylindrical coordinates as the reference's schw_ks_rpz */
enum disco_metric_id  { DISCO_METRIC_NONE = -1, DISCO_METRIC_SCHW_KS_RPZ = 0,
                        DISCO_METRIC_KERR_KS_RPZ = 1 };
enum disco_frame_id   { DISCO_FRAME_NONE = -1, DISCO_FRAME_NORMAL = 0 };
enum disco_boundary_id{ DISCO_BC_FIXED = 0, DISCO_BC_FIXED3D = 1,
                        DISCO_BC_OUTFLOW3D = 2, DISCO_BC_ZEROGRAD = 3,
                        DISCO_BC_ZEROGRAD_OMK = 4, DISCO_BC_ZEROGRAD_OMIN = 5,
                        DISCO_BC_ACCRETE3D = 6, DISCO_BC_FIXRREFZ = 7,
                        DISCO_BC_POLAR3D = 8, DISCO_BC_FIXED_GAP = 9,
                        DISCO_BC_TUBE = 10, DISCO_BC_SURFACEGRAVBOX = 11,
                        DISCO_BC_FLOWTHROUGH = 12, DISCO_BC_POLAR = 13,
                        DISCO_BC_HORIZON3D = 14, DISCO_BC_HORIZON = 15,
                        DISCO_BC_HORIZON_BIN = 16, DISCO_BC_COUNT = 17 };
enum disco_planets_id { DISCO_PL_NONE = 0, DISCO_PL_SUN = 1,
                        DISCO_PL_CIRCULAR = 2, DISCO_PL_CM = 3 };
/* ANALYSIS of Makefile_opt.in: the Diagnostics/ plugin whose ring averages
 * timestep() accumulates (analysis.c:52-108, timestep.c:51) */
enum disco_analysis_id{ DISCO_DIAG_NONE = -1, DISCO_DIAG_EULER = 0,
                        DISCO_DIAG_DISK2D = 1, DISCO_DIAG_CB = 2,
                        DISCO_DIAG_BL = 3, DISCO_DIAG_MHDMRI = 4,
                        DISCO_DIAG_GRMHDMRI = 5 };

#define DISCO_MAX_PLANETS 4
#define DISCO_NUM_G 2   /* ghost rings per side: paul.h:20 NUM_G */

/* Module selection: mirror of Makefile_opt.in (Makefile_opt.in.template). */
typedef struct disco_modules {
   int hydro, initial, boundary, planets;
   int num_c, num_n, ct_mode;    /* NUM_C, NUM_N, CT_MODE */
   char initial_name[64], hydro_name[64], boundary_name[64], planets_name[64];
   int metric, frame;            /* GRMHD: disco_metric_id, disco_frame_id */
   char metric_name[64], frame_name[64];
   int analysis;                 /* ANALYSIS: disco_analysis_id, or -1 when absent */
   char analysis_name[64];
   /* the remaining names the checkpoint records (h5out.c:98-160); "" when absent */
   char geometry_name[64], output_name[64], restart_name[64], hlld_name[64];
} disco_modules;

/* Run-time parameters: the hot-path subset of struct param_list
 * (paul.h:43-141), keyed by the same in.par names (readpar.c:70-175).
 * A key absent from in.par reads as 0, as in the reference. */
typedef struct disco_params {
   double t_min, t_max;
   int Num_R, Num_Z;
   double aspect;
   double rmin, rmax, zmin, zmax, phimax;
   int NoBC_Rmin, NoBC_Rmax, NoBC_Zmin, NoBC_Zmax;
   int LogZoning, R_Periodic, Z_Periodic;
   double LogRadius;
   int Mesh_Motion, Riemann_Solver, Timestep;
   double CFL, PLM, maxDT;
   double Density_Floor, Pressure_Floor;
   int Exact_Mesh_Omega;      double Exact_Mesh_Omega_Par;
   int Energy_Omega;          double Energy_Omega_Par;
   int RotFrame;              double RotOmega, RotD;
   double Adiabatic_Index;
   int visc_flag;             double viscosity;
   int alpha_flag;
   int isothermal_flag;
   int Cs2_Profile;           double Cs2_Par;
   double Disk_Mach, Mass_Ratio;
   int grav2D;
   int CT;
   int metricPar0;  double metricPar1, metricPar2, metricPar3, metricPar4;
   int initPar0;
   double initPar1, initPar2, initPar3, initPar4, initPar5, initPar6,
          initPar7, initPar8;
   int noiseType;   double noiseAbs, noiseRel;
   int sinkType, nozzleType, coolType;
   int dampInnerType, dampOuterType, dampUpperType, dampLowerType;
   double grav_eps;
   int read_errors;   /* number of keys absent (readpar.c: err count) */
   double sinkPar3;   /* Sink_Par3: the softening behind report.c's torque cut radii */
   double coolPar1, coolPar2, coolPar3, coolPar4;            /* Cool_Par1..4 (sink.c:274) */
   double dampTimeInner, dampLenInner, dampTimeOuter, dampLenOuter,
          dampTimeUpper, dampLenUpper, dampTimeLower, dampLenLower;   /* Damp*_Time/_Len (sink.c:329) */
   int maxNp;         /* Max_Np: cap on cells per ring (no reference key; 0 = none) */
   int sinkNumber;    /* Sink_Number: sinks on the first n bodies (0: all) */
   double sinkPar1, sinkPar2, sinkPar4, sinkPar5;             /* Sink_Par1,2,4,5 (sink.c:105) */
   double nozzlePar1, nozzlePar2, nozzlePar3, nozzlePar4;     /* Nozzle_Par1..4 (sink.c:105) */
   /* keys the hot path does not read but the checkpoint records
    * (readpar.c:73-126, h5out.c:168-366) */
   int NumRepts, NumSnaps, NumChecks, Out_LogTime, Initial_Regrid, restart_flag, include_atmos;
   double MaxShort, MaxLong, Eccentricity, Drift_Rate, Drift_Exp;
} disco_params;

/* One point mass: the fields of struct planet (paul.h:259-284) the hot path
 * reads. */
typedef struct disco_planet {
   double r, phi, M, omega, vr, eps;
   int type;
} disco_planet;

/* Host-side domain: grid, ring phases and initial primitives produced by
 * the C set-up (gridsetup.c:15, domain.c:170, domain.c:283 up to
 * prim2cons), owned by the library. */
typedef struct disco_host_domain {
   disco_params par;
   disco_modules mod;
   int Nr, Nz, NgRa, NgRb, NgZa, NgZb;
   int num_q, num_faces;
   long Ncell;            /* total cells incl. ghosts */
   int *Np;               /* [Nr*Nz] */
   long *ring_off;        /* [Nr*Nz+1] exclusive prefix of Np */
   double *r_jph;         /* [Nr+1]; r_jph[0] is the reference's r_jph[-1] */
   double *z_kph;         /* [Nz+1]; z_kph[0] is the reference's z_kph[-1] */
   double phi_max, t;
   double *piph, *dphi;   /* [Ncell] */
   double *prim;          /* [num_q*Ncell]: initial() (+ noise) for real cells */
   int Npl;
   disco_planet planets[DISCO_MAX_PLANETS];
   double ic_aux[4];      /* constants the initial condition derives once at set-up
                             (fm_torus: ell, F(r_in), h(r_pk) - 1, field scale) */
   double *Phi;           /* [num_faces*Ncell] face fluxes read from a checkpoint
                             (disco_host_restart), else NULL: disco_gpu_create then
                             takes them instead of the initial field's */
} disco_host_domain;

/* Host->device state snapshot, filled by disco_gpu_download(). Any pointer
 * may be NULL to skip that field.  Sizes: [Ncell] or [num_q*Ncell]. */
typedef struct disco_state_view {
   double *piph, *dphi, *wiph;
   double *prim, *cons;
   double *Phi;            /* [num_faces*Ncell], CT only */
   double t;
} disco_state_view;

/* Device-side health counters (kernels never trap; they count). */
typedef struct disco_gpu_errs {
   long long nan_cells;       /* cells whose prim went non-finite */
   long long rho_floor_hits;  /* density floor applied (euler.c:107) */
   long long p_floor_hits;    /* pressure floor applied (euler.c:123) */
   long long face_errors;     /* inconsistent sheared-face merge */
   long long steps;           /* timesteps taken on the device */
   long long c2p_no_converge; /* GRMHD: Newton cons2prim stopped at max_iter = 30
                                 (grmhd.c:959-968, which prints and continues) */
   long long async_timeouts;  /* bounded waits for asynchronous (TMA) copies
                                 that ran out; the block then skips its work */
} disco_gpu_errs;

typedef struct disco_gpu disco_gpu;   /* opaque device instance */

/* ---- host set-up (C, no GPU needed) ----------------------------------- */

/* readvar/read_par_file of readpar.c:6-210 with the same key names,
 * separators and x2pi scalings. */
int disco_params_read(const char *in_par_path, disco_params *out);

/* Module names from a Makefile_opt.in (Makefile:12-26). */
int disco_modules_read(const char *makefile_opt_path, disco_modules *out);

/* Serial set-up identical to main.c:34-47 -- grid (gridsetup.c:15),
 * ring phases from glibc rand() after srand(314159) (domain.c:172-233),
 * initial()+noise for real cells (domain.c:319-353).  Free with
 * disco_host_free(). */
int disco_host_setup(const disco_params *par, const disco_modules *mod,
                     disco_host_domain **out);
void disco_host_free(disco_host_domain *dom);

/* ---- device instance ---------------------------------------------------- */

/* precision: 0 = plain FP64 path; 1 = mixed (FP32 reconstruction, fluxes
 * and sources; FP64 positions, face geometry, conserved accumulation, dt). */
int disco_gpu_create(const disco_host_domain *dom, int precision,
                     disco_gpu **out);

/* Replaces getmindt() (misc.c:39): CFL * min over real cells of mindt(). */
int disco_gpu_getmindt(disco_gpu *g, double *dt);

/* Replaces timestep() (timestep.c:7): one full RK step of size dt,
 * including ghost/boundary fill (onestep.c:309-316). */
int disco_gpu_timestep(disco_gpu *g, double dt);

/* Runs n steps of (getmindt; timestep) entirely on the device, dt never
 * leaving the GPU (the main.c:69-74 loop without output/check_dt).
 * If t_end > 0 the last dt is clamped so t does not pass t_end
 * (check_dt, domain.c:433-436). */
int disco_gpu_run(disco_gpu *g, int nsteps, double t_end);

/* Copies the device state to caller-owned host arrays. */
int disco_gpu_download(disco_gpu *g, disco_state_view *v);

/* Overwrites the device state (prim, cons, piph, dphi, wiph may each be
 * NULL to keep the device copy); used to resume from a checkpoint. */
int disco_gpu_upload(disco_gpu *g, const disco_state_view *v);

/* Timed variant of disco_gpu_run for benchmarking: each of the n steps is
 * one CUDA-graph launch bracketed by CUDA events on the library's stream;
 * if flush_bytes > 0 a scratch buffer of that size is overwritten before
 * each step, outside the timed interval, to evict L2.  *ms_total receives
 * the summed device time of the steps. */
int disco_gpu_run_timed(disco_gpu *g, int nsteps, double t_end,
                        size_t flush_bytes, double *ms_total);

/* Per-kernel device time: runs n steps without graphs, each kernel launch
 * bracketed by CUDA events, and reports per kernel name the launch count
 * and summed milliseconds (at most max_out entries). */
typedef struct disco_kernel_time {
   char name[48];
   long long launches;
   double ms;
} disco_kernel_time;
int disco_gpu_profile(disco_gpu *g, int nsteps, disco_kernel_time *out,
                      int max_out, int *n_out);

int disco_gpu_status(disco_gpu *g, disco_gpu_errs *errs);

/* The point masses as the device has advanced them (the analytic orbits of
 * planet.c:236-270, Planets/circular.c, Planets/cm.c): copies min(Npl, max)
 * entries to out; *n = Npl.  The reference keeps them in
 * theDomain->thePlanets, which report() and the checkpoint read. */
int disco_gpu_planets(disco_gpu *g, disco_planet *out, int max, int *n);
double disco_gpu_time(disco_gpu *g);
long disco_gpu_num_cells(disco_gpu *g);       /* total incl. ghosts */
long disco_gpu_num_real_cells(disco_gpu *g);  /* interior cells */
void disco_gpu_free(disco_gpu *g);

/* Kernel launches made by this library since load (for accounting). */
long long disco_gpu_launch_count(void);

const char *disco_last_error(void);
int disco_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
