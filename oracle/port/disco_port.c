/*
 * CHECKER INFRASTRUCTURE (oracle) -- not product code.
 *
 * Plain-C restatement of the reference's RK substep cycle (timestep.c:7 ->
 * onestep.c:86) for the Newtonian hydro (Hydro/euler.c) and MHD
 * (Hydro/mhd.c + hlld.c + bfields.c constrained transport) modules, run
 * serially on the CPU.  It keeps the reference's per-cell records, face
 * records with cell pointers, loop orders and scatter updates, so compiled
 * with gcc (no FMA contraction) it reproduces the reference's numbers
 * bit-for-bit; tests/test_oracle_port.py pins that against the reference
 * binary built from the reference's own sources (oracle/ref).
 *
 * Used as the checker of the GPU path at sizes beyond the golden fixtures
 * and as the timed CPU baseline ("port") in bench.py.  Input: the host-set-up
 * domain of include/disco_gpu.h (grid, ring phases, initial primitives),
 * itself checked bit-for-bit against the reference.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "disco_gpu.h"
#include "../../disco_gb300/csrc/plugins/ic_vortex_gauss.h"
#include "../../disco_gb300/csrc/plugins/ic_disks.h"
#include "../../disco_gb300/csrc/plugins/bc_plugins.h"

enum { RHO, PPP, URR, UPP, UZZ, BRR, BPP, BZZ };
enum { DDD, TAU, SRR, LLL, SZZ };
#define MAXQ 9
#define TOL_HLLD 1e-10

typedef struct pcell {
   double prim[MAXQ], cons[MAXQ], RKcons[MAXQ];
   double gradr[MAXQ], gradp[MAXQ], gradz[MAXQ];
   double piph, dphi, wiph;
   double E[8], B[8], E_phi[4], Phi[5], RK_Phi[5];
   double tempDoub;
   int real;
} pcell;

typedef struct pface {
   pcell *L, *R;
   double dxL, dxR, cm[3], dphi, dl, dA, E, B;
   int LRtype, flip_flag;
} pface;

typedef struct port_domain {
   disco_params par;
   disco_modules mod;
   int Nr, Nz, NgRa, NgRb, NgZa, NgZb, nq, nc, Npl, mhd, ct;
   long N;
   int *Np;
   long *off;
   pcell *cells;
   pcell **ring;          /* ring[jk] = cells + off[jk] */
   double *rj, *zk;       /* rj[j] = reference r_jph[j], j = -1..Nr-1 */
   double Pmax, t;
   pface *faces[2];
   int *fI[2];
   int ntracks[2];
   disco_planet pl[DISCO_MAX_PLANETS];
   double gam;
   int nd;                /* num_diagnostics() of the ANALYSIS plugin */
   double *Qrz, t_avg;    /* struct diagnostic_avg: Qrz[jk*nd + q] */
   /* the bodies' sink accumulators (paul.h:258-276) in report.c's column
    * order: gravL, dM, accL, Ls, kin, therm, linXmom, linYmom; and their RK
    * copies */
   double sacc[DISCO_MAX_PLANETS][8], sacc_rk[DISCO_MAX_PLANETS][8];
} port_domain;

static port_domain *D;   /* the domain being advanced (module statics in the reference) */

/* ---- geometry: Geometry/cylindrical.c:10-75 ---------------------------- */
static double get_dp(double phip, double phim)
{
   double dp = phip - phim;
   while(dp < 0.0) dp += D->Pmax;
   while(dp > D->Pmax) dp -= D->Pmax;
   return dp;
}
static double get_signed_dp(double phip, double phim)
{
   double dp = phip - phim;
   while(dp < -.5*D->Pmax) dp += D->Pmax;
   while(dp > .5*D->Pmax) dp -= D->Pmax;
   return dp;
}
static double centroid(double xp, double xm, int dim)
{
   if(dim == 1) return 2.0*(xp*xp + xp*xm + xm*xm)/(3.0*(xp + xm));
   return 0.5*(xp + xm);
}
static void centroid_arr(const double *xp, const double *xm, double *x)
{
   x[0] = centroid(xp[0], xm[0], 1);
   x[1] = centroid(xp[1], xm[1], 0);
   x[2] = centroid(xp[2], xm[2], 2);
}
static double get_dL(const double *xp, const double *xm, int dim)
{
   double r = .5*(xp[0] + xm[0]);
   double dphi = get_dp(xp[1], xm[1]);
   if(dim == 0) return r*dphi;
   if(dim == 1) return xp[0] - xm[0];
   return xp[2] - xm[2];
}
static double get_dA(const double *xp, const double *xm, int dim)
{
   double r = .5*(xp[0] + xm[0]), dr = xp[0] - xm[0];
   double dphi = get_dp(xp[1], xm[1]), dz = xp[2] - xm[2];
   if(dim == 0) return dr*dz;
   if(dim == 1) return r*dphi*dz;
   return r*dr*dphi;
}
static double get_dV(const double *xp, const double *xm)
{
   double r = .5*(xp[0] + xm[0]), dr = xp[0] - xm[0];
   double dphi = get_dp(xp[1], xm[1]), dz = xp[2] - xm[2];
   return r*dr*dphi*dz;
}

/* ---- omega.c ------------------------------------------------------------ */
static double get_om(const double *x)   /* omega.c:76-100 */
{
   double O0 = D->par.RotOmega;
   if(D->par.Energy_Omega == 0) return 0.0 - O0;
   double r = sqrt(x[0]*x[0] + D->par.grav_eps*D->par.grav_eps);
   switch(D->par.Energy_Omega) {
   case 1: return 1.0 - O0;
   case 2: return 1.0/pow(r, 1.5) - O0;
   case 3: { double n = 8.0; return 1./pow(pow(r, 1.5*n) + 1., 1./n) - O0; }
   case 4: return 10.*exp(-.5*r*r) - O0;
   default: return 0.0 - O0;
   }
}
static double get_om1(const double *x)  /* omega.c:102-126 */
{
   int ch = D->par.Energy_Omega;
   if(ch == 0 || ch == 1) return 0.0;
   double r = sqrt(x[0]*x[0] + D->par.grav_eps*D->par.grav_eps);
   if(ch == 2) return -1.5/pow(r, 2.5);
   if(ch == 3) { double n = 8.0; return -1.5*pow(r, -1 + 1.5*n)/pow(pow(r, 1.5*n) + 1., 1.0 + 1./n); }
   if(ch == 4) return 10.*r*exp(-.5*r*r);
   return 0.0;
}
static double mesh_om(const double *x)  /* omega.c:56-74 */
{
   double r = sqrt(x[0]*x[0] + D->par.grav_eps*D->par.grav_eps);
   if(D->par.Exact_Mesh_Omega == 1) return 1.0;
   if(D->par.Exact_Mesh_Omega == 2) return pow(r, -1.5);
   if(D->par.Exact_Mesh_Omega == 3) { double n = 4.0; return 1./pow(pow(r, 1.5*n) + 1., 1./n); }
   return 0.0;
}
static double fgrav(double M, double r, double eps);
extern double disco_port_phi_order;
static double phigrav(double M, double r, double eps)
{
   double n = disco_port_phi_order;
   return M/pow(pow(r, n) + pow(eps, n), 1./n);
}
static double get_cs2(const double *x)  /* omega.c:157-209 */
{
   double r = x[0], M = D->par.Disk_Mach;
   if(D->par.Cs2_Profile == 1) return 1./(M*M);
   if(D->par.Cs2_Profile == 2) { double nu = .5; return .5/M/M/pow(r, 2.*nu); }
   if(D->par.Cs2_Profile == 3)
      return D->par.metricPar2*D->par.initPar4*D->par.initPar4/(2*D->par.initPar2*D->par.initPar2*D->par.initPar2);
   if(D->par.Cs2_Profile == 4) {
      r = sqrt(r*r + D->par.grav_eps*D->par.grav_eps);
      double v2 = D->par.metricPar2/r;
      return v2/(M*M);
   }
   if(D->par.Cs2_Profile == 5) {
      double gx = r*cos(x[1]), gy = r*sin(x[1]), phip = 0.0;
      for(int p = 0; p < D->Npl; p++) {
         double px = D->pl[p].r*cos(D->pl[p].phi), py = D->pl[p].r*sin(D->pl[p].phi);
         double pr = (px - gx)*(px - gx) + (py - gy)*(py - gy);
         phip += phigrav(D->pl[p].M, sqrt(pr), D->pl[p].eps);
      }
      return phip/(M*M);
   }
   return 1.0;
}
static double get_height_om(const double *x)  /* omega.c:132-155 */
{
   double omtot2 = 0.0, r = x[0], phi = x[1];
   double gx = r*cos(phi), gy = r*sin(phi);
   for(int p = 0; p < D->Npl; p++) {
      double px = D->pl[p].r*cos(D->pl[p].phi), py = D->pl[p].r*sin(D->pl[p].phi);
      double sr = sqrt((px - gx)*(px - gx) + (py - gy)*(py - gy));
      double f1 = fgrav(D->pl[p].M, sr, D->pl[p].eps);
      omtot2 += f1/(sr + 0.0625*D->pl[p].eps);
   }
   return sqrt(omtot2);
}

/* ---- planet.c (point masses) ---------------------------------------------- */
/* planet.c:4 keeps the potential's order in a mutable global, so the
 * reference's pow() calls stay libm calls; an exported global here keeps
 * the compiler from folding pow(x, 2.0) into x*x, which can differ from
 * libm's pow in the last bit. */
double disco_port_phi_order = 2.0;
static double fgrav(double M, double r, double eps)
{
   double n = disco_port_phi_order;
   return M*pow(r, n - 1.)/pow(pow(r, n) + pow(eps, n), 1. + 1./n);
}
static void planetary_force(const disco_planet *pl, double r, double phi, double z,
                            double *fr, double *fp, double *fz)
{
   double rp = pl->r, pp = pl->phi;
   if(D->par.grav2D == 1) z = 0.0;
   else if(D->par.grav2D == 2) { rp = r; pp = phi; z = 1.0; }
   double cosp = cos(phi), sinp = sin(phi);
   double dx = r*cosp - rp*cos(pp);
   double dy = r*sinp - rp*sin(pp);
   double script_r = sqrt(dx*dx + dy*dy + z*z);
   double script_r_perp = sqrt(dx*dx + dy*dy);
   double f1 = -fgrav(pl->M, script_r, pl->eps);
   double cosa = dx/script_r_perp, sina = dy/script_r_perp;
   double cosap = cosa*cosp + sina*sinp;
   double sinap = sina*cosp - cosa*sinp;
   if(script_r_perp <= 0.0) { cosap = 0.0; sinap = 0.0; }
   double sint = script_r_perp/script_r, cost = z/script_r;
   *fr = cosap*f1*sint;
   *fp = sinap*f1*sint;
   *fz = f1*cost;
}
static void planet_src(const disco_planet *pl, const double *prim, double *cons,
                       const double *xp, const double *xm, double dVdt)
{
   double rho = prim[RHO], vr = prim[URR], vz = prim[UZZ], omega = prim[UPP];
   double dphi = get_dp(xp[1], xm[1]);
   double phi = xm[1] + 0.5*dphi;
   double x[3] = {centroid(xp[0], xm[0], 1), phi, centroid(xp[2], xm[2], 2)};
   double F[3];
   planetary_force(pl, x[0], x[1], x[2], &F[0], &F[1], &F[2]);
   double hr = 1.0, hp = x[0], hz = 1.0;
   if(D->par.NoBC_Rmin == 1) {   /* planet.c:13-18, :205-212: polar vector adjustment */
      double adjust = sin(0.5*dphi)/(0.5*dphi);
      F[0] *= adjust; F[1] *= adjust;
   }
   cons[SRR] += rho*hr*F[0]*dVdt;
   cons[LLL] += rho*hp*F[1]*dVdt;
   cons[SZZ] += rho*hz*F[2]*dVdt;
   cons[TAU] += rho*(hr*F[0]*vr + hz*F[2]*vz + hp*F[1]*omega)*dVdt;
}

/* ---- Hydro/euler.c -------------------------------------------------------- */
static void e_prim2cons(const double *prim, double *cons, const double *x, double dV)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double om = get_om(x);
   double vp_off = vp - om*r;
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   double rhoe = Pp/(D->gam - 1.);
   cons[DDD] = rho*dV;
   cons[TAU] = (.5*rho*v2 + rhoe)*dV;
   cons[SRR] = rho*vr*dV;
   cons[LLL] = r*rho*vp*dV;
   cons[SZZ] = rho*vz*dV;
   for(int q = D->nc; q < D->nq; q++) cons[q] = prim[q]*cons[DDD];
}
static void e_getUstar(const double *prim, double *Ustar, const double *x, double Sk, double Ss,
                       const double *n)
{
   double r = x[0], rho = prim[RHO], vr = prim[URR], vp = prim[UPP]*r;
   double vz = prim[UZZ], Pp = prim[PPP];
   double om = get_om(x);
   double vp_off = vp - om*r;
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   double vn = vr*n[0] + vp*n[1] + vz*n[2];
   double vn_off = vn - om*r*n[1];
   double Ss_off = Ss + vn_off - vn;
   double rhoe = Pp/(D->gam - 1.);
   double rhostar = rho*(Sk - vn)/(Sk - Ss);
   double Pstar = Pp*(Ss - vn)/(Sk - Ss);
   double Us = rhoe*(Sk - vn)/(Sk - Ss);
   Ustar[DDD] = rhostar;
   Ustar[SRR] = rhostar*(vr + (Ss - vn)*n[0]);
   Ustar[LLL] = r*rhostar*(vp + (Ss - vn)*n[1]);
   Ustar[SZZ] = rhostar*(vz + (Ss - vn)*n[2]);
   Ustar[TAU] = .5*rhostar*v2 + Us + rhostar*Ss_off*(Ss - vn) + Pstar;
   for(int q = D->nc; q < D->nq; q++) Ustar[q] = prim[q]*Ustar[DDD];
}
static void e_cons2prim(const double *cons, double *prim, const double *x, double dV)
{
   double r = x[0];
   double rho = cons[DDD]/dV;
   if(rho < D->par.Density_Floor) rho = D->par.Density_Floor;
   double Sr = cons[SRR]/dV, Sp = cons[LLL]/dV/r, Sz = cons[SZZ]/dV, E = cons[TAU]/dV;
   double om = get_om(x);
   double vr = Sr/rho, vp = Sp/rho, vp_off = vp - om*r, vz = Sz/rho;
   double KE = .5*(Sr*vr + rho*vp_off*vp_off + Sz*vz);
   double rhoe = E - KE;
   double Pp = (D->gam - 1.)*rhoe;
   if(Pp < D->par.Pressure_Floor*rho) Pp = D->par.Pressure_Floor*rho;
   if(D->par.isothermal_flag) Pp = get_cs2(x)*rho/D->gam;
   prim[RHO] = rho; prim[PPP] = Pp; prim[URR] = vr; prim[UPP] = vp/r; prim[UZZ] = vz;
   for(int q = D->nc; q < D->nq; q++) prim[q] = cons[q]/cons[DDD];
}
static void e_flux(const double *prim, double *f, const double *x, const double *n)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double om = get_om(x);
   double vn = vr*n[0] + vp*n[1] + vz*n[2];
   double wn = om*r*n[1];
   double vp_off = vp - om*r;
   double rhoe = Pp/(D->gam - 1.);
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   f[DDD] = rho*vn;
   f[SRR] = rho*vr*vn + Pp*n[0];
   f[LLL] = r*(rho*vp*vn + Pp*n[1]);
   f[SZZ] = rho*vz*vn + Pp*n[2];
   f[TAU] = (.5*rho*v2 + rhoe + Pp)*vn - Pp*wn;
   for(int q = D->nc; q < D->nq; q++) f[q] = prim[q]*f[DDD];
}
static void e_vel(const double *p1, const double *p2, double *Sl, double *Sr, double *Ss,
                  const double *n, const double *x)
{
   double r = x[0];
   double P1 = p1[PPP], rho1 = p1[RHO];
   double vn1 = p1[URR]*n[0] + p1[UPP]*n[1]*r + p1[UZZ]*n[2];
   double cs1 = sqrt(D->gam*P1/rho1);
   double P2 = p2[PPP], rho2 = p2[RHO];
   double vn2 = p2[URR]*n[0] + p2[UPP]*n[1]*r + p2[UZZ]*n[2];
   double cs2 = sqrt(D->gam*P2/rho2);
   *Ss = (P2 - P1 + rho1*vn1*(-cs1) - rho2*vn2*cs2)/(rho1*(-cs1) - rho2*cs2);
   *Sr = cs1 + vn1;
   *Sl = -cs1 + vn1;
   if(*Sr < cs2 + vn2) *Sr = cs2 + vn2;
   if(*Sl > -cs2 + vn2) *Sl = -cs2 + vn2;
}
static void e_source(const double *prim, double *cons, const double *xp, const double *xm,
                     double dVdt)
{
   double rp = xp[0], rm = xm[0];
   double rho = prim[RHO], Pp = prim[PPP];
   double r = centroid(rp, rm, 1), z = centroid(xp[2], xm[2], 2);
   double r_1 = .5*(rp + rm);
   double vr = prim[URR], omega = prim[UPP], vz = prim[UZZ];
   double x[3] = {r, 0.5*(xm[1] + xp[1]), z};
   double centrifugal = rho*omega*omega*r;
   if(D->par.NoBC_Rmin == 1) {   /* polar_sources (euler.c:26, :195-200): geom_polar_vec_adjust */
      double dphi = get_dp(xp[1], xm[1]);
      centrifugal *= sin(0.5*dphi)/(0.5*dphi);
   }
   double press_bal = Pp/r_1;
   cons[SRR] += dVdt*(centrifugal + press_bal);
   double om = get_om(x), om_r = get_om1(x), om_z = 0.0;
   cons[TAU] += dVdt*rho*(r*vr*om*om - r*r*(omega - om)*(vr*om_r + vz*om_z));
}
static double e_visc_nu(const double *prim, const double *x)   /* euler.c:220-226 */
{
   double nu = D->par.viscosity;
   if(D->par.alpha_flag) {
      double c2 = D->gam*prim[PPP]/prim[RHO];
      nu = D->par.viscosity*c2/get_height_om(x);
   }
   return nu;
}
static void e_visc_flux(const double *prim, const double *gr, const double *gp, const double *gz,
                        double *f, const double *x, const double *n)   /* euler.c:215-256 */
{
   double r = x[0], nu = e_visc_nu(prim, x);
   double rho = prim[RHO], vr = prim[URR], om_off = prim[UPP] - get_om(x), vz = prim[UZZ];
   double divV_o_d = (gr[URR] + gp[UPP] + gz[UZZ] + vr/r)/3.0;
   double srr = gr[URR] - divV_o_d;
   double spp = r*(r*gp[UPP] + vr - r*divV_o_d);
   double szz = gz[UZZ] - divV_o_d;
   double srp = 0.5*(r*r*gr[UPP] + gp[URR]);
   double srz = 0.5*(gr[UZZ] + gz[URR]);
   double spz = 0.5*(gp[UZZ] + r*r*gz[UPP]);
   double nc[3] = {n[0], n[1]/r, n[2]};
   double srn = srr*nc[0] + srp*nc[1] + srz*nc[2];
   double spn = srp*nc[0] + spp*nc[1] + spz*nc[2];
   double szn = srz*nc[0] + spz*nc[1] + szz*nc[2];
   f[SRR] = -2*nu*rho*srn;
   f[LLL] = -2*nu*rho*spn;
   f[SZZ] = -2*nu*rho*szn;
   f[TAU] = -2*nu*rho*(vr*srn + om_off*spn + vz*szn);
}
static void e_visc_source(const double *prim, const double *gr, const double *gp, const double *gz,
                          double *cons, const double *xp, const double *xm, double dVdt)
{                                                               /* euler.c:258-291 */
   double x[3];
   centroid_arr(xp, xm, x);
   double r = x[0], nu = e_visc_nu(prim, x);
   double rho = prim[RHO], vr = prim[URR];
   double divV_o_d = (gr[URR] + gp[UPP] + gz[UZZ] + vr/r)/3.0;
   double spp = (r*gp[UPP] + vr - r*divV_o_d)/(r*r*r);
   cons[SRR] += (-2*r*rho*nu*spp)*dVdt;
   double srp = 0.5*(r*r*gr[UPP] + gp[URR]);
   double spz = 0.5*(gp[UZZ] + r*r*gz[UPP]);
   double om_r = get_om1(x), om_z = 0.0;
   cons[TAU] += (2*rho*nu*(srp*om_r + spz*om_z))*dVdt;
}
static double e_mindt(const double *prim, double w, const double *xp, const double *xm)
{
   double r = centroid(xp[0], xm[0], 1);
   double Pp = prim[PPP], rho = prim[RHO];
   double vp = (prim[UPP] - w)*r, vr = prim[URR], vz = prim[UZZ];
   double cs = sqrt(D->gam*Pp/rho);
   double maxvr = cs + fabs(vr), maxvp = cs + fabs(vp), maxvz = cs + fabs(vz);
   double dtr = get_dL(xp, xm, 1)/maxvr;
   double dtp = get_dL(xp, xm, 0)/maxvp;
   double dtz = get_dL(xp, xm, 2)/maxvz;
   double dt = dtr;
   if(dt > dtp) dt = dtp;
   if(dt > dtz) dt = dtz;
   if(D->par.visc_flag) {   /* euler.c:351-373 */
      double dL0 = get_dL(xp, xm, 0), dL1 = get_dL(xp, xm, 1), dL2 = get_dL(xp, xm, 2);
      double dx = dL0;
      if(dx > dL1) dx = dL1;
      if(dx > dL2) dx = dL2;
      double nu = D->par.viscosity;
      if(D->par.alpha_flag) {
         double x[3];
         centroid_arr(xp, xm, x);
         double c2 = D->gam*prim[PPP]/prim[RHO];
         nu = D->par.viscosity*c2/get_height_om(x);
      }
      double dt_visc = 0.5*dx*dx/nu;
      if(dt > dt_visc) dt = dt_visc;
   }
   return dt;
}

/* ---- Hydro/mhd.c ----------------------------------------------------------- */
static void m_prim2cons(const double *prim, double *cons, const double *x, double dV)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double om = get_om(x);
   double vp_off = vp - om*r;
   double Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   double B2 = Br*Br + Bp*Bp + Bz*Bz;
   double rhoe = Pp/(D->gam - 1.);
   cons[DDD] = rho*dV;
   cons[TAU] = (.5*rho*v2 + rhoe + .5*B2)*dV;
   cons[SRR] = rho*vr*dV;
   cons[LLL] = r*rho*vp*dV;
   cons[SZZ] = rho*vz*dV;
   cons[BRR] = Br*dV*(1.0/r);
   cons[BPP] = Bp*dV/r;
   cons[BZZ] = Bz*dV;
   for(int q = D->nc; q < D->nq; q++) cons[q] = prim[q]*cons[DDD];
}
static void m_cons2prim(const double *cons, double *prim, const double *x, double dV)
{
   double r = x[0];
   double rho = cons[DDD]/dV;
   if(rho < D->par.Density_Floor) rho = D->par.Density_Floor;
   double Sr = cons[SRR]/dV, Sp = cons[LLL]/dV/r, Sz = cons[SZZ]/dV, E = cons[TAU]/dV;
   double om = get_om(x);
   double vr = Sr/rho, vp = Sp/rho, vp_off = vp - om*r, vz = Sz/rho;
   double Br = cons[BRR]/(dV*(1.0/r));
   double Bp = cons[BPP]/dV*r;
   double Bz = cons[BZZ]/dV;
   double B2 = Br*Br + Bp*Bp + Bz*Bz;
   double KE = .5*(Sr*vr + rho*vp_off*vp_off + Sz*vz);
   double rhoe = E - KE - .5*B2;
   double Pp = (D->gam - 1.)*rhoe;
   if(Pp < D->par.Pressure_Floor*rho) Pp = D->par.Pressure_Floor*rho;
   if(D->par.isothermal_flag) Pp = get_cs2(x)*rho/D->gam;
   prim[RHO] = rho; prim[PPP] = Pp; prim[URR] = vr; prim[UPP] = vp/r; prim[UZZ] = vz;
   prim[BRR] = Br; prim[BPP] = Bp; prim[BZZ] = Bz;
   for(int q = D->nc; q < D->nq; q++) prim[q] = cons[q]/cons[DDD];
}
static void m_flux(const double *prim, double *f, const double *x, const double *n)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
   double vn = vr*n[0] + vp*n[1] + vz*n[2];
   double Bn = Br*n[0] + Bp*n[1] + Bz*n[2];
   double vB = vr*Br + vp*Bp + vz*Bz;
   double rhoe = Pp/(D->gam - 1.);
   double v2 = vr*vr + vp*vp + vz*vz;
   double B2 = Br*Br + Bp*Bp + Bz*Bz;
   f[DDD] = rho*vn;
   f[SRR] = rho*vr*vn + (Pp + .5*B2)*n[0] - Br*Bn;
   f[LLL] = r*(rho*vp*vn + (Pp + .5*B2)*n[1] - Bp*Bn);
   f[SZZ] = rho*vz*vn + (Pp + .5*B2)*n[2] - Bz*Bn;
   f[TAU] = (.5*rho*v2 + rhoe + Pp + B2)*vn - vB*Bn;
   f[BRR] = (Br*vn - vr*Bn)*(1.0/r);
   f[BPP] = (Bp*vn - vp*Bn)/r;
   f[BZZ] = Bz*vn - vz*Bn;
   for(int q = D->nc; q < D->nq; q++) f[q] = prim[q]*f[DDD];
}
static void m_source(const double *prim, double *cons, const double *xp, const double *xm,
                     double dVdt)
{
   double rp = xp[0], rm = xm[0];
   double dphi = get_dp(xp[1], xm[1]);
   double rho = prim[RHO], Pp = prim[PPP];
   double r_1 = .5*(rp + rm);
   double r2_3 = (rp*rp + rp*rm + rm*rm)/3.;
   double vr = prim[URR], omega = prim[UPP];
   double r = centroid(rp, rm, 1), z = centroid(xp[2], xm[2], 2);
   double x[3] = {r, 0.5*(xm[1] + xp[1]), z};
   double Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
   double B2 = Br*Br + Bp*Bp + Bz*Bz;
   double centrifugal;
   if(D->NgRa == 0) {
      centrifugal = (rho*omega*omega*r2_3)/r_1*sin(.5*dphi)/(.5*dphi);
      centrifugal -= Bp*Bp/r_1;
   } else {
      centrifugal = rho*omega*omega*r - Bp*Bp/r;
   }
   double press_bal = (Pp + .5*B2)/r_1;
   cons[SRR] += dVdt*(centrifugal + press_bal);
   double om = get_om(x), om1 = get_om1(x);
   cons[TAU] += dVdt*rho*vr*(om*om*r2_3/r_1 - om1*(omega - om)*r2_3);
   if(D->par.visc_flag) cons[SRR] += -dVdt*D->par.viscosity*rho*vr/(r_1*r_1);
}
static void m_flux_to_E(const double *Flux, const double *Ustr, const double *x,
                        double *E1, double *B1, double *E2, double *B2, int dim)
{
   double r = x[0];
   double irfac = 1.0/(1.0/x[0]);
   if(dim == 0) {
      *E1 = Flux[BRR]*irfac; *B1 = Ustr[BRR]*irfac; *E2 = -Flux[BZZ]; *B2 = Ustr[BZZ];
   } else if(dim == 1) {
      *E1 = -Flux[BPP]*r; *B1 = Ustr[BRR]*irfac; *E2 = Flux[BZZ];
   } else {
      *E1 = Flux[BPP]*r; *B1 = Ustr[BZZ]; *E2 = -Flux[BRR]*irfac;
   }
}
static double m_mindt(const double *prim, double w, const double *xp, const double *xm)
{
   double r = centroid(xp[0], xm[0], 1);
   double Pp = prim[PPP], rho = prim[RHO];
   double vp = (prim[UPP] - w)*r, vr = prim[URR], vz = prim[UZZ];
   double cs = sqrt(D->gam*Pp/rho);
   double Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
   double b2 = (Br*Br + Bp*Bp + Bz*Bz)/rho;
   double cf = sqrt(cs*cs + b2);
   double maxvr = cf + fabs(vr), maxvp = cf + fabs(vp), maxvz = cf + fabs(vz);
   double dtr = get_dL(xp, xm, 1)/maxvr;
   double dtp = get_dL(xp, xm, 0)/maxvp;
   double dtz = get_dL(xp, xm, 2)/maxvz;
   double dt = dtr;
   if(dt > dtp) dt = dtp;
   if(dt > dtz) dt = dtz;
   return dt;
}

/* ---- hlld.c: 5-wave solver with face speed w ------------------------------ */
static void h_velocities(const double *pL, const double *pR, const double *n, double *vel,
                         double *Pt_star)
{
   double gam = D->gam;
   double rho_L = pL[RHO], P_L = pL[PPP];
   double u_L = pL[URR]*n[0] + pL[UPP]*n[1] + pL[UZZ]*n[2];
   double Bn_L = pL[BRR]*n[0] + pL[BPP]*n[1] + pL[BZZ]*n[2];
   double B2_L = pL[BRR]*pL[BRR] + pL[BPP]*pL[BPP] + pL[BZZ]*pL[BZZ];
   double Pt_L = P_L + .5*B2_L;
   double rho_R = pR[RHO], P_R = pR[PPP];
   double u_R = pR[URR]*n[0] + pR[UPP]*n[1] + pR[UZZ]*n[2];
   double Bn_R = pR[BRR]*n[0] + pR[BPP]*n[1] + pR[BZZ]*n[2];
   double B2_R = pR[BRR]*pR[BRR] + pR[BPP]*pR[BPP] + pR[BZZ]*pR[BZZ];
   double Pt_R = P_R + .5*B2_R;
   double Bn = .5*(Bn_L + Bn_R);
   double aL = gam*P_L + B2_L, aR = gam*P_R + B2_R;
   double cf2_L = .5*(gam*P_L + B2_L + sqrt(fabs(aL*aL - 4.*gam*P_L*Bn_L*Bn_L)))/rho_L;
   double cf2_R = .5*(gam*P_R + B2_R + sqrt(fabs(aR*aR - 4.*gam*P_R*Bn_R*Bn_R)))/rho_R;
   double cf2 = cf2_L > cf2_R ? cf2_L : cf2_R;
   double umin, umax;
   if(u_L < u_R) { umin = u_L; umax = u_R; } else { umin = u_R; umax = u_L; }
   double S_R = umax + sqrt(fabs(cf2));
   double S_L = umin - sqrt(fabs(cf2));
   double S_M = ((S_R - u_R)*rho_R*u_R - (S_L - u_L)*rho_L*u_L - Pt_R + Pt_L)/
                ((S_R - u_R)*rho_R - (S_L - u_L)*rho_L);
   double rhostar_L = rho_L*(S_L - u_L)/(S_L - S_M);
   double rhostar_R = rho_R*(S_R - u_R)/(S_R - S_M);
   vel[0] = S_L;
   vel[1] = S_M - fabs(Bn)/sqrt(rhostar_L);
   vel[2] = S_M;
   vel[3] = S_M + fabs(Bn)/sqrt(rhostar_R);
   vel[4] = S_R;
   double num = (S_R - u_R)*rho_R*Pt_L - (S_L - u_L)*rho_L*Pt_R +
                rho_L*rho_R*(S_R - u_R)*(S_L - u_L)*(u_R - u_L);
   double denom = (S_R - u_R)*rho_R - (S_L - u_L)*rho_L;
   *Pt_star = num/denom;
}
static void h_prim_to_cons(const double *prim, double *cons)
{
   double rho = prim[RHO], Pp = prim[PPP], vx = prim[URR], vy = prim[UPP], vz = prim[UZZ];
   double Bx = prim[BRR], By = prim[BPP], Bz = prim[BZZ];
   double v2 = vx*vx + vy*vy + vz*vz;
   double rhoe = Pp/(D->gam - 1.);
   double B2 = Bx*Bx + By*By + Bz*Bz;
   cons[DDD] = rho; cons[SRR] = rho*vx; cons[LLL] = rho*vy; cons[SZZ] = rho*vz;
   cons[TAU] = (.5*rho*v2 + rhoe + .5*B2);
   cons[BRR] = Bx; cons[BPP] = By; cons[BZZ] = Bz;
}
static void h_flux(const double *prim, double *flux, const double *n)
{
   double rho = prim[RHO], Pp = prim[PPP], vx = prim[URR], vy = prim[UPP], vz = prim[UZZ];
   double Bx = prim[BRR], By = prim[BPP], Bz = prim[BZZ];
   double v2 = vx*vx + vy*vy + vz*vz;
   double vB = vx*Bx + vy*By + vz*Bz;
   double B2 = Bx*Bx + By*By + Bz*Bz;
   double vn = vx*n[0] + vy*n[1] + vz*n[2];
   double Bn = Bx*n[0] + By*n[1] + Bz*n[2];
   double rhoe = Pp/(D->gam - 1.);
   flux[DDD] = rho*vn;
   flux[SRR] = rho*vx*vn + (Pp + .5*B2)*n[0] - Bx*Bn;
   flux[LLL] = rho*vy*vn + (Pp + .5*B2)*n[1] - By*Bn;
   flux[SZZ] = rho*vz*vn + (Pp + .5*B2)*n[2] - Bz*Bn;
   flux[TAU] = (.5*rho*v2 + rhoe + Pp + B2)*vn - vB*Bn;
   flux[BRR] = Bx*vn - vx*Bn;
   flux[BPP] = By*vn - vy*Bn;
   flux[BZZ] = Bz*vn - vz*Bn;
}
static void h_single_star(const double *prim, double *Us, double S_K, double S_M,
                          double Pt_star, const double *n)
{
   double rho = prim[RHO], vx = prim[URR], vy = prim[UPP], vz = prim[UZZ], Pp = prim[PPP];
   double Bx = prim[BRR], By = prim[BPP], Bz = prim[BZZ];
   double u_K = vx*n[0] + vy*n[1] + vz*n[2];
   double Bn = Bx*n[0] + By*n[1] + Bz*n[2];
   double vdotB = vx*Bx + vy*By + vz*Bz;
   double v2 = vx*vx + vy*vy + vz*vz;
   double B2 = Bx*Bx + By*By + Bz*Bz;
   double Pt = Pp + .5*B2;
   double e = .5*rho*v2 + Pp/(D->gam - 1.) + .5*B2;
   double rhostar = rho*(S_K - u_K)/(S_K - S_M);
   double denom = rho*(S_K - u_K)*(S_K - S_M) - Bn*Bn;
   if(fabs(denom) < TOL_HLLD) denom = TOL_HLLD;
   double vx_s = vx - Bn*Bx*(S_M - u_K)/denom;
   double vy_s = vy - Bn*By*(S_M - u_K)/denom;
   double vz_s = vz - Bn*Bz*(S_M - u_K)/denom;
   double sq = (S_K - u_K)*(S_K - u_K);
   double Bx_s = Bx*(rho*sq - Bn*Bn)/denom;
   double By_s = By*(rho*sq - Bn*Bn)/denom;
   double Bz_s = Bz*(rho*sq - Bn*Bn)/denom;
   double vn_s = vx_s*n[0] + vy_s*n[1] + vz_s*n[2];
   double Bn_s = Bx_s*n[0] + By_s*n[1] + Bz_s*n[2];
   vx_s += (S_M - vn_s)*n[0]; vy_s += (S_M - vn_s)*n[1]; vz_s += (S_M - vn_s)*n[2];
   Bx_s += (Bn - Bn_s)*n[0]; By_s += (Bn - Bn_s)*n[1]; Bz_s += (Bn - Bn_s)*n[2];
   double vB_s = vx_s*Bx_s + vy_s*By_s + vz_s*Bz_s;
   double e_s = ((S_K - u_K)*e - Pt*u_K + Pt_star*S_M + Bn*(vdotB - vB_s))/(S_K - S_M);
   Us[DDD] = rhostar; Us[SRR] = rhostar*vx_s; Us[LLL] = rhostar*vy_s; Us[SZZ] = rhostar*vz_s;
   Us[TAU] = e_s; Us[BRR] = Bx_s; Us[BPP] = By_s; Us[BZZ] = Bz_s;
}
static void h_double_star(const double *UsL, const double *UsR, double *Uss, const double *vel,
                          const double *n, int LR)
{
   double rho_L = UsL[DDD], rho_R = UsR[DDD];
   double rhostar_K = LR == 0 ? rho_L : rho_R;
   double rrh_L = sqrt(rho_L), rrh_R = sqrt(rho_R), rrh_K = sqrt(rhostar_K);
   double vx_L = UsL[SRR]/rho_L, vy_L = UsL[LLL]/rho_L, vz_L = UsL[SZZ]/rho_L;
   double Bx_L = UsL[BRR], By_L = UsL[BPP], Bz_L = UsL[BZZ];
   double vx_R = UsR[SRR]/rho_R, vy_R = UsR[LLL]/rho_R, vz_R = UsR[SZZ]/rho_R;
   double Bx_R = UsR[BRR], By_R = UsR[BPP], Bz_R = UsR[BZZ];
   double Bn_L = Bx_L*n[0] + By_L*n[1] + Bz_L*n[2];
   double Bn_R = Bx_R*n[0] + By_R*n[1] + Bz_R*n[2];
   double Bn = .5*(Bn_L + Bn_R);
   double sB = Bn > 0.0 ? 1.0 : -1.0;
   double den = rrh_L + rrh_R;
   double vx = (rrh_L*vx_L + rrh_R*vx_R + (Bx_R - Bx_L)*sB)/den;
   double vy = (rrh_L*vy_L + rrh_R*vy_R + (By_R - By_L)*sB)/den;
   double vz = (rrh_L*vz_L + rrh_R*vz_R + (Bz_R - Bz_L)*sB)/den;
   double vn = vx*n[0] + vy*n[1] + vz*n[2];
   vx += (vel[2] - vn)*n[0]; vy += (vel[2] - vn)*n[1]; vz += (vel[2] - vn)*n[2];
   double Bx = (rrh_L*Bx_R + rrh_R*Bx_L + rrh_L*rrh_R*(vx_R - vx_L)*sB)/den;
   double By = (rrh_L*By_R + rrh_R*By_L + rrh_L*rrh_R*(vy_R - vy_L)*sB)/den;
   double Bz = (rrh_L*Bz_R + rrh_R*Bz_L + rrh_L*rrh_R*(vz_R - vz_L)*sB)/den;
   double Bns = Bx*n[0] + By*n[1] + Bz*n[2];
   Bx += (Bn - Bns)*n[0]; By += (Bn - Bns)*n[1]; Bz += (Bn - Bns)*n[2];
   double vB_ss = vx*Bx + vy*By + vz*Bz;
   double vBstar, e_star;
   if(LR == 0) { vBstar = vx_L*Bx_L + vy_L*By_L + vz_L*Bz_L; e_star = UsL[TAU]; }
   else { vBstar = vx_R*Bx_R + vy_R*By_R + vz_R*Bz_R; e_star = UsR[TAU]; }
   double pm = LR == 1 ? 1.0 : -1.0;
   double e_ss = e_star + pm*rrh_K*(vBstar - vB_ss)*sB;
   Uss[DDD] = rhostar_K; Uss[SRR] = rhostar_K*vx; Uss[LLL] = rhostar_K*vy; Uss[SZZ] = rhostar_K*vz;
   Uss[TAU] = e_ss; Uss[BRR] = Bx; Uss[BPP] = By; Uss[BZZ] = Bz;
}
static void h_ustar(double w, const double *primL, const double *primR, double *F, double *U,
                    const double *x, const double *n)
{
   double vel[5], Pt_star;
   double hr = 1.0, hp = x[0], hz = 1.0;
   double pL[MAXQ], pR[MAXQ];
   int q, nq = D->nq;
   memcpy(pL, primL, nq*sizeof(double));
   memcpy(pR, primR, nq*sizeof(double));
   pL[URR] *= hr; pR[URR] *= hr;
   pL[UPP] *= hp; pR[UPP] *= hp;
   pL[UZZ] *= hz; pR[UZZ] *= hz;
   h_velocities(pL, pR, n, vel, &Pt_star);
   if(w < vel[2]) {
      double UL[8];
      h_flux(pL, F, n);
      h_prim_to_cons(pL, UL);
      if(w < vel[0]) {
         h_prim_to_cons(pL, U);
      } else if(w < vel[1]) {
         h_single_star(pL, U, vel[0], vel[2], Pt_star, n);
         for(q = 0; q < 8; q++) F[q] += vel[0]*(U[q] - UL[q]);
      } else {
         double UsL[8], UsR[8];
         h_single_star(pL, UsL, vel[0], vel[2], Pt_star, n);
         h_single_star(pR, UsR, vel[4], vel[2], Pt_star, n);
         h_double_star(UsL, UsR, U, vel, n, 0);
         for(q = 0; q < 8; q++) F[q] += vel[1]*(U[q] - UsL[q]) + vel[0]*(UsL[q] - UL[q]);
      }
      for(q = 8; q < nq; q++) { U[q] = pL[q]*U[DDD]; F[q] = pL[q]*F[DDD]; }
   } else {
      double UR[8];
      h_flux(pR, F, n);
      h_prim_to_cons(pR, UR);
      if(w > vel[4]) {
         h_prim_to_cons(pR, U);
      } else if(w > vel[3]) {
         h_single_star(pR, U, vel[4], vel[2], Pt_star, n);
         for(q = 0; q < 8; q++) F[q] += vel[4]*(U[q] - UR[q]);
      } else {
         double UsL[8], UsR[8];
         h_single_star(pL, UsL, vel[0], vel[2], Pt_star, n);
         h_single_star(pR, UsR, vel[4], vel[2], Pt_star, n);
         h_double_star(UsL, UsR, U, vel, n, 1);
         for(q = 0; q < 8; q++) F[q] += vel[3]*(U[q] - UsR[q]) + vel[4]*(UsR[q] - UR[q]);
      }
      for(q = 8; q < nq; q++) { U[q] = pR[q]*U[DDD]; F[q] = pR[q]*F[DDD]; }
   }
   double brfac = 1.0/x[0], bpfac = 1.0, bzfac = 1.0;
   F[SRR] *= hr; F[LLL] *= hp; F[SZZ] *= hz;
   F[BRR] *= brfac/hr; F[BPP] *= bpfac/hp; F[BZZ] *= bzfac/hz;
   U[SRR] *= hr; U[LLL] *= hp; U[SZZ] *= hz;
   U[BRR] *= brfac/hr; U[BPP] *= bpfac/hp; U[BZZ] *= bzfac/hz;
}

/* ---- module dispatch --------------------------------------------------------- */
static void prim2cons(const double *p, double *c, const double *x, double dV)
{ if(D->mhd) m_prim2cons(p, c, x, dV); else e_prim2cons(p, c, x, dV); }
static void cons2prim(const double *c, double *p, const double *x, double dV)
{ if(D->mhd) m_cons2prim(c, p, x, dV); else e_cons2prim(c, p, x, dV); }
static void flux(const double *p, double *f, const double *x, const double *n)
{ if(D->mhd) m_flux(p, f, x, n); else e_flux(p, f, x, n); }
static double mindt(const double *p, double w, const double *xp, const double *xm)
{ return D->mhd ? m_mindt(p, w, xp, xm) : e_mindt(p, w, xp, xm); }

/* ---- riemann.c:216-320 ------------------------------------------------------- */
/* mhd.c's wave-speed bounds for HLL/HLLC (vel, :318-450): the fast
 * magnetosonic speeds of both states bound the fan, the contact speed comes
 * from the total-pressure balance, and Bpack carries the HLL average of B
 * (normal component, r, phi, z) and v.B for the star state. */
static void m_vel(const double *p1, const double *p2, double *Sl, double *Sr, double *Ss,
                  const double *n, const double *x, double *Bpack)
{
   const double r = x[0], gam = D->par.Adiabatic_Index;
   const double *pp[2] = {p1, p2};
   double v[2][3], B[2][3], rho[2], P[2], vn[2], Bn[2], B2[2], cf[2];
   double m[2][3], Fm[2][3], FB[2][3];
   for(int s = 0; s < 2; s++) {
      const double *p = pp[s];
      rho[s] = p[RHO]; P[s] = p[PPP];
      v[s][0] = p[URR]; v[s][1] = r*p[UPP]; v[s][2] = p[UZZ];
      B[s][0] = p[BRR]; B[s][1] = p[BPP]; B[s][2] = p[BZZ];
      vn[s] = v[s][0]*n[0] + v[s][1]*n[1] + v[s][2]*n[2];
      Bn[s] = B[s][0]*n[0] + B[s][1]*n[1] + B[s][2]*n[2];
      B2[s] = B[s][0]*B[s][0] + B[s][1]*B[s][1] + B[s][2]*B[s][2];
      double cs = sqrt(gam*(P[s]/rho[s])), b2 = B2[s]/rho[s];
      double a = cs*cs + b2;
      cf[s] = .5*(cs*cs + b2 + sqrt(fabs(a*a - 4.0*cs*cs*Bn[s]*Bn[s]/rho[s])));
      for(int c = 0; c < 3; c++) {
         FB[s][c] = vn[s]*B[s][c] - Bn[s]*v[s][c];
         m[s][c] = rho[s]*v[s][c];
         Fm[s][c] = rho[s]*v[s][c]*vn[s] + (P[s] + .5*B2[s])*n[c] - B[s][c]*Bn[s];
      }
   }
   double Lm = vn[0] - sqrt(cf[0]), Lp = vn[0] + sqrt(cf[0]);
   if(Lm > vn[1] - sqrt(cf[1])) Lm = vn[1] - sqrt(cf[1]);
   if(Lp < vn[1] + sqrt(cf[1])) Lp = vn[1] + sqrt(cf[1]);
   const double aL = Lp, aR = -Lm;
   double Bh[3], mh[3];
   for(int c = 0; c < 3; c++) {
      Bh[c] = (aR*B[0][c] + aL*B[1][c] + FB[0][c] - FB[1][c])/(aL + aR);
      mh[c] = (aR*m[0][c] + aL*m[1][c] + Fm[0][c] - Fm[1][c])/(aL + aR);
   }
   double Bnh = Bh[0]*n[0] + Bh[1]*n[1] + Bh[2]*n[2];
   double mnL = m[0][0]*n[0] + m[0][1]*n[1] + m[0][2]*n[2];
   double mnR = m[1][0]*n[0] + m[1][1]*n[1] + m[1][2]*n[2];
   double rhoh = (aR*rho[0] + aL*rho[1] + mnL - mnR)/(aL + aR);
   *Ss = (rho[1]*vn[1]*(Lp - vn[1]) - rho[0]*vn[0]*(Lm - vn[0])
          + (P[0] + .5*B2[0] - Bn[0]*Bn[0]) - (P[1] + .5*B2[1] - Bn[1]*Bn[1]))
         /(rho[1]*(Lp - vn[1]) - rho[0]*(Lm - vn[0]));
   double vh[3] = {mh[0]/rhoh, mh[1]/rhoh, mh[2]/rhoh};
   Bpack[0] = Bnh; Bpack[1] = Bh[0]; Bpack[2] = Bh[1]; Bpack[3] = Bh[2];
   Bpack[4] = vh[0]*Bh[0] + vh[1]*Bh[1] + vh[2]*Bh[2];
   *Sl = Lm;
   *Sr = Lp;
}

/* mhd.c's HLLC star state (getUstar, :71-137) of the side with wave speed
 * Sk, contact Ss and the HLL field Bpack of m_vel */
static void m_getUstar(const double *prim, double *Us, const double *x, double Sk, double Ss,
                       const double *n, const double *Bpack)
{
   const double r = x[0], gam = D->par.Adiabatic_Index;
   const double Bsn = Bpack[0], Bs[3] = {Bpack[1], Bpack[2], Bpack[3]}, vBs = Bpack[4];
   const double rho = prim[RHO], Pp = prim[PPP];
   const double v[3] = {prim[URR], prim[UPP]*r, prim[UZZ]};
   const double B[3] = {prim[BRR], prim[BPP], prim[BZZ]};
   double v2 = v[0]*v[0] + v[1]*v[1] + v[2]*v[2], B2 = B[0]*B[0] + B[1]*B[1] + B[2]*B[2];
   double vn = v[0]*n[0] + v[1]*n[1] + v[2]*n[2], Bn = B[0]*n[0] + B[1]*n[1] + B[2]*n[2];
   double vB = v[0]*B[0] + v[1]*B[1] + v[2]*B[2];
   double E = .5*rho*v2 + Pp/(gam - 1.) + .5*B2;
   double Bs2 = Bs[0]*Bs[0] + Bs[1]*Bs[1] + Bs[2]*Bs[2];
   double Ps = rho*(Sk - vn)*(Ss - vn) + (Pp + .5*B2 - Bn*Bn) - .5*Bs2 + Bsn*Bsn;
   double Ds = (Sk - vn)*rho/(Sk - Ss);
   double Ms[3];
   for(int c = 0; c < 3; c++) {
      const double mc = rho*v[c];   /* the momentum first, as mhd.c forms it */
      Ms[c] = ((Sk - vn)*mc + (B[c]*Bn - Bs[c]*Bsn))/(Sk - Ss);
   }
   double Es = ((Sk - vn)*E + (Ps + .5*Bs2)*Ss - (Pp + .5*B2)*vn - vBs*Bsn + vB*Bn)/(Sk - Ss);
   double Msn = Ds*Ss, mn = Ms[0]*n[0] + Ms[1]*n[1] + Ms[2]*n[2];
   for(int c = 0; c < 3; c++) Ms[c] += n[c]*(Msn - mn);
   Us[DDD] = Ds; Us[SRR] = Ms[0]; Us[LLL] = r*Ms[1]; Us[SZZ] = Ms[2]; Us[TAU] = Es;
   Us[BRR] = Bs[0]*(1.0/r);   /* bfield_scale_factor(r, 0) = 1 / r (mhd.c:518) */
   Us[BPP] = Bs[1]/r;
   Us[BZZ] = Bs[2];
   for(int q = D->nc; q < D->nq; q++) Us[q] = prim[q]*Us[DDD];
}

static void solve_riemann(const double *primL, const double *primR, double *consL, double *consR,
                          const double *gLr, const double *gLp, const double *gLz,
                          const double *gRr, const double *gRp, const double *gRz,
                          const double *x, const double *n, double w, double dAdt, int dim,
                          double *E1, double *B1, double *E2, double *B2)
{
   int nq = D->nq, q;
   double Flux[MAXQ] = {0}, Ustr[MAXQ] = {0};
   int solver = D->par.Riemann_Solver;   /* 0 HLL, 1 HLLC, 2 HLLD, 3 HLLC with HLL for r < 0.1 */
   if(solver == 0 || solver == 1 || solver == 3) {
      double Sl, Sr, Ss, Bpack[5];
      if(D->mhd) m_vel(primL, primR, &Sl, &Sr, &Ss, n, x, Bpack);
      else e_vel(primL, primR, &Sl, &Sr, &Ss, n, x);
      if(w < Sl) {
         flux(primL, Flux, x, n);
         prim2cons(primL, Ustr, x, 1.0);
      } else if(w > Sr) {
         flux(primR, Flux, x, n);
         prim2cons(primR, Ustr, x, 1.0);
      } else if(solver == 0 || (x[0] < 0.1 && solver == 3)) {
         double Fl[MAXQ], Fr[MAXQ], Ul[MAXQ], Ur[MAXQ];
         double aL = Sr, aR = -Sl;
         prim2cons(primL, Ul, x, 1.0);
         prim2cons(primR, Ur, x, 1.0);
         flux(primL, Fl, x, n);
         flux(primR, Fr, x, n);
         for(q = 0; q < nq; q++) {
            Flux[q] = (aL*Fl[q] + aR*Fr[q] + aL*aR*(Ul[q] - Ur[q]))/(aL + aR);
            Ustr[q] = (aR*Ul[q] + aL*Ur[q] + Fl[q] - Fr[q])/(aL + aR);
         }
      } else {
         double Uk[MAXQ], Fk[MAXQ];
         if(w < Ss) {
            prim2cons(primL, Uk, x, 1.0);
            if(D->mhd) m_getUstar(primL, Ustr, x, Sl, Ss, n, Bpack);
            else e_getUstar(primL, Ustr, x, Sl, Ss, n);
            flux(primL, Fk, x, n);
            for(q = 0; q < nq; q++) Flux[q] = Fk[q] + Sl*(Ustr[q] - Uk[q]);
         } else {
            prim2cons(primR, Uk, x, 1.0);
            if(D->mhd) m_getUstar(primR, Ustr, x, Sr, Ss, n, Bpack);
            else e_getUstar(primR, Ustr, x, Sr, Ss, n);
            flux(primR, Fk, x, n);
            for(q = 0; q < nq; q++) Flux[q] = Fk[q] + Sr*(Ustr[q] - Uk[q]);
         }
      }
   } else {
      h_ustar(w, primL, primR, Flux, Ustr, x, n);
   }
   if(D->par.visc_flag && !D->mhd) {   /* riemann.c:297-312 (mhd.c has no viscous flux) */
      double vF[MAXQ], pm[MAXQ], gr[MAXQ], gp[MAXQ], gz[MAXQ];
      for(q = 0; q < nq; q++) {
         pm[q] = .5*(primL[q] + primR[q]);
         gr[q] = .5*(gLr[q] + gRr[q]);
         gp[q] = .5*(gLp[q] + gRp[q]);
         gz[q] = .5*(gLz[q] + gRz[q]);
         vF[q] = 0.0;
      }
      e_visc_flux(pm, gr, gp, gz, vF, x, n);
      for(q = 0; q < nq; q++) Flux[q] += vF[q];
   }
   for(q = 0; q < nq; q++) {
      consL[q] -= (Flux[q] - w*Ustr[q])*dAdt;
      consR[q] += (Flux[q] - w*Ustr[q])*dAdt;
   }
   if(D->mhd) m_flux_to_E(Flux, Ustr, x, E1, B1, E2, B2, dim);
}

/* ---- faces: faces_alt.c:36-179 (sequential walk) ------------------------------ */
static void build_faces(int dim)
{
   int Nr = D->Nr, Nz = D->Nz, j, k, i, jk;
   int *I0 = (int *)malloc(sizeof(int)*Nr*Nz);
   for(jk = 0; jk < Nr*Nz; jk++) {
      int found = 0, quad_prev = 0;
      for(i = 0; i < D->Np[jk] && !found; i++) {
         double convert = 2.*M_PI/D->Pmax;
         double ph = D->ring[jk][i].piph;
         double sn = sin(ph*convert), cs = cos(ph*convert);
         if(sn > 0. && cs > 0. && quad_prev) { found = 1; I0[jk] = i; }
         else if(sn < 0. && cs > 0.) quad_prev = 1;
      }
      if(!found) I0[jk] = 0;
   }
   int Nrmax = dim == 1 ? Nr - 1 : Nr;
   int Nzmax = dim == 1 ? Nz : Nz - 1;
   int d0 = dim - 1, n = 0;
   for(k = 0; k < Nzmax; k++) for(j = 0; j < Nrmax; j++) {
      int L = j + Nr*k, R = dim == 1 ? j + 1 + Nr*k : j + Nr*(k + 1);
      D->fI[d0][j + Nrmax*k] = n;
      n += D->Np[L] + D->Np[R];
   }
   D->fI[d0][Nrmax*Nzmax] = n;
   D->ntracks[d0] = Nrmax*Nzmax;
   free(D->faces[d0]);
   D->faces[d0] = (pface *)malloc(sizeof(pface)*(n > 0 ? n : 1));
   const double *rj = D->rj, *zk = D->zk;
   n = 0;
   for(k = 0; k < Nzmax; k++) for(j = 0; j < Nrmax; j++) {
      int jkL = j + Nr*k, jkR = dim == 1 ? j + 1 + Nr*k : j + Nr*(k + 1);
      double dxL, dxR;
      if(dim == 1) {
         double rm = centroid(rj[j], rj[j - 1], 1), rp = centroid(rj[j + 1], rj[j], 1);
         dxL = rj[j] - rm; dxR = rp - rj[j];
      } else {
         double zm = centroid(zk[k], zk[k - 1], 2), zp = centroid(zk[k + 1], zk[k], 2);
         dxL = zk[k] - zm; dxR = zp - zk[k];
      }
      double xp[3] = {rj[j], 0.0, zk[k]}, xm[3] = {rj[j], 0.0, zk[k - 1]};
      if(dim == 2) { xm[0] = rj[j - 1]; xm[2] = zk[k]; }
      int a = I0[jkL], b = I0[jkR], f;
      for(f = 0; f < D->Np[jkL] + D->Np[jkR]; f++) {
         pcell *cL = &D->ring[jkL][a], *cR = &D->ring[jkR][b];
         double dphi = cL->piph - cR->piph;
         while(dphi > .5*D->Pmax) dphi -= D->Pmax;
         while(dphi < -.5*D->Pmax) dphi += D->Pmax;
         int LR = dphi > 0. ? 1 : 0;
         dphi = cL->piph - cL->dphi - cR->piph + cR->dphi;
         while(dphi > .5*D->Pmax) dphi -= D->Pmax;
         while(dphi < -.5*D->Pmax) dphi += D->Pmax;
         int LR_back = dphi < 0. ? 1 : 0;
         xp[1] = LR == 0 ? cL->piph : cR->piph;
         xm[1] = LR_back == 0 ? cL->piph - cL->dphi : cR->piph - cR->dphi;
         pface *F = &D->faces[d0][n];
         double dp = get_dp(xp[1], xm[1]);
         F->cm[0] = dim == 1 ? 0.5*(xp[0] + xm[0]) : centroid(xp[0], xm[0], 1);
         F->cm[1] = get_dp(xp[1], .5*dp);
         F->cm[2] = dim == 2 ? 0.5*(xp[2] + xm[2]) : centroid(xp[2], xm[2], 2);
         F->L = cL; F->R = cR; F->dxL = dxL; F->dxR = dxR;
         F->dphi = dp; F->dA = get_dA(xp, xm, dim);
         F->dl = get_dL(xp, xm, 3 - dim);
         F->E = 0.0; F->B = 0.0; F->LRtype = LR; F->flip_flag = 0;
         n++;
         if(LR == 0) { a++; if(a == D->Np[jkL]) a = 0; }
         else { b++; if(b == D->Np[jkR]) b = 0; }
      }
   }
   free(I0);
}

/* ---- reconstruction: plm.c ----------------------------------------------------- */
static double minmod(double a, double b, double c)
{
   double m = a;
   if(a*b < 0.0) m = 0.0;
   if(fabs(b) < fabs(m)) m = b;
   if(b*c < 0.0) m = 0.0;
   if(fabs(c) < fabs(m)) m = c;
   return m;
}
static void plm_phi(void)
{
   double PLM = D->par.PLM;
   for(int jk = 0; jk < D->Nr*D->Nz; jk++) {
      int Np = D->Np[jk];
      for(int i = 0; i < Np; i++) {
         pcell *c = &D->ring[jk][i], *cL = &D->ring[jk][i == 0 ? Np - 1 : i - 1];
         pcell *cR = &D->ring[jk][(i + 1)%Np];
         double dpL = cL->dphi, dpC = c->dphi, dpR = cR->dphi;
         for(int q = 0; q < D->nq; q++) {
            double pL = cL->prim[q], pC = c->prim[q], pR = cR->prim[q];
            double sL = pC - pL; sL /= .5*(dpC + dpL);
            double sR = pR - pC; sR /= .5*(dpR + dpC);
            double sC = pR - pL; sC /= .5*(dpL + dpR) + dpC;
            c->gradp[q] = minmod(PLM*sL, sC, PLM*sR);
         }
      }
   }
}
static double *gsel(pcell *c, int dim) { return dim == 1 ? c->gradr : c->gradz; }
static void plm_trans(int dim)
{
   int nq = D->nq, q, n, j, k, i;
   for(j = 0; j < D->Nr; j++) for(k = 0; k < D->Nz; k++) {
      int jk = j + D->Nr*k;
      for(i = 0; i < D->Np[jk]; i++) memset(gsel(&D->ring[jk][i], dim), 0, sizeof(double)*MAXQ);
   }
   double PLM = D->par.PLM;
   if(PLM == 0.0) return;
   pface *Fs = D->faces[dim - 1];
   int Nf = D->fI[dim - 1][D->ntracks[dim - 1]];
   for(n = 0; n < Nf; n++) {
      pface *f = &Fs[n];
      double phi = f->cm[1];
      double phiL = f->L->piph - .5*f->L->dphi, phiR = f->R->piph - .5*f->R->dphi;
      double dpL = get_signed_dp(phi, phiL), dpR = get_signed_dp(phiR, phi);
      double *gL = gsel(f->L, dim), *gR = gsel(f->R, dim);
      for(q = 0; q < nq; q++) {
         double WL = f->L->prim[q] + dpL*f->L->gradp[q];
         double WR = f->R->prim[q] - dpR*f->R->gradp[q];
         double S = (WR - WL)/(f->dxR + f->dxL);
         gL[q] += S*f->dA;
         gR[q] += S*f->dA;
      }
   }
   for(j = 0; j < D->Nr; j++) for(k = 0; k < D->Nz; k++) {
      int jk = j + D->Nr*k;
      for(i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double phip = c->piph, phim = phip - c->dphi;
         double xp[3] = {D->rj[j], phip, D->zk[k]}, xm[3] = {D->rj[j - 1], phim, D->zk[k - 1]};
         if(dim == 1) xm[0] = D->rj[j]; else xm[2] = D->zk[k];
         double dAp = get_dA(xp, xm, dim);
         if(dim == 1) { xp[0] = D->rj[j - 1]; xm[0] = D->rj[j - 1]; }
         else { xp[2] = D->zk[k - 1]; xm[2] = D->zk[k - 1]; }
         double dAm = get_dA(xp, xm, dim);
         double dAtot = dAp + dAm;
         if((dim == 1 && j == 0) || (dim == 2 && k == 0)) dAtot = dAp;
         if((dim == 1 && j == D->Nr - 1) || (dim == 2 && k == D->Nz - 1)) dAtot = dAm;
         double *g = gsel(c, dim);
         for(q = 0; q < nq; q++) g[q] /= dAtot;
      }
   }
   for(n = 0; n < Nf; n++) {
      pface *f = &Fs[n];
      double phi = f->cm[1];
      double phiL = f->L->piph - .5*f->L->dphi, phiR = f->R->piph - .5*f->R->dphi;
      double dpL = get_signed_dp(phi, phiL), dpR = get_signed_dp(phiR, phi);
      double *gL = gsel(f->L, dim), *gR = gsel(f->R, dim);
      for(q = 0; q < nq; q++) {
         double WL = f->L->prim[q] + dpL*f->L->gradp[q];
         double WR = f->R->prim[q] - dpR*f->R->gradp[q];
         double S = (WR - WL)/(f->dxR + f->dxL);
         if(S*gL[q] < 0.0) gL[q] = 0.0; else if(fabs(PLM*S) < fabs(gL[q])) gL[q] = PLM*S;
         if(S*gR[q] < 0.0) gR[q] = 0.0; else if(fabs(PLM*S) < fabs(gR[q])) gR[q] = PLM*S;
      }
   }
   /* plm_geom_boundary (plm.c:184-232) at a coordinate inner edge: geom_grad
    * (cylindrical.c:141-173) acts only where the edge is r = 0. */
   if(dim == 1 && D->NgRa == 0 && !(D->rj[0] < 0.0 || fabs(D->rj[-1]) > 1.0e-10*D->rj[0])) {
      for(k = 0; k < D->Nz; k++) {
         double r = centroid(D->rj[0], D->rj[-1], 1);
         for(i = 0; i < D->Np[k*D->Nr]; i++) {
            pcell *c = &D->ring[k*D->Nr][i];
            for(q = 0; q < nq; q++) {
               if(q == URR || (D->nc > BZZ && q == BRR)) {
                  double SL = c->prim[q]/r, S = c->gradr[q];
                  if(S*SL < 0.0) c->gradr[q] = 0.0;
                  else if(fabs(PLM*SL) < fabs(S)) c->gradr[q] = PLM*SL;
               } else {
                  c->gradr[q] = 0.0;
               }
            }
         }
      }
   }
}

/* ---- fluxes: misc.c:378-519, riemann.c:39-214 ------------------------------------- */
static void riemann_phi(pcell *cL, pcell *cR, double *x, double dAdt)
{
   double primL[MAXQ], primR[MAXQ], gp[MAXQ];
   int q;
   for(q = 0; q < D->nq; q++) {
      primL[q] = cL->prim[q] + .5*cL->gradp[q]*cL->dphi;
      primR[q] = cR->prim[q] - .5*cR->gradp[q]*cR->dphi;
      gp[q] = (cR->prim[q] - cL->prim[q])/(0.5*(cR->dphi + cL->dphi));
   }
   double n[3] = {0.0, 1.0, 0.0};
   double hn = x[0];
   if(D->mhd) { double Bp = .5*(primL[BPP] + primR[BPP]); primL[BPP] = Bp; primR[BPP] = Bp; }
   double Er = 0, Ez = 0, Br = 0, Bz = 0;
   solve_riemann(primL, primR, cL->cons, cR->cons, cL->gradr, gp, cL->gradz, cR->gradr, gp, cR->gradz,
                 x, n, hn*cL->wiph, dAdt, 0, &Ez, &Br, &Er, &Bz);
   if(D->mhd && D->ct) {   /* NUM_EDGES == 8 */
      cL->E[0] = .5*Ez; cL->E[1] = .5*Ez; cR->E[2] = .5*Ez; cR->E[3] = .5*Ez;
      cL->B[0] = .5*Br; cL->B[1] = .5*Br; cR->B[2] = .5*Br; cR->B[3] = .5*Br;
      cL->E[4] = .5*Er; cL->E[5] = .5*Er; cR->E[6] = .5*Er; cR->E[7] = .5*Er;
      cL->B[4] = .5*Bz; cL->B[5] = .5*Bz; cR->B[6] = .5*Bz; cR->B[7] = .5*Bz;
   }
}
static void riemann_trans(pface *F, double dt, int dim)
{
   pcell *cL = F->L, *cR = F->R;
   double dAdt = F->dA*dt, phi = F->cm[1];
   double primL[MAXQ], primR[MAXQ], grad[MAXQ];
   double phiL = cL->piph - .5*cL->dphi, phiR = cR->piph - .5*cR->dphi;
   double dpL = get_signed_dp(phi, phiL), dpR = get_signed_dp(phiR, phi);
   double *gL = gsel(cL, dim), *gR = gsel(cR, dim);
   int q;
   for(q = 0; q < D->nq; q++) {
      primL[q] = cL->prim[q] + gL[q]*F->dxL + cL->gradp[q]*dpL;
      primR[q] = cR->prim[q] - gR[q]*F->dxR - cR->gradp[q]*dpR;
      grad[q] = ((cR->prim[q] - cR->gradp[q]*dpR) - (cL->prim[q] + cL->gradp[q]*dpL))/(F->dxL + F->dxR);
   }
   double n[3] = {0.0, 0.0, 0.0};
   if(dim == 1) n[0] = 1.0; else n[2] = 1.0;
   if(D->mhd) {
      int BT = dim == 1 ? BRR : BZZ;
      double Bavg = .5*(primL[BT] + primR[BT]);
      primL[BT] = Bavg; primR[BT] = Bavg;
   }
   double Erz = 0, Brz = 0, Ephi = 0;
   if(dim == 1)
      solve_riemann(primL, primR, cL->cons, cR->cons, grad, cL->gradp, cL->gradz,
                    grad, cR->gradp, cR->gradz, F->cm, n, 0.0, dAdt, dim, &Erz, &Brz, &Ephi, NULL);
   else
      solve_riemann(primL, primR, cL->cons, cR->cons, cL->gradr, cL->gradp, grad,
                    cR->gradr, cR->gradp, grad, F->cm, n, 0.0, dAdt, dim, &Erz, &Brz, &Ephi, NULL);
   if(!(D->mhd && D->ct)) return;
   double fracL = F->dphi/cL->dphi, fracR = F->dphi/cR->dphi;
   if(dim == 1) {
      cL->E[1] += .5*Erz*fracL; cL->E[3] += .5*Erz*fracL;
      cR->E[0] += .5*Erz*fracR; cR->E[2] += .5*Erz*fracR;
      cL->B[1] += .5*Brz*fracL; cL->B[3] += .5*Brz*fracL;
      cR->B[0] += .5*Brz*fracR; cR->B[2] += .5*Brz*fracR;
      if(F->LRtype == 0) cL->E_phi[1] = Ephi; else cR->E_phi[0] = Ephi;
   } else {
      cL->E[5] += .5*Erz*fracL; cL->E[7] += .5*Erz*fracL;
      cR->E[4] += .5*Erz*fracR; cR->E[6] += .5*Erz*fracR;
      cL->B[5] += .5*Brz*fracL; cL->B[7] += .5*Brz*fracL;
      cR->B[4] += .5*Brz*fracR; cR->B[6] += .5*Brz*fracR;
      if(F->LRtype == 0) cL->E_phi[3] = Ephi; else cR->E_phi[2] = Ephi;
   }
}
static void phi_flux(double dt)
{
   int jmin, jmax, kmin, kmax, j, k, i;
   if(D->mhd && D->ct) {
      jmin = D->NgRa == 0 ? 0 : D->NgRa - 1; jmax = D->NgRb == 0 ? D->Nr : D->Nr - D->NgRb + 1;
      kmin = D->NgZa == 0 ? 0 : D->NgZa - 1; kmax = D->NgZb == 0 ? D->Nz : D->Nz - D->NgZb + 1;
   } else {
      jmin = D->NgRa; jmax = D->Nr - D->NgRb; kmin = D->NgZa; kmax = D->Nz - D->NgZb;
   }
   for(k = kmin; k < kmax; k++) {
      double zp = D->zk[k], zm = D->zk[k - 1], z = centroid(zp, zm, 2);
      for(j = jmin; j < jmax; j++) {
         double rp = D->rj[j], rm = D->rj[j - 1], r = centroid(rp, rm, 1);
         int jk = j + D->Nr*k, Np = D->Np[jk];
         pcell *cp = D->ring[jk];
         for(i = 0; i < Np; i++) {
            int ip = i < Np - 1 ? i + 1 : 0;
            double phi = cp[i].piph;
            double xp[3] = {rp, phi, zp}, xm[3] = {rm, phi, zm};
            double dA = get_dA(xp, xm, 0);
            double x[3] = {r, phi, z};
            riemann_phi(&cp[i], &cp[ip], x, dA*dt);
         }
      }
   }
}
static void trans_flux(double dt, int dim)
{
   int jmin, jmax, kmin, kmax, Nfr, j, k;
   int ctx = D->mhd && D->ct;
   if(dim == 1) {
      Nfr = D->Nr - 1;
      jmin = D->NgRa == 0 ? 0 : D->NgRa - 1; jmax = D->NgRb == 0 ? D->Nr - 1 : D->Nr - D->NgRb;
      if(ctx) { kmin = D->NgZa == 0 ? 0 : D->NgZa - 1; kmax = D->NgZb == 0 ? D->Nz : D->Nz - D->NgZb + 1; }
      else { kmin = D->NgZa; kmax = D->Nz - D->NgZb; }
   } else {
      Nfr = D->Nr;
      if(ctx) { jmin = D->NgRa == 0 ? 0 : D->NgRa - 1; jmax = D->NgRb == 0 ? D->Nr : D->Nr - D->NgRb + 1; }
      else { jmin = D->NgRa; jmax = D->Nr - D->NgRb; }
      kmin = D->NgZa == 0 ? 0 : D->NgZa - 1; kmax = D->NgZb == 0 ? D->Nz - 1 : D->Nz - D->NgZb;
   }
   int *fI = D->fI[dim - 1];
   for(k = kmin; k < kmax; k++) for(j = jmin; j < jmax; j++) {
      int JK = j + Nfr*k;
      for(int f = fI[JK]; f < fI[JK + 1]; f++) riemann_trans(&D->faces[dim - 1][f], dt, dim);
   }
}

/* ---- constrained transport: bfields.c ------------------------------------------ */
static void B_faces_to_cells(int type)
{
   int Nr = D->Nr, Nz = D->Nz, j, k, i, n;
   for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
      int jk = j + Nr*k;
      for(i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         c->tempDoub = 0.0;
         if(type == 0) { c->prim[BRR] = 0.0; c->prim[BPP] = 0.0; c->prim[BZZ] = 0.0; }
         else { c->cons[BRR] = 0.0; c->cons[BPP] = 0.0; c->cons[BZZ] = 0.0; }
      }
   }
   int Nf = D->fI[0][D->ntracks[0]];
   for(n = 0; n < Nf; n++) {
      pface *f = &D->faces[0][n];
      double Phi = f->LRtype == 0 ? f->L->Phi[2] : f->R->Phi[1];
      f->L->tempDoub += f->dA;
      f->R->tempDoub += f->dA;
      if(type == 0) { f->L->prim[BRR] += Phi; f->R->prim[BRR] += Phi; }
      else { f->L->cons[BRR] += Phi; f->R->cons[BRR] += Phi; }
   }
   for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
      int jk = j + Nr*k;
      for(i = 0; i < D->Np[jk]; i++) {
         int im = i == 0 ? D->Np[jk] - 1 : i - 1;
         pcell *c = &D->ring[jk][i], *cm = &D->ring[jk][im];
         double xp[3] = {D->rj[j], c->piph, D->zk[k]}, xm[3] = {D->rj[j - 1], cm->piph, D->zk[k - 1]};
         double x[3];
         centroid_arr(xp, xm, x);
         double dA = get_dA(xp, xm, 0), dV = get_dV(xp, xm);
         if(type == 0) {
            c->prim[BRR] /= c->tempDoub;
            c->prim[BPP] = .5*(c->Phi[0] + cm->Phi[0])/dA;
         } else {
            double rfac = 1.0/x[0], hr = 1.0, hp = x[0];
            c->cons[BRR] *= dV*rfac/(c->tempDoub*hr);
            c->cons[BPP] = .5*(c->Phi[0] + cm->Phi[0])*dV/(dA*hp);
         }
      }
   }
   if(Nz > 1) {
      for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
         int jk = j + Nr*k;
         for(i = 0; i < D->Np[jk]; i++) D->ring[jk][i].tempDoub = 0.0;
      }
      int Nfz = D->fI[1][D->ntracks[1]];
      for(n = 0; n < Nfz; n++) {
         pface *f = &D->faces[1][n];
         double Phi = f->LRtype == 0 ? f->L->Phi[4] : f->R->Phi[3];
         f->L->tempDoub += f->dA;
         f->R->tempDoub += f->dA;
         if(type == 0) { f->L->prim[BZZ] += Phi; f->R->prim[BZZ] += Phi; }
         else { f->L->cons[BZZ] += Phi; f->R->cons[BZZ] += Phi; }
      }
      for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
         int jk = j + Nr*k;
         for(i = 0; i < D->Np[jk]; i++) {
            int im = i == 0 ? D->Np[jk] - 1 : i - 1;
            pcell *c = &D->ring[jk][i], *cm = &D->ring[jk][im];
            double xp[3] = {D->rj[j], c->piph, D->zk[k]}, xm[3] = {D->rj[j - 1], cm->piph, D->zk[k - 1]};
            double dV = get_dV(xp, xm);
            if(type == 0) c->prim[BZZ] /= c->tempDoub;
            else c->cons[BZZ] *= dV*1.0/(c->tempDoub*1.0);
         }
      }
   }
}

static void initial(double *prim, const double *x);
static void initial_raw(double *prim, const double *x);

static void set_B_fields(void)
{
   int i, j, k, n;
   for(k = 0; k < D->Nz; k++) {
      double z = centroid(D->zk[k], D->zk[k - 1], 2);
      for(j = 0; j < D->Nr; j++) {
         double r = centroid(D->rj[j], D->rj[j - 1], 1);
         int jk = j + D->Nr*k;
         for(i = 0; i < D->Np[jk]; i++) {
            pcell *c = &D->ring[jk][i];
            double phip = c->piph, phim = phip - c->dphi;
            double xp[3] = {D->rj[j], phip, D->zk[k]}, xm[3] = {D->rj[j - 1], phim, D->zk[k - 1]};
            double x[3] = {r, phip, z};
            double prim[MAXQ];
            initial(prim, x);
            c->Phi[0] = prim[BPP]*get_dA(xp, xm, 0);
         }
      }
   }
   build_faces(1);
   for(n = 0; n < D->fI[0][D->ntracks[0]]; n++) {
      pface *f = &D->faces[0][n];
      double prim[MAXQ];
      initial(prim, f->cm);
      double Phi = prim[BRR]*f->dA;
      if(f->LRtype == 0) f->L->Phi[2] = Phi; else f->R->Phi[1] = Phi;
   }
   if(D->Nz > 1) {
      build_faces(2);
      for(n = 0; n < D->fI[1][D->ntracks[1]]; n++) {
         pface *f = &D->faces[1][n];
         double prim[MAXQ];
         initial(prim, f->cm);
         double Phi = prim[BZZ]*f->dA;
         if(f->LRtype == 0) f->L->Phi[4] = Phi; else f->R->Phi[3] = Phi;
      }
   }
   B_faces_to_cells(0);
   B_faces_to_cells(1);
}

static void avg_Efields(void)
{
   int Nr = D->Nr, Nz = D->Nz, j, k, i, n, d;
   for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
      int jk = j + Nr*k;
      for(i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i], *cp = &D->ring[jk][(i + 1)%D->Np[jk]];
         for(int h = 0; h < 2; h++) {
            int a = 4*h;
            double El = .5*(c->E[a + 0] + cp->E[a + 2]), Er = .5*(c->E[a + 1] + cp->E[a + 3]);
            c->E[a + 0] = El; c->E[a + 1] = Er; cp->E[a + 2] = El; cp->E[a + 3] = Er;
            double Bl = .5*(c->B[a + 0] + cp->B[a + 2]), Br = .5*(c->B[a + 1] + cp->B[a + 3]);
            c->B[a + 0] = Bl; c->B[a + 1] = Br; cp->B[a + 2] = Bl; cp->B[a + 3] = Br;
         }
      }
   }
   for(d = 0; d < 2; d++) {
      if(d == 1 && Nz <= 1) break;
      int a = 4*d;
      int Nf = D->fI[d][D->ntracks[d]];
      pface *Fs = D->faces[d];
      for(n = 0; n < Nf; n++) {
         pface *f = &Fs[n];
         pcell *c1 = f->LRtype == 0 ? f->L : f->R, *c2 = f->LRtype == 0 ? f->R : f->L;
         double dp1 = get_dp(c2->piph, c1->piph);
         double dp2 = c2->dphi - dp1;
         if(f->LRtype == 0) {
            double Eavg = (dp2*c2->E[a + 0] + dp1*c2->E[a + 2])/(dp1 + dp2);
            double Bavg = (dp2*c2->B[a + 0] + dp1*c2->B[a + 2])/(dp1 + dp2);
            f->E = .5*(f->L->E[a + 1] + Eavg);
            f->B = .5*(f->L->B[a + 1] + Bavg);
         } else {
            double Eavg = (dp2*c2->E[a + 1] + dp1*c2->E[a + 3])/(dp1 + dp2);
            double Bavg = (dp2*c2->B[a + 1] + dp1*c2->B[a + 3])/(dp1 + dp2);
            f->E = .5*(f->R->E[a + 0] + Eavg);
            f->B = .5*(f->R->B[a + 0] + Bavg);
         }
      }
      for(n = 0; n < Nf; n++) {
         pface *f = &Fs[n];
         if(f->LRtype == 0) { f->L->E[a + 1] = f->E; f->L->B[a + 1] = f->B; }
         else { f->R->E[a + 0] = f->E; f->R->B[a + 0] = f->B; }
         f->E = 0.0; f->B = 0.0;
      }
   }
   for(j = 0; j < Nr; j++) for(k = 0; k < Nz; k++) {
      int jk = j + Nr*k;
      for(i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i], *cp = &D->ring[jk][(i + 1)%D->Np[jk]];
         cp->E[2] = c->E[0]; cp->E[3] = c->E[1]; cp->B[2] = c->B[0]; cp->B[3] = c->B[1];
         cp->E[6] = c->E[4]; cp->E[7] = c->E[5]; cp->B[6] = c->B[4]; cp->B[7] = c->B[5];
      }
   }
}
static void subtract_advective_B_fluxes(void)
{
   for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
      int jk = j + D->Nr*k;
      double xp[3] = {D->rj[j], 0.0, D->zk[k]}, xm[3] = {D->rj[j - 1], 0.0, D->zk[k - 1]};
      double xc[3];
      centroid_arr(xp, xm, xc);
      double hL = xm[0], hR = xp[0], hD = xc[0], hU = xc[0];
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double wm = c->wiph, wp = c->wiph;
         c->E[0] -= hL*wm*c->B[0];
         c->E[1] -= hR*wp*c->B[1];
         c->E[4] += hD*wm*c->B[4];
         c->E[5] += hU*wp*c->B[5];
      }
   }
}
static int phi_switch(double dphi, int mode)
{
   while(dphi > .5*D->Pmax) dphi -= D->Pmax;
   while(dphi < -.5*D->Pmax) dphi += D->Pmax;
   if(mode == 1) dphi = -dphi;
   return dphi > 0. ? 1 : 0;
}
static int get_which4(double phi, double phiR, double phiU, double phiUR, int *LR_alt,
                      int *UD_alt, int mode)
{
   int LR_D = phi_switch(phi - phiR, mode);
   int LR_U = phi_switch(phiU - phiUR, mode);
   double phi1 = LR_D ? phiR : phi, phi2 = LR_U ? phiUR : phiU;
   int UD = phi_switch(phi1 - phi2, mode);
   int w4 = UD == 0 ? (LR_D == 0 ? 0 : 1) : (LR_U == 0 ? 2 : 3);
   if(mode == 0) {
      *LR_alt = (w4 == 0 || w4 == 1) ? LR_U : LR_D;
      if(w4 == 0 || w4 == 2) *UD_alt = phi_switch(phiR - phiUR, mode);
      else *UD_alt = phi_switch(phi - phiU, mode);
   }
   return w4;
}
static void make_edge_adjust(double dt)
{
   int Nr = D->Nr, Nz = D->Nz, i, j, k, jk;
   int *I0 = (int *)malloc(sizeof(int)*Nr*Nz);
   for(jk = 0; jk < Nr*Nz; jk++) {
      int found = 0, quad_prev = 0;
      for(i = 0; i < D->Np[jk] && !found; i++) {
         double convert = 2.*M_PI/D->Pmax;
         double ph = D->ring[jk][i].piph;
         double sn = sin(ph*convert), cs = cos(ph*convert);
         if(sn > 0. && cs > 0. && quad_prev) { found = 1; I0[jk] = i; }
         else if(sn < 0. && cs > 0.) quad_prev = 1;
      }
      if(!found) I0[jk] = 0;
   }
   for(k = 0; k < Nz - 1; k++) for(j = 0; j < Nr - 1; j++) {
      int a = j + Nr*k, b = j + 1 + Nr*k, u = j + Nr*(k + 1), ur = j + 1 + Nr*(k + 1);
      double xp[3] = {D->rj[j], 0.0, D->zk[k]}, xm[3] = {D->rj[j], 0.0, D->zk[k]};
      int i0 = I0[a], iR = I0[b], iU = I0[u], iUR = I0[ur];
      int Ne = D->Np[a] + D->Np[b] + D->Np[u] + D->Np[ur];
      for(int e = 0; e < Ne; e++) {
         pcell *c = &D->ring[a][i0], *cR = &D->ring[b][iR], *cU = &D->ring[u][iU], *cUR = &D->ring[ur][iUR];
         int LR_alt, UD_alt;
         int w4 = get_which4(c->piph, cR->piph, cU->piph, cUR->piph, &LR_alt, &UD_alt, 0);
         int w4b = get_which4(c->piph - c->dphi, cR->piph - cR->dphi, cU->piph - cU->dphi,
                              cUR->piph - cUR->dphi, NULL, NULL, 1);
         double *PhiL, *PhiR, *PhiU, *PhiD, E;
         if(w4 == 0) {
            PhiL = c->Phi + 4; PhiD = c->Phi + 2;
            E = .25*(c->E_phi[3] + c->E_phi[1]);
            if(LR_alt == 0) { PhiU = cU->Phi + 2; E += .25*cU->E_phi[1]; }
            else { PhiU = cUR->Phi + 1; E += .25*cUR->E_phi[0]; }
            if(UD_alt == 0) { PhiR = cR->Phi + 4; E += .25*cR->E_phi[3]; }
            else { PhiR = cUR->Phi + 3; E += .25*cUR->E_phi[2]; }
         } else if(w4 == 1) {
            PhiR = cR->Phi + 4; PhiD = cR->Phi + 1;
            E = .25*(cR->E_phi[3] + cR->E_phi[0]);
            if(LR_alt == 0) { PhiU = cU->Phi + 2; E += .25*cU->E_phi[1]; }
            else { PhiU = cUR->Phi + 1; E += .25*cUR->E_phi[0]; }
            if(UD_alt == 0) { PhiL = c->Phi + 4; E += .25*c->E_phi[3]; }
            else { PhiL = cU->Phi + 3; E += .25*cU->E_phi[2]; }
         } else if(w4 == 2) {
            PhiL = cU->Phi + 3; PhiU = cU->Phi + 2;
            E = .25*(cU->E_phi[2] + cU->E_phi[1]);
            if(LR_alt == 0) { PhiD = c->Phi + 2; E += .25*c->E_phi[1]; }
            else { PhiD = cR->Phi + 1; E += .25*cR->E_phi[0]; }
            if(UD_alt == 0) { PhiR = cR->Phi + 4; E += .25*cR->E_phi[3]; }
            else { PhiR = cUR->Phi + 3; E += .25*cUR->E_phi[2]; }
         } else {
            PhiR = cUR->Phi + 3; PhiU = cUR->Phi + 1;
            E = .25*(cUR->E_phi[2] + cUR->E_phi[0]);
            if(LR_alt == 0) { PhiD = c->Phi + 2; E += .25*c->E_phi[1]; }
            else { PhiD = cR->Phi + 1; E += .25*cR->E_phi[0]; }
            if(UD_alt == 0) { PhiL = c->Phi + 4; E += .25*c->E_phi[3]; }
            else { PhiL = cU->Phi + 3; E += .25*cU->E_phi[2]; }
         }
         pcell *top = w4 == 0 ? c : w4 == 1 ? cR : w4 == 2 ? cU : cUR;
         pcell *bot = w4b == 0 ? c : w4b == 1 ? cR : w4b == 2 ? cU : cUR;
         xp[1] = top->piph;
         xm[1] = bot->piph - bot->dphi;
         double Edldt = E*get_dL(xp, xm, 0)*dt;
         *PhiL -= Edldt; *PhiR += Edldt; *PhiU -= Edldt; *PhiD += Edldt;
         if(w4 == 0) { if(++i0 == D->Np[a]) i0 = 0; }
         else if(w4 == 1) { if(++iR == D->Np[b]) iR = 0; }
         else if(w4 == 2) { if(++iU == D->Np[u]) iU = 0; }
         else { if(++iUR == D->Np[ur]) iUR = 0; }
      }
   }
   free(I0);
}
static void update_B_fluxes_core(double dt);
static void update_B_fluxes(double dt)
{
   update_B_fluxes_core(dt);
   if(D->Nz > 1) make_edge_adjust(dt);
}
static void update_B_fluxes_core(double dt)
{
   for(int d = 0; d < 2; d++) {
      if(d == 1 && D->Nz <= 1) break;
      pface *Fs = D->faces[d];
      int *Nf = D->fI[d];
      int n0 = 0;
      for(int jk = 0; jk < D->ntracks[d]; jk++) {
         int cnt = Nf[jk] - n0;
         for(int n = 0; n < cnt; n++) {
            pface *f = Fs + n0 + n, *fp = Fs + n0 + (n + 1 == cnt ? 0 : n + 1);
            double E, dl = f->dl;
            if(d == 0) {
               if(f->LRtype == 0) { E = f->L->E[1]; f->L->Phi[2] -= E*dl*dt; f->L->Phi[0] += E*dl*dt; }
               else { E = f->R->E[0]; f->R->Phi[1] -= E*dl*dt; f->R->Phi[0] -= E*dl*dt; }
               if(fp->LRtype == 0) fp->L->Phi[2] += E*dl*dt; else fp->R->Phi[1] += E*dl*dt;
            } else {
               if(f->LRtype == 0) { E = f->L->E[5]; f->L->Phi[4] += E*dl*dt; f->L->Phi[0] -= E*dl*dt; }
               else { E = f->R->E[4]; f->R->Phi[3] += E*dl*dt; f->R->Phi[0] += E*dl*dt; }
               if(fp->LRtype == 0) fp->L->Phi[4] -= E*dl*dt; else fp->R->Phi[3] -= E*dl*dt;
            }
         }
         n0 = Nf[jk];
      }
   }
}
static void check_flipped(int d)
{
   pface *Fs = D->faces[d];
   int *fI = D->fI[d], n0 = 0;
   for(int jk = 0; jk < D->ntracks[d]; jk++) {
      int cnt = fI[jk] - n0;
      for(int n = 0; n < cnt; n++) {
         pface *f = Fs + n0 + n, *fp = Fs + n0 + (n + 1 == cnt ? 0 : n + 1);
         double pm = f->LRtype == 0 ? f->L->piph : f->R->piph;
         double pp = fp->LRtype == 0 ? fp->L->piph : fp->R->piph;
         if(get_signed_dp(pp, pm) < 0.) fp->flip_flag = 1;
      }
      n0 = fI[jk];
   }
}
static void phi_ptr(pface *f, double **P, double **RK, int d)
{
   int lo = d == 0 ? 2 : 4, hi = d == 0 ? 1 : 3;
   if(f->LRtype == 0) { *P = &f->L->Phi[lo]; *RK = &f->L->RK_Phi[lo]; }
   else { *P = &f->R->Phi[hi]; *RK = &f->R->RK_Phi[hi]; }
}
static void flip_fluxes(int d)
{
   pface *Fs = D->faces[d];
   int *fI = D->fI[d], n0 = 0;
   for(int jk = 0; jk < D->ntracks[d]; jk++) {
      int cnt = fI[jk] - n0;
      for(int n = 0; n < cnt; n++) {
         pface *f = Fs + n0 + n;
         if(!f->flip_flag) continue;
         pface *fp = Fs + n0 + (n + 1 == cnt ? 0 : n + 1);
         pface *fm = Fs + n0 + (n == 0 ? cnt - 1 : n - 1);
         double *P, *Pm, *Pp, *RP, *RPm, *RPp;
         phi_ptr(f, &P, &RP, d);
         phi_ptr(fm, &Pm, &RPm, d);
         phi_ptr(fp, &Pp, &RPp, d);
         double Phi = *P, RPhi = *RP;
         *P = *Pm + Phi; *RP = *RPm + RPhi;
         *Pm = -Phi; *RPm = -RPhi;
         *Pp = *Pp + Phi; *RPp = *RPp + RPhi;
         f->LRtype = !f->LRtype;
         fm->LRtype = !fm->LRtype;
      }
      n0 = fI[jk];
   }
}

/* ---- cell loops: misc.c ------------------------------------------------------------- */
static void set_wcell(void)
{
   for(int jk = 0; jk < D->Nr*D->Nz; jk++) {
      int Np = D->Np[jk];
      for(int i = 0; i < Np; i++) {
         double w = 0.0;
         if(D->par.Mesh_Motion) w = .5*(D->ring[jk][i].prim[UPP] + D->ring[jk][(i + 1)%Np].prim[UPP]);
         D->ring[jk][i].wiph = w;
      }
      if(D->par.Mesh_Motion == 3) {
         double w = 0.0;
         for(int i = 0; i < Np; i++) w += D->ring[jk][i].wiph;
         w /= (double)Np;
         for(int i = 0; i < Np; i++) D->ring[jk][i].wiph = w;
      }
      if(D->par.Mesh_Motion == 4) {   /* misc.c:153-167: exact mesh rotation */
         int j = jk % D->Nr, k = jk / D->Nr;
         double x[3] = {centroid(D->rj[j], D->rj[j - 1], 1), 0.0, centroid(D->zk[k], D->zk[k - 1], 2)};
         double w = mesh_om(x);
         for(int i = 0; i < Np; i++) D->ring[jk][i].wiph = w;
      }
   }
}
static void calc_dp(void)
{
   for(int jk = 0; jk < D->Nr*D->Nz; jk++) {
      int Np = D->Np[jk];
      for(int i = 0; i < Np; i++)
         D->ring[jk][i].dphi = get_dp(D->ring[jk][i].piph, D->ring[jk][i == 0 ? Np - 1 : i - 1].piph);
   }
}
static void calc_prim(void)
{
   for(int k = D->NgZa; k < D->Nz - D->NgZb; k++) {
      double zm = D->zk[k - 1], zp = D->zk[k], z = centroid(zp, zm, 2);
      for(int j = D->NgRa; j < D->Nr - D->NgRb; j++) {
         int jk = j + D->Nr*k;
         double rm = D->rj[j - 1], rp = D->rj[j], r = centroid(rp, rm, 1);
         for(int i = 0; i < D->Np[jk]; i++) {
            pcell *c = &D->ring[jk][i];
            double phip = c->piph, phim = phip - c->dphi;
            double xp[3] = {rp, phip, zp}, xm[3] = {rm, phim, zm};
            double x[3] = {r, 0.5*(phim + phip), z};
            cons2prim(c->cons, c->prim, x, get_dV(xp, xm));
         }
      }
   }
}
static void initial(double *prim, const double *x)
{
   initial_raw(prim, x);
   if(D->par.RotFrame) prim[UPP] -= D->par.RotOmega;
}
static void initial_raw(double *prim, const double *x)
{
   const disco_params *p = &D->par;
   if(D->mod.initial == DISCO_IC_VORTEX_GAUSS) {
      struct disco_ic_vortex_gauss V = {p->initPar1, p->initPar2, p->initPar3, p->initPar4,
                                        p->initPar5, p->Adiabatic_Index};
      disco_ic_vortex_gauss_eval(&V, prim, x, D->nc, D->nq);
   } else {
      struct disco_ic_disk Dk;
      disco_ic_disk_from_params(&Dk, p->Adiabatic_Index, p->Disk_Mach, p->initPar1, p->initPar2,
                                p->initPar3, p->initPar4, p->initPar5, p->initPar6);
      if(D->mod.initial == DISCO_IC_DISK_MHD) disco_ic_disk_mhd_eval(&Dk, prim, x, D->nc, D->nq);
      else if(D->mod.initial == DISCO_IC_DISK_PLANET) disco_ic_disk_planet_eval(&Dk, prim, x, D->nc, D->nq);
      else disco_ic_disk_cbd_eval(&Dk, prim, x, D->nc, D->nq);
   }
}
/* Boundary/fixed.c:11-46 (r ghosts) and fixed3d.c via set_cell_init. */
/* set_cells_copy_distant (boundary_functions.c:90-158): ring c takes the
 * phi-overlap average of ring c1's primitives. */
static void copy_distant(pcell *c, int Np, const pcell *c1, int Np1)
{
   double Pmax = D->Pmax;
   int i, q, i1;
   for(i = 0; i < Np; i++) for(q = 0; q < D->nq; q++) c[i].prim[q] = 0.0;
   double phi0 = c[0].piph - c[0].dphi;
   for(i1 = 0; i1 < Np1; i1++) {
      double dp = get_signed_dp(c1[i1].piph, phi0);
      if(dp > 0 && dp - c1[i1].dphi <= 0.0) break;
   }
   if(i1 >= Np1) i1 = 0;
   for(i = 0; i < Np; i++) {
      double hi = c[i].piph, lo = c[i].piph - c[i].dphi, hi1, lo1;
      do {
         hi1 = c1[i1].piph; lo1 = c1[i1].piph - c1[i1].dphi;
         while(hi1 < lo) { hi1 += Pmax; lo1 += Pmax; }
         while(lo1 > hi) { hi1 -= Pmax; lo1 -= Pmax; }
         double w = (hi < hi1 ? hi : hi1) - (lo > lo1 ? lo : lo1);
         for(q = 0; q < D->nq; q++) c[i].prim[q] += c1[i1].prim[q]*w;
         i1 = i1 < Np1 - 1 ? i1 + 1 : 0;
      } while(hi1 < hi);
      i1 = i1 > 0 ? i1 - 1 : Np1 - 1;
   }
   for(i = 0; i < Np; i++) for(q = 0; q < D->nq; q++) c[i].prim[q] /= c[i].dphi;
}

/* The per-side primitives of boundary_functions.c.  copy_side covers
 * boundary_zerograd_* (:269-441, the next ring inward, layer by layer
 * outward, with the diode), boundary_reflect_* (:442-621, the mirror ring,
 * normal velocity negated) and boundary_noslip_* (:914-1101, every
 * velocity negated); init_side covers boundary_fixed_* (:161-268,
 * set_cell_init), boundary_fixed_q_* (:662-773, set_cell_init_q) and
 * boundary_fixed_phi_* (:774-913). */
static void copy_ring(int jk, int jk1, int op, int vq, int sign, int diode)
{
   copy_distant(D->ring[jk], D->Np[jk], D->ring[jk1], D->Np[jk1]);
   for(int i = 0; i < D->Np[jk]; i++) {
      double *p = D->ring[jk][i].prim;
      if(op == DISCO_BCOP_ZEROGRAD && diode && sign*p[vq] > 0) p[vq] = 0.0;
      if(op == DISCO_BCOP_REFLECT) p[vq] = -p[vq];
      if(op == DISCO_BCOP_NOSLIP) { p[URR] = -p[URR]; p[UPP] = -p[UPP]; p[UZZ] = -p[UZZ]; }
   }
}

static void copy_side(const disco_bc_op *o)
{
   int j, k, Nr = D->Nr, Nz = D->Nz, zg = o->op == DISCO_BCOP_ZEROGRAD;
   switch(o->side) {
   case DISCO_SIDE_RINN:
      for(k = 0; k < Nz; k++) for(j = D->NgRa - 1; j >= 0; j--)
         copy_ring(j + Nr*k, (zg ? j + 1 : 2*D->NgRa - j - 1) + Nr*k, o->op, URR, 1, o->arg);
      break;
   case DISCO_SIDE_ROUT:
      for(k = 0; k < Nz; k++) for(j = Nr - D->NgRb; j < Nr; j++)
         copy_ring(j + Nr*k, (zg ? j - 1 : 2*(Nr - D->NgRb) - j - 1) + Nr*k, o->op, URR, -1, o->arg);
      break;
   case DISCO_SIDE_ZBOT:
      for(k = D->NgZa - 1; k >= 0; k--) for(j = 0; j < Nr; j++)
         copy_ring(j + Nr*k, j + Nr*(zg ? k + 1 : 2*D->NgZa - k - 1), o->op, UZZ, 1, o->arg);
      break;
   default:
      for(k = Nz - D->NgZb; k < Nz; k++) for(j = 0; j < Nr; j++)
         copy_ring(j + Nr*k, j + Nr*(zg ? k - 1 : 2*(Nz - D->NgZb) - k - 1), o->op, UZZ, -1, o->arg);
      break;
   }
}

static void init_side(const disco_bc_op *o)
{
   int j0, j1, k0, k1;
   if(o->side == DISCO_SIDE_RINN) { j0 = 0; j1 = D->NgRa; k0 = 0; k1 = D->Nz; }
   else if(o->side == DISCO_SIDE_ROUT) { j0 = D->Nr - D->NgRb; j1 = D->Nr; k0 = 0; k1 = D->Nz; }
   else if(o->side == DISCO_SIDE_ZBOT) { j0 = 0; j1 = D->Nr; k0 = 0; k1 = D->NgZa; }
   else { j0 = 0; j1 = D->Nr; k0 = D->Nz - D->NgZb; k1 = D->Nz; }
   for(int k = k0; k < k1; k++) for(int j = j0; j < j1; j++) {
      int jk = j + D->Nr*k;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double xp[3] = {D->rj[j], c->piph, D->zk[k]}, xm[3] = {D->rj[j - 1], c->piph - c->dphi, D->zk[k - 1]};
         double x[3], prim[MAXQ];
         if(o->op == DISCO_BCOP_FIXED_Q) {
            x[0] = centroid(D->rj[j], D->rj[j - 1], 1);
            x[1] = c->piph - 0.5*c->dphi;
            x[2] = centroid(D->zk[k], D->zk[k - 1], 2);
            initial(prim, x);
            for(int q = 0; q < D->nq; q++) if((o->arg >> q) & 1) c->prim[q] = prim[q];
            continue;
         }
         if(o->op == DISCO_BCOP_FIXED_MEAN) {   /* Boundary/horizon.c's fixed sides */
            x[0] = .5*(D->rj[j] + D->rj[j - 1]);
            x[1] = c->piph - .5*c->dphi;
            x[2] = .5*(D->zk[k] + D->zk[k - 1]);
            initial(c->prim, x);
            continue;
         }
         if(o->op == DISCO_BCOP_FIXED_PHI) {
            double phi = c->piph - 0.5*c->dphi;
            while(phi < o->pa) phi += D->Pmax;
            if(!(phi < o->pb)) continue;
         }
         centroid_arr(xp, xm, x);
         initial(c->prim, x);
      }
   }
}

/* exchangeData (exchange.c:173-279) of a run on one rank with a periodic
 * dimension: the cartesian communicator wraps around, so the rank is its
 * own neighbour on both sides, and ghost ring j < Ng (k < Ng) takes the
 * cells of real ring j + Nreal (k + Nreal), ghost ring j >= N - Ng those of
 * j - Nreal: every field of struct cell_lite (exchange.c:6-15). */
static int periodic_dim(int dim)
{
   return dim == 1 ? (D->par.R_Periodic && D->Nr > 1) : (D->par.Z_Periodic && D->Nz > 1);
}
static void exchange(int dim)
{
   if(!periodic_dim(dim)) return;
   int nreal = dim == 1 ? D->Nr - D->NgRa - D->NgRb : D->Nz - D->NgZa - D->NgZb;
   int ga = dim == 1 ? D->NgRa : D->NgZa, gb = dim == 1 ? D->NgRb : D->NgZb;
   int n = dim == 1 ? D->Nr : D->Nz;
   for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
      int a = dim == 1 ? j : k, s;
      if(a < ga) s = a + nreal;
      else if(a >= n - gb) s = a - nreal;
      else continue;
      int src = dim == 1 ? s + D->Nr*k : j + D->Nr*s;
      int jk = j + D->Nr*k;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         const pcell *o = &D->ring[src][i];
         memcpy(c->prim, o->prim, sizeof c->prim);
         memcpy(c->cons, o->cons, sizeof c->cons);
         memcpy(c->RKcons, o->RKcons, sizeof c->RKcons);
         memcpy(c->Phi, o->Phi, sizeof c->Phi);
         memcpy(c->RK_Phi, o->RK_Phi, sizeof c->RK_Phi);
         c->piph = o->piph;
         c->dphi = o->dphi;
         c->wiph = o->wiph;
      }
   }
}

/* onestep.c:166-172: exchangeData(r); boundary_trans(r) unless R_Periodic;
 * exchangeData(z); boundary_trans(z) unless Z_Periodic */
/* boundary_fixed_horizon (boundary_functions.c:622-660): every ring within
 * R_HOR of the origin, ghost or real, back to initial() at the cell
 * centroid (set_cell_init, :21-31), and out of getmindt (real = 0).
 * cut != 0: Boundary/horizon.c's own cut-out (:73-109), initial() at the
 * arithmetic-mean r, z and the cell's mid phi. */
static void horizon_rings(int cut)
{
   for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
      if(cut ? !disco_bc_horizon_cut_ring(D->rj, D->zk, D->Nz, j, k)
             : !disco_bc_horizon_ring(D->rj, D->zk, j, k)) continue;
      int jk = j + D->Nr*k;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double x[3];
         if(cut) {
            x[0] = 0.5*(D->rj[j - 1] + D->rj[j]);
            x[1] = c->piph - .5*c->dphi;
            x[2] = 0.5*(D->zk[k - 1] + D->zk[k]);
         } else {
            double xp[3] = {D->rj[j], c->piph, D->zk[k]}, xm[3] = {D->rj[j - 1], c->piph - c->dphi, D->zk[k - 1]};
            centroid_arr(xp, xm, x);
         }
         initial(c->prim, x);
         c->real = 0;
      }
   }
}

/* Boundary/horizon_bin.c's cut-outs (:79-179): hole 0, then hole 1; on a
 * candidate ring, a cell whose point (rc, mid phi, zc) lies within the hole
 * goes back to initial() at the arithmetic-mean r, z and its mid phi, and
 * out of getmindt for good (real = 0) */
static void hole_cells(void)
{
   for(int h = 0; h < 2; h++)
      for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
         double rc, zc;
         if(!disco_bc_hole_ring(D->rj, D->zk, D->Nr, D->Nz, j, k, h, &rc, &zc)) continue;
         int jk = j + D->Nr*k;
         for(int i = 0; i < D->Np[jk]; i++) {
            pcell *c = &D->ring[jk][i];
            double phi = c->piph - .5*c->dphi;
            if(!disco_bc_hole_cell(rc, zc, D->Nz, phi, h)) continue;
            double x[3] = {0.5*(D->rj[j - 1] + D->rj[j]), phi, 0.5*(D->zk[k - 1] + D->zk[k])};
            initial(c->prim, x);
            c->real = 0;
         }
      }
}

static void boundary(void)
{
   disco_bc_op ops[DISCO_BC_MAX_OPS];
   int n = disco_bc_plugin_ops(D->mod.boundary, ops);
   exchange(1);
   if(n > 0) {   /* the plugin's primitives in call order: r sides, then z sides */
      int zdone = 0;
      for(int o = 0; o < n; o++) {
         int dim = ops[o].side < 2 ? 1 : 2;
         if(dim == 2 && !zdone) { exchange(2); zdone = 1; }
         if((dim == 1 && D->Nr <= 1) || (dim == 2 && D->Nz <= 1)) continue;
         if(periodic_dim(dim)) continue;
         if(ops[o].op == DISCO_BCOP_HORIZON) horizon_rings(ops[o].arg);
         else if(ops[o].op == DISCO_BCOP_HOLES) hole_cells();
         else if(ops[o].op >= DISCO_BCOP_ZEROGRAD && ops[o].op <= DISCO_BCOP_NOSLIP) copy_side(&ops[o]);
         else init_side(&ops[o]);
      }
      if(!zdone) exchange(2);
      return;
   }
   for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
      int rg = j < D->NgRa || j >= D->Nr - D->NgRb;
      int zg = k < D->NgZa || k >= D->Nz - D->NgZb;
      if(periodic_dim(1)) rg = 0;
      if(periodic_dim(2)) zg = 0;
      int jk = j + D->Nr*k;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double x[3];
         if(D->mod.boundary == DISCO_BC_FIXED) {
            if(!rg || D->Nr <= 1) continue;
            x[0] = .5*(D->rj[j] + D->rj[j - 1]);
            x[1] = c->piph - .5*c->dphi;
            x[2] = .5*(D->zk[k] + D->zk[k - 1]);
         } else {
            if(!((rg && D->Nr > 1) || (zg && D->Nz > 1))) continue;
            double xp[3] = {D->rj[j], c->piph, D->zk[k]}, xm[3] = {D->rj[j - 1], c->piph - c->dphi, D->zk[k - 1]};
            centroid_arr(xp, xm, x);
         }
         initial(c->prim, x);
      }
   }
   exchange(2);
}
/* rotframe.c:32-80 (cylindrical: the rpz / orthonormal conversions reduce
 * to the scale factor r on the phi component) */
static void omega_src(const double *prim, double *cons, const double *xp, const double *xm,
                      double dVdt)
{
   double x[3];
   centroid_arr(xp, xm, x);
   double r = x[0], phi = x[1];
   double O = D->par.RotOmega, d = D->par.RotD;
   double rho = prim[RHO];
   double v0 = prim[URR], v1 = prim[UPP]*r, v2 = prim[UZZ];
   double vr = v0, vom = v1/r;
   double Rr = r - d*cos(phi), Rp = d*sin(phi);
   double f0 = O*O*Rr + 2.*O*r*vom;
   double f1 = O*O*Rp - 2.*O*vr;
   double f2 = 0.0;
   v1 -= r*get_om(x);
   double vf = v0*f0 + v1*f1 + v2*f2;
   f1 *= r;
   cons[SRR] += rho*f0*dVdt;
   cons[LLL] += rho*f1*dVdt;
   cons[SZZ] += rho*f2*dVdt;
   cons[TAU] += rho*vf*dVdt;
}
/* cooling (sink.c:274-326) and damping (sink.c:329-427), the first two
 * terms add_source applies (misc.c:579-580). */
static void planetary_force_m1(const disco_planet *pl, double r, double phi, double z,
                               double *fr, double *fp, double *fz);
static void initial_raw(double *prim, const double *x);

static double orbital_rate(const double *x)
{
   double gx = x[0]*cos(x[1]), gy = x[0]*sin(x[1]), omtot = 0.0;
   for(int p = 0; p < D->Npl; p++) {
      double px = D->pl[p].r*cos(D->pl[p].phi), py = D->pl[p].r*sin(D->pl[p].phi);
      double dx = gx - px, dy = gy - py, mag = sqrt(dx*dx + dy*dy), fr, fp, fz;
      planetary_force_m1(&D->pl[p], x[0], x[1], x[2], &fr, &fp, &fz);
      omtot += sqrt(fr*fr + fp*fp + fz*fz)/mag;
   }
   return sqrt(omtot);
}

static void cooling(const double *prim, double *cons, const double *xp, const double *xm, double dV, double dt)
{
   int type = D->par.coolType;
   if(type != 1 && type != 2) return;
   double x[3];
   centroid_arr(xp, xm, x);
   double gm1 = D->gam - 1.0;
   double enTarget = get_cs2(x)/(D->gam*gm1), enCurrent = prim[PPP]/(prim[RHO]*gm1);
   if(type == 2 || enCurrent > enTarget) {
      double Tm1 = expm1(-dt*orbital_rate(x)/D->par.coolPar1);
      cons[TAU] += prim[RHO]*dV*(enCurrent - enTarget)*Tm1;
   }
}

static void damping(const double *prim, double *cons, const double *xp, const double *xm, double dV, double dt)
{
   const disco_params *p = &D->par;
   int t[4] = {p->dampInnerType, p->dampOuterType, p->dampUpperType, p->dampLowerType};
   if(t[0] + t[1] + t[2] + t[3] <= 0) return;
   double x[3];
   centroid_arr(xp, xm, x);
   /* the last active side's factor is the one applied (ratetot, which the
    * damping times enter, is unused in the reference) */
   double f = 0.0, th;
   if(t[0] > 0) { th = (x[0] - p->rmin)/p->dampLenInner; f = th > 1.0 ? 0.0 : 1.0 - pow(1.0 - pow(th, 2.0), 2.0); }
   if(t[1] > 0) { th = (p->rmax - x[0])/p->dampLenOuter; f = th > 1.0 ? 0.0 : pow(1.0 - pow(th, 2.0), 2.0); }
   if(D->Nz > 1) {
      if(t[2] > 0) { th = (p->zmax - x[2])/p->dampLenUpper; f = th > 1.0 ? 0.0 : pow(1.0 - pow(th, 2.0), 2.0); }
      if(t[3] > 0) { th = (p->zmax - x[2])/p->dampLenLower; f = th > 1.0 ? 0.0 : 1.0 - pow(1.0 - pow(th, 2.0), 2.0); }
   }
   f = expm1(-dt*f);
   double p0[MAXQ], c0[MAXQ], c1[MAXQ];
   initial_raw(p0, x);
   prim2cons(p0, c0, x, dV);
   prim2cons(prim, c1, x, dV);
   cons[DDD] += (c1[DDD] - c0[DDD])*f;
   cons[SRR] += (c1[SRR] - c0[SRR])*f;
   cons[LLL] += (c1[LLL] - c0[LLL])*f;
   cons[SZZ] += (c1[SZZ] - c0[SZZ])*f;
   cons[TAU] += (c1[TAU] - c0[TAU])*f;
}

/* sink_src (sink.c:105-247): the nozzle, then the accreting sinks of the
 * first Sink_Number bodies (all if 0 or not fewer than Npl), accumulating
 * into the bodies' sink accumulators in cell order as the reference does.
 * A cell outside the nozzle returns before the sinks, as in the reference;
 * delta is fmax(0, Sink_Par2), the reference's fmin being overwritten. */
static void sink_src(const double *prim, double *cons, const double *xp, const double *xm, double dV, double dt)
{
   const disco_params *p = &D->par;
   if(p->nozzleType == 1) {
      double R0 = p->nozzlePar1, dR = p->nozzlePar2, v = p->nozzlePar3, mach = p->nozzlePar4;
      double r = 0.5*(xp[0] + xm[0]), phi = 0.5*(xp[1] + xm[1]), z = 0.5*(xp[2] + xm[2]);
      if(phi > M_PI) phi -= 2*M_PI;
      if((r - R0)*(r - R0) + r*r*phi*phi + z*z > dR*dR) return;
      double rhodot = 1.0*3.0/(4.0*M_PI*dR*dR*dR);
      if(D->Nz == 1) rhodot *= 2*sqrt(dR*dR - (r - R0)*(r - R0) - r*r*phi*phi);
      if(rhodot*dV*dt > cons[RHO]) rhodot = cons[RHO]/dV*dt;
      double x[3] = {r, phi, z};
      double om = get_om(x);
      double cs2 = v*v/(mach*mach);
      double eps = cs2/(D->gam*(D->gam - 1));
      cons[RHO] += rhodot*dV*dt;
      cons[LLL] += rhodot*r*v*dV*dt;
      cons[TAU] += (0.5*rhodot*(v - r*om)*(v - r*om) + rhodot*eps)*dV*dt;
      if(D->nq > D->nc) cons[D->nc] += rhodot*dV*dt;
   }
   if(p->sinkType == 0) return;
   double x[3];
   centroid_arr(xp, xm, x);
   double r = x[0], phi = x[1];
   double rho = prim[RHO], vr = prim[URR], vp = prim[UPP]*r, vz = prim[UZZ];
   double cosg = cos(phi), sing = sin(phi), gx = r*cosg, gy = r*sing;
   int ns = D->Npl;
   if(p->sinkNumber > 0 && p->sinkNumber < ns) ns = p->sinkNumber;
   for(int b = 0; b < ns; b++) {
      const disco_planet *q = &D->pl[b];
      double *a = D->sacc[b];
      double cosp = cos(q->phi), sinp = sin(q->phi);
      double dx = gx - q->r*cosp, dy = gy - q->r*sinp;
      double mag = sqrt(dx*dx + dy*dy);
      double arg = 0.0;
      if(p->sinkType == 3) {
         if(mag <= p->sinkPar3) arg = 1.0;
      } else if(p->sinkType == 2) {
         double eps = pow(p->sinkPar3, p->sinkPar4);
         double ef = p->sinkPar5 <= 0.0 ? 1.0 : p->sinkPar5;
         arg = exp(-pow(mag, p->sinkPar4)/(eps*ef));
      } else if(p->sinkType == 1) {
         arg = pow(1.0 - pow(mag/p->sinkPar3, p->sinkPar4), p->sinkPar5);
         if(mag >= p->sinkPar3) arg = 0.0;
      }
      double surfdiff = rho*(p->sinkPar1*q->omega)*arg;
      double delta = fmax(0.0, p->sinkPar2);
      double vpp = q->r*q->omega;
      double vxp = q->vr*cosp - vpp*sinp, vyp = q->vr*sinp + vpp*cosp;
      double vxg = vr*cosg - vp*sing, vyg = vr*sing + vp*cosg;
      double vxr = vxg - vxp, vyr = vyg - vyp;
      double cphi = dx/mag, sphi = dy/mag;
      double af = dV*dt*surfdiff;
      double vpr = cphi*vyr - sphi*vxr;
      a[3] += (1.0 - delta)*mag*vpr*af;
      double vxn = (cphi*cphi + (1.0 - delta)*sphi*sphi)*vxr + delta*sphi*cphi*vyr;
      double vyn = delta*cphi*sphi*vxr + (sphi*sphi + (1.0 - delta)*cphi*cphi)*vyr;
      vxg = vxn + vxp;
      vyg = vyn + vyp;
      double vgr = vxg*cosg + vyg*sing, vgp = -vxg*sing + vyg*cosg;
      a[2] += vgp*r*af;
      cons[DDD] -= af;
      if(delta == 0.0) { vgr = vr; vgp = vp; }
      cons[SRR] -= vgr*af;
      cons[LLL] -= r*vgp*af;
      cons[SZZ] -= vz*af;
      double v2 = vgp*vgp + vgr*vgr + vz*vz;
      cons[TAU] -= af*(0.5*v2 + prim[PPP]/(rho*(D->gam - 1.0)));
      a[1] += af;
      a[4] += 0.5*v2*af;
      a[5] += prim[PPP]*af/(rho*(D->gam - 1.0));
      a[6] += af*vxg;
      a[7] += af*vyg;
      double fr, fp, fz;
      double rho0 = 1.0/(3.0*M_PI*p->viscosity);
      planetary_force_m1(q, r, phi, 0.0, &fr, &fp, &fz);
      a[0] -= (rho - rho0)*q->r*fp*dV*dt;
   }
}

static void add_source(double dt)
{
   for(int k = D->NgZa; k < D->Nz - D->NgZb; k++) for(int j = D->NgRa; j < D->Nr - D->NgRb; j++) {
      int jk = j + D->Nr*k;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double phip = c->piph, phim = c->piph - c->dphi;
         double xp[3] = {D->rj[j], phip, D->zk[k]}, xm[3] = {D->rj[j - 1], phim, D->zk[k - 1]};
         double dV = get_dV(xp, xm);
         cooling(c->prim, c->cons, xp, xm, dV, dt);
         damping(c->prim, c->cons, xp, xm, dV, dt);
         if(D->mhd) m_source(c->prim, c->cons, xp, xm, dV*dt);
         else e_source(c->prim, c->cons, xp, xm, dV*dt);
         for(int p = 0; p < D->Npl; p++) planet_src(&D->pl[p], c->prim, c->cons, xp, xm, dV*dt);
         if(D->par.visc_flag && !D->mhd)
            e_visc_source(c->prim, c->gradr, c->gradp, c->gradz, c->cons, xp, xm, dV*dt);
         if(D->par.RotFrame) omega_src(c->prim, c->cons, xp, xm, dV*dt);
         if(D->par.sinkType || D->par.nozzleType) sink_src(c->prim, c->cons, xp, xm, dV, dt);
      }
   }
}

static void onestep(double RK, double dt, int first)
{
   long c;
   int q;
   if(first) set_wcell();
   for(c = 0; c < D->N; c++) {
      pcell *x = &D->cells[c];
      for(q = 0; q < D->nq; q++) x->cons[q] = (1. - RK)*x->cons[q] + RK*x->RKcons[q];
      if(D->mhd) for(q = 0; q < 5; q++) x->Phi[q] = (1. - RK)*x->Phi[q] + RK*x->RK_Phi[q];
   }
   for(int p = 0; p < D->Npl; p++)   /* adjust_RK_planets_aux, misc.c:258-264 */
      for(q = 0; q < 8; q++) D->sacc[p][q] = (1. - RK)*D->sacc[p][q] + RK*D->sacc_rk[p][q];
   plm_phi();
   if(D->Nr > 1) { build_faces(1); plm_trans(1); }
   if(D->Nz > 1) { build_faces(2); plm_trans(2); }
   phi_flux(dt);
   if(D->Nr > 1) trans_flux(dt, 1);
   if(D->Nz > 1) trans_flux(dt, 2);
   if(D->mhd) { avg_Efields(); subtract_advective_B_fluxes(); update_B_fluxes(dt); }
   add_source(dt);
   if(first) {
      for(c = 0; c < D->N; c++) D->cells[c].piph += D->cells[c].wiph*dt;
      /* movePlanets (Planets/circular.c:44-46) for the analytic orbit */
      if(D->mod.planets == DISCO_PL_CIRCULAR && D->Npl > 1) D->pl[1].phi += D->pl[1].omega*dt;
      if(D->mod.planets == DISCO_PL_CM && D->Npl > 1) {   /* Planets/cm.c:53-59 */
         D->pl[0].phi += D->pl[0].omega*dt;
         D->pl[1].phi += D->pl[1].omega*dt;
         double eps = 0.5/D->par.Disk_Mach + exp(-D->t/30.);
         D->pl[0].eps = eps;
         D->pl[1].eps = eps;
      }
      if(D->mhd) {
         check_flipped(0); flip_fluxes(0);
         if(D->Nz > 1) { check_flipped(1); flip_fluxes(1); }
      }
   }
   for(c = 0; c < D->N; c++) {
      double phi = D->cells[c].piph;
      while(phi > D->Pmax) phi -= D->Pmax;
      while(phi < 0.0) phi += D->Pmax;
      D->cells[c].piph = phi;
   }
   for(int p = 0; p < D->Npl; p++) {   /* clean_pi on planets, misc.c:27-34 */
      double phi = D->pl[p].phi;
      while(phi > D->Pmax) phi -= D->Pmax;
      while(phi < 0.0) phi += D->Pmax;
      D->pl[p].phi = phi;
   }
   calc_dp();
   if(D->mhd && D->ct) B_faces_to_cells(1);
   calc_prim();
   boundary();
}

static double getmindt(void)
{
   double dt = D->par.maxDT/D->par.CFL;
   if(dt <= 0.0) dt = 1.0e100;
   for(int k = D->NgZa; k < D->Nz - D->NgZb; k++) for(int j = D->NgRa; j < D->Nr - D->NgRb; j++) {
      int jk = j + D->Nr*k, Np = D->Np[jk];
      for(int i = 0; i < Np; i++) {
         pcell *c = &D->ring[jk][i];
         if(!c->real) continue;
         double phip = c->piph, phim = phip - c->dphi;
         double xp[3] = {D->rj[j], phip, D->zk[k]}, xm[3] = {D->rj[j - 1], phim, D->zk[k - 1]};
         double w = .5*(D->ring[jk][i == 0 ? Np - 1 : i - 1].wiph + c->wiph);
         double t = mindt(c->prim, w, xp, xm);
         if(dt > t) dt = t;
      }
   }
   return dt*D->par.CFL;
}

/* ---- public checker API --------------------------------------------------------- */
port_domain *disco_port_create(const disco_host_domain *h)
{
   port_domain *d = (port_domain *)calloc(1, sizeof(*d));
   D = d;
   d->par = h->par; d->mod = h->mod;
   d->Nr = h->Nr; d->Nz = h->Nz; d->NgRa = h->NgRa; d->NgRb = h->NgRb;
   d->NgZa = h->NgZa; d->NgZb = h->NgZb; d->nq = h->num_q; d->nc = h->mod.num_c;
   d->mhd = h->mod.hydro == DISCO_HYDRO_MHD;
   d->ct = d->mhd && h->mod.ct_mode == 2 && h->par.CT;
   if(d->mhd && (!d->ct || (h->par.Riemann_Solver != 0 && h->par.Riemann_Solver != 1 &&
                             h->par.Riemann_Solver != 2) || h->NgRa == 0 || h->NgRb == 0 ||
                 h->NgZa == 0 || h->NgZb == 0)) { free(d); return NULL; }
   disco_bc_op bops[DISCO_BC_MAX_OPS];
   if(disco_bc_plugin_ops(h->mod.boundary, bops) < 0) { free(d); return NULL; }
   if(h->par.Timestep != 0 && h->par.Timestep != 3) { free(d); return NULL; }
   if(h->par.sinkType < 0 || h->par.sinkType > 3 || (h->par.nozzleType != 0 && h->par.nozzleType != 1)) {
      free(d);
      return NULL;
   }
   if(h->mod.hydro == DISCO_HYDRO_GRMHD ||
      (h->mod.analysis == DISCO_DIAG_MHDMRI && !d->mhd) || h->mod.analysis > DISCO_DIAG_MHDMRI) {
      free(d); return NULL;
   }
   static const int ndiag[] = {8, 5, 6, 5, 18};
   d->nd = h->mod.analysis >= 0 ? ndiag[h->mod.analysis] : 0;
   d->Qrz = (double *)calloc((size_t)h->Nr*h->Nz*(d->nd ? d->nd : 1), sizeof(double));
   d->N = h->Ncell; d->Pmax = h->phi_max; d->t = h->t; d->Npl = h->Npl;
   d->gam = h->par.Adiabatic_Index;
   memcpy(d->pl, h->planets, sizeof d->pl);
   int R = d->Nr*d->Nz;
   d->Np = (int *)malloc(sizeof(int)*R); memcpy(d->Np, h->Np, sizeof(int)*R);
   d->off = (long *)malloc(sizeof(long)*(R + 1)); memcpy(d->off, h->ring_off, sizeof(long)*(R + 1));
   double *rj = (double *)malloc(sizeof(double)*(d->Nr + 1));
   double *zk = (double *)malloc(sizeof(double)*(d->Nz + 1));
   memcpy(rj, h->r_jph, sizeof(double)*(d->Nr + 1));
   memcpy(zk, h->z_kph, sizeof(double)*(d->Nz + 1));
   d->rj = rj + 1; d->zk = zk + 1;
   d->cells = (pcell *)calloc(d->N, sizeof(pcell));
   d->ring = (pcell **)malloc(sizeof(pcell *)*R);
   for(int jk = 0; jk < R; jk++) d->ring[jk] = d->cells + d->off[jk];
   d->fI[0] = (int *)malloc(sizeof(int)*((d->Nr - 1)*d->Nz + 2));
   d->fI[1] = (int *)malloc(sizeof(int)*(d->Nr*(d->Nz > 1 ? d->Nz - 1 : 0) + 2));
   long c;
   for(c = 0; c < d->N; c++) { d->cells[c].piph = h->piph[c]; d->cells[c].dphi = h->dphi[c]; }
   /* setupCells (domain.c:283-385) */
   int j, k, i, q;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) {
      double z = centroid(d->zk[k], d->zk[k - 1], 2);
      for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
         double r = centroid(d->rj[j], d->rj[j - 1], 1);
         int jk = j + d->Nr*k;
         for(i = 0; i < d->Np[jk]; i++) {
            pcell *x = &d->ring[jk][i];
            double phip = x->piph, phim = phip - x->dphi;
            double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
            double X[3] = {r, x->piph - .5*x->dphi, z};
            for(q = 0; q < d->nq; q++) x->prim[q] = h->prim[(size_t)q*d->N + (x - d->cells)];
            prim2cons(x->prim, x->cons, X, get_dV(xp, xm));
            x->real = 1;
         }
      }
   }
   if(d->ct) set_B_fields();
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) {
      double z = centroid(d->zk[k], d->zk[k - 1], 2);
      for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
         double r = centroid(d->rj[j], d->rj[j - 1], 1);
         int jk = j + d->Nr*k;
         for(i = 0; i < d->Np[jk]; i++) {
            pcell *x = &d->ring[jk][i];
            double phip = x->piph, phim = phip - x->dphi;
            double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
            double X[3] = {r, x->piph - .5*x->dphi, z};
            cons2prim(x->cons, x->prim, X, get_dV(xp, xm));
         }
      }
   }
   set_wcell();
   boundary();
   return d;
}

static void add_diagnostics(double dt);

/* timestep.c:7-54 (Timestep 0), preceded by getmindt (main.c:70). */
double disco_port_step(port_domain *d)
{
   D = d;
   double dt = getmindt();
   for(long c = 0; c < d->N; c++) {
      memcpy(d->cells[c].RKcons, d->cells[c].cons, sizeof(double)*MAXQ);
      memcpy(d->cells[c].RK_Phi, d->cells[c].Phi, sizeof(double)*5);
   }
   memcpy(d->sacc_rk, d->sacc, sizeof d->sacc);   /* planet_RK_copy, timestep.c:25-27 */
   if(d->par.Timestep == 3) {   /* timestep.c:35-42 */
      onestep(0.0, dt, 1);
      d->t += dt;
      onestep(0.75, 0.25*dt, 0);
      d->t -= dt*0.5;
      onestep(1./3., 2.*dt/3., 0);
      d->t += dt*0.5;
   } else {
      onestep(0.0, dt, 1);
      d->t += dt;
      onestep(0.5, 0.5*dt, 0);
   }
   add_diagnostics(dt);
   return dt;
}

/* The sink accumulators of the first nbody bodies, out[8 b + k]. */
void disco_port_sink_accum(const port_domain *d, double *out, int nbody)
{
   for(int b = 0; b < nbody && b < d->Npl; b++)
      for(int k = 0; k < 8; k++) out[8*b + k] = d->sacc[b][k];
}

int disco_port_run(port_domain *d, int nsteps)
{
   for(int s = 0; s < nsteps; s++) disco_port_step(d);
   return 0;
}

/* SoA download, same layout as disco_gpu_download; Phi may be NULL. */
void disco_port_state(const port_domain *d, double *piph, double *dphi, double *prim,
                      double *cons, double *t)
{
   long N = d->N, c;
   for(c = 0; c < N; c++) {
      const pcell *x = &d->cells[c];
      if(piph) piph[c] = x->piph;
      if(dphi) dphi[c] = x->dphi;
      for(int q = 0; q < d->nq; q++) {
         if(prim) prim[(size_t)q*N + c] = x->prim[q];
         if(cons) cons[(size_t)q*N + c] = x->cons[q];
      }
   }
   if(t) *t = d->t;
}

void disco_port_phi(const port_domain *d, double *Phi)
/* per-cell face fluxes Phi[0..4], SoA [5*N] */
{
   for(long c = 0; c < d->N; c++)
      for(int q = 0; q < 5; q++) Phi[(size_t)q*d->N + c] = d->cells[c].Phi[q];
}

/* report.c:4-329: the domain sums of one report line, in the reference's
 * (j, k, i) loop order -- out = {t, q, Mass, Torque, Torque2,
 * Torque1_cut[0], Torque2_cut[0], ..., Torque1_cut[4], Torque2_cut[4]}.
 * planetaryForce's mode 1 takes the components along the planet's
 * direction (planet.c:158-161). */
static void planetary_force_m1(const disco_planet *pl, double r, double phi, double z,
                               double *fr, double *fp, double *fz)
{
   double rp = pl->r, pp = pl->phi;
   if(D->par.grav2D == 1) z = 0.0;
   else if(D->par.grav2D == 2) { rp = r; pp = phi; z = 1.0; }
   double cosp = cos(phi), sinp = sin(phi);
   double dx = r*cosp - rp*cos(pp);
   double dy = r*sinp - rp*sin(pp);
   double script_r = sqrt(dx*dx + dy*dy + z*z);
   double script_r_perp = sqrt(dx*dx + dy*dy);
   double f1 = -fgrav(pl->M, script_r, pl->eps);
   double cosa = dx/script_r_perp, sina = dy/script_r_perp;
   double cosap = cosa*cos(pp) + sina*sin(pp);
   double sinap = sina*cos(pp) - cosa*sin(pp);
   if(script_r_perp <= 0.0) { cosap = 0.0; sinap = 0.0; }
   double sint = script_r_perp/script_r, cost = z/script_r;
   *fr = cosap*f1*sint;
   *fp = sinap*f1*sint;
   *fz = f1*cost;
}

void disco_port_report(port_domain *d, double *out)
{
   D = d;
   double Mass = 0.0, Torque = 0.0, Torque2 = 0.0, T1c[5] = {0}, T2c[5] = {0};
   double soft = d->par.sinkPar3;
   for(int j = d->NgRa; j < d->Nr - d->NgRb; j++)
      for(int k = d->NgZa; k < d->Nz - d->NgZb; k++) {
         int jk = j + d->Nr*k;
         for(int i = 0; i < d->Np[jk]; i++) {
            pcell *c = &d->ring[jk][i];
            double phi = c->piph - .5*c->dphi;
            double rho = c->prim[RHO];
            double phip = c->piph, phim = phip - c->dphi;
            double xp[3] = {d->rj[j], phip, d->zk[k]};
            double xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
            double dV = get_dV(xp, xm);
            double r = centroid(xp[0], xm[0], 1);
            Mass += rho*dV;
            if(d->Npl > 1) {
               double fr, fp, fz, fp2;
               planetary_force_m1(&d->pl[0], r, phi, 0.0, &fr, &fp2, &fz);
               planetary_force_m1(&d->pl[1], r, phi, 0.0, &fr, &fp, &fz);
               double rS = d->pl[0].r, rp = d->pl[1].r, pp = d->pl[1].phi;
               double dx = r*cos(phi) - rp*cos(pp);
               double dy = r*sin(phi) - rp*sin(pp);
               double script_r = sqrt(dx*dx + dy*dy);
               double t1v = (rho - 1.0)*rp*fp*dV;
               double t2v = (rho - 1.0)*rS*fp2*dV;
               Torque -= t1v;
               Torque2 -= t2v;
               for(int n = 0; n < 5; n++) {
                  double r_cut = (double)(n + 1.)*soft;
                  if(script_r > r_cut) { T1c[n] -= t1v; T2c[n] -= t2v; }
               }
            }
         }
      }
   out[0] = d->t;
   out[1] = d->Npl > 1 ? d->pl[1].M/d->pl[0].M : 0.0;
   out[2] = Mass; out[3] = Torque; out[4] = Torque2;
   for(int n = 0; n < 5; n++) { out[5 + 2*n] = T1c[n]; out[6 + 2*n] = T2c[n]; }
}

/* get_diagnostics of the ANALYSIS plugins (Diagnostics/diag_euler.c:18-44,
 * diag_disk2d.c:18-41, diag_cb.c:18-62, diag_bl.c:17-36,
 * diag_mhdmri.c:17-62) at the cell centroid x. */
static void get_diagnostics(const double *x, const double *prim, double *Q)
{
   double r = x[0], phi = x[1], z = x[2];
   double rho = prim[RHO], Pp = prim[PPP], vr = prim[URR], om = prim[UPP], vz = prim[UZZ];
   double Fr, Fp = 0.0, Fz;
   switch(D->mod.analysis) {
   case DISCO_DIAG_EULER:
      if(D->Npl > 1) planetary_force(&D->pl[1], r, phi, z, &Fr, &Fp, &Fz);
      Q[0] = rho;
      Q[1] = 2.*M_PI*r*rho*vr;
      Q[2] = 2.*M_PI*r*rho*vz;
      Q[3] = 2.*M_PI*r*rho*(r*Fp);
      Q[4] = 2.*M_PI*r*rho*(r*r*om*vr);
      Q[5] = om;
      Q[6] = 2.*M_PI*r*rho*r*r*om;
      Q[7] = Pp;
      break;
   case DISCO_DIAG_DISK2D:
      if(D->Npl > 1) planetary_force(&D->pl[1], r, phi, 0.0, &Fr, &Fp, &Fz);
      Q[0] = rho;
      Q[1] = 2.*M_PI*r*rho*vr;
      Q[2] = 2.*M_PI*r*rho*(r*Fp);
      Q[3] = 2.*M_PI*r*rho*(r*r*om*vr);
      Q[4] = om;
      break;
   case DISCO_DIAG_CB: {
      double vp = r*om;
      double gx = r*cos(phi), gy = r*sin(phi);
      double vx = vr*cos(phi) - vp*sin(phi), vy = vr*sin(phi) + vp*cos(phi);
      double vm2 = vx*vx + vy*vy, rdv = vx*gx + vy*gy;
      Q[0] = rho;
      Q[1] = 2.*M_PI*r*rho*vr;
      Q[2] = ((vm2 - 1./r)*gx - rdv*vx)*rho;
      Q[3] = ((vm2 - 1./r)*gy - rdv*vy)*rho;
      Q[4] = 0.0;
      Q[5] = rho*vp;
      for(int p = 0; p < 2 && p < D->Npl; p++) {
         planetary_force_m1(&D->pl[p], r, phi, z, &Fr, &Fp, &Fz);
         Q[4] += rho*D->pl[p].r*Fp;
      }
      break;
   }
   case DISCO_DIAG_BL: {
      double vp = r*om;
      Q[0] = rho; Q[1] = rho*om; Q[2] = rho*vp; Q[3] = rho*vr; Q[4] = rho*vp*vr;
      break;
   }
   case DISCO_DIAG_MHDMRI: {
      double g = D->par.Adiabatic_Index;
      double Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
      double cs2 = g*Pp/rho, B2 = Br*Br + Bp*Bp + Bz*Bz;
      Q[0] = rho; Q[1] = Pp; Q[2] = vr; Q[3] = om; Q[4] = vz;
      Q[5] = Br; Q[6] = Bp; Q[7] = Bz; Q[8] = rho;
      Q[9] = 0.5*rho*(vr*vr + r*r*om*om + vz*vz) + Pp/(g - 1.0) + 0.5*B2;
      Q[10] = rho*vr; Q[11] = r*r*rho*om; Q[12] = rho*vz;
      Q[13] = rho*vr*om; Q[14] = Br*Bp; Q[15] = B2;
      Q[16] = sqrt(cs2); Q[17] = sqrt(B2/rho);
      break;
   }
   default: break;
   }
}

/* add_diagnostics (analysis.c:52-108): per ring, every ghost ring included,
 * Qrz += (sum of Q dV) * dt / (sum of dV); t_avg += dt. */
static void add_diagnostics(double dt)
{
   int nd = D->nd;
   if(!nd) return;
   double Q[18];
   for(int k = 0; k < D->Nz; k++) for(int j = 0; j < D->Nr; j++) {
      int jk = k*D->Nr + j;
      double sum[18] = {0}, vol = 0.0;
      for(int i = 0; i < D->Np[jk]; i++) {
         pcell *c = &D->ring[jk][i];
         double xp[3] = {D->rj[j], c->piph, D->zk[k]};
         double xm[3] = {D->rj[j - 1], c->piph - c->dphi, D->zk[k - 1]};
         double xc[3];
         centroid_arr(xp, xm, xc);
         double dV = get_dV(xp, xm);
         get_diagnostics(xc, c->prim, Q);
         for(int q = 0; q < nd; q++) sum[q] += Q[q]*dV;
         vol += dV;
      }
      for(int q = 0; q < nd; q++) D->Qrz[(size_t)jk*nd + q] += sum[q]*dt/vol;
   }
   D->t_avg += dt;
}

/* Qrz [Nr*Nz*nd] (may be NULL) and t_avg; returns nd. */
int disco_port_diag(const port_domain *d, double *Qrz, double *t_avg)
{
   if(Qrz && d->nd) memcpy(Qrz, d->Qrz, sizeof(double)*(size_t)d->Nr*d->Nz*d->nd);
   if(t_avg) *t_avg = d->t_avg;
   return d->nd;
}

long disco_port_num_real(const port_domain *d)
{
   long n = 0;
   for(int k = d->NgZa; k < d->Nz - d->NgZb; k++)
      for(int j = d->NgRa; j < d->Nr - d->NgRb; j++) n += d->Np[j + d->Nr*k];
   return n;
}

void disco_port_free(port_domain *d)
{
   if(!d) return;
   free(d->Np); free(d->off); free(d->rj - 1); free(d->zk - 1);
   free(d->cells); free(d->ring);
   free(d->faces[0]); free(d->faces[1]); free(d->fI[0]); free(d->fI[1]);
   free(d->Qrz);
   free(d);
}

/* The face tables of dimension dim built from the current positions
 * (faces_alt.c:36-179), in the layout of disco_gpu_debug_faces: fIndex
 * [ntracks + 1], per face L and R as global cell ids, LRtype, cm[1] and dA.
 * Returns the number of faces (arrays may be NULL to size them). */
long disco_port_faces(port_domain *d, int dim, int *fIndex, int *L, int *R, int *LRtype,
                      double *phic, double *dA)
{
   D = d;
   if((dim == 1 && d->Nr <= 1) || (dim == 2 && d->Nz <= 1)) return 0;
   build_faces(dim);
   int d0 = dim - 1, nt = d->ntracks[d0];
   long nf = d->fI[d0][nt];
   if(fIndex) for(int t = 0; t <= nt; t++) fIndex[t] = d->fI[d0][t];
   for(long n = 0; n < nf; n++) {
      const pface *f = &d->faces[d0][n];
      if(L) L[n] = (int)(f->L - d->cells);
      if(R) R[n] = (int)(f->R - d->cells);
      if(LRtype) LRtype[n] = f->LRtype;
      if(phic) phic[n] = f->cm[1];
      if(dA) dA[n] = f->dA;
   }
   return nf;
}

/* plm_phi, then the faces and plm_trans of each dimension (onestep.c:104-130)
 * on the current state; gradp, gradr, gradz as SoA [nq*N] (NULL to skip). */
void disco_port_grad(port_domain *d, double *gradp, double *gradr, double *gradz)
{
   D = d;
   plm_phi();
   if(d->Nr > 1) { build_faces(1); plm_trans(1); }
   if(d->Nz > 1) { build_faces(2); plm_trans(2); }
   for(long c = 0; c < d->N; c++)
      for(int q = 0; q < d->nq; q++) {
         if(gradp) gradp[(size_t)q*d->N + c] = d->cells[c].gradp[q];
         if(gradr) gradr[(size_t)q*d->N + c] = d->cells[c].gradr[q];
         if(gradz) gradz[(size_t)q*d->N + c] = d->cells[c].gradz[q];
      }
}

/* Stage dumps of the CT chain of the first substep (see disco_gpu_debug_ct). */
int disco_port_debug_ct(port_domain *d, int stage, double *E, double *B, double *Ephi, double *Phi)
{
   D = d;
   double dt = getmindt();
   for(long c = 0; c < d->N; c++) {
      memcpy(d->cells[c].RKcons, d->cells[c].cons, sizeof(double)*MAXQ);
      memcpy(d->cells[c].RK_Phi, d->cells[c].Phi, sizeof(double)*5);
   }
   set_wcell();
   plm_phi();
   if(d->Nr > 1) { build_faces(1); plm_trans(1); }
   if(d->Nz > 1) { build_faces(2); plm_trans(2); }
   phi_flux(dt);
   if(stage >= 1 && d->Nr > 1) trans_flux(dt, 1);
   if(stage >= 1 && d->Nz > 1) trans_flux(dt, 2);
   if(stage >= 2) { avg_Efields(); subtract_advective_B_fluxes(); }
   if(stage >= 3) update_B_fluxes_core(dt);
   if(stage >= 4 && d->Nz > 1) make_edge_adjust(dt);
   long N = d->N;
   for(long c = 0; c < N; c++) {
      pcell *x = &d->cells[c];
      for(int q = 0; q < 8; q++) { if(E) E[q*N + c] = x->E[q]; if(B) B[q*N + c] = x->B[q]; }
      for(int q = 0; q < 4; q++) if(Ephi) Ephi[q*N + c] = x->E_phi[q];
      for(int q = 0; q < 5; q++) if(Phi) Phi[q*N + c] = x->Phi[q];
   }
   return 0;
}
