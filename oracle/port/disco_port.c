/*
 * CHECKER INFRASTRUCTURE (oracle) -- not product code.
 *
 * Plain-C restatement of the reference's RK substep cycle (timestep.c:7 ->
 * onestep.c:86) for the Newtonian hydro module (Hydro/euler.c), run serially
 * on the CPU over the same ring layout.  It follows the reference loop by
 * loop -- sequential face walk (faces_alt.c:36-179), scatter updates in face
 * order (riemann.c:314-317), limiter (plm.c:146-179) -- so that compiled
 * with gcc it reproduces the reference's numbers.  It is pinned against the
 * reference binary (oracle/ref) by tests/test_oracle_port.py, and used
 *   - as the checker of the GPU path at sizes beyond the golden fixtures,
 *   - as the timed CPU baseline ("port") in bench.py.
 *
 * Input: the host-set-up domain (grid, ring phases, initial primitives) of
 * include/disco_gpu.h, which tests check bit-for-bit against the reference.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "disco_gpu.h"
#include "../../disco_gb300/csrc/plugins/ic_vortex_gauss.h"
#include "../../disco_gb300/csrc/plugins/ic_disks.h"

enum { RHO, PPP, URR, UPP, UZZ };
enum { DDD, TAU, SRR, LLL, SZZ };
#define MAXQ 9

typedef struct {
   int L, R;            /* global cell ids */
   double dxL, dxR, cm[3], dphi, dA;
   int LRtype;
} pface;

typedef struct port_domain {
   disco_params par;
   disco_modules mod;
   int Nr, Nz, NgRa, NgRb, NgZa, NgZb, nq, nc, Npl;
   long N;
   int *Np;
   long *off;
   double *rj, *zk;      /* rj[j] = reference r_jph[j] for j = -1..Nr-1 */
   double Pmax, t;
   double *piph, *dphi, *wiph;
   double *prim, *cons, *RKcons, *gradp, *gradr, *gradz;   /* [c*nq + q] */
   pface *faces[2];
   int *fI[2];
   int nfaces[2];
   disco_planet pl[DISCO_MAX_PLANETS];
   /* physics */
   double gamma_law, rho_floor, p_floor;
} port_domain;

#define P(d, c) ((d)->prim + (size_t)(c)*(d)->nq)
#define U(d, c) ((d)->cons + (size_t)(c)*(d)->nq)

/* ---- geometry: Geometry/cylindrical.c:10-75 ---------------------------- */
static double get_dp(const port_domain *d, double phip, double phim)
{
   double dp = phip - phim;
   while(dp < 0.0) dp += d->Pmax;
   while(dp > d->Pmax) dp -= d->Pmax;
   return dp;
}
static double get_signed_dp(const port_domain *d, double phip, double phim)
{
   double dp = phip - phim;
   while(dp < -.5*d->Pmax) dp += d->Pmax;
   while(dp > .5*d->Pmax) dp -= d->Pmax;
   return dp;
}
static double centroid(double xp, double xm, int dim)
{
   if(dim == 1) return 2.0*(xp*xp + xp*xm + xm*xm)/(3.0*(xp + xm));
   return 0.5*(xp + xm);
}
static double get_dA(const port_domain *d, const double *xp, const double *xm, int dim)
{
   double r = .5*(xp[0] + xm[0]), dr = xp[0] - xm[0];
   double dphi = get_dp(d, xp[1], xm[1]), dz = xp[2] - xm[2];
   if(dim == 0) return dr*dz;
   if(dim == 1) return r*dphi*dz;
   return r*dr*dphi;
}
static double get_dV(const port_domain *d, const double *xp, const double *xm)
{
   double r = .5*(xp[0] + xm[0]), dr = xp[0] - xm[0];
   double dphi = get_dp(d, xp[1], xm[1]), dz = xp[2] - xm[2];
   return r*dr*dphi*dz;
}

/* ---- omega.c (Energy_Omega 0: om = -RotOmega) ---------------------------- */
static double get_om(const port_domain *d, const double *x)
{
   double r = sqrt(x[0]*x[0] + d->par.grav_eps*d->par.grav_eps);
   switch(d->par.Energy_Omega) {
   case 1: return 1.0 - d->par.RotOmega;
   case 2: return 1.0/pow(r, 1.5) - d->par.RotOmega;
   default: return 0.0 - d->par.RotOmega;
   }
}
static double get_om1(const port_domain *d, const double *x)
{
   double r = sqrt(x[0]*x[0] + d->par.grav_eps*d->par.grav_eps);
   if(d->par.Energy_Omega == 2) return -1.5/pow(r, 2.5);
   return 0.0;
}

/* ---- Hydro/euler.c ------------------------------------------------------- */
static void prim2cons(const port_domain *d, const double *prim, double *cons,
                      const double *x, double dV)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double om = get_om(d, x);
   double vp_off = vp - om*r;
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   double rhoe = Pp/(d->gamma_law - 1.);
   cons[DDD] = rho*dV;
   cons[TAU] = (.5*rho*v2 + rhoe)*dV;
   cons[SRR] = rho*vr*dV;
   cons[LLL] = r*rho*vp*dV;
   cons[SZZ] = rho*vz*dV;
   for(int q = d->nc; q < d->nq; q++) cons[q] = prim[q]*cons[DDD];
}
static void getUstar(const port_domain *d, const double *prim, double *Ustar,
                     const double *x, double Sk, double Ss, const double *n)
{
   double r = x[0], rho = prim[RHO], vr = prim[URR], vp = prim[UPP]*r;
   double vz = prim[UZZ], Pp = prim[PPP];
   double om = get_om(d, x);
   double vp_off = vp - om*r;
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   double vn = vr*n[0] + vp*n[1] + vz*n[2];
   double vn_off = vn - om*r*n[1];
   double Ss_off = Ss + vn_off - vn;
   double rhoe = Pp/(d->gamma_law - 1.);
   double rhostar = rho*(Sk - vn)/(Sk - Ss);
   double Pstar = Pp*(Ss - vn)/(Sk - Ss);
   double Us = rhoe*(Sk - vn)/(Sk - Ss);
   Ustar[DDD] = rhostar;
   Ustar[SRR] = rhostar*(vr + (Ss - vn)*n[0]);
   Ustar[LLL] = r*rhostar*(vp + (Ss - vn)*n[1]);
   Ustar[SZZ] = rhostar*(vz + (Ss - vn)*n[2]);
   Ustar[TAU] = .5*rhostar*v2 + Us + rhostar*Ss_off*(Ss - vn) + Pstar;
   for(int q = d->nc; q < d->nq; q++) Ustar[q] = prim[q]*Ustar[DDD];
}
static void cons2prim(const port_domain *d, const double *cons, double *prim,
                      const double *x, double dV)
{
   double r = x[0];
   double rho = cons[DDD]/dV;
   if(rho < d->rho_floor) rho = d->rho_floor;
   double Sr = cons[SRR]/dV, Sp = cons[LLL]/dV/r, Sz = cons[SZZ]/dV, E = cons[TAU]/dV;
   double om = get_om(d, x);
   double vr = Sr/rho, vp = Sp/rho, vp_off = vp - om*r, vz = Sz/rho;
   double KE = .5*(Sr*vr + rho*vp_off*vp_off + Sz*vz);
   double rhoe = E - KE;
   double Pp = (d->gamma_law - 1.)*rhoe;
   if(Pp < d->p_floor*rho) Pp = d->p_floor*rho;
   if(d->par.isothermal_flag) {
      double rr = sqrt(r*r + d->par.grav_eps*d->par.grav_eps);
      double cs2 = 1.0;
      if(d->par.Cs2_Profile == 1) cs2 = 1./(d->par.Disk_Mach*d->par.Disk_Mach);
      else if(d->par.Cs2_Profile == 4) cs2 = (d->par.metricPar2/rr)/(d->par.Disk_Mach*d->par.Disk_Mach);
      Pp = cs2*rho/d->gamma_law;
   }
   prim[RHO] = rho; prim[PPP] = Pp; prim[URR] = vr; prim[UPP] = vp/r; prim[UZZ] = vz;
   for(int q = d->nc; q < d->nq; q++) prim[q] = cons[q]/cons[DDD];
}
static void flux(const port_domain *d, const double *prim, double *f, const double *x,
                 const double *n)
{
   double r = x[0], rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
   double vp = prim[UPP]*r, vz = prim[UZZ];
   double om = get_om(d, x);
   double vn = vr*n[0] + vp*n[1] + vz*n[2];
   double wn = om*r*n[1];
   double vp_off = vp - om*r;
   double rhoe = Pp/(d->gamma_law - 1.);
   double v2 = vr*vr + vp_off*vp_off + vz*vz;
   f[DDD] = rho*vn;
   f[SRR] = rho*vr*vn + Pp*n[0];
   f[LLL] = r*(rho*vp*vn + Pp*n[1]);
   f[SZZ] = rho*vz*vn + Pp*n[2];
   f[TAU] = (.5*rho*v2 + rhoe + Pp)*vn - Pp*wn;
   for(int q = d->nc; q < d->nq; q++) f[q] = prim[q]*f[DDD];
}
static void vel(const port_domain *d, const double *p1, const double *p2, double *Sl,
                double *Sr, double *Ss, const double *n, const double *x)
{
   double r = x[0];
   double P1 = p1[PPP], rho1 = p1[RHO];
   double vn1 = p1[URR]*n[0] + p1[UPP]*n[1]*r + p1[UZZ]*n[2];
   double cs1 = sqrt(d->gamma_law*P1/rho1);
   double P2 = p2[PPP], rho2 = p2[RHO];
   double vn2 = p2[URR]*n[0] + p2[UPP]*n[1]*r + p2[UZZ]*n[2];
   double cs2 = sqrt(d->gamma_law*P2/rho2);
   *Ss = (P2 - P1 + rho1*vn1*(-cs1) - rho2*vn2*cs2)/(rho1*(-cs1) - rho2*cs2);
   *Sr = cs1 + vn1;
   *Sl = -cs1 + vn1;
   if(*Sr < cs2 + vn2) *Sr = cs2 + vn2;
   if(*Sl > -cs2 + vn2) *Sl = -cs2 + vn2;
}
static void source(const port_domain *d, const double *prim, double *cons,
                   const double *xp, const double *xm, double dVdt)
{
   double rp = xp[0], rm = xm[0];
   double rho = prim[RHO], Pp = prim[PPP];
   double r = centroid(rp, rm, 1), z = centroid(xp[2], xm[2], 2);
   double r_1 = .5*(rp + rm);
   double vr = prim[URR], omega = prim[UPP], vz = prim[UZZ];
   double x[3] = {r, 0.5*(xm[1] + xp[1]), z};
   double centrifugal = rho*omega*omega*r;
   double press_bal = Pp/r_1;
   cons[SRR] += dVdt*(centrifugal + press_bal);
   double om = get_om(d, x), om_r = get_om1(d, x), om_z = 0.0;
   cons[TAU] += dVdt*rho*(r*vr*om*om - r*r*(omega - om)*(vr*om_r + vz*om_z));
}
static double mindt(const port_domain *d, const double *prim, double w,
                    const double *xp, const double *xm)
{
   double r = centroid(xp[0], xm[0], 1);
   double Pp = prim[PPP], rho = prim[RHO];
   double vp = (prim[UPP] - w)*r, vr = prim[URR], vz = prim[UZZ];
   double cs = sqrt(d->gamma_law*Pp/rho);
   double maxvr = cs + fabs(vr), maxvp = cs + fabs(vp), maxvz = cs + fabs(vz);
   double dtr = (xp[0] - xm[0])/maxvr;
   double dtp = (.5*(xp[0] + xm[0])*get_dp(d, xp[1], xm[1]))/maxvp;
   double dtz = (xp[2] - xm[2])/maxvz;
   double dt = dtr;
   if(dt > dtp) dt = dtp;
   if(dt > dtz) dt = dtz;
   return dt;
}

/* ---- Riemann solver: riemann.c:216-320 (HLL / HLLC) ------------------------- */
static void solve_riemann(port_domain *d, const double *primL, const double *primR,
                          double *consL, double *consR, const double *x, const double *n,
                          double w, double dAdt)
{
   int nq = d->nq, q;
   double Flux[MAXQ] = {0}, Ustr[MAXQ] = {0};
   double Sl, Sr, Ss;
   vel(d, primL, primR, &Sl, &Sr, &Ss, n, x);
   if(w < Sl) {
      flux(d, primL, Flux, x, n);
      prim2cons(d, primL, Ustr, x, 1.0);
   } else if(w > Sr) {
      flux(d, primR, Flux, x, n);
      prim2cons(d, primR, Ustr, x, 1.0);
   } else if(d->par.Riemann_Solver == 0) {
      double Fl[MAXQ], Fr[MAXQ], Ul[MAXQ], Ur[MAXQ];
      double aL = Sr, aR = -Sl;
      prim2cons(d, primL, Ul, x, 1.0);
      prim2cons(d, primR, Ur, x, 1.0);
      flux(d, primL, Fl, x, n);
      flux(d, primR, Fr, x, n);
      for(q = 0; q < nq; q++) {
         Flux[q] = (aL*Fl[q] + aR*Fr[q] + aL*aR*(Ul[q] - Ur[q]))/(aL + aR);
         Ustr[q] = (aR*Ul[q] + aL*Ur[q] + Fl[q] - Fr[q])/(aL + aR);
      }
   } else {
      double Uk[MAXQ], Fk[MAXQ];
      if(w < Ss) {
         prim2cons(d, primL, Uk, x, 1.0);
         getUstar(d, primL, Ustr, x, Sl, Ss, n);
         flux(d, primL, Fk, x, n);
         for(q = 0; q < nq; q++) Flux[q] = Fk[q] + Sl*(Ustr[q] - Uk[q]);
      } else {
         prim2cons(d, primR, Uk, x, 1.0);
         getUstar(d, primR, Ustr, x, Sr, Ss, n);
         flux(d, primR, Fk, x, n);
         for(q = 0; q < nq; q++) Flux[q] = Fk[q] + Sr*(Ustr[q] - Uk[q]);
      }
   }
   for(q = 0; q < nq; q++) {
      consL[q] -= (Flux[q] - w*Ustr[q])*dAdt;
      consR[q] += (Flux[q] - w*Ustr[q])*dAdt;
   }
}

/* ---- faces: faces_alt.c:36-179 (sequential walk) ---------------------------- */
static void build_faces(port_domain *d, int dim)
{
   int Nr = d->Nr, Nz = d->Nz, j, k, i, jk;
   int *I0 = (int *)malloc(sizeof(int)*Nr*Nz);
   double convert = 2.*M_PI/d->Pmax;
   for(jk = 0; jk < Nr*Nz; jk++) {
      int found = 0, quad_prev = 0;
      for(i = 0; i < d->Np[jk] && !found; i++) {
         double ph = d->piph[d->off[jk] + i];
         double sn = sin(ph*convert), cs = cos(ph*convert);
         if(sn > 0. && cs > 0. && quad_prev) { found = 1; I0[jk] = i; }
         else if(sn < 0. && cs > 0.) quad_prev = 1;
      }
      if(!found) I0[jk] = 0;
   }
   int Nrmax = dim == 1 ? Nr - 1 : Nr;
   int Nzmax = dim == 1 ? Nz : Nz - 1;
   int d0 = dim - 1;
   int n = 0;
   for(k = 0; k < Nzmax; k++) for(j = 0; j < Nrmax; j++) {
      int JK = j + Nrmax*k;
      int L = j + Nr*k, R = dim == 1 ? j + 1 + Nr*k : j + Nr*(k + 1);
      d->fI[d0][JK] = n;
      n += d->Np[L] + d->Np[R];
   }
   d->fI[d0][Nrmax*Nzmax] = n;
   d->nfaces[d0] = n;
   free(d->faces[d0]);
   d->faces[d0] = (pface *)malloc(sizeof(pface)*(n > 0 ? n : 1));
   const double *rj = d->rj, *zk = d->zk;
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
      for(f = 0; f < d->Np[jkL] + d->Np[jkR]; f++) {
         long cL = d->off[jkL] + a, cR = d->off[jkR] + b;
         double dphi = d->piph[cL] - d->piph[cR];
         while(dphi > .5*d->Pmax) dphi -= d->Pmax;
         while(dphi < -.5*d->Pmax) dphi += d->Pmax;
         int LR = dphi > 0. ? 1 : 0;
         dphi = d->piph[cL] - d->dphi[cL] - d->piph[cR] + d->dphi[cR];
         while(dphi > .5*d->Pmax) dphi -= d->Pmax;
         while(dphi < -.5*d->Pmax) dphi += d->Pmax;
         int LR_back = dphi < 0. ? 1 : 0;
         xp[1] = LR == 0 ? d->piph[cL] : d->piph[cR];
         xm[1] = LR_back == 0 ? d->piph[cL] - d->dphi[cL] : d->piph[cR] - d->dphi[cR];
         /* addFace, faces_alt.c:10-34 */
         pface *F = &d->faces[d0][n];
         double dp = get_dp(d, xp[1], xm[1]);
         double phic = get_dp(d, xp[1], .5*dp);
         F->cm[0] = dim == 1 ? 0.5*(xp[0] + xm[0]) : centroid(xp[0], xm[0], 1);
         F->cm[1] = phic;
         F->cm[2] = dim == 2 ? 0.5*(xp[2] + xm[2]) : centroid(xp[2], xm[2], 2);
         F->L = (int)cL; F->R = (int)cR; F->dxL = dxL; F->dxR = dxR;
         F->dphi = dp; F->dA = get_dA(d, xp, xm, dim); F->LRtype = LR;
         n++;
         if(LR == 0) { a++; if(a == d->Np[jkL]) a = 0; }
         else { b++; if(b == d->Np[jkR]) b = 0; }
      }
   }
   free(I0);
}

/* ---- reconstruction: plm.c ---------------------------------------------------- */
static double minmod(double a, double b, double c)
{
   double m = a;
   if(a*b < 0.0) m = 0.0;
   if(fabs(b) < fabs(m)) m = b;
   if(b*c < 0.0) m = 0.0;
   if(fabs(c) < fabs(m)) m = c;
   return m;
}
static void plm_phi(port_domain *d)
{
   int jk, i, q, nq = d->nq;
   double PLM = d->par.PLM;
   for(jk = 0; jk < d->Nr*d->Nz; jk++) {
      long o = d->off[jk];
      int Np = d->Np[jk];
      for(i = 0; i < Np; i++) {
         long c = o + i, cl = o + (i == 0 ? Np - 1 : i - 1), cr = o + (i + 1)%Np;
         double dpL = d->dphi[cl], dpC = d->dphi[c], dpR = d->dphi[cr];
         for(q = 0; q < nq; q++) {
            double pL = P(d, cl)[q], pC = P(d, c)[q], pR = P(d, cr)[q];
            double sL = pC - pL; sL /= .5*(dpC + dpL);
            double sR = pR - pC; sR /= .5*(dpR + dpC);
            double sC = pR - pL; sC /= .5*(dpL + dpR) + dpC;
            d->gradp[c*nq + q] = minmod(PLM*sL, sC, PLM*sR);
         }
      }
   }
}
static void plm_trans(port_domain *d, int dim)
{
   int nq = d->nq, q, n;
   long c;
   double *G = dim == 1 ? d->gradr : d->gradz;
   memset(G, 0, sizeof(double)*nq*d->N);
   double PLM = d->par.PLM;
   if(PLM == 0.0) return;
   pface *Fs = d->faces[dim - 1];
   int Nf = d->nfaces[dim - 1];
   for(n = 0; n < Nf; n++) {
      pface *f = &Fs[n];
      double phi = f->cm[1];
      double phiL = d->piph[f->L] - .5*d->dphi[f->L], phiR = d->piph[f->R] - .5*d->dphi[f->R];
      double dpL = get_signed_dp(d, phi, phiL), dpR = get_signed_dp(d, phiR, phi);
      for(q = 0; q < nq; q++) {
         double WL = P(d, f->L)[q] + dpL*d->gradp[(size_t)f->L*nq + q];
         double WR = P(d, f->R)[q] - dpR*d->gradp[(size_t)f->R*nq + q];
         double S = (WR - WL)/(f->dxR + f->dxL);
         G[(size_t)f->L*nq + q] += S*f->dA;
         G[(size_t)f->R*nq + q] += S*f->dA;
      }
   }
   int j, k, i;
   for(j = 0; j < d->Nr; j++) for(k = 0; k < d->Nz; k++) {
      int jk = j + d->Nr*k;
      for(i = 0; i < d->Np[jk]; i++) {
         c = d->off[jk] + i;
         double phip = d->piph[c], phim = phip - d->dphi[c];
         double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
         if(dim == 1) xm[0] = d->rj[j]; else xm[2] = d->zk[k];
         double dAp = get_dA(d, xp, xm, dim);
         if(dim == 1) { xp[0] = d->rj[j - 1]; xm[0] = d->rj[j - 1]; }
         else { xp[2] = d->zk[k - 1]; xm[2] = d->zk[k - 1]; }
         double dAm = get_dA(d, xp, xm, dim);
         double dAtot = dAp + dAm;
         if((dim == 1 && j == 0) || (dim == 2 && k == 0)) dAtot = dAp;
         if((dim == 1 && j == d->Nr - 1) || (dim == 2 && k == d->Nz - 1)) dAtot = dAm;
         for(q = 0; q < nq; q++) G[c*nq + q] /= dAtot;
      }
   }
   for(n = 0; n < Nf; n++) {
      pface *f = &Fs[n];
      double phi = f->cm[1];
      double phiL = d->piph[f->L] - .5*d->dphi[f->L], phiR = d->piph[f->R] - .5*d->dphi[f->R];
      double dpL = get_signed_dp(d, phi, phiL), dpR = get_signed_dp(d, phiR, phi);
      for(q = 0; q < nq; q++) {
         double WL = P(d, f->L)[q] + dpL*d->gradp[(size_t)f->L*nq + q];
         double WR = P(d, f->R)[q] - dpR*d->gradp[(size_t)f->R*nq + q];
         double S = (WR - WL)/(f->dxR + f->dxL);
         double *gL = &G[(size_t)f->L*nq + q], *gR = &G[(size_t)f->R*nq + q];
         if(S*(*gL) < 0.0) *gL = 0.0; else if(fabs(PLM*S) < fabs(*gL)) *gL = PLM*S;
         if(S*(*gR) < 0.0) *gR = 0.0; else if(fabs(PLM*S) < fabs(*gR)) *gR = PLM*S;
      }
   }
}

/* ---- fluxes: misc.c:378-519, riemann.c:39-214 --------------------------------- */
static void phi_flux(port_domain *d, double dt)
{
   int j, k, i, q, nq = d->nq;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) {
      double zp = d->zk[k], zm = d->zk[k - 1], z = centroid(zp, zm, 2);
      for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
         double rp = d->rj[j], rm = d->rj[j - 1], r = centroid(rp, rm, 1);
         int jk = j + d->Nr*k, Np = d->Np[jk];
         long o = d->off[jk];
         for(i = 0; i < Np; i++) {
            long cl = o + i, cr = o + (i < Np - 1 ? i + 1 : 0);
            double phi = d->piph[cl];
            double xp[3] = {rp, phi, zp}, xm[3] = {rm, phi, zm};
            double dA = get_dA(d, xp, xm, 0);
            double x[3] = {r, phi, z};
            double primL[MAXQ], primR[MAXQ];
            for(q = 0; q < nq; q++) {
               primL[q] = P(d, cl)[q] + .5*d->gradp[cl*nq + q]*d->dphi[cl];
               primR[q] = P(d, cr)[q] - .5*d->gradp[cr*nq + q]*d->dphi[cr];
            }
            double n[3] = {0.0, 1.0, 0.0};
            double hn = x[0];
            solve_riemann(d, primL, primR, U(d, cl), U(d, cr), x, n, hn*d->wiph[cl], dA*dt);
         }
      }
   }
}
static void trans_flux(port_domain *d, double dt, int dim)
{
   int jmin, jmax, kmin, kmax, Nfr, j, k, q, nq = d->nq;
   if(dim == 1) {
      Nfr = d->Nr - 1;
      jmin = d->NgRa == 0 ? 0 : d->NgRa - 1; jmax = d->NgRb == 0 ? d->Nr - 1 : d->Nr - d->NgRb;
      kmin = d->NgZa; kmax = d->Nz - d->NgZb;
   } else {
      Nfr = d->Nr;
      jmin = d->NgRa; jmax = d->Nr - d->NgRb;
      kmin = d->NgZa == 0 ? 0 : d->NgZa - 1; kmax = d->NgZb == 0 ? d->Nz - 1 : d->Nz - d->NgZb;
   }
   pface *Fs = d->faces[dim - 1];
   int *fI = d->fI[dim - 1];
   for(k = kmin; k < kmax; k++) for(j = jmin; j < jmax; j++) {
      int JK = j + Nfr*k, f;
      for(f = fI[JK]; f < fI[JK + 1]; f++) {
         pface *F = &Fs[f];
         double *gL = (dim == 1 ? d->gradr : d->gradz) + (size_t)F->L*nq;
         double *gR = (dim == 1 ? d->gradr : d->gradz) + (size_t)F->R*nq;
         double phiL = d->piph[F->L] - .5*d->dphi[F->L], phiR = d->piph[F->R] - .5*d->dphi[F->R];
         double dpL = get_signed_dp(d, F->cm[1], phiL), dpR = get_signed_dp(d, phiR, F->cm[1]);
         double primL[MAXQ], primR[MAXQ];
         for(q = 0; q < nq; q++) {
            primL[q] = P(d, F->L)[q] + gL[q]*F->dxL + d->gradp[(size_t)F->L*nq + q]*dpL;
            primR[q] = P(d, F->R)[q] - gR[q]*F->dxR - d->gradp[(size_t)F->R*nq + q]*dpR;
         }
         double n[3] = {0.0, 0.0, 0.0};
         if(dim == 1) n[0] = 1.0; else n[2] = 1.0;
         solve_riemann(d, primL, primR, U(d, F->L), U(d, F->R), F->cm, n, 0.0, F->dA*dt);
      }
   }
}

/* ---- cell loops: misc.c ---------------------------------------------------------- */
static void set_wcell(port_domain *d)
{
   int jk, i;
   for(jk = 0; jk < d->Nr*d->Nz; jk++) {
      long o = d->off[jk];
      int Np = d->Np[jk];
      for(i = 0; i < Np; i++) {
         double w = 0.0;
         if(d->par.Mesh_Motion) w = .5*(P(d, o + i)[UPP] + P(d, o + (i + 1)%Np)[UPP]);
         d->wiph[o + i] = w;
      }
      if(d->par.Mesh_Motion == 3) {
         double w = 0.0;
         for(i = 0; i < Np; i++) w += d->wiph[o + i];
         w /= (double)Np;
         for(i = 0; i < Np; i++) d->wiph[o + i] = w;
      }
   }
}
static void calc_dp(port_domain *d)
{
   int jk, i;
   for(jk = 0; jk < d->Nr*d->Nz; jk++) {
      long o = d->off[jk];
      int Np = d->Np[jk];
      for(i = 0; i < Np; i++) {
         int im = i == 0 ? Np - 1 : i - 1;
         d->dphi[o + i] = get_dp(d, d->piph[o + i], d->piph[o + im]);
      }
   }
}
static void calc_prim(port_domain *d)
{
   int j, k, i;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) {
      double zm = d->zk[k - 1], zp = d->zk[k], z = centroid(zp, zm, 2);
      for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
         int jk = j + d->Nr*k;
         double rm = d->rj[j - 1], rp = d->rj[j], r = centroid(rp, rm, 1);
         for(i = 0; i < d->Np[jk]; i++) {
            long c = d->off[jk] + i;
            double phip = d->piph[c], phim = phip - d->dphi[c];
            double xp[3] = {rp, phip, zp}, xm[3] = {rm, phim, zm};
            double dV = get_dV(d, xp, xm);
            double x[3] = {r, 0.5*(phim + phip), z};
            cons2prim(d, U(d, c), P(d, c), x, dV);
         }
      }
   }
}
static void initial(const port_domain *d, double *prim, const double *x)
{
   const disco_params *p = &d->par;
   if(d->mod.initial == DISCO_IC_VORTEX_GAUSS) {
      struct disco_ic_vortex_gauss V = {p->initPar1, p->initPar2, p->initPar3, p->initPar4,
                                        p->initPar5, p->Adiabatic_Index};
      disco_ic_vortex_gauss_eval(&V, prim, x, d->nc, d->nq);
   } else {
      struct disco_ic_disk D;
      disco_ic_disk_from_params(&D, p->Adiabatic_Index, p->Disk_Mach, p->initPar1, p->initPar2,
                                p->initPar3, p->initPar4, p->initPar5, p->initPar6);
      if(d->mod.initial == DISCO_IC_DISK_MHD) disco_ic_disk_mhd_eval(&D, prim, x, d->nc, d->nq);
      else disco_ic_disk_planet_eval(&D, prim, x, d->nc, d->nq);
   }
   if(p->RotFrame) prim[UPP] -= p->RotOmega;
}
/* Boundary/fixed.c:11-46 (r ghosts) and fixed3d.c via set_cell_init. */
static void boundary(port_domain *d)
{
   int j, k, i;
   for(k = 0; k < d->Nz; k++) for(j = 0; j < d->Nr; j++) {
      int rg = j < d->NgRa || j >= d->Nr - d->NgRb;
      int zg = k < d->NgZa || k >= d->Nz - d->NgZb;
      int jk = j + d->Nr*k;
      for(i = 0; i < d->Np[jk]; i++) {
         long c = d->off[jk] + i;
         double x[3];
         if(d->mod.boundary == DISCO_BC_FIXED) {
            if(!rg || d->Nr <= 1) continue;
            x[0] = .5*(d->rj[j] + d->rj[j - 1]);
            x[1] = d->piph[c] - .5*d->dphi[c];
            x[2] = .5*(d->zk[k] + d->zk[k - 1]);
         } else {
            if(!((rg && d->Nr > 1) || (zg && d->Nz > 1))) continue;
            x[0] = centroid(d->rj[j], d->rj[j - 1], 1);
            x[1] = .5*(d->piph[c] + d->piph[c] - d->dphi[c]);
            x[2] = centroid(d->zk[k], d->zk[k - 1], 2);
         }
         initial(d, P(d, c), x);
      }
   }
}
static void add_source(port_domain *d, double dt)
{
   int j, k, i;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
      int jk = j + d->Nr*k;
      for(i = 0; i < d->Np[jk]; i++) {
         long c = d->off[jk] + i;
         double phip = d->piph[c], phim = d->piph[c] - d->dphi[c];
         double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
         double dV = get_dV(d, xp, xm);
         source(d, P(d, c), U(d, c), xp, xm, dV*dt);
      }
   }
}

static void onestep(port_domain *d, double RK, double dt, int first)
{
   long c;
   int q, nq = d->nq;
   if(first) set_wcell(d);
   for(c = 0; c < d->N; c++)
      for(q = 0; q < nq; q++) U(d, c)[q] = (1. - RK)*U(d, c)[q] + RK*d->RKcons[c*nq + q];
   plm_phi(d);
   if(d->Nr > 1) plm_trans(d, 1);
   if(d->Nz > 1) plm_trans(d, 2);
   phi_flux(d, dt);
   if(d->Nr > 1) trans_flux(d, dt, 1);
   if(d->Nz > 1) trans_flux(d, dt, 2);
   add_source(d, dt);
   if(first) for(c = 0; c < d->N; c++) d->piph[c] += d->wiph[c]*dt;
   for(c = 0; c < d->N; c++) {    /* clean_pi, misc.c:8-26 */
      double phi = d->piph[c];
      while(phi > d->Pmax) phi -= d->Pmax;
      while(phi < 0.0) phi += d->Pmax;
      d->piph[c] = phi;
   }
   calc_dp(d);
   calc_prim(d);
   boundary(d);
}

static double getmindt(port_domain *d)
{
   double dt = d->par.maxDT/d->par.CFL;
   if(dt <= 0.0) dt = 1.0e100;
   int j, k, i;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
      int jk = j + d->Nr*k, Np = d->Np[jk];
      for(i = 0; i < Np; i++) {
         long c = d->off[jk] + i;
         double phip = d->piph[c], phim = phip - d->dphi[c];
         double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
         long cm = d->off[jk] + (i == 0 ? Np - 1 : i - 1);
         double w = .5*(d->wiph[cm] + d->wiph[c]);
         double t = mindt(d, P(d, c), w, xp, xm);
         if(dt > t) dt = t;
      }
   }
   return dt*d->par.CFL;
}

/* ---- public checker API ------------------------------------------------------- */
port_domain *disco_port_create(const disco_host_domain *h)
{
   if(h->mod.hydro != DISCO_HYDRO_EULER) return NULL;
   port_domain *d = (port_domain *)calloc(1, sizeof(*d));
   d->par = h->par; d->mod = h->mod;
   d->Nr = h->Nr; d->Nz = h->Nz; d->NgRa = h->NgRa; d->NgRb = h->NgRb;
   d->NgZa = h->NgZa; d->NgZb = h->NgZb; d->nq = h->num_q; d->nc = h->mod.num_c;
   d->N = h->Ncell; d->Pmax = h->phi_max; d->t = h->t; d->Npl = h->Npl;
   memcpy(d->pl, h->planets, sizeof d->pl);
   d->gamma_law = h->par.Adiabatic_Index;
   d->rho_floor = h->par.Density_Floor; d->p_floor = h->par.Pressure_Floor;
   int R = d->Nr*d->Nz;
   d->Np = (int *)malloc(sizeof(int)*R); memcpy(d->Np, h->Np, sizeof(int)*R);
   d->off = (long *)malloc(sizeof(long)*(R + 1)); memcpy(d->off, h->ring_off, sizeof(long)*(R + 1));
   double *rj = (double *)malloc(sizeof(double)*(d->Nr + 1));
   double *zk = (double *)malloc(sizeof(double)*(d->Nz + 1));
   memcpy(rj, h->r_jph, sizeof(double)*(d->Nr + 1));
   memcpy(zk, h->z_kph, sizeof(double)*(d->Nz + 1));
   d->rj = rj + 1; d->zk = zk + 1;
   long N = d->N;
   int nq = d->nq;
   d->piph = (double *)malloc(sizeof(double)*N); memcpy(d->piph, h->piph, sizeof(double)*N);
   d->dphi = (double *)malloc(sizeof(double)*N); memcpy(d->dphi, h->dphi, sizeof(double)*N);
   d->wiph = (double *)calloc(N, sizeof(double));
   d->prim = (double *)calloc((size_t)nq*N, sizeof(double));
   d->cons = (double *)calloc((size_t)nq*N, sizeof(double));
   d->RKcons = (double *)calloc((size_t)nq*N, sizeof(double));
   d->gradp = (double *)calloc((size_t)nq*N, sizeof(double));
   d->gradr = (double *)calloc((size_t)nq*N, sizeof(double));
   d->gradz = (double *)calloc((size_t)nq*N, sizeof(double));
   d->fI[0] = (int *)malloc(sizeof(int)*((d->Nr - 1)*d->Nz + 2));
   d->fI[1] = (int *)malloc(sizeof(int)*(d->Nr*(d->Nz > 1 ? d->Nz - 1 : 0) + 2));
   /* setupCells: prim2cons then cons2prim for real cells (domain.c:319-382) */
   int j, k, i, q;
   for(k = d->NgZa; k < d->Nz - d->NgZb; k++) {
      double z = centroid(d->zk[k], d->zk[k - 1], 2);
      for(j = d->NgRa; j < d->Nr - d->NgRb; j++) {
         double r = centroid(d->rj[j], d->rj[j - 1], 1);
         int jk = j + d->Nr*k;
         for(i = 0; i < d->Np[jk]; i++) {
            long c = d->off[jk] + i;
            double phip = d->piph[c], phim = phip - d->dphi[c];
            double xp[3] = {d->rj[j], phip, d->zk[k]}, xm[3] = {d->rj[j - 1], phim, d->zk[k - 1]};
            double dV = get_dV(d, xp, xm);
            double x[3] = {r, d->piph[c] - .5*d->dphi[c], z};
            for(q = 0; q < nq; q++) P(d, c)[q] = h->prim[(size_t)q*N + c];
            prim2cons(d, P(d, c), U(d, c), x, dV);
            cons2prim(d, U(d, c), P(d, c), x, dV);
         }
      }
   }
   set_wcell(d);
   boundary(d);
   return d;
}

/* timestep.c:7-54 (Timestep 0), preceded by getmindt (main.c:70). */
double disco_port_step(port_domain *d)
{
   double dt = getmindt(d);
   memcpy(d->RKcons, d->cons, sizeof(double)*d->nq*d->N);
   if(d->Nr > 1) build_faces(d, 1);
   if(d->Nz > 1) build_faces(d, 2);
   onestep(d, 0.0, dt, 1);
   d->t += dt;
   if(d->Nr > 1) build_faces(d, 1);
   if(d->Nz > 1) build_faces(d, 2);
   onestep(d, 0.5, 0.5*dt, 0);
   return dt;
}

int disco_port_run(port_domain *d, int nsteps)
{
   for(int s = 0; s < nsteps; s++) disco_port_step(d);
   return 0;
}

/* SoA download, same layout as disco_gpu_download. */
void disco_port_state(const port_domain *d, double *piph, double *dphi, double *prim,
                      double *cons, double *t)
{
   long N = d->N, c;
   int q, nq = d->nq;
   if(piph) memcpy(piph, d->piph, sizeof(double)*N);
   if(dphi) memcpy(dphi, d->dphi, sizeof(double)*N);
   for(c = 0; c < N; c++) for(q = 0; q < nq; q++) {
      if(prim) prim[(size_t)q*N + c] = d->prim[c*nq + q];
      if(cons) cons[(size_t)q*N + c] = d->cons[c*nq + q];
   }
   if(t) *t = d->t;
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
   free(d->piph); free(d->dphi); free(d->wiph); free(d->prim); free(d->cons);
   free(d->RKcons); free(d->gradp); free(d->gradr); free(d->gradz);
   free(d->faces[0]); free(d->faces[1]); free(d->fI[0]); free(d->fI[1]);
   free(d);
}
