/*
 * fm_torus: the Fishbone-Moncrief (1976) equilibrium torus around a Kerr
 * black hole (mass M, spin a), written for Kerr-Schild CYLINDRICAL
 * coordinates (r, phi, z) -- the coordinates of plugins/metric_kerr.h.  The
 * reference's nearest relative, Initial/torus_fm_grmhd.c, reads x[2] as a
 * polar angle; this plugin takes x = (r, phi, z) like every other initial
 * condition of the cylindrical build.  Same plugin contract: fill prim[] in
 * {RHO, PPP, URR, UPP, UZZ, BRR, BPP, BZZ, passive} order at x.
 *
 * The torus (a published solution, restated from its defining relations):
 *  - constant ell = u^t u_phi, that of the prograde circular equatorial
 *    orbit at the pressure maximum r_pk (Boyer-Lindquist), from the orbit's
 *    u^t and u_phi (Bardeen, Press & Teukolsky 1972);
 *  - enthalpy ln h(R, th) = F(R, th) - F(r_in, pi/2) with, in Boyer-Lindquist
 *    (R, th): Delta = R^2 - 2MR + a^2, Sigma = R^2 + a^2 cos^2 th,
 *    A = (R^2 + a^2)^2 - Delta a^2 sin^2 th, e^2nu = Sigma Delta / A,
 *    e^2psi = A sin^2 th / Sigma, omega = 2 M a R / A, and
 *    F = 1/2 ln((1 + q) / e^2nu) - q/2 - ell omega,
 *    q = sqrt(1 + 4 ell^2 e^2nu / e^2psi);
 *  - polytrope P = K rho^gam with K chosen so that rho = 1 at (r_pk, pi/2):
 *    rho = ((h - 1) / (h_pk - 1))^(1 / (gam - 1));
 *  - purely azimuthal motion: in the frame of the zero-angular-momentum
 *    observer u^(phi) = sqrt((q - 1) / 2), so u^t = sqrt(1 + u^(phi)^2) e^-nu
 *    and u^phi = omega u^t + u^(phi) e^-psi.  With no radial motion the
 *    Boyer-Lindquist and Kerr-Schild u^t, u^phi coincide, and the
 *    cylindrical Kerr-Schild point (r = sqrt(R^2 + a^2) sin th, z = R cos th)
 *    does not move in r or z;
 *  - primitives: the covariant u_r, u_phi / r^2, u_z lowered with the metric;
 *  - outside the torus (h <= 1 or R < r_in): rho = rho_atm, P = rho_atm
 *    cs2_atm, at rest with respect to the normal observer (u_i = 0), as the
 *    reference's torus does;
 *  - poloidal loop field from A_phi = max(rho - acut, 0): with the module's
 *    field primitives sqrt(gamma) B^i / r (prim[BRR], prim[BZZ]) the field
 *    is prim[BRR] = -dA/dz / r, prim[BZZ] = dA/dr / r (divergence-free), by
 *    centred differences, scaled by bscale so that max P / max(B^2 / 2) =
 *    beta over the torus (sampled once by disco_ic_fm_setup).
 * Parameters: gam = Adiabatic_Index, M = Metric_Par2, a = Metric_Par3,
 * r_in = Init_Par1, r_pk = Init_Par2, beta = Init_Par3 (0: no field),
 * acut = Init_Par4, rho_atm = Density_Floor, cs2_atm = Pressure_Floor,
 * passive scalar = 1 inside the torus.
 */
#ifndef DISCO_IC_FM_TORUS_H
#define DISCO_IC_FM_TORUS_H

#include <math.h>
#include "metric_kerr.h"

struct disco_ic_fm {
   double gam, M, a, rin, rpk, beta, acut, rho_atm, cs2_atm;
   /* derived by disco_ic_fm_setup */
   double ell, F_in, hpk1, bscale;
};

/* ell = u^t u_phi of the prograde circular equatorial orbit at radius r */
DISCO_HD static inline double disco_fm_ell(double M, double a, double r)
{
   double sM = sqrt(M), sr = sqrt(r), r32 = r*sr;
   double den = r32 - 3.0*M*sr + 2.0*a*sM;
   double ut2 = (r32 + a*sM)*(r32 + a*sM)/(r32*den);
   double uphi_ut = sM*(r*r - 2.0*a*sM*sr + a*a)/(r32 + a*sM);
   return ut2*uphi_ut;
}

/* F(R, th) of the enthalpy and the pieces the velocity needs */
struct disco_fm_bl {
   double F, q, e2nu, e2psi, omega;
   int ok;     /* outside the horizon and off the axis */
};

DISCO_HD static inline void disco_fm_F(const struct disco_ic_fm *P, double R, double s2,
                                       struct disco_fm_bl *b)
{
   double M = P->M, a = P->a;
   double c2 = 1.0 - s2;
   double Delta = R*R - 2.0*M*R + a*a;
   double Sigma = R*R + a*a*c2;
   double A = (R*R + a*a)*(R*R + a*a) - Delta*a*a*s2;
   b->ok = Delta > 0.0 && s2 > 0.0 && A > 0.0;
   if(!b->ok) return;
   b->e2nu = Sigma*Delta/A;
   b->e2psi = A*s2/Sigma;
   b->omega = 2.0*M*a*R/A;
   b->q = sqrt(1.0 + 4.0*P->ell*P->ell*b->e2nu/b->e2psi);
   b->F = 0.5*log((1.0 + b->q)/b->e2nu) - 0.5*b->q - P->ell*b->omega;
}

/* density (normalised, 0 outside) at the cylindrical Kerr-Schild point,
 * with the Boyer-Lindquist pieces for the velocity */
DISCO_HD static inline double disco_fm_rho(const struct disco_ic_fm *P, double r, double z,
                                           struct disco_fm_bl *b)
{
   double R = disco_kerr_R(r, z, P->a);
   double s2 = r*r/(R*R + P->a*P->a);
   disco_fm_F(P, R, s2, b);
   if(!b->ok || R < P->rin) { b->ok = 0; return 0.0; }
   double lnh = b->F - P->F_in;
   if(lnh <= 0.0) { b->ok = 0; return 0.0; }
   double hm1 = exp(lnh) - 1.0;
   return pow(hm1/P->hpk1, 1.0/(P->gam - 1.0));
}

DISCO_HD static inline double disco_fm_apot(const struct disco_ic_fm *P, double r, double z)
{
   struct disco_fm_bl b;
   double rho = disco_fm_rho(P, r, z, &b);
   double A = rho - P->acut;
   return A > 0.0 ? A : 0.0;
}

/* unscaled field primitives sqrt(gamma) B^r / r and sqrt(gamma) B^z / r */
DISCO_HD static inline void disco_fm_field(const struct disco_ic_fm *P, double r, double z,
                                           double *br, double *bz)
{
   double h = 1.0e-4*(r > 1.0 ? r : 1.0);
   double dAdz = (disco_fm_apot(P, r, z + h) - disco_fm_apot(P, r, z - h))/(2.0*h);
   double dAdr = (disco_fm_apot(P, r + h, z) - disco_fm_apot(P, r - h, z))/(2.0*h);
   *br = -dAdz/r;
   *bz = dAdr/r;
}

DISCO_HD static inline void disco_ic_fm_eval(const struct disco_ic_fm *P, double *prim, const double *x,
                                             int num_c, int num_q)
{
   double r = x[0], z = x[2];
   struct disco_fm_bl b;
   double rho = disco_fm_rho(P, r, z, &b);
   double K = P->hpk1*(P->gam - 1.0)/P->gam;
   double ur = 0.0, up = 0.0, uz = 0.0, Pp, pas = 0.0;
   if(b.ok && rho > 0.0) {
      Pp = K*pow(rho, P->gam);
      pas = 1.0;
      double uzamo = sqrt(0.5*(b.q - 1.0));
      double ut = sqrt(1.0 + uzamo*uzamo)/sqrt(b.e2nu);
      double uphi = b.omega*ut + uzamo/sqrt(b.e2psi);
      struct disco_kerr_pt k;
      disco_kerr_point(r, z, P->M, P->a, 0, &k);
      double lu = ut*k.l[0] + uphi*k.l[2];     /* l_mu u^mu */
      ur = k.H*k.l[1]*lu;
      up = (r*r*uphi + k.H*k.l[2]*lu)/(r*r);
      uz = k.H*k.l[3]*lu;
   } else {
      rho = P->rho_atm;
      Pp = P->rho_atm*P->cs2_atm;
   }
   prim[0] = rho;
   prim[1] = Pp;
   prim[2] = ur;
   prim[3] = up;
   prim[4] = uz;
   if(num_c > 5) {
      double br = 0.0, bz = 0.0;
      if(P->bscale > 0.0) {
         disco_fm_field(P, r, z, &br, &bz);
         br *= P->bscale;
         bz *= P->bscale;
      }
      prim[5] = br;
      prim[6] = 0.0;
      prim[7] = bz;
   }
   for(int q = num_c; q < num_q; q++) prim[q] = pas;
}

/* Derived constants: ell, F(r_in, pi/2), h(r_pk) - 1, and the field scale
 * that makes max P / max(B^2 / 2) = beta, B^2 = gamma_ij B^i B^j, sampled
 * on a 256 x 256 lattice over r in (r_in, 8 r_pk), |z| < 4 r_pk. */
DISCO_HD static inline void disco_ic_fm_setup(struct disco_ic_fm *P)
{
   struct disco_fm_bl b;
   P->ell = disco_fm_ell(P->M, P->a, P->rpk);
   disco_fm_F(P, P->rin, 1.0, &b);
   P->F_in = b.F;
   disco_fm_F(P, P->rpk, 1.0, &b);
   P->hpk1 = exp(b.F - P->F_in) - 1.0;
   P->bscale = 0.0;
   if(!(P->beta > 0.0)) return;
   double K = P->hpk1*(P->gam - 1.0)/P->gam;
   double pmax = 0.0, pmag = 0.0;
   const int n = 256;
   double r0 = sqrt(P->rin*P->rin + P->a*P->a), r1 = 8.0*P->rpk, zr = 4.0*P->rpk;
   for(int i = 0; i < n; i++)
      for(int k = 0; k < n; k++) {
         double r = r0 + (r1 - r0)*(i + 0.5)/n;
         double z = -zr + 2.0*zr*(k + 0.5)/n;
         double rho = disco_fm_rho(P, r, z, &b);
         if(rho <= 0.0) continue;
         double Pp = K*pow(rho, P->gam);
         if(Pp > pmax) pmax = Pp;
         double br, bz, al, gam[9];
         disco_fm_field(P, r, z, &br, &bz);
         double x[3] = {r, 0.0, z};
         disco_kerr_3p1(x, P->M, P->a, &al, 0, gam, 0);
         /* B^i = prim / (sqrt(gamma) / r) = al * prim (sqrt(-g) = r) */
         double Br = al*br, Bz = al*bz;
         double B2 = gam[0]*Br*Br + 2.0*gam[2]*Br*Bz + gam[8]*Bz*Bz;
         if(0.5*B2 > pmag) pmag = 0.5*B2;
      }
   if(pmag > 0.0) P->bscale = sqrt(pmax/(P->beta*pmag));
}

#endif
