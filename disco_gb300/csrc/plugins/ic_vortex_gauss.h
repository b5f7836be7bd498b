/*
 * Initial condition "vortex_gauss": uniform background (rho = 1, P = 1) in
 * rigid rotation Omega0, plus an isentropic Gaussian vortex centred at
 * (r0, phi0) with core radius sigma and peak swirl speed amplitude.
 *
 * This is a new Initial/ plugin (the reference ships no exact match; its
 * nearest relative is Initial/vortex.c).  It follows the reference plugin
 * contract `void initial(double *prim, double *x)` (Initial/vortex.c:6):
 * prim is filled in the reference's primitive order
 * {RHO, PPP, URR, UPP (angular velocity), UZZ, passive...} (paul.h:4).
 *
 * Vortex profile (Yee et al. 1999 isentropic vortex, lengths in units of
 * sigma):  s = |x - x0| / sigma,
 *    swirl speed     v = A s exp((1 - s^2)/2)
 *    temperature     T = 1 - (gamma-1)/(2 gamma) A^2 exp(1 - s^2)
 *    rho = T^(1/(gamma-1)),  P = rho T.
 * The passive scalar (if any) is exp(-s^2).
 *
 * Parameters (in.par):  Init_Par1 = Omega0, Init_Par2 = r0, Init_Par3 = phi0,
 * Init_Par4 = sigma, Init_Par5 = amplitude A;  gamma = Adiabatic_Index.
 *
 * Header-only so the same arithmetic is compiled for the host set-up, the
 * device boundary fill and the CPU checker.
 */
#ifndef DISCO_IC_VORTEX_GAUSS_H
#define DISCO_IC_VORTEX_GAUSS_H

#include <math.h>

#ifndef DISCO_HD
#ifdef __CUDACC__
#define DISCO_HD __host__ __device__
#else
#define DISCO_HD
#endif
#endif

struct disco_ic_vortex_gauss {
   double Omega0, r0, phi0, sigma, amp, gam;
};

DISCO_HD static inline void disco_ic_vortex_gauss_eval(
      const struct disco_ic_vortex_gauss *p, double *prim, const double *x,
      int num_c, int num_q)
{
   double r = x[0];
   double phi = x[1];
   double cp = cos(phi);
   double sp = sin(phi);
   double dx = r*cp - p->r0*cos(p->phi0);
   double dy = r*sp - p->r0*sin(p->phi0);
   double s2 = (dx*dx + dy*dy)/(p->sigma*p->sigma);
   double e = exp(0.5*(1.0 - s2));

   /* Cartesian swirl velocity (-dy, dx) * A e / sigma */
   double vx = -p->amp*e*dy/p->sigma;
   double vy =  p->amp*e*dx/p->sigma;
   double T = 1.0 - (p->gam - 1.0)/(2.0*p->gam)*p->amp*p->amp*e*e;
   double rho = pow(T, 1.0/(p->gam - 1.0));
   double P = rho*T;

   double vr = vx*cp + vy*sp;
   double vp = -vx*sp + vy*cp;

   prim[0] = rho;
   prim[1] = P;
   prim[2] = vr;
   prim[3] = p->Omega0 + vp/r;
   prim[4] = 0.0;
   int q;
   for(q = 5; q < num_c; q++) prim[q] = 0.0;
   for(q = num_c; q < num_q; q++) prim[q] = exp(-s2);
}

#endif
