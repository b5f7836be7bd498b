/*
 * Initial conditions "disk_mhd" and "disk_planet": new Initial/ plugins for
 * the Keplerian-disk synthetic inputs (the reference's nearest relatives are
 * Initial/kepler_mhd.c, Initial/flock.c and Initial/kepler.c).  Same plugin
 * contract as the reference: fill prim[] in {RHO, PPP, URR, UPP, UZZ,
 * [BRR, BPP, BZZ,] passive} order (paul.h:4) at x = (r, phi, z).
 *
 * Units: GM = 1, Keplerian v_K = r^-1/2, locally isothermal sound speed
 * c_s = v_K / Mach (the reference's Cs2_Profile 4 with M = 1, omega.c:157).
 *
 * disk_mhd:  rho = max(exp(-z^2 / (2 H^2)), rho_atm) with H = r / Mach,
 *            P = rho c_s^2 / gamma,  Omega^2 = r^-3 (1 - 1/Mach^2),
 *            net vertical field B_z = sqrt(2 P_mid / beta) (magnetic
 *            pressure B^2/2 as in Hydro/mhd.c:48-53), P_mid = c_s^2/gamma.
 * disk_planet: 2D, Sigma = r^-slope, P = Sigma c_s^2 / gamma,
 *            Omega^2 = r^-3 (1 - (slope + 1)/Mach^2).
 *
 * Parameters (in.par): Init_Par1 = rho_atm (disk_mhd) / slope (disk_planet),
 * Init_Par2 = beta (0 = no field), Init_Par3 = passive-scalar radius,
 * Init_Par4..6 reserved;  Mach_Number;  Adiabatic_Index.
 */
#ifndef DISCO_IC_DISKS_H
#define DISCO_IC_DISKS_H

#include <math.h>

#ifndef DISCO_HD
#ifdef __CUDACC__
#define DISCO_HD __host__ __device__
#else
#define DISCO_HD
#endif
#endif

struct disco_ic_disk {
   double gam, mach, par1, par2, par3, par4, par5, par6;
};

DISCO_HD static inline void disco_ic_disk_from_params(
      struct disco_ic_disk *P, double gam, double mach, double p1, double p2,
      double p3, double p4, double p5, double p6)
{
   P->gam = gam; P->mach = mach; P->par1 = p1; P->par2 = p2; P->par3 = p3;
   P->par4 = p4; P->par5 = p5; P->par6 = p6;
}

DISCO_HD static inline void disco_ic_disk_mhd_eval(
      const struct disco_ic_disk *P, double *prim, const double *x,
      int num_c, int num_q)
{
   double r = x[0];
   double z = x[2];
   double M2 = P->mach*P->mach;
   double cs2 = 1.0/(r*M2);
   double H = r/P->mach;
   double rho = exp(-0.5*z*z/(H*H));
   if(rho < P->par1) rho = P->par1;
   double Pp = rho*cs2/P->gam;
   double omega = sqrt((1.0 - 1.0/M2)/(r*r*r));
   double Bz = 0.0;
   if(P->par2 > 0.0) Bz = sqrt(2.0*(cs2/P->gam)/P->par2);

   prim[0] = rho;
   prim[1] = Pp;
   prim[2] = 0.0;
   prim[3] = omega;
   prim[4] = 0.0;
   if(num_c > 5) { prim[5] = 0.0; prim[6] = 0.0; prim[7] = Bz; }
   int q;
   for(q = num_c; q < num_q; q++) prim[q] = r < P->par3 ? 1.0 : 0.0;
}

DISCO_HD static inline void disco_ic_disk_planet_eval(
      const struct disco_ic_disk *P, double *prim, const double *x,
      int num_c, int num_q)
{
   double r = x[0];
   double M2 = P->mach*P->mach;
   double slope = P->par1;
   double cs2 = 1.0/(r*M2);
   double sig = pow(r, -slope);
   double Pp = sig*cs2/P->gam;
   double omega = sqrt((1.0 - (slope + 1.0)/M2)/(r*r*r));
   prim[0] = sig;
   prim[1] = Pp;
   prim[2] = 0.0;
   prim[3] = omega;
   prim[4] = 0.0;
   int q;
   for(q = 5; q < num_c; q++) prim[q] = 0.0;
   for(q = num_c; q < num_q; q++) prim[q] = r < P->par3 ? 1.0 : 0.0;
}

#endif
