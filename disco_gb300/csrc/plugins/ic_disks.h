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

/* splitmix64 (Steele, Lea, Flood 2014), for the seeded phases below. */
DISCO_HD static inline unsigned long long disco_splitmix64(unsigned long long x)
{
   unsigned long long z = x + 0x9E3779B97F4A7C15ULL;
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
   return z ^ (z >> 31);
}

/*
 * disk_cbd: 3D circumbinary MHD disk around a total mass 1.
 *   rho = max(r^-1 exp(-(r_cav/r)^n) exp(-z^2/(2H^2)) (1 + a dn(phi, r)), rho_atm),
 *   H = r/Mach, P = rho c_s^2 / gamma with c_s^2 = 1/(r Mach^2),
 *   Omega^2 = r^-3 (1 - 2/Mach^2), toroidal field B_phi = sqrt(2 P / beta).
 *   dn is a smooth seeded perturbation: the mean of cos(m phi + p_m) sin(m' ln r + q_m)
 *   over m = 1..8, with the phases p_m, q_m drawn by splitmix64 seeded m.
 * Parameters: Init_Par1 = r_cav, Init_Par2 = beta (0 = no field),
 * Init_Par3 = passive-scalar radius, Init_Par4 = cavity steepness n,
 * Init_Par5 = perturbation amplitude a, Init_Par6 = rho_atm.
 */
DISCO_HD static inline void disco_ic_disk_cbd_eval(
      const struct disco_ic_disk *P, double *prim, const double *x,
      int num_c, int num_q)
{
   double r = x[0], phi = x[1], z = x[2];
   double M2 = P->mach*P->mach;
   double cs2 = 1.0/(r*M2);
   double H = r/P->mach;
   double dn = 0.0;
   int m;
   for(m = 1; m <= 8; m++) {
      double pm = 6.283185307179586*(double)(disco_splitmix64((unsigned long long)m) >> 11)*0x1.0p-53;
      double qm = 6.283185307179586*(double)(disco_splitmix64((unsigned long long)(m + 100)) >> 11)*0x1.0p-53;
      dn += cos(m*phi + pm)*sin(3.0*m*log(r) + qm);
   }
   dn *= 0.125;
   double rho = exp(-pow(P->par1/r, P->par4))*exp(-0.5*z*z/(H*H))*(1.0 + P->par5*dn)/r;
   if(rho < P->par6) rho = P->par6;
   double Pp = rho*cs2/P->gam;
   double omega = sqrt((1.0 - 2.0/M2)/(r*r*r));
   double Bp = 0.0;
   if(P->par2 > 0.0) Bp = sqrt(2.0*Pp/P->par2);
   prim[0] = rho;
   prim[1] = Pp;
   prim[2] = 0.0;
   prim[3] = omega;
   prim[4] = 0.0;
   if(num_c > 5) { prim[5] = 0.0; prim[6] = Bp; prim[7] = 0.0; }
   int q;
   for(q = num_c; q < num_q; q++) prim[q] = r < P->par3 ? 1.0 : 0.0;
}

/*
 * gr_disk: a thin Keplerian GRMHD disk around a Schwarzschild black hole of
 * mass M, in Kerr-Schild cylindrical coordinates (t, r, phi, z) -- the
 * coordinates of the reference's Hydro/Metric/schw_ks_rpz.c, where
 * g = eta + H k k with H = 2M/R, R = sqrt(r^2 + z^2), k = (1, r/R, 0, z/R).
 *   rho  = max(exp(-z^2 / (2 h^2)), 1e-4),  h = hr r;
 *   P    = rho cs^2 / gam,  cs = hr sqrt(M / r);
 *   v^r  = amp sqrt(M / r) sin(3 phi),  v^phi = sqrt(M / r^3),  v^z = 0
 *          (coordinate velocities dx^i/dt);
 *   u^0 from g_{mu nu} u^mu u^nu = -1, l_i = u^0 (g_{i0} + g_{ij} v^j);
 *   prim = {rho, P, l_r, l_phi / r^2, l_z, 0, 0, Bz} with the vertical field
 *   Bz = sqrt(2 P(z = 0) / beta) (the module's B prim is sqrt(gamma) B^i),
 *   passive = 1 inside r < rpass.
 * Parameters: gam = Adiabatic_Index, M = Metric_Par2, hr = Init_Par1,
 * amp = Init_Par2, beta = Init_Par3, rpass = Init_Par4.
 */
struct disco_ic_gr_disk {
   double gam, M, hr, amp, beta, rpass;
};

DISCO_HD static inline void disco_ic_gr_disk_eval(
      const struct disco_ic_gr_disk *P, double *prim, const double *x,
      int num_c, int num_q)
{
   double r = x[0], phi = x[1], z = x[2];
   double M = P->M;
   double R2 = r*r + z*z;
   double R = sqrt(R2);
   double H = 2.0*M/R;
   double g00 = -1.0 + H;
   double g0r = H*r/R, g0z = H*z/R;
   double grr = 1.0 + H*r*r/R2, grz = H*r*z/R2, gzz = 1.0 + H*z*z/R2;
   double gpp = r*r;

   double vk = sqrt(M/r);
   double h = P->hr*r;
   double rho = exp(-0.5*z*z/(h*h));
   if(rho < 1.0e-4) rho = 1.0e-4;
   double cs2 = P->hr*P->hr*vk*vk;
   double Pp = rho*cs2/P->gam;
   double vr = P->amp*vk*sin(3.0*phi);
   double vp = vk/r;
   double vz = 0.0;

   double norm = g00 + 2.0*g0r*vr + 2.0*g0z*vz + grr*vr*vr + 2.0*grz*vr*vz
                 + gzz*vz*vz + gpp*vp*vp;
   double u0 = 1.0/sqrt(-norm);
   double lr = u0*(g0r + grr*vr + grz*vz);
   double lp = u0*gpp*vp;
   double lz = u0*(g0z + grz*vr + gzz*vz);

   prim[0] = rho;
   prim[1] = Pp;
   prim[2] = lr;
   prim[3] = lp/(r*r);
   prim[4] = lz;
   if(num_c > 5) {
      prim[5] = 0.0;
      prim[6] = 0.0;
      prim[7] = P->beta > 0.0 ? sqrt(2.0*cs2/P->gam/P->beta) : 0.0;
   }
   int q;
   for(q = num_c; q < num_q; q++) prim[q] = r < P->rpass ? 1.0 : 0.0;
}

#endif
