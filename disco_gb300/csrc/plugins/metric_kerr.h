/*
 * The Kerr metric (mass M, spin a) in Kerr-Schild cylindrical coordinates
 * (t, r, phi, z): a new Hydro/Metric plugin behind the reference's metric.h
 * hooks (metric_lapse, metric_shift, metric_gam, metric_igam,
 * metric_jacobian, metric_der_g, metric_der_lapse, metric_der_shift,
 * metric_killing; Hydro/metric.h:4-14).  The reference's nearest relative is
 * Hydro/Metric/schw_ks_rpz.c, the a = 0 case.
 *
 * Kerr-Schild form: g_mu,nu = eta_mu,nu + H l_mu l_nu with eta the flat
 * metric in cylindrical coordinates, diag(-1, 1, r^2, 1), and l a null
 * covector.  With x = r cos(phi), y = r sin(phi) the Cartesian Kerr-Schild
 * coordinates, the Boyer-Lindquist radius R(r, z) is the positive root of
 *     R^4 - (r^2 + z^2 - a^2) R^2 - a^2 z^2 = 0,
 * and
 *     H   = 2 M R^3 / (R^4 + a^2 z^2),
 *     l_mu = (1, R r / (R^2 + a^2), -a r^2 / (R^2 + a^2), z / R).
 * Since l is null, det g = det eta, so sqrt(-g) = r (metric_jacobian), and
 *     lapse  alpha = (1 + H)^-1/2,
 *     shift  beta^i = H l^i / (1 + H),   l^i = eta^ij l_j,
 *     gamma_ij = eta_ij + H l_i l_j,  gamma^ij = eta^ij - H l^i l^j / (1 + H).
 * The metric is stationary and axisymmetric: t and phi are Killing
 * directions, so only d/dr and d/dz of it are non-zero.
 *
 * Shared by the host set-up (initial conditions), the device (the GRMHD
 * hooks), and the reference-build plugin that pins the device to the
 * reference's own Hydro/grmhd.c evaluated on this metric.
 */
#ifndef DISCO_METRIC_KERR_H
#define DISCO_METRIC_KERR_H

#include <math.h>

#ifndef DISCO_HD
#ifdef __CUDACC__
#define DISCO_HD __host__ __device__
#else
#define DISCO_HD
#endif
#endif

/* One point of the metric: R, H, the null covector l_mu and the raised
 * spatial l^i, with their r and z derivatives when asked for. */
struct disco_kerr_pt {
   double R, H;
   double l[4];        /* l_mu, mu = t, r, phi, z */
   double lu[3];       /* l^i = eta^ij l_j, i = r, phi, z */
   double dR[2], dH[2];          /* d/dr, d/dz */
   double dl[2][4];              /* d l_mu / dr, d l_mu / dz */
   double dlu[2][3];             /* d l^i / dr, d l^i / dz */
};

DISCO_HD static inline double disco_kerr_R(double r, double z, double a)
{
   double b = r*r + z*z - a*a;
   return sqrt(0.5*(b + sqrt(b*b + 4.0*a*a*z*z)));
}

DISCO_HD static inline void disco_kerr_point(double r, double z, double M, double a, int derivs,
                                             struct disco_kerr_pt *p)
{
   double R = disco_kerr_R(r, z, a);
   double R2 = R*R, a2 = a*a;
   double Sig = R2*R2 + a2*z*z;
   double S2 = R2 + a2;
   p->R = R;
   p->H = 2.0*M*R2*R/Sig;
   p->l[0] = 1.0;
   p->l[1] = R*r/S2;
   p->l[2] = -a*r*r/S2;
   p->l[3] = z/R;
   p->lu[0] = p->l[1];
   p->lu[1] = -a/S2;
   p->lu[2] = p->l[3];
   if(!derivs) return;
   /* implicit differentiation of the quartic for R(r, z) */
   double dRdr = r*R2*R/Sig;
   double dRdz = z*R*S2/Sig;
   double dHdR = 2.0*M*R2*(3.0*a2*z*z - R2*R2)/(Sig*Sig);
   double dHdz_R = -4.0*M*a2*z*R2*R/(Sig*Sig);
   p->dR[0] = dRdr;
   p->dR[1] = dRdz;
   p->dH[0] = dHdR*dRdr;
   p->dH[1] = dHdR*dRdz + dHdz_R;
   double S22 = S2*S2;
   /* d/dr */
   p->dl[0][0] = 0.0;
   p->dl[0][1] = (R*S2 + r*dRdr*(a2 - R2))/S22;
   p->dl[0][2] = -a*(2.0*r*S2 - 2.0*r*r*R*dRdr)/S22;
   p->dl[0][3] = -z*dRdr/R2;
   /* d/dz */
   p->dl[1][0] = 0.0;
   p->dl[1][1] = r*dRdz*(a2 - R2)/S22;
   p->dl[1][2] = 2.0*a*r*r*R*dRdz/S22;
   p->dl[1][3] = (R - z*dRdz)/R2;
   for(int d = 0; d < 2; d++) {
      p->dlu[d][0] = p->dl[d][1];
      p->dlu[d][1] = 2.0*a*R*p->dR[d]/S22;
      p->dlu[d][2] = p->dl[d][3];
   }
}

/* lapse, shift beta^i, gamma_ij, gamma^ij (any pointer may be NULL) */
DISCO_HD static inline void disco_kerr_3p1(const double *x, double M, double a, double *al, double *be,
                                           double *gam, double *igam)
{
   struct disco_kerr_pt p;
   double r = x[0];
   disco_kerr_point(r, x[2], M, a, 0, &p);
   double H = p.H;
   double iH1 = 1.0/(1.0 + H);
   if(al) *al = sqrt(iH1);
   if(be) for(int i = 0; i < 3; i++) be[i] = H*p.lu[i]*iH1;
   const double eta[3] = {1.0, r*r, 1.0};
   const double ieta[3] = {1.0, 1.0/(r*r), 1.0};
   for(int i = 0; i < 3; i++)
      for(int j = 0; j < 3; j++) {
         if(gam) gam[3*i + j] = (i == j ? eta[i] : 0.0) + H*p.l[i + 1]*p.l[j + 1];
         if(igam) igam[3*i + j] = (i == j ? ieta[i] : 0.0) - H*p.lu[i]*p.lu[j]*iH1;
      }
}

/* d g_{mu nu} / d x^i, i = 0..3 (t, r, phi, z); zero for t and phi */
DISCO_HD static inline void disco_kerr_der_g(const double *x, double M, double a, int i, double *dg)
{
   for(int m = 0; m < 16; m++) dg[m] = 0.0;
   if(i != 1 && i != 3) return;
   struct disco_kerr_pt p;
   disco_kerr_point(x[0], x[2], M, a, 1, &p);
   int d = i == 1 ? 0 : 1;
   for(int mu = 0; mu < 4; mu++)
      for(int nu = 0; nu < 4; nu++)
         dg[4*mu + nu] = p.dH[d]*p.l[mu]*p.l[nu] + p.H*(p.dl[d][mu]*p.l[nu] + p.l[mu]*p.dl[d][nu]);
   if(i == 1) dg[10] += 2.0*x[0];   /* d(r^2)/dr of eta_phi,phi */
}

/* d alpha / d x^mu (mu = t, r, phi, z) */
DISCO_HD static inline void disco_kerr_der_lapse(const double *x, double M, double a, double *da)
{
   struct disco_kerr_pt p;
   disco_kerr_point(x[0], x[2], M, a, 1, &p);
   double al = 1.0/sqrt(1.0 + p.H);
   da[0] = 0.0;
   da[1] = -0.5*al*al*al*p.dH[0];
   da[2] = 0.0;
   da[3] = -0.5*al*al*al*p.dH[1];
}

/* d beta^j / d x^mu as db[3*mu + j] */
DISCO_HD static inline void disco_kerr_der_shift(const double *x, double M, double a, double *db)
{
   struct disco_kerr_pt p;
   disco_kerr_point(x[0], x[2], M, a, 1, &p);
   double iH1 = 1.0/(1.0 + p.H);
   double F = p.H*iH1;
   for(int m = 0; m < 12; m++) db[m] = 0.0;
   for(int d = 0; d < 2; d++) {
      int mu = d == 0 ? 1 : 3;
      double dF = p.dH[d]*iH1*iH1;
      for(int j = 0; j < 3; j++) db[3*mu + j] = dF*p.lu[j] + F*p.dlu[d][j];
   }
}

DISCO_HD static inline int disco_kerr_killing(int mu)
{
   return (mu == 1 || mu == 3) ? 0 : 1;
}

#endif
