/*
 * CHECKER INFRASTRUCTURE (oracle): Hydro/Metric plugin for the reference
 * build -- the Kerr metric in Kerr-Schild cylindrical coordinates, behind
 * the reference's metric.h hooks (Hydro/metric.h:4-14), sharing the
 * product's metric header.  Metric_Par2 = M, Metric_Par3 = a (spin).
 */
#include "paul.h"
#include "Hydro/metric.h"
#include "../../../../../disco_gb300/csrc/plugins/metric_kerr.h"

static double M = 1.0;
static double a = 0.0;

void setMetricParams(struct domain *theDomain)
{
   M = theDomain->theParList.metricPar2;
   a = theDomain->theParList.metricPar3;
}

double metric_lapse(const double x[3])
{
   double al;
   disco_kerr_3p1(x, M, a, &al, 0, 0, 0);
   return al;
}

void metric_shift(const double x[3], double b[3])
{
   disco_kerr_3p1(x, M, a, 0, b, 0, 0);
}

void metric_gam(const double x[3], double gam[9])
{
   disco_kerr_3p1(x, M, a, 0, 0, gam, 0);
}

void metric_igam(const double x[3], double igam[9])
{
   disco_kerr_3p1(x, M, a, 0, 0, 0, igam);
}

double metric_jacobian(const double x[3])
{
   return x[0];
}

void metric_der_g(const double x[3], int i, double dg[16])
{
   disco_kerr_der_g(x, M, a, i, dg);
}

void metric_der_lapse(const double x[3], double da[4])
{
   disco_kerr_der_lapse(x, M, a, da);
}

void metric_der_shift(const double x[3], double db[12])
{
   disco_kerr_der_shift(x, M, a, db);
}

int metric_killing(int mu)
{
   return disco_kerr_killing(mu);
}
