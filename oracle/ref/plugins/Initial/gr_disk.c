/*
 * CHECKER INFRASTRUCTURE (oracle): Initial/ plugin for the reference build
 * (contract of Initial/flock_grmhd.c: setICparams + initial) for the thin
 * GRMHD disk synthetic input in Kerr-Schild cylindrical coordinates, using
 * the same header the product's host set-up and device boundary fill use.
 */
#include "paul.h"
#include "../../../../disco_gb300/csrc/plugins/ic_disks.h"

static struct disco_ic_gr_disk P;

void setICparams(struct domain *d)
{
   struct param_list *p = &d->theParList;
   P.gam = p->Adiabatic_Index;
   P.M = p->metricPar2;
   P.hr = p->initPar1;
   P.amp = p->initPar2;
   P.beta = p->initPar3;
   P.rpass = p->initPar4;
}

void initial(double *prim, double *x)
{
   disco_ic_gr_disk_eval(&P, prim, x, NUM_C, NUM_Q);
}
