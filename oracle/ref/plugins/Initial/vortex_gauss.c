/*
 * CHECKER INFRASTRUCTURE (oracle): Initial/ plugin for the reference build.
 * Implements the reference plugin contract setICparams()/initial()
 * (Initial/vortex.c:3-6) for the Gaussian-vortex synthetic input, using the
 * same header the product's host set-up uses, so both sides start from
 * identical primitives.
 */
#include "paul.h"
#include "../../../../disco_gb300/csrc/plugins/ic_vortex_gauss.h"

static struct disco_ic_vortex_gauss P;

void setICparams(struct domain *theDomain)
{
   P.Omega0 = theDomain->theParList.initPar1;
   P.r0     = theDomain->theParList.initPar2;
   P.phi0   = theDomain->theParList.initPar3;
   P.sigma  = theDomain->theParList.initPar4;
   P.amp    = theDomain->theParList.initPar5;
   P.gam    = theDomain->theParList.Adiabatic_Index;
}

void initial(double *prim, double *x)
{
   disco_ic_vortex_gauss_eval(&P, prim, x, NUM_C, NUM_Q);
}
