/*
 * CHECKER INFRASTRUCTURE (oracle): Initial/ plugin for the reference build
 * (contract of Initial/kepler.c) for the 3D circumbinary MHD disk synthetic
 * input, sharing the product's IC header.
 */
#include "paul.h"
#include "../../../../disco_gb300/csrc/plugins/ic_disks.h"

static struct disco_ic_disk P;

void setICparams(struct domain *d)
{
   struct param_list *p = &d->theParList;
   disco_ic_disk_from_params(&P, p->Adiabatic_Index, p->Disk_Mach, p->initPar1, p->initPar2,
                             p->initPar3, p->initPar4, p->initPar5, p->initPar6);
}

void initial(double *prim, double *x)
{
   disco_ic_disk_cbd_eval(&P, prim, x, NUM_C, NUM_Q);
}
