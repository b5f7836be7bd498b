/*
 * CHECKER INFRASTRUCTURE (oracle): Initial/ plugin for the reference build
 * (contract of Initial/torus_fm_grmhd.c: setICparams + initial) -- the
 * Fishbone-Moncrief torus in Kerr-Schild cylindrical coordinates, sharing
 * the product's initial-condition header.
 */
#include "paul.h"
#include "../../../../disco_gb300/csrc/plugins/ic_fm_torus.h"

static struct disco_ic_fm P;

void setICparams(struct domain *d)
{
   struct param_list *p = &d->theParList;
   P.gam = p->Adiabatic_Index; P.M = p->metricPar2; P.a = p->metricPar3;
   P.rin = p->initPar1; P.rpk = p->initPar2; P.beta = p->initPar3; P.acut = p->initPar4;
   P.rho_atm = p->Density_Floor; P.cs2_atm = p->Pressure_Floor;
   disco_ic_fm_setup(&P);
}

void initial(double *prim, double *x)
{
   disco_ic_fm_eval(&P, prim, x, NUM_C, NUM_Q);
}
