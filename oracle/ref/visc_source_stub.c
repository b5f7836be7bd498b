/*
 * CHECKER INFRASTRUCTURE (oracle): Hydro/mhd.c defines no visc_source(),
 * which misc.c:586 references, so the reference MHD build does not link as
 * shipped.  This empty definition lets it link; it is only ever reached when
 * Use_Viscosity=1, which no MHD configuration here sets.
 */
void visc_source(const double *prim, const double *gradr, const double *gradp,
                 const double *gradz, double *cons, const double *xp,
                 const double *xm, double dVdt)
{
   (void)prim; (void)gradr; (void)gradp; (void)gradz; (void)cons;
   (void)xp; (void)xm; (void)dVdt;
}
