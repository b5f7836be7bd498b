/* Ghost-ring boundary plugins (Boundary/*.c) written as the per-side
 * primitives of boundary_functions.c that each plugin's boundary_trans
 * calls, in call order: the dim 1 (r) list, run when Nr > 1, then the
 * dim 2 (z) list, run when Nz > 1.
 *
 * Primitives (boundary_functions.c):
 *   FIXED      boundary_fixed_{rinn,rout,zbot,ztop}     :161-268  set_cell_init (:21)
 *   FIXED_Q    boundary_fixed_q_*                       :662-773  set_cell_init_q (:33) on the q mask
 *   FIXED_PHI  boundary_fixed_phi_*                     :774-913  set_cell_init where phi in [pa, pb)
 *   ZEROGRAD   boundary_zerograd_* (arg: diode)         :269-441  copy of the next ring inward
 *   REFLECT    boundary_reflect_*                       :442-621  copy of the mirror ring, normal velocity negated
 *   NOSLIP     boundary_noslip_*                        :914-1101 copy of the mirror ring, all velocities negated
 *   HORIZON    boundary_fixed_horizon                   :622-660  set_cell_init on every ring within
 *                                                                  R_HOR of the origin, which then leaves
 *                                                                  the CFL minimum (real = 0); arg 1: the
 *                                                                  cut-out of Boundary/horizon.c instead
 *   FIXED_MEAN (Boundary/horizon.c's own fixed sides)             initial() at the arithmetic-mean r, z
 *                                                                  and piph - dphi / 2
 *   HOLES      (Boundary/horizon_bin.c's two cut-outs)            the cells within 0.8 of x = +-5 back to
 *                                                                  initial(), and out of the CFL minimum
 * fixed.c and fixed3d.c keep their own kernel (they fill every ghost ring
 * of their dimensions from initial()).
 */
#ifndef DISCO_BC_PLUGINS_H
#define DISCO_BC_PLUGINS_H

#include <math.h>

#include "disco_gpu.h"

enum { DISCO_BCOP_FIXED = 0, DISCO_BCOP_FIXED_Q = 1, DISCO_BCOP_FIXED_PHI = 2,
       DISCO_BCOP_ZEROGRAD = 3, DISCO_BCOP_REFLECT = 4, DISCO_BCOP_NOSLIP = 5,
       DISCO_BCOP_HORIZON = 6, DISCO_BCOP_FIXED_MEAN = 7, DISCO_BCOP_HOLES = 8 };

#ifdef __CUDACC__
#define DISCO_BC_HD __host__ __device__
#else
#define DISCO_BC_HD
#endif
enum { DISCO_SIDE_RINN = 0, DISCO_SIDE_ROUT = 1, DISCO_SIDE_ZBOT = 2, DISCO_SIDE_ZTOP = 3 };

typedef struct disco_bc_op {
   int op, side;
   int arg;          /* ZEROGRAD: diode; FIXED_Q: bit mask of the primitives set */
   double pa, pb;    /* FIXED_PHI: the phi range */
} disco_bc_op;

#define DISCO_BC_MAX_OPS 8

/* boundary_fixed_horizon's ring test (boundary_functions.c:634-651, R_HOR
 * = 1 at :8): ring (j, k) is excised when its outer edge r_jph[j] and the
 * larger-|z| edge of its layer lie within R_HOR of the origin.  rj and zk
 * are indexed as the reference's r_jph and z_kph (rj[-1] is valid). */
#define DISCO_R_HOR 1.0
static inline int disco_bc_horizon_ring(const double *rj, const double *zk, int j, int k)
{
   double zm = zk[k - 1], zp = zk[k];
   double zo = fabs(zp) > fabs(zm) ? zp : zm;
   if(fabs(zo) > DISCO_R_HOR) return 0;
   double ro = rj[j];
   return sqrt(zo*zo + ro*ro) < DISCO_R_HOR;
}

/* Boundary/horizon.c's cut-out (:73-109): M = 1, cut = 0.7 * 2M; the
 * domain must reach inside the cut, then ring (j, k) is cut when the
 * smaller-|z| edge of its layer and its inner edge lie within it (in 2D,
 * the inner edge alone).  The reference's early exit from the j loop
 * changes nothing: the test only grows stricter with j. */
/* Boundary/horizon_bin.c (:24-31, :79-179): hole h (0, 1) of a binary of
 * total mass M = 1, separation a = 10, mass ratio q = 1 sits at x = a_h
 * (a_0 = q a / (1 + q), a_1 = -a / (1 + q)) with radius 0.8 * 2 M_h.  Ring
 * (j, k) is a candidate when the domain reaches the hole and the ring's
 * nearer edges lie within the cut; *rc and *zc receive those edges.  The
 * reference walks candidate rings cell by cell (disco_bc_hole_cell). */
DISCO_BC_HD static inline int disco_bc_hole_ring(const double *rj, const double *zk, int Nr, int Nz,
                                                 int j, int k, int h, double *rc, double *zc)
{
   const double M = 1.0, a = 1.0e1, q = 1.0;
   const double Mh = h == 0 ? M / (1 + q) : q * M / (1 + q);
   const double ah = h == 0 ? q * a / (1 + q) : -a / (1 + q);
   const double cut = 0.8 * (2 * Mh);
   /* the region test: hole 0 at r ~ a_0, hole 1 at r ~ -a_1 */
   const double s = h == 0 ? ah : -ah;
   if(!(rj[-1] < s + cut && rj[Nr - 1] > s - cut && zk[-1] < cut && zk[Nz - 1] > -cut)) return 0;
   double zp = zk[k], zm = zk[k - 1];
   double z = fabs(zp) < fabs(zm) ? zp : zm;
   if(fabs(z) > cut && Nz > 1) return 0;
   double rp = rj[j], rm = rj[j - 1];
   double r;
   if(h == 0) {
      r = fabs(rp - ah) < fabs(rm - ah) ? rp : rm;
      if(((r - ah)*(r - ah) + z*z > cut*cut && Nz > 1) || fabs(r - ah) > cut) return 0;
   } else {
      r = fabs(rp + ah) < fabs(rm + ah) ? rp : rm;
      if(((r + ah)*(r + ah) + z*z > cut*cut && Nz > 1) || fabs(r + ah) > cut) return 0;
   }
   *rc = r;
   *zc = z;
   return 1;
}
/* the cell test of a candidate ring: the point (rc, phi, zc) within the cut
 * of hole h (phi = piph - dphi / 2) */
DISCO_BC_HD static inline int disco_bc_hole_cell(double rc, double zc, int Nz, double phi, int h)
{
   const double M = 1.0, a = 1.0e1, q = 1.0;
   const double Mh = h == 0 ? M / (1 + q) : q * M / (1 + q);
   const double ah = h == 0 ? q * a / (1 + q) : -a / (1 + q);
   const double cut = 0.8 * (2 * Mh);
   double xc = rc * cos(phi), yc = rc * sin(phi);
   double d2 = Nz > 1 ? (xc - ah)*(xc - ah) + yc*yc + zc*zc : (xc - ah)*(xc - ah) + yc*yc;
   return d2 < cut*cut;
}

#define DISCO_HORIZON_CUT (0.7 * 2.0)
static inline int disco_bc_horizon_cut_ring(const double *rj, const double *zk, int Nz, int j, int k)
{
   const double cut = DISCO_HORIZON_CUT;
   if(!(rj[-1] < cut && zk[-1] < cut && zk[Nz - 1] > -cut)) return 0;
   double zp = zk[k], zm = zk[k - 1];
   double zc = fabs(zp) < fabs(zm) ? zp : zm;
   if(fabs(zc) > cut && Nz > 1) return 0;
   for(int jj = 0; jj <= j; jj++) {
      double rp = rj[jj], rm = rj[jj - 1];
      double rc = fabs(rp) < fabs(rm) ? rp : rm;
      if((rc*rc + zc*zc > cut*cut && Nz > 1) || rc > cut) return 0;
   }
   return 1;
}

static inline disco_bc_op disco_bc_mk(int op, int side, int arg)
{
   disco_bc_op o;
   o.op = op; o.side = side; o.arg = arg; o.pa = 0.0; o.pb = 0.0;
   return o;
}

/* Fills ops (DISCO_BC_MAX_OPS entries) for a plugin that is written as
 * primitives; returns the count, 0 for fixed / fixed3d (own kernel) and -1
 * for an unknown id.  UPP = 3 in the primitive order. */
static inline int disco_bc_plugin_ops(int boundary_id, disco_bc_op *o)
{
   const int upp = 1 << 3;
   int n = 0;
   switch(boundary_id) {
   case DISCO_BC_FIXED: case DISCO_BC_FIXED3D:
      return 0;
   case DISCO_BC_ZEROGRAD:        /* Boundary/zerograd.c */
   case DISCO_BC_OUTFLOW3D: {     /* Boundary/outflow3d.c: with the diode */
      int d = boundary_id == DISCO_BC_OUTFLOW3D;
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_RINN, d);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ROUT, d);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZBOT, d);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, d);
      return n;
   }
   case DISCO_BC_ZEROGRAD_OMK:    /* Boundary/zerograd_omk.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_RINN, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ROUT, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_RINN, upp);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_ROUT, upp);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZBOT, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, 1);
      return n;
   case DISCO_BC_ZEROGRAD_OMIN:   /* Boundary/zerograd_omIN.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_RINN, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_RINN, upp);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZBOT, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, 1);
      return n;
   case DISCO_BC_ACCRETE3D:       /* Boundary/accrete3d.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_RINN, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZTOP, 0);
      return n;
   case DISCO_BC_FIXRREFZ:        /* Boundary/fixRrefZ.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_RINN, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_ZTOP, 0);
      return n;
   case DISCO_BC_POLAR3D:         /* Boundary/polar3d.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZTOP, 0);
      return n;
   case DISCO_BC_POLAR:           /* Boundary/polar.c: initial() at (centroid r, piph - dphi/2,
                                     centroid z), which is set_cell_init_q's position, on every
                                     primitive; without subtract_omega (RotFrame is rejected) */
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_ROUT, 0xffff);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_ZBOT, 0xffff);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_Q, DISCO_SIDE_ZTOP, 0xffff);
      return n;
   case DISCO_BC_HORIZON3D:       /* Boundary/horizon3d.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_HORIZON, DISCO_SIDE_RINN, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZTOP, 0);
      return n;
   case DISCO_BC_HORIZON:         /* Boundary/horizon.c: the cut-out after each pass */
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_HORIZON, DISCO_SIDE_RINN, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ZTOP, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_HORIZON, DISCO_SIDE_ZBOT, 1);
      return n;
   case DISCO_BC_HORIZON_BIN:     /* Boundary/horizon_bin.c: the holes after each pass */
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_HOLES, DISCO_SIDE_RINN, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED_MEAN, DISCO_SIDE_ZTOP, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_HOLES, DISCO_SIDE_ZBOT, 0);
      return n;
   case DISCO_BC_FIXED_GAP:       /* Boundary/fixed_gap.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_RINN, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZBOT, 1);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, 1);
      return n;
   case DISCO_BC_TUBE:            /* Boundary/tube.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, 0);
      return n;
   case DISCO_BC_SURFACEGRAVBOX:  /* Boundary/surfaceGravBox.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_RINN, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_ROUT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_REFLECT, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ZTOP, 1);
      return n;
   case DISCO_BC_FLOWTHROUGH:     /* Boundary/flowthrough.c */
      o[n++] = disco_bc_mk(DISCO_BCOP_NOSLIP, DISCO_SIDE_RINN, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_ZEROGRAD, DISCO_SIDE_ROUT, 1);
      o[n] = disco_bc_mk(DISCO_BCOP_FIXED_PHI, DISCO_SIDE_ROUT, 0);
      o[n].pa = 0.3*M_PI; o[n].pb = 1.7*M_PI; n++;
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZBOT, 0);
      o[n++] = disco_bc_mk(DISCO_BCOP_FIXED, DISCO_SIDE_ZTOP, 0);
      return n;
   default:
      return -1;
   }
}

#endif
