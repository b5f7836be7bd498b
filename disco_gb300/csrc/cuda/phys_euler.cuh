// Newtonian hydro hooks of Hydro/euler.c, restated as device functions
// templated on the arithmetic type R (double for the plain path, float for
// the mixed path).  Same hook set as hydro.h:6-35: prim2cons, getUstar,
// cons2prim, flux, source, visc_flux, visc_source, vel, mindt.
#pragma once
#include "dev_common.cuh"

namespace disco {

template <typename R, int NQ>
struct Euler {
  static constexpr int NC = 5;
  static constexpr bool MHD = false;
  static constexpr bool GR = false;
  template <typename T>
  using Rebind = Euler<T, NQ>;

  // prim2cons, euler.c:37-63.  x = (r, phi, z); only r enters.
  // omf: angular velocity of the frame the velocities are given in (0 in
  // the lab frame); the energy frame get_om moves with it.
  template <typename T>
  DISCO_D static void prim2cons(const DevParams& P, const R* prim, T* cons, R r, R dV, R omf = 0) {
    R rho = prim[RHO], Pp = prim[PPP], vr = prim[URR];
    R vp = prim[UPP] * r, vz = prim[UZZ];
    R om = get_om<R>(P, r) - omf;
    R vp_off = vp - om * r;
    R v2 = vr * vr + vp_off * vp_off + vz * vz;
    R rhoe = Pp / (PRM(R, P, gamma_law) - (R)1.);
    cons[DDD] = rho * dV;
    cons[TAU] = ((R).5 * rho * v2 + rhoe) * dV;
    cons[SRR] = rho * vr * dV;
    cons[LLL] = r * rho * vp * dV;
    cons[SZZ] = rho * vz * dV;
#pragma unroll
    for (int q = NC; q < NQ; ++q) cons[q] = prim[q] * (R)cons[DDD];
  }

  // getUstar, euler.c:65-101 (HLLC star state).
  DISCO_D static void getUstar(const DevParams& P, const R* prim, R* Ustar, R r, R Sk, R Ss,
                               const R* n, const R* Bpack, R omf = 0) {
    R rho = prim[RHO], vr = prim[URR], vp = prim[UPP] * r, vz = prim[UZZ], Pp = prim[PPP];
    R om = get_om<R>(P, r) - omf;
    R vp_off = vp - om * r;
    R v2 = vr * vr + vp_off * vp_off + vz * vz;
    R vn = vr * n[0] + vp * n[1] + vz * n[2];
    R vn_off = vn - om * r * n[1];
    R Ss_off = Ss + vn_off - vn;
    R rhoe = Pp / (PRM(R, P, gamma_law) - (R)1.);
    R rhostar = rho * (Sk - vn) / (Sk - Ss);
    R Pstar = Pp * (Ss - vn) / (Sk - Ss);
    R Us = rhoe * (Sk - vn) / (Sk - Ss);
    Ustar[DDD] = rhostar;
    Ustar[SRR] = rhostar * (vr + (Ss - vn) * n[0]);
    Ustar[LLL] = r * rhostar * (vp + (Ss - vn) * n[1]);
    Ustar[SZZ] = rhostar * (vz + (Ss - vn) * n[2]);
    Ustar[TAU] = (R).5 * rhostar * v2 + Us + rhostar * Ss_off * (Ss - vn) + Pstar;
#pragma unroll
    for (int q = NC; q < NQ; ++q) Ustar[q] = prim[q] * Ustar[DDD];
  }

  // cons2prim, euler.c:103-140.  cons in FP64 (conserved accumulation),
  // prim in R.  Returns a floor-hit bit mask (1 = density, 2 = pressure).
  // Mixed path (R = float): the angular momentum is taken relative to the
  // ring frame Om in FP64 (Lsh = Om r^2), so prim[UPP] comes out as
  // omega - Om with the precision of the motion relative to that frame.
  DISCO_D static int cons2prim(const DevParams& P, const DevPlanet* pl, const double* cons, R* prim,
                               R r, R phi, R dV, double Lsh = 0, R Om = 0) {
    int hits = 0;
    R rho, Sr, Sp, Sz, E;
    R rr = (R)r;
    if (sizeof(R) < sizeof(double)) {   // mixed path: one reciprocal, FP32 products
      R idV = (R)1 / (R)dV;
      rho = to_r<R>(cons[DDD]) * idV; Sr = to_r<R>(cons[SRR]) * idV;
      Sp = to_r<R>(cons[LLL] - cons[DDD] * Lsh) * idV / rr;
      Sz = to_r<R>(cons[SZZ]) * idV; E = to_r<R>(cons[TAU]) * idV;
    } else {
      rho = (R)(cons[DDD] / dV); Sr = (R)(cons[SRR] / dV); Sp = (R)(cons[LLL] / dV / r);
      Sz = (R)(cons[SZZ] / dV); E = (R)(cons[TAU] / dV);
    }
    R rho0 = rho;
    if (rho < PRM(R, P, rho_floor)) { rho = PRM(R, P, rho_floor); hits |= 1; }
    R om = get_om<R>(P, rr);
    R vr = Sr / rho;
    R vp = Sp / rho;                       // relative to the frame
    if (rho != rho0) vp += Om * rr * (rho0 / rho - (R)1);
    R vp_off = vp + (Om - om) * rr;
    R vz = Sz / rho;
    R KE = (R).5 * (Sr * vr + rho * vp_off * vp_off + Sz * vz);
    R rhoe = E - KE;
    R Pp = (PRM(R, P, gamma_law) - (R)1.) * rhoe;
    if (Pp < PRM(R, P, p_floor) * rho) { Pp = PRM(R, P, p_floor) * rho; hits |= 2; }
    if (P.isothermal) {
      R cs2 = get_cs2<R>(P, pl, rr, (R)phi);
      Pp = cs2 * rho / PRM(R, P, gamma_law);
    }
    prim[RHO] = rho;
    prim[PPP] = Pp;
    prim[URR] = vr;
    prim[UPP] = vp / rr;
    prim[UZZ] = vz;
#pragma unroll
    for (int q = NC; q < NQ; ++q)
      prim[q] = sizeof(R) < sizeof(double) ? to_r<R>(cons[q]) / to_r<R>(cons[DDD]) : (R)(cons[q] / cons[DDD]);
    return hits;
  }

  // flux, euler.c:142-170.
  DISCO_D static void flux(const DevParams& P, const R* prim, R* f, R r, const R* n, R omf = 0) {
    R rho = prim[RHO], Pp = prim[PPP], vr = prim[URR], vp = prim[UPP] * r, vz = prim[UZZ];
    R om = get_om<R>(P, r) - omf;
    R vn = vr * n[0] + vp * n[1] + vz * n[2];
    R wn = om * r * n[1];
    R vp_off = vp - om * r;
    R rhoe = Pp / (PRM(R, P, gamma_law) - (R)1.);
    R v2 = vr * vr + vp_off * vp_off + vz * vz;
    f[DDD] = rho * vn;
    f[SRR] = rho * vr * vn + Pp * n[0];
    f[LLL] = r * (rho * vp * vn + Pp * n[1]);
    f[SZZ] = rho * vz * vn + Pp * n[2];
    f[TAU] = ((R).5 * rho * v2 + rhoe + Pp) * vn - Pp * wn;
#pragma unroll
    for (int q = NC; q < NQ; ++q) f[q] = prim[q] * f[DDD];
  }

  // vel, euler.c:301-326: HLLC wave-speed estimates.
  DISCO_D static void vel(const DevParams& P, const R* p1, const R* p2, R* Sl, R* Sr, R* Ss,
                          const R* n, R r, R* Bpack) {
    R P1 = p1[PPP], rho1 = p1[RHO];
    R vn1 = p1[URR] * n[0] + p1[UPP] * n[1] * r + p1[UZZ] * n[2];
    R cs1 = sqrt(PRM(R, P, gamma_law) * P1 / rho1);
    R P2 = p2[PPP], rho2 = p2[RHO];
    R vn2 = p2[URR] * n[0] + p2[UPP] * n[1] * r + p2[UZZ] * n[2];
    R cs2 = sqrt(PRM(R, P, gamma_law) * P2 / rho2);
    *Ss = (P2 - P1 + rho1 * vn1 * (-cs1) - rho2 * vn2 * cs2) / (rho1 * (-cs1) - rho2 * cs2);
    *Sr = cs1 + vn1;
    *Sl = -cs1 + vn1;
    if (*Sr < cs2 + vn2) *Sr = cs2 + vn2;
    if (*Sl > -cs2 + vn2) *Sl = -cs2 + vn2;
  }

  // source, euler.c:172-213 (geometric + energy-frame source).  T is the
  // accumulator type; r_1 = .5 (rp + rm), rc = centroid radius, dphi = cell
  // width (r23 is unused by this module).
  template <typename T>
  DISCO_D static void source(const DevParams& P, const R* prim, T* cons, T dVdt, R r_1, R r23,
                             R r, R dphi) {
    (void)r23;
    R rho = prim[RHO], Pp = prim[PPP];
    R vr = prim[URR], omega = prim[UPP], vz = prim[UZZ];
    R centrifugal = rho * omega * omega * r;
    if (P.polar_sources) centrifugal *= (R)(sin((R)0.5 * dphi) / ((R)0.5 * dphi));
    R press_bal = Pp / r_1;
    cons[SRR] += dVdt * (T)(centrifugal + press_bal);
    R om = get_om<R>(P, r);
    R om_r = get_om1<R>(P, r);
    R om_z = 0.0;
    cons[TAU] += (dVdt * (T)rho) * (T)(r * vr * om * om - r * r * (omega - om) * (vr * om_r + vz * om_z));
  }

  // nu for viscosity: explicit, or alpha c^2 / get_height_om (euler.c:220-226).
  DISCO_D static R visc_nu(const DevParams& P, const DevPlanet* pl, const R* prim, R r, R phi) {
    R nu = PRM(R, P, explicit_viscosity);
    if (P.alpha_flag) {
      R alpha = PRM(R, P, explicit_viscosity);
      R c2 = PRM(R, P, gamma_law) * prim[PPP] / prim[RHO];
      nu = alpha * c2 / get_height_om<R>(P, pl, r, phi);
    }
    return nu;
  }

  // visc_flux, euler.c:215-256.
  DISCO_D static void visc_flux(const DevParams& P, const DevPlanet* pl, const R* prim,
                                const R* gradr, const R* gradp, const R* gradz, R* f, R r,
                                R phi, const R* n, R omf = 0) {
    R nu = visc_nu(P, pl, prim, r, phi);
    R rho = prim[RHO], vr = prim[URR], om = prim[UPP];
    R om_off = om - (get_om<R>(P, r) - omf);
    R vz = prim[UZZ];
    R divV_o_d = (gradr[URR] + gradp[UPP] + gradz[UZZ] + vr / r) / (R)3.0;
    R srr = gradr[URR] - divV_o_d;
    R spp = r * (r * gradp[UPP] + vr - r * divV_o_d);
    R szz = gradz[UZZ] - divV_o_d;
    R srp = (R)0.5 * (r * r * gradr[UPP] + gradp[URR]);
    R srz = (R)0.5 * (gradr[UZZ] + gradz[URR]);
    R spz = (R)0.5 * (gradp[UZZ] + r * r * gradz[UPP]);
    R nc0 = n[0], nc1 = n[1] / r, nc2 = n[2];
    R srn = srr * nc0 + srp * nc1 + srz * nc2;
    R spn = srp * nc0 + spp * nc1 + spz * nc2;
    R szn = srz * nc0 + spz * nc1 + szz * nc2;
    f[SRR] = (R)-2 * nu * rho * srn;
    f[LLL] = (R)-2 * nu * rho * spn;
    f[SZZ] = (R)-2 * nu * rho * szn;
    f[TAU] = (R)-2 * nu * rho * (vr * srn + om_off * spn + vz * szn);
  }

  // visc_source, euler.c:258-291.
  DISCO_D static void visc_source(const DevParams& P, const DevPlanet* pl, const R* prim,
                                  const R* gradr, const R* gradp, const R* gradz, double* cons,
                                  const double* xp, const double* xm, double dVdt) {
    R r = (R)centroid_r(xp[0], xm[0]);
    R phi = (R)(0.5 * (xp[1] + xm[1]));
    R nu = visc_nu(P, pl, prim, r, phi);
    R rho = prim[RHO], vr = prim[URR];
    R divV_o_d = (gradr[URR] + gradp[UPP] + gradz[UZZ] + vr / r) / (R)3.0;
    R spp = (r * gradp[UPP] + vr - r * divV_o_d) / (r * r * r);
    cons[SRR] += (double)(((R)-2 * r * rho * nu * spp) * (R)dVdt);
    R srp = (R)0.5 * (r * r * gradr[UPP] + gradp[URR]);
    R spz = (R)0.5 * (gradp[UZZ] + r * r * gradz[UPP]);
    R om_r = get_om1<R>(P, r);
    R om_z = 0.0;
    cons[TAU] += (double)(((R)2 * rho * nu * (srp * om_r + spz * om_z)) * (R)dVdt);
  }

  // flux_to_E, euler.c:293-299: no magnetic field, nothing to do.
  DISCO_D static void flux_to_E(const R*, const R*, R, R*, R*, R*, R*, int) {}

  // HLLD is rejected for hydro at set-up (riemann.c:19-22); never reached.
  DISCO_D static void hlld(const DevParams&, R, const R*, const R*, R* F, R* U, R, const R*) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) { F[q] = 0; U[q] = 0; }
  }

  // Signal speeds of the CFL bound in R (mixed path): sp[0..2] =
  // cs + |v_r|, cs + |v_phi - w r|, cs + |v_z|; sp[3] = the explicit
  // viscosity nu, 0 without viscosity (euler.c:328-377).
  DISCO_D static void cfl_speeds_r(const DevParams& P, const DevPlanet* pl, const R* prim, R w, R r, R phi,
                                   R* sp) {
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (prim[UPP] - w) * r;
    R cs = sqrt(PRM(R, P, gamma_law) * Pp / rho);
    sp[0] = cs + fabs(prim[URR]);
    sp[1] = cs + fabs(vp);
    sp[2] = cs + fabs(prim[UZZ]);
    sp[3] = (R)0;
    if (P.include_viscosity) {
      R nu = PRM(R, P, explicit_viscosity);
      if (P.alpha_flag) {
        R c2 = PRM(R, P, gamma_law) * Pp / rho;
        nu = PRM(R, P, explicit_viscosity) * c2 / get_height_om<R>(P, pl, r, phi);
      }
      sp[3] = nu;
    }
  }

  // mindt of the mixed path: the same bound in R, with the cell extents
  // dL0 = r dphi, dL1 = dr, dL2 = dz given.
  DISCO_D static R mindt_r(const DevParams& P, const DevPlanet* pl, const R* prim, R w, R dL0, R dL1,
                           R dL2, R r, R phi) {
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (prim[UPP] - w) * r;
    R vr = prim[URR], vz = prim[UZZ];
    R cs = sqrt(PRM(R, P, gamma_law) * Pp / rho);
    R dt = dL1 / (cs + fabs(vr)), dtp = dL0 / (cs + fabs(vp)), dtz = dL2 / (cs + fabs(vz));
    if (dt > dtp) dt = dtp;
    if (dt > dtz) dt = dtz;
    if (P.include_viscosity) {
      R dx = dL0;
      if (dx > dL1) dx = dL1;
      if (dx > dL2) dx = dL2;
      R nu = PRM(R, P, explicit_viscosity);
      if (P.alpha_flag) {
        R c2 = PRM(R, P, gamma_law) * prim[PPP] / prim[RHO];
        nu = PRM(R, P, explicit_viscosity) * c2 / get_height_om<R>(P, pl, r, phi);
      }
      R dt_visc = (R)0.5 * dx * dx / nu;
      if (dt > dt_visc) dt = dt_visc;
    }
    return dt;
  }

  // mindt, euler.c:328-377.
  DISCO_D static double mindt(const DevParams& P, const DevPlanet* pl, const R* prim, double w,
                              const double* xp, const double* xm, double r) {
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (R)((double)prim[UPP] - w) * (R)r;
    R vr = prim[URR], vz = prim[UZZ];
    R cs = sqrt(PRM(R, P, gamma_law) * Pp / rho);
    R maxvr = cs + fabs(vr), maxvp = cs + fabs(vp), maxvz = cs + fabs(vz);
    double dL1 = xp[0] - xm[0];
    double dL0 = .5 * (xp[0] + xm[0]) * get_dp(xp[1], xm[1], P.phi_max);
    double dL2 = xp[2] - xm[2];
    double dtr, dtp, dtz;
    if (sizeof(R) < sizeof(double)) {
      dtr = (double)((R)dL1 / maxvr); dtp = (double)((R)dL0 / maxvp); dtz = (double)((R)dL2 / maxvz);
    } else {
      dtr = dL1 / (double)maxvr; dtp = dL0 / (double)maxvp; dtz = dL2 / (double)maxvz;
    }
    double dt = dtr;
    if (dt > dtp) dt = dtp;
    if (dt > dtz) dt = dtz;
    if (P.include_viscosity) {
      double dx = dL0;
      if (dx > dL1) dx = dL1;
      if (dx > dL2) dx = dL2;
      R nu = PRM(R, P, explicit_viscosity);
      if (P.alpha_flag) {
        R c2 = PRM(R, P, gamma_law) * prim[PPP] / prim[RHO];
        nu = PRM(R, P, explicit_viscosity) * c2 /
             get_height_om<R>(P, pl, (R)r, (R)(0.5 * (xp[1] + xm[1])));
      }
      double dt_visc = 0.5 * dx * dx / (double)nu;
      if (dt > dt_visc) dt = dt_visc;
    }
    return dt;
  }
};

}  // namespace disco
