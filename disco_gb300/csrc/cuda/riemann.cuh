// solve_riemann (riemann.c:216-320) as a device function templated on the
// hydro module.  Returns Flux - w U* (the quantity every caller scales by
// dA dt and scatters, riemann.c:314-317) and, for MHD, the star state used
// by flux_to_E.
#pragma once
#include "dev_common.cuh"

namespace disco {

template <typename Phys, typename R, int NQ>
DISCO_D void solve_riemann(const DevParams& P, const DevPlanet* pl, const R* primL, const R* primR,
                           const R* gLr, const R* gLp, const R* gLz, const R* gRr, const R* gRp,
                           const R* gRz, R r, R phi, const R* n, R w, R* Fw, R* Flux_out,
                           R* Ustr_out, R omf = 0) {
  R Flux[NQ], Ustr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) { Flux[q] = 0; Ustr[q] = 0; }

  if (P.riemann_solver == SOLVER_HLL || P.riemann_solver == SOLVER_HLLC ||
      P.riemann_solver == SOLVER_HLLC_DAMP) {
    R Sl, Sr, Ss;
    R Bpack[5];
    Phys::vel(P, primL, primR, &Sl, &Sr, &Ss, n, r, Bpack);
    if (w < Sl) {
      Phys::flux(P, primL, Flux, r, n, omf);
      Phys::template prim2cons<R>(P, primL, Ustr, r, (R)1.0, omf);
    } else if (w > Sr) {
      Phys::flux(P, primR, Flux, r, n, omf);
      Phys::template prim2cons<R>(P, primR, Ustr, r, (R)1.0, omf);
    } else {
      if (P.riemann_solver == SOLVER_HLL || (r < (R)0.1 && P.riemann_solver == SOLVER_HLLC_DAMP)) {
        R Fl[NQ], Fr[NQ], Ul[NQ], Ur[NQ];
        R aL = Sr, aR = -Sl;
        Phys::template prim2cons<R>(P, primL, Ul, r, (R)1.0, omf);
        Phys::template prim2cons<R>(P, primR, Ur, r, (R)1.0, omf);
        Phys::flux(P, primL, Fl, r, n, omf);
        Phys::flux(P, primR, Fr, r, n, omf);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          Flux[q] = (aL * Fl[q] + aR * Fr[q] + aL * aR * (Ul[q] - Ur[q])) / (aL + aR);
          Ustr[q] = (aR * Ul[q] + aL * Ur[q] + Fl[q] - Fr[q]) / (aL + aR);
        }
      } else {
        R Uk[NQ], Fk[NQ];
        if (w < Ss) {
          Phys::template prim2cons<R>(P, primL, Uk, r, (R)1.0, omf);
          Phys::getUstar(P, primL, Ustr, r, Sl, Ss, n, Bpack, omf);
          Phys::flux(P, primL, Fk, r, n, omf);
#pragma unroll
          for (int q = 0; q < NQ; ++q) Flux[q] = Fk[q] + Sl * (Ustr[q] - Uk[q]);
        } else {
          Phys::template prim2cons<R>(P, primR, Uk, r, (R)1.0, omf);
          Phys::getUstar(P, primR, Ustr, r, Sr, Ss, n, Bpack, omf);
          Phys::flux(P, primR, Fk, r, n, omf);
#pragma unroll
          for (int q = 0; q < NQ; ++q) Flux[q] = Fk[q] + Sr * (Ustr[q] - Uk[q]);
        }
      }
    }
  } else {
    Phys::hlld(P, w, primL, primR, Flux, Ustr, r, n);
  }

  if (P.include_viscosity) {
    R vFlux[NQ], prim[NQ], gr[NQ], gp[NQ], gz[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      prim[q] = (R).5 * (primL[q] + primR[q]);
      gr[q] = (R).5 * (gLr[q] + gRr[q]);
      gp[q] = (R).5 * (gLp[q] + gRp[q]);
      gz[q] = (R).5 * (gLz[q] + gRz[q]);
      vFlux[q] = 0.0;
    }
    Phys::visc_flux(P, pl, prim, gr, gp, gz, vFlux, r, phi, n, omf);
#pragma unroll
    for (int q = 0; q < NQ; ++q) Flux[q] += vFlux[q];
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) Fw[q] = Flux[q] - w * Ustr[q];
  if (Flux_out) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) { Flux_out[q] = Flux[q]; Ustr_out[q] = Ustr[q]; }
  }
}

// The HLL branch of solve_riemann (riemann.c:238-271) for the GR module,
// whose hooks take the face position x = (r, phi, z): Fw = Flux - w U*.
// No viscous flux and no EMFs (the GR module is built without viscosity
// and with cell-centred B).
template <typename Phys, int NQ>
DISCO_D void solve_riemann_gr(const DevParams& P, const double* primL, const double* primR, const double* x,
                              const double* n, double w, double* Fw) {
  double Flux[NQ], Ustr[NQ];
  double Sl, Sr;
  Phys::vel_x(P, primL, primR, &Sl, &Sr, n, x);
  if (w < Sl) {
    Phys::flux_x(P, primL, Flux, x, n);
    Phys::prim2cons_x(P, primL, Ustr, x, 1.0);
  } else if (w > Sr) {
    Phys::flux_x(P, primR, Flux, x, n);
    Phys::prim2cons_x(P, primR, Ustr, x, 1.0);
  } else {
    double Fl[NQ], Fr[NQ], Ul[NQ], Ur[NQ];
    const double aL = Sr, aR = -Sl;
    Phys::prim2cons_x(P, primL, Ul, x, 1.0);
    Phys::prim2cons_x(P, primR, Ur, x, 1.0);
    Phys::flux_x(P, primL, Fl, x, n);
    Phys::flux_x(P, primR, Fr, x, n);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      Flux[q] = (aL * Fl[q] + aR * Fr[q] + aL * aR * (Ul[q] - Ur[q])) / (aL + aR);
      Ustr[q] = (aR * Ul[q] + aL * Ur[q] + Fl[q] - Fr[q]) / (aL + aR);
    }
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) Fw[q] = Flux[q] - w * Ustr[q];
}

}  // namespace disco
