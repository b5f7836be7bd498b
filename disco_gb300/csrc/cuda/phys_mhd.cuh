// Newtonian MHD hooks of Hydro/mhd.c and the HLLD solver of hlld.c as device
// functions templated on the arithmetic type R.  Magnetic field primitives
// are B^r, B^phi (orthonormal), B^z; conserved B^r is scaled by 1/r
// (bfield_scale_factor, mhd.c:518).
#pragma once
#include "dev_common.cuh"

namespace disco {

template <typename R, int NQ>
struct Mhd {
  static constexpr int NC = 8;
  static constexpr bool MHD = true;
  static constexpr bool GR = false;
  template <typename T>
  using Rebind = Mhd<T, NQ>;

  // prim2cons, mhd.c:35-69
  template <typename T>
  DISCO_D static void prim2cons(const DevParams& P, const R* prim, T* cons, R r, R dV, R omf = 0) {
    R rho = prim[RHO], Pp = prim[PPP], vr = prim[URR], vp = prim[UPP] * r, vz = prim[UZZ];
    R om = get_om<R>(P, r) - omf;
    R vp_off = vp - om * r;
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R v2 = vr * vr + vp_off * vp_off + vz * vz;
    R B2 = Br * Br + Bp * Bp + Bz * Bz;
    R rhoe = Pp / (PRM(R, P, gamma_law) - (R)1.);
    cons[DDD] = rho * dV;
    cons[TAU] = ((R).5 * rho * v2 + rhoe + (R).5 * B2) * dV;
    cons[SRR] = rho * vr * dV;
    cons[LLL] = r * rho * vp * dV;
    cons[SZZ] = rho * vz * dV;
    cons[BRR] = Br * dV * ((R)1.0 / r);
    cons[BPP] = Bp * dV / r;
    cons[BZZ] = Bz * dV;
#pragma unroll
    for (int q = NC; q < NQ; ++q) cons[q] = prim[q] * (R)cons[DDD];
  }

  // cons2prim, mhd.c:138-185 (FP64 conserved in, R primitives out)
  // Mixed path: prim[UPP] relative to the ring frame Om (Lsh = Om r^2), as
  // in the hydro module.
  DISCO_D static int cons2prim(const DevParams& P, const DevPlanet* pl, const double* cons, R* prim,
                               R r, R phi, R dV, double Lsh = 0, R Om = 0) {
    int hits = 0;
    R rho, Sr, Sp, Sz, E, Br, Bp, Bz;
    R rr = (R)r;
    if (sizeof(R) < sizeof(double)) {   // mixed path: one reciprocal, FP32 products
      R idV = (R)1 / (R)dV;
      rho = to_r<R>(cons[DDD]) * idV; Sr = to_r<R>(cons[SRR]) * idV;
      Sp = to_r<R>(cons[LLL] - cons[DDD] * Lsh) * idV / rr;
      Sz = to_r<R>(cons[SZZ]) * idV; E = to_r<R>(cons[TAU]) * idV;
      Br = to_r<R>(cons[BRR]) * idV * rr; Bp = to_r<R>(cons[BPP]) * idV * rr; Bz = to_r<R>(cons[BZZ]) * idV;
    } else {
      rho = (R)(cons[DDD] / dV); Sr = (R)(cons[SRR] / dV); Sp = (R)(cons[LLL] / dV / r);
      Sz = (R)(cons[SZZ] / dV); E = (R)(cons[TAU] / dV);
      Br = (R)(cons[BRR] / (dV * (1.0 / r))); Bp = (R)(cons[BPP] / dV * r); Bz = (R)(cons[BZZ] / dV);
    }
    R rho0 = rho;
    if (rho < PRM(R, P, rho_floor)) { rho = PRM(R, P, rho_floor); hits |= 1; }
    R om = get_om<R>(P, rr);
    R vr = Sr / rho, vp = Sp / rho, vz = Sz / rho;   // vp relative to the frame
    if (rho != rho0) vp += Om * rr * (rho0 / rho - (R)1);
    R vp_off = vp + (Om - om) * rr;
    R B2 = Br * Br + Bp * Bp + Bz * Bz;
    R KE = (R).5 * (Sr * vr + rho * vp_off * vp_off + Sz * vz);
    R rhoe = E - KE - (R).5 * B2;
    R Pp = (PRM(R, P, gamma_law) - (R)1.) * rhoe;
    if (Pp < PRM(R, P, p_floor) * rho) { Pp = PRM(R, P, p_floor) * rho; hits |= 2; }
    if (P.isothermal) {
      R cs2 = get_cs2<R>(P, pl, rr, (R)phi);
      Pp = cs2 * rho / PRM(R, P, gamma_law);
    }
    prim[RHO] = rho; prim[PPP] = Pp; prim[URR] = vr; prim[UPP] = vp / rr; prim[UZZ] = vz;
    prim[BRR] = Br; prim[BPP] = Bp; prim[BZZ] = Bz;
#pragma unroll
    for (int q = NC; q < NQ; ++q)
      prim[q] = sizeof(R) < sizeof(double) ? to_r<R>(cons[q]) / to_r<R>(cons[DDD]) : (R)(cons[q] / cons[DDD]);
    return hits;
  }

  // flux, mhd.c:187-223
  // (omf is accepted for the common hook signature: this flux has no energy frame)
  DISCO_D static void flux(const DevParams& P, const R* prim, R* f, R r, const R* n, R omf = 0) {
    (void)omf;
    R rho = prim[RHO], Pp = prim[PPP], vr = prim[URR], vp = prim[UPP] * r, vz = prim[UZZ];
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R vn = vr * n[0] + vp * n[1] + vz * n[2];
    R Bn = Br * n[0] + Bp * n[1] + Bz * n[2];
    R vB = vr * Br + vp * Bp + vz * Bz;
    R rhoe = Pp / (PRM(R, P, gamma_law) - (R)1.);
    R v2 = vr * vr + vp * vp + vz * vz;
    R B2 = Br * Br + Bp * Bp + Bz * Bz;
    f[DDD] = rho * vn;
    f[SRR] = rho * vr * vn + (Pp + (R).5 * B2) * n[0] - Br * Bn;
    f[LLL] = r * (rho * vp * vn + (Pp + (R).5 * B2) * n[1] - Bp * Bn);
    f[SZZ] = rho * vz * vn + (Pp + (R).5 * B2) * n[2] - Bz * Bn;
    f[TAU] = ((R).5 * rho * v2 + rhoe + Pp + B2) * vn - vB * Bn;
    f[BRR] = (Br * vn - vr * Bn) * ((R)1.0 / r);
    f[BPP] = (Bp * vn - vp * Bn) / r;
    f[BZZ] = Bz * vn - vz * Bn;
#pragma unroll
    for (int q = NC; q < NQ; ++q) f[q] = prim[q] * f[DDD];
  }

  // source, mhd.c:225-262.  T is the accumulator type (FP64 conserved
  // state, or the R sum of the mixed path); r_1 = .5 (rp + rm),
  // r23 = (rp^2 + rp rm + rm^2) / 3, rc = centroid radius, dphi = cell width.
  template <typename T>
  DISCO_D static void source(const DevParams& P, const R* prim, T* cons, T dVdt, R r_1, R r2_3,
                             R r, R dphi) {
    R rho = prim[RHO], Pp = prim[PPP];
    R vr = prim[URR], omega = prim[UPP];
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R B2 = Br * Br + Bp * Bp + Bz * Bz;
    R centrifugal;
    if (P.polar_sources) {
      centrifugal = (rho * omega * omega * r2_3) / r_1 * (R)sin((R).5 * dphi) / (R)((R).5 * dphi);
      centrifugal -= Bp * Bp / r_1;
    } else {
      centrifugal = rho * omega * omega * r - Bp * Bp / r;
    }
    R press_bal = (Pp + (R).5 * B2) / r_1;
    cons[SRR] += dVdt * (T)(centrifugal + press_bal);
    R om = get_om<R>(P, r), om1 = get_om1<R>(P, r);
    cons[TAU] += ((dVdt * (T)rho) * (T)vr) * (T)(om * om * r2_3 / r_1 - om1 * (omega - om) * r2_3);
    if (P.include_viscosity)
      cons[SRR] += -dVdt * (T)P.explicit_viscosity * (T)rho * (T)vr / (T)(r_1 * r_1);
  }

  // mhd.c defines neither visc_flux nor visc_source with content.
  DISCO_D static void visc_flux(const DevParams&, const DevPlanet*, const R*, const R*, const R*,
                                const R*, R*, R, R, const R*, R = 0) {}
  DISCO_D static void visc_source(const DevParams&, const DevPlanet*, const R*, const R*, const R*,
                                  const R*, double*, const double*, const double*, double) {}

  // flux_to_E, mhd.c:293-316: edge EMFs from the face flux / star state.
  DISCO_D static void flux_to_E(const R* Flux, const R* Ustr, R r, R* E1, R* B1, R* E2, R* B2,
                                int dim) {
    R irfac = (R)1.0 / ((R)1.0 / r);
    if (dim == 0) {
      *E1 = Flux[BRR] * irfac; *B1 = Ustr[BRR] * irfac; *E2 = -Flux[BZZ]; *B2 = Ustr[BZZ];
    } else if (dim == 1) {
      *E1 = -Flux[BPP] * r; *B1 = Ustr[BRR] * irfac; *E2 = Flux[BZZ];
    } else {
      *E1 = Flux[BPP] * r; *B1 = Ustr[BZZ]; *E2 = -Flux[BRR] * irfac;
    }
  }

  // ---- mhd.c's HLL/HLLC hooks (FP64 path; the mixed path rejects these
  // solvers at set-up) ----------------------------------------------------
  // vel (mhd.c:318-450): fast magnetosonic bounds of both states, the
  // contact speed from the total-pressure balance, and in Bpack the HLL
  // average of B (normal, r, phi, z) and v.B for the star state.
  DISCO_D static void vel(const DevParams& P, const R* p1, const R* p2, R* Sl, R* Sr, R* Ss, const R* n,
                          R r, R* Bpack) {
    const R gam = PRM(R, P, gamma_law);
    const R* pp[2] = {p1, p2};
    R v[2][3], B[2][3], rho[2], Pr[2], vn[2], Bn[2], B2[2], cf[2], m[2][3], Fm[2][3], FB[2][3];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const R* p = pp[s];
      rho[s] = p[RHO]; Pr[s] = p[PPP];
      v[s][0] = p[URR]; v[s][1] = r * p[UPP]; v[s][2] = p[UZZ];
      B[s][0] = p[BRR]; B[s][1] = p[BPP]; B[s][2] = p[BZZ];
      vn[s] = v[s][0] * n[0] + v[s][1] * n[1] + v[s][2] * n[2];
      Bn[s] = B[s][0] * n[0] + B[s][1] * n[1] + B[s][2] * n[2];
      B2[s] = B[s][0] * B[s][0] + B[s][1] * B[s][1] + B[s][2] * B[s][2];
      R cs = sqrt(gam * (Pr[s] / rho[s])), b2 = B2[s] / rho[s];
      R a = cs * cs + b2;
      cf[s] = (R).5 * (cs * cs + b2 + sqrt(fabs(a * a - (R)4.0 * cs * cs * Bn[s] * Bn[s] / rho[s])));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        FB[s][c] = vn[s] * B[s][c] - Bn[s] * v[s][c];
        m[s][c] = rho[s] * v[s][c];
        Fm[s][c] = rho[s] * v[s][c] * vn[s] + (Pr[s] + (R).5 * B2[s]) * n[c] - B[s][c] * Bn[s];
      }
    }
    R Lm = vn[0] - sqrt(cf[0]), Lp = vn[0] + sqrt(cf[0]);
    if (Lm > vn[1] - sqrt(cf[1])) Lm = vn[1] - sqrt(cf[1]);
    if (Lp < vn[1] + sqrt(cf[1])) Lp = vn[1] + sqrt(cf[1]);
    const R aL = Lp, aR = -Lm;
    R Bh[3], mh[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Bh[c] = (aR * B[0][c] + aL * B[1][c] + FB[0][c] - FB[1][c]) / (aL + aR);
      mh[c] = (aR * m[0][c] + aL * m[1][c] + Fm[0][c] - Fm[1][c]) / (aL + aR);
    }
    R Bnh = Bh[0] * n[0] + Bh[1] * n[1] + Bh[2] * n[2];
    R mnL = m[0][0] * n[0] + m[0][1] * n[1] + m[0][2] * n[2];
    R mnR = m[1][0] * n[0] + m[1][1] * n[1] + m[1][2] * n[2];
    R rhoh = (aR * rho[0] + aL * rho[1] + mnL - mnR) / (aL + aR);
    *Ss = (rho[1] * vn[1] * (Lp - vn[1]) - rho[0] * vn[0] * (Lm - vn[0]) +
           (Pr[0] + (R).5 * B2[0] - Bn[0] * Bn[0]) - (Pr[1] + (R).5 * B2[1] - Bn[1] * Bn[1])) /
          (rho[1] * (Lp - vn[1]) - rho[0] * (Lm - vn[0]));
    R vh0 = mh[0] / rhoh, vh1 = mh[1] / rhoh, vh2 = mh[2] / rhoh;
    Bpack[0] = Bnh; Bpack[1] = Bh[0]; Bpack[2] = Bh[1]; Bpack[3] = Bh[2];
    Bpack[4] = vh0 * Bh[0] + vh1 * Bh[1] + vh2 * Bh[2];
    *Sl = Lm;
    *Sr = Lp;
  }
  // getUstar (mhd.c:71-137): the HLLC star state of the side with wave
  // speed Sk and contact Ss, with the HLL field Bpack of vel
  DISCO_D static void getUstar(const DevParams& P, const R* prim, R* Us, R r, R Sk, R Ss, const R* n,
                               const R* Bpack, R = 0) {
    const R gam = PRM(R, P, gamma_law);
    const R Bsn = Bpack[0], Bs[3] = {Bpack[1], Bpack[2], Bpack[3]}, vBs = Bpack[4];
    const R rho = prim[RHO], Pp = prim[PPP];
    const R v[3] = {prim[URR], prim[UPP] * r, prim[UZZ]};
    const R B[3] = {prim[BRR], prim[BPP], prim[BZZ]};
    R v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    R vn = v[0] * n[0] + v[1] * n[1] + v[2] * n[2], Bn = B[0] * n[0] + B[1] * n[1] + B[2] * n[2];
    R vB = v[0] * B[0] + v[1] * B[1] + v[2] * B[2];
    R E = (R).5 * rho * v2 + Pp / (gam - (R)1.) + (R).5 * B2;
    R Bs2 = Bs[0] * Bs[0] + Bs[1] * Bs[1] + Bs[2] * Bs[2];
    R Ps = rho * (Sk - vn) * (Ss - vn) + (Pp + (R).5 * B2 - Bn * Bn) - (R).5 * Bs2 + Bsn * Bsn;
    R Ds = (Sk - vn) * rho / (Sk - Ss);
    R Ms[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const R mc = rho * v[c];
      Ms[c] = ((Sk - vn) * mc + (B[c] * Bn - Bs[c] * Bsn)) / (Sk - Ss);
    }
    R Es = ((Sk - vn) * E + (Ps + (R).5 * Bs2) * Ss - (Pp + (R).5 * B2) * vn - vBs * Bsn + vB * Bn) / (Sk - Ss);
    R Msn = Ds * Ss, mn = Ms[0] * n[0] + Ms[1] * n[1] + Ms[2] * n[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) Ms[c] += n[c] * (Msn - mn);
    Us[DDD] = Ds; Us[SRR] = Ms[0]; Us[LLL] = r * Ms[1]; Us[SZZ] = Ms[2]; Us[TAU] = Es;
    Us[BRR] = Bs[0] * ((R)1.0 / r);   // bfield_scale_factor(r, 0) = 1 / r (mhd.c:518)
    Us[BPP] = Bs[1] / r;
    Us[BZZ] = Bs[2];
#pragma unroll
    for (int q = 8; q < NQ; ++q) Us[q] = prim[q] * Us[DDD];
  }

  // ---- hlld.c ----------------------------------------------------------------
  DISCO_D static void h_velocities(R gam, const R* pL, const R* pR, const R* n, R* vel, R* Pt_star) {
    R rho_L = pL[RHO], P_L = pL[PPP];
    R u_L = pL[URR] * n[0] + pL[UPP] * n[1] + pL[UZZ] * n[2];
    R Bn_L = pL[BRR] * n[0] + pL[BPP] * n[1] + pL[BZZ] * n[2];
    R B2_L = pL[BRR] * pL[BRR] + pL[BPP] * pL[BPP] + pL[BZZ] * pL[BZZ];
    R Pt_L = P_L + (R).5 * B2_L;
    R rho_R = pR[RHO], P_R = pR[PPP];
    R u_R = pR[URR] * n[0] + pR[UPP] * n[1] + pR[UZZ] * n[2];
    R Bn_R = pR[BRR] * n[0] + pR[BPP] * n[1] + pR[BZZ] * n[2];
    R B2_R = pR[BRR] * pR[BRR] + pR[BPP] * pR[BPP] + pR[BZZ] * pR[BZZ];
    R Pt_R = P_R + (R).5 * B2_R;
    R Bn = (R).5 * (Bn_L + Bn_R);
    R aL = gam * P_L + B2_L, aR = gam * P_R + B2_R;
    R cf2_L = (R).5 * (gam * P_L + B2_L + sqrt(fabs(aL * aL - (R)4. * gam * P_L * Bn_L * Bn_L))) / rho_L;
    R cf2_R = (R).5 * (gam * P_R + B2_R + sqrt(fabs(aR * aR - (R)4. * gam * P_R * Bn_R * Bn_R))) / rho_R;
    R cf2 = cf2_L > cf2_R ? cf2_L : cf2_R;
    R umin, umax;
    if (u_L < u_R) { umin = u_L; umax = u_R; } else { umin = u_R; umax = u_L; }
    R S_R = umax + sqrt(fabs(cf2));
    R S_L = umin - sqrt(fabs(cf2));
    R S_M = ((S_R - u_R) * rho_R * u_R - (S_L - u_L) * rho_L * u_L - Pt_R + Pt_L) /
            ((S_R - u_R) * rho_R - (S_L - u_L) * rho_L);
    R rhostar_L = rho_L * (S_L - u_L) / (S_L - S_M);
    R rhostar_R = rho_R * (S_R - u_R) / (S_R - S_M);
    vel[0] = S_L;
    vel[1] = S_M - fabs(Bn) / sqrt(rhostar_L);
    vel[2] = S_M;
    vel[3] = S_M + fabs(Bn) / sqrt(rhostar_R);
    vel[4] = S_R;
    R num = (S_R - u_R) * rho_R * Pt_L - (S_L - u_L) * rho_L * Pt_R +
            rho_L * rho_R * (S_R - u_R) * (S_L - u_L) * (u_R - u_L);
    R denom = (S_R - u_R) * rho_R - (S_L - u_L) * rho_L;
    *Pt_star = num / denom;
  }
  DISCO_D static void h_prim_to_cons(R gam, const R* p, R* c) {
    R rho = p[RHO], Pp = p[PPP], vx = p[URR], vy = p[UPP], vz = p[UZZ];
    R Bx = p[BRR], By = p[BPP], Bz = p[BZZ];
    R v2 = vx * vx + vy * vy + vz * vz;
    R rhoe = Pp / (gam - (R)1.);
    R B2 = Bx * Bx + By * By + Bz * Bz;
    c[DDD] = rho; c[SRR] = rho * vx; c[LLL] = rho * vy; c[SZZ] = rho * vz;
    c[TAU] = ((R).5 * rho * v2 + rhoe + (R).5 * B2);
    c[BRR] = Bx; c[BPP] = By; c[BZZ] = Bz;
  }
  DISCO_D static void h_flux(R gam, const R* p, R* f, const R* n) {
    R rho = p[RHO], Pp = p[PPP], vx = p[URR], vy = p[UPP], vz = p[UZZ];
    R Bx = p[BRR], By = p[BPP], Bz = p[BZZ];
    R v2 = vx * vx + vy * vy + vz * vz;
    R vB = vx * Bx + vy * By + vz * Bz;
    R B2 = Bx * Bx + By * By + Bz * Bz;
    R vn = vx * n[0] + vy * n[1] + vz * n[2];
    R Bn = Bx * n[0] + By * n[1] + Bz * n[2];
    R rhoe = Pp / (gam - (R)1.);
    f[DDD] = rho * vn;
    f[SRR] = rho * vx * vn + (Pp + (R).5 * B2) * n[0] - Bx * Bn;
    f[LLL] = rho * vy * vn + (Pp + (R).5 * B2) * n[1] - By * Bn;
    f[SZZ] = rho * vz * vn + (Pp + (R).5 * B2) * n[2] - Bz * Bn;
    f[TAU] = ((R).5 * rho * v2 + rhoe + Pp + B2) * vn - vB * Bn;
    f[BRR] = Bx * vn - vx * Bn;
    f[BPP] = By * vn - vy * Bn;
    f[BZZ] = Bz * vn - vz * Bn;
  }
  DISCO_D static void h_single_star(R gam, const R* p, R* Us, R S_K, R S_M, R Pt_star, const R* n) {
    R rho = p[RHO], vx = p[URR], vy = p[UPP], vz = p[UZZ], Pp = p[PPP];
    R Bx = p[BRR], By = p[BPP], Bz = p[BZZ];
    R u_K = vx * n[0] + vy * n[1] + vz * n[2];
    R Bn = Bx * n[0] + By * n[1] + Bz * n[2];
    R vdotB = vx * Bx + vy * By + vz * Bz;
    R v2 = vx * vx + vy * vy + vz * vz;
    R B2 = Bx * Bx + By * By + Bz * Bz;
    R Pt = Pp + (R).5 * B2;
    R e = (R).5 * rho * v2 + Pp / (gam - (R)1.) + (R).5 * B2;
    R rhostar = rho * (S_K - u_K) / (S_K - S_M);
    R denom = rho * (S_K - u_K) * (S_K - S_M) - Bn * Bn;
    if (fabs(denom) < (R)1e-10) denom = (R)1e-10;   // hlld.c:12 TOL
    R vx_s = vx - Bn * Bx * (S_M - u_K) / denom;
    R vy_s = vy - Bn * By * (S_M - u_K) / denom;
    R vz_s = vz - Bn * Bz * (S_M - u_K) / denom;
    R sq = (S_K - u_K) * (S_K - u_K);
    R Bx_s = Bx * (rho * sq - Bn * Bn) / denom;
    R By_s = By * (rho * sq - Bn * Bn) / denom;
    R Bz_s = Bz * (rho * sq - Bn * Bn) / denom;
    R vn_s = vx_s * n[0] + vy_s * n[1] + vz_s * n[2];
    R Bn_s = Bx_s * n[0] + By_s * n[1] + Bz_s * n[2];
    vx_s += (S_M - vn_s) * n[0]; vy_s += (S_M - vn_s) * n[1]; vz_s += (S_M - vn_s) * n[2];
    Bx_s += (Bn - Bn_s) * n[0]; By_s += (Bn - Bn_s) * n[1]; Bz_s += (Bn - Bn_s) * n[2];
    R vB_s = vx_s * Bx_s + vy_s * By_s + vz_s * Bz_s;
    R e_s = ((S_K - u_K) * e - Pt * u_K + Pt_star * S_M + Bn * (vdotB - vB_s)) / (S_K - S_M);
    Us[DDD] = rhostar; Us[SRR] = rhostar * vx_s; Us[LLL] = rhostar * vy_s; Us[SZZ] = rhostar * vz_s;
    Us[TAU] = e_s; Us[BRR] = Bx_s; Us[BPP] = By_s; Us[BZZ] = Bz_s;
  }
  DISCO_D static void h_double_star(const R* UsL, const R* UsR, R* Uss, const R* vel, const R* n, int LR) {
    R rho_L = UsL[DDD], rho_R = UsR[DDD];
    R rhostar_K = LR == 0 ? rho_L : rho_R;
    R rrh_L = sqrt(rho_L), rrh_R = sqrt(rho_R), rrh_K = sqrt(rhostar_K);
    R vx_L = UsL[SRR] / rho_L, vy_L = UsL[LLL] / rho_L, vz_L = UsL[SZZ] / rho_L;
    R Bx_L = UsL[BRR], By_L = UsL[BPP], Bz_L = UsL[BZZ];
    R vx_R = UsR[SRR] / rho_R, vy_R = UsR[LLL] / rho_R, vz_R = UsR[SZZ] / rho_R;
    R Bx_R = UsR[BRR], By_R = UsR[BPP], Bz_R = UsR[BZZ];
    R Bn_L = Bx_L * n[0] + By_L * n[1] + Bz_L * n[2];
    R Bn_R = Bx_R * n[0] + By_R * n[1] + Bz_R * n[2];
    R Bn = (R).5 * (Bn_L + Bn_R);
    R sB = Bn > (R)0.0 ? (R)1.0 : (R)-1.0;
    R den = rrh_L + rrh_R;
    R vx = (rrh_L * vx_L + rrh_R * vx_R + (Bx_R - Bx_L) * sB) / den;
    R vy = (rrh_L * vy_L + rrh_R * vy_R + (By_R - By_L) * sB) / den;
    R vz = (rrh_L * vz_L + rrh_R * vz_R + (Bz_R - Bz_L) * sB) / den;
    R vn = vx * n[0] + vy * n[1] + vz * n[2];
    vx += (vel[2] - vn) * n[0]; vy += (vel[2] - vn) * n[1]; vz += (vel[2] - vn) * n[2];
    R Bx = (rrh_L * Bx_R + rrh_R * Bx_L + rrh_L * rrh_R * (vx_R - vx_L) * sB) / den;
    R By = (rrh_L * By_R + rrh_R * By_L + rrh_L * rrh_R * (vy_R - vy_L) * sB) / den;
    R Bz = (rrh_L * Bz_R + rrh_R * Bz_L + rrh_L * rrh_R * (vz_R - vz_L) * sB) / den;
    R Bns = Bx * n[0] + By * n[1] + Bz * n[2];
    Bx += (Bn - Bns) * n[0]; By += (Bn - Bns) * n[1]; Bz += (Bn - Bns) * n[2];
    R vB_ss = vx * Bx + vy * By + vz * Bz;
    R vBstar, e_star;
    if (LR == 0) { vBstar = vx_L * Bx_L + vy_L * By_L + vz_L * Bz_L; e_star = UsL[TAU]; }
    else { vBstar = vx_R * Bx_R + vy_R * By_R + vz_R * Bz_R; e_star = UsR[TAU]; }
    R pm = LR == 1 ? (R)1.0 : (R)-1.0;
    R e_ss = e_star + pm * rrh_K * (vBstar - vB_ss) * sB;
    Uss[DDD] = rhostar_K; Uss[SRR] = rhostar_K * vx; Uss[LLL] = rhostar_K * vy; Uss[SZZ] = rhostar_K * vz;
    Uss[TAU] = e_ss; Uss[BRR] = Bx; Uss[BPP] = By; Uss[BZZ] = Bz;
  }
  // get_Ustar_HLLD, hlld.c:282-401
  DISCO_D static void hlld(const DevParams& P, R w, const R* primL, const R* primR, R* F, R* U, R r,
                           const R* n) {
    R gam = PRM(R, P, gamma_law);
    R vel[5], Pt_star;
    R hr = 1.0, hp = r, hz = 1.0;
    R pL[NQ], pR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) { pL[q] = primL[q]; pR[q] = primR[q]; }
    pL[URR] *= hr; pR[URR] *= hr;
    pL[UPP] *= hp; pR[UPP] *= hp;
    pL[UZZ] *= hz; pR[UZZ] *= hz;
    h_velocities(gam, pL, pR, n, vel, &Pt_star);
    if (w < vel[2]) {
      R UL[8];
      h_flux(gam, pL, F, n);
      h_prim_to_cons(gam, pL, UL);
      if (w < vel[0]) {
        h_prim_to_cons(gam, pL, U);
      } else if (w < vel[1]) {
        h_single_star(gam, pL, U, vel[0], vel[2], Pt_star, n);
#pragma unroll
        for (int q = 0; q < 8; ++q) F[q] += vel[0] * (U[q] - UL[q]);
      } else {
        R UsL[8], UsR[8];
        h_single_star(gam, pL, UsL, vel[0], vel[2], Pt_star, n);
        h_single_star(gam, pR, UsR, vel[4], vel[2], Pt_star, n);
        h_double_star(UsL, UsR, U, vel, n, 0);
#pragma unroll
        for (int q = 0; q < 8; ++q) F[q] += vel[1] * (U[q] - UsL[q]) + vel[0] * (UsL[q] - UL[q]);
      }
#pragma unroll
      for (int q = 8; q < NQ; ++q) { U[q] = pL[q] * U[DDD]; F[q] = pL[q] * F[DDD]; }
    } else {
      R UR[8];
      h_flux(gam, pR, F, n);
      h_prim_to_cons(gam, pR, UR);
      if (w > vel[4]) {
        h_prim_to_cons(gam, pR, U);
      } else if (w > vel[3]) {
        h_single_star(gam, pR, U, vel[4], vel[2], Pt_star, n);
#pragma unroll
        for (int q = 0; q < 8; ++q) F[q] += vel[4] * (U[q] - UR[q]);
      } else {
        R UsL[8], UsR[8];
        h_single_star(gam, pL, UsL, vel[0], vel[2], Pt_star, n);
        h_single_star(gam, pR, UsR, vel[4], vel[2], Pt_star, n);
        h_double_star(UsL, UsR, U, vel, n, 1);
#pragma unroll
        for (int q = 0; q < 8; ++q) F[q] += vel[3] * (U[q] - UsR[q]) + vel[4] * (UsR[q] - UR[q]);
      }
#pragma unroll
      for (int q = 8; q < NQ; ++q) { U[q] = pR[q] * U[DDD]; F[q] = pR[q] * F[DDD]; }
    }
    R brfac = (R)1.0 / r, bpfac = 1.0, bzfac = 1.0;
    F[SRR] *= hr; F[LLL] *= hp; F[SZZ] *= hz;
    F[BRR] *= brfac / hr; F[BPP] *= bpfac / hp; F[BZZ] *= bzfac / hz;
    U[SRR] *= hr; U[LLL] *= hp; U[SZZ] *= hz;
    U[BRR] *= brfac / hr; U[BPP] *= bpfac / hp; U[BZZ] *= bzfac / hz;
  }

  // Signal speeds of the CFL bound in R (mixed path): sp[0..2] = c_f + |v|
  // per direction, c_f the fast speed bound sqrt(cs^2 + B^2 / rho) of
  // mhd.c:452-483; sp[3] = 0 (no explicit viscosity).
  DISCO_D static void cfl_speeds_r(const DevParams& P, const DevPlanet*, const R* prim, R w, R r, R phi,
                                   R* sp) {
    (void)phi;
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (prim[UPP] - w) * r;
    R cs2 = PRM(R, P, gamma_law) * Pp / rho;
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R cf = sqrt(cs2 + (Br * Br + Bp * Bp + Bz * Bz) / rho);
    sp[0] = cf + fabs(prim[URR]);
    sp[1] = cf + fabs(vp);
    sp[2] = cf + fabs(prim[UZZ]);
    sp[3] = (R)0;
  }

  // mindt of the mixed path: the same bound in R, with the cell extents
  // dL0 = r dphi, dL1 = dr, dL2 = dz given.
  DISCO_D static R mindt_r(const DevParams& P, const DevPlanet*, const R* prim, R w, R dL0, R dL1,
                           R dL2, R r, R phi) {
    (void)phi;
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (prim[UPP] - w) * r;
    R vr = prim[URR], vz = prim[UZZ];
    R cs = sqrt(PRM(R, P, gamma_law) * Pp / rho);
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R b2 = (Br * Br + Bp * Bp + Bz * Bz) / rho;
    R cf = sqrt(cs * cs + b2);
    R dt = dL1 / (cf + fabs(vr)), dtp = dL0 / (cf + fabs(vp)), dtz = dL2 / (cf + fabs(vz));
    if (dt > dtp) dt = dtp;
    if (dt > dtz) dt = dtz;
    return dt;
  }

  // mindt, mhd.c:452-483
  DISCO_D static double mindt(const DevParams& P, const DevPlanet*, const R* prim, double w,
                              const double* xp, const double* xm, double r) {
    R Pp = prim[PPP], rho = prim[RHO];
    R vp = (R)((double)prim[UPP] - w) * (R)r;
    R vr = prim[URR], vz = prim[UZZ];
    R cs = sqrt(PRM(R, P, gamma_law) * Pp / rho);
    R Br = prim[BRR], Bp = prim[BPP], Bz = prim[BZZ];
    R b2 = (Br * Br + Bp * Bp + Bz * Bz) / rho;
    R cf = sqrt(cs * cs + b2);
    R maxvr = cf + fabs(vr), maxvp = cf + fabs(vp), maxvz = cf + fabs(vz);
    double dL1 = xp[0] - xm[0];
    double dL0 = .5 * (xp[0] + xm[0]) * get_dp(xp[1], xm[1], P.phi_max);
    double dL2 = xp[2] - xm[2];
    double dt, dtp, dtz;
    if (sizeof(R) < sizeof(double)) {
      dt = (double)((R)dL1 / maxvr); dtp = (double)((R)dL0 / maxvp); dtz = (double)((R)dL2 / maxvz);
    } else {
      dt = dL1 / (double)maxvr; dtp = dL0 / (double)maxvp; dtz = dL2 / (double)maxvz;
    }
    if (dt > dtp) dt = dtp;
    if (dt > dtz) dt = dtz;
    return dt;
  }
};

}  // namespace disco
