// GRMHD module (Hydro/grmhd.c) on the Schwarzschild metric in Kerr-Schild
// cylindrical coordinates (Hydro/Metric/schw_ks_rpz.c) or the Kerr metric
// of spin a in the same coordinates (plugins/metric_kerr.h), with the normal
// observer frame (Hydro/Frame/normal.c).  FP64 only.
//
// Unlike the Newtonian modules every hook depends on the full position
// x = (r, phi, z) through the metric, so the hooks take x explicitly and the
// kernels call them through `if constexpr (Phys::GR)` branches.  Each
// formula keeps the reference's operation order (the FP64 units are built
// without FMA contraction), so the results track the reference to rounding.
//
// B is cell-centred (CT_MODE 0): prim[BRR..BZZ] = sqrt(gamma) B^i (with the
// r^-1 / r scalings of the reference), conserved B evolves by the face
// fluxes like the other components.  Primitive velocities are the covariant
// u_i: prim[URR] = u_r, prim[UPP] = u_phi / r^2, prim[UZZ] = u_z.
#pragma once
#include "dev_common.cuh"
#include "../plugins/metric_kerr.h"

namespace disco {

// ---- Hydro/Metric/schw_ks_rpz.c -------------------------------------------
// metric_lapse :20, metric_shift :26, metric_gam :39, metric_igam :63,
// metric_jacobian :88, metric_der_g :93, metric_der_lapse :142,
// metric_der_shift :159, metric_killing :184.
// kerr != 0 selects the Kerr metric of spin a (metric_kerr.h); else the
// Schwarzschild formulas of schw_ks_rpz.c in the reference's operation order.
struct KsMetric {
  double al, be[3], gam[9], igam[9], jac;   // jac = metric_jacobian / r

  DISCO_D KsMetric(const double* x, double M, double a, int kerr) {
    if (kerr) {
      disco_kerr_3p1(x, M, a, &al, be, gam, igam);
      jac = 1.0;   // metric_jacobian (r) / r
      return;
    }
    const double r = x[0], z = x[2];
    const double R = sqrt(r * r + z * z);
    al = 1.0 / sqrt(1.0 + 2 * M / R);
    const double a2 = 1.0 / (1.0 + 2 * M / R);
    be[0] = 2 * M * r / (R * R) * a2;
    be[1] = 0.0;
    be[2] = 2 * M * z / (R * R) * a2;
    const double H = 2 * M / R;
    const double st = r / R, ct = z / R;
    gam[0] = 1.0 + H * st * st; gam[1] = 0.0; gam[2] = H * st * ct;
    gam[3] = 0.0; gam[4] = r * r; gam[5] = 0.0;
    gam[6] = H * st * ct; gam[7] = 0.0; gam[8] = 1.0 + H * ct * ct;
    const double b2 = 1.0 / (1.0 + H);
    igam[0] = (1.0 + H * ct * ct) * b2; igam[1] = 0.0; igam[2] = -H * st * ct * b2;
    igam[3] = 0.0; igam[4] = 1.0 / (r * r); igam[5] = 0.0;
    igam[6] = -H * st * ct * b2; igam[7] = 0.0; igam[8] = (1.0 + H * st * st) * b2;
    jac = x[0] / r;
  }
};

DISCO_D int ks_killing(int mu) { return (mu == 1 || mu == 3) ? 0 : 1; }

// d g_{mu nu} / d x^i (i = 1: r, i = 3: z; zero otherwise)
DISCO_D void ks_der_g(const double* x, double M, double a, int kerr, int i, double* dg) {
  if (kerr) {
    disco_kerr_der_g(x, M, a, i, dg);
    return;
  }
  for (int mu = 0; mu < 16; ++mu) dg[mu] = 0.0;
  if (i != 1 && i != 3) return;
  const double r = x[0], z = x[2];
  const double R = sqrt(r * r + z * z);
  const double st = r / R, ct = z / R;
  const double MoR2 = M / (R * R), MoR3 = M / (R * R * R), MoR4 = M / (R * R * R * R);
  if (i == 1) {
    dg[0] = -2 * MoR2 * st;
    dg[1] = 2 * MoR2 * (1.0 - 2 * st * st);
    dg[3] = -4 * MoR3 * z * st;
    dg[5] = 2 * MoR3 * r * (2.0 - 3.0 * st * st);
    dg[7] = 2 * MoR3 * z * (1.0 - 3.0 * st * st);
    dg[10] = 2 * r;
    dg[15] = -6 * MoR4 * z * z * st;
  } else {
    dg[0] = -2 * MoR2 * ct;
    dg[1] = -4 * MoR3 * r * ct;
    dg[3] = 2 * MoR2 * (1.0 - 2 * ct * ct);
    dg[5] = -6 * MoR4 * r * r * ct;
    dg[7] = 2 * MoR3 * r * (1.0 - 3.0 * ct * ct);
    dg[15] = 2 * MoR3 * z * (2.0 - 3.0 * ct * ct);
  }
  dg[4] = dg[1];
  dg[12] = dg[3];
  dg[13] = dg[7];
}

// frame_U (normal.c:9): the normal observer, U = (1, -beta) / alpha
DISCO_D void ks_frame_U(const KsMetric& g, double* U) {
  const double ia = 1.0 / g.al;
  U[0] = ia;
  U[1] = -ia * g.be[0];
  U[2] = -ia * g.be[1];
  U[3] = -ia * g.be[2];
}

// frame_der_U (normal.c:21) with metric_der_lapse / metric_der_shift
DISCO_D void ks_frame_der_U(const double* x, double M, double spin, int kerr, const KsMetric& g, double* dU) {
  double da[4], db[12];
  if (kerr) {
    disco_kerr_der_lapse(x, M, spin, da);
    disco_kerr_der_shift(x, M, spin, db);
  } else {
    const double r = x[0], z = x[2];
    const double R = sqrt(r * r + z * z);
    const double st = r / R, ct = z / R;
    // metric_der_lapse
    const double MoR2 = M / (R * R);
    const double a = 1.0 / sqrt(1.0 + 2 * M / R);
    da[0] = 0.0; da[1] = a * a * a * MoR2 * st; da[2] = 0.0; da[3] = a * a * a * MoR2 * ct;
    // metric_der_shift
    const double denom = 1.0 / (R * R + 2 * M * R);
    const double d_denom = -denom * denom * 2 * (R + M);
    for (int i = 0; i < 3; ++i) db[i] = 0;
    db[3] = 2 * M * denom + 2 * M * r * d_denom * st;
    db[4] = 0.0;
    db[5] = 2 * M * z * d_denom * st;
    for (int i = 0; i < 3; ++i) db[6 + i] = 0;
    db[9] = 2 * M * r * d_denom * ct;
    db[10] = 0.0;
    db[11] = 2 * M * denom + 2 * M * z * d_denom * ct;
  }
  const double ia = 1.0 / g.al;
  for (int i = 0; i < 16; ++i) dU[i] = 0.0;
  for (int i = 0; i < 4; ++i) {
    if (ks_killing(i)) continue;
    dU[4 * i] = -ia * ia * da[i];
    for (int j = 0; j < 3; ++j) dU[4 * i + j + 1] = g.be[j] * ia * ia * da[i] - db[3 * i + j] * ia;
  }
}

template <typename R, int NQ>
struct Grmhd {
  static_assert(sizeof(R) == sizeof(double), "the GRMHD module runs in FP64 only");
  static constexpr int NC = 8;
  static constexpr bool MHD = true;   // B components present (cell-centred)
  static constexpr bool GR = true;
  template <typename T>
  using Rebind = Grmhd<T, NQ>;

  // shared pieces of prim2cons / flux (grmhd.c:65-155, :247-337)
  struct State {
    double l[3], B[3], U[4], w, u0, l0, uU, uB, b0, bd[3], B2, b2, UB, Ub, sqrtgam;
  };
  DISCO_D static void state(const KsMetric& g, const double* prim, double r, State& s) {
    s.sqrtgam = g.jac / g.al;
    s.l[0] = prim[URR]; s.l[1] = r * r * prim[UPP]; s.l[2] = prim[UZZ];
    s.B[0] = prim[BRR] / s.sqrtgam; s.B[1] = prim[BPP] / (r * s.sqrtgam); s.B[2] = prim[BZZ] / s.sqrtgam;
    ks_frame_U(g, s.U);
    double igaml[3];
    for (int i = 0; i < 3; ++i) {
      igaml[i] = 0.0;
      for (int j = 0; j < 3; ++j) igaml[i] += g.igam[3 * i + j] * s.l[j];
    }
    const double u2 = s.l[0] * igaml[0] + s.l[1] * igaml[1] + s.l[2] * igaml[2];
    s.w = sqrt(1.0 + u2);
    s.u0 = s.w / g.al;
    s.l0 = -g.al * s.w + g.be[0] * s.l[0] + g.be[1] * s.l[1] + g.be[2] * s.l[2];
    s.uU = s.U[0] * s.l0 + s.U[1] * s.l[0] + s.U[2] * s.l[1] + s.U[3] * s.l[2];
    s.uB = s.l[0] * s.B[0] + s.l[1] * s.B[1] + s.l[2] * s.B[2];
    s.b0 = s.uB / g.al;
    for (int i = 0; i < 3; ++i)
      s.bd[i] = (g.gam[3 * i] * s.B[0] + g.gam[3 * i + 1] * s.B[1] + g.gam[3 * i + 2] * s.B[2] +
                 s.l[i] * s.uB) / s.w;
    s.B2 = 0.0;
    s.UB = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        s.B2 += g.gam[3 * i + j] * s.B[i] * s.B[j];
        s.UB += g.gam[3 * i + j] * s.B[i] * (s.U[0] * g.be[j] + s.U[j + 1]);
      }
    s.b2 = (s.B2 + s.uB * s.uB) / (s.w * s.w);
    s.Ub = (s.UB + s.uU * s.uB) / s.w;
  }

  // prim2cons, grmhd.c:65-155
  DISCO_D static void prim2cons_x(const DevParams& P, const double* prim, double* cons, const double* x,
                                  double dV) {
    const double r = x[0];
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    State s;
    state(g, prim, r, s);
    const double gl = P.gamma_law;
    const double rho = prim[RHO], Pp = prim[PPP];
    const double rhoh = rho + gl / (gl - 1.0) * Pp + s.b2;
    const double rhoe = Pp / (gl - 1.0);
    cons[DDD] = g.jac * rho * s.u0 * dV;
    cons[SRR] = g.jac * (rhoh * s.u0 * s.l[0] - s.b0 * s.bd[0]) * dV;
    cons[LLL] = g.jac * (rhoh * s.u0 * s.l[1] - s.b0 * s.bd[1]) * dV;
    cons[SZZ] = g.jac * (rhoh * s.u0 * s.l[2] - s.b0 * s.bd[2]) * dV;
    cons[TAU] = g.jac * (-(rhoe + 0.5 * s.b2) * s.uU * s.u0 - (Pp + 0.5 * s.b2) * (s.uU * s.u0 + s.U[0]) -
                         rho * (s.uU + 1.0) * s.u0 + s.Ub * s.b0) * dV;
    cons[BRR] = s.sqrtgam * s.B[0] / r * dV;
    cons[BPP] = s.sqrtgam * s.B[1] * dV;
    cons[BZZ] = s.sqrtgam * s.B[2] * dV;
#pragma unroll
    for (int q = NC; q < NQ; ++q) cons[q] = prim[q] * cons[DDD];
  }

  // flux, grmhd.c:247-337
  DISCO_D static void flux_x(const DevParams& P, const double* prim, double* f, const double* x,
                             const double* n) {
    const double r = x[0];
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    State s;
    state(g, prim, r, s);
    // u^i and v^i = u^i / u^0 (the reference forms igaml again; same values)
    double u[3], v[3];
    for (int i = 0; i < 3; ++i) {
      double igl = 0.0;
      for (int j = 0; j < 3; ++j) igl += g.igam[3 * i + j] * s.l[j];
      u[i] = igl - g.be[i] * s.u0;
    }
    for (int i = 0; i < 3; ++i) v[i] = u[i] / s.u0;
    const double un = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
    const double Bn = s.B[0] * n[0] + s.B[1] * n[1] + s.B[2] * n[2];
    const double Un = s.U[1] * n[0] + s.U[2] * n[1] + s.U[3] * n[2];
    const double vn = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
    const double hn = n[0] + r * n[1] + n[2];
    const double bn = (Bn + s.uB * un) / s.w;
    const double gl = P.gamma_law;
    const double rho = prim[RHO], Pp = prim[PPP];
    const double rhoh = rho + gl / (gl - 1.0) * Pp + s.b2;
    const double rhoe = Pp / (gl - 1.0);
    const double Pt = Pp + 0.5 * s.b2;
    f[DDD] = g.jac * hn * rho * un;
    f[SRR] = g.jac * hn * (rhoh * un * s.l[0] + Pt * n[0] - s.bd[0] * bn);
    f[LLL] = g.jac * hn * (rhoh * un * s.l[1] + Pt * n[1] - s.bd[1] * bn);
    f[SZZ] = g.jac * hn * (rhoh * un * s.l[2] + Pt * n[2] - s.bd[2] * bn);
    f[TAU] = g.jac * hn * (-(rhoe + 0.5 * s.b2) * s.uU * un - Pt * (s.uU * un + Un) -
                           rho * (s.uU + 1.0) * un + s.Ub * bn);
    f[BRR] = s.sqrtgam * hn * (s.B[0] * vn - Bn * v[0]) / r;
    f[BPP] = s.sqrtgam * hn * (s.B[1] * vn - Bn * v[1]);
    f[BZZ] = s.sqrtgam * hn * (s.B[2] * vn - Bn * v[2]);
#pragma unroll
    for (int q = NC; q < NQ; ++q) f[q] = prim[q] * f[DDD];
  }

  // vel, grmhd.c:489-646: the outer wave speeds (the contact speed Ss is
  // used by HLLC only and is not formed)
  DISCO_D static void vel_x(const DevParams& P, const double* p1, const double* p2, double* Sl, double* Sr,
                            const double* n, const double* x) {
    const double r = x[0];
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    const double sqrtgam = g.jac * r / (g.al * r);   // metric_jacobian(x) / (al r)
    const double gl = P.gamma_law;
    const double* pr[2] = {p1, p2};
    double sl[2], sr[2];
    const double bn = g.be[0] * n[0] + g.be[1] * n[1] + g.be[2] * n[2];
    const double ign = g.igam[0] * n[0] + g.igam[4] * n[1] + g.igam[8] * n[2];
    const double hn = n[0] + r * n[1] + n[2];
    for (int k = 0; k < 2; ++k) {
      const double* p = pr[k];
      const double rho = p[RHO], Pp = p[PPP];
      const double l[3] = {p[URR], r * r * p[UPP], p[UZZ]};
      const double B[3] = {p[BRR] / sqrtgam, p[BPP] / (r * sqrtgam), p[BZZ] / sqrtgam};
      const double cs2 = gl * Pp / (rho + gl / (gl - 1.0) * Pp);
      double uS[3], u2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        uS[i] = 0.0;
        for (int j = 0; j < 3; ++j) uS[i] += g.igam[3 * i + j] * l[j];
        u2 += uS[i] * l[i];
      }
      const double w = sqrt(1.0 + u2);
      const double v2 = u2 / (w * w);
      const double uB = l[0] * B[0] + l[1] * B[1] + l[2] * B[2];
      double BB = 0.0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) BB += g.gam[3 * i + j] * B[i] * B[j];
      const double b2 = (BB + uB * uB) / (w * w);
      const double va2 = b2 / (rho + gl / (gl - 1.0) * Pp + b2);
      const double cf2 = cs2 + va2 - cs2 * va2;
      const double vSn = (uS[0] * n[0] + uS[1] * n[1] + uS[2] * n[2]) / w;
      const double dv = sqrt(cf2 * (ign - vSn * vSn - cf2 * (ign * v2 - vSn * vSn))) / w;
      sl[k] = hn * (g.al * (vSn * (1.0 - cf2) - dv) / (1.0 - v2 * cf2) - bn);
      sr[k] = hn * (g.al * (vSn * (1.0 - cf2) + dv) / (1.0 - v2 * cf2) - bn);
    }
    *Sr = sr[0] > sr[1] ? sr[0] : sr[1];
    *Sl = sl[0] < sl[1] ? sl[0] : sl[1];
  }

  // source, grmhd.c:339-454.  xp, xm: the cell's upper / lower corners.
  DISCO_D static void source_x(const DevParams& P, const double* prim, double* cons, const double* xp,
                               const double* xm, double dVdt) {
    const double x[3] = {0.5 * (xm[0] + xp[0]), 0.5 * (xm[1] + xp[1]), 0.5 * (xm[2] + xp[2])};
    const double M = P.gr_M;
    const double r = x[0];
    KsMetric g(x, M, P.gr_a, P.gr_kerr);
    double U[4], dU[16];
    ks_frame_U(g, U);
    ks_frame_der_U(x, M, P.gr_a, P.gr_kerr, g, dU);
    const double sqrtgam = g.jac / g.al;
    const double gl = P.gamma_law;
    const double rho = prim[RHO], Pp = prim[PPP];
    double l[4] = {0.0, prim[URR], r * r * prim[UPP], prim[UZZ]};
    const double B[3] = {prim[BRR] / sqrtgam, prim[BPP] / (r * sqrtgam), prim[BZZ] / sqrtgam};
    double ig[16];
    const double ia2 = 1.0 / (g.al * g.al);
    ig[0] = -ia2;
    for (int mu = 0; mu < 3; ++mu) {
      ig[mu + 1] = g.be[mu] * ia2;
      ig[4 * (mu + 1)] = ig[mu + 1];
      for (int nu = 0; nu < 3; ++nu) ig[4 * (mu + 1) + nu + 1] = g.igam[3 * mu + nu] - g.be[mu] * g.be[nu] * ia2;
    }
    double igaml[3];
    igaml[0] = g.igam[0] * l[1] + g.igam[1] * l[2] + g.igam[2] * l[3];
    igaml[1] = g.igam[3] * l[1] + g.igam[4] * l[2] + g.igam[5] * l[3];
    igaml[2] = g.igam[6] * l[1] + g.igam[7] * l[2] + g.igam[8] * l[3];
    const double u2 = l[1] * igaml[0] + l[2] * igaml[1] + l[3] * igaml[2];
    const double w = sqrt(1.0 + u2);
    double u[4];
    u[0] = w / g.al;
    for (int i = 0; i < 3; ++i) u[i + 1] = igaml[i] - g.be[i] * u[0];
    l[0] = -g.al * w + g.be[0] * l[1] + g.be[1] * l[2] + g.be[2] * l[3];
    const double uB = l[1] * B[0] + l[2] * B[1] + l[3] * B[2];
    double b[4], bd[4];
    b[0] = uB / g.al;
    b[1] = (B[0] + u[1] * uB) / w;
    b[2] = (B[1] + u[2] * uB) / w;
    b[3] = (B[2] + u[3] * uB) / w;
    bd[1] = (g.gam[0] * B[0] + g.gam[1] * B[1] + g.gam[2] * B[2] + l[1] * uB) / w;
    bd[2] = (g.gam[3] * B[0] + g.gam[4] * B[1] + g.gam[5] * B[2] + l[2] * uB) / w;
    bd[3] = (g.gam[6] * B[0] + g.gam[7] * B[1] + g.gam[8] * B[2] + l[3] * uB) / w;
    double B2 = 0.0, beB = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        beB += g.gam[3 * i + j] * g.be[i] * B[j];
        B2 += g.gam[3 * i + j] * B[i] * B[j];
      }
    bd[0] = (beB + l[0] * uB) / w;
    const double b2 = (B2 + uB * uB) / (w * w);
    const double rhoh = rho + gl / (gl - 1.0) * Pp + b2;
    const double Pt = Pp + 0.5 * b2;
    const double rp = xp[0], rm = xm[0];
    const double r2_3 = (rp * rp + rp * rm + rm * rm) / 3.0;
    const double dphi = get_dp(xp[1], xm[1], P.phi_max);
    const double rcorr = r2_3 / (r * r);
    const double pcorr = sin(0.5 * dphi) / (0.5 * dphi);
    double Sk[3];
    for (int i = 0; i < 3; ++i) {
      Sk[i] = 0.0;
      if (ks_killing(i + 1)) continue;
      double dg[16];
      ks_der_g(x, M, P.gr_a, P.gr_kerr, i + 1, dg);
      for (int mu = 0; mu < 4; ++mu)
        for (int nu = 0; nu < 4; ++nu)
          Sk[i] += (rhoh * u[mu] * u[nu] * rcorr * pcorr + ig[4 * mu + nu] * Pt - b[mu] * b[nu]) *
                   dg[4 * mu + nu];
      Sk[i] *= 0.5;
    }
    double S0 = -U[1] * Sk[0] - U[2] * Sk[1] - U[3] * Sk[2];
    for (int mu = 0; mu <= 3; ++mu)
      for (int nu = 0; nu <= 3; ++nu) {
        if (mu == nu)
          S0 += -(rhoh * u[mu] * l[nu] + Pt - b[mu] * bd[nu]) * dU[4 * mu + nu];
        else
          S0 += -(rhoh * u[mu] * l[nu] - b[mu] * bd[nu]) * dU[4 * mu + nu];
      }
    cons[SRR] += g.jac * Sk[0] * dVdt;
    cons[LLL] += g.jac * Sk[1] * dVdt;
    cons[SZZ] += g.jac * Sk[2] * dVdt;
    cons[TAU] += g.jac * S0 * dVdt;
  }

  // ---- cons2prim (grmhd.c:228-245, cons2prim_solve_adiabatic_noble2d
  // :813-1029) in three parts: the invariants of the conserved state, a
  // Newton-Raphson solve of Noble et al. (2006)'s two equations in
  // (v^2, eta) from a given starting point, and the recovery of the
  // primitives.  FP64; each formula keeps the reference's operation order.

  // What the two Noble equations depend on: s2 = S^2 / D^2, the energy e,
  // Q = sqrt(gamma) B^2 / D and psi = sqrt(gamma) (B.S)^2 / D^3, with
  // n = (gamma_law - 1) / gamma_law.  Kept with the pieces the recovery uses.
  struct C2PInv {
    double D, S[3], B[3], B2, BS, s2, e, Q, psi, n, sqrtgam, r;
  };

  DISCO_D static void c2p_invariants(const DevParams& P, const double* cons, const KsMetric& g, double r,
                                     C2PInv& v) {
    v.r = r;
    v.D = cons[DDD];
    v.S[0] = cons[SRR]; v.S[1] = cons[LLL]; v.S[2] = cons[SZZ];
    const double tau = cons[TAU];
    v.sqrtgam = g.jac / g.al;
    double U[4];
    ks_frame_U(g, U);
    v.B[0] = r * cons[BRR] / v.sqrtgam; v.B[1] = cons[BPP] / v.sqrtgam; v.B[2] = cons[BZZ] / v.sqrtgam;
    double s2 = 0.0, Us = 0.0, BS = 0.0, B2 = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s2 += g.igam[3 * i + j] * v.S[i] * v.S[j];
    s2 /= v.D * v.D;
    for (int i = 0; i < 3; ++i) Us += v.S[i] * (g.be[i] * U[0] + U[i + 1]);
    Us /= v.D;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) B2 += g.gam[3 * i + j] * v.B[i] * v.B[j];
    for (int i = 0; i < 3; ++i) BS += v.B[i] * v.S[i];
    v.s2 = s2;
    v.B2 = B2;
    v.BS = BS;
    v.Q = v.sqrtgam * B2 / v.D;
    v.psi = v.sqrtgam * BS * BS / (v.D * v.D * v.D);
    v.e = (tau / v.D + Us + 1.0) / (g.al * U[0]);
    v.n = (P.gamma_law - 1.0) / P.gamma_law;
  }

  // The two residuals at (v2, eta), each relative to the term it balances.
  DISCO_D static double c2p_residual(const C2PInv& v, double v2, double eta) {
    if (!(v2 >= 0.0 && v2 < 1.0 && eta >= 1.0)) return 1.0e300;
    const double w = 1.0 / sqrt(1.0 - v2);
    const double Q = v.Q, psi = v.psi;
    const double fa = (eta + Q) * (eta + Q) * v2 - psi * (2 * eta + Q) / (eta * eta) - v.s2;
    const double fb = eta - v.n * (1 - v2) * (eta - w) + 0.5 * Q * (1 + v2) - 0.5 * psi / (eta * eta) - v.e;
    const double r = fabs(fa) / ((eta + Q) * (eta + Q)) + fabs(fb) / eta;
    return r == r ? r : 1.0e300;
  }

  // Newton-Raphson from (v20, eta0): at most 30 iterations, 10 more after
  // the relative change of eta first falls below 1e-12.  Returns the status
  // word: 4 if the iteration hit its cap.  *kconv = the iteration at which
  // the change first fell below the tolerance (0 if it never did), *iters =
  // the iterations taken.
  DISCO_D static int noble2d_solve(const C2PInv& v, double v20, double eta0, double* v2_out, double* eta_out,
                                   int* kconv, int* iters) {
    const double prec = 1.0e-12;
    const int max_iter = 30;
    const int Nextra = 10;
    const double Q = v.Q, psi = v.psi, s2 = v.s2, e = v.e, n = v.n;
    double v2, v21 = v20, eta, eta1 = eta0;
    int it = 0, clean = -1, kc = 0;
    while (1) {
      v2 = v21;
      eta = eta1;
      const double w = 1.0 / sqrt(1.0 - v2);
      const double fa = (eta + Q) * (eta + Q) * v2 - psi * (2 * eta + Q) / (eta * eta) - s2;
      const double fb = eta - n * (1 - v2) * (eta - w) + 0.5 * Q * (1 + v2) - 0.5 * psi / (eta * eta) - e;
      const double dfadv2 = (eta + Q) * (eta + Q);
      const double dfadet = 2 * (eta + Q) * (v2 + psi / (eta * eta * eta));
      const double dfbdv2 = n * (eta - 0.5 * w) + 0.5 * Q;
      const double dfbdet = 1 - n * (1 - v2) + psi / (eta * eta * eta);
      const double detj = dfadv2 * dfbdet - dfbdv2 * dfadet;
      v21 = v2 - (dfbdet * fa - dfadet * fb) / detj;
      eta1 = eta - (-dfbdv2 * fa + dfadv2 * fb) / detj;
      it++;
      if (v21 > 1.0) v21 = 0.5 * (v2 + 1.0);
      if (v21 < 0.0) v21 = 0.5 * v2;
      if (eta1 < 1.0) eta1 = 0.5 * (eta + 1.0);
      const double err = (eta1 - eta) / eta;
      if (fabs(err) < prec && clean < 0) {
        clean = Nextra + 1;
        kc = it;
      }
      if (clean >= 0) clean--;
      if (clean == 0 || it == max_iter) break;
    }
    *v2_out = v21;
    *eta_out = eta1;
    *kconv = kc;
    *iters = it;
    return it == max_iter ? 4 : 0;
  }

  // The starting point the reference uses: the previous primitives' v^2 and
  // eta = W h.
  DISCO_D static void c2p_warm_start(const DevParams& P, const KsMetric& g, const double* prim, double r,
                                     double* v20, double* eta0) {
    double u2 = 0.0;
    const double l[3] = {prim[URR], r * r * prim[UPP], prim[UZZ]};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) u2 += g.igam[3 * i + j] * l[i] * l[j];
    const double w = sqrt(1.0 + u2);
    const double gl = P.gamma_law;
    *v20 = u2 / (1.0 + u2);
    *eta0 = w * (1.0 + gl / (gl - 1.0) * prim[PPP] / prim[RHO]);
  }

  // Primitives from the converged (v2, eta); returns the floor-hit mask
  // (1 density, 2 pressure).
  DISCO_D static int c2p_recover(const DevParams& P, const KsMetric& g, const C2PInv& v, const double* cons,
                                 double v2, double eta, double* prim) {
    int hits = 0;
    const double gl = P.gamma_law, r = v.r, D = v.D, sqrtgam = v.sqrtgam;
    const double w = 1.0 / sqrt(1 - v2);
    const double u0 = w / g.al;
    double h = eta / w;
    double rho = D / (g.jac * u0);
    if (rho < P.rho_floor) { rho = P.rho_floor; hits |= 1; }
    double Pp = v.n * rho * (h - 1.0);
    if (Pp < P.p_floor * rho) { Pp = P.p_floor * rho; hits |= 2; }
    h = 1.0 + gl / (gl - 1.0) * Pp / rho;
    const double* B = v.B;
    double Bd[3];
    Bd[0] = g.gam[0] * B[0] + g.gam[1] * B[1] + g.gam[2] * B[2];
    Bd[1] = g.gam[3] * B[0] + g.gam[4] * B[1] + g.gam[5] * B[2];
    Bd[2] = g.gam[6] * B[0] + g.gam[7] * B[1] + g.gam[8] * B[2];
    const double BS = v.BS, B2 = v.B2;
    double l[3];
    l[0] = (v.S[0] + sqrtgam * BS * Bd[0] / (D * h * w)) / (D * h + sqrtgam * B2 / w);
    l[1] = (v.S[1] + sqrtgam * BS * Bd[1] / (D * h * w)) / (D * h + sqrtgam * B2 / w);
    l[2] = (v.S[2] + sqrtgam * BS * Bd[2] / (D * h * w)) / (D * h + sqrtgam * B2 / w);
    prim[RHO] = rho;
    prim[URR] = l[0];
    prim[UPP] = l[1] / (r * r);
    prim[UZZ] = l[2];
    prim[PPP] = Pp;
    prim[BRR] = sqrtgam * B[0];
    prim[BPP] = sqrtgam * r * B[1];
    prim[BZZ] = sqrtgam * B[2];
#pragma unroll
    for (int q = NC; q < NQ; ++q) prim[q] = cons[q] / cons[DDD];
    return hits;
  }

  // The previous primitives' log(W^2 - 1) and log(P / rho): the point the
  // reference starts from (v20 = u2 / (1 + u2), eta0 = W h), in the
  // variables the learned correction uses.
  DISCO_D static void c2p_warm_logs(const KsMetric& g, const double* prim, double r, double* lu2, double* lth) {
    double u2 = 0.0;
    const double l[3] = {prim[URR], r * r * prim[UPP], prim[UZZ]};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) u2 += g.igam[3 * i + j] * l[i] * l[j];
    *lu2 = log(fmax(u2, 1.0e-30));
    *lth = log(fmax(prim[PPP] / prim[RHO], 1.0e-30));
  }
  // The ten features of the learned correction: the Noble invariants (log e,
  // log s2, log Q, the squared cosine between B and S), the rest mass log D,
  // the lapse, log r, log |e^2 - s2|, and the previous primitives'
  // log(W^2 - 1) and log(P / rho).
  DISCO_D static void c2p_features(const C2PInv& v, const KsMetric& g, double lu2, double lth, float* f) {
    f[0] = logf((float)fmax(v.e, 1.0e-30));
    f[1] = logf((float)(v.s2 + 1.0e-20));
    f[2] = logf((float)(v.Q + 1.0e-20));
    f[3] = (float)(v.psi / (v.Q * v.s2 + 1.0e-30));
    f[4] = logf((float)fmax(v.D, 1.0e-30));
    f[5] = (float)g.al;
    f[6] = logf((float)v.r);
    f[7] = logf((float)(fabs(v.e * v.e - v.s2) + 1.0e-20));
    f[8] = (float)lu2;
    f[9] = (float)lth;
  }
  // Targets from a converged (v2, eta): the changes of log(W^2 - 1) and of
  // log(P / rho) from the previous primitives' values.
  DISCO_D static void c2p_targets(const C2PInv& v, double v2, double eta, double lu2, double lth, float* y) {
    const double u2 = v2 / (1.0 - v2);
    const double w = sqrt(1.0 + u2);
    const double th = v.n * (eta / w - 1.0);
    y[0] = (float)(log(fmax(u2, 1.0e-30)) - lu2);
    y[1] = (float)(log(fmax(th, 1.0e-30)) - lth);
  }
  // The starting point (v2, eta) of the outputs: W^2 - 1 = exp(lu2 + y0),
  // P / rho = exp(lth + y1), eta = W h, h = 1 + gamma / (gamma - 1) P / rho.
  DISCO_D static void c2p_guess_from(const C2PInv& v, const float* y, double lu2, double lth, double* g2) {
    const double u2 = exp(lu2 + (double)y[0]);
    const double th = exp(lth + (double)y[1]);
    g2[0] = u2 / (1.0 + u2);
    g2[1] = sqrt(1.0 + u2) * (1.0 + th / v.n);
  }

  // Per-call record of the solve: iteration at first convergence, the
  // iterations taken, and whether a supplied guess replaced the warm start.
  struct C2PRec {
    int kconv, iters, guessed;
  };

  // cons2prim at x: the conserved state cons_in (times dV) to prim (in: the
  // previous primitives, the warm start; out: the new ones).  guess, when
  // given, is a starting point (v^2, eta) that replaces the warm start if
  // its residual is the smaller (the warm start stays the fallback).
  // Returns the status word: 1 density floor, 2 pressure floor, 4 Newton
  // cap.
  DISCO_D static int cons2prim_x(const DevParams& P, const double* cons_in, double* prim, const double* x,
                                 double dV, const double* guess = nullptr, C2PRec* rec = nullptr) {
    double cons[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) cons[q] = cons_in[q] / dV;
    const double r = x[0];
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    C2PInv v;
    c2p_invariants(P, cons, g, r, v);
    double v20, eta0;
    c2p_warm_start(P, g, prim, r, &v20, &eta0);
    int guessed = 0;
    if (guess && c2p_residual(v, guess[0], guess[1]) < c2p_residual(v, v20, eta0)) {
      v20 = guess[0];
      eta0 = guess[1];
      guessed = 1;
    }
    double v2, eta;
    int kc, it;
    int status = noble2d_solve(v, v20, eta0, &v2, &eta, &kc, &it);
    status |= c2p_recover(P, g, v, cons, v2, eta, prim);
    if (rec) { rec->kconv = kc; rec->iters = it; rec->guessed = guessed; }
    return status;
  }

  // mindt, grmhd.c:648-721 (wc: the cell's mesh angular velocity)
  DISCO_D static double mindt_x(const DevParams& P, const double* prim, double wc, const double* xp,
                                const double* xm) {
    const double x[3] = {0.5 * (xm[0] + xp[0]), 0.5 * (xm[1] + xp[1]), 0.5 * (xm[2] + xp[2])};
    const double r = x[0];
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    const double sqrtgam = g.jac * r / (r * g.al);   // metric_jacobian(x) / (r al)
    const double gl = P.gamma_law;
    const double rho = prim[RHO], Pp = prim[PPP];
    const double l[3] = {prim[URR], r * r * prim[UPP], prim[UZZ]};
    const double B[3] = {prim[BRR] / sqrtgam, prim[BPP] / (r * sqrtgam), prim[BZZ] / sqrtgam};
    const double cs = sqrt(gl * Pp / (rho + gl / (gl - 1) * Pp));
    double uS[3], u2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      uS[i] = 0.0;
      for (int j = 0; j < 3; ++j) uS[i] += g.igam[3 * i + j] * l[j];
      u2 += uS[i] * l[i];
    }
    const double w = sqrt(1.0 + u2);
    double vS[3];
    for (int i = 0; i < 3; ++i) vS[i] = uS[i] / w;
    const double v2 = u2 / (w * w);
    const double uB = l[0] * B[0] + l[1] * B[1] + l[2] * B[2];
    double B2 = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) B2 += g.gam[3 * i + j] * B[i] * B[j];
    const double b2 = (B2 + uB * uB) / (w * w);
    const double va2 = b2 / (rho + gl / (gl - 1.0) * Pp + b2);
    const double cf = sqrt(cs * cs + va2 - cs * cs * va2);
    const double sig = 1 - cf * cf;
    const double dvr = cf * sqrt(g.igam[0] * (1 - cf * cf * v2) - sig * vS[0] * vS[0]) / w;
    const double vrl = fabs(g.al * (vS[0] * sig - dvr) / (1 - v2 * cf * cf) - g.be[0]);
    const double vrr = fabs(g.al * (vS[0] * sig + dvr) / (1 - v2 * cf * cf) - g.be[0]);
    const double dvp = cf * sqrt(g.igam[4] * (1 - cf * cf * v2) - sig * vS[1] * vS[1]) / w;
    const double vpl = fabs(r * (g.al * (vS[1] * sig - dvp) / (1 - v2 * cf * cf) - g.be[1] - wc));
    const double vpr = fabs(r * (g.al * (vS[1] * sig + dvp) / (1 - v2 * cf * cf) - g.be[1] - wc));
    const double dvz = cf * sqrt(g.igam[8] * (1 - cf * cf * v2) - sig * vS[2] * vS[2]) / w;
    const double vzl = fabs(g.al * (vS[2] * sig - dvz) / (1 - v2 * cf * cf) - g.be[2]);
    const double vzr = fabs(g.al * (vS[2] * sig + dvz) / (1 - v2 * cf * cf) - g.be[2]);
    const double maxvr = vrr > vrl ? vrr : vrl;
    const double maxvp = vpr > vpl ? vpr : vpl;
    const double maxvz = vzr > vzl ? vzr : vzl;
    // get_dL, cylindrical.c: dim 1 = dr, dim 0 = r dphi at the mean radius, dim 2 = dz
    const double dLr = xp[0] - xm[0];
    const double dLp = .5 * (xp[0] + xm[0]) * get_dp(xp[1], xm[1], P.phi_max);
    const double dLz = xp[2] - xm[2];
    const double dtr = dLr / maxvr, dtp = dLp / maxvp, dtz = dLz / maxvz;
    double dt = dtr;
    dt = dt < dtp ? dt : dtp;
    dt = dt < dtz ? dt : dtz;
    return dt;
  }
};

}  // namespace disco
