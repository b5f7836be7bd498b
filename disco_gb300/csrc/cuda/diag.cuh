// Ring diagnostics accumulated by every timestep: add_diagnostics
// (analysis.c:52-108, called at timestep.c:51) with the quantities of the
// Diagnostics/ plugin the configuration names (diag_euler.c, diag_disk2d.c,
// diag_cb.c, diag_bl.c, diag_mhdmri.c).
//
// For every ring (ghost rings included, as in the reference) the step adds
//   Qrz[jk][q] += (sum_i Q_q(x_i, prim_i) dV_i) * dt / (sum_i dV_i)
// and t_avg += dt.  One block per ring: each thread sums a strided share of
// the ring's cells, then a fixed shuffle/shared-memory tree adds the shares,
// so the result is deterministic and equal to the reference's serial sum to
// rounding.  On the mixed path the per-cell quantities and each thread's
// share of the ring are formed in R from the R primitives; the tree is FP64.
#pragma once
#include "kernels.cuh"
#include "phys_grmhd.cuh"

namespace disco {

constexpr int kDiagBlock = 128;
constexpr int kDiagMax = 48;

// num_diagnostics() of each plugin
DISCO_HD inline int diag_count(int id) {
  switch (id) {
    case 0: return 8;    // diag_euler.c:10
    case 1: return 5;    // diag_disk2d.c:10
    case 2: return 6;    // diag_cb.c:10
    case 3: return 5;    // diag_bl.c:10
    case 4: return 18;   // diag_mhdmri.c:9
    case 5: return 48;   // diag_grmhdmri.c:12
    default: return 0;
  }
}

// planetaryForce (planet.c:138-188) for the mixed path's diagnostics, in
// the planet's frame: with D = phi - phi_p formed in FP64 and s = sin(D/2),
//   |x - x_p|_perp^2 = (r - r_p)^2 + 4 r r_p s^2,
//   sin(a - phi) |x - x_p|_perp = r_p sin D,  cos(a - phi) |...| = (r - r_p) + 2 r_p s^2
// (mode 1, along the planet's direction: r sin D and (r - r_p) - 2 r s^2),
// so f_phi = -M r_p sin D / (|x - x_p|^2 + eps^2)^(3/2) keeps FP32's relative
// precision next to the planet, where the lab-frame differences
// r cos(phi) - r_p cos(phi_p) cancel.  The torque a ring sums is a small
// residual of such terms of both signs.
template <typename R>
DISCO_D void planetary_force_mix(const DevParams& P, const DevPlanet& pl, double r, double phi, double z,
                                 R* fr, R* fp, R* fz, int mode) {
  double rp = pl.r, pp = pl.phi;
  if (P.grav2D == 1) z = 0.0;
  else if (P.grav2D == 2) { rp = r; pp = phi; z = 1.0; }
  double del = phi - pp;
  if (del > M_PI) del -= 2.0 * M_PI;
  if (del > M_PI) del -= 2.0 * M_PI;
  if (del < -M_PI) del += 2.0 * M_PI;
  if (del < -M_PI) del += 2.0 * M_PI;
  R sh, ch;
  sincos((R)(0.5 * del), &sh, &ch);
  const R sinD = (R)2.0 * sh * ch;
  const R rr = (R)r, rpp = (R)rp, zz = (R)z, dr = (R)(r - rp);
  const R srp2 = dr * dr + (R)4.0 * rr * rpp * sh * sh;
  const R sr2 = srp2 + zz * zz;
  R f1_sr = 0.0;   // fgrav / |x - x_p|, with the sign of f1
  if (pl.type == PL_POINTMASS) {
    const R d = sr2 + (R)pl.eps * (R)pl.eps;
    f1_sr = -(R)pl.M / (d * sqrt(d));
  } else if (pl.type == PL_SURFACEGRAV) {
    f1_sr = -(R)pl.M / sqrt(sr2);
  }
  R s_ap, c_ap;   // sin/cos of the force's angle to the cell's (planet's) radial, times |x - x_p|_perp
  if (mode == 1) { s_ap = rr * sinD; c_ap = dr - (R)2.0 * rr * sh * sh; }
  else { s_ap = rpp * sinD; c_ap = dr + (R)2.0 * rpp * sh * sh; }
  if (!(srp2 > (R)0.0)) { s_ap = 0.0; c_ap = 0.0; }
  *fr = c_ap * f1_sr;
  *fp = s_ap * f1_sr;
  *fz = f1_sr * zz;
}

// The second body seen from one ring, for the mixed path's per-cell torque:
// everything but the azimuth is a ring constant.
template <typename R>
struct RingBody {
  double pp;          // the body's azimuth (FP64)
  R rr, rpp, dr, zz;  // ring radius, body radius, their difference (FP64 first), z
  R M, eps2;
  int type;
};

template <typename R>
DISCO_D RingBody<R> ring_body(const DevParams& P, const DevPlanet& pl, double r, double z) {
  RingBody<R> b;
  double rp = pl.r, pp = pl.phi;
  if (P.grav2D == 1) z = 0.0;
  b.pp = pp;
  b.rr = (R)r; b.rpp = (R)rp; b.dr = (R)(r - rp); b.zz = (R)z;
  b.M = (R)pl.M; b.eps2 = (R)pl.eps * (R)pl.eps;
  b.type = pl.type;
  return b;
}

// planetary_force_mix (mode 0) with the ring constants of RingBody: per cell
// one FP64 difference piph - phi_p, wrapped to [-pi, pi] in FP64 and
// rounded to FP32 on the integer pipe; the half width comes off in FP32.
template <typename R>
DISCO_D R ring_body_fphi(const RingBody<R>& b, double piph, R dph) {
  double d = piph - b.pp;
  if (d > M_PI) d -= 2.0 * M_PI;
  if (d < -M_PI) d += 2.0 * M_PI;
  R del = d2f_int(d) - (R)0.5 * dph;
  if (del < (R)-M_PI) del += (R)(2.0 * M_PI);
  R sh, ch;
  sincos((R)0.5 * del, &sh, &ch);
  const R srp2 = b.dr * b.dr + (R)4.0 * b.rr * b.rpp * sh * sh;
  const R sr2 = srp2 + b.zz * b.zz;
  R f1_sr = 0.0;
  if (b.type == PL_POINTMASS) {
    const R dd = sr2 + b.eps2;
    f1_sr = -b.M / (dd * sqrt(dd));
  } else if (b.type == PL_SURFACEGRAV) {
    f1_sr = -b.M / sqrt(sr2);
  }
  if (!(srp2 > (R)0.0)) return (R)0.0;
  return b.rpp * ((R)2.0 * sh * ch) * f1_sr;
}

// planetaryForce at the cell centroid: the reference's operation order on
// the FP64 path, the planet-frame form above on the mixed path
template <typename R>
DISCO_D void diag_force(const DevParams& P, const DevPlanet& pl, double r, double phi, double z, R* fr,
                        R* fp, R* fz, int mode) {
  if constexpr (kMix<R>) planetary_force_mix<R>(P, pl, r, phi, z, fr, fp, fz, mode);
  else planetary_force<R>(P, pl, r, phi, z, fr, fp, fz, mode);
}

// get_diagnostics of plugin D at the cell centroid (rd, phid, zd)
// (Om: the ring frame's rotation, added back to the mixed path's relative
// azimuthal velocity; 0 on the FP64 path)
template <typename R, int NQ, int D>
DISCO_D void diag_cell(const DevParams& P, const DevState<R>& S, int c, double Om, double rd, double phid,
                       double zd, R* Q, const RingBody<R>* rb = nullptr, double piph = 0.0, R dph = 0) {
  const int N = S.N;
  const R r = (R)rd, phi = (R)phid;
  const R rho = S.prim[RHO * N + c], Pp = S.prim[PPP * N + c];
  const R vr = S.prim[URR * N + c], vz = S.prim[UZZ * N + c];
  const R omega = S.prim[UPP * N + c] + (R)Om;
  const R twopi = (R)(2. * M_PI);
  if constexpr (D == 0) {   // diag_euler.c:18-44
    R Fr, Fp = 0.0, Fz;
    if (P.Npl > 1) {
      if (kMix<R> && rb) Fp = ring_body_fphi<R>(*rb, piph, dph);
      else diag_force<R>(P, S.planets[1], rd, phid, zd, &Fr, &Fp, &Fz, 0);
    }
    Q[0] = rho;
    Q[1] = twopi * r * rho * vr;
    Q[2] = twopi * r * rho * vz;
    Q[3] = twopi * r * rho * (r * Fp);
    Q[4] = twopi * r * rho * (r * r * omega * vr);
    Q[5] = omega;
    Q[6] = twopi * r * rho * r * r * omega;
    Q[7] = Pp;
  } else if constexpr (D == 1) {   // diag_disk2d.c:18-41
    R Fr, Fp = 0.0, Fz;
    if (P.Npl > 1) {
      if (kMix<R> && rb) Fp = ring_body_fphi<R>(*rb, piph, dph);
      else diag_force<R>(P, S.planets[1], rd, phid, 0.0, &Fr, &Fp, &Fz, 0);
    }
    Q[0] = rho;
    Q[1] = twopi * r * rho * vr;
    Q[2] = twopi * r * rho * (r * Fp);
    Q[3] = twopi * r * rho * (r * r * omega * vr);
    Q[4] = omega;
  } else if constexpr (D == 2) {   // diag_cb.c:18-62
    const R vp = r * omega;
    Q[0] = rho;
    Q[1] = twopi * r * rho * vr;
    const R cp = cos(phi), sp = sin(phi);
    const R gx = r * cp, gy = r * sp;
    const R vx = vr * cp - vp * sp;
    const R vy = vr * sp + vp * cp;
    const R vm2 = vx * vx + vy * vy;
    const R rdv = vx * gx + vy * gy;
    Q[2] = (vm2 - (R)1. / r) * gx - rdv * vx;
    Q[2] *= rho;
    Q[3] = (vm2 - (R)1. / r) * gy - rdv * vy;
    Q[3] *= rho;
    Q[4] = 0.0;
    Q[5] = rho * vp;
    for (int pi = 0; pi < 2 && pi < P.Npl; ++pi) {   // both bodies of the binary
      R Fr, Fp, Fz;
      diag_force<R>(P, S.planets[pi], rd, phid, zd, &Fr, &Fp, &Fz, 1);
      const R rp = (R)S.planets[pi].r;
      Q[4] += rho * rp * Fp;
    }
  } else if constexpr (D == 3) {   // diag_bl.c:17-36
    const R vp = r * omega;
    Q[0] = rho;
    Q[1] = rho * omega;
    Q[2] = rho * vp;
    Q[3] = rho * vr;
    Q[4] = rho * vp * vr;
  } else if constexpr (D == 4) {   // diag_mhdmri.c:17-62
    if constexpr (NQ >= 8) {
      const R g = (R)P.gamma_law;
      const R Br = S.prim[BRR * N + c], Bp = S.prim[BPP * N + c], Bz = S.prim[BZZ * N + c];
      const R vp = omega;
      const R cs2 = g * Pp / rho;
      const R B2 = Br * Br + Bp * Bp + Bz * Bz;
      const R sr = rho * vr;
      const R spp = r * r * rho * vp;
      const R sz = rho * vz;
      const R e = (R)0.5 * rho * (vr * vr + r * r * vp * vp + vz * vz) + Pp / (g - (R)1.0) + (R)0.5 * B2;
      Q[0] = rho; Q[1] = Pp; Q[2] = vr; Q[3] = vp; Q[4] = vz;
      Q[5] = Br; Q[6] = Bp; Q[7] = Bz;
      Q[8] = rho; Q[9] = e; Q[10] = sr; Q[11] = spp; Q[12] = sz;
      Q[13] = rho * vr * vp;
      Q[14] = Br * Bp;
      Q[15] = B2;
      Q[16] = sqrt(cs2);
      Q[17] = sqrt(B2 / rho);
    }
  } else if constexpr (D == 5) {   // diag_grmhdmri.c:19-163 (FP64 GRMHD path)
    if constexpr (NQ >= 8 && !kMix<R>) {
      const double gl = P.gamma_law;
      const double x[3] = {rd, phid, zd};
      const KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
      const double al = g.al, jac = g.jac;
      const double* be = g.be;
      const double* gam = g.gam;
      const double* igam = g.igam;
      const double sqrtgam = jac / al;
      const double l[3] = {vr, S.prim[UPP * N + c], vz};
      const double B[3] = {S.prim[BRR * N + c] / sqrtgam, S.prim[BPP * N + c] / (rd * sqrtgam),
                           S.prim[BZZ * N + c] / sqrtgam};
      double U[4];
      ks_frame_U(g, U);
      double igaml[3];
      for (int i = 0; i < 3; ++i) {
        igaml[i] = 0.0;
        for (int j = 0; j < 3; ++j) igaml[i] += igam[3 * i + j] * l[j];
      }
      const double u2 = l[0] * igaml[0] + l[1] * igaml[1] + l[2] * igaml[2];
      const double w = sqrt(1.0 + u2);
      const double u0 = w / al;
      double u[3];
      for (int i = 0; i < 3; ++i) u[i] = igaml[i] - be[i] * u0;
      const double l0 = -al * w + be[0] * l[0] + be[1] * l[1] + be[2] * l[2];
      const double uU = U[0] * l0 + U[1] * l[0] + U[2] * l[1] + U[3] * l[2];
      const double uB = l[0] * B[0] + l[1] * B[1] + l[2] * B[2];
      const double b0 = uB / al;
      double bd[3], b[3];
      for (int i = 0; i < 3; ++i) {
        bd[i] = (gam[3 * i] * B[0] + gam[3 * i + 1] * B[1] + gam[3 * i + 2] * B[2] + l[i] * uB) / w;
        b[i] = (B[i] + uB * u[i]) / w;
      }
      double B2 = 0.0, UB = 0.0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          B2 += gam[3 * i + j] * B[i] * B[j];
          UB += gam[3 * i + j] * B[i] * (U[0] * be[j] + U[j + 1]);
        }
      const double b2 = (B2 + uB * uB) / (w * w);
      const double Ub = (UB + uU * uB) / w;
      const double rhoh = rho + gl / (gl - 1.0) * Pp + b2;
      const double rhoe = Pp / (gl - 1.0);
      const double rhohs = rhoh + b2;
      const double tauU = jac * (-(rhoe + 0.5 * b2) * uU * u0 - (Pp + 0.5 * b2) * (uU * u0 + U[0]) -
                                 rho * (uU + 1.0) * u0 + Ub * b0);
      const double tau = sqrtgam * ((rhoe + 0.5 * b2) * w * w + (Pp + 0.5 * b2) * u2 + rho * w * u2 / (w + 1) -
                                    b0 * b0);
      const double bd0 = -al * al * b0 + be[0] * bd[0] + be[1] * bd[1] + be[2] * bd[2];
      const double uu[4] = {u0, u[0], u[1], u[2]};
      const double uud[4] = {l0, l[0], l[1], l[2]};
      const double bb[4] = {b0, b[0], b[1], b[2]};
      const double bbd[4] = {bd0, bd[0], bd[1], bd[2]};
      Q[0] = rho; Q[1] = Pp;
      Q[2] = l[0]; Q[3] = l[1]; Q[4] = l[2];
      Q[5] = B[0]; Q[6] = B[1]; Q[7] = B[2];
      Q[8] = jac * rho * u0;
      Q[9] = tauU;
      for (int i = 0; i < 3; ++i) Q[10 + i] = jac * (rhohs * u0 * l[i] - b0 * bd[i]);
      for (int i = 0; i < 3; ++i) Q[13 + i] = jac * rho * uu[1 + i];
      for (int i = 1; i < 4; ++i)
        for (int j = 1; j < 4; ++j) {
          const int n = 3 * (i - 1) + (j - 1);
          Q[16 + n] = jac * (rhoh * uud[i] * uu[j]);
          Q[25 + n] = jac * (b2 * uud[i] * uu[j]);
          Q[34 + n] = jac * (-bbd[i] * bb[j]);
        }
      Q[43] = B2;
      Q[44] = b2;
      Q[45] = sqrt(gl * Pp / rhoh);
      Q[46] = sqrt(b2 / rhohs);
      Q[47] = tau;
    }
  }
}

// One block per ring jk; Qrz is [Nr*Nz][ND], t_avg lives in scal[SC_TAVG].
template <typename R, int NQ, int D>
DISCO_D void k_diag_body(const DevParams& P, const DevState<R>& S, double* Qrz, int bx_, int by_) {
  constexpr int ND = D == 0 ? 8 : D == 1 ? 5 : D == 2 ? 6 : D == 3 ? 5 : D == 4 ? 18 : 48;
  const int jk = bx_;
  const int k = jk / P.Nr, j = jk - k * P.Nr;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const double rp = S.r_jph[j + 1], rm = S.r_jph[j];   // r_jph[j], r_jph[j-1]
  const double zp = S.z_kph[k + 1], zm = S.z_kph[k];
  const double rc = centroid_r(rp, rm);
  const double zc = .5 * (zp + zm);
  const double rdr = (.5 * (rp + rm)) * (rp - rm), dz = zp - zm;
  const double Om = kMix<R> ? S.ring_Om[jk] : 0.0;
  // Each cell's Q dV is formed in R (FP32 on the mixed path, whose cell
  // volume comes from the cell's own width; FP64 with the reference's get_dV
  // otherwise); every sum, each thread's share and the tree across threads,
  // is FP64 on both paths.
  // the mixed path's torque (diag_euler, diag_disk2d) takes the ring
  // constants once; the other forms need each cell's centroid azimuth
  const bool ring_force = kMix<R> && (D == 0 || D == 1) && P.Npl > 1 && P.grav2D != 2;
  const bool need_phi = !ring_force && (D == 2 || D == 5 || ((D == 0 || D == 1) && P.Npl > 1));
  RingBody<R> rb;
  if (ring_force) rb = ring_body<R>(P, S.planets[1], rc, D == 1 ? 0.0 : zc);
  double sum[ND + 1];
#pragma unroll
  for (int q = 0; q <= ND; ++q) sum[q] = 0.0;
#pragma unroll 4
  for (int i = threadIdx.x; i < Np; i += kDiagBlock) {
    const int c = off + i;
    double phic = 0.0;
    R dV;
    double piph = 0.0;
    R dphf = 0;
    if constexpr (kMix<R>) {
      const double dph = S.dphi[c];
      if (need_phi) phic = S.piph[c] - .5 * dph;
      if (ring_force) piph = S.piph[c];
      dphf = d2f_int(dph);
      dV = (R)rdr * dphf * (R)dz;
    } else {
      const double phip = S.piph[c];
      const double phim = phip - S.dphi[c];
      phic = .5 * (phip + phim);   // get_centroid(dim 0)
      dV = rdr * get_dp(phip, phim, P.phi_max) * dz;   // get_dV, cylindrical.c:56-63
    }
    R Q[ND];
    diag_cell<R, NQ, D>(P, S, c, Om, rc, phic, zc, Q, ring_force ? &rb : nullptr, piph, dphf);
#pragma unroll
    for (int q = 0; q < ND; ++q) sum[q] += from_r<R>(Q[q] * dV);
    sum[ND] += from_r<R>(dV);
  }
  __shared__ double red[ND + 1][kDiagBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q <= ND; ++q) {
    double x = sum[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[q][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < ND) {
    double s = 0.0, v = 0.0;
#pragma unroll
    for (int w = 0; w < kDiagBlock / 32; ++w) { s += red[threadIdx.x][w]; v += red[ND][w]; }
    const double dt = S.scal[SC_DT];
    Qrz[(size_t)jk * ND + threadIdx.x] += s * dt / v;
  }
  if (jk == 0 && threadIdx.x == 0) S.scal[SC_TAVG] += S.scal[SC_DT];
}
template <typename R, int NQ, int D>
__global__ void __launch_bounds__(kDiagBlock) k_diag(DevParams P, DevState<R> S, double* Qrz) {
  k_diag_body<R, NQ, D>(P, S, Qrz, (int)blockIdx.x, (int)blockIdx.y);
}

}  // namespace disco
