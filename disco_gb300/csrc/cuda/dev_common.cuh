// Device-side parameters, state arrays and the small geometry / frame /
// gravity helpers the hot path calls per cell and per face.  Every helper
// names the reference function it restates; arithmetic follows the same
// operation order so the FP64 path tracks the reference to rounding.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <math.h>

#define DISCO_HD __host__ __device__
#define DISCO_D __device__ __forceinline__

namespace disco {

// primitive / conserved component indices (paul.h:4-5)
enum { RHO = 0, PPP = 1, URR = 2, UPP = 3, UZZ = 4, BRR = 5, BPP = 6, BZZ = 7 };
enum { DDD = 0, TAU = 1, SRR = 2, LLL = 3, SZZ = 4 };
enum { PL_POINTMASS = 0, PL_PW = 1, PL_SURFACEGRAV = 2, PL_SPLINE = 3, PL_WEGGC = 4 };
enum { SOLVER_HLL = 0, SOLVER_HLLC = 1, SOLVER_HLLD = 2, SOLVER_HLLC_DAMP = 3 };

constexpr int MAX_Q = 9;
constexpr int MAX_PL = 4;

struct DevPlanet {
  double r, phi, M, omega, vr, eps;
  int type;
};

// Hot-path parameters (the module-static values the reference pushes with
// set*Params, domain.c:259-270), passed by value to every kernel.
struct DevParams {
  int Nr, Nz, NgRa, NgRb, NgZa, NgZb;
  long long Ncell;
  int num_q, num_c;
  double phi_max;
  // Hydro/euler.c:6-27 and Hydro/mhd.c:6-22
  double gamma_law, rho_floor, p_floor, explicit_viscosity, mach;
  int include_viscosity, isothermal, alpha_flag, polar_sources;
  // riemann.c:7-10, misc.c, plm.c
  int riemann_solver, mesh_motion;
  double PLM, CFL, maxDT;
  // omega.c:4-38
  int meshOmChoice, enOmChoice, cs2Choice;
  double Omega0, om_M, om_r1, om_H0, eps;
  // rotframe.c:4-12
  int rot_flag;
  double rot_omega, rot_d;
  // planet.c:4-35
  int grav2D, polar_r, polar_p;
  // plm_geom_boundary (plm.c:184-186) acts on the inner ring when it has no
  // ghosts and geom_grad (cylindrical.c:150-155) finds its edge at r = 0
  int geom_bd_r;
  // cooling and damping (sink.c:274-427): Cool_Type, Cool_Par1 (beta);
  // Damp{Inner,Outer,Upper,Lower}_{Type,Time,Len}; the domain edges they use
  int cool_type, cool_damp, twoD;
  double cool_beta;
  int damp_type[4];
  double damp_time[4], damp_len[4];
  double dom_rmin, dom_rmax, dom_zmax;
  // accreting sinks and the nozzle (sink.c:105-247): Sink_Type, the number
  // of sink bodies (Sink_Number capped at Npl), Sink_Par1..5, Nozzle_Type,
  // Nozzle_Par1..4
  int sink_type, sink_bodies, nozzle_type;
  double sink_par[5], nozzle_par[4];
  int Npl;
  // GRMHD: the black-hole mass of the Kerr-Schild metric (Metric_Par2)
  double gr_M;
  double gr_a;     // GRMHD: black-hole spin (Metric_Par3) of the Kerr metric
  int gr_kerr;     // GRMHD: 1 for METRIC kerr_ks_rpz, 0 for schw_ks_rpz
  // initial / boundary plugins
  int initial_id, boundary_id;
  double ic[8];
  double ic_aux[4];   // constants the initial condition derived at set-up (disco_host_domain)
  double t_end;
  // exact division by Nr and Nr - 1 (ring and r-pair indices) by 40-bit
  // reciprocals: ceil(2^40 / d)
  unsigned long long mul_nr, mul_nr1;
  // FP32 copies of the parameters the mixed-precision kernels use per cell
  // or face (a conversion from FP64 would issue on the slow FP64 pipe)
  struct {
    float gamma_law, rho_floor, p_floor, explicit_viscosity, mach, PLM;
    float Omega0, om_M, om_r1, om_H0, eps;
  } f;
};

// A parameter in the arithmetic type R: the FP32 copy on the mixed path.
#define PRM(R, P, x) (sizeof(R) < sizeof(double) ? (R)(P).f.x : (R)(P).x)

// n / d for 0 <= n < 2^24 and 1 <= d < 2^16, given m = ceil(2^40 / d): the
// rounding excess of m is below n / 2^40 < 2^-16 < 1 / d, so the floor is
// exact.  Replaces a runtime integer division (tens of instructions).
DISCO_HD inline int div_fast(int n, unsigned long long m) {
  return (int)(((unsigned long long)n * m) >> 40);
}

// FP64 <-> FP32 conversions on the integer pipes, without branches.  A
// hardware conversion to or from FP64 issues on the FP64 pipe, which on this
// part runs at a small fraction of the FP32 rate.  They are used where they
// measured faster: conserved-state reads and writes in the update, in
// cons2prim and in the constrained-transport flux kernels.  In the Riemann
// flux kernels, whose FP64 pipe is mostly idle, the hardware conversion
// measured faster and stays.
//
// d2f_int: in the normal FP32 range it rounds to nearest, ties away from
// zero (IEEE's ties-to-even differs on exact ties only; the error is at most
// half an ulp either way).  Results below the smallest normal FP32 number
// flush to signed zero; overflow gives infinity, NaN stays NaN.
#ifdef __CUDACC__
__device__ inline float d2f_int(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned s = (unsigned)(b >> 32) & 0x80000000u;
  unsigned long long a = b & 0x7fffffffffffffffull;
  unsigned e = (unsigned)(a >> 52);
  // add half an FP32 ulp, drop 29 mantissa bits, rebias the exponent by
  // 1023 - 127 = 896 (a carry out of the mantissa lands in the exponent;
  // the arithmetic is modulo 2^32 and the result fits in 31 bits)
  unsigned m = (unsigned)((a + (1ull << 28)) >> 29) - (896u << 23);
  unsigned big = (a > 0x7ff0000000000000ull) ? 0x7fc00000u : 0x7f800000u;
  m = e < 897u ? 0u : (e > 1150u ? big : m);
  return __uint_as_float(s | m);
}
// f2d_int: exact for normal FP32 numbers, zero, infinity and NaN; FP32
// subnormals flush to signed zero.
__device__ inline double f2d_int(float x) {
  unsigned u = __float_as_uint(x);
  unsigned s = u & 0x80000000u;
  unsigned a = u & 0x7fffffffu;
  unsigned e = a >> 23;
  unsigned hi = (a >> 3) + (e == 255u ? (1792u << 20) : (896u << 20));
  hi = e == 0u ? 0u : hi;
  unsigned lo = e == 0u ? 0u : (a << 29);
  return __hiloint2double((int)(s | hi), (int)lo);
}
// to_r: a double into the reconstruction type R (identity for R = double)
template <typename R>
__device__ inline R to_r(double x) {
  if constexpr (sizeof(R) < sizeof(double)) return d2f_int(x);
  else return x;
}
template <typename R>
__device__ inline double from_r(R x) {
  if constexpr (sizeof(R) < sizeof(double)) return f2d_int(x);
  else return x;
}
#endif

// ---- cylindrical geometry: Geometry/cylindrical.c ------------------------
DISCO_HD inline double get_dp(double phip, double phim, double phi_max) {
  double dp = phip - phim;                       // cylindrical.c:10-15
  while (dp < 0.0) dp += phi_max;
  while (dp > phi_max) dp -= phi_max;
  return dp;
}
DISCO_HD inline double get_signed_dp(double phip, double phim, double phi_max) {
  double dp = phip - phim;                       // cylindrical.c:17-22
  while (dp < -.5 * phi_max) dp += phi_max;
  while (dp > .5 * phi_max) dp -= phi_max;
  return dp;
}
#ifdef __CUDACC__
// clean_pi (misc.c:8) and get_dp with their comparisons on the bit patterns
// instead of FP64 compares: the integer order of non-negative doubles is
// their numeric order, and a negative non-zero double's bits exceed 2^63 as
// unsigned.  Same results as the FP64-compare loops for finite values;
// infinities and NaN pass through instead of looping.
__device__ inline double clean_pi_bits(double p, double pmax) {
  const long long bmax = __double_as_longlong(pmax);
  long long b = __double_as_longlong(p);
  while (b > bmax && b < 0x7ff0000000000000LL) { p -= pmax; b = __double_as_longlong(p); }
  while ((unsigned long long)b > 0x8000000000000000ull && (unsigned long long)b < 0xfff0000000000000ull) {
    p += pmax;
    b = __double_as_longlong(p);
  }
  return p;
}
__device__ inline double get_dp_bits(double phip, double phim, double pmax) {
  double dp = phip - phim;
  long long b = __double_as_longlong(dp);
  while ((unsigned long long)b > 0x8000000000000000ull && (unsigned long long)b < 0xfff0000000000000ull) {
    dp += pmax;
    b = __double_as_longlong(dp);
  }
  const long long bmax = __double_as_longlong(pmax);
  while (b > bmax && b < 0x7ff0000000000000LL) { dp -= pmax; b = __double_as_longlong(dp); }
  return dp;
}
// get_signed_dp (cylindrical.c:17-22) with the comparisons against
// +-pmax/2 on the bit patterns (ordered by magnitude within each sign).
__device__ inline double get_signed_dp_bits(double phip, double phim, double pmax) {
  const double half = .5 * pmax;
  const unsigned long long hb = (unsigned long long)__double_as_longlong(half);
  double dp = phip - phim;
  unsigned long long b = (unsigned long long)__double_as_longlong(dp);
  // dp < -half: negative with magnitude above half (and not NaN)
  while (b > (0x8000000000000000ull | hb) && b < 0xfff0000000000000ull) {
    dp += pmax;
    b = (unsigned long long)__double_as_longlong(dp);
  }
  // dp > half: non-negative above half (and not NaN or infinity)
  while (b > hb && b < 0x7ff0000000000000ull) {
    dp -= pmax;
    b = (unsigned long long)__double_as_longlong(dp);
  }
  return dp;
}
// while (p < 0) p += pmax; while (p > pmax) p -= pmax; on the bit patterns
__device__ inline double wrap_pos_bits(double p, double pmax) {
  const long long bmax = __double_as_longlong(pmax);
  long long b = __double_as_longlong(p);
  while ((unsigned long long)b > 0x8000000000000000ull && (unsigned long long)b < 0xfff0000000000000ull) {
    p += pmax;
    b = __double_as_longlong(p);
  }
  while (b > bmax && b < 0x7ff0000000000000LL) { p -= pmax; b = __double_as_longlong(p); }
  return p;
}
#endif
DISCO_HD inline double centroid_r(double xp, double xm) {
  return 2.0 * (xp * xp + xp * xm + xm * xm) / (3.0 * (xp + xm));  // cylindrical.c:24-30
}
DISCO_HD inline double centroid_z(double xp, double xm) { return 0.5 * (xp + xm); }

// ---- omega.c ----------------------------------------------------------------
template <typename R>
DISCO_D R mesh_om(const DevParams& P, R r) {           // omega.c:56-74
  r = sqrt(r * r + PRM(R, P, eps) * PRM(R, P, eps));
  if (P.meshOmChoice == 1) return (R)1.0;
  if (P.meshOmChoice == 2) return pow(r, (R)-1.5);
  if (P.meshOmChoice == 3) { R n = 4.0; return (R)1. / pow(pow(r, (R)1.5 * n) + (R)1., (R)1. / n); }
  return (R)0.0;
}
template <typename R>
DISCO_D R get_om(const DevParams& P, R r) {            // omega.c:76-100
  if (P.enOmChoice == 0) return (R)0.0 - PRM(R, P, Omega0);
  r = sqrt(r * r + PRM(R, P, eps) * PRM(R, P, eps));
  if (P.enOmChoice == 1) return (R)1.0 - PRM(R, P, Omega0);
  if (P.enOmChoice == 2) return (R)1.0 / pow(r, (R)1.5) - PRM(R, P, Omega0);
  if (P.enOmChoice == 3) { R n = 8.0; return (R)1. / pow(pow(r, (R)1.5 * n) + (R)1., (R)1. / n) - PRM(R, P, Omega0); }
  if (P.enOmChoice == 4) return (R)10. * exp((R)-.5 * r * r) - PRM(R, P, Omega0);
  return (R)0.0 - PRM(R, P, Omega0);
}
template <typename R>
DISCO_D R get_om1(const DevParams& P, R r) {           // omega.c:102-126
  if (P.enOmChoice == 0 || P.enOmChoice == 1) return (R)0.0;
  r = sqrt(r * r + PRM(R, P, eps) * PRM(R, P, eps));
  if (P.enOmChoice == 2) return (R)-1.5 / pow(r, (R)2.5);
  if (P.enOmChoice == 3) {
    R n = 8.0;
    return (R)-1.5 * pow(r, (R)-1 + (R)1.5 * n) / pow(pow(r, (R)1.5 * n) + (R)1., (R)1.0 + (R)1. / n);
  }
  if (P.enOmChoice == 4) return (R)10. * r * exp((R)-.5 * r * r);
  return (R)0.0;
}

// ---- planet.c ---------------------------------------------------------------
template <typename R>
DISCO_D R phigrav(R M, R r, R eps, int type) {          // planet.c:37-73 (point mass)
  if (type == PL_POINTMASS) {
    R n = 2.0;
    return M / pow(pow(r, n) + pow(eps, n), (R)1. / n);
  }
  return (R)0.0;
}
template <typename R>
DISCO_D R fgrav(R M, R r, R eps, int type) {            // planet.c:75-112 (point mass)
  if (type == PL_POINTMASS) {
    R n = 2.0;
    return M * pow(r, n - (R)1.) / pow(pow(r, n) + pow(eps, n), (R)1. + (R)1. / n);
  }
  if (type == PL_SURFACEGRAV) return M;
  return (R)0.0;
}

template <typename R>
DISCO_D R get_cs2(const DevParams& P, const DevPlanet* pl, R r, R phi) {  // omega.c:157-209
  if (P.cs2Choice == 1) return (R)1. / (PRM(R, P, mach) * PRM(R, P, mach));
  if (P.cs2Choice == 2) { R nu = .5; return (R).5 / PRM(R, P, mach) / PRM(R, P, mach) / pow(r, (R)2. * nu); }
  if (P.cs2Choice == 3) return PRM(R, P, om_M) * PRM(R, P, om_H0) * PRM(R, P, om_H0) / ((R)2 * PRM(R, P, om_r1) * PRM(R, P, om_r1) * PRM(R, P, om_r1));
  if (P.cs2Choice == 4) {
    r = sqrt(r * r + PRM(R, P, eps) * PRM(R, P, eps));
    R v2 = PRM(R, P, om_M) / r;
    return v2 / (PRM(R, P, mach) * PRM(R, P, mach));
  }
  if (P.cs2Choice == 5) {
    R cosp = cos(phi), sinp = sin(phi);
    R gx = r * cosp, gy = r * sinp;
    R phip = 0.0;
    for (int p = 0; p < P.Npl; ++p) {
      R px = (R)pl[p].r * cos((R)pl[p].phi);
      R py = (R)pl[p].r * sin((R)pl[p].phi);
      R pr = (px - gx) * (px - gx) + (py - gy) * (py - gy);
      phip += phigrav<R>((R)pl[p].M, sqrt(pr), (R)pl[p].eps, pl[p].type);
    }
    return phip / (PRM(R, P, mach) * PRM(R, P, mach));
  }
  return (R)1.0;
}

// planetaryForce (planet.c:138-188).  mode 1 (report.c) takes the force
// components along the planet's direction instead of the cell's.
template <typename R>
DISCO_D void planetary_force(const DevParams& P, const DevPlanet& pl, R r, R phi, R z,
                             R* fr, R* fp, R* fz, int mode = 0) {
  R rp = (R)pl.r, pp = (R)pl.phi;
  if (P.grav2D == 1) z = 0.0;
  else if (P.grav2D == 2) { rp = r; pp = phi; z = 1.0; }
  R cosp = cos(phi), sinp = sin(phi);
  R dx = r * cosp - rp * cos(pp);
  R dy = r * sinp - rp * sin(pp);
  R script_r = sqrt(dx * dx + dy * dy + z * z);
  R script_r_perp = sqrt(dx * dx + dy * dy);
  R f1 = -fgrav<R>((R)pl.M, script_r, (R)pl.eps, pl.type);
  R cosa = dx / script_r_perp, sina = dy / script_r_perp;
  R cosap = cosa * cosp + sina * sinp;
  R sinap = sina * cosp - cosa * sinp;
  if (mode == 1) {
    cosap = cosa * cos(pp) + sina * sin(pp);
    sinap = sina * cos(pp) - cosa * sin(pp);
  }
  if (script_r_perp <= (R)0.0) { cosap = 0.0; sinap = 0.0; }
  R sint = script_r_perp / script_r;
  R cost = z / script_r;
  *fr = cosap * f1 * sint;
  *fp = sinap * f1 * sint;
  *fz = f1 * cost;
}

// planet_src (planet.c:190-234) for one planet, cylindrical coordinates, at
// the cell centre (rc, phi, z) of a cell of width dphi; T is the accumulator
// type (FP64 conserved state, or the R sum of the mixed path).
template <typename R, typename T>
DISCO_D void planet_src(const DevParams& P, const DevPlanet& pl, const R* prim, T* cons, R phi,
                        R x2, T dVdt, R rc, R dphi) {
  R rho = prim[RHO], vr = prim[URR], vz = prim[UZZ], omega = prim[UPP];
  R x0 = rc;
  R F0, F1, F2;
  planetary_force<R>(P, pl, x0, phi, x2, &F0, &F1, &F2);
  R hr = 1.0, hp = x0, hz = 1.0;
  if (P.polar_r || P.polar_p) {
    // geom_polar_vec_adjust, cylindrical.c:175-183
    R adjust = (R)(sin((R)0.5 * dphi) / ((R)0.5 * dphi));
    if (P.polar_r) F0 *= adjust;
    if (P.polar_p) F1 *= adjust;
  }
  cons[SRR] += (T)(rho * hr * F0 * (R)dVdt);
  cons[LLL] += (T)(rho * hp * F1 * (R)dVdt);
  cons[SZZ] += (T)(rho * hz * F2 * (R)dVdt);
  cons[TAU] += (T)(rho * (hr * F0 * vr + hz * F2 * vz + hp * F1 * omega) * (R)dVdt);
}

// get_height_om (omega.c:132-155): sqrt(sum_p fgrav / script_r).
template <typename R>
DISCO_D R get_height_om(const DevParams& P, const DevPlanet* pl, R r, R phi) {
  R omtot2 = 0.0;
  R gx = r * cos(phi), gy = r * sin(phi);
  for (int p = 0; p < P.Npl; ++p) {
    R px = (R)pl[p].r * cos((R)pl[p].phi);
    R py = (R)pl[p].r * sin((R)pl[p].phi);
    R sr = sqrt((px - gx) * (px - gx) + (py - gy) * (py - gy));
    R f1 = fgrav<R>((R)pl[p].M, sr, (R)pl[p].eps, pl[p].type);
    omtot2 += f1 / (sr + (R)0.0625 * (R)pl[p].eps);
  }
  return sqrt(omtot2);
}

// Health counters written by kernels (never trap).
struct DevErrs {
  unsigned long long nan_cells, rho_floor_hits, p_floor_hits, face_errors, steps;
  unsigned long long c2p_no_converge;   // GRMHD Newton cons2prim at its iteration cap
  // GRMHD Newton cons2prim: calls, the summed iteration at first convergence
  // (k_converge), the summed iterations taken, and the calls whose starting
  // point came from a supplied guess instead of the previous primitives
  unsigned long long c2p_calls, c2p_kconv, c2p_iters, c2p_guessed;
  unsigned long long async_timeouts;   // bounded waits on asynchronous copies that ran out
};

#ifdef __CUDACC__
// Adds one cons2prim record to the counters, one atomic per warp for each
// (the calling threads may be any subset of the warp).
__device__ inline void c2p_count(DevErrs* e, int kconv, int iters, int guessed) {
  const unsigned m = __activemask();
  const unsigned kc = __reduce_add_sync(m, (unsigned)kconv);
  const unsigned it = __reduce_add_sync(m, (unsigned)iters);
  const unsigned gs = __reduce_add_sync(m, (unsigned)guessed);
  if ((threadIdx.x & 31) == (unsigned)(__ffs(m) - 1)) {
    atomicAdd(&e->c2p_calls, (unsigned long long)__popc(m));
    atomicAdd(&e->c2p_kconv, (unsigned long long)kc);
    atomicAdd(&e->c2p_iters, (unsigned long long)it);
    if (gs) atomicAdd(&e->c2p_guessed, (unsigned long long)gs);
  }
}
#endif

}  // namespace disco
