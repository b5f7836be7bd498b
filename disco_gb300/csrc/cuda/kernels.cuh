// Kernels of one RK substep (onestep.c:86-186) on ragged SoA ring arrays.
//
// Layout in HBM (N = cells incl. ghosts, ring jk = j + Nr*k):
//   cell c of ring jk lives at ring_off[jk] + i;  per-component arrays are
//   SoA: prim[q*N + c] (R), cons/RKcons[q*N + c] (FP64; RKdU in R on the
//   mixed path), gradp/gradr/gradz
//   [q*N + c] (R), piph/dphi/wiph[c] (FP64).
//   Sheared r (dim 1) and z (dim 2) faces are stored per ring pair in a
//   static block face_off[pair] .. face_off[pair+1] (the count Np_L + Np_R
//   never changes, faces_alt.c:87-100); only their contents are rebuilt.
#pragma once
#include "dev_common.cuh"
#include "riemann.cuh"
#include "../plugins/ic_vortex_gauss.h"
#include "../plugins/ic_disks.h"
#include "../plugins/ic_fm_torus.h"
#include "../plugins/bc_plugins.h"

namespace disco {

// accumulators per sink body, in report.c's column order (report.c:81-88)
enum { SA_GRAVL = 0, SA_DM, SA_ACCL, SA_LS, SA_KIN, SA_THERM, SA_XMOM, SA_YMOM, kSinkAcc };

template <typename R>
struct DevState {
  int N;                       // cells incl. ghosts
  const int* cell_ring;        // [N] ring id of each cell
  const int* ring_off;         // [Nr*Nz+1]
  const double* r_jph;         // [Nr+1], index shifted: r_jph[j+1] = reference r_jph[j]
  const double* z_kph;         // [Nz+1]
  const double* piph;          // [N] current positions
  double* piph_out;            // [N] positions after move_cells (first substep)
  double* dphi;                // [N]
  double* wiph;                // [N]
  R* prim;                     // [NQ*N]
  double* cons;                // [NQ*N]
  double* RKcons;              // [NQ*N] FP64 path: conserved state at the substep start
  R* RKdU;                     // [NQ*N] mixed path: the first substep's increment (R)
  R* gradp;                    // [NQ*N]
  R* gradr;                    // [NQ*N]
  R* gradz;                    // [NQ*N]
  R* fphi;                     // [NQ*N]  (F - wU*) dA dt of the phi face i|i+1
  // ring anchors (faces_alt.c:57-79)
  int* anchor;                 // [Nr*Nz]
  // sheared faces, index d = 0 (r) / 1 (z)
  const int* face_off[2];      // [npairs+1]
  int* fL[2];                  // [Nf] global cell id
  int* fR[2];
  signed char* fLR[2];         // LRtype
  double* fphic[2];            // cm[1]
  R* fdA[2];                   // dA
  R* fdpL[2];                  // signed phi offset face centre - L cell centre
  R* fdpR[2];                  // signed phi offset R cell centre - face centre
  R* ffrL[2];                  // face dphi / L cell dphi (edge EMF weight, CT)
  R* ffrR[2];                  // face dphi / R cell dphi
  R* fdp1[2];                  // avg_Efields interpolation weights (CT)
  R* fdp2[2];
  double* ring_rc;             // per ring: centroid radius (cylindrical.c:24)
  double* ring_r23;            // per ring: (rp^2 + rp rm + rm^2) / 3 (mhd.c:239)
  // Per-ring constants in R for the mixed path (the FP64 path evaluates the
  // reference's own expressions instead): centroid radius, .5 (rp + rm),
  // dV / dphi, phi-face area, total r / z face area per unit dphi
  // (plm.c:113-143), r / z face edge length (bfields.c:338-356).
  R* ring_rc_r;
  R* ring_r1_r;
  R* ring_vol_r;
  R* ring_dA_r;
  R* ring_r23_r;
  R* ring_zc_r;
  R* ring_At_r[2];
  R* ring_dl_r[2];
  double* ring_cfl;            // [3 * Nr*Nz]: .5 (rp + rm), 1 / dr, 1 / dz (CFL bound, FP64)
  R* dphi_r;                   // [N] dphi in R (the same array as dphi when R is double)
  // Ring frame of the mixed path: there prim[UPP] holds omega - Om of the
  // cell's ring, so the FP32 value keeps the precision of the motion
  // relative to the mesh (Om is fixed at set-up; 0 on the FP64 path).
  double* ring_Om;             // per ring: Om
  R* ring_Om_r;                // Om in R
  double* ring_Lsh;            // Om rc^2: angular momentum per unit mass of the frame
  R* ring_gL_r;                // Om (rc - r_lower), Om (rc - r_upper): EMF frame terms
  R* ring_gR_r;
  R* pdOm[2];                  // per pair: Om(R ring) - Om(L ring)
  R* pcX[2];                   // per pair: EMF frame term of the R cell, +-(Om_R - Om_L) r
  R* pdxL[2];                  // per pair: dxL, dxR, dxL + dxR, face radius
  R* pdxR[2];
  R* pdxs[2];
  R* prad[2];
  R* pidxs[2];                 // per pair: 1 / (dxL + dxR)
  R* pdA[2];                   // per pair: face area per unit dphi
  R* fflux[2];                 // [NQ*Nf] (F - wU*) dA dt
  R* fslope;                   // [NQ*max Nf] face slopes of one dimension (plm_trans)
  // chunks of kTileCells consecutive cells of one ring (tiled face gathers)
  const int* chunk_ring;
  const int* chunk_i0;
  int nchunk;
  // the ghost cells the boundary plugin fills, as chunks of up to
  // kTileCells consecutive cells of one ring (k_boundary: one block each)
  const int* ghost_ring;
  const int* ghost_i0;
  int nghost;
  const double* ghost_tab;     // [nring][NQ]: fixed ghosts of an axisymmetric initial condition
  int* run_up_s[2];            // per cell: first face where the cell is L (pair above)
  int* run_up_e[2];
  int* run_dn_s[2];            // per cell: first face where the cell is R (pair below)
  int* run_dn_e[2];
  // Boundary/horizon3d.c: rings boundary_fixed_horizon resets (list) and
  // the same as a per-ring flag, which drops their cells from the CFL
  // minimum; null / 0 without that plugin
  const int* hor_rings;
  const unsigned char* ring_excised;
  int nhor;
  // Boundary/horizon_bin.c: candidate (ring, hole) entries, 2 jk + hole,
  // and the per-cell flag its cut-outs set for good (real = 0)
  const int* hole_list;
  unsigned char* cell_excised;
  int nhole;
  int* nb_up[2];               // per cell: the R cell of its last face in the pair above
  int* nb_dn[2];               // per cell: the L cell of its last face in the pair below
  int nf[2];
  // constrained transport (MHD): edge EMFs written by the flux kernels
  int ct;
  R* Eraw;                     // [8*N] E[8] of the reference cell
  R* Braw;                     // [8*N] B[8]
  R* fErz[2];                  // per face flux_to_E outputs
  R* fBrz[2];
  R* fEphi[2];
  DevPlanet* planets;          // [Npl], device copy (moves for analytic orbits)
  double* sink_acc;            // [2][MAX_PL * kSinkAcc]: the sink bodies' accumulators, then their RK copy
  double* sink_part;           // [blocks of k_sink_acc][MAX_PL * kSinkAcc]: per-block partial sums
  double* scal;                // [0] dt, [1] t, [2] min-dt accumulator (bits)
  DevErrs* errs;
};

// scal: [SC_DT] dt (FP64), [SC_T] t, [SC_MIN] min-dt accumulator (bits),
// [SC_DTF] dt rounded to FP32, stored in the first 4 bytes of the slot,
// [SC_TAVG] the time the ring diagnostics have accumulated over.
enum { SC_DT = 0, SC_T = 1, SC_MIN = 2, SC_DTF = 3, SC_TAVG = 4, SC_COUNT = 5 };

// The mixed path (R = float) keeps positions, conserved sums and face
// fluxes of B in FP64 but does every other product in R.
template <typename R>
constexpr bool kMix = sizeof(R) < sizeof(double);

// dt in R: the FP32 copy on the mixed path, the FP64 value otherwise.
template <typename R>
DISCO_D R dt_r(const double* scal) {
  if constexpr (kMix<R>) return *(const float*)&scal[SC_DTF];
  else return scal[SC_DT];
}

// Wrap a phi difference into [0, Pmax] (get_dp) / [-Pmax/2, Pmax/2]
// (get_signed_dp) in R, for differences already formed in FP64.
template <typename R>
DISCO_D R wrap_dp(R dp, R Pmax) {
  while (dp < (R)0) dp += Pmax;
  while (dp > Pmax) dp -= Pmax;
  return dp;
}
template <typename R>
DISCO_D R wrap_signed(R dp, R Pmax) {
  while (dp < (R)-.5 * Pmax) dp += Pmax;
  while (dp > (R).5 * Pmax) dp -= Pmax;
  return dp;
}

// Order-preserving integer key of a double: integer comparison of keys
// equals IEEE comparison of the values (and +0 == -0), so phi orderings run
// on the integer pipe.
DISCO_D long long phi_key(double v) {
  long long b = __double_as_longlong(v);
  return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}
DISCO_D double phi_unkey(long long k) {
  return k >= 0 ? __longlong_as_double(k) : __longlong_as_double((-k) | (long long)0x8000000000000000ULL);
}

DISCO_D bool is_real(const DevParams& P, int j, int k) {
  return j >= P.NgRa && j < P.Nr - P.NgRb && k >= P.NgZa && k < P.Nz - P.NgZb;
}

// CT sweep ranges (misc.c:393-407, :464-500): one ring beyond the interior.
DISCO_D bool ring_in_phi_range(const DevParams& P, int j, int k) {
  int jmin = P.NgRa == 0 ? 0 : P.NgRa - 1, jmax = P.NgRb == 0 ? P.Nr : P.Nr - P.NgRb + 1;
  int kmin = P.NgZa == 0 ? 0 : P.NgZa - 1, kmax = P.NgZb == 0 ? P.Nz : P.Nz - P.NgZb + 1;
  return j >= jmin && j < jmax && k >= kmin && k < kmax;
}
DISCO_D bool pair_in_flux_range(const DevParams& P, int dim, int pair) {
  int j, k, jmin, jmax, kmin, kmax;
  if (dim == 1) {
    k = div_fast(pair, P.mul_nr1); j = pair - k * (P.Nr - 1);
    jmin = P.NgRa == 0 ? 0 : P.NgRa - 1; jmax = P.NgRb == 0 ? P.Nr - 1 : P.Nr - P.NgRb;
    kmin = P.NgZa == 0 ? 0 : P.NgZa - 1; kmax = P.NgZb == 0 ? P.Nz : P.Nz - P.NgZb + 1;
  } else {
    k = div_fast(pair, P.mul_nr); j = pair - k * P.Nr;
    jmin = P.NgRa == 0 ? 0 : P.NgRa - 1; jmax = P.NgRb == 0 ? P.Nr : P.Nr - P.NgRb + 1;
    kmin = P.NgZa == 0 ? 0 : P.NgZa - 1; kmax = P.NgZb == 0 ? P.Nz - 1 : P.Nz - P.NgZb;
  }
  return j >= jmin && j < jmax && k >= kmin && k < kmax;
}

// ---- initial() dispatch (plugin chosen by Makefile_opt.in INITIAL) --------
DISCO_D void initial_raw(const DevParams& P, double* prim, const double* x) {
  if (P.initial_id == 0) {
    disco_ic_vortex_gauss V{P.ic[0], P.ic[1], P.ic[2], P.ic[3], P.ic[4], P.gamma_law};
    disco_ic_vortex_gauss_eval(&V, prim, x, P.num_c, P.num_q);
  } else {
    disco_ic_disk D;
    disco_ic_disk_from_params(&D, P.gamma_law, P.mach, P.ic[0], P.ic[1], P.ic[2], P.ic[3],
                              P.ic[4], P.ic[5]);
    if (P.initial_id == 1) {
      disco_ic_disk_mhd_eval(&D, prim, x, P.num_c, P.num_q);
    } else if (P.initial_id == 2) {
      disco_ic_disk_planet_eval(&D, prim, x, P.num_c, P.num_q);
    } else if (P.initial_id == 3) {
      disco_ic_disk_cbd_eval(&D, prim, x, P.num_c, P.num_q);
    } else if (P.initial_id == 4) {   // gr_disk (Metric_Par2 = M, Init_Par1..4)
      disco_ic_gr_disk G{P.gamma_law, P.gr_M, P.ic[0], P.ic[1], P.ic[2], P.ic[3]};
      disco_ic_gr_disk_eval(&G, prim, x, P.num_c, P.num_q);
    } else {   // 5: fm_torus (Metric_Par2,3 = M, a; Init_Par1..4; the set-up's derived constants)
      disco_ic_fm F{P.gamma_law, P.gr_M, P.gr_a, P.ic[0], P.ic[1], P.ic[2], P.ic[3], P.rho_floor,
                    P.p_floor, P.ic_aux[0], P.ic_aux[1], P.ic_aux[2], P.ic_aux[3]};
      disco_ic_fm_eval(&F, prim, x, P.num_c, P.num_q);
    }
  }
}
// initial() followed by subtract_omega (rotframe.c:15), as set_cell_init does
DISCO_D void initial_eval(const DevParams& P, double* prim, const double* x) {
  initial_raw(P, prim, x);
  if (P.rot_flag) prim[UPP] -= P.rot_omega;
}

// ---- set_wcell, misc.c:101-168 --------------------------------------------
template <typename R, int NQ>
DISCO_D void k_wcell_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  int c = bx_ * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  double w = 0.0;
  if (P.mesh_motion == 4) {
    double r = centroid_r(S.r_jph[j + 1], S.r_jph[j]);
    w = (double)mesh_om<double>(P, r);
  } else if (P.mesh_motion) {
    int ip = (i + 1) % Np;
    double wL = (double)S.prim[UPP * S.N + c];        // get_omega: prim[UPP]
    double wR = (double)S.prim[UPP * S.N + off + ip];
    w = .5 * (wL + wR);
    if constexpr (kMix<R>) w += S.ring_Om[jk];          // ring frame -> lab
  }
  (void)k;
  S.wiph[c] = w;
}
template <typename R, int NQ>
__global__ void k_wcell(DevParams P, DevState<R> S) {
  k_wcell_body<R, NQ>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// Mixed path, Mesh_Motion 3: the ring average of .5 (w_i + w_i+1) is the
// ring average of w_i = prim[UPP]; one block per ring sums it as an FP64
// tree (the mesh speed enters F - wU, where its rounding is amplified) and
// writes the mean to every cell of the ring.
template <typename R>
DISCO_D void k_wcell_ring_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  __shared__ double part[32];
  int jk = bx_;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  double s = 0;
  for (int i = threadIdx.x; i < Np; i += blockDim.x) s += (double)S.prim[UPP * S.N + off + i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = s;
  __syncthreads();
  if (wid == 0) {
    s = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) part[0] = s / (double)Np + S.ring_Om[jk];   // ring frame -> lab
  }
  __syncthreads();
  double w = part[0];
  for (int i = threadIdx.x; i < Np; i += blockDim.x) S.wiph[off + i] = w;
}
template <typename R>
__global__ void k_wcell_ring(DevParams P, DevState<R> S) {
  k_wcell_ring_body<R>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// Mesh_Motion 3: ring average of w (misc.c:138-152), one block per ring.  The
// ring is staged in shared memory and summed by one thread in the
// reference's order, so the mesh speed rounds exactly like the reference's
// (it can coincide with a contact speed, where HLLD branches on equality).
template <typename R>
DISCO_D void k_wcell_avg_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  extern __shared__ double wsm[];
  int jk = bx_;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  for (int i = threadIdx.x; i < Np; i += blockDim.x) wsm[i] = S.wiph[off + i];
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < Np; ++i) s += wsm[i];
    wsm[Np] = s / (double)Np;
  }
  __syncthreads();
  double w = wsm[Np];
  for (int i = threadIdx.x; i < Np; i += blockDim.x) S.wiph[off + i] = w;
}
template <typename R>
__global__ void k_wcell_avg(DevParams P, DevState<R> S) {
  k_wcell_avg_body<R>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// dphi in R for the mixed path (after an upload or at set-up).
template <typename R>
__global__ void k_dphi_r(DevState<R> S) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < S.N) S.dphi_r[c] = (R)S.dphi[c];
}

// ---- plm_phi, plm.c:6-51 ------------------------------------------------
template <typename R>
DISCO_D R minmod(R a, R b, R c) {
  R m = a;
  if (a * b < (R)0.0) m = 0.0;
  if (fabs(b) < fabs(m)) m = b;
  if (b * c < (R)0.0) m = 0.0;
  if (fabs(c) < fabs(m)) m = c;
  return m;
}

template <typename R, int NQ>
DISCO_D void k_plm_phi_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  int c = bx_ * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  int cm = off + (i == 0 ? Np - 1 : i - 1);
  int cp = off + (i + 1 == Np ? 0 : i + 1);
  R dpL = S.dphi_r[cm], dpC = S.dphi_r[c], dpR = S.dphi_r[cp];
  R PLM = PRM(R, P, PLM);
  const int N = S.N;
  R iL = 0, iR = 0, iC = 0;
  if constexpr (kMix<R>) {   // three reciprocals instead of 3 NQ divisions
    iL = (R)1 / ((R).5 * (dpC + dpL));
    iR = (R)1 / ((R).5 * (dpR + dpC));
    iC = (R)1 / ((R).5 * (dpL + dpR) + dpC);
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    R pL = S.prim[q * N + cm], pC = S.prim[q * N + c], pR = S.prim[q * N + cp];
    R sL = pC - pL, sR = pR - pC, sC = pR - pL;
    if constexpr (kMix<R>) {
      sL *= iL; sR *= iR; sC *= iC;
    } else {
      sL /= (R).5 * (dpC + dpL);
      sR /= (R).5 * (dpR + dpC);
      sC /= (R).5 * (dpL + dpR) + dpC;
    }
    S.gradp[q * N + c] = minmod<R>(PLM * sL, sC, PLM * sR);
  }
}
template <typename R, int NQ>
__global__ void k_plm_phi(DevParams P, DevState<R> S) {
  k_plm_phi_body<R, NQ>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- ring anchors, faces_alt.c:57-79 -----------------------------------------
// Quadrant tests of sin/cos(piph * 2pi/Pmax) done as exact comparisons of the
// double theta against the doubles bracketing pi/2, pi, 3pi/2, 2pi: the sign
// of sin/cos of a double is fixed by which side of those irrationals it lies.
DISCO_D int quadrant_q1(double th) {  // sin > 0 && cos > 0
  const double PI_2_LO = 1.5707963267948965579989817342720925807952880859375;   // < pi/2
  const double TWO_PI_LO = 6.28318530717958623199592693708837032318115234375;    // < 2pi
  return (th > 0.0 && th <= PI_2_LO) || (th > TWO_PI_LO);
}
DISCO_D int quadrant_q4(double th) {  // sin < 0 && cos > 0
  const double THREE_PI_2_LO = 4.71238898038468967399694520281627774238586425781250;  // < 3pi/2
  const double TWO_PI_LO = 6.28318530717958623199592693708837032318115234375;
  return th > THREE_PI_2_LO && th <= TWO_PI_LO;
}

// One warp per ring: I0 = first Q1 cell after the first Q4 cell, else 0.
template <typename R>
DISCO_D void k_anchor_body(const DevParams& P, const DevState<R>& S, int nring, int bx_, int by_) {
  int warp = (bx_ * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nring) return;
  int off = S.ring_off[warp], Np = S.ring_off[warp + 1] - off;
  double convert = 2. * M_PI / P.phi_max;
  // phi_max = 2 pi (convert == 1): th = piph exactly, and the quadrant tests
  // compare bit patterns (the integer order of finite non-negative doubles
  // is their numeric order; negative values and NaN fail both tests as the
  // FP64 compares do)
  const bool unit = convert == 1.0;
  const long long kPi2 = 0x3ff921fb54442d18LL;     // bits of quadrant_q1's PI_2_LO
  const long long k3Pi2 = 0x4012d97c7f3321d2LL;    // bits of quadrant_q4's THREE_PI_2_LO
  const long long k2Pi = 0x401921fb54442d18LL;     // bits of TWO_PI_LO
  const long long kInf = 0x7ff0000000000000LL;
  auto q4 = [&](double p) {
    if (!unit) return quadrant_q4(p * convert) != 0;
    long long b = __double_as_longlong(p);
    return b > k3Pi2 && b <= k2Pi;
  };
  auto q1 = [&](double p) {
    if (!unit) return quadrant_q1(p * convert) != 0;
    long long b = __double_as_longlong(p);
    return (b > 0 && b <= kPi2) || (b > k2Pi && b <= kInf);
  };
  int firstQ4 = 0x7fffffff;
  for (int i = lane; i < Np; i += 32)
    if (q4(S.piph[off + i])) { firstQ4 = min(firstQ4, i); }
  for (int o = 16; o > 0; o >>= 1) firstQ4 = min(firstQ4, __shfl_xor_sync(0xffffffffu, firstQ4, o));
  int I0 = 0x7fffffff;
  for (int i = lane; i < Np; i += 32)
    if (i > firstQ4 && q1(S.piph[off + i])) { I0 = min(I0, i); }
  for (int o = 16; o > 0; o >>= 1) I0 = min(I0, __shfl_xor_sync(0xffffffffu, I0, o));
  if (lane == 0) S.anchor[warp] = (I0 == 0x7fffffff) ? 0 : I0;
}
template <typename R>
__global__ void k_anchor(DevParams P, DevState<R> S, int nring) {
  k_anchor_body<R>(P, S, nring, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- sheared faces, faces_alt.c:36-179 ---------------------------------------
// One block per ring pair.  The reference walks both rings from their anchors,
// advancing the ring whose upper cell edge comes first (ties advance L).  That
// walk is a merge of the two circular sequences; face n sits at merge-path
// state (a, b), a + b = n.  Each thread binary-searches the state at the start
// of its chunk using exact (lap, phi) keys, then walks the chunk with the
// reference's own wrapped comparison.
struct PairInfo {
  int L, R, jL, kL;  // ring ids and (j, k) of the L ring
};

DISCO_D PairInfo pair_info(const DevParams& P, int dim, int pair) {
  PairInfo pi;
  if (dim == 1) {
    int k = div_fast(pair, P.mul_nr1), j = pair - k * (P.Nr - 1);
    pi.L = j + P.Nr * k; pi.R = j + 1 + P.Nr * k; pi.jL = j; pi.kL = k;
  } else {
    int k = div_fast(pair, P.mul_nr), j = pair - k * P.Nr;
    pi.L = j + P.Nr * k; pi.R = j + P.Nr * (k + 1); pi.jL = j; pi.kL = k;
  }
  return pi;
}

// First index in [lo0, hi0] at which the monotone predicate (true ... true,
// false ... false) is false, searched outward from the hint h with doubling
// steps and finished by bisection: O(log |answer - h|) predicate calls.
template <typename F>
DISCO_D int gallop_search(int lo0, int hi0, int h, F&& pred) {
  if (hi0 <= lo0) return lo0;
  if (h < lo0) h = lo0;
  if (h > hi0 - 1) h = hi0 - 1;
  int lo, hi;
  if (pred(h)) {
    lo = h + 1; hi = hi0;
    for (int step = 1;; step <<= 1) {
      int p = h + step;
      if (p >= hi0) break;
      if (!pred(p)) { hi = p; break; }
      lo = p + 1;
    }
  } else {
    lo = lo0; hi = h;
    for (int step = 1;; step <<= 1) {
      int p = h - step;
      if (p < lo0) break;
      if (pred(p)) { lo = p + 1; break; }
      hi = p;
    }
  }
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (pred(mid)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <typename R>
DISCO_D void k_faces_body(const DevParams& P, const DevState<R>& S, int dim, int bx_, int by_) {
  extern __shared__ long long fkeys[];
  const int d = dim - 1;
  int pair = bx_;
  PairInfo pi = pair_info(P, dim, pair);
  int offL = S.ring_off[pi.L], NL = S.ring_off[pi.L + 1] - offL;
  int offR = S.ring_off[pi.R], NR = S.ring_off[pi.R + 1] - offR;
  int I0L = S.anchor[pi.L], I0R = S.anchor[pi.R];
  int Nf = NL + NR;
  int base = S.face_off[d][pair];
  // anchor-rotated upper cell edges of both rings as integer keys
  long long* sL = fkeys;
  long long* sR = fkeys + NL;
  int* sA = (int*)(fkeys + NL + NR);
  signed char* sLR = (signed char*)(sA + NL + NR);
  const double Pmax = P.phi_max;

  for (int m = threadIdx.x; m < NL; m += blockDim.x) {
    int t = I0L + m; t -= t >= NL ? NL : 0;
    sL[m] = phi_key(S.piph[offL + t]);
  }
  for (int m = threadIdx.x; m < NR; m += blockDim.x) {
    int t = I0R + m; t -= t >= NR ? NR : 0;
    sR[m] = phi_key(S.piph[offR + t]);
  }
  __syncthreads();

  // lap offset of R relative to L from the anchors' wrapped comparison
  int offlap = 0;
  {
    double raw = phi_unkey(sL[0]) - phi_unkey(sR[0]);
    if (raw > .5 * Pmax) offlap = 1;
    else if (raw < -.5 * Pmax) offlap = -1;
  }
  const long long A0 = sL[0], B0 = sR[0];
  // key of merge index a (any a >= 0: lap counts completed turns)
  auto keyL = [&](int a, int& lap, long long& ph) {
    int m = a;
    lap = 0;
    while (m >= NL) { m -= NL; ++lap; }
    ph = sL[m];
    lap += (m > 0 && ph < A0) ? 1 : 0;
  };
  auto keyR = [&](int b, int& lap, long long& ph) {
    int m = b;
    lap = offlap;
    while (m >= NR) { m -= NR; ++lap; }
    ph = sR[m];
    lap += (m > 0 && ph < B0) ? 1 : 0;
  };

  int j = pi.jL, k = pi.kL;
  const double* rj = S.r_jph + 1;  // rj[j] == reference r_jph[j]
  const double* zk = S.z_kph + 1;
  const float ratio = (float)NL / (float)Nf;

  // Each face n is found independently: merge-path state (a, b), a + b = n,
  // searched from the proportional guess a ~ n NL / Nf; consecutive threads
  // take consecutive faces so every output array is written coalesced.
  int nerr = 0;
  for (int n = threadIdx.x; n < Nf; n += blockDim.x) {
    int a = gallop_search(0, n, __float2int_rn((float)n * ratio), [&](int mid) {
      int la, lb; long long pa, pb;
      keyL(mid, la, pa);
      keyR(n - 1 - mid, lb, pb);
      return (la < lb) || (la == lb && pa <= pb);
    });
    int b = n - a;
    int am = a - (a >= NL ? NL : 0), bm = b - (b >= NR ? NR : 0);
    if (am >= NL || bm >= NR) { ++nerr; continue; }
    int tL = I0L + am; tL -= tL >= NL ? NL : 0;
    int tR = I0R + bm; tR -= tR >= NR ? NR : 0;
    int iL = offL + tL;
    int iR = offR + tR;
    double pL = phi_unkey(sL[am]), pR = phi_unkey(sR[bm]);
    int gf = base + n;
    S.fL[d][gf] = iL;
    S.fR[d][gf] = iR;
    int LR;
    if constexpr (kMix<R>) {
      // LRtype from the merge order itself (the face ends at whichever upper
      // edge comes first; ties advance L); every offset relative to pL in R
      // from the single FP64 difference pR - pL.
      int la, lb; long long ka, kb;
      keyL(a, la, ka);
      keyR(b, lb, kb);
      LR = ((la < lb) || (la == lb && ka <= kb)) ? 0 : 1;
      const R Pm = (R)Pmax;
      R dLr = S.dphi_r[iL], dRr = S.dphi_r[iR];
      // wrapped in FP64 first: across phi = 0 the raw difference is ~2 pi,
      // where an FP32 rounding would be as large as a sliver face
      R dLR = d2f_int(get_signed_dp_bits(pR, pL, Pmax));
      int LR_back = wrap_signed<R>(dRr - dLr - dLR, Pm) < (R)0 ? 1 : 0;
      R xp = LR == 0 ? (R)0 : dLR;                  // upper edge - pL
      R xm = LR_back == 0 ? -dLr : dLR - dRr;      // lower edge - pL
      R dpr = wrap_dp<R>(xp - xm, Pm);
      R pc = xp - (R).5 * dpr;                     // face centre - pL
      double phic = wrap_pos_bits(pL + f2d_int(pc), Pmax);
      S.fLR[d][gf] = (signed char)LR;
      S.fphic[d][gf] = phic;
      S.fdA[d][gf] = S.pdA[d][pair] * dpr;
      S.fdpL[d][gf] = wrap_signed<R>(pc + (R).5 * dLr, Pm);
      S.fdpR[d][gf] = wrap_signed<R>(dLR - pc - (R).5 * dRr, Pm);
      if (S.ct) {
        S.ffrL[d][gf] = dpr / dLr;
        S.ffrR[d][gf] = dpr / dRr;
        R dp1 = wrap_dp<R>(LR == 0 ? dLR : -dLR, Pm);
        S.fdp1[d][gf] = dp1;
        S.fdp2[d][gf] = (LR == 0 ? dRr : dLr) - dp1;
      }
    } else {
      double dL = S.dphi[iL], dR = S.dphi[iR];
      // LRtype and the face's lower edge: the reference's FP64 comparisons
      double dphi = pL - pR;
      while (dphi > .5 * Pmax) dphi -= Pmax;
      while (dphi < -.5 * Pmax) dphi += Pmax;
      LR = dphi > 0. ? 1 : 0;
      dphi = pL - dL - pR + dR;
      while (dphi > .5 * Pmax) dphi -= Pmax;
      while (dphi < -.5 * Pmax) dphi += Pmax;
      int LR_back = dphi < 0. ? 1 : 0;
      double xp1 = LR == 0 ? pL : pR;
      double xm1 = LR_back == 0 ? pL - dL : pR - dR;
      // addFace, faces_alt.c:10-34
      double dp = get_dp(xp1, xm1, Pmax);
      double phic = get_dp(xp1, .5 * dp, Pmax);
      S.fLR[d][gf] = (signed char)LR;
      S.fphic[d][gf] = phic;
      double dA;
      if (dim == 1) dA = (.5 * (rj[j] + rj[j])) * dp * (zk[k] - zk[k - 1]);
      else dA = (.5 * (rj[j] + rj[j - 1])) * (rj[j] - rj[j - 1]) * dp;
      S.fdA[d][gf] = (R)dA;
      // plm.c:93-96 / riemann.c:127-130 offsets, fixed until the next rebuild
      S.fdpL[d][gf] = (R)get_signed_dp(phic, pL - .5 * dL, Pmax);
      S.fdpR[d][gf] = (R)get_signed_dp(pR - .5 * dR, phic, Pmax);
      if (S.ct) {
        S.ffrL[d][gf] = (R)(dp / dL);   // riemann.c:172-173
        S.ffrR[d][gf] = (R)(dp / dR);
        // avg_Efields weights (bfields.c:461-465): c1 owns the face's end edge
        double p1 = LR == 0 ? pL : pR, p2 = LR == 0 ? pR : pL, dc2 = LR == 0 ? dR : dL;
        double dp1 = get_dp(p2, p1, Pmax);
        S.fdp1[d][gf] = (R)dp1;
        S.fdp2[d][gf] = (R)(dc2 - dp1);
      }
    }
    sLR[n] = (signed char)LR;
    sA[n] = a;
  }
  __syncthreads();
  // the walk must end with both rings consumed exactly once (a = NL, b = NR)
  if (threadIdx.x == 0) {
    int alast = sA[Nf - 1] + (sLR[Nf - 1] == 0 ? 1 : 0);
    if (alast != NL) ++nerr;
  }
  if (nerr) atomicAdd(&S.errs->face_errors, (unsigned long long)nerr);
  // runs: face n starts L's run if the previous face advanced L (circularly)
  for (int n = threadIdx.x; n < Nf; n += blockDim.x) {
    int gf = base + n;
    int prev = sLR[n == 0 ? Nf - 1 : n - 1];
    int cur = sLR[n];
    int iL = S.fL[d][gf], iR = S.fR[d][gf];
    if (prev == 0) S.run_up_s[d][iL] = gf;
    if (cur == 0) { S.run_up_e[d][iL] = gf; S.nb_up[d][iL] = iR; }
    if (prev == 1) S.run_dn_s[d][iR] = gf;
    if (cur == 1) { S.run_dn_e[d][iR] = gf; S.nb_dn[d][iR] = iL; }
  }
}
template <typename R>
__global__ void k_faces(DevParams P, DevState<R> S, int dim) {
  k_faces_body<R>(P, S, dim, (int)blockIdx.x, (int)blockIdx.y);
}

// Iterate the faces of a circular run [s, e] of a pair block [base, base+Nf)
// in ascending face order (the reference's loop order).
template <typename F>
DISCO_D void for_run(int s, int e, int base, int Nf, F&& fn) {
  if (s <= e) {
    for (int f = s; f <= e; ++f) fn(f);
  } else {
    for (int f = base; f <= e; ++f) fn(f);
    for (int f = s; f < base + Nf; ++f) fn(f);
  }
}

// The faces of a run in for_run's order, two at a time: fn(f0, f1, two),
// f1 meaningful only when two (else f1 = f0).  The caller issues both faces'
// loads before it consumes the first, and consumes them in order.
template <typename F>
DISCO_D void for_run2(int s, int e, int base, int Nf, F&& fn) {
  const int first0 = s <= e ? s : base;
  const int n1 = s <= e ? e - s + 1 : e - base + 1;   // faces before the wrap
  const int n = s <= e ? n1 : n1 + (base + Nf - s);
  for (int t = 0; t < n; t += 2) {
    int f0 = t < n1 ? first0 + t : s + (t - n1);
    bool two = t + 1 < n;
    int f1 = t + 1 < n1 ? first0 + t + 1 : s + (t + 1 - n1);
    fn(f0, two ? f1 : f0, two);
  }
}

DISCO_D int pair_above(const DevParams& P, int dim, int j, int k) {
  if (dim == 1) return (j < P.Nr - 1) ? j + (P.Nr - 1) * k : -1;
  return (k < P.Nz - 1) ? j + P.Nr * k : -1;
}
DISCO_D int pair_below(const DevParams& P, int dim, int j, int k) {
  if (dim == 1) return (j > 0) ? (j - 1) + (P.Nr - 1) * k : -1;
  return (k > 0) ? j + P.Nr * (k - 1) : -1;
}

// pair spacing dxL + dxR (faces_alt.c:112-135)
DISCO_D void pair_dx(const DevParams& P, const double* r_jph, const double* z_kph, int dim,
                     int pair, double* dxL, double* dxR) {
  const double* rj = r_jph + 1;
  const double* zk = z_kph + 1;
  if (dim == 1) {
    int j = pair - div_fast(pair, P.mul_nr1) * (P.Nr - 1);
    double rm = centroid_r(rj[j], rj[j - 1]);
    double rp = centroid_r(rj[j + 1], rj[j]);
    *dxL = rj[j] - rm;
    *dxR = rp - rj[j];
  } else {
    int k = div_fast(pair, P.mul_nr);
    double zm = centroid_z(zk[k], zk[k - 1]);
    double zp = centroid_z(zk[k + 1], zk[k]);
    *dxL = zk[k] - zm;
    *dxR = zp - zk[k];
  }
}

// Static per-ring radii, computed once with the path's rounding.
template <typename R>
__global__ void k_ring_geom(DevParams P, DevState<R> S, int nring) {
  int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= nring) return;
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  double rp = S.r_jph[j + 1], rm = S.r_jph[j];
  double zp = S.z_kph[k + 1], zm = S.z_kph[k];
  S.ring_rc[jk] = centroid_r(rp, rm);
  S.ring_r23[jk] = (rp * rp + rp * rm + rm * rm) / 3.;
  double r1 = .5 * (rp + rm), dr = rp - rm, dz = zp - zm;
  S.ring_rc_r[jk] = (R)centroid_r(rp, rm);
  S.ring_r1_r[jk] = (R)r1;
  S.ring_vol_r[jk] = (R)(r1 * dr * dz);
  S.ring_dA_r[jk] = (R)(dr * dz);
  S.ring_r23_r[jk] = (R)((rp * rp + rp * rm + rm * rm) / 3.);
  S.ring_zc_r[jk] = (R)centroid_z(zp, zm);
  double Om = S.ring_Om[jk], rc = centroid_r(rp, rm);
  S.ring_Om_r[jk] = (R)Om;
  S.ring_Lsh[jk] = Om * rc * rc;
  S.ring_gL_r[jk] = (R)(Om * (rc - rm));
  S.ring_gR_r[jk] = (R)(Om * (rc - rp));
  // total face area per unit dphi, one side only at the domain's edge rings
  double atr = (rp + rm) * dz, atz = 2. * r1 * dr;
  if (j == 0) atr = rp * dz;
  if (j == P.Nr - 1) atr = rm * dz;
  if (k == 0 || k == P.Nz - 1) atz = r1 * dr;
  S.ring_At_r[0][jk] = (R)atr;
  S.ring_At_r[1][jk] = (R)atz;
  S.ring_dl_r[0][jk] = (R)dz;
  S.ring_dl_r[1][jk] = (R)dr;
  // CFL extents in FP64: .5 (rp + rm) (times dphi: r dphi), 1 / dr, 1 / dz
  S.ring_cfl[3 * jk + 0] = r1;
  S.ring_cfl[3 * jk + 1] = 1.0 / dr;
  S.ring_cfl[3 * jk + 2] = 1.0 / dz;
}

// Static per-pair geometry (faces_alt.c:112-135, the face radius cm[0]).
template <typename R>
__global__ void k_pair_geom(DevParams P, DevState<R> S, int dim, int npair) {
  int pair = blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= npair) return;
  const int d = dim - 1;
  double dxL, dxR;
  pair_dx(P, S.r_jph, S.z_kph, dim, pair, &dxL, &dxR);
  const double* rj = S.r_jph + 1;
  int pj = pair % (dim == 1 ? (P.Nr - 1) : P.Nr);
  double r = dim == 1 ? .5 * (rj[pj] + rj[pj]) : centroid_r(rj[pj], rj[pj - 1]);
  S.pdxL[d][pair] = (R)dxL;
  S.pdxR[d][pair] = (R)dxR;
  S.pdxs[d][pair] = (R)(dxR + dxL);
  S.prad[d][pair] = (R)r;
  S.pidxs[d][pair] = (R)1 / (R)(dxR + dxL);
  int pk = pair / (dim == 1 ? (P.Nr - 1) : P.Nr);
  const double* zk = S.z_kph + 1;
  double a = dim == 1 ? (.5 * (rj[pj] + rj[pj])) * (zk[pk] - zk[pk - 1])
                      : (.5 * (rj[pj] + rj[pj - 1])) * (rj[pj] - rj[pj - 1]);
  S.pdA[d][pair] = (R)a;
  PairInfo pi = pair_info(P, dim, pair);
  double dOm = S.ring_Om[pi.R] - S.ring_Om[pi.L];
  S.pdOm[d][pair] = (R)dOm;
  S.pcX[d][pair] = (R)((dim == 1 ? -dOm : dOm) * r);
}

// ---- plm_trans, plm.c:56-195 ------------------------------------------------
// Two passes, as the reference's own face loop: k_plm_slopes computes every
// face's slope S = (W_R - W_L) / (dxL + dxR) once (plm.c:87-110), then
// k_plm_trans gathers each cell's faces in the reference's order: sum S dA,
// divide by the total area, limit.  The reference limiter loop
// (plm.c:146-179) reduces to: zero if any face slope has the opposite sign
// (or is zero), else the smallest of |g| and |PLM S| -- a function of the
// extremes of PLM S over the faces only, independent of face order.
constexpr int kSlopeFaces = 4;   // faces per thread in k_plm_slopes (loads in flight)

template <typename R, int NQ>
DISCO_D void k_plm_slopes_body(const DevParams& P, const DevState<R>& S, int dim, int bx_, int by_) {
  const int d = dim - 1;
  int pair = bx_;
  int base = S.face_off[d][pair], Nf = S.face_off[d][pair + 1] - base;
  const int N = S.N, NF = S.nf[d];
  R dxs = S.pdxs[d][pair];
  R idxs = kMix<R> ? S.pidxs[d][pair] : (R)0;
  R dOm = kMix<R> ? S.pdOm[d][pair] : (R)0;
#pragma unroll
  for (int u = 0; u < kSlopeFaces; ++u) {
    int n = (by_ * kSlopeFaces + u) * blockDim.x + threadIdx.x;
    if (n >= Nf) break;
    int f = base + n;
    int cL = S.fL[d][f], cR = S.fR[d][f];
    R dpL = S.fdpL[d][f], dpR = S.fdpR[d][f];
    // every component's reconstructed pair before the first store: the
    // stores may alias the inputs as far as the compiler knows, so loads
    // placed after one would wait for it
    R WL[NQ], WR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      WL[q] = S.prim[q * N + cL] + dpL * S.gradp[q * N + cL];
      WR[q] = S.prim[q * N + cR] - dpR * S.gradp[q * N + cR];
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      R Sl;
      if constexpr (kMix<R>) Sl = ((WR[q] - WL[q]) + (q == UPP ? dOm : (R)0)) * idxs;   // frames of the rings
      else Sl = (WR[q] - WL[q]) / dxs;
      S.fslope[(size_t)q * NF + f] = Sl;
    }
  }
}
template <typename R, int NQ>
__global__ void k_plm_slopes(DevParams P, DevState<R> S, int dim) {
  k_plm_slopes_body<R, NQ>(P, S, dim, (int)blockIdx.x, (int)blockIdx.y);
}

// The components are independent: blockIdx.y selects a group of QPT of them.
constexpr int kPlmQ = 9;        // components per thread in k_plm_trans (one group for NQ <= 9)
constexpr int kTileCells = 128; // cells per block of a tiled face gather
constexpr int kTileCap = 4 * kTileCells;   // faces staged per side
template <int NQ>
constexpr int plm_groups() { return (NQ + kPlmQ - 1) / kPlmQ; }

// The faces where consecutive cells of a ring are L (or R) form one circular
// interval of the pair's face block, because the merge walk assigns faces to
// the cells of each ring in ring order.  A block takes kTileCells consecutive
// cells of one ring, stages that interval's face data in shared memory with
// coalesced loads, and each thread then walks its own run in the reference's
// order from shared memory.
template <typename R, int NQ>
DISCO_D void k_plm_trans_body(const DevParams& P, const DevState<R>& S, int dim, int bx_, int by_) {
  constexpr int QPT = kPlmQ;
  constexpr int NG = plm_groups<NQ>();
  // components of this block: [q0, q0 + QPT) within NQ (q0 = 0 at compile
  // time for a single group)
  constexpr int QB = NG == 1 ? NQ : QPT;
  __shared__ R sS[QB][kTileCap];
  __shared__ R sA[kTileCap];
  __shared__ int rng[2];
  const int item = bx_;
  const int q0 = NG == 1 ? 0 : by_ * QPT;
  const int d = dim - 1;
  const int N = S.N, NF = S.nf[d];
  const int jk = S.chunk_ring[item], i0 = S.chunk_i0[item];
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const int i1 = min(Np, i0 + kTileCells);
  const int i = i0 + threadIdx.x;
  const bool valid = i < i1;
  const int c = off + i;
  const int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  R* grad = dim == 1 ? S.gradr : S.gradz;
  const R PLM = PRM(R, P, PLM);
  if (PLM == (R)0) {
    if (valid)
#pragma unroll
      for (int t = 0; t < QB; ++t)
        if (q0 + t < NQ) grad[(q0 + t) * N + c] = 0;
    return;
  }
  // The limiter needs only the extremes of PLM S over the faces: for g > 0
  // it is zero if any PLM S <= 0, else min(g, min PLM S); for g < 0
  // symmetric.  Rounding is monotonic, so min(PLM S) = PLM min(S) exactly
  // for PLM > 0 (max for PLM < 0): the extremes of S are tracked and scaled
  // once.
  R sum[QB], mn[QB], mx[QB];
#pragma unroll
  for (int t = 0; t < QB; ++t) {
    sum[t] = 0;
    mn[t] = (R)INFINITY;
    mx[t] = -(R)INFINITY;
  }
  auto take = [&](int t, R Sl, R dA) {
    sum[t] += Sl * dA;
    mn[t] = fmin(mn[t], Sl);
    mx[t] = fmax(mx[t], Sl);
  };

  for (int side = 0; side < 2; ++side) {   // pair below (cell is R), then above (cell is L)
    const int p = side == 0 ? pair_below(P, dim, j, k) : pair_above(P, dim, j, k);
    if (p < 0) continue;                    // uniform over the block (one ring)
    const int base = S.face_off[d][p], Nf = S.face_off[d][p + 1] - base;
    const int* rs = side == 0 ? S.run_dn_s[d] : S.run_up_s[d];
    const int* re = side == 0 ? S.run_dn_e[d] : S.run_up_e[d];
    if (threadIdx.x == 0) {
      int st = rs[off + i0], en = re[off + i1 - 1];
      int dd = en - st;
      if (dd < 0) dd += Nf;
      rng[0] = st;
      rng[1] = dd + 1;
    }
    __syncthreads();
    const int st = rng[0], cnt = rng[1];
    if (cnt <= kTileCap) {   // uniform over the block
      for (int t = threadIdx.x; t < cnt; t += kTileCells) {
        int f = st + t;
        if (f >= base + Nf) f -= Nf;
        sA[t] = S.fdA[d][f];
#pragma unroll
        for (int u = 0; u < QB; ++u)
          if (q0 + u < NQ) sS[u][t] = S.fslope[(size_t)(q0 + u) * NF + f];
      }
      __syncthreads();
      if (valid) {
        for_run(rs[c], re[c], base, Nf, [&](int f) {
          int o = f - st;
          if (o < 0) o += Nf;
          R dA = sA[o];
#pragma unroll
          for (int t = 0; t < QB; ++t)
            if (q0 + t < NQ) take(t, sS[t][o], dA);
        });
      }
    } else if (valid) {
      for_run(rs[c], re[c], base, Nf, [&](int f) {
        R dA = S.fdA[d][f];
#pragma unroll
        for (int t = 0; t < QB; ++t)
          if (q0 + t < NQ) take(t, S.fslope[(size_t)(q0 + t) * NF + f], dA);
      });
    }
    __syncthreads();
  }
  if (!valid) return;
#pragma unroll
  for (int t = 0; t < QB; ++t) {
    R a = PLM * mn[t], b = PLM * mx[t];
    mn[t] = PLM > (R)0 ? a : b;
    mx[t] = PLM > (R)0 ? b : a;
  }

  // total weight, plm.c:113-143
  R dAt, idAt = 0;
  if constexpr (kMix<R>) {
    dAt = S.ring_At_r[d][jk] * S.dphi_r[c];
    idAt = (R)1 / dAt;
  } else {
    const double Pmax = P.phi_max;
    const double* rj = S.r_jph + 1;
    const double* zk = S.z_kph + 1;
    double phip = S.piph[c], phim = phip - S.dphi[c];
    double dph = get_dp(phip, phim, Pmax);
    double dAp, dAm;
    if (dim == 1) {
      double dz = zk[k] - zk[k - 1];
      dAp = (.5 * (rj[j] + rj[j])) * dph * dz;
      dAm = (.5 * (rj[j - 1] + rj[j - 1])) * dph * dz;
    } else {
      double dr = rj[j] - rj[j - 1];
      double r = .5 * (rj[j] + rj[j - 1]);
      dAp = r * dr * dph;
      dAm = r * dr * dph;
    }
    double dAtot = dAp + dAm;
    int idx = dim == 1 ? j : k;
    int nmax = dim == 1 ? P.Nr : P.Nz;
    if (idx == 0) dAtot = dAp;
    if (idx == nmax - 1) dAtot = dAm;
    dAt = (R)dAtot;
  }

  bool geom_bd = (dim == 1 && j == 0 && P.geom_bd_r);
  R rcen = kMix<R> ? S.ring_rc_r[jk] : (R)S.ring_rc[jk];
#pragma unroll
  for (int t = 0; t < QB; ++t) {
    const int q = q0 + t;
    if (q >= NQ) break;
    R g;
    if constexpr (kMix<R>) g = sum[t] * idAt;
    else g = sum[t] / dAt;
    if (g > (R)0) {
      if (!(mn[t] > (R)0)) g = 0;
      else if (mn[t] < g) g = mn[t];
    } else if (g < (R)0) {
      if (!(mx[t] < (R)0)) g = 0;
      else if (mx[t] > g) g = mx[t];
    }
    if (geom_bd) {  // plm_geom_boundary + geom_grad, cylindrical.c:141-173
      if (q == URR || (P.num_c > BZZ && q == BRR)) {
        R SL = S.prim[q * N + c] / rcen;
        if (g * SL < (R)0) g = 0;
        else if (fabs(PLM * SL) < fabs(g)) g = PLM * SL;
      } else {
        g = 0;
      }
    }
    grad[q * N + c] = g;
  }
}
template <typename R, int NQ>
__global__ void __launch_bounds__(kTileCells) k_plm_trans(DevParams P, DevState<R> S, int dim) {
  k_plm_trans_body<R, NQ>(P, S, dim, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- cooling (sink.c:274-326) and damping (sink.c:329-427) of one cell -----
// add_source runs them first (misc.c:579-580).  x is the cell centroid; the
// planets' summed |f|/|x - x_p| (mode-1 forces) sets the orbital rate of the
// beta cooling and of the type-2 damping times.  Damping relaxes DDD, SRR,
// LLL, SZZ and TAU towards initial() with expm1(-dt f), f the damping
// factor of the last active side (the reference's ratetot is unused).
template <typename Phys, typename R, int NQ>
DISCO_D void cool_damp_src(const DevParams& P, const DevPlanet* pl, const R* prim, double* U,
                           const double* xp, const double* xm, double dV, double dt) {
  const double x[3] = {centroid_r(xp[0], xm[0]), .5 * (xp[1] + xm[1]), centroid_z(xp[2], xm[2])};
  auto orbital = [&]() {
    const double gx = x[0] * cos(x[1]), gy = x[0] * sin(x[1]);
    double omtot = 0.0;
    for (int p = 0; p < P.Npl; ++p) {
      const double px = pl[p].r * cos(pl[p].phi), py = pl[p].r * sin(pl[p].phi);
      const double dx = gx - px, dy = gy - py;
      const double mag = sqrt(dx * dx + dy * dy);
      double fr, fp, fz;
      planetary_force<double>(P, pl[p], x[0], x[1], x[2], &fr, &fp, &fz, 1);
      omtot += sqrt(fr * fr + fp * fp + fz * fz) / mag;
    }
    return sqrt(omtot);
  };
  if (P.cool_type == 1 || P.cool_type == 2) {   // COOL_BETA, COOL_BETA_RELAX
    const double press = prim[PPP], rho = prim[RHO];
    const double gm1 = P.gamma_law - 1.0;
    const double enTarget = get_cs2<double>(P, pl, x[0], x[1]) / (P.gamma_law * gm1);
    const double enCurrent = press / (rho * gm1);
    if (P.cool_type == 2 || enCurrent > enTarget) {
      const double omtot = orbital();
      const double Tm1 = expm1(-dt * omtot / P.cool_beta);
      U[TAU] += rho * dV * (enCurrent - enTarget) * Tm1;
    }
  }
  if (P.damp_type[0] + P.damp_type[1] + P.damp_type[2] + P.damp_type[3] > 0) {
    // inner, outer, upper, lower (upper and lower only in 3D); both z sides
    // measure from the upper edge, as the reference does.  The damping times
    // (and the orbital rate of type 2) enter only the reference's unused
    // ratetot, so they play no part here.
    double dampFactor = 0.0;
    for (int side = 0; side < 4; ++side) {
      if (P.damp_type[side] <= 0 || (side >= 2 && P.twoD)) continue;
      const double theta = side == 0 ? (x[0] - P.dom_rmin) / P.damp_len[0]
                         : side == 1 ? (P.dom_rmax - x[0]) / P.damp_len[1]
                                     : (P.dom_zmax - x[2]) / P.damp_len[side];
      const bool rising = side == 1 || side == 2;   // outer, upper: pow(1 - theta^2, 2)
      if (theta > 1.0) dampFactor = 0.0;
      else dampFactor = rising ? pow(1.0 - pow(theta, 2.0), 2.0) : 1.0 - pow(1.0 - pow(theta, 2.0), 2.0);
    }
    dampFactor = expm1(-dt * dampFactor);
    double p0[MAX_Q];
    initial_raw(P, p0, x);
    R p0r[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) p0r[q] = (R)p0[q];
    double c0[NQ], c1[NQ];
    Phys::template prim2cons<double>(P, p0r, c0, (R)x[0], (R)dV);
    Phys::template prim2cons<double>(P, prim, c1, (R)x[0], (R)dV);
    U[DDD] += (c1[DDD] - c0[DDD]) * dampFactor;
    U[SRR] += (c1[SRR] - c0[SRR]) * dampFactor;
    U[LLL] += (c1[LLL] - c0[LLL]) * dampFactor;
    U[SZZ] += (c1[SZZ] - c0[SZZ]) * dampFactor;
    U[TAU] += (c1[TAU] - c0[TAU]) * dampFactor;
  }
}

// sink_src (sink.c:105-247), the last term of add_source: the gas nozzle
// (Nozzle_Type 1) and the accreting sinks of the first sink_bodies bodies
// (Sink_Type 1 compact polynomial, 2 exponential, 3 top hat).  A cell
// outside the nozzle takes neither term, as in the reference (its early
// return).  U gets the cell's changes; acc, when given, gets the cell's
// share of each sink body's accumulators (SA_*).  The reference's
// fmin(Sink_Par2, 1) is overwritten by fmax(0, Sink_Par2), so delta is the
// latter.
template <typename R>
DISCO_D void sink_src(const DevParams& P, const DevPlanet* pl, const R* prim, double* U, const double* xp,
                      const double* xm, double dV, double dt, double* acc) {
  if (P.nozzle_type == 1) {
    const double r = .5 * (xp[0] + xm[0]);
    double phi = .5 * (xp[1] + xm[1]);
    const double z = .5 * (xp[2] + xm[2]);
    if (phi > M_PI) phi -= 2 * M_PI;
    const double R0 = P.nozzle_par[0], dR = P.nozzle_par[1], v = P.nozzle_par[2], mach = P.nozzle_par[3];
    const double d2 = (r - R0) * (r - R0) + r * r * phi * phi + z * z;
    if (d2 > dR * dR) return;
    double rhodot = 1.0 * 3.0 / (4.0 * M_PI * dR * dR * dR);
    if (P.twoD) rhodot *= 2 * sqrt(dR * dR - (r - R0) * (r - R0) - r * r * phi * phi);
    if (rhodot * dV * dt > U[RHO]) rhodot = U[RHO] / dV * dt;
    const double om = get_om<double>(P, r);
    const double cs2 = v * v / (mach * mach);
    const double eps = cs2 / (P.gamma_law * (P.gamma_law - 1));
    U[RHO] += rhodot * dV * dt;
    U[LLL] += rhodot * r * v * dV * dt;
    U[TAU] += (0.5 * rhodot * (v - r * om) * (v - r * om) + rhodot * eps) * dV * dt;
    if (P.num_q > P.num_c) U[P.num_c] += rhodot * dV * dt;
  }
  if (P.sink_type == 0) return;
  const double r = centroid_r(xp[0], xm[0]), phi = .5 * (xp[1] + xm[1]);
  const double rho = prim[RHO], vr = prim[URR], vp = (double)prim[UPP] * r, vz = prim[UZZ], pres = prim[PPP];
  const double cosg = cos(phi), sing = sin(phi);
  const double gx = r * cosg, gy = r * sing;
  const double delta = fmax(0.0, P.sink_par[1]);
  const double gm1 = P.gamma_law - 1.0;
  for (int b = 0; b < P.sink_bodies; ++b) {
    const DevPlanet& q = pl[b];
    const double cosp = cos(q.phi), sinp = sin(q.phi);
    const double dx = gx - q.r * cosp, dy = gy - q.r * sinp;
    const double mag = sqrt(dx * dx + dy * dy);
    double arg = 0.0;
    if (P.sink_type == 3) {
      if (mag <= P.sink_par[2]) arg = 1.0;
    } else if (P.sink_type == 2) {
      const double eps = pow(P.sink_par[2], P.sink_par[3]);
      const double ef = P.sink_par[4] <= 0.0 ? 1.0 : P.sink_par[4];
      arg = exp(-pow(mag, P.sink_par[3]) / (eps * ef));
    } else if (P.sink_type == 1) {
      const double eps = P.sink_par[2];
      arg = pow(1.0 - pow(mag / eps, P.sink_par[3]), P.sink_par[4]);
      if (mag >= eps) arg = 0.0;
    }
    const double surfdiff = rho * (P.sink_par[0] * q.omega) * arg;
    // the gas velocity relative to the body, its radial part kept and its
    // azimuthal part (about the body) removed in proportion delta
    const double vpp = q.r * q.omega;
    const double vxp = q.vr * cosp - vpp * sinp, vyp = q.vr * sinp + vpp * cosp;
    double vxg = vr * cosg - vp * sing, vyg = vr * sing + vp * cosg;
    const double vxr = vxg - vxp, vyr = vyg - vyp;
    const double cphi = dx / mag, sphi = dy / mag;
    const double af = dV * dt * surfdiff;
    const double vpr = cphi * vyr - sphi * vxr;
    const double vxn = (cphi * cphi + (1.0 - delta) * sphi * sphi) * vxr + delta * sphi * cphi * vyr;
    const double vyn = delta * cphi * sphi * vxr + (sphi * sphi + (1.0 - delta) * cphi * cphi) * vyr;
    vxg = vxn + vxp;
    vyg = vyn + vyp;
    double vgr = vxg * cosg + vyg * sing, vgp = -vxg * sing + vyg * cosg;
    const double accL = vgp * r * af;
    U[RHO] -= af;
    if (delta == 0.0) { vgr = vr; vgp = vp; }
    U[URR] -= vgr * af;
    U[UPP] -= r * vgp * af;
    U[UZZ] -= vz * af;
    const double v2 = vgp * vgp + vgr * vgr + vz * vz;
    U[PPP] -= af * (0.5 * v2 + pres / (rho * gm1));
    if (acc) {
      double fr, fp, fz;
      planetary_force<double>(P, q, r, phi, 0.0, &fr, &fp, &fz, 1);
      const double rho0 = 1.0 / (3.0 * M_PI * P.explicit_viscosity);
      double* a = acc + b * kSinkAcc;
      a[SA_LS] += (1.0 - delta) * mag * vpr * af;
      a[SA_ACCL] += accL;
      a[SA_DM] += af;
      a[SA_KIN] += 0.5 * v2 * af;
      a[SA_THERM] += pres * af / (rho * gm1);
      a[SA_XMOM] += af * vxg;
      a[SA_YMOM] += af * vyg;
      a[SA_GRAVL] -= (rho - rho0) * q.r * fp * dV * dt;
    }
  }
}

// The sink bodies' accumulators over this substep's real cells, from the
// state add_source sees (the primitives and positions before the update):
// each block's partial sums, by a fixed tree, to part[block].
template <typename Phys, typename R, int NQ>
__global__ void __launch_bounds__(256) k_sink_acc(DevParams P, DevState<R> S, double fac) {
  constexpr int NA = MAX_PL * kSinkAcc;
  __shared__ double red[8][NA];
  double acc[NA];
#pragma unroll
  for (int q = 0; q < NA; ++q) acc[q] = 0.0;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < S.N) {
    const int jk = S.cell_ring[c];
    const int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
    if (is_real(P, j, k)) {
      const double* rj = S.r_jph + 1;
      const double* zk = S.z_kph + 1;
      const double piph = S.piph[c], dphi = S.dphi[c];
      const double xp[3] = {rj[j], piph, zk[k]};
      const double xm[3] = {rj[j - 1], piph - dphi, zk[k - 1]};
      const double dV = (.5 * (xp[0] + xm[0])) * (xp[0] - xm[0]) * get_dp(xp[1], xm[1], P.phi_max) * (xp[2] - xm[2]);
      const double dt = fac * S.scal[SC_DT];
      R pr[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * S.N + c];
      if constexpr (kMix<R>) pr[UPP] += S.ring_Om_r[jk];   // lab omega
      double U[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) U[q] = 0.0;
      U[RHO] = 1.0e300;   // no nozzle cap from here: only acc is kept
      sink_src<R>(P, S.planets, pr, U, xp, xm, dV, dt, acc);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < NA) {
    double v = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v += red[i][threadIdx.x];
    S.sink_part[(size_t)blockIdx.x * NA + threadIdx.x] = v;
  }
}

// adjust_RK_planets_aux (misc.c:258-264, planet.c:261-270) and the sum of
// this substep's contributions: acc = (1 - RK) acc + RK acc_RK + the block
// partials in block order.  The first substep first copies acc to acc_RK
// (planet_RK_copy at the start of timestep, timestep.c:25-27).
static __global__ void k_sink_final(double* sink_acc, const double* part, int nblocks, double RK, int first,
                                    int nbody) {
  constexpr int NA = MAX_PL * kSinkAcc;
  const int t = threadIdx.x;
  if (t >= nbody * kSinkAcc) return;
  double* cur = sink_acc;
  double* rk = sink_acc + NA;
  if (first) rk[t] = cur[t];
  double a = (1. - RK) * cur[t] + RK * rk[t];
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * NA + t];
  cur[t] = a + s;
}

// Occupancy: on the mixed path the flux and update kernels are capped at
// 64 registers per thread (4 blocks of 256 per SM), measured faster than
// their natural 70+; the FP64 versions would spill, so they are not capped.

// ---- phi fluxes, misc.c:378-436 + riemann_phi, riemann.c:39-112 -------------
// The phi face between cell c and its successor cp of ring jk (j, k), from
// their primitives pC, pP, phi gradients gC, gP and widths dL, dR: the
// reconstruction, the Riemann solve, the face flux into fphi and, with
// constrained transport, the edge EMFs.  Shared by k_flux_phi and the
// staged sweep k_phi_sweep.
template <typename Phys, typename R, int NQ>
DISCO_D void flux_phi_face(const DevParams& P, const DevState<R>& S, double fac, int c, int cp, int jk, int j, int k,
                           const R* pC, const R* pP, const R* gC, const R* gP, R dL, R dR) {
  const int N = S.N;
  R r, dAdt_r = 0;
  double dAdt = 0;
  if constexpr (kMix<R>) {
    r = S.ring_rc_r[jk];
    dAdt_r = S.ring_dA_r[jk] * ((R)fac * dt_r<R>(S.scal));
  } else {
    const double* rj = S.r_jph + 1;
    const double* zk = S.z_kph + 1;
    double rp = rj[j], rm = rj[j - 1], zp = zk[k], zm = zk[k - 1];
    r = S.ring_rc[jk];
    double dA = (rp - rm) * (zp - zm);         // get_dA(.., 0) = dr dz
    dAdt = dA * (fac * S.scal[SC_DT]);
  }
  // the face angle enters the Riemann solver through the viscous flux only
  double phi = P.include_viscosity ? S.piph[c] : 0.0;
  R primL[NQ], primR[NQ], gp[NQ], gLr[NQ], gLz[NQ], gRr[NQ], gRz[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    R pL = pC[q], pR = pP[q];
    primL[q] = pL + (R).5 * gC[q] * dL;
    primR[q] = pR - (R).5 * gP[q] * dR;
    gp[q] = (pR - pL) / ((R)0.5 * (dR + dL));
  }
  if (P.include_viscosity) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      gLr[q] = S.gradr[q * N + c]; gLz[q] = S.gradz[q * N + c];
      gRr[q] = S.gradr[q * N + cp]; gRz[q] = S.gradz[q * N + cp];
    }
  }
  if (Phys::MHD) {
    R Bp = (R).5 * (primL[BPP] + primR[BPP]);
    primL[BPP] = Bp; primR[BPP] = Bp;
  }
  R n[3] = {0, 1, 0};
  R hn = (R)r;
  R Fw[NQ], Fl[NQ], Us[NQ];
  if constexpr (kMix<R>) {
    // Riemann problem in the ring frame: mesh speed and energy frame
    // relative to Om, then Fw back to the lab (the mass flux through the
    // moving face is frame invariant; L and, for the total energy of the
    // MHD module, TAU pick up the frame's share).
    R Om = S.ring_Om_r[jk];
    R w = hn * (R)(S.wiph[c] - S.ring_Om[jk]);
    solve_riemann<Phys, R, NQ>(P, S.planets, primL, primR, gLr, gp, gLz, gRr, gp, gRz, r,
                               (R)phi, n, w, Fw, Fl, Us, Om);
    R Omr2 = Om * r * r;
    if (Phys::MHD) Fw[TAU] += Om * Fw[LLL] + (R).5 * Om * Omr2 * Fw[DDD];
    Fw[LLL] += Omr2 * Fw[DDD];
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.fphi[q * N + c] = Fw[q] * dAdt_r;
  } else if constexpr (Phys::GR) {   // x = (centroid r, phi, centroid z), misc.c:396-411
    const double* zk = S.z_kph + 1;
    const double xg[3] = {r, S.piph[c], .5 * (zk[k] + zk[k - 1])};
    const double nd[3] = {0.0, 1.0, 0.0};
    solve_riemann_gr<Phys, NQ>(P, primL, primR, xg, nd, (double)(hn * S.wiph[c]), Fw);
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.fphi[q * N + c] = (R)((double)Fw[q] * dAdt);
  } else {
    R w = hn * (R)S.wiph[c];
    solve_riemann<Phys, R, NQ>(P, S.planets, primL, primR, gLr, gp, gLz, gRr, gp, gRz, (R)r,
                               (R)phi, n, w, Fw, Fl, Us);
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.fphi[q * N + c] = (R)((double)Fw[q] * dAdt);
  }
  if constexpr (!Phys::GR) if (S.ct) {   // riemann.c:86-111 (NUM_EDGES == 8)
    R Ez, Br, Er, Bz;
    Phys::flux_to_E(Fl, Us, (R)r, &Ez, &Br, &Er, &Bz, 0);
    R hEz = (R).5 * Ez, hBr = (R).5 * Br, hEr = (R).5 * Er, hBz = (R).5 * Bz;
    if constexpr (kMix<R>) {
      // ring-frame EMFs X = E + s h Om B (s = -1 on r edges, +1 on z edges);
      // the Er slots reduce to the frame-relative value exactly
      R hEzL = (R).5 * (Ez + S.ring_gL_r[jk] * Br), hEzR = (R).5 * (Ez + S.ring_gR_r[jk] * Br);
      S.Eraw[0 * N + c] = hEzL; S.Eraw[1 * N + c] = hEzR; S.Eraw[2 * N + cp] = hEzL; S.Eraw[3 * N + cp] = hEzR;
    } else {
      S.Eraw[0 * N + c] = hEz; S.Eraw[1 * N + c] = hEz; S.Eraw[2 * N + cp] = hEz; S.Eraw[3 * N + cp] = hEz;
    }
    S.Braw[0 * N + c] = hBr; S.Braw[1 * N + c] = hBr; S.Braw[2 * N + cp] = hBr; S.Braw[3 * N + cp] = hBr;
    S.Eraw[4 * N + c] = hEr; S.Eraw[5 * N + c] = hEr; S.Eraw[6 * N + cp] = hEr; S.Eraw[7 * N + cp] = hEr;
    S.Braw[4 * N + c] = hBz; S.Braw[5 * N + c] = hBz; S.Braw[6 * N + cp] = hBz; S.Braw[7 * N + cp] = hBz;
  }
}

template <typename Phys, typename R, int NQ>
DISCO_D void k_flux_phi_body(const DevParams& P, const DevState<R>& S, double fac, int bx_, int by_) {
  int c = bx_ * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (S.ct ? !ring_in_phi_range(P, j, k) : !is_real(P, j, k)) return;
  const int N = S.N;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  int cp = off + (i < Np - 1 ? i + 1 : 0);
  R pC[NQ], pP[NQ], gC[NQ], gP[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    pC[q] = S.prim[q * N + c]; pP[q] = S.prim[q * N + cp];
    gC[q] = S.gradp[q * N + c]; gP[q] = S.gradp[q * N + cp];
  }
  flux_phi_face<Phys, R, NQ>(P, S, fac, c, cp, jk, j, k, pC, pP, gC, gP, S.dphi_r[c], S.dphi_r[cp]);
}
template <typename Phys, typename R, int NQ>
__global__ void __launch_bounds__(256, kMix<R> ? 4 : 1) k_flux_phi(DevParams P, DevState<R> S, double fac) {
  k_flux_phi_body<Phys, R, NQ>(P, S, fac, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- r/z fluxes, misc.c:441-519 + riemann_trans, riemann.c:114-214 ----------
// Grid: x = pair within the active range, y = chunk of 256 faces.
// One face of the r / z flux sweep (misc.c:441-519, riemann.c:114-214):
// reconstruction at the face from the two cells' primitives and gradients,
// the Riemann solve, the fluxes times dA dt, and the CT face terms.  ld(s, q,
// &p, &gp, &gd) gives cell s's (0: L, 1: R) component q: primitive, phi
// gradient and gradient across the face.
template <typename Phys, typename R, int NQ, typename Load>
DISCO_D void flux_trans_face(const DevParams& P, const DevState<R>& S, int dim, int pair, int pj, int pk, int f,
                             int cL, int cR, double fac, Load&& ld) {
  const int d = dim - 1;
  const int N = S.N;
  // the face angle enters the Riemann solver through the viscous flux only
  R phi = P.include_viscosity ? (R)S.fphic[d][f] : (R)0;
  R dpL = S.fdpL[d][f], dpR = S.fdpR[d][f];
  R rdxL = S.pdxL[d][pair], rdxR = S.pdxR[d][pair];
  R ridxs = kMix<R> ? S.pidxs[d][pair] : (R)0;
  R primL[NQ], primR[NQ], grad[NQ];
  R gLp[NQ], gRp[NQ], gLo[NQ], gRo[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    R pL, gpL, gdL, pR, gpR, gdR;
    ld(0, q, &pL, &gpL, &gdL);
    ld(1, q, &pR, &gpR, &gdR);
    primL[q] = pL + gdL * rdxL + gpL * dpL;
    primR[q] = pR - gdR * rdxR - gpR * dpR;
    if constexpr (kMix<R>) grad[q] = ((pR - gpR * dpR) - (pL + gpL * dpL)) * ridxs;
    else grad[q] = ((pR - gpR * dpR) - (pL + gpL * dpL)) / (rdxL + rdxR);
    gLp[q] = gpL; gRp[q] = gpR;
  }
  R OmL = 0;
  if constexpr (kMix<R>) {   // the R cell's omega into the L ring's frame
    R dOm = S.pdOm[d][pair];
    primR[UPP] += dOm;
    grad[UPP] += dOm * ridxs;
    OmL = S.ring_Om_r[pj + P.Nr * pk];   // the pair's L ring
  }
  if (P.include_viscosity) {
    const R* go = dim == 1 ? S.gradz : S.gradr;
#pragma unroll
    for (int q = 0; q < NQ; ++q) { gLo[q] = go[q * N + cL]; gRo[q] = go[q * N + cR]; }
  }
  R n3[3] = {0, 0, 0};
  if (dim == 1) n3[0] = 1; else n3[2] = 1;
  if (Phys::MHD) {
    int BT = dim == 1 ? BRR : BZZ;
    R Bavg = (R).5 * (primL[BT] + primR[BT]);
    primL[BT] = Bavg; primR[BT] = Bavg;
  }
  // face x = cm: r is the face radius for r faces, the centroid for z faces
  R r = S.prad[d][pair];
  R Fw[NQ], Fl[NQ], Us[NQ];
  if constexpr (Phys::GR) {
    // face centre cm (faces_alt.c:10-20): z mid-layer on r faces, the face's z on z faces
    const double* zk = S.z_kph + 1;
    const double xg[3] = {r, S.fphic[d][f], dim == 1 ? .5 * (zk[pk] + zk[pk - 1]) : zk[pk]};
    const double nd[3] = {n3[0], n3[1], n3[2]};
    solve_riemann_gr<Phys, NQ>(P, primL, primR, xg, nd, 0.0, Fw);
    (void)Fl; (void)Us;
  } else if (dim == 1) {
    solve_riemann<Phys, R, NQ>(P, S.planets, primL, primR, grad, gLp, gLo, grad, gRp, gRo, (R)r,
                               phi, n3, (R)0.0, Fw, Fl, Us, OmL);
  } else {
    solve_riemann<Phys, R, NQ>(P, S.planets, primL, primR, gLo, gLp, grad, gRo, gRp, grad, (R)r,
                               phi, n3, (R)0.0, Fw, Fl, Us, OmL);
  }
  if constexpr (kMix<R>) {   // back to the lab frame (fixed face: F = Fw)
    R Omr2 = OmL * r * r;
    if (Phys::MHD) Fw[TAU] += OmL * Fw[LLL] + (R).5 * OmL * Omr2 * Fw[DDD];
    Fw[LLL] += Omr2 * Fw[DDD];
  }
  R* out = S.fflux[d];
  const int NF = S.nf[d];
  R dAdt;
  if constexpr (kMix<R>) dAdt = S.fdA[d][f] * ((R)fac * dt_r<R>(S.scal));
  else dAdt = S.fdA[d][f] * (R)(fac * S.scal[SC_DT]);
#pragma unroll
  for (int q = 0; q < NQ; ++q) out[(size_t)q * NF + f] = Fw[q] * dAdt;
  if constexpr (!Phys::GR) if (S.ct) {
    R E1, B1, E2, B2;
    Phys::flux_to_E(Fl, Us, r, &E1, &B1, &E2, &B2, dim);
    S.fErz[d][f] = E1; S.fBrz[d][f] = B1; S.fEphi[d][f] = E2;
  }
}

template <typename Phys, typename R, int NQ>
DISCO_D void k_flux_trans_body(const DevParams& P, const DevState<R>& S, int dim, int jmin, int jcount, int kmin, double fac, int bx_, int by_) {
  const int d = dim - 1;
  int pj = jmin + (int)bx_ % jcount;
  int pk = kmin + (int)bx_ / jcount;
  int pair = dim == 1 ? pj + (P.Nr - 1) * pk : pj + P.Nr * pk;
  int base = S.face_off[d][pair], Nf = S.face_off[d][pair + 1] - base;
  int n = by_ * blockDim.x + threadIdx.x;
  if (n >= Nf) return;
  int f = base + n;
  const int N = S.N;
  const int cL = S.fL[d][f], cR = S.fR[d][f];
  const R* gradD = dim == 1 ? S.gradr : S.gradz;
  flux_trans_face<Phys, R, NQ>(P, S, dim, pair, pj, pk, f, cL, cR, fac, [&](int s, int q, R* p, R* gp, R* gd) {
    const int c = s ? cR : cL;
    *p = S.prim[q * N + c];
    *gp = S.gradp[q * N + c];
    *gd = gradD[q * N + c];
  });
}

template <typename Phys, typename R, int NQ>
__global__ void __launch_bounds__(256, kMix<R> ? 4 : 1) k_flux_trans(DevParams P, DevState<R> S, int dim, int jmin, int jcount, int kmin, double fac) {
  k_flux_trans_body<Phys, R, NQ>(P, S, dim, jmin, jcount, kmin, fac, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- conserved update + sources + move + cons2prim -----------------------------
// adjust_RK_cons (misc.c:226), flux scatter (riemann.c:314-317) as a gather in
// the reference's order, add_source (misc.c:550), move_cells/clean_pi/calc_dp
// (misc.c:266, :8, :281), calc_prim (misc.c:300).
// Variants kept out of the common instantiation, which runs at the mixed
// path's 64-register cap with every component's loads in flight: CD with
// cooling / damping, MID for a middle substep (RK3's second), whose store of
// the running increment would otherwise sit in the component loop.
template <typename Phys, typename R, int NQ, bool CD, bool MID>
DISCO_D void k_update_body(const DevParams& P, const DevState<R>& S, double RK, double fac, int first, int do_c2p, int bx_, int by_) {
  constexpr bool mid = MID;
  int c = bx_ * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  const double Pmax = P.phi_max;
  double dt = fac * S.scal[SC_DT];
  bool real = is_real(P, j, k);

  double piph = S.piph[c], dphi = S.dphi[c];
  constexpr bool MIX = kMix<R>;
  // move_cells + clean_pi + calc_dp (first substep only): new positions
  double piph_new = piph, dphi_new = dphi;
  if (first) {
    int cm = off + (i == 0 ? Np - 1 : i - 1);
    double pn = piph + S.wiph[c] * dt;
    double pm = S.piph[cm] + S.wiph[cm] * dt;
    if constexpr (MIX) {   // the same wraps with integer compares
      pn = clean_pi_bits(pn, Pmax);
      pm = clean_pi_bits(pm, Pmax);
      dphi_new = get_dp_bits(pn, pm, Pmax);
    } else {
      while (pn > Pmax) pn -= Pmax;
      while (pn < 0.0) pn += Pmax;
      while (pm > Pmax) pm -= Pmax;
      while (pm < 0.0) pm += Pmax;
      dphi_new = get_dp(pn, pm, Pmax);
    }
    piph_new = pn;
  }
  if (real) {
    double U[NQ];
    // adjust_RK_cons: before the flux terms on the FP64 path (they are added
    // to U in order); after the R sums on the mixed path (shorter live range)
    auto load_rk = [&]() {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        double u = S.cons[q * N + c];
        if (first) {
          S.RKcons[q * N + c] = u;
        } else {
          u = (1. - RK) * u + RK * S.RKcons[q * N + c];
        }
        U[q] = u;
      }
    };
    if constexpr (!MIX) load_rk();
    else (void)load_rk;
    // Mixed path: fluxes and sources are summed in R (FP32) into dU, and dU
    // is added once to the FP64 conserved state.  The FP64 path adds every
    // term to U directly, in the reference's order.
    R dU[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) dU[q] = 0;
    auto add = [&](int q, R v) { if (MIX) dU[q] += v; else U[q] += (double)v; };
    // phi faces: cell i receives +F_{i-1} then -F_i (for i = 0: -F_0, +F_{Np-1})
    int cm = off + (i == 0 ? Np - 1 : i - 1);
    if (i == 0) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) { add(q, -S.fphi[q * N + c]); add(q, S.fphi[q * N + cm]); }
    } else {
#pragma unroll
      for (int q = 0; q < NQ; ++q) { add(q, S.fphi[q * N + cm]); add(q, -S.fphi[q * N + c]); }
    }
    // r then z faces: lower pair (cell is R: +=) then upper pair (cell is L: -=)
#pragma unroll
    for (int dim = 1; dim <= 2; ++dim) {
      if (dim == 1 && P.Nr <= 1) continue;
      if (dim == 2 && P.Nz <= 1) continue;
      const int d = dim - 1;
      const R* Fb = S.fflux[d];
      const int NF = S.nf[d];
      int pb = pair_below(P, dim, j, k);
      int pa = pair_above(P, dim, j, k);
      if (pb >= 0) {
        int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
        for_run(S.run_dn_s[d][c], S.run_dn_e[d][c], base, Nf, [&](int f) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) add(q, Fb[(size_t)q * NF + f]);
        });
      }
      if (pa >= 0) {
        int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
        for_run(S.run_up_s[d][c], S.run_up_e[d][c], base, Nf, [&](int f) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) add(q, -Fb[(size_t)q * NF + f]);
        });
      }
    }
    // sources (misc.c:569-590) at the pre-move geometry
    R pr[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * N + c];
    double xp[3] = {rj[j], piph, zk[k]};
    double xm[3] = {rj[j - 1], piph - dphi, zk[k - 1]};
    double dVdt = 0, dVc = 0;
    if constexpr (MIX) {   // sources summed in R into dU with the flux terms
      pr[UPP] += S.ring_Om_r[jk];   // lab omega for the source terms
      R dph = S.dphi_r[c];
      R dVdt_r = S.ring_vol_r[jk] * dph * (to_r<R>(fac) * dt_r<R>(S.scal));
      R rc = S.ring_rc_r[jk];
      Phys::template source<R>(P, pr, dU, dVdt_r, S.ring_r1_r[jk], S.ring_r23_r[jk], rc, dph);
      if (P.Npl) {
        R phc = to_r<R>(piph) - (R).5 * dph;
        for (int p = 0; p < P.Npl; ++p)
          if (S.planets[p].M != 0.0)
            planet_src<R, R>(P, S.planets[p], pr, dU, phc, S.ring_zc_r[jk], dVdt_r, rc, dph);
      }
      // adjust_RK_cons on the mixed path.  The first substep adds its
      // increment d1 (summed in R; plus the FP64 viscous / rotating-frame
      // sources, below) to cons and keeps d1 in R; the second substep's
      // RK RKcons + (1 - RK) cons is then cons - RK d1 (to FP64 rounding:
      // nothing else writes the cons of a real cell between the two updates,
      // except the B components of a CT run, which are rebuilt from the face
      // fluxes after every update and never read from here).  So
      // U = cons + (dU - RK d1): one FP64 add per component, and the RK
      // copy of the state is R instead of FP64.
      // A middle substep (RK3's second) keeps the increment since the step
      // start current for the last one: d_k = d_(k-1) + (U_k - U_(k-1)).
      const R rk = to_r<R>(RK);
      const bool whole = P.include_viscosity || P.rot_flag || CD;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        double u = S.cons[q * N + c];
        R d = dU[q];
        if (first) {
          S.RKdU[q * N + c] = d;
        } else {
          const R dold = S.RKdU[q * N + c];
          d = fma(-rk, dold, d);
          if constexpr (MID) {
            if (!whole) S.RKdU[q * N + c] = dold + d;
          }
        }
        U[q] = u + from_r<R>(d);
      }
      if (P.include_viscosity || P.rot_flag || CD) {
        double dV = (.5 * (xp[0] + xm[0])) * (xp[0] - xm[0]) * get_dp(xp[1], xm[1], Pmax) * (xp[2] - xm[2]);
        dVdt = dV * dt;
        dVc = dV;
        if constexpr (!Phys::GR)
          if constexpr (CD) cool_damp_src<Phys, R, NQ>(P, S.planets, pr, U, xp, xm, dV, dt);
      }
    } else {
      double dV = (.5 * (xp[0] + xm[0])) * (xp[0] - xm[0]) * get_dp(xp[1], xm[1], Pmax) * (xp[2] - xm[2]);
      dVdt = dV * dt;
      dVc = dV;
      if constexpr (Phys::GR) {   // grmhd.c:339 (metric and frame sources; no planets)
        Phys::source_x(P, pr, U, xp, xm, dVdt);
      } else {
        if constexpr (CD) cool_damp_src<Phys, R, NQ>(P, S.planets, pr, U, xp, xm, dV, dt);
        double dph = get_dp(xp[1], xm[1], Pmax);
        double rc = S.ring_rc[jk];
        Phys::template source<double>(P, pr, U, dVdt, (R)(.5 * (xp[0] + xm[0])), (R)S.ring_r23[jk], (R)rc,
                                      (R)dph);
        for (int p = 0; p < P.Npl; ++p)
          if (S.planets[p].M != 0.0)
            planet_src<R, double>(P, S.planets[p], pr, U, (R)(xm[1] + 0.5 * dph),
                                  (R)centroid_z(xp[2], xm[2]), dVdt, (R)rc, (R)dph);
      }
    }
    if constexpr (!Phys::GR) if (P.include_viscosity) {
      R gr[NQ], gp[NQ], gz[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        gr[q] = S.gradr[q * N + c]; gp[q] = S.gradp[q * N + c]; gz[q] = S.gradz[q * N + c];
      }
      Phys::visc_source(P, S.planets, pr, gr, gp, gz, U, xp, xm, dVdt);
    }
    if constexpr (!Phys::GR) if (P.rot_flag) {  // omega_src, rotframe.c:32-80
      double r = S.ring_rc[jk];
      double ph = .5 * (xp[1] + xm[1]);
      double rho = pr[RHO];
      double v0 = pr[URR], v1 = (double)pr[UPP] * r, v2 = pr[UZZ];
      double vr = v0, vom = v1 / r;
      double Rr = r - P.rot_d * cos(ph), Rp = P.rot_d * sin(ph);
      double f0 = P.rot_omega * P.rot_omega * Rr + 2. * P.rot_omega * r * vom;
      double f1 = P.rot_omega * P.rot_omega * Rp - 2. * P.rot_omega * vr;
      double f2 = 0.0;
      v1 -= r * (double)get_om<double>(P, r);
      double vf = v0 * f0 + v1 * f1 + v2 * f2;
      f1 *= r;
      U[SRR] += rho * f0 * dVdt;
      U[LLL] += rho * f1 * dVdt;
      U[SZZ] += rho * f2 * dVdt;
      U[TAU] += rho * vf * dVdt;
    }
    if constexpr (CD && !Phys::GR)   // sink_src, the last source (misc.c:587)
      if (P.sink_type || P.nozzle_type) sink_src<R>(P, S.planets, pr, U, xp, xm, dVc, dt, nullptr);
    if constexpr (MIX) {
      // the viscous and rotating-frame sources go to U in FP64 after the R
      // sum: the increment kept for the second substep is then the whole
      // change of this substep
      if ((first || mid) && (P.include_viscosity || P.rot_flag || CD)) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const R dold = first ? (R)0 : S.RKdU[q * N + c];
          S.RKdU[q * N + c] = dold + to_r<R>(U[q] - S.cons[q * N + c]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.cons[q * N + c] = U[q];
    if constexpr (MIX) {
      if (do_c2p) {   // calc_prim at the post-move geometry, from U in registers
        R pr2[NQ];
        R dph = first ? to_r<R>(dphi_new) : S.dphi_r[c];
        int hits = Phys::cons2prim(P, S.planets, U, pr2, S.ring_rc_r[jk],
                                   to_r<R>(piph_new) - (R).5 * dph, S.ring_vol_r[jk] * dph,
                                   S.ring_Lsh[jk], S.ring_Om_r[jk]);
        bool bad = false;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          S.prim[q * N + c] = pr2[q];
          if (!isfinite(pr2[q])) bad = true;
        }
        if (bad) atomicAdd(&S.errs->nan_cells, 1ull);
        if (hits & 1) atomicAdd(&S.errs->rho_floor_hits, 1ull);
        if (hits & 2) atomicAdd(&S.errs->p_floor_hits, 1ull);
      }
    }
  }

  if (first) {
    piph = piph_new;
    dphi = dphi_new;
    S.piph_out[c] = piph;
    S.dphi[c] = dphi;
    if constexpr (MIX) S.dphi_r[c] = to_r<R>(dphi);
  }

  if (!MIX && real && do_c2p) {  // calc_prim at the post-move geometry
    R pr[NQ];
    int hits;
    {
      double rp = rj[j], rm = rj[j - 1], zp = zk[k], zm = zk[k - 1];
      double phim = piph - dphi;
      double xp1 = piph;
      double dV = (.5 * (rp + rm)) * (rp - rm) * get_dp(xp1, phim, Pmax) * (zp - zm);
      double r = S.ring_rc[jk];
      double U[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) U[q] = S.cons[q * N + c];
      if constexpr (Phys::GR) {   // Newton iteration seeded with the previous primitives
#pragma unroll
        for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * N + c];
        const double xg[3] = {r, .5 * (phim + piph), .5 * (zp + zm)};
        typename Phys::C2PRec rec;
        hits = Phys::cons2prim_x(P, U, pr, xg, dV, nullptr, &rec);
        c2p_count(S.errs, rec.kconv, rec.iters, rec.guessed);
      } else {
        hits = Phys::cons2prim(P, S.planets, U, pr, r, .5 * (phim + piph), dV);
      }
    }
    bool bad = false;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      S.prim[q * N + c] = pr[q];
      if (!isfinite(pr[q])) bad = true;
    }
    if (bad) atomicAdd(&S.errs->nan_cells, 1ull);
    if (hits & 1) atomicAdd(&S.errs->rho_floor_hits, 1ull);
    if (hits & 2) atomicAdd(&S.errs->p_floor_hits, 1ull);
    if (hits & 4) atomicAdd(&S.errs->c2p_no_converge, 1ull);
  }
}
template <typename Phys, typename R, int NQ, bool CD = false, bool MID = false>
__global__ void __launch_bounds__(256, kMix<R> ? 4 : 1) k_update(DevParams P, DevState<R> S, double RK, double fac, int first, int do_c2p) {
  k_update_body<Phys, R, NQ, CD, MID>(P, S, RK, fac, first, do_c2p, (int)blockIdx.x, (int)blockIdx.y);
}

// ---- FP64 primitives in and out of the device layout --------------------------
// The C ABI's views hold FP64 primitives with prim[UPP] the lab omega; the
// device holds R, relative to the ring frame on the mixed path.  The same
// arithmetic the host would do (FP64 difference, then one rounding to R; the
// widening and FP64 sum back), over all NQ * N values in a grid-stride loop.
template <typename R, int NQ>
__global__ void k_prim_in(DevState<R> S, const double* src) {
  const size_t n = (size_t)NQ * S.N;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = src[i];
    if constexpr (kMix<R>) {
      if (i / (size_t)S.N == (size_t)UPP) v -= S.ring_Om[S.cell_ring[i - (size_t)UPP * S.N]];
    }
    S.prim[i] = (R)v;
  }
}
template <typename R, int NQ>
__global__ void k_prim_out(DevState<R> S, double* dst) {
  const size_t n = (size_t)NQ * S.N;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = (double)S.prim[i];
    if constexpr (kMix<R>) {
      if (i / (size_t)S.N == (size_t)UPP) v += S.ring_Om[S.cell_ring[i - (size_t)UPP * S.N]];
    }
    dst[i] = v;
  }
}

// ---- ghost rings: boundary_trans of Boundary/fixed.c and Boundary/fixed3d.c ----
// fixed.c:11-46 evaluates initial() at the arithmetic-mean radius on r ghosts
// only; fixed3d.c uses set_cell_init (boundary_functions.c:21) on r and z
// ghosts.  The state after the prim update is position-dependent only.
template <typename R, int NQ>
DISCO_D void k_boundary_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  // one block per chunk of ghost cells (the list holds the rings the plugin
  // fills: fixed.c r ghosts, fixed3d.c r and z ghosts)
  const int jk = S.ghost_ring[bx_], i0 = S.ghost_i0[bx_];
  const int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const int i = i0 + threadIdx.x;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  // r and z of the evaluation point are those of the ring in both plugins
  const double xr = P.boundary_id == 0 ? .5 * (rj[j] + rj[j - 1]) : centroid_r(rj[j], rj[j - 1]);
  const double xz = P.boundary_id == 0 ? .5 * (zk[k] + zk[k - 1]) : centroid_z(zk[k], zk[k - 1]);
  // the disk initial conditions do not depend on phi (or time): their ghost
  // values come from the per-ring table made at set-up (k_ghost_tab)
  if (i >= Np || i >= i0 + kTileCells) return;
  const int c = off + i;
  double prim[MAX_Q];
  if (S.ghost_tab) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) prim[q] = S.ghost_tab[(size_t)jk * NQ + q];
  } else {
    double x[3];
    x[0] = xr;
    x[1] = P.boundary_id == 0 ? S.piph[c] - .5 * S.dphi[c] : .5 * (S.piph[c] + (S.piph[c] - S.dphi[c]));
    x[2] = xz;
    initial_eval(P, prim, x);
  }
  if constexpr (kMix<R>) prim[UPP] -= S.ring_Om[jk];   // ring frame
#pragma unroll
  for (int q = 0; q < NQ; ++q) S.prim[q * S.N + c] = (R)prim[q];
}
// exchangeData with one rank and a periodic dimension (exchange.c:173-279:
// the cartesian communicator wraps around, so the rank is its own left and
// right neighbour): every cell of ghost ring dst[b] takes the state of the
// same cell of ring src[b] -- primitives, conserved state and its RK copy,
// position, width and mesh speed, and with CT the face fluxes and their RK
// copy (struct cell_lite, exchange.c:6-15).  The two rings have the same Np
// (set at set-up, as the exchange's Np message does), and on the mixed path
// the same ring frame, so the frame-relative omega copies as it is.
template <typename R, int NQ>
__global__ void __launch_bounds__(kTileCells) k_periodic_copy(DevParams P, DevState<R> S, double* Phi,
                                                              double* RKPhi, const int* dst, const int* src) {
  (void)P;
  const int jd = dst[blockIdx.x], js = src[blockIdx.x];
  const int od = S.ring_off[jd], os = S.ring_off[js];
  const int np = S.ring_off[js + 1] - os;
  const int N = S.N;
  double* piph = const_cast<double*>(S.piph);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int cd = od + i, cs = os + i;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      S.prim[q * N + cd] = S.prim[q * N + cs];
      S.cons[q * N + cd] = S.cons[q * N + cs];
      if constexpr (kMix<R>) S.RKdU[q * N + cd] = S.RKdU[q * N + cs];
      else S.RKcons[q * N + cd] = S.RKcons[q * N + cs];
    }
    piph[cd] = piph[cs];
    S.dphi[cd] = S.dphi[cs];
    S.wiph[cd] = S.wiph[cs];
    if constexpr (kMix<R>) S.dphi_r[cd] = S.dphi_r[cs];
    if (Phi) {
#pragma unroll
      for (int f = 0; f < 5; ++f) {
        Phi[f * N + cd] = Phi[f * N + cs];
        RKPhi[f * N + cd] = RKPhi[f * N + cs];
      }
    }
  }
}

template <typename R, int NQ>
__global__ void __launch_bounds__(kTileCells) k_boundary(DevParams P, DevState<R> S) {
  k_boundary_body<R, NQ>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// Per-ring ghost values of fixed.c / fixed3d.c for the axisymmetric disk
// initial conditions (ids 1, 2), evaluated once at set-up at the points
// k_boundary uses (phi plays no part): one thread per ring.
template <typename R, int NQ>
__global__ void k_ghost_tab(DevParams P, int nring, double* tab, const double* r_jph, const double* z_kph) {
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= nring) return;
  const int k = jk / P.Nr, j = jk - k * P.Nr;
  const double* rj = r_jph + 1;
  const double* zk = z_kph + 1;
  double x[3];
  x[0] = P.boundary_id == 0 ? .5 * (rj[j] + rj[j - 1]) : centroid_r(rj[j], rj[j - 1]);
  x[1] = 0.0;
  x[2] = P.boundary_id == 0 ? .5 * (zk[k] + zk[k - 1]) : centroid_z(zk[k], zk[k - 1]);
  double prim[MAX_Q];
  initial_eval(P, prim, x);
  for (int q = 0; q < NQ; ++q) tab[(size_t)jk * NQ + q] = prim[q];
}

// ---- ghost rings copied from other rings: boundary_functions.c:90-158 ----
// boundary_zerograd_* (:269-441) copy the next ring inward onto each ghost
// ring, layer by layer from the real domain outward (with an optional
// diode on the normal velocity, as outflow3d.c asks); boundary_reflect_*
// (:442-621) and boundary_noslip_* (:914-1101) copy the mirror ring and
// negate the normal velocity (reflect) or every velocity (noslip,
// reflect_prims in all three directions).  The copy is the phi-overlap
// average of set_cells_copy_distant.  One thread per ghost ring of a layer
// walks both rings in the reference's order (the same overlaps summed in
// the same order); the layers are separate launches.  On the mixed path
// the copy is made in the frame of the reference's primitives (ring
// frames added and removed in FP64).
// dim 1: rings (layer, k) for all k; dim 2: rings (j, layer) for all j.
// mode 0 zerograd (source layer +- 1), 1 reflect, 2 noslip (mirror source).
template <typename R, int NQ>
__global__ void k_bc_copy(DevParams P, DevState<R> S, int dim, int side, int layer, int mode, int diode) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int j, k, j1, k1;
  if (dim == 1) {
    if (t >= P.Nz) return;
    k = k1 = t;
    j = layer;
    if (mode == 0) j1 = side == 0 ? j + 1 : j - 1;
    else j1 = side == 0 ? 2 * P.NgRa - j - 1 : 2 * (P.Nr - P.NgRb) - j - 1;
  } else {
    if (t >= P.Nr) return;
    j = j1 = t;
    k = layer;
    if (mode == 0) k1 = side == 0 ? k + 1 : k - 1;
    else k1 = side == 0 ? 2 * P.NgZa - k - 1 : 2 * (P.Nz - P.NgZb) - k - 1;
  }
  const int jk = j + P.Nr * k, jk1 = j1 + P.Nr * k1;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const int off1 = S.ring_off[jk1], Np1 = S.ring_off[jk1 + 1] - off1;
  const double Pmax = P.phi_max;
  const int N = S.N;
  const double Om = kMix<R> ? S.ring_Om[jk] : 0.0, Om1 = kMix<R> ? S.ring_Om[jk1] : 0.0;
  // the first source cell that holds the lower edge of cell 0
  int i1 = 0;
  {
    const double phi0 = S.piph[off] - S.dphi[off];
    for (i1 = 0; i1 < Np1; ++i1) {
      const double dphip = get_signed_dp(S.piph[off1 + i1], phi0, Pmax);
      const double dphim = dphip - S.dphi[off1 + i1];
      if (dphip > 0 && dphim <= 0.0) break;
    }
    if (i1 >= Np1) i1 = 0;
  }
  const int qn = dim == 1 ? URR : UZZ;
  for (int i = 0; i < Np; ++i) {
    const int c = off + i;
    const double phip = S.piph[c], phim = S.piph[c] - S.dphi[c];
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
    double phip1, phim1;
    int walk = 0;   // at most one turn of the source ring (guards a non-finite phi)
    do {
      const int c1 = off1 + i1;
      phip1 = S.piph[c1];
      phim1 = S.piph[c1] - S.dphi[c1];
      for (int w = 0; w < 4 && phip1 < phim; ++w) { phip1 += Pmax; phim1 += Pmax; }
      for (int w = 0; w < 4 && phim1 > phip; ++w) { phip1 -= Pmax; phim1 -= Pmax; }
      const double p1 = phip < phip1 ? phip : phip1;
      const double p2 = phim > phim1 ? phim : phim1;
      const double dphi = p1 - p2;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        double v = (double)S.prim[q * N + c1];
        if (kMix<R> && q == UPP) v += Om1;
        acc[q] += v * dphi;
      }
      i1 = i1 < Np1 - 1 ? i1 + 1 : 0;
    } while (phip1 < phip && ++walk <= Np1);
    i1 = i1 > 0 ? i1 - 1 : Np1 - 1;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double v = acc[q] / S.dphi[c];
      if (mode == 0 && diode && q == qn && (side == 0 ? v > 0 : v < 0)) v = 0.0;
      if ((mode == 1 && q == qn) || (mode == 2 && (q == URR || q == UPP || q == UZZ))) v = -v;
      if (kMix<R> && q == UPP) v -= Om;
      S.prim[q * N + c] = (R)v;
    }
  }
}

// ---- ghost rings from the initial condition, one side at a time ----------
// boundary_fixed_* (boundary_functions.c:161-268: set_cell_init at the
// cell centroid), boundary_fixed_q_* (:662-773: set_cell_init_q, at
// phi = piph - dphi/2, only the primitives in qmask) and
// boundary_fixed_phi_* (:774-913: set_cell_init where the cell's phi,
// raised past pa by whole turns, is below pb).  One block per ghost ring:
// dim 1 rings (j, k) of the side's ng layers for all k, dim 2 (j, k) for
// all j.  mode 0 fixed, 1 fixed_q, 2 fixed_phi.
template <typename R, int NQ>
DISCO_D void bc_init_ring(const DevParams& P, const DevState<R>& S, int j, int k, int mode, int qmask,
                          double pa, double pb) {
  const int jk = j + P.Nr * k;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  // mode 3 (Boundary/horizon.c): arithmetic-mean r and z
  const double xr = mode == 3 ? .5 * (rj[j] + rj[j - 1]) : centroid_r(rj[j], rj[j - 1]);
  const double xz = mode == 3 ? .5 * (zk[k] + zk[k - 1]) : centroid_z(zk[k], zk[k - 1]);
  const int N = S.N;
  for (int i = threadIdx.x; i < Np; i += blockDim.x) {
    const int c = off + i;
    const double phip = S.piph[c], dph = S.dphi[c];
    double x[3] = {xr, 0.0, xz};
    if (mode == 1 || mode == 3) {
      x[1] = phip - .5 * dph;
    } else {
      if (mode == 2) {
        double phi = phip - .5 * dph;
        for (int w = 0; w < 4 && phi < pa; ++w) phi += P.phi_max;
        if (!(phi < pb)) continue;
      }
      x[1] = .5 * (phip + (phip - dph));   // get_centroid(dim 0)
    }
    double prim[MAX_Q];
    initial_eval(P, prim, x);
    if constexpr (kMix<R>) prim[UPP] -= S.ring_Om[jk];   // ring frame
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (mode != 1 || ((qmask >> q) & 1)) S.prim[q * N + c] = (R)prim[q];
  }
}
template <typename R, int NQ>
__global__ void __launch_bounds__(128) k_bc_init(DevParams P, DevState<R> S, int dim, int side, int mode,
                                                 int qmask, double pa, double pb) {
  int j, k;
  if (dim == 1) {
    const int ng = side ? P.NgRb : P.NgRa;
    const int l = blockIdx.x % ng;
    k = blockIdx.x / ng;
    j = side ? P.Nr - P.NgRb + l : l;
  } else {
    const int ng = side ? P.NgZb : P.NgZa;
    const int l = blockIdx.x % ng;
    j = blockIdx.x / ng;
    k = side ? P.Nz - P.NgZb + l : l;
  }
  bc_init_ring<R, NQ>(P, S, j, k, mode, qmask, pa, pb);
}
// Boundary/horizon_bin.c's cut-outs (:79-179): on a candidate ring of hole
// h, every cell whose point (rc, mid phi, zc) lies within the hole goes back
// to initial() at the arithmetic-mean r, z and its mid phi, and leaves the
// CFL minimum for good (one block a candidate entry)
template <typename R, int NQ>
__global__ void __launch_bounds__(128) k_bc_holes(DevParams P, DevState<R> S) {
  const int e = S.hole_list[blockIdx.x], jk = e >> 1, h = e & 1;
  const int k = jk / P.Nr, j = jk - k * P.Nr;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double rc, zc;
  if (!disco_bc_hole_ring(rj, zk, P.Nr, P.Nz, j, k, h, &rc, &zc)) return;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off, N = S.N;
  for (int i = threadIdx.x; i < Np; i += blockDim.x) {
    const int c = off + i;
    const double phi = S.piph[c] - .5 * S.dphi[c];
    if (!disco_bc_hole_cell(rc, zc, P.Nz, phi, h)) continue;
    double x[3] = {.5 * (rj[j - 1] + rj[j]), phi, .5 * (zk[k - 1] + zk[k])};
    double prim[MAX_Q];
    initial_eval(P, prim, x);
    if constexpr (kMix<R>) prim[UPP] -= S.ring_Om[jk];   // ring frame
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.prim[q * N + c] = (R)prim[q];
    S.cell_excised[c] = 1;
  }
}

// boundary_fixed_horizon (boundary_functions.c:622-660): set_cell_init on
// every cell of the excised rings, real and ghost alike (one block a ring);
// mode 3 for Boundary/horizon.c's cut-out (arithmetic-mean positions)
template <typename R, int NQ>
__global__ void __launch_bounds__(128) k_bc_horizon(DevParams P, DevState<R> S, int mode) {
  const int jk = S.hor_rings[blockIdx.x];
  const int k = jk / P.Nr, j = jk - k * P.Nr;
  bc_init_ring<R, NQ>(P, S, j, k, mode, 0, 0.0, 0.0);
}

// ---- getmindt, misc.c:39-84 -------------------------------------------------
// The CFL bound of cell c, +1e300 for ghost cells: the module's mindt hook
// on the FP64 path, 1 / cell_rate on the mixed path (FP64 extents and dt).
template <typename Phys, typename R, int NQ>
DISCO_D double cell_rate(const DevParams& P, const DevState<R>& S, int c);

template <typename Phys, typename R, int NQ>
DISCO_D double cell_mindt(const DevParams& P, const DevState<R>& S, int c) {
  if constexpr (kMix<R>) {
    const double rate = cell_rate<Phys, R, NQ>(P, S, c);
    return rate > 0.0 ? 1.0 / rate : 1.0e300;
  } else {
    int jk = S.cell_ring[c];
    int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
    if (!is_real(P, j, k) || (S.ring_excised && S.ring_excised[jk]) || (S.cell_excised && S.cell_excised[c]))
      return 1.0e300;
    int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
    int i = c - off;
    int im = off + (i == 0 ? Np - 1 : i - 1);
    const double* rj = S.r_jph + 1;
    const double* zk = S.z_kph + 1;
    double phip = S.piph[c], phim = phip - S.dphi[c];
    double xp[3] = {rj[j], phip, zk[k]};
    double xm[3] = {rj[j - 1], phim, zk[k - 1]};
    double w = .5 * (S.wiph[im] + S.wiph[c]);
    R pr[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * S.N + c];
    if constexpr (Phys::GR) return Phys::mindt_x(P, pr, w, xp, xm);
    else return Phys::mindt(P, S.planets, pr, w, xp, xm, S.ring_rc[jk]);
  }
}

// Mixed path: the cell's inverse time step.  The signal speeds are physics
// and FP32, as in the Riemann solvers; the cell extents, the rates, their
// maximum and dt are FP64: dt = 1 / max(s_r / dr, s_phi / (r dphi),
// s_z / dz [, 2 nu / dx^2]).  0 for a ghost cell, and for a rate that is
// not a number (such a cell drops out of the minimum, as in getmindt).
template <typename Phys, typename R, int NQ>
DISCO_D double cell_rate(const DevParams& P, const DevState<R>& S, int c) {
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!is_real(P, j, k) || (S.ring_excised && S.ring_excised[jk]) || (S.cell_excised && S.cell_excised[c]))
    return 0.0;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  int im = off + (i == 0 ? Np - 1 : i - 1);
  const double phip = S.piph[c];
  const double w = .5 * (S.wiph[im] + S.wiph[c]);
  R pr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * S.N + c];
  R sp[4];
  const R wr = (R)(w - S.ring_Om[jk]);   // relative to the ring frame, as prim[UPP]
  const double dph = S.dphi[c];
  Phys::cfl_speeds_r(P, S.planets, pr, wr, S.ring_rc_r[jk], (R)(phip - .5 * dph), sp);
  const double* g = S.ring_cfl + 3 * jk;
  const double iphi = 1.0 / (g[0] * dph);
  double rate = fmax(f2d_int(sp[0]) * g[1], fmax(f2d_int(sp[1]) * iphi, f2d_int(sp[2]) * g[2]));
  if (sp[3] > (R)0) {   // explicit viscosity: dt_visc = dx^2 / (2 nu), dx the smallest extent
    const double ix = fmax(iphi, fmax(g[1], g[2]));
    rate = fmax(rate, 2.0 * f2d_int(sp[3]) * ix * ix);
  }
  return rate >= 0.0 ? rate : 0.0;
}

template <typename Phys, typename R, int NQ>
DISCO_D void k_mindt_body(const DevParams& P, const DevState<R>& S, int bx_, int by_) {
  int c = bx_ * blockDim.x + threadIdx.x;
  // dt > 0: its IEEE bits order like unsigned integers; NaN sorts above.
  // The mixed path reduces the largest rate instead and divides once per
  // block: 1 / x rounds monotonically, so 1 / max(rate) is the smallest
  // 1 / rate bit for bit.
  __shared__ unsigned long long red[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long b;
  if constexpr (kMix<R>) {
    b = __double_as_longlong(c < S.N ? cell_rate<Phys, R, NQ>(P, S, c) : 0.0);
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  } else {
    b = __double_as_longlong(c < S.N ? cell_mindt<Phys, R, NQ>(P, S, c) : 1.0e300);
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (lane == 0) red[wid] = b;
  __syncthreads();
  if (wid == 0) {
    if constexpr (kMix<R>) {
      b = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
      for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
      const double rmax = __longlong_as_double(b);
      b = __double_as_longlong(rmax > 0.0 ? 1.0 / rmax : 1.0e300);
    } else {
      b = lane < (int)(blockDim.x >> 5) ? red[lane] : ~0ull;
      for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if (lane == 0) atomicMin((unsigned long long*)&S.scal[SC_MIN], b);
  }
}
template <typename Phys, typename R, int NQ>
__global__ void k_mindt(DevParams P, DevState<R> S) {
  k_mindt_body<Phys, R, NQ>(P, S, (int)blockIdx.x, (int)blockIdx.y);
}

// dt = CFL * min (misc.c:52-78); clamp to T_End (check_dt, domain.c:433).
DISCO_D void dt_finalize_one(const DevParams& P, double* scal) {
  double m = __longlong_as_double(*(long long*)&scal[SC_MIN]);
  double dt0 = P.maxDT / P.CFL;
  if (dt0 <= 0.0) dt0 = 1.0e100;
  double dt = dt0 < m ? dt0 : m;
  dt *= P.CFL;
  if (P.t_end > 0.0 && scal[SC_T] + dt > P.t_end) dt = P.t_end - scal[SC_T];
  scal[SC_DT] = dt;
  *(float*)&scal[SC_DTF] = (float)dt;
  *(unsigned long long*)&scal[SC_MIN] = 0x7ff0000000000000ull;   // +inf
}
static __global__ void k_dt_finalize(DevParams P, double* scal) { dt_finalize_one(P, scal); }

// After the first substep: t += dt (timestep.c:136), analytic planet motion
// (Planets/circular.c:44-46), clean_pi on planets (misc.c:27-34).
DISCO_D void after_first_one(const DevParams& P, double* scal, DevPlanet* pl, int planets_id,
                              DevErrs* errs) {
  double dt = scal[SC_DT];
  double t = scal[SC_T];   // movePlanets sees the time before the step's update
  scal[SC_T] += dt;
  if (planets_id == 2 && P.Npl > 1) pl[1].phi += pl[1].omega * dt;
  if (planets_id == 3 && P.Npl > 1) {   // Planets/cm.c:53-59
    pl[0].phi += pl[0].omega * dt;
    pl[1].phi += pl[1].omega * dt;
    double eps = 0.5 / P.mach + exp(-t / 30.);
    pl[0].eps = eps;
    pl[1].eps = eps;
  }
  for (int p = 0; p < P.Npl; ++p) {
    double phi = pl[p].phi;
    while (phi > P.phi_max) phi -= P.phi_max;
    while (phi < 0.0) phi += P.phi_max;
    pl[p].phi = phi;
  }
  errs->steps += 1;
}
static __global__ void k_after_first(DevParams P, double* scal, DevPlanet* pl, int planets_id,
                              DevErrs* errs) { after_first_one(P, scal, pl, planets_id, errs); }

// ---- calc_prim (misc.c:300-335) as its own pass (after B_faces_to_cells) --------
template <typename Phys, typename R, int NQ>
DISCO_D void c2p_cell(const DevParams& P, const DevState<R>& S, int c, int jk, int j, int k) {
  const int N = S.N;
  double U[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) U[q] = S.cons[q * N + c];
  R pr[NQ];
  int hits;
  if constexpr (kMix<R>) {
    R dph = S.dphi_r[c];
    hits = Phys::cons2prim(P, S.planets, U, pr, S.ring_rc_r[jk], to_r<R>(S.piph[c]) - (R).5 * dph,
                           S.ring_vol_r[jk] * dph, S.ring_Lsh[jk], S.ring_Om_r[jk]);
  } else {
    const double* rj = S.r_jph + 1;
    const double* zk = S.z_kph + 1;
    double piph = S.piph[c], dphi = S.dphi[c];
    double rp = rj[j], rm = rj[j - 1], zp = zk[k], zm = zk[k - 1];
    double phim = piph - dphi;
    double dV = (.5 * (rp + rm)) * (rp - rm) * get_dp(piph, phim, P.phi_max) * (zp - zm);
    double r = S.ring_rc[jk];
    if constexpr (Phys::GR) {   // Newton iteration seeded with the previous primitives
#pragma unroll
      for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * N + c];
      const double xg[3] = {r, .5 * (phim + piph), .5 * (zp + zm)};
      typename Phys::C2PRec rec;
      hits = Phys::cons2prim_x(P, U, pr, xg, dV, nullptr, &rec);
      c2p_count(S.errs, rec.kconv, rec.iters, rec.guessed);
    } else {
      hits = Phys::cons2prim(P, S.planets, U, pr, r, .5 * (phim + piph), dV);
    }
  }
  bool bad = false;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    S.prim[q * N + c] = pr[q];
    if (!isfinite(pr[q])) bad = true;
  }
  if (bad) atomicAdd(&S.errs->nan_cells, 1ull);
  if (hits & 1) atomicAdd(&S.errs->rho_floor_hits, 1ull);
  if (hits & 2) atomicAdd(&S.errs->p_floor_hits, 1ull);
  if (hits & 4) atomicAdd(&S.errs->c2p_no_converge, 1ull);
}

template <typename Phys, typename R, int NQ>
__global__ void k_c2p(DevParams P, DevState<R> S) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!is_real(P, j, k)) return;
  c2p_cell<Phys, R, NQ>(P, S, c, jk, j, k);
}

// ---- set-up: prim2cons + cons2prim for real cells (domain.c:349, :379) ---------
template <typename Phys, typename R, int NQ>
__global__ void k_init_cells(DevParams P, DevState<R> S, const double* prim0, int do_c2p) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!is_real(P, j, k)) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) { S.prim[q * N + c] = (R)0; S.cons[q * N + c] = 0; }
    return;
  }
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double piph = S.piph[c], dphi = S.dphi[c];
  double rp = rj[j], rm = rj[j - 1], zp = zk[k], zm = zk[k - 1];
  double dV = (.5 * (rp + rm)) * (rp - rm) * get_dp(piph, piph - dphi, P.phi_max) * (zp - zm);
  double r = centroid_r(rp, rm);
  double pr[NQ], U[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) pr[q] = prim0[q * N + c];
  R out[NQ];
  if constexpr (Phys::GR) {
    // setupCells (domain.c:176-238): prim2cons, then cons2prim seeded with
    // the initial primitives, both at x = (centroid r, phi, centroid z)
    const double xg[3] = {r, piph - .5 * dphi, .5 * (zp + zm)};
    Phys::prim2cons_x(P, pr, U, xg, dV);
#pragma unroll
    for (int q = 0; q < NQ; ++q) out[q] = pr[q];
    if (do_c2p) Phys::cons2prim_x(P, U, out, xg, dV);
  } else if (do_c2p) {
    using Phys64 = typename Phys::template Rebind<double>;
    Phys64::template prim2cons<double>(P, pr, U, r, dV);
    Phys::cons2prim(P, S.planets, U, out, r, piph - .5 * dphi, dV, S.ring_Lsh[jk], (R)S.ring_Om[jk]);
  } else {
    using Phys64 = typename Phys::template Rebind<double>;
    Phys64::template prim2cons<double>(P, pr, U, r, dV);
    for (int q = 0; q < NQ; ++q) out[q] = (R)pr[q];
    if constexpr (kMix<R>) out[UPP] = (R)(pr[UPP] - S.ring_Om[jk]);   // ring frame
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) { S.cons[q * N + c] = U[q]; S.prim[q * N + c] = out[q]; }
}

}  // namespace disco
