// Constrained transport (bfields.c) on the device.
//
// Per cell: Eraw/Braw[8] edge EMFs and fields (E[8], B[8] of struct cell),
// Ephi[4] azimuthal-edge EMFs (E_phi), Phi/RKPhi[5] face fluxes (FP64).
// Face flux ownership follows the reference exactly: the r face ending at
// cell L's upper phi edge (LRtype 0) stores its flux in L.Phi[2], the one
// ending at R's upper edge (LRtype 1) in R.Phi[1]; z faces use Phi[4]/[3].
// Every cell owns exactly one face on each side, the last face of its run
// in that pair (run_up_e / run_dn_e), so the reference's scatter updates
// become per-cell gathers.
#pragma once
#include "kernels.cuh"

namespace disco {

template <typename R>
struct CtStateT {
  double* Phi;      // [5*N] face fluxes: conserved, FP64 in both paths
  double* RKPhi;    // [5*N]
  R* Efin;          // [4*N]: E0, E1, E4, E5 after averaging and advective subtraction
  R* Ephi;          // [4*N]
  unsigned long long* errs;  // [0] edge-order mismatches
  int last_pair[2]; // index of the last pair of each dimension (skipped by update_B_fluxes)
  // edge-walk events of the last walk (make_edge_adjust): the four cells,
  // the branch bits and the edge length, replayed by the next step's first
  // substep, whose positions are the same (nullptr: no cache)
  int4* ev_cid;
  unsigned char* ev_flag;   // bit 0-1 w4, bit 2 LR_alt, bit 3 UD_alt, bit 7 valid
  R* ev_dl;
  const int* quad_ev_off;   // [quads + 1]: first event of each quad
  int* ev_ok;               // device flag: the cache matches the current positions
};

// ---- edge gathers (riemann.c:172-212) ------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256, kMix<R> ? 6 : 1) k_ct_gather(DevParams P, DevState<R> S, CtStateT<R> C) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!ring_in_phi_range(P, j, k)) return;
#pragma unroll
  for (int dim = 1; dim <= 2; ++dim) {
    if (dim == 1 && P.Nr <= 1) continue;
    if (dim == 2 && P.Nz <= 1) continue;
    const int d = dim - 1;
    const int a = 4 * d;
    int pb = pair_below(P, dim, j, k), pa = pair_above(P, dim, j, k);
    if (pb >= 0 && pair_in_flux_range(P, dim, pb)) {
      R e0 = S.Eraw[(a + 0) * N + c], e2 = S.Eraw[(a + 2) * N + c];
      R b0 = S.Braw[(a + 0) * N + c], b2 = S.Braw[(a + 2) * N + c];
      int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
      // mixed path: the face EMF was solved in the L ring's frame; this cell
      // (R) stores it relative to its own ring's frame
      R cX = kMix<R> ? S.pcX[d][pb] : (R)0;
      auto acc = [&](R fr, R ef, R bz) {
        if constexpr (kMix<R>) ef += cX * bz;
        e0 += (R).5 * ef * fr; e2 += (R).5 * ef * fr;
        b0 += (R).5 * bz * fr; b2 += (R).5 * bz * fr;
      };
      // two faces' loads in flight per iteration, accumulated in run order
      for_run2(S.run_dn_s[d][c], S.run_dn_e[d][c], base, Nf, [&](int f0, int f1, bool two) {
        R fr0 = S.ffrR[d][f0], ef0 = S.fErz[d][f0], bz0 = S.fBrz[d][f0];
        R fr1 = S.ffrR[d][f1], ef1 = S.fErz[d][f1], bz1 = S.fBrz[d][f1];
        acc(fr0, ef0, bz0);
        if (two) acc(fr1, ef1, bz1);
      });
      S.Eraw[(a + 0) * N + c] = e0; S.Eraw[(a + 2) * N + c] = e2;
      S.Braw[(a + 0) * N + c] = b0; S.Braw[(a + 2) * N + c] = b2;
      C.Ephi[(2 * d + 0) * N + c] = S.fEphi[d][S.run_dn_e[d][c]];
    }
    if (pa >= 0 && pair_in_flux_range(P, dim, pa)) {
      R e1 = S.Eraw[(a + 1) * N + c], e3 = S.Eraw[(a + 3) * N + c];
      R b1 = S.Braw[(a + 1) * N + c], b3 = S.Braw[(a + 3) * N + c];
      int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
      auto acc = [&](R fr, R ef, R bz) {
        e1 += (R).5 * ef * fr; e3 += (R).5 * ef * fr;
        b1 += (R).5 * bz * fr; b3 += (R).5 * bz * fr;
      };
      for_run2(S.run_up_s[d][c], S.run_up_e[d][c], base, Nf, [&](int f0, int f1, bool two) {
        R fr0 = S.ffrL[d][f0], ef0 = S.fErz[d][f0], bz0 = S.fBrz[d][f0];
        R fr1 = S.ffrL[d][f1], ef1 = S.fErz[d][f1], bz1 = S.fBrz[d][f1];
        acc(fr0, ef0, bz0);
        if (two) acc(fr1, ef1, bz1);
      });
      S.Eraw[(a + 1) * N + c] = e1; S.Eraw[(a + 3) * N + c] = e3;
      S.Braw[(a + 1) * N + c] = b1; S.Braw[(a + 3) * N + c] = b3;
      C.Ephi[(2 * d + 1) * N + c] = S.fEphi[d][S.run_up_e[d][c]];
    }
  }
}

// ---- avg_Efields (bfields.c:392-644) + subtract_advective_B_fluxes (:646-690)
// d1: neighbour average along phi; d2: face average with the interpolated
// value from the overlapping cell of the other ring; then E -= h w B.
//
// edge_avg_at: slot e of cell x after the phi-neighbour averaging pass, for
// a cell of the ring whose first cell and size are given (a face
// neighbour's ring follows from the pair, so its bounds load in parallel
// with the face lookup instead of after it).
template <typename R>
DISCO_D R edge_avg_at(const R* A, int N, int e, int x, int off, int Np) {
  int i = x - off;
  int xp = off + (i + 1 == Np ? 0 : i + 1), xm = off + (i == 0 ? Np - 1 : i - 1);
  int h = e & 4, s = e & 3;
  if (s == 0) return (R).5 * (A[(h + 0) * N + x] + A[(h + 2) * N + xp]);
  if (s == 1) return (R).5 * (A[(h + 1) * N + x] + A[(h + 3) * N + xp]);
  if (s == 2) return (R).5 * (A[(h + 0) * N + xm] + A[(h + 2) * N + x]);
  return (R).5 * (A[(h + 1) * N + xm] + A[(h + 3) * N + x]);
}

template <typename R>
__global__ void k_ct_avg(DevParams P, DevState<R> S, CtStateT<R> C) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  R outE[4], outB[4];
  // mixed path: the B average split by the ring whose frame the EMFs were
  // stored in (own ring / the neighbouring ring across the face)
  R ownB[4], othB[4], dOmo[4];
  bool has[4] = {false, false, false, false};
  // slots: 0 -> E0 (r lower), 1 -> E1 (r upper), 2 -> E4 (z lower), 3 -> E5 (z upper)
  const int slot_e[4] = {0, 1, 4, 5};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    outE[s] = edge_avg_at(S.Eraw, N, slot_e[s], c, off, Np);
    outB[s] = edge_avg_at(S.Braw, N, slot_e[s], c, off, Np);
    ownB[s] = outB[s]; othB[s] = 0; dOmo[s] = 0;
  }
#pragma unroll
  for (int dim = 1; dim <= 2; ++dim) {
    if (dim == 1 && P.Nr <= 1) continue;
    if (dim == 2 && P.Nz <= 1) continue;
    const int d = dim - 1, a = 4 * d;
    const int stride = dim == 1 ? 1 : P.Nr;   // ring index step across the pair
    int pa = pair_above(P, dim, j, k), pb = pair_below(P, dim, j, k);
    if (pa >= 0) {   // LRtype 0 face owned by c (c = L = c1, c2 = R)
      const int o2 = S.ring_off[jk + stride], n2 = S.ring_off[jk + stride + 1] - o2;
      int f = S.run_up_e[d][c];
      int c2 = S.nb_up[d][c];   // = fR of face f, loaded beside f
      R dp1 = S.fdp1[d][f], dp2 = S.fdp2[d][f];
      R Eavg = (dp2 * edge_avg_at(S.Eraw, N, a + 0, c2, o2, n2) + dp1 * edge_avg_at(S.Eraw, N, a + 2, c2, o2, n2)) / (dp1 + dp2);
      R Bavg = (dp2 * edge_avg_at(S.Braw, N, a + 0, c2, o2, n2) + dp1 * edge_avg_at(S.Braw, N, a + 2, c2, o2, n2)) / (dp1 + dp2);
      const int s = 2 * d + 1;
      outE[s] = (R).5 * (outE[s] + Eavg);
      outB[s] = (R).5 * (outB[s] + Bavg);
      has[s] = true; othB[s] = Bavg;
      if constexpr (kMix<R>) dOmo[s] = S.pdOm[d][pa];
    }
    if (pb >= 0) {   // LRtype 1 face owned by c (c = R = c1, c2 = L)
      const int o2 = S.ring_off[jk - stride], n2 = S.ring_off[jk - stride + 1] - o2;
      int f = S.run_dn_e[d][c];
      int c2 = S.nb_dn[d][c];   // = fL of face f, loaded beside f
      R dp1 = S.fdp1[d][f], dp2 = S.fdp2[d][f];
      R Eavg = (dp2 * edge_avg_at(S.Eraw, N, a + 1, c2, o2, n2) + dp1 * edge_avg_at(S.Eraw, N, a + 3, c2, o2, n2)) / (dp1 + dp2);
      R Bavg = (dp2 * edge_avg_at(S.Braw, N, a + 1, c2, o2, n2) + dp1 * edge_avg_at(S.Braw, N, a + 3, c2, o2, n2)) / (dp1 + dp2);
      const int s = 2 * d + 0;
      outE[s] = (R).5 * (outE[s] + Eavg);
      outB[s] = (R).5 * (outB[s] + Bavg);
      has[s] = true; othB[s] = Bavg;
      if constexpr (kMix<R>) dOmo[s] = -S.pdOm[d][pb];
    }
  }
  const double* rj = S.r_jph + 1;
  if constexpr (kMix<R>) {
    // E_lab - h w B = X + s h ((w - Om_own) B_own + (w - Om_other) B_other),
    // all frame differences small and exact to FP32 rounding
    R wrel = to_r<R>(S.wiph[c] - S.ring_Om[jk]);
    R hL = to_r<R>(rj[j - 1]), hR = to_r<R>(rj[j]), hC = S.ring_rc_r[jk];
    const R h[4] = {hL, hR, hC, hC};
    const R sg[4] = {(R)-1, (R)-1, (R)1, (R)1};
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      R bt = has[s] ? (R).5 * (wrel * ownB[s] + (wrel - dOmo[s]) * othB[s]) : wrel * ownB[s];
      C.Efin[s * N + c] = outE[s] + sg[s] * h[s] * bt;
    }
  } else {
    (void)ownB; (void)othB; (void)dOmo; (void)has;
    double hL = rj[j - 1], hR = rj[j];
    double hC = S.ring_rc[jk];
    double w = S.wiph[c];
    C.Efin[0 * N + c] = outE[0] - (R)(hL * w) * outB[0];
    C.Efin[1 * N + c] = outE[1] - (R)(hR * w) * outB[1];
    C.Efin[2 * N + c] = outE[2] + (R)(hC * w) * outB[2];
    C.Efin[3 * N + c] = outE[3] + (R)(hC * w) * outB[3];
  }
}

// ---- update_B_fluxes (bfields.c:313-382): Stokes circulation per face --------
// The reference's loop skips the last pair of each dimension (it visits pair
// jk-1 at index jk, jk < N_ftracks); that is reproduced.
template <typename R>
DISCO_D R face_emf(const DevState<R>& S, const CtStateT<R>& C, int d, int f) {
  const int N = S.N;
  if (S.fLR[d][f] == 0) return C.Efin[(2 * d + 1) * N + S.fL[d][f]];
  return C.Efin[(2 * d + 0) * N + S.fR[d][f]];
}

// Mixed path: each slot's circulation E dl dt is formed in R, summed per
// slot into dph and added to the FP64 flux once (the FP64 path below keeps
// the reference's terms).
template <typename R>
DISCO_D void ct_bflux_mixed(const DevParams& P, const DevState<R>& S, const CtStateT<R>& C,
                            double fac, int c, R* dph) {
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  R dtf = to_r<R>(fac) * dt_r<R>(S.scal);
#pragma unroll
  for (int q = 0; q < 5; ++q) dph[q] = 0;
  R dph0 = 0;
#pragma unroll
  for (int dim = 1; dim <= 2; ++dim) {
    if (dim == 1 && P.Nr <= 1) continue;
    if (dim == 2 && P.Nz <= 1) continue;
    const int d = dim - 1;
    R dldt = S.ring_dl_r[d][jk] * dtf;
    int pb = pair_below(P, dim, j, k), pa = pair_above(P, dim, j, k);
    if (pb >= 0 && pb != C.last_pair[d]) {
      int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
      int f = S.run_dn_e[d][c];
      int g = f == base ? base + Nf - 1 : f - 1;
      R Ef = C.Efin[(2 * d + 0) * N + c];
      R Eg = face_emf(S, C, d, g);
      int slot = dim == 1 ? 1 : 3;
      R dv = dim == 1 ? (Eg - Ef) * dldt : (Ef - Eg) * dldt;
      dph[slot] += dv;
      dph0 += dim == 1 ? -Ef * dldt : Ef * dldt;
    }
    if (pa >= 0 && pa != C.last_pair[d]) {
      int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
      int f = S.run_up_e[d][c];
      int g = f == base ? base + Nf - 1 : f - 1;
      R Ef = C.Efin[(2 * d + 1) * N + c];
      R Eg = face_emf(S, C, d, g);
      int slot = dim == 1 ? 2 : 4;
      R dv = dim == 1 ? (Eg - Ef) * dldt : (Ef - Eg) * dldt;
      dph[slot] += dv;
      dph0 += dim == 1 ? Ef * dldt : -Ef * dldt;
    }
  }
  dph[0] += dph0;
}

// The RK adjustment of the face fluxes (Phi -> (1 - RK) Phi + RK RKPhi, or
// RKPhi = Phi on the first substep) is done here, in registers, before the
// circulation terms: nothing reads Phi between the edge gathers and this
// kernel, so one pass over Phi serves both.
template <typename R>
__global__ void k_ct_bflux(DevParams P, DevState<R> S, CtStateT<R> C, double fac, double RK, int first) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  double ph[5];
  if constexpr (kMix<R>) {
    // circulation terms summed in R first, then Phi = RK RKPhi + ((1 - RK) Phi + d)
    R dph[5];
    ct_bflux_mixed<R>(P, S, C, fac, c, dph);
    const double a1 = 1. - RK;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      double v = C.Phi[q * N + c], d = from_r<R>(dph[q]);
      if (first) {
        C.RKPhi[q * N + c] = v;
        v += d;
      } else {
        v = fma(RK, C.RKPhi[q * N + c], fma(a1, v, d));
      }
      C.Phi[q * N + c] = v;
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    double v = C.Phi[q * N + c];
    if (first) C.RKPhi[q * N + c] = v;
    else v = (1. - RK) * v + RK * C.RKPhi[q * N + c];
    ph[q] = v;
  }
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  double dt = fac * S.scal[SC_DT];
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double ph0 = ph[0];
#pragma unroll
  for (int dim = 1; dim <= 2; ++dim) {
    if (dim == 1 && P.Nr <= 1) continue;
    if (dim == 2 && P.Nz <= 1) continue;
    const int d = dim - 1;
    double dl = dim == 1 ? (zk[k] - zk[k - 1]) : (rj[j] - rj[j - 1]);
    double sgn = dim == 1 ? 1.0 : -1.0;   // z faces circulate with the opposite sign
    int pb = pair_below(P, dim, j, k), pa = pair_above(P, dim, j, k);
    // lower pair: c is R, owns the LRtype-1 face run_dn_e (slot Phi[1] or Phi[3])
    if (pb >= 0 && pb != C.last_pair[d]) {
      int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
      int f = S.run_dn_e[d][c];
      int g = f == base ? base + Nf - 1 : f - 1;
      double Ef = (double)C.Efin[(2 * d + 0) * N + c];
      double Eg = (double)face_emf(S, C, d, g);
      int slot = dim == 1 ? 1 : 3;
      double v = ph[slot];
      if (dim == 1) {
        if (f == base) { v -= Ef * dl * dt; v += Eg * dl * dt; }
        else { v += Eg * dl * dt; v -= Ef * dl * dt; }
        ph0 -= Ef * dl * dt;
      } else {
        if (f == base) { v += Ef * dl * dt; v -= Eg * dl * dt; }
        else { v -= Eg * dl * dt; v += Ef * dl * dt; }
      }
      ph[slot] = v;
      if (dim == 2) ph0 += Ef * dl * dt;
    }
    if (pa >= 0 && pa != C.last_pair[d]) {
      int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
      int f = S.run_up_e[d][c];
      int g = f == base ? base + Nf - 1 : f - 1;
      double Ef = (double)C.Efin[(2 * d + 1) * N + c];
      double Eg = (double)face_emf(S, C, d, g);
      int slot = dim == 1 ? 2 : 4;
      double v = ph[slot];
      if (dim == 1) {
        if (f == base) { v -= Ef * dl * dt; v += Eg * dl * dt; }
        else { v += Eg * dl * dt; v -= Ef * dl * dt; }
        ph0 += Ef * dl * dt;
      } else {
        if (f == base) { v += Ef * dl * dt; v -= Eg * dl * dt; }
        else { v -= Eg * dl * dt; v += Ef * dl * dt; }
        ph0 -= Ef * dl * dt;
      }
      ph[slot] = v;
    }
    (void)sgn;
  }
  ph[0] = ph0;
#pragma unroll
  for (int q = 0; q < 5; ++q) C.Phi[q * N + c] = ph[q];
}

// ---- make_edge_adjust (bfields.c:888-1127) -------------------------------------
// The reference walks, for each corner line (r_j, z_k), the four rings around
// it in phi order (a 4-way merge of their upper cell edges, ties ordered
// c < cR < cU < cUR) and adds E_phi dl dt to the four faces meeting there.
// Every walk event advances exactly one cell, so events map one-to-one onto
// the cells of the four rings: here each thread takes one cell, finds the
// heads of the other three rings by binary search, and evaluates that event.
// Contributions from different events to one face are summed with FP64
// atomics (order may differ from the reference at rounding level).
DISCO_D int phi_switch(double dphi, double Pmax, int mode) {
  while (dphi > .5 * Pmax) dphi -= Pmax;
  while (dphi < -.5 * Pmax) dphi += Pmax;
  if (mode == 1) dphi = -dphi;
  return dphi > 0. ? 1 : 0;
}
DISCO_D int get_which4(double phi, double phiR, double phiU, double phiUR, int* LR_alt, int* UD_alt,
                       int mode, double Pmax) {
  int LR_D = phi_switch(phi - phiR, Pmax, mode);
  int LR_U = phi_switch(phiU - phiUR, Pmax, mode);
  double phi1 = LR_D ? phiR : phi, phi2 = LR_U ? phiUR : phiU;
  int UD = phi_switch(phi1 - phi2, Pmax, mode);
  int w4 = UD == 0 ? (LR_D == 0 ? 0 : 1) : (LR_U == 0 ? 2 : 3);
  if (mode == 0) {
    *LR_alt = (w4 == 0 || w4 == 1) ? LR_U : LR_D;
    if (w4 == 0 || w4 == 2) *UD_alt = phi_switch(phiR - phiUR, Pmax, mode);
    else *UD_alt = phi_switch(phi - phiU, Pmax, mode);
  }
  return w4;
}

// The four face fluxes an edge event adjusts and its averaged E_phi
// (bfields.c:955-1110): from the ring that advanced (w4), the two branch
// bits and the four current cells (c, cR, cU, cUR).
template <typename R>
DISCO_D void edge_targets(const CtStateT<R>& C, int N, int w4, int LR_alt, int UD_alt, int c, int cR,
                          int cU, int cUR, double** PL, double** PR, double** PU, double** PD, R* Eo) {
  const R* Ep = C.Ephi;
  R E;
  double *PhiL, *PhiR, *PhiU, *PhiD;
  double* Ph = C.Phi;
  if (w4 == 0) {
    PhiL = Ph + 4 * N + c; PhiD = Ph + 2 * N + c;
    E = (R).25 * (Ep[3 * N + c] + Ep[1 * N + c]);
    if (LR_alt == 0) { PhiU = Ph + 2 * N + cU; E += (R).25 * Ep[1 * N + cU]; }
    else { PhiU = Ph + 1 * N + cUR; E += (R).25 * Ep[0 * N + cUR]; }
    if (UD_alt == 0) { PhiR = Ph + 4 * N + cR; E += (R).25 * Ep[3 * N + cR]; }
    else { PhiR = Ph + 3 * N + cUR; E += (R).25 * Ep[2 * N + cUR]; }
  } else if (w4 == 1) {
    PhiR = Ph + 4 * N + cR; PhiD = Ph + 1 * N + cR;
    E = (R).25 * (Ep[3 * N + cR] + Ep[0 * N + cR]);
    if (LR_alt == 0) { PhiU = Ph + 2 * N + cU; E += (R).25 * Ep[1 * N + cU]; }
    else { PhiU = Ph + 1 * N + cUR; E += (R).25 * Ep[0 * N + cUR]; }
    if (UD_alt == 0) { PhiL = Ph + 4 * N + c; E += (R).25 * Ep[3 * N + c]; }
    else { PhiL = Ph + 3 * N + cU; E += (R).25 * Ep[2 * N + cU]; }
  } else if (w4 == 2) {
    PhiL = Ph + 3 * N + cU; PhiU = Ph + 2 * N + cU;
    E = (R).25 * (Ep[2 * N + cU] + Ep[1 * N + cU]);
    if (LR_alt == 0) { PhiD = Ph + 2 * N + c; E += (R).25 * Ep[1 * N + c]; }
    else { PhiD = Ph + 1 * N + cR; E += (R).25 * Ep[0 * N + cR]; }
    if (UD_alt == 0) { PhiR = Ph + 4 * N + cR; E += (R).25 * Ep[3 * N + cR]; }
    else { PhiR = Ph + 3 * N + cUR; E += (R).25 * Ep[2 * N + cUR]; }
  } else {
    PhiR = Ph + 3 * N + cUR; PhiU = Ph + 1 * N + cUR;
    E = (R).25 * (Ep[2 * N + cUR] + Ep[0 * N + cUR]);
    if (LR_alt == 0) { PhiD = Ph + 2 * N + c; E += (R).25 * Ep[1 * N + c]; }
    else { PhiD = Ph + 1 * N + cR; E += (R).25 * Ep[0 * N + cR]; }
    if (UD_alt == 0) { PhiL = Ph + 4 * N + c; E += (R).25 * Ep[3 * N + c]; }
    else { PhiL = Ph + 3 * N + cU; E += (R).25 * Ep[2 * N + cU]; }
  }
  *PL = PhiL; *PR = PhiR; *PU = PhiU; *PD = PhiD; *Eo = E;
}

// E dl dt of one event (FP64 on the FP64 path, R on the mixed path).
template <typename R>
DISCO_D double edge_edldt(R E, R dl, R dtf, double dt) {
  if constexpr (kMix<R>) return from_r<R>(E * (dl * dtf));
  else return (double)E * dl * dt;
}

// mode 0: always walk; mode 1: walk only if the cache is stale (first
// substep); mode 2: walk and record the events for the next step.
template <typename R>
__global__ void k_ct_edge(DevParams P, DevState<R> S, CtStateT<R> C, double fac, int mode) {
  extern __shared__ double sm[];
  if (mode == 1 && C.ev_ok && *C.ev_ok) return;
  const bool cache = mode == 2 && C.ev_cid != nullptr;
  int q = blockIdx.x;   // quad (j, k): rings j, j+1 at layers k, k+1
  const long ev0 = cache ? (long)C.quad_ev_off[q] : 0;
  int k = div_fast(q, P.mul_nr1), j = q - k * (P.Nr - 1);
  const int N = S.N;
  int ring[4] = {j + P.Nr * k, j + 1 + P.Nr * k, j + P.Nr * (k + 1), j + 1 + P.Nr * (k + 1)};
  int off[4], np[4], I0[4], base[4];
  int tot = 0;
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    off[x] = S.ring_off[ring[x]];
    np[x] = S.ring_off[ring[x] + 1] - off[x];
    I0[x] = S.anchor[ring[x]];
    base[x] = tot;
    tot += np[x];
  }
  // rotated piph of the four rings as IEEE bit patterns: positions are
  // non-negative, so integer order equals numeric order and the merge-order
  // search runs on the integer pipe.
  long long* sp = (long long*)sm;
  for (int x = 0; x < 4; ++x)
    for (int m = threadIdx.x; m < np[x]; m += blockDim.x) {
      int t = I0[x] + m;   // I0 < np, m < np: one conditional wrap
      t -= t >= np[x] ? np[x] : 0;
      sp[base[x] + m] = __double_as_longlong(S.piph[off[x] + t]);
    }
  __syncthreads();
  const double Pmax = P.phi_max;
  int lapoff[4];
  lapoff[0] = 0;
#pragma unroll
  for (int x = 1; x < 4; ++x) {
    double raw = __longlong_as_double(sp[base[0]]) - __longlong_as_double(sp[base[x]]);
    lapoff[x] = raw > .5 * Pmax ? 1 : (raw < -.5 * Pmax ? -1 : 0);
  }
  // m is in [-1, np[x]]: one wrap at most, no integer division needed
  // (x may be a runtime ring index: selects keep the small arrays in registers)
  auto pick = [](const int* a, int x) { return x == 0 ? a[0] : x == 1 ? a[1] : x == 2 ? a[2] : a[3]; };
  auto key = [&](int x, int m, int& lap, long long& ph) {
    int npx = pick(np, x), bx = pick(base, x);
    int wrap = m >= npx ? 1 : (m < 0 ? -1 : 0);
    int mm = m - wrap * npx;
    ph = sp[bx + mm];
    lap = wrap + ((mm > 0 && ph < sp[bx]) ? 1 : 0) + pick(lapoff, x);
  };
  double dt = fac * S.scal[SC_DT];
  const double rjj = S.r_jph[j + 1];
  const R rjr = (R)rjj;
  R dtf = 0;
  if constexpr (kMix<R>) dtf = to_r<R>(fac) * dt_r<R>(S.scal);
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int rx = t >= base[3] ? 3 : t >= base[2] ? 2 : t >= base[1] ? 1 : 0;
    int m = t - pick(base, rx);
    int lx; long long px;
    key(rx, m, lx, px);
    int head[4];
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      if (y == rx) { head[y] = m; continue; }
      // number of Y elements ordered before X[m]: (lap, phi, rank)
      // lexicographic, searched from the proportional position
      int hint = __float2int_rn((float)m * ((float)np[y] / (float)pick(np, rx)));
      head[y] = gallop_search(0, np[y], hint, [&](int mid) {
        int ly; long long py;
        key(y, mid, ly, py);
        return (ly < lx) || (ly == lx && (py < px || (py == px && y < rx)));
      });
    }
    int cid[4];
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      int t2 = I0[y] + head[y];
      t2 -= t2 >= np[y] ? np[y] : 0;
      t2 -= t2 >= np[y] ? np[y] : 0;
      cid[y] = off[y] + t2;
    }
    int LR_alt, UD_alt, w4, w4b;
    double pp[4], pb[4];
    double xp1, xm1;
    if constexpr (kMix<R>) {
      // get_which4 on the merge keys: the heads' upper edges, and the
      // predecessors' upper edges for the lower edges ("after" = strictly
      // later in the (lap, phi) order, the wrapped comparison's meaning)
      int hl[4], bl[4];
      long long hk[4], bk[4];
#pragma unroll
      for (int y = 0; y < 4; ++y) { key(y, head[y], hl[y], hk[y]); key(y, head[y] - 1, bl[y], bk[y]); }
      auto after = [](int la, long long pa, int lb, long long pb_) {
        return la > lb || (la == lb && pa > pb_);
      };
      // (selects instead of runtime indices keep the arrays in registers)
      int LR_D = after(hl[0], hk[0], hl[1], hk[1]);
      int LR_U = after(hl[2], hk[2], hl[3], hk[3]);
      int l1 = LR_D ? hl[1] : hl[0], l2 = LR_U ? hl[3] : hl[2];
      long long k1 = LR_D ? hk[1] : hk[0], k2 = LR_U ? hk[3] : hk[2];
      int UD = after(l1, k1, l2, k2);
      w4 = UD == 0 ? (LR_D == 0 ? 0 : 1) : (LR_U == 0 ? 2 : 3);
      LR_alt = (w4 == 0 || w4 == 1) ? LR_U : LR_D;
      UD_alt = (w4 == 0 || w4 == 2) ? after(hl[1], hk[1], hl[3], hk[3]) : after(hl[0], hk[0], hl[2], hk[2]);
      int LB_D = after(bl[1], bk[1], bl[0], bk[0]);
      int LB_U = after(bl[3], bk[3], bl[2], bk[2]);
      int m1 = LB_D ? bl[1] : bl[0], m2 = LB_U ? bl[3] : bl[2];
      long long n1 = LB_D ? bk[1] : bk[0], n2 = LB_U ? bk[3] : bk[2];
      int UB = after(m2, n2, m1, n1);
      w4b = UB == 0 ? (LB_D == 0 ? 0 : 1) : (LB_U == 0 ? 2 : 3);
      xp1 = phi_unkey(UD == 0 ? k1 : k2);
      xm1 = phi_unkey(UB == 0 ? n1 : n2);
      (void)pp; (void)pb;
    } else {
#pragma unroll
      for (int y = 0; y < 4; ++y) { pp[y] = S.piph[cid[y]]; pb[y] = pp[y] - S.dphi[cid[y]]; }
      w4 = get_which4(pp[0], pp[1], pp[2], pp[3], &LR_alt, &UD_alt, 0, Pmax);
      w4b = get_which4(pb[0], pb[1], pb[2], pb[3], nullptr, nullptr, 1, Pmax);
      xp1 = w4 == 0 ? pp[0] : w4 == 1 ? pp[1] : w4 == 2 ? pp[2] : pp[3];
      xm1 = w4b == 0 ? pb[0] : w4b == 1 ? pb[1] : w4b == 2 ? pb[2] : pb[3];
    }
    if (w4 != rx) {
      atomicAdd(C.errs, 1ull);
      if (cache) C.ev_flag[ev0 + t] = 0;
      continue;
    }
    int c = cid[0], cR = cid[1], cU = cid[2], cUR = cid[3];
    R E;
    double *PhiL, *PhiR, *PhiU, *PhiD;
    edge_targets<R>(C, N, w4, LR_alt, UD_alt, c, cR, cU, cUR, &PhiL, &PhiR, &PhiU, &PhiD, &E);
    R dl;   // edge length r dphi (the phi extent wrapped in FP64)
    if constexpr (kMix<R>) {
      // xp1, xm1 in [0, Pmax]: one FP64 difference, at most one wrap (the
      // bits of a negative non-zero double exceed 2^63 as unsigned), converted
      // on the integer pipe
      double dp = xp1 - xm1;
      if ((unsigned long long)__double_as_longlong(dp) > 0x8000000000000000ull) dp += Pmax;
      dl = rjr * d2f_int(dp);
    } else {
      dl = (.5 * (rjj + rjj)) * get_dp(xp1, xm1, Pmax);
    }
    if (cache) {
      long e = ev0 + t;
      C.ev_cid[e] = make_int4(c, cR, cU, cUR);
      C.ev_flag[e] = (unsigned char)(w4 | (LR_alt << 2) | (UD_alt << 3) | 0x80);
      C.ev_dl[e] = dl;
    }
    double Edldt = edge_edldt<R>(E, dl, dtf, dt);
    atomicAdd(PhiL, -Edldt);
    atomicAdd(PhiR, Edldt);
    atomicAdd(PhiU, -Edldt);
    atomicAdd(PhiD, Edldt);
  }
}

// Replay of the recorded edge events (first substep, cache current): the
// same targets, average and edge length as the walk, from the current E_phi.
template <typename R>
__global__ void k_ct_edge_replay(DevParams P, DevState<R> S, CtStateT<R> C, double fac, long nev) {
  if (!*C.ev_ok) return;
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nev) return;
  unsigned fl = C.ev_flag[e];
  if (!(fl & 0x80)) return;
  int4 cc = C.ev_cid[e];
  R E;
  double *PhiL, *PhiR, *PhiU, *PhiD;
  edge_targets<R>(C, S.N, fl & 3, (fl >> 2) & 1, (fl >> 3) & 1, cc.x, cc.y, cc.z, cc.w,
                  &PhiL, &PhiR, &PhiU, &PhiD, &E);
  double dt = fac * S.scal[SC_DT];
  R dtf = 0;
  if constexpr (kMix<R>) dtf = to_r<R>(fac) * dt_r<R>(S.scal);
  double Edldt = edge_edldt<R>(E, C.ev_dl[e], dtf, dt);
  atomicAdd(PhiL, -Edldt);
  atomicAdd(PhiR, Edldt);
  atomicAdd(PhiU, -Edldt);
  atomicAdd(PhiD, Edldt);
}

static __global__ void k_set_flag(int* f, int v) { *f = v; }

// ---- check_flipped + flip_fluxes (bfields.c:693-814), first substep --------------
// One block per pair; flags in parallel, then the sequential repair (rare).
template <typename R>
__global__ void k_ct_flip(DevParams P, DevState<R> S, CtStateT<R> C, int dim) {
  extern __shared__ unsigned char fsm[];
  const int d = dim - 1;
  int pair = blockIdx.x;
  if (pair == C.last_pair[d]) return;   // the reference loops skip the last pair
  int base = S.face_off[d][pair], Nf = S.face_off[d][pair + 1] - base;
  // shared: lr[Nf] (int8), then the ascending list of flagged faces (int)
  signed char* lr = (signed char*)fsm;
  int* list = (int*)(fsm + ((Nf + 15) & ~15));
  __shared__ int cnt[256];
  for (int n = threadIdx.x; n < Nf; n += blockDim.x) lr[n] = S.fLR[d][base + n];
  __syncthreads();
  // each thread flags a contiguous chunk, so a prefix over the per-thread
  // counts lists the flagged faces in ascending order
  const int chunk = (Nf + blockDim.x - 1) / blockDim.x;
  const int n0 = threadIdx.x * chunk, n1 = min(Nf, n0 + chunk);
  unsigned long long bits = 0;   // chunk <= 64 (Nf <= 16384)
  int mine = 0;
  // the end edge of face n: piph of its L cell (LRtype 0) or of its R cell
  auto edge = [&](int n) {
    const int f = base + n;
    return S.piph[lr[n] == 0 ? S.fL[d][f] : S.fR[d][f]];
  };
  double pm = n0 < n1 ? edge(n0) : 0.0;   // carried from face to face: one gather each
#pragma unroll 4
  for (int n = n0; n < n1; ++n) {
    int np = n + 1 == Nf ? 0 : n + 1;   // face np is flagged when its end edge precedes face n's
    const double pp = edge(np);
    bool flip;
    if constexpr (kMix<R>) {   // the same test with the wrap on bit patterns
      double dp = get_signed_dp_bits(pp, pm, P.phi_max);
      flip = (unsigned long long)__double_as_longlong(dp) > 0x8000000000000000ull &&
             (unsigned long long)__double_as_longlong(dp) < 0xfff0000000000000ull;
    } else {
      flip = get_signed_dp(pp, pm, P.phi_max) < 0.;
    }
    if (flip) { bits |= 1ull << (n - n0); ++mine; }
    pm = pp;
  }
  cnt[threadIdx.x] = mine;
  // nothing flagged in this pair (the common case): fLR stays, no repair
  if (!__syncthreads_or(mine)) return;
  if (threadIdx.x == 0) {   // exclusive scan of 256 counts (cheap, one thread)
    int acc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) { int v = cnt[t]; cnt[t] = acc; acc += v; }
    list[Nf] = acc;
  }
  __syncthreads();
  {
    int w = cnt[threadIdx.x];
    for (int n = n0; n < n1; ++n)
      if (bits >> (n - n0) & 1ull) list[w++] = n + 1 == Nf ? 0 : n + 1;
  }
  __syncthreads();   // the list is complete before anyone reads it
  __shared__ int last_start;
  const int nflag = list[Nf];
  // flip_fluxes in ascending face order (the list holds n + 1 for each n;
  // the wrap-around face 0 comes from the last chunk, so it is visited first)
  const bool wrap0 = list[nflag - 1] == 0;
  auto ord = [&](int t) { return wrap0 ? (t == 0 ? 0 : list[t - 1]) : list[t]; };
  // Faces x < y (the last face one chain touches, the first face the next
  // chain touches) leave the two chains independent when they are distinct
  // faces and share neither their L nor their R cell: the cells of a pair's
  // faces advance monotonically with the face index, so no face up to x then
  // shares a cell (hence a flux slot) with a face from y on.
  auto apart = [&](int x, int y) {
    if (y <= x) return false;
    int fx = base + (x >= Nf ? x - Nf : x), fy = base + (y >= Nf ? y - Nf : y);
    return S.fL[d][fx] != S.fL[d][fy] && S.fR[d][fx] != S.fR[d][fy];
  };
  // entry t (> 0) starts a chain when it is apart from entry t - 1
  auto starts = [&](int t) { return apart(ord(t - 1) + 1, ord(t) - 1); };
  if (threadIdx.x == 0) {   // the last chain's first entry (see below)
    int t = nflag - 1;
    while (t > 0 && !starts(t)) --t;
    last_start = t;
  }
  __syncthreads();
  const int N = S.N;
  int lo = d == 0 ? 2 : 4, hi = d == 0 ? 1 : 3;
  auto slot = [&](int n) -> long long {
    int f = base + n;
    return lr[n] == 0 ? (long long)lo * N + S.fL[d][f] : (long long)hi * N + S.fR[d][f];
  };
  auto repair = [&](int n) {
    int np = n + 1 == Nf ? 0 : n + 1, nm = n == 0 ? Nf - 1 : n - 1;
    long long s = slot(n), sm_ = slot(nm), sp = slot(np);
    double Phi = C.Phi[s], RPhi = C.RKPhi[s];
    C.Phi[s] = C.Phi[sm_] + Phi; C.RKPhi[s] = C.RKPhi[sm_] + RPhi;
    C.Phi[sm_] = -Phi; C.RKPhi[sm_] = -RPhi;
    C.Phi[sp] = C.Phi[sp] + Phi; C.RKPhi[sp] = C.RKPhi[sp] + RPhi;
    lr[n] = !lr[n];
    lr[nm] = !lr[nm];
  };
  if (Nf <= 6) {   // every face within two of every other: one serial chain
    if (threadIdx.x == 0)
      for (int t = 0; t < nflag; ++t) repair(ord(t));
  } else {
    // repair(n) touches the slots of faces n - 1, n, n + 1 and flips lr[n - 1]
    // and lr[n]: flagged faces that are not apart form a chain and are
    // repaired in order by one thread; different chains touch disjoint slots
    // and lr entries, so they run in parallel with the same result.  The
    // first and the last chain are one chain when they meet across the wrap
    // (face Nf - 1 next to face 0): the first chain's thread then continues
    // with the last chain, which keeps the ascending order.
    const bool linked = nflag > 1 && !apart(ord(nflag - 1) + 1, ord(0) - 1 + Nf);
    for (int t = threadIdx.x; t < nflag; t += blockDim.x) {
      if (t > 0 && !starts(t)) continue;                   // not a chain start
      if (linked && t > 0 && t == last_start) continue;   // done by chain 0
      int u = t;
      repair(ord(u));
      while (u + 1 < nflag && !starts(u + 1)) repair(ord(++u));
      if (t == 0 && linked && last_start > u)
        for (int v = last_start; v < nflag; ++v) repair(ord(v));
    }
  }
  __syncthreads();
  for (int n = threadIdx.x; n < Nf; n += blockDim.x) S.fLR[d][base + n] = lr[n];
}

// ---- B_faces_to_cells type 1 (bfields.c:88-309): cell B from face fluxes ---------
template <typename R, int NQ>
DISCO_D void ct_b2c_cell(const DevParams& P, const DevState<R>& S, const CtStateT<R>& C, int c,
                         int prim_out) {
  const int N = S.N;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!prim_out && !is_real(P, j, k)) return;
  int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  int i = c - off;
  int cm = off + (i == 0 ? Np - 1 : i - 1);
  if constexpr (kMix<R>) {   // face fluxes summed in R
    R sums[2] = {0, 0}, areas[2] = {0, 0};
#pragma unroll
    for (int dim = 1; dim <= 2; ++dim) {
      if (dim == 1 && P.Nr <= 1) continue;
      if (dim == 2 && P.Nz <= 1) continue;
      const int d = dim - 1;
      int lo = d == 0 ? 2 : 4, hi = d == 0 ? 1 : 3;
      int pb = pair_below(P, dim, j, k), pa = pair_above(P, dim, j, k);
      // the owning cell's slot of a face: L's lo slot or R's hi slot
      auto slot = [&](int f) {
        return S.fLR[d][f] == 0 ? lo * N + S.fL[d][f] : hi * N + S.fR[d][f];
      };
      // two faces' loads in flight per iteration, summed in run order
      auto visit2 = [&](int f0, int f1, bool two) {
        int s0 = slot(f0), s1 = slot(f1);
        R a0 = S.fdA[d][f0], a1 = S.fdA[d][f1];
        double p0 = C.Phi[s0], p1 = C.Phi[s1];
        areas[d] += a0;
        sums[d] += to_r<R>(p0);
        if (two) {
          areas[d] += a1;
          sums[d] += to_r<R>(p1);
        }
      };
      if (pb >= 0) {
        int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
        for_run2(S.run_dn_s[d][c], S.run_dn_e[d][c], base, Nf, visit2);
      }
      if (pa >= 0) {
        int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
        for_run2(S.run_up_s[d][c], S.run_up_e[d][c], base, Nf, visit2);
      }
    }
    R Bphi = (R).5 * to_r<R>(C.Phi[c] + C.Phi[cm]);
    R dA = S.ring_dA_r[jk];
    R x0 = S.ring_rc_r[jk];
    if (prim_out) {
      S.prim[BRR * N + c] = sums[0] / areas[0];
      S.prim[BPP * N + c] = Bphi / dA;
      if (P.Nz > 1) S.prim[BZZ * N + c] = sums[1] / areas[1];
    } else {
      R dV = S.ring_vol_r[jk] * S.dphi_r[c];
      S.cons[BRR * N + c] = from_r<R>(sums[0] * (dV / (areas[0] * x0)));
      S.cons[BPP * N + c] = from_r<R>(Bphi * dV / (dA * x0));
      if (P.Nz > 1) S.cons[BZZ * N + c] = from_r<R>(sums[1] * (dV / areas[1]));
    }
    return;
  }
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double xp0 = rj[j], xm0 = rj[j - 1], xp2 = zk[k], xm2 = zk[k - 1];
  double xp1 = S.piph[c], xm1 = S.piph[cm];
  double x0 = S.ring_rc[jk];
  double dA = (xp0 - xm0) * (xp2 - xm2);
  double dV = (.5 * (xp0 + xm0)) * (xp0 - xm0) * get_dp(xp1, xm1, P.phi_max) * (xp2 - xm2);
  double sums[2] = {0, 0}, areas[2] = {0, 0};
  for (int dim = 1; dim <= 2; ++dim) {
    if (dim == 1 && P.Nr <= 1) continue;
    if (dim == 2 && P.Nz <= 1) continue;
    const int d = dim - 1;
    int lo = d == 0 ? 2 : 4, hi = d == 0 ? 1 : 3;
    int pb = pair_below(P, dim, j, k), pa = pair_above(P, dim, j, k);
    auto visit = [&](int f) {
      double ph = S.fLR[d][f] == 0 ? C.Phi[lo * N + S.fL[d][f]] : C.Phi[hi * N + S.fR[d][f]];
      areas[d] += (double)S.fdA[d][f];
      sums[d] += ph;
    };
    if (pb >= 0) {
      int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
      for_run(S.run_dn_s[d][c], S.run_dn_e[d][c], base, Nf, visit);
    }
    if (pa >= 0) {
      int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
      for_run(S.run_up_s[d][c], S.run_up_e[d][c], base, Nf, visit);
    }
  }
  double Bphi = .5 * (C.Phi[c] + C.Phi[cm]);
  if (prim_out) {   // type 0 (primitive B), used once at set-up
    S.prim[BRR * N + c] = (R)(sums[0] / areas[0]);
    S.prim[BPP * N + c] = (R)(Bphi / dA);
    if (P.Nz > 1) S.prim[BZZ * N + c] = (R)(sums[1] / areas[1]);
  } else {
    double rfac = 1.0 / x0, hr = 1.0, hp = x0;
    S.cons[BRR * N + c] = sums[0] * (dV * rfac / (areas[0] * hr));
    S.cons[BPP * N + c] = Bphi * dV / (dA * hp);
    if (P.Nz > 1) S.cons[BZZ * N + c] = sums[1] * (dV * 1.0 / (areas[1] * 1.0));
  }
}


template <typename R, int NQ>
__global__ void k_ct_b2c(DevParams P, DevState<R> S, CtStateT<R> C, int prim_out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  ct_b2c_cell<R, NQ>(P, S, C, c, prim_out);
}

// B_faces_to_cells then calc_prim of the same real cell (onestep.c:285-296),
// one pass over the conserved state instead of two.
template <typename Phys, typename R, int NQ>
__global__ void k_ct_b2c_c2p(DevParams P, DevState<R> S, CtStateT<R> C) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (!is_real(P, j, k)) return;
  ct_b2c_cell<R, NQ>(P, S, C, c, 0);
  c2p_cell<Phys, R, NQ>(P, S, c, jk, j, k);
}

// ---- set_B_fields (bfields.c:13-86): face fluxes of the initial field ------------
template <typename R>
__global__ void k_ct_init_phi0(DevParams P, DevState<R> S, CtStateT<R> C) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  int jk = S.cell_ring[c];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double x[3] = {S.ring_rc[jk], S.piph[c], centroid_z(zk[k], zk[k - 1])};
  double prim[MAX_Q];
  initial_eval(P, prim, x);
  double dA = (rj[j] - rj[j - 1]) * (zk[k] - zk[k - 1]);
  C.Phi[c] = prim[BPP] * dA;
}

template <typename R>
__global__ void k_ct_init_face_phi(DevParams P, DevState<R> S, CtStateT<R> C, int dim) {
  const int d = dim - 1;
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= S.nf[d]) return;
  // face centre cm = (r, phic, z) of its pair
  int cL = S.fL[d][f];
  int jk = S.cell_ring[cL];
  int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  double x[3];
  if (dim == 1) { x[0] = .5 * (rj[j] + rj[j]); x[2] = centroid_z(zk[k], zk[k - 1]); }
  else { x[0] = centroid_r(rj[j], rj[j - 1]); x[2] = .5 * (zk[k] + zk[k]); }
  x[1] = S.fphic[d][f];
  double prim[MAX_Q];
  initial_eval(P, prim, x);
  double Phi = (dim == 1 ? prim[BRR] : prim[BZZ]) * (double)S.fdA[d][f];
  const int N = S.N;
  if (S.fLR[d][f] == 0) C.Phi[(dim == 1 ? 2 : 4) * N + cL] = Phi;
  else C.Phi[(dim == 1 ? 1 : 3) * N + S.fR[d][f]] = Phi;
}

}  // namespace disco
