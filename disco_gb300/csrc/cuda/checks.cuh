// Checks of the device state that the reference's hot path does not run
// itself: the divergence of B held as face fluxes, and a kernel that applies
// the integer-pipe FP64 <-> FP32 conversions to a buffer so that they can be
// compared with the hardware conversions.
#pragma once
#include "ct_kernels.cuh"

namespace disco {

// Net outward magnetic flux of every cell, from the face fluxes that
// constrained transport evolves (the sum Python/discopy/geom.py:370-520
// (calcDivB) forms on a checkpoint):
//   Phi[0] of the cell (its upper phi face) - Phi[0] of its phi neighbour
//   below, + every r / z face above the cell - every face below it.
// A sheared face's flux lives in the cell that owns the face's end edge
// (bfields.c:52-76): L.Phi[2] (r) / L.Phi[4] (z) for LRtype 0, else
// R.Phi[1] / R.Phi[3].  `scale` gets the sum of the absolute face fluxes of
// the cell, so |div| / scale is the divergence relative to the flux through
// the cell.  Cells without a neighbour ring on every side get div = 0 and
// scale = -1 (not evaluated).  Faces are visited in ascending order, so the
// result is deterministic.
template <typename R>
__global__ void k_divb(DevParams P, DevState<R> S, CtStateT<R> C, double* div, double* scale) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.N) return;
  const int N = S.N;
  const int jk = S.cell_ring[c];
  const int k = jk / P.Nr, j = jk - k * P.Nr;
  bool inner = (P.Nr <= 1 || (j > 0 && j < P.Nr - 1)) && (P.Nz <= 1 || (k > 0 && k < P.Nz - 1));
  if (!inner) { div[c] = 0.0; scale[c] = -1.0; return; }
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const int i = c - off;
  const int cm = off + (i == 0 ? Np - 1 : i - 1);
  const double* Phi = C.Phi;
  double s = Phi[c] - Phi[cm];
  double a = fabs(Phi[c]) + fabs(Phi[cm]);
  for (int dim = 1; dim <= 2; ++dim) {
    if ((dim == 1 && P.Nr <= 1) || (dim == 2 && P.Nz <= 1)) continue;
    const int d = dim - 1;
    auto flux = [&](int f) {
      return S.fLR[d][f] == 0 ? Phi[(size_t)(2 + 2 * d) * N + S.fL[d][f]]
                              : Phi[(size_t)(1 + 2 * d) * N + S.fR[d][f]];
    };
    const int pa = pair_above(P, dim, j, k), pb = pair_below(P, dim, j, k);
    {
      const int base = S.face_off[d][pa], Nf = S.face_off[d][pa + 1] - base;
      for_run(S.run_up_s[d][c], S.run_up_e[d][c], base, Nf, [&](int f) {
        double x = flux(f);
        s += x;
        a += fabs(x);
      });
    }
    {
      const int base = S.face_off[d][pb], Nf = S.face_off[d][pb + 1] - base;
      for_run(S.run_dn_s[d][c], S.run_dn_e[d][c], base, Nf, [&](int f) {
        double x = flux(f);
        s -= x;
        a += fabs(x);
      });
    }
  }
  div[c] = s;
  scale[c] = a;
}

// The conversions of dev_common.cuh and the hardware's, element by element.
static __global__ void k_convert_check(const double* in, long n, float* f_int, float* f_hw,
                                const float* fin, double* d_int, double* d_hw) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const double x = in[t];
    f_int[t] = d2f_int(x);
    f_hw[t] = __double2float_rn(x);
    const float y = fin[t];
    d_int[t] = f2d_int(y);
    d_hw[t] = (double)y;
  }
}

}  // namespace disco
