// The GRMHD cons2prim pass that uses the learned starting point (mlp.cuh):
// calc_prim (misc.c:300-335 with grmhd.c:228) with the network's corrected
// start, or with the reference's start while recording training pairs.
#pragma once
#include "kernels.cuh"
#include "mlp.cuh"

namespace disco {

// Geometry of the cons2prim of real cell c (the FP64 calc_prim of k_update):
// dV and the point x at which the reference evaluates the metric.
template <typename R>
DISCO_D void c2p_geometry(const DevParams& P, const DevState<R>& S, int c, int jk, int j, int k, double* dV,
                          double* x) {
  const double* rj = S.r_jph + 1;
  const double* zk = S.z_kph + 1;
  const double piph = S.piph[c], dphi = S.dphi[c];
  const double rp = rj[j], rm = rj[j - 1], zp = zk[k], zm = zk[k - 1];
  const double phim = piph - dphi;
  *dV = (.5 * (rp + rm)) * (rp - rm) * get_dp(piph, phim, P.phi_max) * (zp - zm);
  x[0] = S.ring_rc[jk];
  x[1] = .5 * (phim + piph);
  x[2] = .5 * (zp + zm);
}

// Where the cons2prim pass records training pairs (X null: nowhere): for
// every stride-th real cell, the features and the change of log(W^2 - 1)
// and log(P / rho) from the previous primitives to the converged solution.
struct C2PRecord {
  float* X;
  float* Y;
  long cap;
  unsigned long long* count;
  int stride;
};

// calc_prim of the GRMHD module with the learned starting point: each warp
// evaluates the network for its 32 cells on the tensor cores, then every
// thread solves its cell from the corrected start -- or from the previous
// primitives where the corrected start's residual is not below m.warm_ratio
// times theirs, where theirs is at most m.warm_floor, or where Newton from
// the corrected start does not converge: the reference's own start is the
// fallback -- and recovers its primitives as calc_prim does.  use_guess 0 starts every cell from the previous primitives (the
// reference's calc_prim) and may record training pairs.  256 threads per
// block.
template <typename Phys, typename R, int NQ>
__global__ void __launch_bounds__(256) k_c2p_guess(DevParams P, DevState<R> S, MlpDev m, int use_guess,
                                                   C2PRecord rec) {
  __shared__ MlpSmem w;
  __shared__ __align__(16) bf16 Xs[8][32 * kLdX];
  __shared__ float Ys[8][32 * kMlpOut];
  mlp_load_smem(m, w);
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int N = S.N;
  bool valid = false;
  int jk = 0, j = 0, k = 0;
  if (c < N) {
    jk = S.cell_ring[c];
    k = div_fast(jk, P.mul_nr);
    j = jk - k * P.Nr;
    valid = is_real(P, j, k);
  }
  double dV = 1.0, x[3] = {1.0, 0.0, 0.0}, cons[NQ], prim[NQ], lu2 = 0.0, lth = 0.0;
  float f[kMlpIn];
  typename Phys::C2PInv v;
  if (valid) {
    c2p_geometry(P, S, c, jk, j, k, &dV, x);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      cons[q] = S.cons[q * N + c] / dV;
      prim[q] = S.prim[q * N + c];
    }
    KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
    Phys::c2p_invariants(P, cons, g, x[0], v);
    Phys::c2p_warm_logs(g, prim, x[0], &lu2, &lth);
    Phys::c2p_features(v, g, lu2, lth, f);
  }
  if (use_guess) {
    mlp_put_row(m, &Xs[wid][lane * kLdX], f, valid);
    mlp_infer_warp(m, w, Xs[wid], Ys[wid]);   // every lane of the warp takes part
  }
  if (!valid) return;
  KsMetric g(x, P.gr_M, P.gr_a, P.gr_kerr);
  double v2w, etaw;   // the previous primitives' start
  Phys::c2p_warm_start(P, g, prim, x[0], &v2w, &etaw);
  double v20 = v2w, eta0 = etaw;
  int guessed = 0;
  if (use_guess) {
    double guess[2];
    Phys::c2p_guess_from(v, &Ys[wid][lane * kMlpOut], lu2, lth, guess);
    const double rw = Phys::c2p_residual(v, v20, eta0);
    if (rw > m.warm_floor && Phys::c2p_residual(v, guess[0], guess[1]) < m.warm_ratio * rw) {
      v20 = guess[0];
      eta0 = guess[1];
      guessed = 1;
    }
  }
  double v2, eta;
  int kc, it;
  int hits = Phys::noble2d_solve(v, v20, eta0, &v2, &eta, &kc, &it);
  if (guessed && (kc == 0 || (hits & 4))) {
    // Newton from the learned start did not converge: solve again from the
    // previous primitives, as the reference does.  The wasted iterations
    // count toward this call's k_converge and iterations, and the call
    // counts as not guessed.
    int kc2, it2;
    hits = Phys::noble2d_solve(v, v2w, etaw, &v2, &eta, &kc2, &it2);
    kc = kc2 ? it + kc2 : 0;
    it += it2;
    guessed = 0;
  }
  if (rec.X && !(hits & 4) && (c % rec.stride) == 0) {   // a training pair from this solve
    float y[kMlpOut];
    Phys::c2p_targets(v, v2, eta, lu2, lth, y);
    bool ok = isfinite(y[0]) && isfinite(y[1]);
#pragma unroll
    for (int q = 0; q < kMlpIn; ++q) ok = ok && isfinite(f[q]);
    if (ok) {
      const unsigned long long at = atomicAdd(rec.count, 1ull);
      if ((long)at < rec.cap) {
#pragma unroll
        for (int q = 0; q < kMlpIn; ++q) rec.X[at * kMlpIn + q] = f[q];
        rec.Y[at * kMlpOut + 0] = y[0];
        rec.Y[at * kMlpOut + 1] = y[1];
      }
    }
  }
  hits |= Phys::c2p_recover(P, g, v, cons, v2, eta, prim);
  c2p_count(S.errs, kc, it, guessed);
  bool bad = false;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    S.prim[q * N + c] = prim[q];
    if (!isfinite(prim[q])) bad = true;
  }
  if (bad) atomicAdd(&S.errs->nan_cells, 1ull);
  if (hits & 1) atomicAdd(&S.errs->rho_floor_hits, 1ull);
  if (hits & 2) atomicAdd(&S.errs->p_floor_hits, 1ull);
  if (hits & 4) atomicAdd(&S.errs->c2p_no_converge, 1ull);
}

}  // namespace disco
