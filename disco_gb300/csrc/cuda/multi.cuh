// Many instances of one hydro module and precision advanced by one launch
// per stage: the batching form of the step.  Each stage kernel is
// persistent -- a grid of a few CTAs per SM -- and its blocks walk a work
// list of (instance, tile) items, the tiles being the blocks each instance
// would have launched on its own (cells, ring chunks, ring pairs, rings).
// A block takes a contiguous range of the list, so it stays on one instance
// for many tiles; whenever the instance changes, the block copies that
// instance's parameters and array pointers into shared memory, and the
// kernel bodies read them from there.  Bodies that use shared memory of
// their own end each tile with a block barrier (SYNC); the others run
// their tiles back to back, with a barrier only around a change of
// instance.
//
// The bodies are the single-instance kernels' own (k_*_body), so a member
// advanced in a batch computes exactly what it computes alone.
#pragma once
#include "kernels.cuh"
#include "diag.cuh"

namespace disco {

// One member of a batch: its parameters and arrays (with the piph buffers
// of one parity), and the range of ring pairs its r / z flux sweeps cover
// (jmin, jcount, kmin per dimension; jcount 0: no sweep).
template <typename R>
struct MultiMember {
  DevParams P;
  DevState<R> S;
  int fr[2][3];
  int planets_id;
  double* qrz;   // the ring-diagnostics accumulators (null: no ANALYSIS)
};

// A work item: member, block index x, block index y.
struct MultiTile {
  int m, x, y, pad;
};

#ifdef __CUDACC__
// Walks this block's contiguous share of the work list, calling
// body(member, bx, by) with the member staged in shared memory.  Every
// thread sees the same tiles, so `cur` (a register) and the branches on it
// are block-uniform.
template <typename R, bool SYNC, typename F>
DISCO_D void multi_walk(const MultiMember<R>* tab, const MultiTile* tiles, int ntiles, F&& body) {
  __shared__ MultiMember<R> sm;
  const int per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
  int cur = -1;
  for (int t = t0; t < t1; ++t) {
    const MultiTile w = tiles[t];
    if (w.m != cur) {   // stage the member's parameters
      if (!SYNC && cur >= 0) __syncthreads();   // every thread is done with the previous member
      const int* src = reinterpret_cast<const int*>(&tab[w.m]);
      int* dst = reinterpret_cast<int*>(&sm);
      for (int i = threadIdx.x; i < (int)(sizeof(MultiMember<R>) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      cur = w.m;
    }
    body(sm, w.x, w.y);
    if constexpr (SYNC) __syncthreads();
  }
}

#define DISCO_MULTI_KERNEL(NAME, LB, TPL, SYNC, BODYCALL)                                             \
  TPL __global__ void LB NAME(const MultiMember<R>* tab, const MultiTile* tiles, int ntiles,             \
                              double a0, double a1, int i0, int i1) {                                    \
    (void)a0; (void)a1; (void)i0; (void)i1;                                                              \
    multi_walk<R, SYNC>(tab, tiles, ntiles, [&](const MultiMember<R>& M, int bx, int by) { BODYCALL; }); \
  }

#define DISCO_TPL_RN template <typename R, int NQ>
#define DISCO_TPL_R template <typename R>
#define DISCO_TPL_PRN template <typename Phys, typename R, int NQ>
// SYNC: the bodies with shared memory of their own (mindt, wcell_ring,
// wcell_avg, faces, plm_trans; diag below)
DISCO_MULTI_KERNEL(km_mindt, __launch_bounds__(256), DISCO_TPL_PRN, true, (k_mindt_body<Phys, R, NQ>(M.P, M.S, bx, by)))
DISCO_MULTI_KERNEL(km_wcell, , DISCO_TPL_RN, false, (k_wcell_body<R, NQ>(M.P, M.S, bx, by)))
DISCO_MULTI_KERNEL(km_wcell_ring, , DISCO_TPL_R, true, (k_wcell_ring_body<R>(M.P, M.S, bx, by)))
DISCO_MULTI_KERNEL(km_wcell_avg, , DISCO_TPL_R, true, (k_wcell_avg_body<R>(M.P, M.S, bx, by)))
DISCO_MULTI_KERNEL(km_plm_phi, , DISCO_TPL_RN, false, (k_plm_phi_body<R, NQ>(M.P, M.S, bx, by)))
DISCO_MULTI_KERNEL(km_anchor, , DISCO_TPL_R, false, (k_anchor_body<R>(M.P, M.S, (int)(M.P.Nr * M.P.Nz), bx, by)))
DISCO_MULTI_KERNEL(km_faces, , DISCO_TPL_R, true, (k_faces_body<R>(M.P, M.S, i0, bx, by)))
DISCO_MULTI_KERNEL(km_plm_slopes, , DISCO_TPL_RN, false, (k_plm_slopes_body<R, NQ>(M.P, M.S, i0, bx, by)))
DISCO_MULTI_KERNEL(km_plm_trans, __launch_bounds__(kTileCells), DISCO_TPL_RN, true,
                   (k_plm_trans_body<R, NQ>(M.P, M.S, i0, bx, by)))
DISCO_MULTI_KERNEL(km_flux_phi, __launch_bounds__(256, kMix<R> ? 4 : 1), DISCO_TPL_PRN, false,
                   (k_flux_phi_body<Phys, R, NQ>(M.P, M.S, a0, bx, by)))
DISCO_MULTI_KERNEL(km_flux_trans, __launch_bounds__(256, kMix<R> ? 4 : 1), DISCO_TPL_PRN, false,
                   (k_flux_trans_body<Phys, R, NQ>(M.P, M.S, i0, M.fr[i0 - 1][0], M.fr[i0 - 1][1],
                                                   M.fr[i0 - 1][2], a0, bx, by)))
DISCO_MULTI_KERNEL(km_boundary, __launch_bounds__(kTileCells), DISCO_TPL_RN, false,
                   (k_boundary_body<R, NQ>(M.P, M.S, bx, by)))
#undef DISCO_TPL_RN
#undef DISCO_TPL_R
#undef DISCO_TPL_PRN

// k_update of every member (the same template variant for all)
template <typename Phys, typename R, int NQ, bool CD, bool MID>
__global__ void __launch_bounds__(256, kMix<R> ? 4 : 1) km_update(const MultiMember<R>* tab, const MultiTile* tiles,
                                                                  int ntiles, double RK, double fac, int first,
                                                                  int do_c2p) {
  multi_walk<R, false>(tab, tiles, ntiles, [&](const MultiMember<R>& M, int bx, int by) {
    k_update_body<Phys, R, NQ, CD, MID>(M.P, M.S, RK, fac, first, do_c2p, bx, by);
  });
}

// ring diagnostics of every member, into its own accumulators
template <typename R, int NQ, int D>
__global__ void __launch_bounds__(kDiagBlock) km_diag(const MultiMember<R>* tab, const MultiTile* tiles, int ntiles) {
  multi_walk<R, true>(tab, tiles, ntiles, [&](const MultiMember<R>& M, int bx, int by) {
    (void)by;
    k_diag_body<R, NQ, D>(M.P, M.S, M.qrz, bx, 0);
  });
}

// dt of every member (one thread each): dt_finalize of k_dt_finalize
template <typename R>
__global__ void km_dt_finalize(const MultiMember<R>* tab, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n) dt_finalize_one(tab[m].P, tab[m].S.scal);
}

// time and analytic orbits of every member after its first substep
template <typename R>
__global__ void km_after_first(const MultiMember<R>* tab, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n) after_first_one(tab[m].P, tab[m].S.scal, tab[m].S.planets, tab[m].planets_id, tab[m].S.errs);
}
#endif

}  // namespace disco
