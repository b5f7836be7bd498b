// The azimuthal sweep of the mixed path in one pass: plm_phi (plm.c:6-51)
// and the phi-face fluxes (misc.c:378-436, riemann.c:39-112) of a chunk of
// kTileCells consecutive cells of one ring, from a single shared-memory
// stage of the ring's primitives and widths.
//
// Staging: the chunk's window -- ring cells i0-1 .. i0+T+1 (w = 0 .. T+2),
// the periodic phi stencil of plm_phi and of the face fluxes -- is brought
// in by the tensor memory accelerator, one 1-D bulk tensor copy per
// component row of prim (SoA: row q starts at element q N) and one of
// dphi, all completing on one mbarrier.  A copy must start on a 16-byte
// boundary, so each row starts at its first element rounded down to a
// multiple of four and the kernel indexes from the remainder.  Window cells
// that wrap around the ring's ends (i0 = 0 on the left, the ring's last
// chunk on the right) are patched with plain loads after the wait.
//
// Every wait is bounded in time (about a second of SM clock): on a timeout
// the block counts it in the health counters, waits (again bounded) for its
// copies in flight and returns.  A debug mode issues no copies, so that a
// test can make the wait run out and read the count.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include "kernels.cuh"
#include "mlp.cuh"

namespace disco {

constexpr int kSweepBox = 136;    // elements per staged row: 128 + 3 halo, + up to 3 of alignment, 16-byte multiple
constexpr int kSweepSlot = 160;   // floats per shared-memory row slot (640 B, a multiple of 128 B)
constexpr long long kSweepMaxCycles = 1LL << 31;   // about 1 s at 2 GHz

#ifdef __CUDACC__
__device__ inline void tma_load_1d(void* dst, const CUtensorMap* map, int x, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];\n" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(smem_u32(bar))
      : "memory");
}
__device__ inline void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ inline void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ inline void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ inline bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ inline bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kSweepMaxCycles) return false;
  return true;
}

template <typename Phys, typename R, int NQ>
__global__ void __launch_bounds__(kTileCells) k_phi_sweep(DevParams P, DevState<R> S, double fac,
                                                         const __grid_constant__ CUtensorMap tm_prim,
                                                         const __grid_constant__ CUtensorMap tm_dphi,
                                                         int no_copies) {
  static_assert(sizeof(R) == 4, "the staged sweep is the mixed path's");
  __shared__ __align__(128) float stage[(NQ + 1) * kSweepSlot];
  __shared__ float gsh[NQ][kTileCells + 2];   // gradp of window cells w = 1 .. T+1
  __shared__ __align__(8) unsigned long long bar;
  const int ch = blockIdx.x, t = threadIdx.x;
  const int jk = S.chunk_ring[ch], i0 = S.chunk_i0[ch];
  const int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
  const int T = min(kTileCells, Np - i0);
  const int N = S.N;
  const int c0 = off + i0;
  // row q of the window starts at element q N + c0 - 1; the copy at that
  // element rounded down to a multiple of 4, the window at the remainder
  auto row_start = [&](int q) { return (long long)q * N + c0 - 1; };
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (t == 0 && !no_copies) {
    mbar_expect_tx(&bar, (unsigned)((NQ + 1) * kSweepBox * sizeof(float)));
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const long long x = row_start(q);
      tma_load_1d(&stage[q * kSweepSlot], &tm_prim, (int)(x - (x & 3)), &bar);
    }
    const long long xd = (long long)c0 - 1;
    tma_load_1d(&stage[NQ * kSweepSlot], &tm_dphi, (int)(xd - (xd & 3)), &bar);
  }
  // every thread waits (bounded); the block leaves together if any ran out
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (__syncthreads_or(!ok)) {
    if (t == 0) atomicAdd(&S.errs->async_timeouts, 1ull);
    if (!ok) mbar_wait_bounded(&bar, 0);   // the copies in flight, once more, bounded
    return;
  }
  auto V = [&](int q, int w) -> float& { return stage[q * kSweepSlot + (int)(row_start(q) & 3) + w]; };
  auto D = [&](int w) -> float& { return stage[NQ * kSweepSlot + (int)(((long long)c0 - 1) & 3) + w]; };
  // window cells past the ring's ends come from the other end of the ring
  if (t < 3) {
    const int w = t == 0 ? 0 : T + t;
    const int iw = i0 - 1 + w;
    if (iw < 0 || iw >= Np) {
      const int g = off + (iw < 0 ? iw + Np : iw - Np);
#pragma unroll
      for (int q = 0; q < NQ; ++q) V(q, w) = S.prim[q * N + g];
      D(w) = S.dphi_r[g];
    }
  }
  __syncthreads();
  // plm_phi for w = t + 1 (and w = T + 1, the successor of the last cell)
  const R PLM = PRM(R, P, PLM);
  auto plm = [&](int w) {
    const R dpL = D(w - 1), dpC = D(w), dpR = D(w + 1);
    const R iL = (R)1 / ((R).5 * (dpC + dpL));
    const R iR = (R)1 / ((R).5 * (dpR + dpC));
    const R iC = (R)1 / ((R).5 * (dpL + dpR) + dpC);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const R pL = V(q, w - 1), pC = V(q, w), pR = V(q, w + 1);
      const R sL = (pC - pL) * iL, sR = (pR - pC) * iR, sC = (pR - pL) * iC;
      gsh[q][w - 1] = minmod<R>(PLM * sL, sC, PLM * sR);
    }
  };
  if (t < T) {
    plm(t + 1);
#pragma unroll
    for (int q = 0; q < NQ; ++q) S.gradp[q * N + c0 + t] = gsh[q][t];
  }
  if (t == 0) plm(T + 1);
  __syncthreads();
  // the phi face between cell i0 + t and its successor
  const int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
  if (t < T && (S.ct ? ring_in_phi_range(P, j, k) : is_real(P, j, k))) {
    const int i = i0 + t, c = c0 + t;
    const int cp = off + (i + 1 < Np ? i + 1 : 0);
    R pC[NQ], pP[NQ], gC[NQ], gP[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      pC[q] = V(q, t + 1); pP[q] = V(q, t + 2);
      gC[q] = gsh[q][t]; gP[q] = gsh[q][t + 1];
    }
    flux_phi_face<Phys, R, NQ>(P, S, fac, c, cp, jk, j, k, pC, pP, gC, gP, D(t + 1), D(t + 2));
  }
}
#endif

// A rank-1 tensor map over n FP32 elements at base (16-byte aligned), box
// kSweepBox, no swizzle, out-of-range elements read as zero: the copies of
// the staged sweep.  The driver's cuTensorMapEncodeTiled, reached through
// the runtime's entry-point lookup.  0 on success.
inline int make_sweep_tmap(CUtensorMap* map, const float* base, unsigned long long n) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return -1;
    fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  cuuint64_t dims[1] = {n};
  cuuint64_t strides[1] = {n * sizeof(float)};
  cuuint32_t box[1] = {(cuuint32_t)kSweepBox};
  cuuint32_t es[1] = {1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, (void*)base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

}  // namespace disco
