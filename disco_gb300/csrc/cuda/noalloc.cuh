// CFL reduction into a statically sized __device__ scratch array: the
// kernels behind disco_gpu_getmindt_noalloc (include/disco_gpu_noalloc.h).
//
// The array has internal linkage, so every translation unit that includes
// this header (one per hydro module and precision) owns its own copy; the
// kernels that use it live in the same unit.
#pragma once
#include <cuda_runtime.h>

#include <mutex>

#include "disco_gpu_noalloc.h"
#include "kernels.cuh"

namespace disco {

constexpr int kNoallocBlock = 256;
constexpr long kNoallocMaxBlocks = DISCO_NOALLOC_MAX_CELLS / kNoallocBlock;

// [0, kNoallocMaxBlocks): per-block minima (IEEE bits of dt); [kNoallocMaxBlocks]: dt.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoallocMaxBlocks + 32];

// Device address of the scratch array, looked up once per device.
static unsigned long long* noalloc_scratch(int dev) {
  static std::mutex mu;
  static unsigned long long* addr[64] = {};
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
    addr[dev] = (unsigned long long*)p;
  }
  return addr[dev];
}

// Per-block minimum of the cells' mindt (misc.c:39-84), the same per-cell
// bound and the same in-block reduction as k_mindt, written to the block's
// own slot instead of an atomic on the instance's accumulator.
template <typename Phys, typename R, int NQ>
__global__ void k_mindt_blocks(DevParams P, DevState<R> S, unsigned long long* part) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  double dtc = 1.0e300;
  float dtf = 3.0e38f;
  if (c < S.N) {
    int jk = S.cell_ring[c];
    int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
    if (is_real(P, j, k)) {
      int off = S.ring_off[jk], Np = S.ring_off[jk + 1] - off;
      int i = c - off;
      int im = off + (i == 0 ? Np - 1 : i - 1);
      R pr[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) pr[q] = S.prim[q * S.N + c];
      if constexpr (kMix<R>) {
        R w = (R)(.5 * (S.wiph[im] + S.wiph[c]) - S.ring_Om[jk]);
        R dph = S.dphi_r[c];
        dtf = Phys::mindt_r(P, S.planets, pr, w, S.ring_r1_r[jk] * dph, S.ring_dl_r[1][jk],
                            S.ring_dl_r[0][jk], S.ring_rc_r[jk], (R)S.piph[c] - (R).5 * dph);
      } else {
        const double* rj = S.r_jph + 1;
        const double* zk = S.z_kph + 1;
        double phip = S.piph[c], phim = phip - S.dphi[c];
        double xp[3] = {rj[j], phip, zk[k]};
        double xm[3] = {rj[j - 1], phim, zk[k - 1]};
        double w = .5 * (S.wiph[im] + S.wiph[c]);
        if constexpr (Phys::GR) dtc = Phys::mindt_x(P, pr, w, xp, xm);
        else dtc = Phys::mindt(P, S.planets, pr, w, xp, xm, S.ring_rc[jk]);
      }
    }
  }
  __shared__ unsigned long long red[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long b;
  if constexpr (kMix<R>) {
    unsigned u = __float_as_uint(dtf);
    for (int o = 16; o > 0; o >>= 1) u = min(u, __shfl_xor_sync(0xffffffffu, u, o));
    b = __double_as_longlong(u >= 0x7f000000u ? 1.0e300 : (double)__uint_as_float(u));
  } else {
    b = __double_as_longlong(dtc);
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  (void)dtc; (void)dtf;
  if (lane == 0) red[wid] = b;
  __syncthreads();
  if (wid == 0) {
    b = lane < (int)(blockDim.x >> 5) ? red[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
    if (lane == 0) part[blockIdx.x] = b;
  }
}

// One block: minimum over the nb partials, then dt = CFL * min(maxDT / CFL, m)
// as k_dt_finalize does with no end-time clamp; dt goes to part[kNoallocMaxBlocks].
static __global__ void k_mindt_final(DevParams P, unsigned long long* part, int nb) {
  __shared__ unsigned long long red[32];
  unsigned long long b = ~0ull;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) b = min(b, part[i]);
  for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = b;
  __syncthreads();
  if (wid == 0) {
    b = lane < (int)(blockDim.x >> 5) ? red[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
    if (lane == 0) {
      double m = __longlong_as_double((long long)b);
      double dt0 = P.maxDT / P.CFL;
      if (dt0 <= 0.0) dt0 = 1.0e100;
      double dt = dt0 < m ? dt0 : m;
      dt *= P.CFL;
      part[kNoallocMaxBlocks] = (unsigned long long)__double_as_longlong(dt);
    }
  }
}

}  // namespace disco
