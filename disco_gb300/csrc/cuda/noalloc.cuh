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
  double dtc = c < S.N ? cell_mindt<Phys, R, NQ>(P, S, c) : 1.0e300;
  __shared__ unsigned long long red[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long b = __double_as_longlong(dtc);
  for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
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
  // seeded with +inf as k_dt_finalize's accumulator is, so partials that are
  // all NaN give the maxDT-capped dt there and here alike
  unsigned long long b = 0x7ff0000000000000ull;
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
