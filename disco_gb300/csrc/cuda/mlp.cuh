// The learned starting point of the GRMHD Newton cons2prim: a 2 x 64 MLP
// (10 features: 8 of the conserved state and the metric, 2 of the previous
// primitives -> the changes of log(W^2 - 1) and log(P / rho) from the
// previous primitives' values), trained and evaluated on the tensor cores.
//
// Arithmetic: BF16 operands (inputs, weights, activations, backpropagated
// deltas) in mma.sync.m16n8k16 with FP32 accumulation; biases, tanh, the
// loss and the Adam update in FP32 (FP32 master weights).  Operands reach
// the tensor cores through ldmatrix from shared memory, or -- between the
// layers of one 16-row tile -- straight from the previous layer's
// accumulator registers (the m16n8 accumulator layout of two adjacent
// column tiles is the m16k16 A-operand layout).
//
// Layout: weights [out][in] row-major (FP32 masters in one flat vector,
// BF16 copies beside them); a sample is a row, features in columns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace disco {

constexpr int kMlpIn = 10;         // features
constexpr int kMlpInPad = 16;      // K of the first layer
constexpr int kMlpH = 64;          // hidden width
constexpr int kMlpOut = 2;         // outputs
constexpr int kMlpOutPad = 8;      // N of the last layer
// flat FP32 parameter vector: W1[64][16] b1[64] W2[64][64] b2[64] W3[8][64] b3[8]
constexpr int kOffW1 = 0, kOffB1 = 1024, kOffW2 = 1088, kOffB2 = 5184, kOffW3 = 5248, kOffB3 = 5760;
constexpr int kMlpParams = 5768;
// shared-memory row strides (elements): rows padded so that the eight rows
// an ldmatrix reads fall in different banks
constexpr int kLd1 = 24, kLd2 = 72, kLdX = 24;

typedef __nv_bfloat16 bf16;

// The model as kernels see it: BF16 weight copies W1b[64][16], W2b[64][64],
// W3b[16][64] (rows 2..15 zero), FP32 biases (in the master vector) and the
// standardisation of features and targets.
struct MlpDev {
  const bf16* W1b;
  const bf16* W2b;
  const bf16* W3b;
  const float* params;   // FP32 masters (biases read from here)
  float xm[kMlpIn], xs[kMlpIn], ym[kMlpOut], ys[kMlpOut];
  // cons2prim considers the learned start only where the previous
  // primitives leave a residual of the two Noble equations above
  // warm_floor, and takes it where its own residual is below warm_ratio
  // times theirs
  double warm_floor, warm_ratio;
};

struct __align__(16) MlpSmem {
  bf16 W1[kMlpH * kLd1];
  bf16 W2[kMlpH * kLd2];
  bf16 W3[16 * kLd2];
  float b1[kMlpH], b2[kMlpH], b3[kMlpOutPad];
};

#ifdef __CUDACC__
__device__ inline unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ inline void ldsm_x4(unsigned* r, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ inline void ldsm_x4_t(unsigned* r, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
// D = A (16 x 16, row) * B (16 x 8, col) + D, BF16 in, FP32 accumulate
__device__ inline void mma_bf16(float* c, const unsigned* a, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ inline unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}

// Weights and biases into shared memory (padded rows), by the whole block.
__device__ inline void mlp_load_smem(const MlpDev& m, MlpSmem& w) {
  for (int e = threadIdx.x; e < kMlpH * kMlpInPad; e += blockDim.x)
    w.W1[(e / kMlpInPad) * kLd1 + e % kMlpInPad] = m.W1b[e];
  for (int e = threadIdx.x; e < kMlpH * kMlpH; e += blockDim.x) w.W2[(e / kMlpH) * kLd2 + e % kMlpH] = m.W2b[e];
  for (int e = threadIdx.x; e < 16 * kMlpH; e += blockDim.x) w.W3[(e / kMlpH) * kLd2 + e % kMlpH] = m.W3b[e];
  for (int e = threadIdx.x; e < kMlpH; e += blockDim.x) {
    w.b1[e] = m.params[kOffB1 + e];
    w.b2[e] = m.params[kOffB2 + e];
  }
  for (int e = threadIdx.x; e < kMlpOutPad; e += blockDim.x) w.b3[e] = m.params[kOffB3 + e];
}

// One 16-row tile through the network by one warp.  X: 16 rows of
// kMlpInPad BF16 features (stride kLdX).  Out: h1, h2 (FP32 after tanh) and
// y (the first accumulator tile of the last layer) in accumulator layout:
// thread (g = lane / 4, t = lane % 4) holds, for column tile j, rows g and
// g + 8 at columns 8 j + 2 t and 8 j + 2 t + 1.
__device__ inline void mlp_fwd_tile(const MlpSmem& w, const bf16* X, float (*h1)[4], float (*h2)[4], float* y) {
  const int lane = threadIdx.x & 31, t = lane & 3, i8 = lane >> 3, r8 = lane & 7;
  unsigned a[4];
  ldsm_x4(a, X + (lane & 15) * kLdX + (lane >> 4) * 8);
#pragma unroll
  for (int jp = 0; jp < 4; ++jp) {   // layer 1: N = 64 in four pairs of 8-column tiles, K = 16
    unsigned b[4];
    ldsm_x4(b, w.W1 + (16 * jp + (i8 >> 1) * 8 + r8) * kLd1 + (i8 & 1) * 8);
#pragma unroll
    for (int e = 0; e < 4; ++e) { h1[2 * jp][e] = 0.f; h1[2 * jp + 1][e] = 0.f; }
    mma_bf16(h1[2 * jp], a, b[0], b[1]);
    mma_bf16(h1[2 * jp + 1], a, b[2], b[3]);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float c0 = w.b1[8 * j + 2 * t], c1 = w.b1[8 * j + 2 * t + 1];
    h1[j][0] = tanhf(h1[j][0] + c0); h1[j][1] = tanhf(h1[j][1] + c1);
    h1[j][2] = tanhf(h1[j][2] + c0); h1[j][3] = tanhf(h1[j][3] + c1);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) h2[j][e] = 0.f;
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {   // layer 2: K = 64 from h1's registers
    const unsigned ak[4] = {pack_bf16(h1[2 * kt][0], h1[2 * kt][1]), pack_bf16(h1[2 * kt][2], h1[2 * kt][3]),
                            pack_bf16(h1[2 * kt + 1][0], h1[2 * kt + 1][1]),
                            pack_bf16(h1[2 * kt + 1][2], h1[2 * kt + 1][3])};
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
      unsigned b[4];
      ldsm_x4(b, w.W2 + (16 * jp + (i8 >> 1) * 8 + r8) * kLd2 + 16 * kt + (i8 & 1) * 8);
      mma_bf16(h2[2 * jp], ak, b[0], b[1]);
      mma_bf16(h2[2 * jp + 1], ak, b[2], b[3]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float c0 = w.b2[8 * j + 2 * t], c1 = w.b2[8 * j + 2 * t + 1];
    h2[j][0] = tanhf(h2[j][0] + c0); h2[j][1] = tanhf(h2[j][1] + c1);
    h2[j][2] = tanhf(h2[j][2] + c0); h2[j][3] = tanhf(h2[j][3] + c1);
  }
  float y2[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int e = 0; e < 4; ++e) y[e] = 0.f;
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {   // layer 3: N = 8 (+ 8 zero rows of W3), K = 64
    const unsigned ak[4] = {pack_bf16(h2[2 * kt][0], h2[2 * kt][1]), pack_bf16(h2[2 * kt][2], h2[2 * kt][3]),
                            pack_bf16(h2[2 * kt + 1][0], h2[2 * kt + 1][1]),
                            pack_bf16(h2[2 * kt + 1][2], h2[2 * kt + 1][3])};
    unsigned b[4];
    ldsm_x4(b, w.W3 + ((i8 >> 1) * 8 + r8) * kLd2 + 16 * kt + (i8 & 1) * 8);
    mma_bf16(y, ak, b[0], b[1]);
    mma_bf16(y2, ak, b[2], b[3]);
  }
  y[0] += w.b3[2 * t]; y[1] += w.b3[2 * t + 1];
  y[2] += w.b3[2 * t]; y[3] += w.b3[2 * t + 1];
}

// Standardised features of one sample into a BF16 row (10 used of 16).
__device__ inline void mlp_put_row(const MlpDev& m, bf16* row, const float* f, bool valid) {
#pragma unroll
  for (int q = 0; q < kMlpInPad; ++q) {
    float v = 0.f;
    if (valid && q < kMlpIn) v = (f[q] - m.xm[q]) / m.xs[q];
    row[q] = __float2bfloat16_rn(v);
  }
}

// Inference for 32 consecutive samples of a warp: Xw [32][kLdX] BF16 rows
// (filled by mlp_put_row), Yw [32][2] the destandardised outputs.
__device__ inline void mlp_infer_warp(const MlpDev& m, const MlpSmem& w, const bf16* Xw, float* Yw) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  __syncwarp();
#pragma unroll 1
  for (int tile = 0; tile < 2; ++tile) {
    float h1[8][4], h2[8][4], y[4];
    mlp_fwd_tile(w, Xw + 16 * tile * kLdX, h1, h2, y);
    if (t == 0) {
      Yw[(16 * tile + g) * 2 + 0] = y[0] * m.ys[0] + m.ym[0];
      Yw[(16 * tile + g) * 2 + 1] = y[1] * m.ys[1] + m.ym[1];
      Yw[(16 * tile + g + 8) * 2 + 0] = y[2] * m.ys[0] + m.ym[0];
      Yw[(16 * tile + g + 8) * 2 + 1] = y[3] * m.ys[1] + m.ym[1];
    }
  }
  __syncwarp();
}
#endif

}  // namespace disco
