// Training of the cons2prim MLP (mlp.cuh) on the tensor cores: one step is
// k_mlp_fwdbwd (forward, loss and backpropagated deltas of 16-sample tiles,
// one warp per tile), k_mlp_wgrad (the weight gradients as BF16 GEMMs over
// the batch), k_mlp_adam (FP32 masters) and k_mlp_bf16 (the BF16 copies).
// Included by one translation unit only.
#pragma once
#include "mlp.cuh"

namespace disco {

// splitmix64 (Steele, Lea, Flood 2014): the batch's sample indices
__device__ inline unsigned long long mlp_mix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// BF16 copies of the FP32 masters: W1b[64][16], W2b[64][64], W3b[16][64]
// (rows 8..15 zero).
static __global__ void k_mlp_bf16(const float* p, bf16* W1b, bf16* W2b, bf16* W3b) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kMlpH * kMlpH; e += gridDim.x * blockDim.x) {
    W2b[e] = __float2bfloat16_rn(p[kOffW2 + e]);
    if (e < kMlpH * kMlpInPad) W1b[e] = __float2bfloat16_rn(p[kOffW1 + e]);
    if (e < 16 * kMlpH) W3b[e] = __float2bfloat16_rn(e < kMlpOutPad * kMlpH ? p[kOffW3 + e] : 0.f);
  }
}

// Per-sample tile buffers of one batch (BF16, rows = samples): X [B][16],
// dY [B][16] (columns 0, 1 used), H1, H2, dZ1, dZ2 [B][64].
struct MlpBatch {
  bf16 *X, *dY, *H1, *H2, *Z1, *Z2;
};

// One warp per 16-sample tile: forward, loss, dY = 2 (y - t) / B, and the
// deltas dZ2 = (dY W3) (1 - h2^2), dZ1 = (dZ2 W2) (1 - h1^2).  Samples come
// from the data set (X raw features [n][8], Y raw targets [n][2]): sample s
// of the batch is data row mix(seed + s) mod n, or row s when seed is ~0.
static __global__ void __launch_bounds__(128) k_mlp_fwdbwd(MlpDev m, const float* Xd, const float* Yd, long n,
                                                           int B, unsigned long long seed, MlpBatch bt,
                                                           float* loss) {
  __shared__ MlpSmem w;
  __shared__ __align__(16) bf16 Xs[4][16 * kLdX];
  mlp_load_smem(m, w);
  __syncthreads();
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int i8 = lane >> 3, r8 = lane & 7;
  const int tile = blockIdx.x * 4 + wid;
  if (tile * 16 >= B) return;   // whole warps leave together
  const int s0 = tile * 16;
  long row[2] = {0, 0};   // the data rows of this lane's two tile rows (read only below B)
  for (int h = 0; h < 2; ++h) {
    const int s = s0 + g + 8 * h;
    row[h] = seed == ~0ull ? (long)s : (long)(mlp_mix(seed + (unsigned long long)s) % (unsigned long long)n);
  }
  if (lane < 16) {
    const int s = s0 + lane;
    const long r = seed == ~0ull ? (long)s : (long)(mlp_mix(seed + (unsigned long long)s) % (unsigned long long)n);
    float f[kMlpIn];
    if (s < B)   // a partial last tile's padding rows read nothing
#pragma unroll
      for (int q = 0; q < kMlpIn; ++q) f[q] = Xd[r * kMlpIn + q];
    mlp_put_row(m, &Xs[wid][lane * kLdX], f, s < B);
    // the BF16 row for the first layer's weight gradient
#pragma unroll
    for (int q = 0; q < kMlpInPad; ++q) bt.X[(size_t)s * kMlpInPad + q] = Xs[wid][lane * kLdX + q];
  }
  __syncwarp();
  float h1[8][4], h2[8][4], y[4];
  mlp_fwd_tile(w, Xs[wid], h1, h2, y);
  // loss and dY: columns 0, 1 live in the t == 0 lanes
  float dy[4] = {0.f, 0.f, 0.f, 0.f};
  float l = 0.f;
  if (t == 0) {
    const float invB = 1.0f / (float)B;
    for (int h = 0; h < 2; ++h) {
      if (s0 + g + 8 * h >= B) continue;   // a partial last tile's padding rows
      for (int o = 0; o < kMlpOut; ++o) {
        const float tn = (Yd[row[h] * kMlpOut + o] - m.ym[o]) / m.ys[o];
        const float d = y[2 * h + o] - tn;
        l += d * d;
        dy[2 * h + o] = 2.f * d * invB;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if (lane == 0) atomicAdd(loss, l);
  {   // dY as BF16 rows for dW3 / db3: columns 2 t, 2 t + 1 of rows g, g + 8
    const unsigned u0 = pack_bf16(dy[0], dy[1]), u1 = pack_bf16(dy[2], dy[3]);
    *reinterpret_cast<unsigned*>(&bt.dY[(size_t)(s0 + g) * 16 + 2 * t]) = u0;
    *reinterpret_cast<unsigned*>(&bt.dY[(size_t)(s0 + g + 8) * 16 + 2 * t]) = u1;
    *reinterpret_cast<unsigned*>(&bt.dY[(size_t)(s0 + g) * 16 + 8 + 2 * t]) = 0u;
    *reinterpret_cast<unsigned*>(&bt.dY[(size_t)(s0 + g + 8) * 16 + 8 + 2 * t]) = 0u;
  }
  // dH2 = dY W3: A = dY (K = 16 outputs), B(k = out, n = in) = W3[out][in]
  const unsigned ay[4] = {pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], dy[3]), 0u, 0u};
  float d2[8][4];
#pragma unroll
  for (int jp = 0; jp < 4; ++jp) {
    unsigned b[4];
    ldsm_x4_t(b, w.W3 + ((i8 & 1) * 8 + r8) * kLd2 + 16 * jp + (i8 >> 1) * 8);
#pragma unroll
    for (int e = 0; e < 4; ++e) { d2[2 * jp][e] = 0.f; d2[2 * jp + 1][e] = 0.f; }
    mma_bf16(d2[2 * jp], ay, b[0], b[1]);
    mma_bf16(d2[2 * jp + 1], ay, b[2], b[3]);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) d2[j][e] *= 1.f - h2[j][e] * h2[j][e];
  // dH1 = dZ2 W2: A = dZ2 (K = 64 from registers), B(k = out, n = in) = W2[out][in]
  float d1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) d1[j][e] = 0.f;
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    const unsigned ak[4] = {pack_bf16(d2[2 * kt][0], d2[2 * kt][1]), pack_bf16(d2[2 * kt][2], d2[2 * kt][3]),
                            pack_bf16(d2[2 * kt + 1][0], d2[2 * kt + 1][1]),
                            pack_bf16(d2[2 * kt + 1][2], d2[2 * kt + 1][3])};
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
      unsigned b[4];
      ldsm_x4_t(b, w.W2 + (16 * kt + (i8 & 1) * 8 + r8) * kLd2 + 16 * jp + (i8 >> 1) * 8);
      mma_bf16(d1[2 * jp], ak, b[0], b[1]);
      mma_bf16(d1[2 * jp + 1], ak, b[2], b[3]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) d1[j][e] *= 1.f - h1[j][e] * h1[j][e];
  // the activations and deltas as BF16 rows for the weight gradients
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const size_t o0 = (size_t)(s0 + g) * kMlpH + 8 * j + 2 * t, o1 = o0 + 8 * kMlpH;
    *reinterpret_cast<unsigned*>(&bt.H1[o0]) = pack_bf16(h1[j][0], h1[j][1]);
    *reinterpret_cast<unsigned*>(&bt.H1[o1]) = pack_bf16(h1[j][2], h1[j][3]);
    *reinterpret_cast<unsigned*>(&bt.H2[o0]) = pack_bf16(h2[j][0], h2[j][1]);
    *reinterpret_cast<unsigned*>(&bt.H2[o1]) = pack_bf16(h2[j][2], h2[j][3]);
    *reinterpret_cast<unsigned*>(&bt.Z1[o0]) = pack_bf16(d1[j][0], d1[j][1]);
    *reinterpret_cast<unsigned*>(&bt.Z1[o1]) = pack_bf16(d1[j][2], d1[j][3]);
    *reinterpret_cast<unsigned*>(&bt.Z2[o0]) = pack_bf16(d2[j][0], d2[j][1]);
    *reinterpret_cast<unsigned*>(&bt.Z2[o1]) = pack_bf16(d2[j][2], d2[j][3]);
  }
}

// Weight gradients over the batch, FP32 accumulation of BF16 products:
// dW2 = dZ2^T H1, dW1 = dZ1^T X, dW3 = dY^T H2, and the bias gradients as
// column sums of dZ1, dZ2, dY.  Each block takes kWgSamples samples in
// stages of 64 staged in shared memory; warps 0-3: dW2 rows 16 w..16 w+15,
// warps 4-7: dW1 rows, warp 8: dW3, warp 9: the biases; the block's sums are
// added to grad (flat, the parameter layout) atomically.
constexpr int kWgSamples = 256;
constexpr int kWgStage = 64;

static __global__ void __launch_bounds__(320) k_mlp_wgrad(MlpBatch bt, int B, float* grad) {
  __shared__ __align__(16) bf16 Z2s[kWgStage * kLd2];
  __shared__ __align__(16) bf16 H1s[kWgStage * kLd2];
  __shared__ __align__(16) bf16 Z1s[kWgStage * kLd2];
  __shared__ __align__(16) bf16 H2s[kWgStage * kLd2];
  __shared__ __align__(16) bf16 Xs[kWgStage * kLdX];
  __shared__ __align__(16) bf16 Ys[kWgStage * kLdX];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int i8 = lane >> 3, r8 = lane & 7;
  float acc[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
  float bs[5] = {0.f, 0.f, 0.f, 0.f, 0.f};   // warp 9: db1 (2 columns), db2 (2), db3 (lane 0, 1)
  const int sb = blockIdx.x * kWgSamples;
  for (int st0 = sb; st0 < sb + kWgSamples && st0 < B; st0 += kWgStage) {
    const int ns = min(kWgStage, B - st0);
    __syncthreads();
    // stage 64 samples (16-byte loads; rows past the batch are zero)
    for (int e = threadIdx.x; e < kWgStage * 8; e += blockDim.x) {
      const int rr = e >> 3, cc = (e & 7) * 8;
      uint4 z = {0u, 0u, 0u, 0u}, a = z, b = z, c = z, d = z;
      if (rr < ns) {
        const size_t o = (size_t)(st0 + rr) * kMlpH + cc;
        a = *reinterpret_cast<const uint4*>(&bt.Z2[o]);
        b = *reinterpret_cast<const uint4*>(&bt.H1[o]);
        c = *reinterpret_cast<const uint4*>(&bt.Z1[o]);
        d = *reinterpret_cast<const uint4*>(&bt.H2[o]);
      }
      *reinterpret_cast<uint4*>(&Z2s[rr * kLd2 + cc]) = a;
      *reinterpret_cast<uint4*>(&H1s[rr * kLd2 + cc]) = b;
      *reinterpret_cast<uint4*>(&Z1s[rr * kLd2 + cc]) = c;
      *reinterpret_cast<uint4*>(&H2s[rr * kLd2 + cc]) = d;
    }
    for (int e = threadIdx.x; e < kWgStage * 2; e += blockDim.x) {
      const int rr = e >> 1, cc = (e & 1) * 8;
      uint4 z = {0u, 0u, 0u, 0u}, a = z, b = z;
      if (rr < ns) {
        const size_t o = (size_t)(st0 + rr) * 16 + cc;
        a = *reinterpret_cast<const uint4*>(&bt.X[o]);
        b = *reinterpret_cast<const uint4*>(&bt.dY[o]);
      }
      *reinterpret_cast<uint4*>(&Xs[rr * kLdX + cc]) = a;
      *reinterpret_cast<uint4*>(&Ys[rr * kLdX + cc]) = b;
    }
    __syncthreads();
    if (wid < 9) {
      // A = (deltas)^T: A(m = out, k = sample) from rows [sample][out]
      const bf16* As = wid < 4 ? Z2s : (wid < 8 ? Z1s : Ys);
      const int lda = wid < 8 ? kLd2 : kLdX;
      const int m0 = wid < 4 ? 16 * wid : (wid < 8 ? 16 * (wid - 4) : 0);
      // B(k = sample, n = in) from rows [sample][in]
      const bf16* Bs = wid < 4 ? H1s : (wid < 8 ? Xs : H2s);
      const int ldb = wid < 4 ? kLd2 : (wid < 8 ? kLdX : kLd2);
      const int npair = wid >= 4 && wid < 8 ? 1 : 4;
#pragma unroll
      for (int kt = 0; kt < kWgStage / 16; ++kt) {
        unsigned a[4];
        ldsm_x4_t(a, As + (16 * kt + (i8 >> 1) * 8 + r8) * lda + m0 + (i8 & 1) * 8);
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
          if (jp >= npair) break;
          unsigned b[4];
          ldsm_x4_t(b, Bs + (16 * kt + (i8 & 1) * 8 + r8) * ldb + 16 * jp + (i8 >> 1) * 8);
          mma_bf16(acc[2 * jp], a, b[0], b[1]);
          mma_bf16(acc[2 * jp + 1], a, b[2], b[3]);
        }
      }
    } else {   // bias gradients: column sums over the staged samples
      for (int rr = 0; rr < ns; ++rr) {
        bs[0] += __bfloat162float(Z1s[rr * kLd2 + 2 * lane]);
        bs[1] += __bfloat162float(Z1s[rr * kLd2 + 2 * lane + 1]);
        bs[2] += __bfloat162float(Z2s[rr * kLd2 + 2 * lane]);
        bs[3] += __bfloat162float(Z2s[rr * kLd2 + 2 * lane + 1]);
        if (lane < kMlpOut) bs[4] += __bfloat162float(Ys[rr * kLdX + lane]);
      }
    }
  }
  // the block's sums into grad
  if (wid < 4) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int o = 16 * wid + g, i = 8 * j + 2 * t;
      atomicAdd(&grad[kOffW2 + o * kMlpH + i], acc[j][0]);
      atomicAdd(&grad[kOffW2 + o * kMlpH + i + 1], acc[j][1]);
      atomicAdd(&grad[kOffW2 + (o + 8) * kMlpH + i], acc[j][2]);
      atomicAdd(&grad[kOffW2 + (o + 8) * kMlpH + i + 1], acc[j][3]);
    }
  } else if (wid < 8) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int o = 16 * (wid - 4) + g, i = 8 * j + 2 * t;
      atomicAdd(&grad[kOffW1 + o * kMlpInPad + i], acc[j][0]);
      atomicAdd(&grad[kOffW1 + o * kMlpInPad + i + 1], acc[j][1]);
      atomicAdd(&grad[kOffW1 + (o + 8) * kMlpInPad + i], acc[j][2]);
      atomicAdd(&grad[kOffW1 + (o + 8) * kMlpInPad + i + 1], acc[j][3]);
    }
  } else if (wid == 8) {
    if (g < kMlpOutPad) {   // rows 0..7 of the 16-row tile: W3's rows
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int i = 8 * j + 2 * t;
        atomicAdd(&grad[kOffW3 + g * kMlpH + i], acc[j][0]);
        atomicAdd(&grad[kOffW3 + g * kMlpH + i + 1], acc[j][1]);
      }
    }
  } else {
    atomicAdd(&grad[kOffB1 + 2 * lane], bs[0]);
    atomicAdd(&grad[kOffB1 + 2 * lane + 1], bs[1]);
    atomicAdd(&grad[kOffB2 + 2 * lane], bs[2]);
    atomicAdd(&grad[kOffB2 + 2 * lane + 1], bs[3]);
    if (lane < kMlpOut) atomicAdd(&grad[kOffB3 + lane], bs[4]);
  }
}

// Adam (Kingma & Ba 2015) on the FP32 masters; bc1, bc2 = 1 - beta^step.
static __global__ void k_mlp_adam(float* p, float* m1, float* m2, const float* grad, float lr, float b1, float b2,
                                  float eps, float bc1, float bc2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kMlpParams) return;
  const float gr = grad[e];
  const float a = b1 * m1[e] + (1.f - b1) * gr;
  const float v = b2 * m2[e] + (1.f - b2) * gr * gr;
  m1[e] = a;
  m2[e] = v;
  p[e] -= lr * (a / bc1) / (sqrtf(v / bc2) + eps);
}

// Inference on given raw feature rows (the same warp routine calc_prim uses).
static __global__ void __launch_bounds__(128) k_mlp_predict(MlpDev m, const float* X, long n, float* Y) {
  __shared__ MlpSmem w;
  __shared__ __align__(16) bf16 Xs[4][32 * kLdX];
  __shared__ float Ys[4][32 * kMlpOut];
  mlp_load_smem(m, w);
  __syncthreads();
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  float f[kMlpIn];
  const bool valid = s < n;
  if (valid)
#pragma unroll
    for (int q = 0; q < kMlpIn; ++q) f[q] = X[s * kMlpIn + q];
  mlp_put_row(m, &Xs[wid][lane * kLdX], f, valid);
  mlp_infer_warp(m, w, Xs[wid], Ys[wid]);
  if (valid) {
    Y[s * kMlpOut + 0] = Ys[wid][lane * kMlpOut + 0];
    Y[s * kMlpOut + 1] = Ys[wid][lane * kMlpOut + 1];
  }
}

}  // namespace disco
