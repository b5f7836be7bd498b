// report.c (report.c:4-329) as a device reduction: the domain sums the
// reference prints at every report -- the gas mass, and with a second body
// the gravitational torques of the gas on both bodies, in total and outside
// five cut radii around the second body.
//
// The reference sums cell by cell in (j, k, i) order; here each block sums
// its cells in a fixed tree and a single block adds the block partials in
// block order, so the result is deterministic and equal to the serial sum
// to rounding.  The planets' sink/accretion accumulators the reference also
// prints are zero in this build (sinks are not built).
#pragma once
#include "kernels.cuh"

namespace disco {

// sums: Mass, Torque, Torque2, Torque1_cut[5], Torque2_cut[5]
constexpr int kReportSums = 13;
constexpr int kReportBlock = 256;

template <typename R, int NQ>
__global__ void __launch_bounds__(kReportBlock) k_report_blocks(DevParams P, DevState<R> S, double soft,
                                                                double* part) {
  double v[kReportSums];
#pragma unroll
  for (int s = 0; s < kReportSums; ++s) v[s] = 0.0;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < S.N) {
    const int jk = S.cell_ring[c];
    const int k = div_fast(jk, P.mul_nr), j = jk - k * P.Nr;
    if (is_real(P, j, k)) {   // report.c:110-206: j in [NgRa, Nr-NgRb), k in [NgZa, Nz-NgZb)
      const double* rj = S.r_jph + 1;
      const double* zk = S.z_kph + 1;
      const double phip = S.piph[c], dph = S.dphi[c];
      const double phi = phip - .5 * dph;
      const double phim = phip - dph;
      const double rho = (double)S.prim[RHO * S.N + c];
      // get_dV and get_centroid (cylindrical.c)
      const double rp = rj[j], rm = rj[j - 1];
      const double dV = (.5 * (rp + rm)) * (rp - rm) * get_dp(phip, phim, P.phi_max) * (zk[k] - zk[k - 1]);
      const double r = centroid_r(rp, rm);
      v[0] = rho * dV;
      if (P.Npl > 1) {
        double fr, fp, fp2, fz;
        planetary_force<double>(P, S.planets[0], r, phi, 0.0, &fr, &fp2, &fz, 1);
        planetary_force<double>(P, S.planets[1], r, phi, 0.0, &fr, &fp, &fz, 1);
        const double rS = S.planets[0].r, rp1 = S.planets[1].r, pp = S.planets[1].phi;
        const double dx = r * cos(phi) - rp1 * cos(pp);
        const double dy = r * sin(phi) - rp1 * sin(pp);
        const double script_r = sqrt(dx * dx + dy * dy);
        const double t1v = (rho - 1.0) * rp1 * fp * dV;
        const double t2v = (rho - 1.0) * rS * fp2 * dV;
        v[1] = -t1v;
        v[2] = -t2v;
#pragma unroll
        for (int n = 0; n < 5; ++n) {
          const double r_cut = (double)(n + 1.) * soft;
          if (script_r > r_cut) {
            v[3 + n] = -t1v;
            v[8 + n] = -t2v;
          }
        }
      }
    }
  }
  // block tree: warp shuffles, then the warps' partials
  __shared__ double red[kReportSums][kReportBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < kReportSums; ++s) {
    double x = v[s];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[s][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < kReportSums) {
    double x = 0.0;
    for (int w = 0; w < kReportBlock / 32; ++w) x += red[threadIdx.x][w];
    part[(size_t)blockIdx.x * kReportSums + threadIdx.x] = x;
  }
}

// One block: the block partials of each sum added in block order.
static __global__ void k_report_final(const double* part, int nb, double* out) {
  const int s = threadIdx.x;
  if (s >= kReportSums) return;
  double x = 0.0;
  for (int b = 0; b < nb; ++b) x += part[(size_t)b * kReportSums + s];
  out[s] = x;
}

}  // namespace disco
