/*
 * Device moment up-pass over a fixed tree topology (FP64).
 *
 * The host tree build (changa_gb300/host/tree.cpp) accumulates every node's
 * moments particle by particle and child by child, as
 * MultipoleMoments::operator+= does (MultipoleMoments.h:206-352); the sums
 * it forms are, for the node's particle range P:
 *   totalMass = sum_P m,        cm = sum_P m x / totalMass,
 *   soft      = sum_P m s / totalMass,
 *   xx..zz    = sum_P m (x - cm)_a (x - cm)_b   (about the centre of mass).
 * This kernel forms the same sums directly over each node's contiguous
 * particle range (GPU order), one warp per node, without atomics, so the
 * result does not depend on scheduling.  It refreshes the moments after the
 * particles move when the tree topology is kept (a differentiated leapfrog
 * reusing one step's lists, or a caller that rebuilds the tree less often
 * than it moves particles).  The radius (slot 0) is left unchanged: it only
 * drives the walk's opening test, which a fixed topology does not repeat.
 */
#include "chg_internal.h"

namespace chg {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__global__ void __launch_bounds__(256) node_moments_kernel(const double* __restrict__ parts,
                                                           long long n_parts,
                                                           const int* __restrict__ first,
                                                           const int* __restrict__ count,
                                                           long long n_moments,
                                                           double* __restrict__ moments) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long node = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
       node < n_moments; node += warps) {
    const long long f = __ldg(first + node);
    const long long c = __ldg(count + node);
    if (f < 0 || c <= 0 || f + c > n_parts) continue;
    double m = 0, mx = 0, my = 0, mz = 0, ms = 0;
    for (long long k = f + lane; k < f + c; k += 32) {
      const double* p = parts + 5 * k;
      const double pm = p[0];
      m += pm;
      ms += pm * p[1];
      mx += pm * p[2];
      my += pm * p[3];
      mz += pm * p[4];
    }
    m = warp_sum(m);
    ms = warp_sum(ms);
    mx = warp_sum(mx);
    my = warp_sum(my);
    mz = warp_sum(mz);
    if (!(m > 0.0)) continue;
    const double cx = mx / m, cy = my / m, cz = mz / m;
    double xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0;
    for (long long k = f + lane; k < f + c; k += 32) {
      const double* p = parts + 5 * k;
      const double pm = p[0];
      const double dx = p[2] - cx, dy = p[3] - cy, dz = p[4] - cz;
      xx += pm * dx * dx;
      xy += pm * dx * dy;
      xz += pm * dx * dz;
      yy += pm * dy * dy;
      yz += pm * dy * dz;
      zz += pm * dz * dz;
    }
    xx = warp_sum(xx);
    xy = warp_sum(xy);
    xz = warp_sum(xz);
    yy = warp_sum(yy);
    yz = warp_sum(yz);
    zz = warp_sum(zz);
    if (lane == 0) {
      double* o = moments + 12 * node;
      o[1] = ms / m;
      o[2] = m;
      o[3] = cx;
      o[4] = cy;
      o[5] = cz;
      o[6] = xx;
      o[7] = xy;
      o[8] = xz;
      o[9] = yy;
      o[10] = yz;
      o[11] = zz;
    }
  }
}

}  // namespace
}  // namespace chg

using namespace chg;

extern "C" int changa_tree_moments(const double* parts, long long n_parts, const int* first,
                                   const int* count, long long n_moments, double* moments,
                                   cudaStream_t s) {
  if (n_parts < 0 || n_moments < 0 || (n_moments > 0 && (!parts || !first || !count || !moments)))
    return record_error(CHANGA_E_INVALID_ARG, "changa_tree_moments: arrays", __FILE__, __LINE__);
  if (n_moments == 0) return 0;
  long long blocks = (n_moments + 7) / 8;
  const long long cap = (long long)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  {
    TimingScope ts(kKidMoments, s);
    node_moments_kernel<<<(int)blocks, 256, 0, s>>>(parts, n_parts, first, count, n_moments,
                                                     moments);
  }
  count_launch();
  CHG_CUDA(cudaGetLastError());
  return 0;
}
