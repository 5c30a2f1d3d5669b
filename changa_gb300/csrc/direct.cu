/*
 * Direct-sum accuracy yardstick: the force on sampled particles from every
 * particle, without a tree.  No reference counterpart (ChaNGa checks its
 * tree against nothing at run time); it gives the "error against the
 * direct sum" of every force form on workloads far too large for the CPU.
 *
 * Open boundaries: a_i = sum_j m_j b(r) r, pot_i = -sum_j m_j a(r), with
 * SPLINE's softening (gravity.h:147-182; twoh = soft_i + soft_j).
 *
 * Periodic cube of side L (G = 1, uniform neutralising background, the
 * convention of ChaNGa's Ewald sum, Ewald.cpp:72-281) by Ewald summation
 * with splitting parameter alpha:
 *   real space (minimum image, |r| < r_cut):
 *     a_i += m_j r [erfc(alpha r) / r^3 + 2 alpha / sqrt(pi) exp(-alpha^2 r^2) / r^2]
 *     and, for |r| < twoh, the softening correction m_j r (b_spline(r) - 1/r^3);
 *   k space (k = 2 pi n / L, 0 < |k| < k_cut):
 *     a_i += -(4 pi / L^3) sum_k exp(-k^2 / 4 alpha^2) / k^2  k  Im(e^{i k.x_i} conj(S(k))),
 *     S(k) = sum_j m_j e^{i k.x_j}.
 * alpha r_cut = 4.2 (erfc 2.6e-9) and exp(-k_cut^2 / 4 alpha^2) = 1e-9.
 * Pair terms are FP32 on bucket-free split coordinates (hi + lo parts, so
 * close pairs keep FP32 relative accuracy of the separation) with Kahan
 * sums per thread and FP64 totals; S(k) and the k-space sum are FP64.
 * Accuracy about 1e-6 of |a|: ample for judging tree errors of 1e-4..1e-2.
 */
#include <math.h>

#include "chg_internal.h"

namespace chg {
namespace {

constexpr int kDsThreads = 128;  // targets per block of the pair kernel
constexpr int kDsTile = 256;     // sources per shared-memory tile
constexpr int kSkThreads = 256;
constexpr int kSkKPT = 4;        // k-vectors per thread in the S(k) kernel
constexpr int kSkTileP = 32;     // particles per S(k) table tile
constexpr int kMaxN = 24;        // largest |n| per axis of the k-space sum

__device__ __forceinline__ void kahan(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

/* b(r) of SPLINE inside the softening (gravity.h:152-176), FP32. */
__device__ float spline_b(float r, float twoh) {
  const float dih = 2.0f / twoh;
  const float u = r * dih;
  const float dih3 = dih * dih * dih;
  if (u < 1.0f) return dih3 * (4.0f / 3.0f - 6.0f / 5.0f * u * u + 0.5f * u * u * u);
  const float ir = 1.0f / r;
  return -1.0f / 15.0f * ir * ir * ir +
         dih3 * (8.0f / 3.0f - 3.0f * u + 6.0f / 5.0f * u * u - 1.0f / 6.0f * u * u * u);
}

__device__ float spline_a(float r, float twoh) {
  const float dih = 2.0f / twoh;
  const float u = r * dih;
  const float u2 = u * u;
  if (u < 1.0f) return dih * (7.0f / 5.0f - 2.0f / 3.0f * u2 + 3.0f / 10.0f * u2 * u2 - 0.1f * u2 * u2 * u);
  return -1.0f / 15.0f / r +
         dih * (8.0f / 5.0f - 4.0f / 3.0f * u2 + u2 * u - 3.0f / 10.0f * u2 * u2 + u2 * u2 * u / 30.0f);
}

struct PairArgs {
  const float4* parts;  // packed {hi.xyz, m} {lo.xyz, soft}
  long long n;
  const int* idx;
  long long n_idx;
  float L;         // 0: open boundaries
  float rcut2;     // periodic real-space cutoff squared
  float alpha;
  long long split; // sources per block column
  double* partial; // gridDim.y x n_idx x 4
};

/* Pair sum over one column of sources for a block of targets. */
template <bool PERIODIC>
__global__ void __launch_bounds__(kDsThreads) ds_pair_kernel(const PairArgs a) {
  __shared__ float4 sh[kDsTile], sl[kDsTile];
  const long long t = blockIdx.x * (long long)kDsThreads + threadIdx.x;
  const bool active = t < a.n_idx;
  long long ti = active ? a.idx[t] : 0;
  if (ti < 0 || ti >= a.n) ti = 0;
  const float4 th = a.parts[2 * ti], tl = a.parts[2 * ti + 1];
  const float halfL = 0.5f * a.L;
  const float a2 = a.alpha * a.alpha;
  const float c2a = 1.1283791670955126f * a.alpha;  // 2 alpha / sqrt(pi)
  float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;
  const long long j0 = blockIdx.y * a.split;
  const long long j1 = min(a.n, j0 + a.split);
  for (long long jt = j0; jt < j1; jt += kDsTile) {
    const int nt = (int)min((long long)kDsTile, j1 - jt);
    __syncthreads();
    for (int k = threadIdx.x; k < nt; k += kDsThreads) {
      sh[k] = a.parts[2 * (jt + k)];
      sl[k] = a.parts[2 * (jt + k) + 1];
    }
    __syncthreads();
    if (!active) continue;
    for (int k = 0; k < nt; ++k) {
      const float4 h = sh[k], l = sl[k];
      float dx = h.x - th.x, dy = h.y - th.y, dz = h.z - th.z;
      if (PERIODIC) {
        dx = dx > halfL ? dx - a.L : (dx < -halfL ? dx + a.L : dx);
        dy = dy > halfL ? dy - a.L : (dy < -halfL ? dy + a.L : dy);
        dz = dz > halfL ? dz - a.L : (dz < -halfL ? dz + a.L : dz);
      }
      dx += l.x - tl.x;
      dy += l.y - tl.y;
      dz += l.z - tl.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (r2 == 0.f) continue;
      if (PERIODIC && r2 >= a.rcut2) continue;
      const float r = sqrtf(r2);
      const float ir = 1.0f / r;
      const float ir3 = ir * ir * ir;
      const float twoh = l.w + tl.w;
      float f, pot = 0.f;
      if (PERIODIC) {
        const float ar = a.alpha * r;
        f = erfcf(ar) * ir3 + c2a * expf(-a2 * r2) * ir * ir;
        if (r < twoh) f += spline_b(r, twoh) - ir3;
      } else {
        f = r < twoh ? spline_b(r, twoh) : ir3;
        pot = -h.w * (r < twoh ? spline_a(r, twoh) : ir);
      }
      const float fm = f * h.w;
      kahan(sx, cx, fm * dx);
      kahan(sy, cy, fm * dy);
      kahan(sz, cz, fm * dz);
      kahan(sp, cp, pot);
    }
  }
  if (active) {
    double* o = a.partial + ((size_t)blockIdx.y * a.n_idx + t) * 4;
    o[0] = (double)sx - (double)cx;
    o[1] = (double)sy - (double)cy;
    o[2] = (double)sz - (double)cz;
    o[3] = (double)sp - (double)cp;
  }
}

__global__ void ds_sum_kernel(const double* __restrict__ partial, int splits, long long n_idx,
                              double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 4 * n_idx;
       i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += partial[(size_t)k * 4 * n_idx + i];
    out[i] = s;
  }
}

/* S(k) for the half-space k-vectors kv[] (integer n per axis): per tile of
 * particles, e^{i 2 pi n x / L} tables per axis in shared memory, then each
 * thread accumulates its kSkKPT k-vectors over the tile. */
__global__ void __launch_bounds__(kSkThreads) ds_sk_kernel(const double* __restrict__ parts,
                                                           long long n, const int4* __restrict__ kv,
                                                           int nk, int nmax, double L,
                                                           long long split,
                                                           double2* __restrict__ S) {
  extern __shared__ double2 tab[];  // kSkTileP x 3 x (2 nmax + 1)
  const int W = 2 * nmax + 1;
  double2 acc[kSkKPT];
  int4 myk[kSkKPT];
#pragma unroll
  for (int q = 0; q < kSkKPT; ++q) {
    acc[q] = make_double2(0.0, 0.0);
    const int kk = (blockIdx.x * kSkThreads + threadIdx.x) * kSkKPT + q;
    myk[q] = kk < nk ? kv[kk] : make_int4(0, 0, 0, -1);
  }
  const double w = 2.0 * M_PI / L;
  const long long p0 = blockIdx.y * split;
  const long long p1 = min(n, p0 + split);
  for (long long pt = p0; pt < p1; pt += kSkTileP) {
    const int np = (int)min((long long)kSkTileP, p1 - pt);
    __syncthreads();
    for (int e = threadIdx.x; e < np * 3 * W; e += kSkThreads) {
      const int p = e / (3 * W), rem = e - p * 3 * W, ax = rem / W, nn = rem - ax * W - nmax;
      const double* r = parts + 5 * (pt + p);
      double sv, cv;
      sincos(w * (double)nn * r[2 + ax], &sv, &cv);
      const double m = ax == 2 ? r[0] : 1.0;  // fold the mass into the z table
      tab[e] = make_double2(m * cv, m * sv);
    }
    __syncthreads();
    for (int p = 0; p < np; ++p) {
      const double2* tp = tab + p * 3 * W;
#pragma unroll
      for (int q = 0; q < kSkKPT; ++q) {
        if (myk[q].w < 0) continue;
        const double2 ex = tp[myk[q].x + nmax], ey = tp[W + myk[q].y + nmax],
                      ez = tp[2 * W + myk[q].z + nmax];
        const double xr = ex.x * ey.x - ex.y * ey.y, xi = ex.x * ey.y + ex.y * ey.x;
        acc[q].x += xr * ez.x - xi * ez.y;
        acc[q].y += xr * ez.y + xi * ez.x;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kSkKPT; ++q) {
    if (myk[q].w < 0) continue;
    const int kk = (blockIdx.x * kSkThreads + threadIdx.x) * kSkKPT + q;
    atomicAdd(&S[kk].x, acc[q].x);
    atomicAdd(&S[kk].y, acc[q].y);
  }
}

/* k-space acceleration of the targets (FP64), added to out. */
__global__ void ds_kspace_kernel(const double* __restrict__ parts, long long n,
                                 const int* __restrict__ idx, long long n_idx,
                                 const int4* __restrict__ kv, const double2* __restrict__ S,
                                 int nk, double L, double alpha, double* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n_idx;
       t += (long long)gridDim.x * blockDim.x) {
    long long i = idx[t];
    if (i < 0 || i >= n) continue;
    const double* r = parts + 5 * i;
    const double w = 2.0 * M_PI / L;
    const double pref = -2.0 * 4.0 * M_PI / (L * L * L);  // x2: half-space sum
    double ax = 0, ay = 0, az = 0;
    for (int k = 0; k < nk; ++k) {
      const int4 q = kv[k];
      const double kx = w * q.x, ky = w * q.y, kz = w * q.z;
      const double k2 = kx * kx + ky * ky + kz * kz;
      const double g = exp(-k2 / (4.0 * alpha * alpha)) / k2;
      double sv, cv;
      sincos(kx * r[2] + ky * r[3] + kz * r[4], &sv, &cv);
      // Im(e^{i k.x} conj(S)) = sin(k.x) S.re - cos(k.x) S.im
      const double im = sv * S[k].x - cv * S[k].y;
      ax += g * kx * im;
      ay += g * ky * im;
      az += g * kz * im;
    }
    out[4 * t] += pref * ax;
    out[4 * t + 1] += pref * ay;
    out[4 * t + 2] += pref * az;
  }
}

}  // namespace
}  // namespace chg

using namespace chg;

extern "C" int changa_direct_forces(const double* parts, long long n_parts, const int* idx,
                                    long long n_idx, double L, double rcut_frac, double* out,
                                    cudaStream_t s) {
  if (n_parts < 0 || n_idx < 0 || (n_idx > 0 && (!parts || !idx || !out)) || L < 0 ||
      rcut_frac < 0 || rcut_frac > 0.5)
    return record_error(CHANGA_E_INVALID_ARG, "changa_direct_forces: arguments", __FILE__,
                        __LINE__);
  if (n_idx == 0) return 0;
  if (n_parts == 0) return (int)cudaMemsetAsync(out, 0, (size_t)n_idx * 4 * sizeof(double), s);
  const bool periodic = L > 0;
  const double rc = (rcut_frac > 0 ? rcut_frac : 0.5) * L;
  const double alpha = periodic ? 4.2 / rc : 0.0;
  /* k-space: exp(-k^2 / 4 alpha^2) >= 1e-9 -> |n| <= alpha L sqrt(ln 1e9) / pi */
  const int nmax = periodic ? (int)floor(alpha * L * sqrt(log(1e9)) / M_PI) : 0;
  if (nmax > kMaxN)
    return record_error(CHANGA_E_TOO_LARGE, "changa_direct_forces: r_cut too small", __FILE__,
                        __LINE__);
  /* half-space k-vectors with |n|^2 <= nmax^2 */
  int4* hk = nullptr;
  int nk = 0;
  if (periodic) {
    const int cap = (2 * nmax + 1) * (2 * nmax + 1) * (nmax + 1);
    hk = new int4[cap > 0 ? cap : 1];
    for (int z = 0; z <= nmax; ++z)
      for (int y = -nmax; y <= nmax; ++y)
        for (int x = -nmax; x <= nmax; ++x) {
          if (x * x + y * y + z * z > nmax * nmax || x * x + y * y + z * z == 0) continue;
          if (z == 0 && (y < 0 || (y == 0 && x < 0))) continue;
          hk[nk++] = make_int4(x, y, z, 0);
        }
  }
  const int grid_x = (int)((n_idx + kDsThreads - 1) / kDsThreads);
  int splits = (sm_count() * 8 + grid_x - 1) / grid_x;
  if (splits < 1) splits = 1;
  const long long split = (n_parts + splits - 1) / splits;
  splits = (int)((n_parts + split - 1) / split);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t pb = al((size_t)n_parts * kPartPackF4 * sizeof(float4));
  const size_t qb = al((size_t)splits * n_idx * 4 * sizeof(double));
  const size_t kb = al((size_t)(nk > 0 ? nk : 1) * sizeof(int4));
  const size_t sb = al((size_t)(nk > 0 ? nk : 1) * sizeof(double2));
  char* block = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&block, pb + qb + kb + sb, s);
  if (e != cudaSuccess) {
    delete[] hk;
    return record_error((int)e, "changa_direct_forces: scratch", __FILE__, __LINE__);
  }
  float4* pp = (float4*)block;
  double* partial = (double*)(block + pb);
  int4* dk = (int4*)(block + pb + qb);
  double2* S = (double2*)(block + pb + qb + kb);
  int rc_out = 0;
  do {
    if (nk > 0) {
      if ((e = cudaMemcpyAsync(dk, hk, (size_t)nk * sizeof(int4), cudaMemcpyHostToDevice, s)) !=
              cudaSuccess ||
          (e = cudaMemsetAsync(S, 0, (size_t)nk * sizeof(double2), s)) != cudaSuccess)
        break;
    }
    if ((e = launch_pack_parts(parts, n_parts, pp, s)) != cudaSuccess) break;
    PairArgs pa;
    pa.parts = pp;
    pa.n = n_parts;
    pa.idx = idx;
    pa.n_idx = n_idx;
    pa.L = (float)L;
    pa.rcut2 = (float)(rc * rc);
    pa.alpha = (float)alpha;
    pa.split = split;
    pa.partial = partial;
    dim3 g(grid_x, splits);
    if (periodic) ds_pair_kernel<true><<<g, kDsThreads, 0, s>>>(pa);
    else ds_pair_kernel<false><<<g, kDsThreads, 0, s>>>(pa);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    ds_sum_kernel<<<(int)((4 * n_idx + 255) / 256 < 4096 ? (4 * n_idx + 255) / 256 : 4096), 256, 0,
                    s>>>(partial, splits, n_idx, out);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if (nk > 0) {
      const int W = 2 * nmax + 1;
      const size_t smem = (size_t)kSkTileP * 3 * W * sizeof(double2);
      if ((e = cudaFuncSetAttribute(ds_sk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem)) != cudaSuccess)
        break;
      const int gx = (nk + kSkThreads * kSkKPT - 1) / (kSkThreads * kSkKPT);
      int gy = (sm_count() * 4 + gx - 1) / gx;
      const long long psplit = (n_parts + gy - 1) / gy;
      gy = (int)((n_parts + psplit - 1) / psplit);
      ds_sk_kernel<<<dim3(gx, gy), kSkThreads, smem, s>>>(parts, n_parts, dk, nk, nmax, L, psplit,
                                                           S);
      count_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      ds_kspace_kernel<<<(int)((n_idx + 127) / 128), 128, 0, s>>>(parts, n_parts, idx, n_idx, dk,
                                                                   S, nk, L, alpha, out);
      count_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
  } while (0);
  if (e != cudaSuccess) rc_out = record_error((int)e, "changa_direct_forces", __FILE__, __LINE__);
  cudaFreeAsync(block, s);
  /* hk is read by the copy above before the stream moves on */
  cudaStreamSynchronize(s);
  delete[] hk;
  return rc_out;
}
