/*
 * Periodic Ewald correction kernels.
 *
 * Reference: BucketEwald (Ewald.cpp:72-281) on the CPU and EwaldKernel
 * (HostCUDA.cu:1958-2192) on the GPU.  Per target particle at d = x - cm:
 * a real-space sum over replicas |i| <= nEwReps (terms with r^2 beyond
 * (fEwCut L)^2 skipped unless inside the "hole" |i| <= nReps, where erfc is
 * replaced by -erf to cancel the tree's own replicas), a series expansion
 * about the origin when r^2 < fInner2, then the k-space sum over the
 * h-table.  One thread per particle, as the work per particle is uniform.
 *
 * Root data travel as a __grid_constant__ kernel parameter (the reference
 * writes __constant__ symbols per call, a race between concurrent streams).
 * Forms:
 *   ewald_f32_kernel  the drop-in form on the FP32 ABI: the reference's
 *                     algorithm and constants, including its single-precision
 *                     fInner2 = 1.1e-2 L^2;
 *   ewald_f64_kernel  all FP64 with the CPU constants (fInner2 = 1.2e-3 L^2);
 *   ewald_mix_kernel  FP32-mixed: d = x - cm in FP64 rounded once; each warp
 *                     first culls the replica lattice against the bounding box
 *                     of its 32 particles (so threads loop over ~90 candidate
 *                     replicas, not 343, each kept as packed offsets and its
 *                     hole flag); hole terms with alpha^2 r^2 < 1 use
 *                     the convergent power series of the g_n (no cancellation
 *                     between -erf(ar)/r and the 1/r^k terms); other terms use
 *                     a rational erfc with fractional error < 1.2e-7 (Press et
 *                     al., Numerical Recipes, "erfcc", a Chebyshev fit) and
 *                     the hardware exp2; the k-space phase is reduced to one
 *                     turn from the integer h before the hardware sin/cos.
 */
#include <cmath>
#include <type_traits>
#include <vector>

#include "chg_internal.h"
#include "f32x2.cuh"

namespace chg {
namespace {

struct EwaldF32Args {
  EwaldReadOnlyData ro;
  EwtData ewt[NEWH];
};

__global__ void __launch_bounds__(128) ewald_f32_kernel(const CompactPartData* __restrict__ parts,
                                                        VariablePartData* __restrict__ vars,
                                                        const int* __restrict__ markers,
                                                        int largephase, int first, int last,
                                                        const __grid_constant__ EwaldF32Args P) {
  const EwaldReadOnlyData& ro = P.ro;
  int id;
  if (largephase) {
    id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id > last) return;
    id = markers[id];
  } else {
    id = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (id > last) return;
  }
  const CompactPartData p = parts[id];
  const MultipoleMomentsData& mom = ro.mm;
#ifdef HEXADECAPOLE
  /* traces of the complete root moments (Ewald.cpp:99-111) */
  const MomcData& mc = ro.momcRoot;
  const float Q4xx = 0.5f * (mc.xxxx + mc.xxyy + mc.xxzz);
  const float Q4xy = 0.5f * (mc.xxxy + mc.xyyy + mc.xyzz);
  const float Q4xz = 0.5f * (mc.xxxz + mc.xyyz + mc.xzzz);
  const float Q4yy = 0.5f * (mc.xxyy + mc.yyyy + mc.yyzz);
  const float Q4yz = 0.5f * (mc.xxyz + mc.yyyz + mc.yzzz);
  const float Q4zz = 0.5f * (mc.xxzz + mc.yyzz + mc.zzzz);
  const float Q4 = 0.25f * (Q4xx + Q4yy + Q4zz);
  const float Q3x = 0.5f * (mc.xxx + mc.xyy + mc.xzz);
  const float Q3y = 0.5f * (mc.xxy + mc.yyy + mc.yzz);
  const float Q3z = 0.5f * (mc.xxz + mc.yyz + mc.zzz);
  const float Q2 = 0.5f * (mc.xx + mc.yy + mc.zz);
#else
  const float Q2 = 0.5f * (mom.xx + mom.yy + mom.zz);
#endif
  float ax = 0.f, ay = 0.f, az = 0.f;
  float fPot = mom.totalMass * ro.k1;
  const float xdif = p.position.x - mom.cmx, ydif = p.position.y - mom.cmy,
              zdif = p.position.z - mom.cmz;
  const int nE = ro.nEwReps, nR = ro.nReps;
  for (int ix = -nE; ix <= nE; ++ix) {
    const bool hx = (ix >= -nR && ix <= nR);
    const float x = xdif + ix * ro.L;
    for (int iy = -nE; iy <= nE; ++iy) {
      const bool hxy = hx && (iy >= -nR && iy <= nR);
      const float y = ydif + iy * ro.L;
      for (int iz = -nE; iz <= nE; ++iz) {
        const bool hole = hxy && (iz >= -nR && iz <= nR);
        const float z = zdif + iz * ro.L;
        float r2 = x * x + y * y + z * z;
        if (r2 > ro.fEwCut2 && !hole) continue;
        float g0, g1, g2, g3;
#ifdef HEXADECAPOLE
        float g4, g5;
#endif
        if (r2 < ro.fInner2) {
          float alphan = ro.ka;
          r2 *= ro.alpha2;
          g0 = alphan * ((1.0f / 3.0f) * r2 - 1.0f);
          alphan *= 2.f * ro.alpha2;
          g1 = alphan * ((1.0f / 5.0f) * r2 - (1.0f / 3.0f));
          alphan *= 2.f * ro.alpha2;
          g2 = alphan * ((1.0f / 7.0f) * r2 - (1.0f / 5.0f));
          alphan *= 2.f * ro.alpha2;
          g3 = alphan * ((1.0f / 9.0f) * r2 - (1.0f / 7.0f));
#ifdef HEXADECAPOLE
          alphan *= 2.f * ro.alpha2;
          g4 = alphan * ((1.0f / 11.0f) * r2 - (1.0f / 9.0f));
          alphan *= 2.f * ro.alpha2;
          g5 = alphan * ((1.0f / 13.0f) * r2 - (1.0f / 11.0f));
#endif
        } else {
          const float dir = rsqrtf(r2);
          const float dir2 = dir * dir;
          float a = expf(-r2 * ro.alpha2);
          a *= ro.ka * dir2;
          const float ar = ro.alpha * (r2 * dir);
          g0 = hole ? -erff(ar) : erfcf(ar);
          g0 *= dir;
          g1 = g0 * dir2 + a;
          float alphan = 2.f * ro.alpha2;
          g2 = 3.f * g1 * dir2 + alphan * a;
          alphan *= 2.f * ro.alpha2;
          g3 = 5.f * g2 * dir2 + alphan * a;
#ifdef HEXADECAPOLE
          alphan *= 2.f * ro.alpha2;
          g4 = 7.f * g3 * dir2 + alphan * a;
          alphan *= 2.f * ro.alpha2;
          g5 = 9.f * g4 * dir2 + alphan * a;
#endif
        }
#ifdef HEXADECAPOLE
        /* the hexadecapole expansion term (Ewald.cpp:203-240) */
        const float xx = 0.5f * x * x, yy = 0.5f * y * y, zz = 0.5f * z * z;
        const float xy = x * y, xz = x * z, yz = y * z, xyz = xy * z;
        const float xxx = (1.0f / 3.0f) * xx * x, yyy = (1.0f / 3.0f) * yy * y,
                    zzz = (1.0f / 3.0f) * zz * z;
        const float xxy = xx * y, xxz = xx * z, xyy = yy * x, yyz = yy * z, xzz = zz * x,
                    yzz = zz * y;
        const float Q2mirx = mc.xx * x + mc.xy * y + mc.xz * z;
        const float Q2miry = mc.xy * x + mc.yy * y + mc.yz * z;
        const float Q2mirz = mc.xz * x + mc.yz * y + mc.zz * z;
        const float Q3mirx = mc.xxx * xx + mc.xxy * xy + mc.xxz * xz + mc.xyy * yy +
                             mc.xyz * yz + mc.xzz * zz;
        const float Q3miry = mc.xxy * xx + mc.xyy * xy + mc.xyz * xz + mc.yyy * yy +
                             mc.yyz * yz + mc.yzz * zz;
        const float Q3mirz = mc.xxz * xx + mc.xyz * xy + mc.xzz * xz + mc.yyz * yy +
                             mc.yzz * yz + mc.zzz * zz;
        const float Q4mirx = mc.xxxx * xxx + mc.xxxy * xxy + mc.xxxz * xxz + mc.xxyy * xyy +
                             mc.xxyz * xyz + mc.xxzz * xzz + mc.xyyy * yyy + mc.xyyz * yyz +
                             mc.xyzz * yzz + mc.xzzz * zzz;
        const float Q4miry = mc.xxxy * xxx + mc.xxyy * xxy + mc.xxyz * xxz + mc.xyyy * xyy +
                             mc.xyyz * xyz + mc.xyzz * xzz + mc.yyyy * yyy + mc.yyyz * yyz +
                             mc.yyzz * yzz + mc.yzzz * zzz;
        const float Q4mirz = mc.xxxz * xxx + mc.xxyz * xxy + mc.xxzz * xxz + mc.xyyz * xyy +
                             mc.xyzz * xyz + mc.xzzz * xzz + mc.yyyz * yyy + mc.yyzz * yyz +
                             mc.yzzz * yzz + mc.zzzz * zzz;
        const float Q4x = Q4xx * x + Q4xy * y + Q4xz * z;
        const float Q4y = Q4xy * x + Q4yy * y + Q4yz * z;
        const float Q4z = Q4xz * x + Q4yz * y + Q4zz * z;
        const float Q2mir = 0.5f * (Q2mirx * x + Q2miry * y + Q2mirz * z) -
                            (Q3x * x + Q3y * y + Q3z * z) + Q4;
        const float Q3mir = (1.0f / 3.0f) * (Q3mirx * x + Q3miry * y + Q3mirz * z) -
                            0.5f * (Q4x * x + Q4y * y + Q4z * z);
        const float Q4mir = 0.25f * (Q4mirx * x + Q4miry * y + Q4mirz * z);
        const float Qta = g1 * mc.m - g2 * Q2 + g3 * Q2mir + g4 * Q3mir + g5 * Q4mir;
        fPot -= g0 * mc.m - g1 * Q2 + g2 * Q2mir + g3 * Q3mir + g4 * Q4mir;
        ax += g2 * (Q2mirx - Q3x) + g3 * (Q3mirx - Q4x) + g4 * Q4mirx - x * Qta;
        ay += g2 * (Q2miry - Q3y) + g3 * (Q3miry - Q4y) + g4 * Q4miry - y * Qta;
        az += g2 * (Q2mirz - Q3z) + g3 * (Q3mirz - Q4z) + g4 * Q4mirz - z * Qta;
#else
        const float Q2mirx = mom.xx * x + mom.xy * y + mom.xz * z;
        const float Q2miry = mom.xy * x + mom.yy * y + mom.yz * z;
        const float Q2mirz = mom.xz * x + mom.yz * y + mom.zz * z;
        const float Q2mir = 0.5f * (Q2mirx * x + Q2miry * y + Q2mirz * z);
        const float Qta = g1 * mom.totalMass - g2 * Q2 + g3 * Q2mir;
        fPot -= g0 * mom.totalMass - g1 * Q2 + g2 * Q2mir;
        ax += g2 * Q2mirx - x * Qta;
        ay += g2 * Q2miry - y * Qta;
        az += g2 * Q2mirz - z * Qta;
#endif
      }
    }
  }
  for (int i = 0; i < ro.nEwhLoop; ++i) {
    const EwtData& e = P.ewt[i];
    const float hdotx = e.hx * xdif + e.hy * ydif + e.hz * zdif;
    float s, c;
    sincosf(hdotx, &s, &c);
    fPot += e.hCfac * c + e.hSfac * s;
    const float t = e.hCfac * s - e.hSfac * c;
    ax += e.hx * t;
    ay += e.hy * t;
    az += e.hz * t;
  }
  VariablePartData& v = vars[id];
  v.a.x += ax;
  v.a.y += ay;
  v.a.z += az;
  v.potential += fPot;
}
/* The hexadecapole build's root for the extension forms: complete moments
 * (EwaldCUDA.h MomcData order) and their traces (Ewald.cpp:99-111). */
template <typename T>
struct HexRoot {
  T c[32];
  T Q4xx, Q4xy, Q4xz, Q4yy, Q4yz, Q4zz, Q4, Q3x, Q3y, Q3z, Q2;
};

template <typename T>
void fill_hex_root(const double* mc, HexRoot<T>& R) {
  for (int k = 0; k < 32; ++k) R.c[k] = (T)mc[k];
  R.Q4xx = (T)(0.5 * (mc[13] + mc[19] + mc[26]));
  R.Q4xy = (T)(0.5 * (mc[15] + mc[14] + mc[27]));
  R.Q4xz = (T)(0.5 * (mc[17] + mc[21] + mc[28]));
  R.Q4yy = (T)(0.5 * (mc[19] + mc[16] + mc[29]));
  R.Q4yz = (T)(0.5 * (mc[20] + mc[18] + mc[30]));
  R.Q4zz = (T)(0.5 * (mc[26] + mc[29] + mc[31]));
  R.Q4 = (T)(0.25 * (0.5 * (mc[13] + mc[19] + mc[26]) + 0.5 * (mc[19] + mc[16] + mc[29]) +
                     0.5 * (mc[26] + mc[29] + mc[31])));
  R.Q3x = (T)(0.5 * (mc[6] + mc[7] + mc[23]));
  R.Q3y = (T)(0.5 * (mc[8] + mc[9] + mc[24]));
  R.Q3z = (T)(0.5 * (mc[10] + mc[11] + mc[25]));
  R.Q2 = (T)(0.5 * (mc[1] + mc[2] + mc[22]));
}

/* One real-space term of the hexadecapole expansion about the root
 * (Ewald.cpp:203-240) at offset (x, y, z) with g0..g5.  MomcData indices:
 * 0 m; 1 xx 2 yy 3 xy 4 xz 5 yz; 6 xxx 7 xyy 8 xxy 9 yyy 10 xxz 11 yyz
 * 12 xyz; 13 xxxx 14 xyyy 15 xxxy 16 yyyy 17 xxxz 18 yyyz 19 xxyy 20 xxyz
 * 21 xyyz; 22 zz; 23 xzz 24 yzz 25 zzz; 26 xxzz 27 xyzz 28 xzzz 29 yyzz
 * 30 yzzz 31 zzzz. */
template <typename T>
__device__ __forceinline__ void hex_ewald_term(const HexRoot<T>& R, T x, T y, T z, T g0, T g1,
                                               T g2, T g3, T g4, T g5, T& fPot, T& ax, T& ay,
                                               T& az) {
  const T* c = R.c;
  const T third = T(1) / T(3);
  const T xx = T(0.5) * x * x, yy = T(0.5) * y * y, zz = T(0.5) * z * z;
  const T xy = x * y, xz = x * z, yz = y * z, xyz = xy * z;
  const T xxx = third * xx * x, yyy = third * yy * y, zzz = third * zz * z;
  const T xxy = xx * y, xxz = xx * z, xyy = yy * x, yyz = yy * z, xzz = zz * x, yzz = zz * y;
  const T Q2mirx = c[1] * x + c[3] * y + c[4] * z;
  const T Q2miry = c[3] * x + c[2] * y + c[5] * z;
  const T Q2mirz = c[4] * x + c[5] * y + c[22] * z;
  const T Q3mirx = c[6] * xx + c[8] * xy + c[10] * xz + c[7] * yy + c[12] * yz + c[23] * zz;
  const T Q3miry = c[8] * xx + c[7] * xy + c[12] * xz + c[9] * yy + c[11] * yz + c[24] * zz;
  const T Q3mirz = c[10] * xx + c[12] * xy + c[23] * xz + c[11] * yy + c[24] * yz + c[25] * zz;
  const T Q4mirx = c[13] * xxx + c[15] * xxy + c[17] * xxz + c[19] * xyy + c[20] * xyz +
                   c[26] * xzz + c[14] * yyy + c[21] * yyz + c[27] * yzz + c[28] * zzz;
  const T Q4miry = c[15] * xxx + c[19] * xxy + c[20] * xxz + c[14] * xyy + c[21] * xyz +
                   c[27] * xzz + c[16] * yyy + c[18] * yyz + c[29] * yzz + c[30] * zzz;
  const T Q4mirz = c[17] * xxx + c[20] * xxy + c[26] * xxz + c[21] * xyy + c[27] * xyz +
                   c[28] * xzz + c[18] * yyy + c[29] * yyz + c[30] * yzz + c[31] * zzz;
  const T Q4x = R.Q4xx * x + R.Q4xy * y + R.Q4xz * z;
  const T Q4y = R.Q4xy * x + R.Q4yy * y + R.Q4yz * z;
  const T Q4z = R.Q4xz * x + R.Q4yz * y + R.Q4zz * z;
  const T Q2mir = T(0.5) * (Q2mirx * x + Q2miry * y + Q2mirz * z) -
                  (R.Q3x * x + R.Q3y * y + R.Q3z * z) + R.Q4;
  const T Q3mir = third * (Q3mirx * x + Q3miry * y + Q3mirz * z) -
                  T(0.5) * (Q4x * x + Q4y * y + Q4z * z);
  const T Q4mir = T(0.25) * (Q4mirx * x + Q4miry * y + Q4mirz * z);
  const T M = c[0];
  const T Qta = g1 * M - g2 * R.Q2 + g3 * Q2mir + g4 * Q3mir + g5 * Q4mir;
  fPot -= g0 * M - g1 * R.Q2 + g2 * Q2mir + g3 * Q3mir + g4 * Q4mir;
  ax += g2 * (Q2mirx - R.Q3x) + g3 * (Q3mirx - Q4x) + g4 * Q4mirx - x * Qta;
  ay += g2 * (Q2miry - R.Q3y) + g3 * (Q3miry - Q4y) + g4 * Q4miry - y * Qta;
  az += g2 * (Q2mirz - R.Q3z) + g3 * (Q3mirz - Q4z) + g4 * Q4mirz - z * Qta;
}

struct EwaldFpArgs {
  double mom[12];
  HexRoot<double> hex;  // the hexadecapole build's root (HEX kernels only)
  double L, fEwCut2, alpha, alpha2, k1, ka;
  int nReps, nEwReps, nEwhLoop;
  double ewt[CHANGA_MAX_EWH][5];
};

/* FP64 real-space term (Ewald.cpp:137-240): quadrupole, or with HEX the
 * hexadecapole expansion of the complete root moments (g4, g5 added). */
template <bool HEX>
__device__ __forceinline__ void ewald_term_f64(const EwaldFpArgs& P, double x, double y, double z,
                                               bool hole, double fInner2, double& fPot,
                                               double& ax, double& ay, double& az) {
  const double* mom = P.mom;
  double r2 = x * x + y * y + z * z;
  double g0, g1, g2, g3, g4 = 0.0, g5 = 0.0;
  if (r2 < fInner2) {
    double alphan = P.ka;
    r2 *= P.alpha2;
    g0 = alphan * ((1.0 / 3.0) * r2 - 1.0);
    alphan *= 2 * P.alpha2;
    g1 = alphan * ((1.0 / 5.0) * r2 - (1.0 / 3.0));
    alphan *= 2 * P.alpha2;
    g2 = alphan * ((1.0 / 7.0) * r2 - (1.0 / 5.0));
    alphan *= 2 * P.alpha2;
    g3 = alphan * ((1.0 / 9.0) * r2 - (1.0 / 7.0));
    if constexpr (HEX) {
      alphan *= 2 * P.alpha2;
      g4 = alphan * ((1.0 / 11.0) * r2 - (1.0 / 9.0));
      alphan *= 2 * P.alpha2;
      g5 = alphan * ((1.0 / 13.0) * r2 - (1.0 / 11.0));
    }
  } else {
    const double dir = rsqrt(r2);
    const double dir2 = dir * dir;
    double a = exp(-r2 * P.alpha2);
    a *= P.ka * dir2;
    const double ar = P.alpha * (r2 * dir);
    g0 = hole ? -erf(ar) : erfc(ar);
    g0 *= dir;
    g1 = g0 * dir2 + a;
    double alphan = 2 * P.alpha2;
    g2 = 3 * g1 * dir2 + alphan * a;
    alphan *= 2 * P.alpha2;
    g3 = 5 * g2 * dir2 + alphan * a;
    if constexpr (HEX) {
      alphan *= 2 * P.alpha2;
      g4 = 7 * g3 * dir2 + alphan * a;
      alphan *= 2 * P.alpha2;
      g5 = 9 * g4 * dir2 + alphan * a;
    }
  }
  if constexpr (HEX) {
    hex_ewald_term<double>(P.hex, x, y, z, g0, g1, g2, g3, g4, g5, fPot, ax, ay, az);
    return;
  }
  const double Q2 = 0.5 * (mom[6] + mom[9] + mom[11]);
  const double Q2mirx = mom[6] * x + mom[7] * y + mom[8] * z;
  const double Q2miry = mom[7] * x + mom[9] * y + mom[10] * z;
  const double Q2mirz = mom[8] * x + mom[10] * y + mom[11] * z;
  const double Q2mir = 0.5 * (Q2mirx * x + Q2miry * y + Q2mirz * z);
  const double Qta = g1 * mom[2] - g2 * Q2 + g3 * Q2mir;
  fPot -= g0 * mom[2] - g1 * Q2 + g2 * Q2mir;
  ax += g2 * Q2mirx - x * Qta;
  ay += g2 * Q2miry - y * Qta;
  az += g2 * Q2mirz - z * Qta;
}


template <bool HEX>
__global__ void __launch_bounds__(128) ewald_f64_kernel(const double* __restrict__ parts,
                                                        long long n_parts,
                                                        const int* __restrict__ idx,
                                                        long long n_idx, double* __restrict__ vars,
                                                        const __grid_constant__ EwaldFpArgs P) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= n_idx) return;
  const long long j = idx ? (long long)idx[k] : k;
  if (j < 0 || j >= n_parts) return;
  const double* p = parts + 5 * j;
  const double dxd = p[2] - P.mom[3], dyd = p[3] - P.mom[4], dzd = p[4] - P.mom[5];
  const int nE = P.nEwReps, nR = P.nReps;
  double fPot = P.mom[2] * P.k1, ax = 0, ay = 0, az = 0;
  const double fInner2 = 1.2e-3 * P.L * P.L;
  for (int ix = -nE; ix <= nE; ++ix) {
    const bool hx = (ix >= -nR && ix <= nR);
    const double x = dxd + ix * P.L;
    for (int iy = -nE; iy <= nE; ++iy) {
      const bool hxy = hx && (iy >= -nR && iy <= nR);
      const double y = dyd + iy * P.L;
      for (int iz = -nE; iz <= nE; ++iz) {
        const bool hole = hxy && (iz >= -nR && iz <= nR);
        const double z = dzd + iz * P.L;
        const double r2 = x * x + y * y + z * z;
        if (r2 > P.fEwCut2 && !hole) continue;
        ewald_term_f64<HEX>(P, x, y, z, hole, fInner2, fPot, ax, ay, az);
      }
    }
  }
  for (int i = 0; i < P.nEwhLoop; ++i) {
    const double* e = P.ewt[i];
    const double hdotx = e[0] * dxd + e[1] * dyd + e[2] * dzd;
    double s, c;
    sincos(hdotx, &s, &c);
    fPot += e[3] * c + e[4] * s;
    const double t = e[3] * s - e[4] * c;
    ax += e[0] * t;
    ay += e[1] * t;
    az += e[2] * t;
  }
  double* v = vars + 5 * j;
  v[0] += ax;
  v[1] += ay;
  v[2] += az;
  v[3] += fPot;
}

/* ---- FP32-mixed form ---- */

constexpr int kMixMaxReps = 4;                       // nEwReps limit of the mixed kernel
constexpr int kMixMaxRepl = (2 * kMixMaxReps + 1) * (2 * kMixMaxReps + 1) * (2 * kMixMaxReps + 1);
constexpr int kMixWarps = 4;

struct EwaldMixArgs {
  double cm[3];
  float M, xx, xy, xz, yy, yz, zz, Q2;
  HexRoot<float> hex;  // the hexadecapole build's root (HEX kernels only)
  float L, alpha2, ka, cut2, k1M, twopi_over_L;
  int nReps, nEwReps, nEwhLoop;
  float4 h[CHANGA_MAX_EWH];  // integer h as floats, hCfac
  float hs[CHANGA_MAX_EWH];  // hSfac
};

/* Series of the hole terms, g_n = -(2 alpha^2)^n ka S_n(s), s = alpha^2 r^2,
 * S_n(s) = sum_j (-1)^j s^j / (j! (2j + 2n + 1)): the Taylor series of
 * -erf(alpha r)/r and of its derivatives g_{n+1} = -(1/r) dg_n/dr.  For
 * s < 1, twelve terms reach FP32 rounding and every term is smaller than
 * the previous one, so nothing cancels. */
__host__ __device__ constexpr double hole_coef(int n, int j) {
  double f = 1.0;
  for (int q = 2; q <= j; ++q) f *= q;
  return ((j & 1) ? -1.0 : 1.0) / (f * (2 * j + 2 * n + 1));
}

template <int NN>
__device__ __forceinline__ float hole_series(float s) {
  constexpr float c0 = (float)hole_coef(NN, 0), c1 = (float)hole_coef(NN, 1);
  constexpr float c2 = (float)hole_coef(NN, 2), c3 = (float)hole_coef(NN, 3);
  constexpr float c4 = (float)hole_coef(NN, 4), c5 = (float)hole_coef(NN, 5);
  constexpr float c6 = (float)hole_coef(NN, 6), c7 = (float)hole_coef(NN, 7);
  constexpr float c8 = (float)hole_coef(NN, 8), c9 = (float)hole_coef(NN, 9);
  constexpr float c10 = (float)hole_coef(NN, 10), c11 = (float)hole_coef(NN, 11);
  float a = c11;
  a = fmaf(a, s, c10);
  a = fmaf(a, s, c9);
  a = fmaf(a, s, c8);
  a = fmaf(a, s, c7);
  a = fmaf(a, s, c6);
  a = fmaf(a, s, c5);
  a = fmaf(a, s, c4);
  a = fmaf(a, s, c3);
  a = fmaf(a, s, c2);
  a = fmaf(a, s, c1);
  return fmaf(a, s, c0);
}

/* erfc(x) for x >= 0 with fractional error below 1.2e-7: the rational
 * Chebyshev fit of Press, Teukolsky, Vetterling & Flannery, Numerical
 * Recipes (2nd ed., section 6.2, "erfcc"); e = exp(-x^2 - 1.26551223 + ...)
 * evaluated with the hardware exp2. */
__device__ __forceinline__ float erfc_nr(float x, float x2) {
  const float t = __fdividef(1.0f, fmaf(0.5f, x, 1.0f));
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  p = fmaf(p, t, -1.26551223f);
  return t * __expf(p - x2);
}

template <bool HEX>
__global__ void __launch_bounds__(kMixWarps * 32) ewald_mix_kernel(
    const double* __restrict__ parts, long long n_parts, const int* __restrict__ idx,
    long long n_idx, double* __restrict__ vars, const __grid_constant__ EwaldMixArgs P) {
  __shared__ short repl[kMixWarps][kMixMaxRepl];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long j = -1;
  if (k < n_idx) {
    j = idx ? (long long)idx[k] : k;
    if (j < 0 || j >= n_parts) j = -1;
  }
  const bool live = j >= 0;
  float dx = 0.f, dy = 0.f, dz = 0.f;
  if (live) {
    const double* p = parts + 5 * j;
    dx = (float)(p[2] - P.cm[0]);
    dy = (float)(p[3] - P.cm[1]);
    dz = (float)(p[4] - P.cm[2]);
  }
  /* bounding box of the warp's offsets */
  float lo[3] = {live ? dx : 1e30f, live ? dy : 1e30f, live ? dz : 1e30f};
  float hi[3] = {live ? dx : -1e30f, live ? dy : -1e30f, live ? dz : -1e30f};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  const int nE = P.nEwReps, nR = P.nReps, side = 2 * nE + 1, nrep = side * side * side;
  const float L = P.L;
  /* candidate replicas: the hole's first (all of them), then those within
   * the cut of some point of the warp's box */
  int count = 0, nhole = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int base = 0; base < nrep; base += 32) {
      const int r = base + lane;
      bool keep = false;
      int ix = 0, iy = 0, iz = 0;
      bool hole = false;
      if (r < nrep) {
        ix = r / (side * side) - nE;
        iy = (r / side) % side - nE;
        iz = r % side - nE;
        hole = ix >= -nR && ix <= nR && iy >= -nR && iy <= nR && iz >= -nR && iz <= nR;
        if (pass == 0) {
          keep = hole;
        } else if (!hole) {
          float d2 = 0.f;
          const int ii[3] = {ix, iy, iz};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float a = lo[c] + ii[c] * L, b = hi[c] + ii[c] * L;
            const float m = a > 0.f ? a : (b < 0.f ? -b : 0.f);
            d2 = fmaf(m, m, d2);
          }
          keep = d2 <= P.cut2 * 1.0001f;
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      /* the replica as packed offsets (each + 8 in four bits) and its hole
       * flag, so the term loop decodes it with shifts instead of integer
       * divisions */
      if (keep)
        repl[warp][count + __popc(bal & ((1u << lane) - 1u))] =
            (short)((ix + 8) | ((iy + 8) << 4) | ((iz + 8) << 8) | ((int)hole << 12));
      count += __popc(bal);
    }
    if (pass == 0) nhole = count;
  }
  __syncwarp();
  if (!live) return;

  const float a2 = P.alpha2, twoa2 = 2.f * a2, foura4 = twoa2 * twoa2, ka = P.ka;
  const float M = P.M, Q2 = P.Q2;
  float fp = P.k1M, fx = 0.f, fy = 0.f, fz = 0.f;
  /* a packed offset nibble k (0..15) as the float k - 8: k placed in the
   * mantissa of 2^23 (exact), then 2^23 + 8 subtracted (exact) */
  auto nibr = [](int v, int sh) { return __int_as_float(0x4B000000 | ((v >> sh) & 15)); };
  auto nib = [&](int v, int sh) { return nibr(v, sh) - 8388616.0f; };
  if constexpr (HEX) {
    const float alpha = sqrtf(a2);
    for (int q = 0; q < count; ++q) {
      const int pk = repl[warp][q];
      const bool hole = (pk >> 12) & 1;
      const float x = fmaf(nib(pk, 0), L, dx), y = fmaf(nib(pk, 4), L, dy),
                  z = fmaf(nib(pk, 8), L, dz);
      const float r2 = x * x + y * y + z * z;
      if (r2 > P.cut2 && !hole) continue;
      const float s = a2 * r2;
      float g0, g1, g2, g3, g4 = 0.f, g5 = 0.f;
      if (hole && s < 1.0f) {
        g0 = -ka * hole_series<0>(s);
        g1 = -twoa2 * ka * hole_series<1>(s);
        g2 = -foura4 * ka * hole_series<2>(s);
        g3 = -foura4 * twoa2 * ka * hole_series<3>(s);
        if constexpr (HEX) {
          g4 = -foura4 * foura4 * ka * hole_series<4>(s);
          g5 = -foura4 * foura4 * twoa2 * ka * hole_series<5>(s);
        }
      } else {
        const float dir = rsqrtf(r2);
        const float dir2 = dir * dir;
        const float ar = alpha * (r2 * dir);  // alpha r from the reciprocal root
        const float e = __expf(-s);
        const float a = ka * dir2 * e;
        const float ec = erfc_nr(ar, s);
        g0 = (hole ? ec - 1.0f : ec) * dir;
        g1 = fmaf(g0, dir2, a);
        g2 = fmaf(3.f * g1, dir2, twoa2 * a);
        g3 = fmaf(5.f * g2, dir2, foura4 * a);
        if constexpr (HEX) {
          g4 = fmaf(7.f * g3, dir2, foura4 * twoa2 * a);
          g5 = fmaf(9.f * g4, dir2, foura4 * foura4 * a);
        }
      }
      if constexpr (HEX) {
        hex_ewald_term<float>(P.hex, x, y, z, g0, g1, g2, g3, g4, g5, fp, fx, fy, fz);
        continue;
      }
      const float Q2mirx = P.xx * x + P.xy * y + P.xz * z;
      const float Q2miry = P.xy * x + P.yy * y + P.yz * z;
      const float Q2mirz = P.xz * x + P.yz * y + P.zz * z;
      const float Q2mir = 0.5f * (Q2mirx * x + Q2miry * y + Q2mirz * z);
      const float Qta = g1 * M - g2 * Q2 + g3 * Q2mir;
      fp -= g0 * M - g1 * Q2 + g2 * Q2mir;
      fx += g2 * Q2mirx - x * Qta;
      fy += g2 * Q2miry - y * Qta;
      fz += g2 * Q2mirz - z * Qta;
    }
  } else {
    /* two culled replicas per step as packed .f32x2 pairs; a replica past
     * the cut (outside the hole), or the padding of an odd count, is
     * evaluated and multiplied by 0 (its terms are finite) */
    const f2 dx2 = pk2(dx, dx), dy2 = pk2(dy, dy), dz2 = pk2(dz, dz), L2 = pk2(L, L);
    const float alpha = sqrtf(a2);
    const f2 alphap = pk2(alpha, alpha);
    const f2 a2p = pk2(a2, a2), kap = pk2(ka, ka), twoa2p = pk2(twoa2, twoa2),
             foura4p = pk2(foura4, foura4), Mp = pk2(M, M), Q2p = pk2(Q2, Q2);
    const f2 xx = pk2(P.xx, P.xx), xy = pk2(P.xy, P.xy), xz = pk2(P.xz, P.xz),
             yy = pk2(P.yy, P.yy), yz = pk2(P.yz, P.yz), zz = pk2(P.zz, P.zz);
    f2 fp2 = 0ull, fx2 = 0ull, fy2 = 0ull, fz2 = 0ull;
    const f2 bias2 = pk2(8388616.0f, 8388616.0f);
    /* one step over culled replicas q and q + 1 of a region ending at
     * qend: the hole's (H, every replica kept, the series near the root)
     * or the rest (no hole terms, the cut per replica) */
    auto step = [&](int q, int qend, auto holes) {
      constexpr bool H = decltype(holes)::value;
      const bool two = q + 1 < qend;
      const int pk0 = repl[warp][q], pk1 = two ? repl[warp][q + 1] : pk0;
      const bool hole0 = H, hole1 = H;
      const f2 x = fma2(sub2(pk2(nibr(pk0, 0), nibr(pk1, 0)), bias2), L2, dx2);
      const f2 y = fma2(sub2(pk2(nibr(pk0, 4), nibr(pk1, 4)), bias2), L2, dy2);
      const f2 z = fma2(sub2(pk2(nibr(pk0, 8), nibr(pk1, 8)), bias2), L2, dz2);
      const f2 r2 = fma2(x, x, fma2(y, y, mul2(z, z)));
      float r20, r21;
      up2(r2, r20, r21);
      const bool k0 = hole0 || r20 <= P.cut2, k1 = two && (hole1 || r21 <= P.cut2);
      if (!(k0 || k1)) return;
      const f2 s2 = mul2(a2p, r2);
      float s0, s1;
      up2(s2, s0, s1);
      /* the erfc form (Numerical Recipes erfcc, as erfc_nr) on both halves */
      const f2 dir = pk2(rsqrtf(r20), rsqrtf(r21));
      const f2 dir2 = mul2(dir, dir);
      /* alpha r = alpha r^2 / r, from the reciprocal root already taken */
      float ar0, ar1;
      up2(mul2(alphap, mul2(r2, dir)), ar0, ar1);
      const f2 e = pk2(__expf(-s0), __expf(-s1));
      const f2 av = mul2(kap, mul2(dir2, e));
      const f2 t = pk2(__fdividef(1.0f, fmaf(0.5f, ar0, 1.0f)), __fdividef(1.0f, fmaf(0.5f, ar1, 1.0f)));
      f2 pp = pk2(0.17087277f, 0.17087277f);
      pp = fma2(pp, t, pk2(-0.82215223f, -0.82215223f));
      pp = fma2(pp, t, pk2(1.48851587f, 1.48851587f));
      pp = fma2(pp, t, pk2(-1.13520398f, -1.13520398f));
      pp = fma2(pp, t, pk2(0.27886807f, 0.27886807f));
      pp = fma2(pp, t, pk2(-0.18628806f, -0.18628806f));
      pp = fma2(pp, t, pk2(0.09678418f, 0.09678418f));
      pp = fma2(pp, t, pk2(0.37409196f, 0.37409196f));
      pp = fma2(pp, t, pk2(1.00002368f, 1.00002368f));
      pp = fma2(pp, t, pk2(-1.26551223f, -1.26551223f));
      float p0, p1;
      up2(sub2(pp, s2), p0, p1);
      const f2 ec = mul2(t, pk2(__expf(p0), __expf(p1)));
      f2 g0 = mul2(H ? sub2(ec, pk2(1.f, 1.f)) : ec, dir);
      f2 g1 = fma2(g0, dir2, av);
      f2 g2 = fma2(mul2(pk2(3.f, 3.f), g1), dir2, mul2(twoa2p, av));
      f2 g3 = fma2(mul2(pk2(5.f, 5.f), g2), dir2, mul2(foura4p, av));
      /* hole terms with alpha^2 r^2 < 1: the convergent series instead */
      const bool ser0 = H && s0 < 1.0f, ser1 = H && two && s1 < 1.0f;
      if (H && (ser0 || ser1)) {
        float a0_, a1_, b0_, b1_, c0_, c1_, d0_, d1_;
        up2(g0, a0_, a1_);
        up2(g1, b0_, b1_);
        up2(g2, c0_, c1_);
        up2(g3, d0_, d1_);
        if (ser0) {
          a0_ = -ka * hole_series<0>(s0);
          b0_ = -twoa2 * ka * hole_series<1>(s0);
          c0_ = -foura4 * ka * hole_series<2>(s0);
          d0_ = -foura4 * twoa2 * ka * hole_series<3>(s0);
        }
        if (ser1) {
          a1_ = -ka * hole_series<0>(s1);
          b1_ = -twoa2 * ka * hole_series<1>(s1);
          c1_ = -foura4 * ka * hole_series<2>(s1);
          d1_ = -foura4 * twoa2 * ka * hole_series<3>(s1);
        }
        g0 = pk2(a0_, a1_);
        g1 = pk2(b0_, b1_);
        g2 = pk2(c0_, c1_);
        g3 = pk2(d0_, d1_);
      }
      const f2 keep = pk2(k0 ? 1.f : 0.f, k1 ? 1.f : 0.f);
      g0 = mul2(g0, keep);
      g1 = mul2(g1, keep);
      g2 = mul2(g2, keep);
      g3 = mul2(g3, keep);
      const f2 Q2mirx = fma2(xx, x, fma2(xy, y, mul2(xz, z)));
      const f2 Q2miry = fma2(xy, x, fma2(yy, y, mul2(yz, z)));
      const f2 Q2mirz = fma2(xz, x, fma2(yz, y, mul2(zz, z)));
      const f2 Q2mir =
          mul2(pk2(0.5f, 0.5f), fma2(Q2mirx, x, fma2(Q2miry, y, mul2(Q2mirz, z))));
      const f2 Qta = fma2(g3, Q2mir, sub2(mul2(g1, Mp), mul2(g2, Q2p)));
      fp2 = sub2(fp2, fma2(g2, Q2mir, sub2(mul2(g0, Mp), mul2(g1, Q2p))));
      fx2 = fma2(g2, Q2mirx, sub2(fx2, mul2(x, Qta)));
      fy2 = fma2(g2, Q2miry, sub2(fy2, mul2(y, Qta)));
      fz2 = fma2(g2, Q2mirz, sub2(fz2, mul2(z, Qta)));
    };
    for (int q = 0; q < nhole; q += 2) step(q, nhole, std::true_type{});
    for (int q = nhole; q < count; q += 2) step(q, count, std::false_type{});
    float u0, u1;
    up2(fp2, u0, u1);
    fp += u0 + u1;
    up2(fx2, u0, u1);
    fx += u0 + u1;
    up2(fy2, u0, u1);
    fy += u0 + u1;
    up2(fz2, u0, u1);
    fz += u0 + u1;
  }
  /* k-space: phase = 2 pi (h . d) / L, reduced to one turn */
  const float invL = 1.0f / L;
  const float ux = dx * invL, uy = dy * invL, uz = dz * invL;
  float kx = 0.f, ky = 0.f, kz = 0.f;
  for (int i = 0; i < P.nEwhLoop; ++i) {
    const float4 h = P.h[i];
    float f = fmaf(h.x, ux, fmaf(h.y, uy, h.z * uz));
    f -= rintf(f);
    float sn, cs;
    __sincosf(6.28318530717958647692f * f, &sn, &cs);
    const float hs = P.hs[i];
    fp += h.w * cs + hs * sn;
    const float t = h.w * sn - hs * cs;
    kx = fmaf(h.x, t, kx);
    ky = fmaf(h.y, t, ky);
    kz = fmaf(h.z, t, kz);
  }
  const float tl = P.twopi_over_L;
  double* v = vars + 5 * j;
  v[0] += (double)fx + (double)(tl * kx);
  v[1] += (double)fy + (double)(tl * ky);
  v[2] += (double)fz + (double)(tl * kz);
  v[3] += (double)fp;
}

}  // namespace

cudaError_t launch_ewald_f32(const CompactPartData* parts, VariablePartData* vars,
                             const int* markers, int largephase, int first, int last,
                             const EwaldReadOnlyData& ro, const EwtData* ewt, cudaStream_t s) {
  int n = last - first + 1;
  if (n <= 0) return cudaSuccess;
  EwaldF32Args P;
  P.ro = ro;
  int nh = ro.nEwhLoop < NEWH ? ro.nEwhLoop : NEWH;
  P.ro.nEwhLoop = nh;
  for (int i = 0; i < nh; ++i) P.ewt[i] = ewt[i];
  for (int i = nh; i < NEWH; ++i) P.ewt[i] = EwtData{0, 0, 0, 0, 0};
  int blocks = (n + 127) / 128;
  TimingScope ts(kKidEwaldF32, s);
  ewald_f32_kernel<<<blocks, 128, 0, s>>>(parts, vars, markers, largephase, first, last, P);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ewald_fp(int form, const double* parts, long long n_parts, const int* idx,
                            long long n_idx, const ChangaEwaldParams& p, double* vars,
                            cudaStream_t s, bool hex) {
  if (n_idx <= 0) return cudaSuccess;
  if (p.nEwhLoop < 0 || p.nEwhLoop > CHANGA_MAX_EWH || (p.nEwhLoop > 0 && !p.ewt) || !(p.L > 0) ||
      (hex && !p.momc))
    return cudaErrorInvalidValue;
  const double L = p.L;
  const double alpha = 2.0 / L, alpha2 = alpha * alpha;
  const int nE0 = (int)ceil(p.fEwCut);
  const int nE = nE0 > p.nReps ? nE0 : p.nReps;
  if (form == kF64) {
    EwaldFpArgs P;
    for (int i = 0; i < 12; ++i) P.mom[i] = p.root[i];
    P.L = L;
    P.fEwCut2 = p.fEwCut * p.fEwCut * L * L;
    P.alpha = alpha;
    P.alpha2 = alpha2;
    P.k1 = M_PI / (alpha2 * L * L * L);
    P.ka = 2.0 * alpha / sqrt(M_PI);
    P.nReps = p.nReps;
    P.nEwReps = nE;
    P.nEwhLoop = p.nEwhLoop;
    for (int i = 0; i < p.nEwhLoop; ++i)
      for (int k = 0; k < 5; ++k) P.ewt[i][k] = p.ewt[5 * i + k];
    if (hex) fill_hex_root(p.momc, P.hex);
    int blocks = (int)((n_idx + 127) / 128);
    TimingScope ts(kKidEwaldF64, s);
    if (hex) ewald_f64_kernel<true><<<blocks, 128, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
    else ewald_f64_kernel<false><<<blocks, 128, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
    count_launch();
    return cudaGetLastError();
  }
  if (nE > kMixMaxReps) return cudaErrorInvalidValue;
  EwaldMixArgs P;
  for (int c = 0; c < 3; ++c) P.cm[c] = p.root[3 + c];
  P.M = (float)p.root[2];
  P.xx = (float)p.root[6];
  P.xy = (float)p.root[7];
  P.xz = (float)p.root[8];
  P.yy = (float)p.root[9];
  P.yz = (float)p.root[10];
  P.zz = (float)p.root[11];
  P.Q2 = (float)(0.5 * (p.root[6] + p.root[9] + p.root[11]));
  P.L = (float)L;
  P.alpha2 = (float)alpha2;
  P.ka = (float)(2.0 * alpha / sqrt(M_PI));
  P.cut2 = (float)(p.fEwCut * p.fEwCut * L * L);
  P.k1M = (float)(p.root[2] * M_PI / (alpha2 * L * L * L));
  P.twopi_over_L = (float)(2.0 * M_PI / L);
  P.nReps = p.nReps;
  P.nEwReps = nE;
  /* The terms of h and -h are equal: the cosine coefficient is even in h,
   * the sine coefficient and the phase odd.  The table (EwaldInit's loop
   * over the cube of h) holds both; one of each pair is kept with its
   * coefficients doubled (exact in floating point), which halves the
   * k-space loop.  Entries without an exact mirror are kept as they are. */
  {
    const double f = L / (2.0 * M_PI);
    const int n = p.nEwhLoop;
    std::vector<int> hi(3 * (size_t)n);
    std::vector<char> used((size_t)n, 0);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) hi[3 * i + k] = (int)rint(p.ewt[5 * i + k] * f);
    int m = 0;
    for (int i = 0; i < n; ++i) {
      if (used[i]) continue;
      const double* e = p.ewt + 5 * i;
      double scale = 1.0;
      for (int j = i + 1; j < n; ++j) {
        const double* g = p.ewt + 5 * j;
        if (!used[j] && hi[3 * j] == -hi[3 * i] && hi[3 * j + 1] == -hi[3 * i + 1] &&
            hi[3 * j + 2] == -hi[3 * i + 2] && g[3] == e[3] && g[4] == -e[4]) {
          used[j] = 1;
          scale = 2.0;
          break;
        }
      }
      P.h[m] = make_float4((float)hi[3 * i], (float)hi[3 * i + 1], (float)hi[3 * i + 2],
                           (float)(scale * e[3]));
      P.hs[m] = (float)(scale * e[4]);
      ++m;
    }
    P.nEwhLoop = m;
  }
  if (hex) fill_hex_root(p.momc, P.hex);
  int threads = kMixWarps * 32;
  int blocks = (int)((n_idx + threads - 1) / threads);
  TimingScope ts(kKidEwaldMix, s);
  if (hex) ewald_mix_kernel<true><<<blocks, threads, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
  else ewald_mix_kernel<false><<<blocks, threads, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
  count_launch();
  return cudaGetLastError();
}

namespace {

/* ---- adjoint of the Ewald term (quadrupole build, FP64) ----
 *
 * The forward term of one replica at r (particle - root centre + replica
 * shift) is a = g2 q - r S with q = Q r, S = g1 M - g2 Q2 + g3 w, Q2 = tr Q
 * / 2, w = r.q / 2 (Ewald.cpp:137-240), and the Fourier part adds
 * h' C_h sin(h'.d) with C_h = -g0(h) M - g2(h) h.Q.h / 2 (Ewald.cpp:285-383).
 * With D_n = -(1/r) dg_n/dr (= g_{n+1} on the erfc branch; on the series
 * branch below fInner2 the derivative of its truncated polynomial), the
 * vector-Jacobian product of lam . a is
 *   d/dr:  g2 Q lam - S lam - D2 (lam.q) r - g3 (lam.r) q
 *          + (lam.r)(D1 M - D2 Q2 + D3 w) r,
 *   d/dM:  -g1 (lam.r),
 *   d/dQ_kl (both entries of a symmetric pair):
 *          g2 lam_k r_l + g2 (lam.r) delta_kl / 2 - g3 (lam.r) r_k r_l / 2,
 * and the Fourier part gives (lam.h') C cos(h'.d) h' to d/dr and
 * (lam.h') sin(h'.d) dC/d(M, Q) to the root moments.  The root's centre
 * enters through r = x - cm, so d/dcm is minus the sum of every particle's
 * d/dr.  ewald_vjp_kernel adds each particle's d/dr to its gradient and
 * sums the root-moment gradients; ewald_vjp_chain_kernel carries those to
 * every particle through M = sum m, cm = sum m x / M, Q = sum m (x-cm)(x-cm). */

struct EwaldVjpArgs {
  double mom[12];
  double L, fEwCut2, fInner2, alpha, alpha2, ka;
  int nReps, nEwReps, nEwhLoop;
  double ewt[CHANGA_MAX_EWH][4];  // h' (2 pi / L h) and C_h
  double hg[CHANGA_MAX_EWH][4];   // integer h and -g2(h) / 2 (dC/dQ_kl = -g2 h_k h_l / 2)
  double g0h[CHANGA_MAX_EWH];     // -g0(h) = dC/dM
};

/* acc: 10 sums {dL/dcm (3), dL/dM, dL/dQ xx xy xz yy yz zz (stored, symmetric)} */
__global__ void __launch_bounds__(128) ewald_vjp_kernel(const double* __restrict__ parts,
                                                        long long n_parts,
                                                        const double* __restrict__ lam,
                                                        double* __restrict__ grad,
                                                        double* __restrict__ acc,
                                                        const __grid_constant__ EwaldVjpArgs P) {
  __shared__ double red[10][4];
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double sums[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (j < n_parts) {
    const double* p = parts + 5 * j;
    const double lx = lam[3 * j], ly = lam[3 * j + 1], lz = lam[3 * j + 2];
    const double dxd = p[2] - P.mom[3], dyd = p[3] - P.mom[4], dzd = p[4] - P.mom[5];
    const double M = P.mom[2];
    const double xx = P.mom[6], xy = P.mom[7], xz = P.mom[8], yy = P.mom[9], yz = P.mom[10],
                 zz = P.mom[11];
    const double Q2 = 0.5 * (xx + yy + zz);
    const double qlx = xx * lx + xy * ly + xz * lz, qly = xy * lx + yy * ly + yz * lz,
                 qlz = xz * lx + yz * ly + zz * lz;  // Q lam
    double gx = 0, gy = 0, gz = 0, gM = 0, gxx = 0, gxy = 0, gxz = 0, gyy = 0, gyz = 0, gzz = 0;
    const int nE = P.nEwReps, nR = P.nReps;
    for (int ix = -nE; ix <= nE; ++ix) {
      const bool hx = (ix >= -nR && ix <= nR);
      const double x = dxd + ix * P.L;
      for (int iy = -nE; iy <= nE; ++iy) {
        const bool hxy = hx && (iy >= -nR && iy <= nR);
        const double y = dyd + iy * P.L;
        for (int iz = -nE; iz <= nE; ++iz) {
          const bool hole = hxy && (iz >= -nR && iz <= nR);
          const double z = dzd + iz * P.L;
          const double r2 = x * x + y * y + z * z;
          if (r2 > P.fEwCut2 && !hole) continue;
          double g1, g2, g3, D1, D2, D3;
          if (r2 < P.fInner2) {
            /* the forward's series: g_n = A_n (u / (2n+3) - 1 / (2n+1)),
             * u = alpha^2 r^2, A_{n+1} = 2 alpha^2 A_n */
            const double u = r2 * P.alpha2, a2 = 2 * P.alpha2;
            const double A1 = P.ka * a2, A2 = A1 * a2, A3 = A2 * a2;
            g1 = A1 * ((1.0 / 5.0) * u - (1.0 / 3.0));
            g2 = A2 * ((1.0 / 7.0) * u - (1.0 / 5.0));
            g3 = A3 * ((1.0 / 9.0) * u - (1.0 / 7.0));
            D1 = -A1 * a2 * (1.0 / 5.0);
            D2 = -A2 * a2 * (1.0 / 7.0);
            D3 = -A3 * a2 * (1.0 / 9.0);
          } else {
            const double dir = rsqrt(r2);
            const double dir2 = dir * dir;
            double a = exp(-r2 * P.alpha2);
            a *= P.ka * dir2;
            const double ar = P.alpha * (r2 * dir);
            double g0 = hole ? -erf(ar) : erfc(ar);
            g0 *= dir;
            g1 = g0 * dir2 + a;
            double alphan = 2 * P.alpha2;
            g2 = 3 * g1 * dir2 + alphan * a;
            alphan *= 2 * P.alpha2;
            g3 = 5 * g2 * dir2 + alphan * a;
            alphan *= 2 * P.alpha2;
            const double g4 = 7 * g3 * dir2 + alphan * a;
            D1 = g2;
            D2 = g3;
            D3 = g4;
          }
          const double qx = xx * x + xy * y + xz * z, qy = xy * x + yy * y + yz * z,
                       qz = xz * x + yz * y + zz * z;
          const double w = 0.5 * (qx * x + qy * y + qz * z);
          const double S = g1 * M - g2 * Q2 + g3 * w;
          const double lr = lx * x + ly * y + lz * z, lq = lx * qx + ly * qy + lz * qz;
          const double T = lr * (D1 * M - D2 * Q2 + D3 * w) - D2 * lq;
          gx += g2 * qlx - S * lx - g3 * lr * qx + T * x;
          gy += g2 * qly - S * ly - g3 * lr * qy + T * y;
          gz += g2 * qlz - S * lz - g3 * lr * qz + T * z;
          gM -= g1 * lr;
          const double hd = 0.5 * g2 * lr, h3 = 0.5 * g3 * lr;
          gxx += g2 * lx * x + hd - h3 * x * x;
          gyy += g2 * ly * y + hd - h3 * y * y;
          gzz += g2 * lz * z + hd - h3 * z * z;
          gxy += g2 * (lx * y + ly * x) - g3 * lr * x * y;
          gxz += g2 * (lx * z + lz * x) - g3 * lr * x * z;
          gyz += g2 * (ly * z + lz * y) - g3 * lr * y * z;
        }
      }
    }
    for (int i = 0; i < P.nEwhLoop; ++i) {
      const double* e = P.ewt[i];
      const double hdotx = e[0] * dxd + e[1] * dyd + e[2] * dzd;
      double s, c;
      sincos(hdotx, &s, &c);
      const double lh = lx * e[0] + ly * e[1] + lz * e[2];
      const double t = lh * e[3] * c;
      gx += t * e[0];
      gy += t * e[1];
      gz += t * e[2];
      const double ls = lh * s;
      gM += ls * P.g0h[i];
      const double* h = P.hg[i];
      const double f = ls * h[3];
      gxx += f * h[0] * h[0];
      gyy += f * h[1] * h[1];
      gzz += f * h[2] * h[2];
      gxy += 2 * f * h[0] * h[1];
      gxz += 2 * f * h[0] * h[2];
      gyz += 2 * f * h[1] * h[2];
    }
    double* g = grad + 4 * j;
    g[0] += gx;
    g[1] += gy;
    g[2] += gz;
    const double v[10] = {-gx, -gy, -gz, gM, gxx, gxy, gxz, gyy, gyz, gzz};
#pragma unroll
    for (int k = 0; k < 10; ++k) sums[k] = v[k];
  }
  /* the block's sums, one FP64 atomic per value and block */
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    double v = sums[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    const double v = red[threadIdx.x][0] + red[threadIdx.x][1] + red[threadIdx.x][2] +
                     red[threadIdx.x][3];
    atomicAdd(acc + threadIdx.x, v);
  }
}

/* The root-moment gradients acc to every particle: M = sum m, cm = sum m x
 * / M, Q = sum m (x - cm)(x - cm) (the cm dependence of Q vanishes, as
 * sum m (x - cm) = 0).  With G the symmetric matrix of dL/dQ (diagonal
 * entries, halves of the off-diagonal ones) and e = x - cm:
 *   dL/dx += m / M dL/dcm + 2 m G e,   dL/dm += dL/dM + dL/dcm . e / M + e.G e. */
__global__ void ewald_vjp_chain_kernel(const double* __restrict__ parts, long long n_parts,
                                       const double* __restrict__ acc, double M, double cmx,
                                       double cmy, double cmz, double* __restrict__ grad) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n_parts;
       j += (long long)gridDim.x * blockDim.x) {
    const double* p = parts + 5 * j;
    const double m = p[0], ex = p[2] - cmx, ey = p[3] - cmy, ez = p[4] - cmz;
    const double gcx = acc[0], gcy = acc[1], gcz = acc[2], gM = acc[3];
    const double Gxx = acc[4], Gxy = 0.5 * acc[5], Gxz = 0.5 * acc[6], Gyy = acc[7],
                 Gyz = 0.5 * acc[8], Gzz = acc[9];
    const double Gex = Gxx * ex + Gxy * ey + Gxz * ez, Gey = Gxy * ex + Gyy * ey + Gyz * ez,
                 Gez = Gxz * ex + Gyz * ey + Gzz * ez;
    double* g = grad + 4 * j;
    const double mM = M != 0 ? m / M : 0.0, iM = M != 0 ? 1.0 / M : 0.0;
    g[0] += mM * gcx + 2 * m * Gex;
    g[1] += mM * gcy + 2 * m * Gey;
    g[2] += mM * gcz + 2 * m * Gez;
    g[3] += gM + (gcx * ex + gcy * ey + gcz * ez) * iM + (ex * Gex + ey * Gey + ez * Gez);
  }
}

}  // namespace

cudaError_t launch_ewald_vjp(const double* parts, long long n_parts, const ChangaEwaldParams& p,
                             const double* lam, double* grad, double* acc, cudaStream_t s) {
  if (n_parts <= 0) return cudaSuccess;
  if (p.nEwhLoop < 0 || p.nEwhLoop > CHANGA_MAX_EWH || (p.nEwhLoop > 0 && !p.ewt) || !(p.L > 0))
    return cudaErrorInvalidValue;
  const double L = p.L;
  EwaldVjpArgs P;
  for (int i = 0; i < 12; ++i) P.mom[i] = p.root[i];
  P.L = L;
  P.alpha = 2.0 / L;
  P.alpha2 = P.alpha * P.alpha;
  P.ka = 2.0 * P.alpha / sqrt(M_PI);
  P.fEwCut2 = p.fEwCut * p.fEwCut * L * L;
  P.fInner2 = 1.2e-3 * L * L;  // the FP64 forward's series radius
  P.nReps = p.nReps;
  const int nE0 = (int)ceil(p.fEwCut);
  P.nEwReps = nE0 > p.nReps ? nE0 : p.nReps;
  P.nEwhLoop = p.nEwhLoop;
  const double k4 = M_PI * M_PI / (P.alpha2 * L * L);
  for (int i = 0; i < p.nEwhLoop; ++i) {
    const double* e = p.ewt + 5 * i;
    for (int k = 0; k < 4; ++k) P.ewt[i][k] = e[k];
    /* the integer h and the gammas of the table's row (changa_ewald_table) */
    double h[3], h2 = 0;
    for (int k = 0; k < 3; ++k) {
      h[k] = std::round(e[k] * L / (2 * M_PI));
      h2 += h[k] * h[k];
    }
    const double g0 = h2 > 0 ? std::exp(-k4 * h2) / (M_PI * h2 * L) : 0.0;
    const double g2 = -(2 * M_PI / L) * (2 * M_PI / L) * g0;
    for (int k = 0; k < 3; ++k) P.hg[i][k] = h[k];
    P.hg[i][3] = -0.5 * g2;
    P.g0h[i] = -g0;
  }
  const int blocks = (int)((n_parts + 127) / 128);
  cudaError_t e = cudaMemsetAsync(acc, 0, 10 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  ewald_vjp_kernel<<<blocks, 128, 0, s>>>(parts, n_parts, lam, grad, acc, P);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int cb = blocks < sm_count() * 8 ? blocks : sm_count() * 8;
  ewald_vjp_chain_kernel<<<cb, 128, 0, s>>>(parts, n_parts, acc, p.root[2], p.root[3], p.root[4],
                                            p.root[5], grad);
  count_launch();
  return cudaGetLastError();
}

}  // namespace chg
