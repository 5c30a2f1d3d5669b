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
 *   ewald_f32_kernel  the drop-in form on the FP32 ABI (reference constants,
 *                     including its single-precision fInner2 = 1.1e-2 L^2);
 *   kF64              all FP64 with the CPU constants (fInner2 = 1.2e-3 L^2);
 *   kMix              FP32 everywhere except the terms with r^2 < 0.05 L^2
 *                     (only the central replica can get there), which are
 *                     evaluated in FP64 where the hole's -erf and the 1/r^k
 *                     terms cancel.  d = x - cm is formed in FP64 and
 *                     rounded once, so it is accurate to FP32 rounding of d.
 */
#include "chg_internal.h"

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
  const float Q2 = 0.5f * (mom.xx + mom.yy + mom.zz);
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
        }
        const float Q2mirx = mom.xx * x + mom.xy * y + mom.xz * z;
        const float Q2miry = mom.xy * x + mom.yy * y + mom.yz * z;
        const float Q2mirz = mom.xz * x + mom.yz * y + mom.zz * z;
        const float Q2mir = 0.5f * (Q2mirx * x + Q2miry * y + Q2mirz * z);
        const float Qta = g1 * mom.totalMass - g2 * Q2 + g3 * Q2mir;
        fPot -= g0 * mom.totalMass - g1 * Q2 + g2 * Q2mir;
        ax += g2 * Q2mirx - x * Qta;
        ay += g2 * Q2miry - y * Qta;
        az += g2 * Q2mirz - z * Qta;
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

struct EwaldFpArgs {
  double mom[12];
  double L, fEwCut2, alpha, alpha2, k1, ka;
  int nReps, nEwReps, nEwhLoop;
  double ewt[CHANGA_MAX_EWH][5];
};

/* FP64 real-space term (Ewald.cpp:137-196, quadrupole). */
__device__ __forceinline__ void ewald_term_f64(const EwaldFpArgs& P, double x, double y, double z,
                                               bool hole, double fInner2, double& fPot,
                                               double& ax, double& ay, double& az) {
  const double* mom = P.mom;
  double r2 = x * x + y * y + z * z;
  double g0, g1, g2, g3;
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

constexpr double kMixInner = 0.05;  // FP64 below r^2 < 0.05 L^2 in the mixed form

template <int FORM>
__global__ void __launch_bounds__(128) ewald_fp_kernel(const double* __restrict__ parts,
                                                       long long n_parts,
                                                       const int* __restrict__ idx, long long n_idx,
                                                       double* __restrict__ vars,
                                                       const __grid_constant__ EwaldFpArgs P) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= n_idx) return;
  const long long j = idx ? (long long)idx[k] : k;
  if (j < 0 || j >= n_parts) return;
  const double* p = parts + 5 * j;
  const double dxd = p[2] - P.mom[3], dyd = p[3] - P.mom[4], dzd = p[4] - P.mom[5];
  const int nE = P.nEwReps, nR = P.nReps;
  double fPot = P.mom[2] * P.k1, ax = 0, ay = 0, az = 0;
  if constexpr (FORM == kF64) {
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
          ewald_term_f64(P, x, y, z, hole, fInner2, fPot, ax, ay, az);
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
  } else {
    const float L = (float)P.L, alpha = (float)P.alpha, alpha2 = (float)P.alpha2;
    const float ka = (float)P.ka, cut2 = (float)P.fEwCut2;
    const float inner2 = (float)(kMixInner * P.L * P.L);
    const float M = (float)P.mom[2];
    const float mxx = (float)P.mom[6], mxy = (float)P.mom[7], mxz = (float)P.mom[8];
    const float myy = (float)P.mom[9], myz = (float)P.mom[10], mzz = (float)P.mom[11];
    const float Q2 = 0.5f * (mxx + myy + mzz);
    const float dx = (float)dxd, dy = (float)dyd, dz = (float)dzd;
    float fx = 0.f, fy = 0.f, fz = 0.f, fp = 0.f;
    for (int ix = -nE; ix <= nE; ++ix) {
      const bool hx = (ix >= -nR && ix <= nR);
      const float x = dx + ix * L;
      for (int iy = -nE; iy <= nE; ++iy) {
        const bool hxy = hx && (iy >= -nR && iy <= nR);
        const float y = dy + iy * L;
        for (int iz = -nE; iz <= nE; ++iz) {
          const bool hole = hxy && (iz >= -nR && iz <= nR);
          const float z = dz + iz * L;
          const float r2 = x * x + y * y + z * z;
          if (r2 > cut2 && !hole) continue;
          if (r2 < inner2) {
            ewald_term_f64(P, dxd + ix * P.L, dyd + iy * P.L, dzd + iz * P.L, hole,
                           1.2e-3 * P.L * P.L, fPot, ax, ay, az);
            continue;
          }
          const float dir = rsqrtf(r2);
          const float dir2 = dir * dir;
          const float a = expf(-r2 * alpha2) * (ka * dir2);
          const float ar = alpha * (r2 * dir);
          float g0 = hole ? -erff(ar) : erfcf(ar);
          g0 *= dir;
          const float g1 = g0 * dir2 + a;
          const float g2 = 3.f * g1 * dir2 + (2.f * alpha2) * a;
          const float g3 = 5.f * g2 * dir2 + (4.f * alpha2 * alpha2) * a;
          const float Q2mirx = mxx * x + mxy * y + mxz * z;
          const float Q2miry = mxy * x + myy * y + myz * z;
          const float Q2mirz = mxz * x + myz * y + mzz * z;
          const float Q2mir = 0.5f * (Q2mirx * x + Q2miry * y + Q2mirz * z);
          const float Qta = g1 * M - g2 * Q2 + g3 * Q2mir;
          fp -= g0 * M - g1 * Q2 + g2 * Q2mir;
          fx += g2 * Q2mirx - x * Qta;
          fy += g2 * Q2miry - y * Qta;
          fz += g2 * Q2mirz - z * Qta;
        }
      }
    }
    for (int i = 0; i < P.nEwhLoop; ++i) {
      const double* e = P.ewt[i];
      const float hx = (float)e[0], hy = (float)e[1], hz = (float)e[2];
      const float hc = (float)e[3], hs = (float)e[4];
      const float hdotx = hx * dx + hy * dy + hz * dz;
      float s, c;
      sincosf(hdotx, &s, &c);
      fp += hc * c + hs * s;
      const float t = hc * s - hs * c;
      fx += hx * t;
      fy += hy * t;
      fz += hz * t;
    }
    fPot += fp;
    ax += fx;
    ay += fy;
    az += fz;
  }
  double* v = vars + 5 * j;
  v[0] += ax;
  v[1] += ay;
  v[2] += az;
  v[3] += fPot;
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
  ewald_f32_kernel<<<blocks, 128, 0, s>>>(parts, vars, markers, largephase, first, last, P);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ewald_fp(int form, const double* parts, long long n_parts, const int* idx,
                            long long n_idx, const ChangaEwaldParams& p, double* vars,
                            cudaStream_t s) {
  if (n_idx <= 0) return cudaSuccess;
  if (p.nEwhLoop < 0 || p.nEwhLoop > CHANGA_MAX_EWH || (p.nEwhLoop > 0 && !p.ewt))
    return cudaErrorInvalidValue;
  EwaldFpArgs P;
  for (int i = 0; i < 12; ++i) P.mom[i] = p.root[i];
  const double L = p.L;
  P.L = L;
  P.fEwCut2 = p.fEwCut * p.fEwCut * L * L;
  P.alpha = 2.0 / L;
  P.alpha2 = P.alpha * P.alpha;
  P.k1 = M_PI / (P.alpha2 * L * L * L);
  P.ka = 2.0 * P.alpha / sqrt(M_PI);
  P.nReps = p.nReps;
  int nE = (int)ceil(p.fEwCut);
  P.nEwReps = nE > p.nReps ? nE : p.nReps;
  P.nEwhLoop = p.nEwhLoop;
  for (int i = 0; i < p.nEwhLoop; ++i)
    for (int k = 0; k < 5; ++k) P.ewt[i][k] = p.ewt[5 * i + k];
  int blocks = (int)((n_idx + 127) / 128);
  if (form == kF64)
    ewald_fp_kernel<kF64><<<blocks, 128, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
  else
    ewald_fp_kernel<kMix><<<blocks, 128, 0, s>>>(parts, n_parts, idx, n_idx, vars, P);
  count_launch();
  return cudaGetLastError();
}

}  // namespace chg
