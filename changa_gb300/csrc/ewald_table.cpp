/*
 * Host producer of the Ewald Fourier-space table.
 *
 * Restates TreePiece::EwaldInit (Ewald.cpp:285-383, quadrupole build): for
 * every integer h with 0 < |h|^2 <= dEwhCut^2, in hx, hy, hz loop order,
 * the cosine coefficient is QEVAL (Ewald.cpp:48-69) of the root expansion at
 * h with the even gamma factors g0 = exp(-pi^2 |h|^2 / (alpha L)^2) /
 * (pi |h|^2 L), g2 = -(2 pi / L)^2 g0 (alpha = 2/L):
 *     hCfac = -g2 * Qmir(h) - g0 * M,   Qmir(h) = h.Q.h / 2.
 * The sine coefficient is QEVAL with the even gammas zeroed, which leaves
 * nothing in the quadrupole build (it needs odd moments, and the dipole
 * vanishes about the centre of mass): hSfac = 0 exactly, as there.
 * The GPU kernels consume the table; it is built once per force evaluation.
 */
#include <cmath>

#include "changa_gb300.h"

extern "C" int changa_ewald_table(const double* root, double L, double dEwhCut, double* ewt,
                                  int max_h) {
  if (!root || !ewt || !(L > 0) || max_h < 0) return -1;
  const int hReps = (int)std::ceil(dEwhCut);
  const double alpha = 2.0 / L;
  const double k4 = M_PI * M_PI / (alpha * alpha * L * L);
  const double M = root[2];
  const double xx = root[6], xy = root[7], xz = root[8], yy = root[9], yz = root[10], zz = root[11];
  int i = 0;
  for (int hx = -hReps; hx <= hReps; ++hx)
    for (int hy = -hReps; hy <= hReps; ++hy)
      for (int hz = -hReps; hz <= hReps; ++hz) {
        const int h2 = hx * hx + hy * hy + hz * hz;
        if (h2 == 0 || h2 > dEwhCut * dEwhCut) continue;
        if (i >= max_h) return -1;
        const double g0 = std::exp(-k4 * h2) / (M_PI * h2 * L);
        const double g1 = 2 * M_PI / L * g0;
        const double g2 = -2 * M_PI / L * g1;
        const double Qmirx = xz * hz + xy * hy + xx * hx;
        const double Qmiry = yz * hz + xy * hx + yy * hy;
        const double Qmirz = yz * hy + xz * hx + zz * hz;
        const double Qmir = 0.5 * (Qmirx * hx + Qmiry * hy + Qmirz * hz);
        double mfacc = 0.0;
        mfacc -= g2 * Qmir;
        mfacc -= g0 * M;
        ewt[5 * i + 0] = 2 * M_PI / L * hx;
        ewt[5 * i + 1] = 2 * M_PI / L * hy;
        ewt[5 * i + 2] = 2 * M_PI / L * hz;
        ewt[5 * i + 3] = mfacc;
        ewt[5 * i + 4] = 0.0;
        ++i;
      }
  return i;
}

/*
 * The hexadecapole build's table (Ewald.cpp:285-383 with HEXADECAPOLE).
 * EwaldInit first turns the root's scaled reduced moments into complete
 * moments in physical units: each order-k moment times radius^k
 * (momRescaleFmomr, moments.c:238-267), then the trace-determined
 * components filled in (momFmomr2Momc, moments.c:1563-1597).  QEVAL of those
 * complete moments at h splits into the cosine coefficient (even orders,
 * gammas 0, 2, 4) and the sine coefficient (the octupole, gamma 3):
 *     hCfac = -(g0 M + g2 T2[h,h]/2 + g4 T4[h,h,h,h]/24),
 *     hSfac = -g3 T3[h,h,h]/6,
 * with g0 as in the quadrupole table and g_{k+1} = (-1)^(k+1) (2 pi / L) g_k.
 */
namespace {

/* MomcData order: m, xx yy xy xz yz, xxx xyy xxy yyy xxz yyz xyz, xxxx xyyy
 * xxxy yyyy xxxz yyyz xxyy xxyz xyyz, zz, xzz yzz zzz, xxzz xyzz xzzz yyzz
 * yzzz zzzz */
enum {
  cM, cXX, cYY, cXY, cXZ, cYZ, cXXX, cXYY, cXXY, cYYY, cXXZ, cYYZ, cXYZ, cXXXX, cXYYY, cXXXY,
  cYYYY, cXXXZ, cYYYZ, cXXYY, cXXYZ, cXYYZ, cZZ, cXZZ, cYZZ, cZZZ, cXXZZ, cXYZZ, cXZZZ, cYYZZ,
  cYZZZ, cZZZZ, cCount
};

/* root: 27 doubles {radius, soft, M, cm.xyz, xx xy xz yy yz, xxx xyy xxy
 * yyy xxz yyz xyz, xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz} */
void complete_moments(const double* root, double* c) {
  const double r = root[0];
  const double s2 = r * r, s3 = s2 * r, s4 = s3 * r;
  c[cM] = root[2];
  c[cXX] = root[6] * s2;
  c[cXY] = root[7] * s2;
  c[cXZ] = root[8] * s2;
  c[cYY] = root[9] * s2;
  c[cYZ] = root[10] * s2;
  c[cXXX] = root[11] * s3;
  c[cXYY] = root[12] * s3;
  c[cXXY] = root[13] * s3;
  c[cYYY] = root[14] * s3;
  c[cXXZ] = root[15] * s3;
  c[cYYZ] = root[16] * s3;
  c[cXYZ] = root[17] * s3;
  c[cXXXX] = root[18] * s4;
  c[cXYYY] = root[19] * s4;
  c[cXXXY] = root[20] * s4;
  c[cYYYY] = root[21] * s4;
  c[cXXXZ] = root[22] * s4;
  c[cYYYZ] = root[23] * s4;
  c[cXXYY] = root[24] * s4;
  c[cXXYZ] = root[25] * s4;
  c[cXYYZ] = root[26] * s4;
  /* trace-free: every trace vanishes */
  c[cZZ] = -(c[cXX] + c[cYY]);
  c[cXZZ] = -(c[cXXX] + c[cXYY]);
  c[cYZZ] = -(c[cXXY] + c[cYYY]);
  c[cZZZ] = -(c[cXXZ] + c[cYYZ]);
  c[cXXZZ] = -(c[cXXXX] + c[cXXYY]);
  c[cXYZZ] = -(c[cXXXY] + c[cXYYY]);
  c[cXZZZ] = -(c[cXXXZ] + c[cXYYZ]);
  c[cYYZZ] = -(c[cXXYY] + c[cYYYY]);
  c[cYZZZ] = -(c[cXXYZ] + c[cYYYZ]);
  c[cZZZZ] = -(c[cXXZZ] + c[cYYZZ]);
}

/* full contractions of the complete moments with h: T2[h,h], T3[h,h,h],
 * T4[h,h,h,h] */
void contractions(const double* c, double x, double y, double z, double& t2, double& t3,
                  double& t4) {
  t2 = c[cXX] * x * x + c[cYY] * y * y + c[cZZ] * z * z +
       2.0 * (c[cXY] * x * y + c[cXZ] * x * z + c[cYZ] * y * z);
  t3 = c[cXXX] * x * x * x + c[cYYY] * y * y * y + c[cZZZ] * z * z * z +
       3.0 * (c[cXXY] * x * x * y + c[cXXZ] * x * x * z + c[cXYY] * x * y * y +
              c[cYYZ] * y * y * z + c[cXZZ] * x * z * z + c[cYZZ] * y * z * z) +
       6.0 * c[cXYZ] * x * y * z;
  t4 = c[cXXXX] * x * x * x * x + c[cYYYY] * y * y * y * y + c[cZZZZ] * z * z * z * z +
       4.0 * (c[cXXXY] * x * x * x * y + c[cXXXZ] * x * x * x * z + c[cXYYY] * x * y * y * y +
              c[cYYYZ] * y * y * y * z + c[cXZZZ] * x * z * z * z + c[cYZZZ] * y * z * z * z) +
       6.0 * (c[cXXYY] * x * x * y * y + c[cXXZZ] * x * x * z * z + c[cYYZZ] * y * y * z * z) +
       12.0 * (c[cXXYZ] * x * x * y * z + c[cXYYZ] * x * y * y * z + c[cXYZZ] * x * y * z * z);
}

}  // namespace

extern "C" int changa_ewald_table_hex(const double* root, double L, double dEwhCut, double* ewt,
                                      int max_h, double* momc) {
  if (!root || !ewt || !(L > 0) || max_h < 0) return -1;
  double c[cCount];
  complete_moments(root, c);
  if (momc)
    for (int k = 0; k < cCount; ++k) momc[k] = c[k];
  const int hReps = (int)std::ceil(dEwhCut);
  const double alpha = 2.0 / L;
  const double k4 = M_PI * M_PI / (alpha * alpha * L * L);
  const double w = 2 * M_PI / L;
  int i = 0;
  for (int hx = -hReps; hx <= hReps; ++hx)
    for (int hy = -hReps; hy <= hReps; ++hy)
      for (int hz = -hReps; hz <= hReps; ++hz) {
        const int h2 = hx * hx + hy * hy + hz * hz;
        if (h2 == 0 || h2 > dEwhCut * dEwhCut) continue;
        if (i >= max_h) return -1;
        const double g0 = std::exp(-k4 * h2) / (M_PI * h2 * L);
        const double g1 = w * g0, g2 = -w * g1, g3 = w * g2, g4 = -w * g3;
        double t2, t3, t4;
        contractions(c, hx, hy, hz, t2, t3, t4);
        ewt[5 * i + 0] = w * hx;
        ewt[5 * i + 1] = w * hy;
        ewt[5 * i + 2] = w * hz;
        ewt[5 * i + 3] = -(g0 * c[cM] + g2 * t2 / 2.0 + g4 * t4 / 24.0);
        ewt[5 * i + 4] = -(g3 * t3 / 6.0);
        ++i;
      }
  return i;
}
