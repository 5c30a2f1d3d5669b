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
