/*
 * Plain-C restatement of ChaNGa's CPU gravity force path (quadrupole build).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle on machines without the
 * reference sources and the timed CPU baseline ("port").  It is pinned
 * against ChaNGa's own gravity.h / Ewald.cpp (oracle/_ref) and against the
 * committed fixtures in tests/golden.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it; the product never does.
 *
 * Every routine states the reference lines it follows.  Arithmetic order is
 * kept where it affects rounding; all arithmetic is FP64 (cosmoType=double,
 * cosmoType.h:6-14).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_api.h"

/* SPLINEQ, gravity.h:22-66 (Hernquist & Katz 1989 A1/A2 with Stadel's
 * higher-derivative terms c, d for quadrupole spline softening). */
static inline void splineq(double invr, double r2, double twoh,
                           double* a, double* b, double* c, double* d) {
  double u, dih, dir = invr;
  if (r2 < twoh * twoh) {
    dih = 2.0 / twoh;
    u = dih / dir;
    if (u < 1.0) {
      *a = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                  - 1.0 / 10.0 * u * u * u * u * u);
      *b = dih * dih * dih * (4.0 / 3.0 - 6.0 / 5.0 * u * u + 1.0 / 2.0 * u * u * u);
      *c = dih * dih * dih * dih * dih * (12.0 / 5.0 - 3.0 / 2.0 * u);
      *d = 3.0 / 2.0 * dih * dih * dih * dih * dih * dih * dir;
    } else {
      *a = -1.0 / 15.0 * dir
           + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                    - 3.0 / 10.0 * u * u * u * u + 1.0 / 30.0 * u * u * u * u * u);
      *b = -1.0 / 15.0 * dir * dir * dir
           + dih * dih * dih * (8.0 / 3.0 - 3.0 * u + 6.0 / 5.0 * u * u - 1.0 / 6.0 * u * u * u);
      *c = -1.0 / 5.0 * dir * dir * dir * dir * dir + 3.0 * dih * dih * dih * dih * dir
           + dih * dih * dih * dih * dih * (-12.0 / 5.0 + 1.0 / 2.0 * u);
      *d = -dir * dir * dir * dir * dir * dir * dir
           + 3.0 * dih * dih * dih * dih * dir * dir * dir
           - 1.0 / 2.0 * dih * dih * dih * dih * dih * dih * dir;
    }
  } else {
    *a = dir;
    *b = (*a) * (*a) * (*a);
    *c = 3.0 * (*b) * (*a) * (*a);
    *d = 5.0 * (*c) * (*a) * (*a);
  }
}

/* SPLINE, gravity.h:147-182 (compact-support cubic spline for P-P). */
static inline void spline(double r2, double twoh, double* a, double* b) {
  double r, u, dih, dir;
  r = sqrt(r2);
  if (r < twoh) {
    dih = 2.0 / twoh;
    u = r * dih;
    if (u < 1.0) {
      *a = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                  - 1.0 / 10.0 * u * u * u * u * u);
      *b = dih * dih * dih * (4.0 / 3.0 - 6.0 / 5.0 * u * u + 1.0 / 2.0 * u * u * u);
    } else {
      dir = 1.0 / r;
      *a = -1.0 / 15.0 * dir
           + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                    - 3.0 / 10.0 * u * u * u * u + 1.0 / 30.0 * u * u * u * u * u);
      *b = -1.0 / 15.0 * dir * dir * dir
           + dih * dih * dih * (8.0 / 3.0 - 3.0 * u + 6.0 / 5.0 * u * u - 1.0 / 6.0 * u * u * u);
    }
  } else {
    *a = 1.0 / r;
    *b = (*a) * (*a) * (*a);
  }
}

/* TreePiece::decodeOffset, ParallelGravity.h:2064-2073 (cubic period). */
static inline void decode_offset(int offsetID, double fperiod, double off[3]) {
  int code = offsetID >> 22;
  off[0] = ((code & 0x7) - 3) * fperiod;
  off[1] = (((code >> 3) & 0x7) - 3) * fperiod;
  off[2] = (((code >> 6) & 0x7) - 3) * fperiod;
}

/* nodeBucketForce (quadrupole), gravity.h:398-475, for one cell and the
 * targets [s, s+n).  The CPU reference has no rsq == 0 guard; the cell lists
 * never hold a node whose centre of mass coincides with a target (nodes of
 * <= 6 particles are always opened, gravity.h:659-663). */
static void node_bucket_force(const double* m, const double* off, const double* parts,
                              double* vars, int s, int n) {
  double cm0 = m[3] + off[0], cm1 = m[4] + off[1], cm2 = m[5] + off[2];
  double mass = m[2], msoft = m[1];
  double xx = m[6], xy = m[7], xz = m[8], yy = m[9], yz = m[10], zz = m[11];
  for (int j = s; j < s + n; ++j) {
    const double* p = parts + 5 * (size_t)j;
    double* v = vars + 5 * (size_t)j;
    double rx = p[2] - cm0, ry = p[3] - cm1, rz = p[4] - cm2;
    double rsq = rx * rx + ry * ry + rz * rz;
    double dir = 1.0 / sqrt(rsq);
    double twoh = msoft + p[1];
    double a, b, c, d;
    splineq(dir, rsq, twoh, &a, &b, &c, &d);
    double qirx = xx * rx + xy * ry + xz * rz;
    double qiry = xy * rx + yy * ry + yz * rz;
    double qirz = xz * rx + yz * ry + zz * rz;
    double qir = 0.5 * (qirx * rx + qiry * ry + qirz * rz);
    double tr = 0.5 * (xx + yy + zz);
    double qir3 = b * mass + d * qir - c * tr;
    v[3] -= mass * a + c * qir - b * tr;
    v[0] -= qir3 * rx - c * qirx;
    v[1] -= qir3 * ry - c * qiry;
    v[2] -= qir3 * rz - c * qirz;
    double idt2 = (p[0] + mass) * b;
    if (idt2 > v[4]) v[4] = idt2;
  }
}

/* partBucketForce, gravity.h:267-303, for one source particle. */
static void part_bucket_force(const double* src, const double* off, const double* tgts,
                              double* vars, int s, int n) {
  for (int j = s; j < s + n; ++j) {
    const double* p = tgts + 5 * (size_t)j;
    double* v = vars + 5 * (size_t)j;
    double rx = off[0] + src[2] - p[2];
    double ry = off[1] + src[3] - p[3];
    double rz = off[2] + src[4] - p[4];
    double rsq = rx * rx + ry * ry + rz * rz;
    double twoh = src[1] + p[1];
    if (rsq != 0) {
      double a, b;
      spline(rsq, twoh, &a, &b);
      double idt2 = (p[0] + src[0]) * b;
      double bm = b * src[0];
      v[0] += rx * bm;
      v[1] += ry * bm;
      v[2] += rz * bm;
      v[3] -= src[0] * a;
      if (idt2 > v[4]) v[4] = idt2;
    }
  }
}

int oracle_cell_list_forces(const double* moments, long n_moments,
                            const double* parts, long n_parts,
                            const int* list, const int* markers,
                            const int* starts, const int* sizes, int n_buckets,
                            const int* bucket_ids, int n_ids,
                            double fperiod, double* vars, int nthreads) {
  (void)n_parts;
  int nwork = bucket_ids ? n_ids : n_buckets;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int w = 0; w < nwork; ++w) {
    int b = bucket_ids ? bucket_ids[w] : w;
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_moments) continue;
      double off[3];
      decode_offset(list[2 * (size_t)e + 1], fperiod, off);
      node_bucket_force(moments + 12 * (size_t)idx, off, parts, vars, starts[b], sizes[b]);
    }
  }
  return 0;
}

int oracle_part_list_forces(const double* sources, long n_sources,
                            const double* targets, long n_targets,
                            const int* list, const int* markers,
                            const int* starts, const int* sizes, int n_buckets,
                            const int* bucket_ids, int n_ids,
                            double fperiod, double* vars, int nthreads) {
  (void)n_targets;
  int nwork = bucket_ids ? n_ids : n_buckets;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int w = 0; w < nwork; ++w) {
    int b = bucket_ids ? bucket_ids[w] : w;
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_sources) continue;
      double off[3];
      decode_offset(list[2 * (size_t)e + 1], fperiod, off);
      part_bucket_force(sources + 5 * (size_t)idx, off, targets, vars, starts[b], sizes[b]);
    }
  }
  return 0;
}

/* ---- hexadecapole build ---- */

/* momEvalFmomrcm, moments.c:1469-1525: the scaled reduced moments mo[6..26]
 * of a cell with radius mo[0] and mass mo[2], evaluated at r = target - cm,
 * dir = 1/|r|; the same expressions in the same order, so the FP64 results
 * are those of the reference. */
static void hex_eval(const double* mo, double dir, double x, double y, double z, double* v) {
  /* the reference's constant is the single-precision 1/3 (1.0f / 3.0f),
   * promoted: kept so the FP64 results are bit-identical */
  const double onethird = (double)(1.0f / 3.0f);
  const double mxx = mo[6], mxy = mo[7], mxz = mo[8], myy = mo[9], myz = mo[10];
  const double mxxx = mo[11], mxyy = mo[12], mxxy = mo[13], myyy = mo[14], mxxz = mo[15],
               myyz = mo[16], mxyz = mo[17];
  const double mxxxx = mo[18], mxyyy = mo[19], mxxxy = mo[20], myyyy = mo[21], mxxxz = mo[22],
               myyyz = mo[23], mxxyy = mo[24], mxxyz = mo[25], mxyyz = mo[26];
  double u = mo[0];
  u *= dir;
  double g0 = dir;
  double g2 = 3 * dir * u * u;
  double g3 = 5 * g2 * u;
  double g4 = 7 * g3 * u;
  x *= dir;
  y *= dir;
  z *= dir;
  double xx = 0.5 * x * x;
  double xy = x * y;
  double xz = x * z;
  double yy = 0.5 * y * y;
  double yz = y * z;
  double zz = 0.5 * z * z;
  double xxx = x * (onethird * xx - zz);
  double xxz = z * (xx - onethird * zz);
  double yyy = y * (onethird * yy - zz);
  double yyz = z * (yy - onethird * zz);
  xx -= zz;
  yy -= zz;
  double xxy = y * xx;
  double xyy = x * yy;
  double xyz = xy * z;
  double tx = g4 * (mxxxx * xxx + mxyyy * yyy + mxxxy * xxy + mxxxz * xxz + mxxyy * xyy +
                    mxxyz * xyz + mxyyz * yyz);
  double ty = g4 * (mxyyy * xyy + mxxxy * xxx + myyyy * yyy + myyyz * yyz + mxxyy * xxy +
                    mxxyz * xxz + mxyyz * xyz);
  double tz = g4 * (-mxxxx * xxz - (mxyyy + mxxxy) * xyz - myyyy * yyz + mxxxz * xxx +
                    myyyz * yyy - mxxyy * (xxz + yyz) + mxxyz * xxy + mxyyz * xyy);
  g4 = 0.25 * (tx * x + ty * y + tz * z);
  xxx = g3 * (mxxx * xx + mxyy * yy + mxxy * xy + mxxz * xz + mxyz * yz);
  xxy = g3 * (mxyy * xy + mxxy * xx + myyy * yy + myyz * yz + mxyz * xz);
  xxz = g3 * (-(mxxx + mxyy) * xz - (mxxy + myyy) * yz + mxxz * xx + myyz * yy + mxyz * xy);
  g3 = onethird * (xxx * x + xxy * y + xxz * z);
  xx = g2 * (mxx * x + mxy * y + mxz * z);
  xy = g2 * (myy * y + mxy * x + myz * z);
  xz = g2 * (-(mxx + myy) * z + mxz * x + myz * y);
  g2 = 0.5 * (xx * x + xy * y + xz * z);
  g0 *= mo[2];
  v[3] += -(g0 + g2 + g3 + g4);
  g0 += 5 * g2 + 7 * g3 + 9 * g4;
  v[0] += dir * (xx + xxx + tx - x * g0);
  v[1] += dir * (xy + xxy + ty - y * g0);
  v[2] += dir * (xz + xxz + tz - z * g0);
}

/* openSoftening, gravity.h:252-260 (closed balls, as the walk uses):
 * geom = {bucket cm.xyz, bucket soft, bbox lesser xyz, greater xyz}. */
static int open_softening(const double* mo, const double* off, const double* geom) {
  const double c0 = mo[3] + off[0], c1 = mo[4] + off[1], c2 = mo[5] + off[2];
  const double r = 2.0 * mo[1];
  double dx = geom[0] - c0, dy = geom[1] - c1, dz = geom[2] - c2;
  const double rr = 2.0 * geom[3] + r;
  if (dx * dx + dy * dy + dz * dz <= rr * rr) return 1;
  double d2 = 0.0, d;
  if ((d = geom[4] - c0) > 0) d2 += d * d;
  else if ((d = c0 - geom[7]) > 0) d2 += d * d;
  if ((d = geom[5] - c1) > 0) d2 += d * d;
  else if ((d = c1 - geom[8]) > 0) d2 += d * d;
  if ((d = geom[6] - c2) > 0) d2 += d * d;
  else if ((d = c2 - geom[9]) > 0) d2 += d * d;
  return d2 <= r * r;
}

/* nodeBucketForce with HEXADECAPOLE, gravity.h:398-421, 439-446. */
static void node_bucket_force_hex(const double* mo, const double* off, const double* geom,
                                  const double* parts, double* vars, int s, int n) {
  if (open_softening(mo, off, geom)) {
    const double src[5] = {mo[2], mo[1], mo[3], mo[4], mo[5]};
    part_bucket_force(src, off, parts, vars, s, n);
    return;
  }
  const double cm0 = mo[3] + off[0], cm1 = mo[4] + off[1], cm2 = mo[5] + off[2];
  for (int j = s; j < s + n; ++j) {
    const double* p = parts + 5 * (size_t)j;
    double* v = vars + 5 * (size_t)j;
    const double rx = p[2] - cm0, ry = p[3] - cm1, rz = p[4] - cm2;
    const double rsq = rx * rx + ry * ry + rz * rz;
    const double dir = 1.0 / sqrt(rsq);
    hex_eval(mo, dir, rx, ry, rz, v);
    const double idt2 = (p[0] + mo[2]) * dir * dir * dir;
    if (idt2 > v[4]) v[4] = idt2;
  }
}

int oracle_cell_list_forces_hex(const double* moments, long n_moments, const double* parts,
                                long n_parts, const int* list, const int* markers,
                                const int* starts, const int* sizes, int n_buckets,
                                const double* geom, double fperiod, double* vars, int nthreads) {
  (void)n_parts;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int b = 0; b < n_buckets; ++b) {
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      const int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_moments) continue;
      double off[3];
      decode_offset(list[2 * (size_t)e + 1], fperiod, off);
      node_bucket_force_hex(moments + 27 * (size_t)idx, off, geom + 10 * (size_t)b, parts, vars,
                            starts[b], sizes[b]);
    }
  }
  return 0;
}

/* QEVAL (quadrupole), Ewald.cpp:48-69: evaluates the root expansion with
 * the gamma factors gam[0..3] at (dx, dy, dz). */
static void qeval(const double* mom, const double gam[6], double dx, double dy, double dz,
                  double* ax, double* ay, double* az, double* fPot) {
  double xx = mom[6], xy = mom[7], xz = mom[8], yy = mom[9], yz = mom[10], zz = mom[11];
  double Qmirx, Qmiry, Qmirz, Qmir, Qta = 0.0;
  Qmirx = xz * dz + xy * dy + xx * dx;
  Qmiry = yz * dz + xy * dx + yy * dy;
  Qmirz = yz * dy + xz * dx + zz * dz;
  Qmir = 0.5 * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
  *fPot -= gam[2] * Qmir;
  Qta += gam[3] * Qmir;
  *ax += gam[2] * Qmirx;
  *ay += gam[2] * Qmiry;
  *az += gam[2] * Qmirz;
  *fPot -= gam[0] * mom[2];
  Qta += gam[1] * mom[2];
  *ax -= dx * Qta;
  *ay -= dy * Qta;
  *az -= dz * Qta;
}

/* TreePiece::EwaldInit h-table, Ewald.cpp:285-383 (quadrupole). */
int oracle_ewald_table(const double* root, double L, double dEwhCut, double* ewt, int max_h) {
  int hReps = (int)ceil(dEwhCut);
  double alpha = 2.0 / L;
  double k4 = M_PI * M_PI / (alpha * alpha * L * L);
  int i = 0;
  for (int hx = -hReps; hx <= hReps; ++hx)
    for (int hy = -hReps; hy <= hReps; ++hy)
      for (int hz = -hReps; hz <= hReps; ++hz) {
        int h2 = hx * hx + hy * hy + hz * hz;
        if (h2 == 0) continue;
        if (h2 > dEwhCut * dEwhCut) continue;
        if (i >= max_h) return -1;
        double gam[6], ax = 0, ay = 0, az = 0, mfacc = 0.0, mfacs = 0.0;
        gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
        gam[1] = 2 * M_PI / L * gam[0];
        gam[2] = -2 * M_PI / L * gam[1];
        gam[3] = 2 * M_PI / L * gam[2];
        gam[4] = -2 * M_PI / L * gam[3];
        gam[5] = 2 * M_PI / L * gam[4];
        gam[1] = 0.0; gam[3] = 0.0; gam[5] = 0.0;
        qeval(root, gam, hx, hy, hz, &ax, &ay, &az, &mfacc);
        gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
        gam[1] = 2 * M_PI / L * gam[0];
        gam[2] = -2 * M_PI / L * gam[1];
        gam[3] = 2 * M_PI / L * gam[2];
        gam[4] = -2 * M_PI / L * gam[3];
        gam[5] = 2 * M_PI / L * gam[4];
        gam[0] = 0.0; gam[2] = 0.0; gam[4] = 0.0;
        ax = ay = az = 0.0;
        qeval(root, gam, hx, hy, hz, &ax, &ay, &az, &mfacs);
        ewt[5 * i + 0] = 2 * M_PI / L * hx;
        ewt[5 * i + 1] = 2 * M_PI / L * hy;
        ewt[5 * i + 2] = 2 * M_PI / L * hz;
        ewt[5 * i + 3] = mfacc;
        ewt[5 * i + 4] = mfacs;
        ++i;
      }
  return i;
}

/* TreePiece::BucketEwald (quadrupole), Ewald.cpp:72-281, for one particle:
 * real-space sum over replicas |i| <= nEwReps with the erf "hole" for
 * |i| <= nReps, the series expansion inside fInner2, then the h-loop. */
static void ewald_one(const double* p, const double* mom, double L, int nReps, double fEwCut,
                      const double* ewt, int nEwhLoop, double* v) {
  double Q2 = 0.5 * (mom[6] + mom[9] + mom[11]);
  double M = mom[2];
  int nEwReps = (int)ceil(fEwCut);
  double fEwCut2 = fEwCut * fEwCut * L * L;
  double fInner2 = 1.2e-3 * L * L;
  if (nReps > nEwReps) nEwReps = nReps;
  double alpha = 2.0 / L;
  double alpha2 = alpha * alpha;
  double k1 = M_PI / (alpha2 * L * L * L);
  double ka = 2.0 * alpha / sqrt(M_PI);
  double fPot = M * k1, ax = 0.0, ay = 0.0, az = 0.0;
  double dx = p[2] - mom[3], dy = p[3] - mom[4], dz = p[4] - mom[5];
  for (int ix = -nEwReps; ix <= nEwReps; ++ix) {
    int bInHolex = (ix >= -nReps && ix <= nReps);
    double x = dx + ix * L;
    for (int iy = -nEwReps; iy <= nEwReps; ++iy) {
      int bInHolexy = (bInHolex && iy >= -nReps && iy <= nReps);
      double y = dy + iy * L;
      for (int iz = -nEwReps; iz <= nEwReps; ++iz) {
        int bInHole = (bInHolexy && iz >= -nReps && iz <= nReps);
        double z = dz + iz * L;
        double r2 = x * x + y * y + z * z;
        if (r2 > fEwCut2 && !bInHole) continue;
        double g0, g1, g2, g3, alphan;
        if (r2 < fInner2) {
          alphan = ka;
          r2 *= alpha2;
          g0 = alphan * ((1.0 / 3.0) * r2 - 1.0);
          alphan *= 2 * alpha2;
          g1 = alphan * ((1.0 / 5.0) * r2 - (1.0 / 3.0));
          alphan *= 2 * alpha2;
          g2 = alphan * ((1.0 / 7.0) * r2 - (1.0 / 5.0));
          alphan *= 2 * alpha2;
          g3 = alphan * ((1.0 / 9.0) * r2 - (1.0 / 7.0));
        } else {
          double dir = 1 / sqrt(r2);
          double dir2 = dir * dir;
          double a = exp(-r2 * alpha2);
          a *= ka * dir2;
          if (bInHole) g0 = -erf(alpha / dir);
          else g0 = erfc(alpha / dir);
          g0 *= dir;
          g1 = g0 * dir2 + a;
          alphan = 2 * alpha2;
          g2 = 3 * g1 * dir2 + alphan * a;
          alphan *= 2 * alpha2;
          g3 = 5 * g2 * dir2 + alphan * a;
        }
        double Q2mirx = mom[6] * x + mom[7] * y + mom[8] * z;
        double Q2miry = mom[7] * x + mom[9] * y + mom[10] * z;
        double Q2mirz = mom[8] * x + mom[10] * y + mom[11] * z;
        double Q2mir = 0.5 * (Q2mirx * x + Q2miry * y + Q2mirz * z);
        double Qta = g1 * M - g2 * Q2 + g3 * Q2mir;
        fPot -= g0 * M - g1 * Q2 + g2 * Q2mir;
        ax += g2 * (Q2mirx) - x * Qta;
        ay += g2 * (Q2miry) - y * Qta;
        az += g2 * (Q2mirz) - z * Qta;
      }
    }
  }
  for (int i = 0; i < nEwhLoop; ++i) {
    const double* e = ewt + 5 * i;
    double hdotx = e[0] * dx + e[1] * dy + e[2] * dz;
    double c = cos(hdotx), s = sin(hdotx);
    fPot += e[3] * c + e[4] * s;
    ax += e[0] * (e[3] * s - e[4] * c);
    ay += e[1] * (e[3] * s - e[4] * c);
    az += e[2] * (e[3] * s - e[4] * c);
  }
  v[3] += fPot;
  v[0] += ax;
  v[1] += ay;
  v[2] += az;
}

int oracle_ewald_forces(const double* parts, long n_parts, const int* idx, long n_idx,
                        const double* root, double L, int nReps, double fEwCut, double dEwhCut,
                        double* vars, int nthreads) {
  (void)n_parts;
  double ewt[5 * 4096];
  int nh = oracle_ewald_table(root, L, dEwhCut, ewt, 4096);
  if (nh < 0) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (long k = 0; k < n_idx; ++k) {
    long j = idx ? idx[k] : k;
    ewald_one(parts + 5 * (size_t)j, root, L, nReps, fEwCut, ewt, nh, vars + 5 * (size_t)k);
  }
  return 0;
}
