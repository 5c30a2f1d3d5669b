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

/* Potential energy of an open system by direct summation,
 * 0.5 sum_i m_i phi_i with phi_i = -sum_{j != i} m_j a(r_ij): a is the
 * SPLINE potential of partBucketForce (gravity.h:147-182, 290) at
 * twoh = soft_i + soft_j, coincident pairs skipped as there.  Every pair
 * once, OpenMP over i with a reduction. */
double oracle_direct_energy(const double* parts, long n, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  double u = 0.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : u)
  for (long i = 0; i < n; ++i) {
    const double* p = parts + 5 * (size_t)i;
    double s = 0.0;
    for (long j = i + 1; j < n; ++j) {
      const double* q = parts + 5 * (size_t)j;
      const double rx = q[2] - p[2], ry = q[3] - p[3], rz = q[4] - p[4];
      const double rsq = rx * rx + ry * ry + rz * rz;
      if (rsq != 0) {
        double a, b;
        spline(rsq, p[1] + q[1], &a, &b);
        s += q[0] * a;
      }
    }
    u -= p[0] * s;
  }
  return u;
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

/* ---- hexadecapole build of the Ewald correction ---- */

/* Complete moments (moments.h MOMC) of a hexadecapole root given as 27
 * doubles {radius, soft, M, cm.xyz, xx xy xz yy yz, xxx xyy xxy yyy xxz yyz
 * xyz, xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz}: momRescaleFmomr to
 * unit scale (moments.c:238-267, f = radius) then momFmomr2Momc
 * (moments.c:1563-1597), as EwaldInit does (Ewald.cpp:291-296). */
typedef struct {
  double m, xx, yy, xy, xz, yz;
  double xxx, xyy, xxy, yyy, xxz, yyz, xyz;
  double xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz;
  double zz, xzz, yzz, zzz, xxzz, xyzz, xzzz, yyzz, yzzz, zzzz;
} momc_t;

static void momc_from_root(const double* r, momc_t* c) {
  double f = r[0] / 1.0, s = f;
  s *= f;
  c->m = r[2];
  c->xx = r[6] * s;
  c->xy = r[7] * s;
  c->xz = r[8] * s;
  c->yy = r[9] * s;
  c->yz = r[10] * s;
  s *= f;
  c->xxx = r[11] * s;
  c->xyy = r[12] * s;
  c->xxy = r[13] * s;
  c->yyy = r[14] * s;
  c->xxz = r[15] * s;
  c->yyz = r[16] * s;
  c->xyz = r[17] * s;
  s *= f;
  c->xxxx = r[18] * s;
  c->xyyy = r[19] * s;
  c->xxxy = r[20] * s;
  c->yyyy = r[21] * s;
  c->xxxz = r[22] * s;
  c->yyyz = r[23] * s;
  c->xxyy = r[24] * s;
  c->xxyz = r[25] * s;
  c->xyyz = r[26] * s;
  c->zz = -(c->xx + c->yy);
  c->xzz = -(c->xxx + c->xyy);
  c->yzz = -(c->xxy + c->yyy);
  c->zzz = -(c->xxz + c->yyz);
  c->xxzz = -(c->xxxx + c->xxyy);
  c->xyzz = -(c->xxxy + c->xyyy);
  c->xzzz = -(c->xxxz + c->xyyz);
  c->yyzz = -(c->xxyy + c->yyyy);
  c->yzzz = -(c->xxyz + c->yyyz);
  c->zzzz = -(c->xxzz + c->yyzz);
}

/* QEVAL (hexadecapole), Ewald.cpp:6-46: the root expansion of complete
 * moments with gamma factors gam[0..5] at (dx, dy, dz). */
static void qeval_hex(const momc_t* mom, const double gam[6], double dx, double dy, double dz,
                      double* ax, double* ay, double* az, double* fPot) {
  double Qmirx, Qmiry, Qmirz, Qmir, Qta = 0.0;
  Qmirx = (1.0 / 6.0) * (mom->xzzz * dz * dz * dz + 3 * mom->xyzz * dy * dz * dz +
                         3 * mom->xyyz * dy * dy * dz + mom->xyyy * dy * dy * dy +
                         3 * mom->xxzz * dx * dz * dz + 6 * mom->xxyz * dx * dy * dz +
                         3 * mom->xxyy * dx * dy * dy + 3 * mom->xxxz * dx * dx * dz +
                         3 * mom->xxxy * dx * dx * dy + mom->xxxx * dx * dx * dx);
  Qmiry = (1.0 / 6.0) * (mom->yzzz * dz * dz * dz + 3 * mom->xyzz * dx * dz * dz +
                         3 * mom->xxyz * dx * dx * dz + mom->xxxy * dx * dx * dx +
                         3 * mom->yyzz * dy * dz * dz + 6 * mom->xyyz * dx * dy * dz +
                         3 * mom->xxyy * dx * dx * dy + 3 * mom->yyyz * dy * dy * dz +
                         3 * mom->xyyy * dx * dy * dy + mom->yyyy * dy * dy * dy);
  Qmirz = (1.0 / 6.0) * (mom->yyyz * dy * dy * dy + 3 * mom->xyyz * dx * dy * dy +
                         3 * mom->xxyz * dx * dx * dy + mom->xxxz * dx * dx * dx +
                         3 * mom->yyzz * dy * dy * dz + 6 * mom->xyzz * dx * dy * dz +
                         3 * mom->xxzz * dx * dx * dz + 3 * mom->yzzz * dy * dz * dz +
                         3 * mom->xzzz * dx * dz * dz + mom->zzzz * dz * dz * dz);
  Qmir = (1.0 / 4.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
  *fPot -= gam[4] * Qmir;
  Qta += gam[5] * Qmir;
  *ax += gam[4] * Qmirx;
  *ay += gam[4] * Qmiry;
  *az += gam[4] * Qmirz;
  Qmirx = (1.0 / 2.0) * (mom->xzz * dz * dz + 2 * mom->xyz * dy * dz + mom->xyy * dy * dy +
                         2 * mom->xxz * dx * dz + 2 * mom->xxy * dx * dy + mom->xxx * dx * dx);
  Qmiry = (1.0 / 2.0) * (mom->yzz * dz * dz + 2 * mom->xyz * dx * dz + mom->xxy * dx * dx +
                         2 * mom->yyz * dy * dz + 2 * mom->xyy * dx * dy + mom->yyy * dy * dy);
  Qmirz = (1.0 / 2.0) * (mom->yyz * dy * dy + 2 * mom->xyz * dx * dy + mom->xxz * dx * dx +
                         2 * mom->yzz * dy * dz + 2 * mom->xzz * dx * dz + mom->zzz * dz * dz);
  Qmir = (1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
  *fPot -= gam[3] * Qmir;
  Qta += gam[4] * Qmir;
  *ax += gam[3] * Qmirx;
  *ay += gam[3] * Qmiry;
  *az += gam[3] * Qmirz;
  Qmirx = (1.0 / 1.0) * (mom->xz * dz + mom->xy * dy + mom->xx * dx);
  Qmiry = (1.0 / 1.0) * (mom->yz * dz + mom->xy * dx + mom->yy * dy);
  Qmirz = (1.0 / 1.0) * (mom->yz * dy + mom->xz * dx + mom->zz * dz);
  Qmir = (1.0 / 2.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
  *fPot -= gam[2] * Qmir;
  Qta += gam[3] * Qmir;
  *ax += gam[2] * Qmirx;
  *ay += gam[2] * Qmiry;
  *az += gam[2] * Qmirz;
  *fPot -= gam[0] * mom->m;
  Qta += gam[1] * mom->m;
  *ax -= dx * Qta;
  *ay -= dy * Qta;
  *az -= dz * Qta;
}

static void momc_out(const momc_t* c, double* o) {
  /* EwaldCUDA.h MomcData order */
  const double v[32] = {c->m,    c->xx,   c->yy,   c->xy,   c->xz,   c->yz,   c->xxx,  c->xyy,
                        c->xxy,  c->yyy,  c->xxz,  c->yyz,  c->xyz,  c->xxxx, c->xyyy, c->xxxy,
                        c->yyyy, c->xxxz, c->yyyz, c->xxyy, c->xxyz, c->xyyz, c->zz,   c->xzz,
                        c->yzz,  c->zzz,  c->xxzz, c->xyzz, c->xzzz, c->yyzz, c->yzzz, c->zzzz};
  for (int k = 0; k < 32; ++k) o[k] = v[k];
}

/* TreePiece::EwaldInit h-table, Ewald.cpp:285-383 (hexadecapole). */
int oracle_ewald_table_hex(const double* root, double L, double dEwhCut, double* ewt, int max_h,
                           double* momc) {
  momc_t c;
  momc_from_root(root, &c);
  if (momc) momc_out(&c, momc);
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
        qeval_hex(&c, gam, hx, hy, hz, &ax, &ay, &az, &mfacc);
        gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
        gam[1] = 2 * M_PI / L * gam[0];
        gam[2] = -2 * M_PI / L * gam[1];
        gam[3] = 2 * M_PI / L * gam[2];
        gam[4] = -2 * M_PI / L * gam[3];
        gam[5] = 2 * M_PI / L * gam[4];
        gam[0] = 0.0; gam[2] = 0.0; gam[4] = 0.0;
        ax = ay = az = 0.0;
        qeval_hex(&c, gam, hx, hy, hz, &ax, &ay, &az, &mfacs);
        ewt[5 * i + 0] = 2 * M_PI / L * hx;
        ewt[5 * i + 1] = 2 * M_PI / L * hy;
        ewt[5 * i + 2] = 2 * M_PI / L * hz;
        ewt[5 * i + 3] = mfacc;
        ewt[5 * i + 4] = mfacs;
        ++i;
      }
  return i;
}

/* TreePiece::BucketEwald (hexadecapole), Ewald.cpp:72-281 for one
 * particle: the complete root moments to fourth order, g0..g5. */
static void ewald_one_hex(const double* p, const double* root, const momc_t* mom, double L,
                          int nReps, double fEwCut, const double* ewt, int nEwhLoop, double* v) {
  const double onethird = 1.0 / 3.0;
  double Q4xx = 0.5 * (mom->xxxx + mom->xxyy + mom->xxzz);
  double Q4xy = 0.5 * (mom->xxxy + mom->xyyy + mom->xyzz);
  double Q4xz = 0.5 * (mom->xxxz + mom->xyyz + mom->xzzz);
  double Q4yy = 0.5 * (mom->xxyy + mom->yyyy + mom->yyzz);
  double Q4yz = 0.5 * (mom->xxyz + mom->yyyz + mom->yzzz);
  double Q4zz = 0.5 * (mom->xxzz + mom->yyzz + mom->zzzz);
  double Q4 = 0.25 * (Q4xx + Q4yy + Q4zz);
  double Q3x = 0.5 * (mom->xxx + mom->xyy + mom->xzz);
  double Q3y = 0.5 * (mom->xxy + mom->yyy + mom->yzz);
  double Q3z = 0.5 * (mom->xxz + mom->yyz + mom->zzz);
  double Q2 = 0.5 * (mom->xx + mom->yy + mom->zz);
  int nEwReps = (int)ceil(fEwCut);
  double fEwCut2 = fEwCut * fEwCut * L * L;
  double fInner2 = 1.2e-3 * L * L;
  if (nReps > nEwReps) nEwReps = nReps;
  double alpha = 2.0 / L;
  double alpha2 = alpha * alpha;
  double k1 = M_PI / (alpha2 * L * L * L);
  double ka = 2.0 * alpha / sqrt(M_PI);
  double fPot = root[2] * k1, ax = 0.0, ay = 0.0, az = 0.0;
  double dx = p[2] - root[3], dy = p[3] - root[4], dz = p[4] - root[5];
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
        double g0, g1, g2, g3, g4, g5, alphan;
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
          alphan *= 2 * alpha2;
          g4 = alphan * ((1.0 / 11.0) * r2 - (1.0 / 9.0));
          alphan *= 2 * alpha2;
          g5 = alphan * ((1.0 / 13.0) * r2 - (1.0 / 11.0));
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
          alphan *= 2 * alpha2;
          g4 = 7 * g3 * dir2 + alphan * a;
          alphan *= 2 * alpha2;
          g5 = 9 * g4 * dir2 + alphan * a;
        }
        double xx = 0.5 * x * x;
        double xxx = onethird * xx * x;
        double xxy = xx * y;
        double xxz = xx * z;
        double yy = 0.5 * y * y;
        double yyy = onethird * yy * y;
        double xyy = yy * x;
        double yyz = yy * z;
        double zz = 0.5 * z * z;
        double zzz = onethird * zz * z;
        double xzz = zz * x;
        double yzz = zz * y;
        double xy = x * y;
        double xyz = xy * z;
        double xz = x * z;
        double yz = y * z;
        double Q2mirx = mom->xx * x + mom->xy * y + mom->xz * z;
        double Q2miry = mom->xy * x + mom->yy * y + mom->yz * z;
        double Q2mirz = mom->xz * x + mom->yz * y + mom->zz * z;
        double Q3mirx = mom->xxx * xx + mom->xxy * xy + mom->xxz * xz + mom->xyy * yy +
                        mom->xyz * yz + mom->xzz * zz;
        double Q3miry = mom->xxy * xx + mom->xyy * xy + mom->xyz * xz + mom->yyy * yy +
                        mom->yyz * yz + mom->yzz * zz;
        double Q3mirz = mom->xxz * xx + mom->xyz * xy + mom->xzz * xz + mom->yyz * yy +
                        mom->yzz * yz + mom->zzz * zz;
        double Q4mirx = mom->xxxx * xxx + mom->xxxy * xxy + mom->xxxz * xxz + mom->xxyy * xyy +
                        mom->xxyz * xyz + mom->xxzz * xzz + mom->xyyy * yyy + mom->xyyz * yyz +
                        mom->xyzz * yzz + mom->xzzz * zzz;
        double Q4miry = mom->xxxy * xxx + mom->xxyy * xxy + mom->xxyz * xxz + mom->xyyy * xyy +
                        mom->xyyz * xyz + mom->xyzz * xzz + mom->yyyy * yyy + mom->yyyz * yyz +
                        mom->yyzz * yzz + mom->yzzz * zzz;
        double Q4mirz = mom->xxxz * xxx + mom->xxyz * xxy + mom->xxzz * xxz + mom->xyyz * xyy +
                        mom->xyzz * xyz + mom->xzzz * xzz + mom->yyyz * yyy + mom->yyzz * yyz +
                        mom->yzzz * yzz + mom->zzzz * zzz;
        double Q4x = Q4xx * x + Q4xy * y + Q4xz * z;
        double Q4y = Q4xy * x + Q4yy * y + Q4yz * z;
        double Q4z = Q4xz * x + Q4yz * y + Q4zz * z;
        double Q2mir = 0.5 * (Q2mirx * x + Q2miry * y + Q2mirz * z) - (Q3x * x + Q3y * y + Q3z * z) + Q4;
        double Q3mir = onethird * (Q3mirx * x + Q3miry * y + Q3mirz * z) - 0.5 * (Q4x * x + Q4y * y + Q4z * z);
        double Q4mir = 0.25 * (Q4mirx * x + Q4miry * y + Q4mirz * z);
        double Qta = g1 * mom->m - g2 * Q2 + g3 * Q2mir + g4 * Q3mir + g5 * Q4mir;
        fPot -= g0 * mom->m - g1 * Q2 + g2 * Q2mir + g3 * Q3mir + g4 * Q4mir;
        ax += g2 * (Q2mirx - Q3x) + g3 * (Q3mirx - Q4x) + g4 * Q4mirx - x * Qta;
        ay += g2 * (Q2miry - Q3y) + g3 * (Q3miry - Q4y) + g4 * Q4miry - y * Qta;
        az += g2 * (Q2mirz - Q3z) + g3 * (Q3mirz - Q4z) + g4 * Q4mirz - z * Qta;
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

int oracle_ewald_forces_hex(const double* parts, long n_parts, const int* idx, long n_idx,
                            const double* root, double L, int nReps, double fEwCut,
                            double dEwhCut, double* vars, int nthreads) {
  (void)n_parts;
  double ewt[5 * 4096];
  momc_t c;
  momc_from_root(root, &c);
  int nh = oracle_ewald_table_hex(root, L, dEwhCut, ewt, 4096, NULL);
  if (nh < 0) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (long k = 0; k < n_idx; ++k) {
    long j = idx ? idx[k] : k;
    ewald_one_hex(parts + 5 * (size_t)j, root, &c, L, nReps, fEwCut, ewt, nh,
                  vars + 5 * (size_t)k);
  }
  return 0;
}
