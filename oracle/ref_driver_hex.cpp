/*
 * Drives ChaNGa's own CPU cell-list force code in its hexadecapole build
 * (-DHEXADECAPOLE, the reference's default configuration) as an oracle.
 *
 * TEST INFRASTRUCTURE ONLY (built into oracle/_ref/ with the reference's
 * moments.c by oracle/Makefile when the reference sources are present;
 * loaded only by tests).
 *
 * gravity.h is included unmodified.  With HEXADECAPOLE, nodeBucketForce
 * (gravity.h:398-421, 439-446) evaluates a cell with momEvalFmomrcm
 * (moments.c:1469-1525) unless the cell's softening sphere meets the bucket
 * (openSoftening, gravity.h:252-260), in which case the cell acts as a
 * softened point mass through partBucketForce.  The bucket therefore needs
 * its centre of mass, softening and bounding box; they come in geom.
 *
 * Ewald.cpp is included unmodified as well: with HEXADECAPOLE, EwaldInit
 * forms the root's complete moments (momRescaleFmomr, momFmomr2Momc) and the
 * h-table from them, and BucketEwald expands about the root to fourth order.
 */
#include "ref_shim.h"
#include "gravity.h"
#include "Ewald.cpp"

#include <vector>
#include "../oracle_api.h"

#ifdef _OPENMP
#include <omp.h>
#endif

cosmoType theta = 0.7;
cosmoType thetaMono = 0.7 * 0.7 * 0.7 * 0.7;

static inline Vector3D<cosmoType> decode_offset(int offsetID, double fperiod) {
  int code = offsetID >> 22;
  int x = (code & 0x7) - 3, y = ((code >> 3) & 0x7) - 3, z = ((code >> 6) & 0x7) - 3;
  return Vector3D<cosmoType>(x * fperiod, y * fperiod, z * fperiod);
}

extern "C" int oracle_cell_list_forces_hex(const double* moments, long n_moments,
                                           const double* parts, long n_parts, const int* list,
                                           const int* markers, const int* starts,
                                           const int* sizes, int n_buckets, const double* geom,
                                           double fperiod, double* vars, int nthreads) {
  std::vector<GravityParticle> gp((size_t)n_parts);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int b = 0; b < n_buckets; ++b) {
    const int s = starts[b], n = sizes[b];
    for (int j = s; j < s + n; ++j) {
      const double* p = parts + 5 * (size_t)j;
      gp[j].mass = p[0];
      gp[j].soft = p[1];
      gp[j].position = Vector3D<cosmoType>(p[2], p[3], p[4]);
      const double* v = vars + 5 * (size_t)j;
      gp[j].treeAcceleration = Vector3D<cosmoType>(v[0], v[1], v[2]);
      gp[j].potential = v[3];
      gp[j].dtGrav = v[4];
      gp[j].rung = 0;
    }
    GenericTreeNode req;
    req.myType = Tree::Bucket;
    req.firstParticle = s;
    req.lastParticle = s + n - 1;
    req.particleCount = n;
    const double* g = geom + 10 * (size_t)b;
    req.moments.cm = Vector3D<cosmoType>(g[0], g[1], g[2]);
    req.moments.soft = g[3];
    req.boundingBox.lesser_corner = Vector3D<double>(g[4], g[5], g[6]);
    req.boundingBox.greater_corner = Vector3D<double>(g[7], g[8], g[9]);
    GenericTreeNode node;
    node.myType = Tree::Internal;
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      const int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_moments) continue;
      const double* m = moments + 27 * (size_t)idx;
      node.moments.radius = m[0];
      node.moments.soft = m[1];
      node.moments.totalMass = m[2];
      node.moments.cm = Vector3D<cosmoType>(m[3], m[4], m[5]);
      FMOMR& f = node.moments.mom;
      f.m = m[2];
      f.xx = m[6];
      f.xy = m[7];
      f.xz = m[8];
      f.yy = m[9];
      f.yz = m[10];
      f.xxx = m[11];
      f.xyy = m[12];
      f.xxy = m[13];
      f.yyy = m[14];
      f.xxz = m[15];
      f.yyz = m[16];
      f.xyz = m[17];
      f.xxxx = m[18];
      f.xyyy = m[19];
      f.xxxy = m[20];
      f.yyyy = m[21];
      f.xxxz = m[22];
      f.yyyz = m[23];
      f.xxyy = m[24];
      f.xxyz = m[25];
      f.xyyz = m[26];
      nodeBucketForce(&node, &req, gp.data(), decode_offset(list[2 * (size_t)e + 1], fperiod), 0);
    }
    for (int j = s; j < s + n; ++j) {
      double* v = vars + 5 * (size_t)j;
      v[0] = gp[j].treeAcceleration.x;
      v[1] = gp[j].treeAcceleration.y;
      v[2] = gp[j].treeAcceleration.z;
      v[3] = gp[j].potential;
      v[4] = gp[j].dtGrav;
    }
  }
  return 0;
}

/* The hexadecapole root as the reference's MultipoleMoments (27 values). */
static void fill_root_hex(GenericTreeNode& root, const double* m) {
  root.moments.radius = m[0];
  root.moments.soft = m[1];
  root.moments.totalMass = m[2];
  root.moments.cm = Vector3D<cosmoType>(m[3], m[4], m[5]);
  FMOMR& f = root.moments.mom;
  f.m = m[2];
  f.xx = m[6];
  f.xy = m[7];
  f.xz = m[8];
  f.yy = m[9];
  f.yz = m[10];
  f.xxx = m[11];
  f.xyy = m[12];
  f.xxy = m[13];
  f.yyy = m[14];
  f.xxz = m[15];
  f.yyz = m[16];
  f.xyz = m[17];
  f.xxxx = m[18];
  f.xyyy = m[19];
  f.xxxy = m[20];
  f.yyyy = m[21];
  f.xxxz = m[22];
  f.yyyz = m[23];
  f.xxyy = m[24];
  f.xxyz = m[25];
  f.xyyz = m[26];
}

static void copy_momc(const MOMC& c, double* o) {
  const double v[32] = {c.m,    c.xx,   c.yy,   c.xy,   c.xz,   c.yz,   c.xxx,  c.xyy,
                        c.xxy,  c.yyy,  c.xxz,  c.yyz,  c.xyz,  c.xxxx, c.xyyy, c.xxxy,
                        c.yyyy, c.xxxz, c.yyyz, c.xxyy, c.xxyz, c.xyyz, c.zz,   c.xzz,
                        c.yzz,  c.zzz,  c.xxzz, c.xyzz, c.xzzz, c.yyzz, c.yzzz, c.zzzz};
  for (int k = 0; k < 32; ++k) o[k] = v[k];
}

extern "C" int oracle_ewald_table_hex(const double* root_moments, double L, double dEwhCut,
                                      double* ewt, int max_h, double* momc) {
  TreePiece tp;
  GenericTreeNode root;
  fill_root_hex(root, root_moments);
  tp.root = &root;
  tp.fPeriod = Vector3D<cosmoType>(L, L, L);
  tp.dEwhCut = dEwhCut;
  tp.EwaldInit();
  if (tp.nEwhLoop > max_h) return -1;
  for (int i = 0; i < tp.nEwhLoop; ++i) {
    ewt[5 * i + 0] = tp.ewt[i].hx;
    ewt[5 * i + 1] = tp.ewt[i].hy;
    ewt[5 * i + 2] = tp.ewt[i].hz;
    ewt[5 * i + 3] = tp.ewt[i].hCfac;
    ewt[5 * i + 4] = tp.ewt[i].hSfac;
  }
  if (momc) copy_momc(tp.momcRoot, momc);
  return tp.nEwhLoop;
}

extern "C" int oracle_ewald_forces_hex(const double* parts, long n_parts, const int* idx,
                                       long n_idx, const double* root_moments, double L,
                                       int nReps, double fEwCut, double dEwhCut, double* vars,
                                       int nthreads) {
  (void)n_parts;
  GenericTreeNode root;
  fill_root_hex(root, root_moments);
  std::vector<GravityParticle> gp((size_t)n_idx);
  for (long k = 0; k < n_idx; ++k) {
    long j = idx ? idx[k] : k;
    const double* p = parts + 5 * (size_t)j;
    gp[k].mass = p[0];
    gp[k].soft = p[1];
    gp[k].position = Vector3D<cosmoType>(p[2], p[3], p[4]);
    const double* v = vars + 5 * (size_t)k;
    gp[k].treeAcceleration = Vector3D<cosmoType>(v[0], v[1], v[2]);
    gp[k].potential = v[3];
    gp[k].dtGrav = v[4];
  }
  /* One EwaldInit (the table and momcRoot), then BucketEwald over chunks. */
  TreePiece proto;
  proto.root = &root;
  proto.fPeriod = Vector3D<cosmoType>(L, L, L);
  proto.dEwhCut = dEwhCut;
  proto.nReplicas = nReps;
  proto.fEwCut = fEwCut;
  proto.EwaldInit();
  const long chunk = 256;
  long nchunks = (n_idx + chunk - 1) / chunk;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (long c = 0; c < nchunks; ++c) {
    TreePiece tp;
    tp.root = &root;
    tp.fPeriod = proto.fPeriod;
    tp.dEwhCut = dEwhCut;
    tp.nReplicas = nReps;
    tp.fEwCut = fEwCut;
    tp.momcRoot = proto.momcRoot;
    tp.nEwhLoop = proto.nEwhLoop;
    if (proto.nEwhLoop > tp.nMaxEwhLoop) {
      delete[] tp.ewt;
      tp.nMaxEwhLoop = proto.nEwhLoop;
      tp.ewt = new EWT[tp.nMaxEwhLoop];
    }
    for (int i = 0; i < proto.nEwhLoop; ++i) tp.ewt[i] = proto.ewt[i];
    tp.myParticles = gp.data();
    GenericTreeNode req;
    req.firstParticle = (int)(c * chunk);
    req.lastParticle = (int)((c + 1) * chunk < n_idx ? (c + 1) * chunk - 1 : n_idx - 1);
    tp.BucketEwald(&req, nReps, fEwCut);
  }
  for (long k = 0; k < n_idx; ++k) {
    double* v = vars + 5 * (size_t)k;
    v[0] = gp[k].treeAcceleration.x;
    v[1] = gp[k].treeAcceleration.y;
    v[2] = gp[k].treeAcceleration.z;
    v[3] = gp[k].potential;
    v[4] = gp[k].dtGrav;
  }
  return 0;
}
