/*
 * Drives ChaNGa's own CPU force code as an oracle.
 *
 * TEST INFRASTRUCTURE ONLY (built into oracle/_ref/ by oracle/Makefile when
 * the reference sources are present; loaded only by tests and bench.py's
 * CPU-baseline leg).
 *
 * gravity.h and Ewald.cpp are included straight from the reference tree,
 * unmodified; oracle/shim provides the few types they need.  The loops below
 * mirror how the reference CPU path calls them:
 *   - ListCompute::calcNodeForces -> nodeBucketForce per cell-list entry
 *     (Compute.cpp:1328-1358, gravity.h:398-475)
 *   - ListCompute::calcParticleForces -> partBucketForce once per source
 *     particle (Compute.cpp:1360-1392, gravity.h:267-303)
 *   - TreePiece::EwaldInit / BucketEwald (Ewald.cpp:72-383)
 * The offset of a list entry is TreePiece::decodeOffset (ParallelGravity.h:
 * 2064-2073) with a cubic period.
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
cosmoType thetaMono = 0.7 * 0.7 * 0.7;

static inline Vector3D<cosmoType> decode_offset(int offsetID, double fperiod) {
  int code = offsetID >> 22;
  int x = (code & 0x7) - 3, y = ((code >> 3) & 0x7) - 3, z = ((code >> 6) & 0x7) - 3;
  return Vector3D<cosmoType>(x * fperiod, y * fperiod, z * fperiod);
}

static void load_targets(GravityParticle* gp, const double* parts, const double* vars, int s, int n) {
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
}

static void store_targets(const GravityParticle* gp, double* vars, int s, int n) {
  for (int j = s; j < s + n; ++j) {
    double* v = vars + 5 * (size_t)j;
    v[0] = gp[j].treeAcceleration.x;
    v[1] = gp[j].treeAcceleration.y;
    v[2] = gp[j].treeAcceleration.z;
    v[3] = gp[j].potential;
    v[4] = gp[j].dtGrav;
  }
}

extern "C" int oracle_cell_list_forces(const double* moments, long n_moments,
                                       const double* parts, long n_parts,
                                       const int* list, const int* markers,
                                       const int* starts, const int* sizes, int n_buckets,
                                       const int* bucket_ids, int n_ids,
                                       double fperiod, double* vars, int nthreads) {
  int nwork = bucket_ids ? n_ids : n_buckets;
  std::vector<GravityParticle> gp((size_t)n_parts);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int w = 0; w < nwork; ++w) {
    int b = bucket_ids ? bucket_ids[w] : w;
    int s = starts[b], n = sizes[b];
    load_targets(gp.data(), parts, vars, s, n);
    GenericTreeNode req;
    req.myType = Tree::Bucket;
    req.firstParticle = s;
    req.lastParticle = s + n - 1;
    req.particleCount = n;
    GenericTreeNode node;
    node.myType = Tree::Internal;
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_moments) continue;
      const double* m = moments + 12 * (size_t)idx;
      node.moments.radius = m[0];
      node.moments.soft = m[1];
      node.moments.totalMass = m[2];
      node.moments.cm = Vector3D<cosmoType>(m[3], m[4], m[5]);
      node.moments.xx = m[6];
      node.moments.xy = m[7];
      node.moments.xz = m[8];
      node.moments.yy = m[9];
      node.moments.yz = m[10];
      node.moments.zz = m[11];
      nodeBucketForce(&node, &req, gp.data(), decode_offset(list[2 * (size_t)e + 1], fperiod), 0);
    }
    store_targets(gp.data(), vars, s, n);
  }
  return 0;
}

extern "C" int oracle_part_list_forces(const double* sources, long n_sources,
                                       const double* targets, long n_targets,
                                       const int* list, const int* markers,
                                       const int* starts, const int* sizes, int n_buckets,
                                       const int* bucket_ids, int n_ids,
                                       double fperiod, double* vars, int nthreads) {
  int nwork = bucket_ids ? n_ids : n_buckets;
  std::vector<GravityParticle> gp((size_t)n_targets);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int w = 0; w < nwork; ++w) {
    int b = bucket_ids ? bucket_ids[w] : w;
    int s = starts[b], n = sizes[b];
    load_targets(gp.data(), targets, vars, s, n);
    GenericTreeNode req;
    req.myType = Tree::Bucket;
    req.firstParticle = s;
    req.lastParticle = s + n - 1;
    req.particleCount = n;
    ExternalGravityParticle src;
    for (int e = markers[b]; e < markers[b + 1]; ++e) {
      int idx = list[2 * (size_t)e];
      if (idx < 0 || idx >= n_sources) continue;
      const double* p = sources + 5 * (size_t)idx;
      src.mass = p[0];
      src.soft = p[1];
      src.position = Vector3D<cosmoType>(p[2], p[3], p[4]);
      partBucketForce(&src, &req, gp.data(), decode_offset(list[2 * (size_t)e + 1], fperiod), 0);
    }
    store_targets(gp.data(), vars, s, n);
  }
  return 0;
}

static void fill_root(GenericTreeNode& root, const double* m) {
  root.moments.radius = m[0];
  root.moments.soft = m[1];
  root.moments.totalMass = m[2];
  root.moments.cm = Vector3D<cosmoType>(m[3], m[4], m[5]);
  root.moments.xx = m[6];
  root.moments.xy = m[7];
  root.moments.xz = m[8];
  root.moments.yy = m[9];
  root.moments.yz = m[10];
  root.moments.zz = m[11];
}

extern "C" int oracle_ewald_table(const double* root_moments, double L, double dEwhCut,
                                  double* ewt, int max_h) {
  TreePiece tp;
  GenericTreeNode root;
  fill_root(root, root_moments);
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
  return tp.nEwhLoop;
}

extern "C" int oracle_ewald_forces(const double* parts, long n_parts, const int* idx, long n_idx,
                                   const double* root_moments, double L, int nReps,
                                   double fEwCut, double dEwhCut, double* vars, int nthreads) {
  (void)n_parts;
  GenericTreeNode root;
  fill_root(root, root_moments);
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
  /* One EwaldInit, then BucketEwald over chunks of the particle array. */
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
