/*
 * Interaction-list walk on the GPU (the reference has a prototype of the
 * same idea, gpuLocalTreeWalk, HostCUDA.cu:724-942).
 *
 * The host walk (changa_gb300/host/tree.cpp) is ChaNGa's dual walk
 * (LocalTargetWalk::dft, TreeWalk.cpp:308-397 with ListCompute's actions):
 * every check-list entry is tested against the local node at each level,
 * accepted as a cell, opened (children join the same level's check list),
 * opened into its particles when it is a bucket, or deferred to the next
 * local level when undecided (openCriterionNode, gravity.h:652-723).
 * Which entries a bucket finally holds depends only on the tests against
 * the local nodes on the path from the root to that bucket.  So one thread
 * per target bucket reproduces the same per-bucket sets with a depth-first
 * stack of (source node, local level, replica) entries: it tests against
 * the local node of its level and pushes deferred entries one level down.
 * The lists hold the same entries as the host walk's, in depth-first
 * instead of level order.
 *
 * Two launches: a count pass (per-bucket list lengths) and, after the
 * caller has turned the counts into offsets, a fill pass.
 *
 * Decisions equal the host walk's FP64 decisions.  GB300 issues FP64 at a
 * small fraction of its FP32 rate, so each opening test is first made in
 * FP32 from rounded copies of the node data, with a bound on how far the
 * FP32 distance can lie from the FP64 one: the clipped box distance and the
 * farthest-corner distance are 1-Lipschitz in the coordinates, so an input
 * error of delta moves a squared distance g^2 by at most 2 g delta +
 * delta^2.  Only tests whose FP32 value lies within that margin of the
 * threshold are repeated in FP64, with the host's expressions (this file is
 * compiled without FMA contraction, as the host code is).
 */
#include "chg_internal.h"

namespace chg {
namespace {

constexpr int kWalkThreads = 128;
constexpr int kStack = 256;

struct WalkArgs {
  const double* geom;  // n_nodes x 6 {cm.xyz, radius, soft, mass}
  const double* bbox;  // n_nodes x 6
  const int* info;     // n_nodes x 4 {child0, child1, first, count}
  const int* parent;   // n_nodes
  long long n_nodes;
  const int* bucket_node;  // n_buckets: moment index of each bucket
  int n_buckets;
  double theta, theta_mono, period;
  int order, n_replicas;
  /* count pass */
  int* n_cells;
  int* n_parts;
  int* n_soft;
  /* fill pass */
  const long long* off_cells;
  const long long* off_parts;
  const long long* off_soft;
  int2* cells;
  int2* parts;
  int2* soft;
  int* error;
  /* FP32 copies for the screening test */
  const float4* nodef;  // n_nodes: {cm.xyz, rn32(opening radius^2)}
  const float4* boxf;   // 2 n_nodes: {lesser.xyz, 0}, {greater.xyz, 0}
  float period32;
};

constexpr float kU = 5.9604645e-08f;  // 2^-24, the FP32 unit roundoff

/* FP32 copies of each node's centre, box and opening radius squared, the
 * last formed in FP64 exactly as open_criterion forms it. */
__global__ void walk_prep_kernel(const double* __restrict__ geom, const double* __restrict__ bbox,
                                 long long n_nodes, double theta, float4* __restrict__ nodef,
                                 float4* __restrict__ boxf) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n_nodes;
       g += (long long)gridDim.x * blockDim.x) {
    const double* gg = geom + 6 * g;
    const double kOpenGeom = 2.0 / sqrt(3.0);
    double radius = kOpenGeom * gg[3] / theta;
    if (radius < gg[3]) radius = gg[3];
    nodef[g] = make_float4((float)gg[0], (float)gg[1], (float)gg[2], (float)(radius * radius));
    const double* b = bbox + 6 * g;
    boxf[2 * g] = make_float4((float)b[0], (float)b[1], (float)b[2], 0.0f);
    boxf[2 * g + 1] = make_float4((float)b[3], (float)b[4], (float)b[5], 0.0f);
  }
}

/* v <= r2 decided from an FP32 value v within e of the FP64 one and r2 =
 * rn32 of the FP64 threshold: 1 certainly, 0 certainly not, -1 too close.
 * The margins carry one extra unit roundoff for the rounding of the two
 * sums compared here; NaN or infinity give -1. */
__device__ __forceinline__ int screen_le(float v, float e, float r2) {
  const float er = 2.0f * kU * r2;
  if (v + e < r2 - er) return 1;
  if (v - e > r2 + er) return 0;
  return -1;
}

__device__ __forceinline__ void decode(int off, double period, double* o) {
  o[0] = ((off & 7) - 3) * period;
  o[1] = (((off >> 3) & 7) - 3) * period;
  o[2] = (((off >> 6) & 7) - 3) * period;
}

__device__ __forceinline__ double box_dist2(const double* b, const double* c) {
  double d2 = 0.0, d;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if ((d = b[k] - c[k]) > 0) d2 += d * d;
    else if ((d = c[k] - b[3 + k]) > 0) d2 += d * d;
  }
  return d2;
}

/* openSoftening (gravity.h:252-260), as tree.cpp's open_softening. */
__device__ bool open_softening(const WalkArgs& a, int g, int local, const double* c) {
  const double r = 2.0 * a.geom[6 * g + 4];
  const double* lg = a.geom + 6 * (size_t)local;
  const double dx = c[0] - lg[0], dy = c[1] - lg[1], dz = c[2] - lg[2];
  const double rr = r + 2.0 * lg[4];
  if (dx * dx + dy * dy + dz * dz <= rr * rr) return true;
  return box_dist2(a.bbox + 6 * (size_t)local, c) <= r * r;
}

/* openCriterionNode (gravity.h:652-723), quadrupole and hexadecapole
 * forms: 1 open, -1 undecided, 0 accept. */
__device__ int open_criterion(const WalkArgs& a, int g, int local, bool local_bucket, int off) {
  const int count = a.info[4 * (size_t)g + 3];
  if (count <= 6) return 1;
  const double* gg = a.geom + 6 * (size_t)g;
  const double kOpenGeom = 2.0 / sqrt(3.0);
  double radius = kOpenGeom * gg[3] / a.theta;
  if (radius < gg[3]) radius = gg[3];
  double o[3];
  decode(off, a.period, o);
  const double c[3] = {gg[0] + o[0], gg[1] + o[1], gg[2] + o[2]};
  const double* b = a.bbox + 6 * (size_t)local;
  const double d2 = box_dist2(b, c);
  const double r2 = radius * radius;
  const bool inter = d2 <= r2;
  if (inter) {
    if (local_bucket) return 1;
    double f2 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double a1 = c[k] - b[k], a2 = b[3 + k] - c[k];
      a1 *= a1;
      a2 *= a2;
      f2 += a1 > a2 ? a1 : a2;
    }
    return f2 <= r2 ? 1 : -1;
  }
  if (a.order != 4) return 0;
  if (!open_softening(a, g, local, c)) return 0;
  const double rm = kOpenGeom * gg[3] / a.theta_mono;
  return d2 <= rm * rm ? 1 : 0;
}

/* open_criterion screened in FP32.  Per axis the FP32 inputs (centre,
 * replica offset, box faces) and the FP32 sums and differences carry at
 * most u (3|cm| + 4|o| + 2|b|) of error against the FP64 values; delta =
 * 6u (|cm| + |o| + |lesser| + |greater|) covers that and the FP64 path's own
 * rounding (the 1e-30 floor covers conversions that land on FP32
 * subnormals).  Squares and the three-term sum add 2u of the total,
 * bounded here by 4u. */
__device__ int open_criterion_screened(const WalkArgs& a, int g, int local, bool local_bucket,
                                       int off) {
  if (a.info[4 * (size_t)g + 3] <= 6) return 1;
  const float4 nf = a.nodef[g];
  const float4 lo = a.boxf[2 * (size_t)local], hi = a.boxf[2 * (size_t)local + 1];
  const float cm[3] = {nf.x, nf.y, nf.z};
  const float o[3] = {(float)((off & 7) - 3) * a.period32,
                      (float)(((off >> 3) & 7) - 3) * a.period32,
                      (float)(((off >> 6) & 7) - 3) * a.period32};
  const float bl[3] = {lo.x, lo.y, lo.z}, bh[3] = {hi.x, hi.y, hi.z};
  float c[3], dl[3];
  float d2 = 0.0f, e = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c[k] = cm[k] + o[k];
    dl[k] = 6.0f * kU * (fabsf(cm[k]) + fabsf(o[k]) + fabsf(bl[k]) + fabsf(bh[k])) + 1e-30f;
    const float gk = fmaxf(0.0f, fmaxf(bl[k] - c[k], c[k] - bh[k]));
    d2 += gk * gk;
    e += 2.0f * gk * dl[k] + 3.0f * dl[k] * dl[k];
  }
  e += 4.0f * kU * d2;
  const int inter = screen_le(d2, e, nf.w);
  if (inter < 0) return open_criterion(a, g, local, local_bucket, off);
  if (inter == 1) {
    if (local_bucket) return 1;
    float f2 = 0.0f, ef = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float mk = fmaxf(fabsf(c[k] - bl[k]), fabsf(bh[k] - c[k]));
      f2 += mk * mk;
      ef += 2.0f * mk * dl[k] + 3.0f * dl[k] * dl[k];
    }
    ef += 4.0f * kU * f2;
    const int far = screen_le(f2, ef, nf.w);
    if (far < 0) return open_criterion(a, g, local, local_bucket, off);
    return far ? 1 : -1;
  }
  /* outside the opening sphere: accepted, unless the hexadecapole rules
   * (softening, monopole radius) open it, which stay in FP64 */
  if (a.order != 4) return 0;
  return open_criterion(a, g, local, local_bucket, off);
}

template <bool FILL>
__global__ void __launch_bounds__(kWalkThreads) walk_kernel(const WalkArgs a) {
  const int b = blockIdx.x * kWalkThreads + threadIdx.x;
  if (b >= a.n_buckets) return;
  const int bn = a.bucket_node[b];
  if (bn < 0 || bn >= a.n_nodes) return;
  /* local nodes from the root down to this bucket */
  int chain[64];
  int depth = 0;
  {
    int tmp[64];
    int n = 0;
    for (int x = bn; x >= 0 && x < a.n_nodes && n < 64; x = a.parent[x]) tmp[n++] = x;
    if (n >= 64 || tmp[n - 1] != 0) {
      atomicExch(a.error, 1);
      return;
    }
    for (int i = 0; i < n; ++i) chain[i] = tmp[n - 1 - i];
    depth = n - 1;  // chain[depth] == bn
  }
  int nc = 0, np = 0, ns = 0;
  long long oc = 0, op = 0, os = 0;
  if (FILL) {
    oc = a.off_cells[b];
    op = a.off_parts[b];
    os = a.off_soft ? a.off_soft[b] : 0;
  }
  /* stack entries: node, level << 16 | replica code */
  int2 st[kStack];
  int sp = 0;
  const int nr = a.n_replicas;
  for (int x = -nr; x <= nr; ++x)
    for (int y = -nr; y <= nr; ++y)
      for (int z = -nr; z <= nr; ++z)
        if (sp < kStack) st[sp++] = make_int2(0, (x + 3) | ((y + 3) << 3) | ((z + 3) << 6));
  while (sp > 0) {
    const int2 e = st[--sp];
    const int g = e.x, level = e.y >> 16, code = e.y & 0xffff;
    if (g < 0 || g >= a.n_nodes) continue;  // memory safety
    const int local = chain[level];
    const bool local_bucket = level == depth;
    const int open = open_criterion_screened(a, g, local, local_bucket, code);
    const int* gi = a.info + 4 * (size_t)g;
    if (open == 0) {
      bool softened = false;
      if (a.order == 4) {
        double o[3];
        decode(code, a.period, o);
        const double* gg = a.geom + 6 * (size_t)g;
        const double c[3] = {gg[0] + o[0], gg[1] + o[1], gg[2] + o[2]};
        softened = open_softening(a, g, bn, c);
      }
      if (softened) {
        if (FILL) a.soft[os + ns] = make_int2(g, code << 22);
        ++ns;
      } else {
        if (FILL) a.cells[oc + nc] = make_int2(g, code << 22);
        ++nc;
      }
      continue;
    }
    if (gi[0] < 0 && gi[1] < 0) {  // a source bucket: its particles
      if (FILL)
        for (int k = 0; k < gi[3]; ++k) a.parts[op + np + k] = make_int2(gi[2] + k, code << 22);
      np += gi[3];
      continue;
    }
    if (open == 1 || local_bucket) {
      if (sp + 2 > kStack) {
        atomicExch(a.error, 2);
        break;
      }
      if (gi[1] >= 0) st[sp++] = make_int2(gi[1], (level << 16) | code);
      if (gi[0] >= 0) st[sp++] = make_int2(gi[0], (level << 16) | code);
    } else {
      if (sp + 1 > kStack) {
        atomicExch(a.error, 2);
        break;
      }
      st[sp++] = make_int2(g, ((level + 1) << 16) | code);
    }
  }
  if (!FILL) {
    a.n_cells[b] = nc;
    a.n_parts[b] = np;
    if (a.n_soft) a.n_soft[b] = ns;
  }
}

}  // namespace
}  // namespace chg

using namespace chg;

static int walk_launch(const ChangaTreeView* t, const ChangaWalkParams* p, bool fill, int* nc,
                       int* np, int* ns, const long long* oc, const long long* op,
                       const long long* os, ILCell* cells, ILCell* parts, ILCell* soft,
                       cudaStream_t s) {
  if (!t || !p || !t->geom || !t->bbox || !t->info || !t->parent || !t->bucket_node ||
      t->n_nodes <= 0 || t->n_buckets < 0 || p->theta <= 0 || (p->order != 2 && p->order != 4) ||
      p->n_replicas < 0 || p->n_replicas > 3)
    return record_error(CHANGA_E_INVALID_ARG, "walk: arguments", __FILE__, __LINE__);
  if (t->n_buckets == 0) return 0;
  prepare_pool();
  char* block = nullptr;
  const size_t nn = (size_t)t->n_nodes;
  CHG_CUDA(cudaMallocAsync((void**)&block, 256 + nn * 3 * sizeof(float4), s));
  int* err = (int*)block;
  float4* nodef = (float4*)(block + 256);
  float4* boxf = nodef + nn;
  CHG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  {
    long long g = (t->n_nodes + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    walk_prep_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(t->geom, t->bbox, t->n_nodes,
                                                              p->theta, nodef, boxf);
    count_launch();
  }
  WalkArgs a;
  a.geom = t->geom;
  a.bbox = t->bbox;
  a.info = t->info;
  a.parent = t->parent;
  a.n_nodes = t->n_nodes;
  a.bucket_node = t->bucket_node;
  a.n_buckets = t->n_buckets;
  a.theta = p->theta;
  a.theta_mono = p->theta * p->theta * p->theta * p->theta;
  a.period = p->period;
  a.order = p->order;
  a.n_replicas = p->n_replicas;
  a.n_cells = nc;
  a.n_parts = np;
  a.n_soft = ns;
  a.off_cells = oc;
  a.off_parts = op;
  a.off_soft = os;
  a.cells = (int2*)cells;
  a.parts = (int2*)parts;
  a.soft = (int2*)soft;
  a.error = err;
  a.nodef = nodef;
  a.boxf = boxf;
  a.period32 = (float)p->period;
  const int grid = (t->n_buckets + kWalkThreads - 1) / kWalkThreads;
  if (fill) walk_kernel<true><<<grid, kWalkThreads, 0, s>>>(a);
  else walk_kernel<false><<<grid, kWalkThreads, 0, s>>>(a);
  count_launch();
  CHG_CUDA(cudaGetLastError());
  int h_err = 0;
  CHG_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CHG_CUDA(cudaFreeAsync(block, s));
  CHG_CUDA(cudaStreamSynchronize(s));
  if (h_err)
    return record_error(CHANGA_E_TOO_LARGE, h_err == 1 ? "walk: tree deeper than 64 levels"
                                                       : "walk: traversal stack exhausted",
                        __FILE__, __LINE__);
  return 0;
}

extern "C" int changa_walk_count(const ChangaTreeView* tree, const ChangaWalkParams* p,
                                 int* n_cells, int* n_parts, int* n_soft, cudaStream_t s) {
  if (!n_cells || !n_parts || (p && p->order == 4 && !n_soft))
    return record_error(CHANGA_E_INVALID_ARG, "walk_count: outputs", __FILE__, __LINE__);
  return walk_launch(tree, p, false, n_cells, n_parts, n_soft, nullptr, nullptr, nullptr, nullptr,
                     nullptr, nullptr, s);
}

extern "C" int changa_walk_fill(const ChangaTreeView* tree, const ChangaWalkParams* p,
                                const long long* off_cells, const long long* off_parts,
                                const long long* off_soft, ILCell* cells, ILCell* parts,
                                ILCell* soft, cudaStream_t s) {
  if (!off_cells || !off_parts || !cells || !parts ||
      (p && p->order == 4 && (!off_soft || !soft)))
    return record_error(CHANGA_E_INVALID_ARG, "walk_fill: outputs", __FILE__, __LINE__);
  return walk_launch(tree, p, true, nullptr, nullptr, nullptr, off_cells, off_parts, off_soft,
                     cells, parts, soft, s);
}
