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
 * the local nodes on the path from the root to that bucket, not on the
 * order of the tests.  So one warp per target bucket reproduces the same
 * per-bucket sets from a stack of (source node, local level, replica)
 * entries in shared memory: each step pops up to 32 entries, tests each on
 * its own lane against the local node of its level, and pushes opened
 * children (or, when undecided, the entry one level down) back in lane
 * order.  The lanes keep 32 independent tests in flight per bucket, where a
 * thread per bucket would chain thousands of dependent loads; the stack
 * stays within a few hundred entries (a 32-wide last-in-first-out frontier)
 * and its capacity is checked.  The lists hold the same entries as the host
 * walk's, in this traversal's order, and each list's entries of one step
 * are written contiguously.
 *
 * Two launches: a count pass (per-bucket list lengths) and, after the
 * counts have become offsets, a fill pass; changa_walk runs both and the
 * prefix sums in between.
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
#include <atomic>
#include <cstring>
#include <type_traits>
#include <vector>

#include "chg_internal.h"
#include "list_eval.cuh"

namespace chg {
namespace {

constexpr int kWalkWarps = 4;      // warps (buckets) per block
constexpr int kWarpStack = 512;    // stack entries per warp (the deepest seen: 211)
constexpr int kWarpStackLarge = 1024;  // the re-run after a warp exhausted kWarpStack
constexpr int kChunk = 256;        // entries per pool chunk of the append pass
constexpr int kMaxChunks = 128;    // chunks per bucket and list in the append pass
enum { kCount = 0, kFill = 1, kAppend = 2 };

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
  /* append pass: per list a pool of kChunk-entry chunks, each chunk's
   * bucket and rank in that bucket's list; bucket_stride > 1 walks every
   * bucket_stride-th bucket only (the sampled count pass) and writes its
   * counts at b / bucket_stride */
  int2* pool[3];
  int* chunk_bucket[3];
  int* chunk_rank[3];
  unsigned int* pool_next;
  long long pool_chunks[3];
  int* overflow;
  int bucket_stride;
  /* per node, one 32-byte record for the traversal (see WalkNode) */
  const struct WalkNode* nodes;
  const float4* boxf;   // 2 n_nodes: {lesser.xyz, 0}, {greater.xyz, 0}
  const float2* hexf;   // n_nodes: {softening, monopole opening radius^2} (hexadecapole rules)
  float period32;
  /* two-phase walk.  Groups: nodes whose subtree holds few buckets (each
   * bucket in exactly one group, the group node on its chain).  Phase 1
   * walks a group node's chain once for all its buckets: its units are the
   * groups (group_node), the counts/offsets/lists above are the group's
   * prefix lists (entries accepted against the shared local nodes) and
   * entries still undecided at the group node go to the frontier.  Phase 2
   * walks each bucket from its group's frontier, after copying the group's
   * prefix lists into its own. */
  const int* group_node;     // n_groups
  int n_groups;
  const int* bucket_group;   // n_buckets: group of each bucket
  int* n_front;              // phase 1 count pass: frontier entries per group
  const long long* off_front;  // phase 1 fill pass: frontier offsets; phase 2: CSR over groups
  int2* front;               // phase 1 fill pass output, phase 2 input: {node, replica code}
  const long long* pre_off[2];  // phase 2: CSR over groups of the prefix cells / particles
  const int2* pre[2];
};

/* What the traversal reads of a source node, in one 32-byte record (two
 * 16-byte loads from one sector): FP32 centre and opening radius^2 for the
 * screened test, then {child0, child1, first, count}. */
struct __align__(32) WalkNode {
  float4 geo;
  int4 link;
};


constexpr float kU = 5.9604645e-08f;  // 2^-24, the FP32 unit roundoff

/* Each node's traversal record (FP32 centre and opening radius squared,
 * the latter formed in FP64 exactly as open_criterion forms it, and its
 * links) and its FP32 box. */
__global__ void walk_prep_kernel(const double* __restrict__ geom, const double* __restrict__ bbox,
                                 const int* __restrict__ info, long long n_nodes, double theta,
                                 double theta_mono, WalkNode* __restrict__ nodes,
                                 float4* __restrict__ boxf, float2* __restrict__ hexf) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n_nodes;
       g += (long long)gridDim.x * blockDim.x) {
    const double* gg = geom + 6 * g;
    const double kOpenGeom = 2.0 / sqrt(3.0);
    double radius = kOpenGeom * gg[3] / theta;
    if (radius < gg[3]) radius = gg[3];
    const int* f = info + 4 * g;
    nodes[g].geo = make_float4((float)gg[0], (float)gg[1], (float)gg[2], (float)(radius * radius));
    nodes[g].link = make_int4(f[0], f[1], f[2], f[3]);
    const double* b = bbox + 6 * g;
    boxf[2 * g] = make_float4((float)b[0], (float)b[1], (float)b[2], 0.0f);
    boxf[2 * g + 1] = make_float4((float)b[3], (float)b[4], (float)b[5], 0.0f);
    /* the monopole radius as open_criterion forms it, squared in FP64 */
    const double rm = kOpenGeom * gg[3] / theta_mono;
    hexf[g] = make_float2((float)gg[4], (float)(rm * rm));
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

/* v <= t decided from an FP32 value v within ev of the FP64 one and an
 * FP32 threshold t within et of the FP64 one: 1 certainly, 0 certainly
 * not, -1 too close (NaN or infinity give -1).  Each side carries two more
 * unit roundoffs for the rounding of the sums compared here. */
__device__ __forceinline__ int screen_le_t(float v, float ev, float t, float et) {
  const float mv = ev + 2.0f * kU * v, mt = et + 2.0f * kU * t;
  if (v + mv < t - mt) return 1;
  if (v - mv > t + mt) return 0;
  return -1;
}

/* open_softening in FP32 for a source g at c = cm + offset (FP32, with
 * the per-axis inputs cm and o for the error bound) against node `node`:
 * 1 certainly true, 0 certainly false, -1 too close to call.  Errors as in
 * open_criterion_screened: per axis the FP32 inputs and their sums carry at
 * most delta = 6u (|cm| + |o| + |node's cm or box face|) against the FP64
 * values; the softening sums 2 s_g + 2 s_node carry at most 3u of their
 * value, so their square at most 7u (bounded here by 8u). */
__device__ int open_softening_screened(const WalkArgs& a, float sg, const float* c,
                                       const float* cm, const float* o, int node) {
  const float4 nc = a.nodes[node].geo;
  const float sn = a.hexf[node].x;
  const float4 lo = a.boxf[2 * (size_t)node], hi = a.boxf[2 * (size_t)node + 1];
  const float ncm[3] = {nc.x, nc.y, nc.z};
  const float bl[3] = {lo.x, lo.y, lo.z}, bh[3] = {hi.x, hi.y, hi.z};
  float v = 0.0f, ev = 0.0f, d2 = 0.0f, e = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dk = 6.0f * kU * (fabsf(cm[k]) + fabsf(o[k]) + fabsf(ncm[k])) + 1e-30f;
    const float dx = c[k] - ncm[k];
    v += dx * dx;
    ev += 2.0f * fabsf(dx) * dk + 3.0f * dk * dk;
    const float db = 6.0f * kU * (fabsf(cm[k]) + fabsf(o[k]) + fabsf(bl[k]) + fabsf(bh[k])) + 1e-30f;
    const float gk = fmaxf(0.0f, fmaxf(bl[k] - c[k], c[k] - bh[k]));
    d2 += gk * gk;
    e += 2.0f * gk * db + 3.0f * db * db;
  }
  ev += 4.0f * kU * v;
  e += 4.0f * kU * d2;
  const float rr = 2.0f * sg + 2.0f * sn, rr2 = rr * rr;
  const int sph = screen_le_t(v, ev, rr2, 8.0f * kU * rr2);
  if (sph == 1) return 1;
  const float r2 = 4.0f * sg * sg;  // (2 s_g)^2
  const int box = screen_le_t(d2, e, r2, 4.0f * kU * r2);
  if (box == 1) return 1;
  return sph == 0 && box == 0 ? 0 : -1;
}

/* open_softening for source g at replica code `off` against node `node`:
 * the FP32 screen, then the FP64 test when too close to call. */
__device__ bool open_softening_fast(const WalkArgs& a, int g, int off, int node) {
  const float4 gf = a.nodes[g].geo;
  const float cm[3] = {gf.x, gf.y, gf.z};
  const float o[3] = {(float)((off & 7) - 3) * a.period32, (float)(((off >> 3) & 7) - 3) * a.period32,
                      (float)(((off >> 6) & 7) - 3) * a.period32};
  const float c[3] = {cm[0] + o[0], cm[1] + o[1], cm[2] + o[2]};
  const int r = open_softening_screened(a, a.hexf[g].x, c, cm, o, node);
  if (r >= 0) return r == 1;
  double o64[3];
  decode(off, a.period, o64);
  const double* gg = a.geom + 6 * (size_t)g;
  const double c64[3] = {gg[0] + o64[0], gg[1] + o64[1], gg[2] + o64[2]};
  return open_softening(a, g, node, c64);
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
__device__ int open_criterion_screened(const WalkArgs& a, const WalkNode& nd, int g, int local,
                                       bool local_bucket, int off) {
  if (nd.link.w <= 6) return 1;
  const float4 nf = nd.geo;
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
   * open it: a softening sphere that meets the local node, and then the
   * monopole radius (both screened in FP32, FP64 when too close to call) */
  if (a.order != 4) return 0;
  const int sof = open_softening_screened(a, a.hexf[g].x, c, cm, o, local);
  if (sof < 0) return open_criterion(a, g, local, local_bucket, off);
  if (sof == 0) return 0;
  const int mono = screen_le(d2, e, a.hexf[g].y);
  if (mono < 0) return open_criterion(a, g, local, local_bucket, off);
  return mono;
}

__device__ __forceinline__ int warp_excl_scan(int v, int& total) {
  const int lane = threadIdx.x & 31;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

/* Append pass: before a step adds `total` entries to list k (cnt so far),
 * the bucket's chunks are extended to hold them (lane 0, one atomic; the
 * warp's table maps list ranks to chunks; -1 once the pool is short). */
__device__ __forceinline__ void ensure_chunks(const WalkArgs& a, int k, int b, int* tab, int& nalloc,
                                              long long cnt, int total) {
  const int need = (int)((cnt + total + kChunk - 1) / kChunk);
  if (need > nalloc) {  // uniform over the warp
    if ((threadIdx.x & 31) == 0) {
      const int m = need - nalloc;
      long long c0 = -1;
      if (need <= kMaxChunks) {
        c0 = atomicAdd(a.pool_next + k, (unsigned)m);
        if (c0 + m > a.pool_chunks[k]) c0 = -1;
      }
      if (c0 < 0) atomicExch(a.overflow, 1);
      for (int i = 0; i < m && nalloc + i < kMaxChunks; ++i) {
        tab[nalloc + i] = c0 < 0 ? -1 : (int)(c0 + i);
        if (c0 >= 0) {
          a.chunk_bucket[k][c0 + i] = b;
          a.chunk_rank[k][c0 + i] = nalloc + i;
        }
      }
    }
    nalloc = need;
    __syncwarp();
  }
}

/* Entry q of list k of this bucket into its chunk. */
__device__ __forceinline__ void append_at(const WalkArgs& a, int k, const int* tab, long long q,
                                          int2 e) {
  const long long r = q / kChunk;
  const int c = r < kMaxChunks ? tab[r] : -1;
  if (c >= 0) a.pool[k][(size_t)c * kChunk + (q - r * kChunk)] = e;
}

/* PHASE 0: the whole walk of each bucket; 1: the shared walk of each group
 * down to its group node (prefix lists and frontier); 2: each bucket from
 * its group's frontier, after its group's prefix lists. */
template <int MODE, int STACK, int PHASE>
__global__ void __launch_bounds__(kWalkWarps * 32) walk_kernel(const WalkArgs a) {
  constexpr bool FILL = MODE == kFill;
  __shared__ int2 stk[kWalkWarps][STACK];
  __shared__ int chain[kWalkWarps][64];
  __shared__ int ctab[MODE == kAppend ? kWalkWarps : 1][3][MODE == kAppend ? kMaxChunks : 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const long long bl = ((long long)blockIdx.x * kWalkWarps + warp) * a.bucket_stride;
  if (bl >= (PHASE == 1 ? (long long)a.n_groups : (long long)a.n_buckets)) return;  // whole warp
  const int b = (int)bl;  // the unit: a bucket, or a group in phase 1
  const int bn = PHASE == 1 ? a.group_node[b] : a.bucket_node[b];
  if (bn < 0 || bn >= a.n_nodes) return;
  const int gid = PHASE == 2 ? a.bucket_group[b] : 0;
  const int gnode = PHASE == 2 ? a.group_node[gid] : -1;
  /* local nodes from the root down to this unit (and, phase 2, the level
   * of the bucket's group node on that chain) */
  int depth = 0, gdepth = -1;
  if (lane == 0) {
    int n = 0;
    for (int x = bn; x >= 0 && x < a.n_nodes && n < 65; x = a.parent[x]) ++n;
    if (n > 64) {
      depth = -1;
    } else {
      int k = n - 1;
      for (int x = bn; k >= 0; x = a.parent[x]) {
        if (x == gnode) gdepth = k;
        chain[warp][k--] = x;
      }
      depth = chain[warp][0] == 0 ? n - 1 : -1;
    }
  }
  depth = __shfl_sync(full, depth, 0);
  gdepth = __shfl_sync(full, gdepth, 0);
  if (depth < 0 || (PHASE == 2 && gdepth < 0)) {
    if (lane == 0) atomicExch(a.error, 1);
    return;
  }
  /* a group node with children is not a bucket: entries undecided at its
   * level go to the frontier instead of being opened */
  const bool unit_bucket = PHASE != 1 || (a.info[4 * (size_t)bn] < 0 && a.info[4 * (size_t)bn + 1] < 0);
  long long oc = 0, op = 0, os = 0, of = 0;
  if (FILL) {
    oc = a.off_cells[b];
    op = a.off_parts[b];
    os = a.off_soft ? a.off_soft[b] : 0;
    if (PHASE == 1) of = a.off_front[b];
  }
  int sp = 0;
  long long fpos = 0, fend = 0;  // phase 2: the group's frontier, fed when the stack is empty
  if (PHASE == 2) {
    fpos = a.off_front[gid];
    fend = a.off_front[gid + 1];
  } else {
    /* the root of every replica on the check list */
    const int nr = a.n_replicas, side = 2 * nr + 1, nrep = side * side * side;
    if (nrep > STACK) {  // uniform; the host re-runs the launch with the larger stack
      if (lane == 0) atomicExch(a.error, 2);
      return;
    }
    for (int r = lane; r < nrep; r += 32) {
      const int x = r / (side * side) - nr, y = (r / side) % side - nr, z = r % side - nr;
      stk[warp][r] = make_int2(0, (x + 3) | ((y + 3) << 3) | ((z + 3) << 6));
    }
    sp = nrep;
  }
  long long nc = 0, np = 0, ns = 0, nf = 0;
  int na[3] = {0, 0, 0};  // append pass: chunks taken per list
  if (PHASE == 2) {
    /* the group's prefix lists (entries accepted against the local nodes
     * the group walk covered, the same for every bucket of the group) */
    if (a.order == 4) {
      /* hexadecapole: the group's accepted cells split here into cells and
       * softened cells, by openSoftening against this bucket, as the
       * one-phase walk splits them when it accepts them */
      const unsigned below = (1u << lane) - 1u;
      const long long p0 = a.pre_off[0][gid], cnt = a.pre_off[0][gid + 1] - p0;
      for (long long j0 = 0; j0 < cnt; j0 += 32) {
        const int tot = (int)(cnt - j0 < 32 ? cnt - j0 : 32);
        int2 e = make_int2(-1, 0);
        bool soft = false;
        if (lane < tot) {
          e = a.pre[0][p0 + j0 + lane];
          if (e.x >= 0 && e.x < a.n_nodes) soft = open_softening_fast(a, e.x, (e.y >> 22) & 0x1ff, bn);
        }
        const unsigned mc = __ballot_sync(full, lane < tot && !soft);
        const unsigned ms = __ballot_sync(full, lane < tot && soft);
        if (MODE == kAppend) {
          if (mc) ensure_chunks(a, 0, b, ctab[warp][0], na[0], nc, __popc(mc));
          if (ms) ensure_chunks(a, 2, b, ctab[warp][2], na[2], ns, __popc(ms));
        }
        if (MODE != kCount && lane < tot) {
          if (!soft) {
            const long long q = nc + __popc(mc & below);
            if (FILL) a.cells[oc + q] = e;
            if (MODE == kAppend) append_at(a, 0, ctab[warp][0], q, e);
          } else {
            const long long q = ns + __popc(ms & below);
            if (FILL) a.soft[os + q] = e;
            if (MODE == kAppend) append_at(a, 2, ctab[warp][2], q, e);
          }
        }
        nc += __popc(mc);
        ns += __popc(ms);
      }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k == 0 && a.order == 4) continue;  // split above
      const long long p0 = a.pre_off[k][gid], cnt = a.pre_off[k][gid + 1] - p0;
      long long& n_k = k == 0 ? nc : np;
      if (MODE != kCount) {
        for (long long j0 = 0; j0 < cnt; j0 += 32) {
          const int tot = (int)(cnt - j0 < 32 ? cnt - j0 : 32);
          if (MODE == kAppend) ensure_chunks(a, k, b, ctab[warp][k], na[k], n_k + j0, tot);
          if (lane < tot) {
            const int2 e = a.pre[k][p0 + j0 + lane];
            if (FILL) (k == 0 ? a.cells[oc + n_k + j0 + lane] : a.parts[op + n_k + j0 + lane]) = e;
            if (MODE == kAppend) append_at(a, k, ctab[warp][k], n_k + j0 + lane, e);
          }
        }
      }
      n_k += cnt;
    }
  }
  __syncwarp();
  while (sp > 0 || fpos < fend) {
    int n;
    int2 e = make_int2(-1, 0);
    if (sp > 0) {
      n = sp < 32 ? sp : 32;
      const int top = sp - n;
      if (lane < n) e = stk[warp][top + lane];
      sp = top;
    } else {  // phase 2: the next frontier entries, tested one level below the group node
      n = (int)(fend - fpos < 32 ? fend - fpos : 32);
      if (lane < n) {
        const int2 f = a.front[fpos + lane];
        e = make_int2(f.x, ((gdepth + 1) << 16) | (f.y & 0xffff));
      }
      fpos += n;
    }
    __syncwarp();  // popped before anything is pushed over them
    /* kind: 0 cell, 1 softened cell, 2 particles, 3 open, 4 defer, 5 frontier
     * (phase 1: undecided at the group node), -1 none */
    int kind = -1, c0 = -1, c1 = -1, pfirst = 0, pcount = 0;
    const int g = e.x, level = e.y >> 16, code = e.y & 0xffff;
    if (g >= 0 && g < a.n_nodes && level <= depth) {  // memory safety
      const int local = chain[warp][level];
      const bool local_bucket = level == depth && unit_bucket;
      const WalkNode nd = a.nodes[g];
      const int open = open_criterion_screened(a, nd, g, local, local_bucket, code);
      if (open == 0) {
        bool softened = false;
        if (a.order == 4 && PHASE != 1)  // phase 2 splits the group's cells per bucket
          softened = open_softening_fast(a, g, code, bn);
        kind = softened ? 1 : 0;
      } else if (nd.link.x < 0 && nd.link.y < 0) {  // a source bucket: its particles
        kind = 2;
        pfirst = nd.link.z;
        pcount = nd.link.w;
      } else if (open == 1 || local_bucket) {
        kind = 3;
        c0 = nd.link.x;
        c1 = nd.link.y;
      } else {
        kind = level == depth ? 5 : 4;  // 5 only in phase 1 (level == depth is a bucket otherwise)
      }
    }
    /* pushes, in lane order; within a lane child 1 below child 0 */
    const int npush = kind == 3 ? (c0 >= 0) + (c1 >= 0) : (kind == 4 ? 1 : 0);
    int tpush;
    int pos = sp + warp_excl_scan(npush, tpush);
    if (sp + tpush > STACK) {  // uniform: every lane sees tpush
      if (lane == 0) atomicExch(a.error, 2);
      break;
    }
    if (kind == 3) {
      if (c1 >= 0) stk[warp][pos++] = make_int2(c1, (level << 16) | code);
      if (c0 >= 0) stk[warp][pos++] = make_int2(c0, (level << 16) | code);
    } else if (kind == 4) {
      stk[warp][pos] = make_int2(g, ((level + 1) << 16) | code);
    }
    sp += tpush;
    /* accepted cells, softened cells and particles, contiguous per step */
    const unsigned below = (1u << lane) - 1u;
    const unsigned mc = __ballot_sync(full, kind == 0), ms = __ballot_sync(full, kind == 1);
    int tpart;
    const int ppos = warp_excl_scan(kind == 2 ? pcount : 0, tpart);
    if (MODE == kAppend) {
      if (mc) ensure_chunks(a, 0, b, ctab[warp][0], na[0], nc, __popc(mc));
      if (ms) ensure_chunks(a, 2, b, ctab[warp][2], na[2], ns, __popc(ms));
      if (tpart) ensure_chunks(a, 1, b, ctab[warp][1], na[1], np, tpart);
    }
    if (kind == 0) {
      const long long q = nc + __popc(mc & below);
      if (FILL) a.cells[oc + q] = make_int2(g, code << 22);
      if (MODE == kAppend) append_at(a, 0, ctab[warp][0], q, make_int2(g, code << 22));
    }
    if (kind == 1) {
      const long long q = ns + __popc(ms & below);
      if (FILL) a.soft[os + q] = make_int2(g, code << 22);
      if (MODE == kAppend) append_at(a, 2, ctab[warp][2], q, make_int2(g, code << 22));
    }
    if (MODE != kCount && tpart) {
      /* the step's particle entries, 32 at a time: entry j belongs to the
       * first lane whose run ends after j (a binary search over the lanes'
       * inclusive ends), which lies ppos(owner) into that lane's run */
      const int incl = ppos + (kind == 2 ? pcount : 0);
      for (int j0 = 0; j0 < tpart; j0 += 32) {
        const int j = j0 + lane;
        int owner = 0;
#pragma unroll
        for (int bit = 16; bit > 0; bit >>= 1)
          if (__shfl_sync(full, incl, owner + bit - 1) <= j) owner += bit;
        const int o_pos = __shfl_sync(full, ppos, owner);
        const int o_first = __shfl_sync(full, pfirst, owner);
        const int o_code = __shfl_sync(full, code, owner);
        if (j < tpart) {
          const int2 e = make_int2(o_first + (j - o_pos), o_code << 22);
          if (FILL) a.parts[op + np + j] = e;
          if (MODE == kAppend) append_at(a, 1, ctab[warp][1], np + j, e);
        }
      }
    }
    if (PHASE == 1) {
      const unsigned mf = __ballot_sync(full, kind == 5);
      if (FILL && kind == 5) a.front[of + nf + __popc(mf & below)] = make_int2(g, code);
      nf += __popc(mf);
    }
    nc += __popc(mc);
    ns += __popc(ms);
    np += tpart;
    __syncwarp();  // pushes visible to the next pops
  }
  if (!FILL && lane == 0) {
    const int i = b / a.bucket_stride;
    a.n_cells[i] = (int)nc;
    a.n_parts[i] = (int)np;
    if (a.n_soft) a.n_soft[i] = (int)ns;
    if (PHASE == 1) a.n_front[i] = (int)nf;
  }
}

/* ---- fused walk and evaluation (FP32-mixed form, quadrupole) ----
 *
 * Phase 2 of the two-phase walk with the forces evaluated as the entries
 * are decided, instead of written to lists (the reference's prototype of a
 * walk that evaluates as it goes is gpuLocalTreeWalk, HostCUDA.cu:724-942).
 * A warp takes buckets from a work queue.  Per chunk of up to 32 targets it
 * keeps the paired target-parallel evaluation of the list kernels (lanes
 * own targets in G = 32 / nt groups; list_kernel_tp2): blocks of 32
 * entries are gathered, finished relative to the bucket, staged in pairs
 * and evaluated with pc_pair / pp_pair, and each block's sums are folded
 * into Kahan-compensated totals.  The blocks come, in this order of
 * preference, from the group's prefix cells and particles (phase 1's
 * output, shared by the group's buckets), from the cells the walk has
 * accepted so far, and from the particles of the source buckets it has
 * opened (queued as runs); a walk step runs only when no block is ready,
 * so each step adds at most 32 cells and 32 runs to buffers of 64.  Each of
 * the two evaluations has one call site in the kernel.  A bucket of more
 * than 32 targets is walked once per chunk.  The decisions, and so the
 * interactions, are the list walk's; only the summation order differs. */
constexpr int kFusedWarps = 4;        // warps per block (2 with the re-run's larger stack)
constexpr int kFusedWarpsPerSM = 16;  // the register cap: 128 per thread

struct FusedArgs {
  ListArgs cells;       // src: packed FP32-mixed cells, n_src: nodes; fperiod_f
  ListArgs parts;       // src: packed FP32-mixed particles, n_src: particles
  double* vars;         // n_src(parts) x 5 FP64, written per target
  unsigned int* queue;  // bucket counter, zero at launch
};

/* One loop per list, not unrolled, with the softening test on every block:
 * the walk and both evaluations share the SM's instruction cache, which the
 * list kernels' four unrolled loop copies per list overran (nfw8m: 83.9 ms
 * this way, 89.5 ms with those copies, 132 ms with one loop unrolled by 2;
 * a 168-register budget of 12 warps per SM was slower still). */
template <int STACK, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, kFusedWarpsPerSM / WARPS)
    walk_eval_kernel(const WalkArgs a, const FusedArgs f) {
  __shared__ int2 stk[WARPS][STACK];
  __shared__ int chain[WARPS][64];
  __shared__ int2 pcell[WARPS][64];  // accepted cells waiting for a block
  __shared__ int4 prun[WARPS][64];   // opened source buckets {first, count, code}
  __shared__ __align__(16) float4 stage[WARPS][16 * 6];
  __shared__ float ssoft[WARPS][32];
  __shared__ double red[WARPS][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const float4* pp = static_cast<const float4*>(f.parts.src);
  using CellT = std::integral_constant<bool, true>;
  using PartT = std::integral_constant<bool, false>;
  using Mark = std::integral_constant<bool, true>;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(f.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) return;
    const int bn = a.bucket_node[b];
    const int gid = a.bucket_group[b];
    if (bn < 0 || bn >= a.n_nodes || gid < 0 || gid >= a.n_groups) {  // memory safety
      if (lane == 0) atomicExch(a.error, 1);
      continue;
    }
    const int gnode = a.group_node[gid];
    int depth = 0, gdepth = -1;
    if (lane == 0) {
      int n = 0;
      for (int x = bn; x >= 0 && x < a.n_nodes && n < 65; x = a.parent[x]) ++n;
      if (n > 64) {
        depth = -1;
      } else {
        int k = n - 1;
        for (int x = bn; k >= 0; x = a.parent[x]) {
          if (x == gnode) gdepth = k;
          chain[warp][k--] = x;
        }
        depth = chain[warp][0] == 0 ? n - 1 : -1;
      }
    }
    depth = __shfl_sync(kFull, depth, 0);
    gdepth = __shfl_sync(kFull, gdepth, 0);
    const long long tbase = a.info[4 * (size_t)bn + 2];
    const int n = a.info[4 * (size_t)bn + 3];
    if (depth < 0 || gdepth < 0) {
      if (lane == 0) atomicExch(a.error, 1);
      continue;
    }
    if (n == 0) continue;  // no targets
    if (n < 0 || tbase < 0 || tbase + n > f.parts.n_src) {  // memory safety
      if (lane == 0) atomicExch(a.error, 3);
      continue;
    }
    /* the bucket's reference point: its first particle's split position */
    const float4 h0 = __ldg(pp + kPartPackF4 * tbase), l0 = __ldg(pp + kPartPackF4 * tbase + 1);
    const float3 chi = make_float3(h0.x, h0.y, h0.z), clo = make_float3(l0.x, l0.y, l0.z);

    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt, grp = lane / nt;
      const bool active = grp < G;
      const long long ti = tbase + t0 + (active ? lane - grp * nt : 0);
      const float4 th = __ldg(pp + kPartPackF4 * ti), tl = __ldg(pp + kPartPackF4 * ti + 1);
      const float tx = (th.x - chi.x) + (tl.x - clo.x), ty = (th.y - chi.y) + (tl.y - clo.y),
                  tz = (th.z - chi.z) + (tl.z - clo.z);
      const float tmass = th.w, tsoft = tl.w;
      const float tsmax = warp_max(active ? tsoft : 0.f);
      const float3 blo = make_float3(warp_min(active ? tx : 3.4e38f),
                                     warp_min(active ? ty : 3.4e38f),
                                     warp_min(active ? tz : 3.4e38f));
      const float3 bhi = make_float3(warp_max(active ? tx : -3.4e38f),
                                     warp_max(active ? ty : -3.4e38f),
                                     warp_max(active ? tz : -3.4e38f));
      const f2 tx2 = pk2(tx, tx), ty2 = pk2(ty, ty), tz2 = pk2(tz, tz);
      const f2 tmc = pk2(-tmass, -tmass), tmp = pk2(tmass, tmass);
      float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;
      float idc = 0.f;  // cells: the minimum of -(m_t + M) b (pc_pair's form)
      float idp = 0.f;  // particles: the maximum of (m_t + m) b

      /* One block: this lane's entry ent (valid when v) gathered, finished
       * and staged, then every staged pair on this lane's target. */
      auto eval_block = [&](int2 ent, bool v, auto cellc) {
        constexpr bool CELL = decltype(cellc)::value;
        constexpr int PW = CELL ? 6 : 2;
        const ListArgs& la = CELL ? f.cells : f.parts;
        RawRec<kMix, CELL> raw;
        gather_raw_entry<kMix, CELL>(la, v ? ent : make_int2(0, 0x49 << 22), raw);
        float4 rec[3];
        const float ls = finish_raw<kMix, CELL>(la, raw, v, chi, clo, rec);
        {
          float* pb = reinterpret_cast<float*>(stage[warp] + (lane >> 1) * PW);
          const int h = lane & 1;
          if constexpr (CELL) {
            stage_cell_half(pb, h, rec[0], rec[1], rec[2]);
          } else {
            pb[pair_slot(0, h)] = rec[0].x;
            pb[pair_slot(1, h)] = rec[0].y;
            pb[pair_slot(2, h)] = rec[0].z;
            pb[pair_slot(3, h)] = rec[0].w;
          }
        }
        ssoft[warp][lane] = ls;
        const float ss = warp_max(ls) + tsmax;
        const float near2 = ss * ss;
        __syncwarp();
        const float4* st = stage[warp];
        f2 ax2 = 0ull, ay2 = 0ull, az2 = 0ull, pot2 = 0ull, pw2 = 0ull;
        unsigned nmask = 0;
        float ex = 0.f, ey = 0.f, ez = 0.f, ep = 0.f;
        if constexpr (CELL) {
          auto body = [&](int p, auto near) {
            pc_pair<decltype(near)::value>(st + p * PW, &ssoft[warp][2 * p], tx2, ty2, tz2, tmc,
                                           tsoft, near2, pot2, pw2, ax2, ay2, az2, idc);
          };
          if (active) {
#pragma unroll 1
            for (int p = grp; p < 16; p += G) body(p, Mark{});
          }
        } else {
          auto body = [&](int p, auto mark) {
            pp_pair<decltype(mark)::value>(st + p * PW, p, tx2, ty2, tz2, tmp, near2, pot2, ax2,
                                           ay2, az2, idp, nmask);
          };
          if (active) {
#pragma unroll 1
            for (int p = grp; p < 16; p += G) body(p, Mark{});
          }
          pp_soft_pass(st, ssoft[warp], nmask, tx, ty, tz, tsoft, tmass, ex, ey, ez, ep, idp);
        }
        float x0, x1, y0, y1, z0, z1, p0, p1;
        up2(ax2, x0, x1);
        up2(ay2, y0, y1);
        up2(az2, z0, z1);
        up2(pot2, p0, p1);
        float pblk;
        if constexpr (CELL) {
          float w0_, w1_;
          up2(pw2, w0_, w1_);
          pblk = (p0 + p1) - 0.5f * (w0_ + w1_);
        } else {
          pblk = -((p0 + p1) + ep);
        }
        kahan_add(sx, cx, (x0 + x1) + ex);
        kahan_add(sy, cy, (y0 + y1) + ey);
        kahan_add(sz, cz, (z0 + z1) + ez);
        kahan_add(sp, cp, pblk);
        __syncwarp();  // the stage is rewritten by the next block
      };

      long long pc_pos = a.pre_off[0][gid], pc_end = a.pre_off[0][gid + 1];
      long long pp_pos = a.pre_off[1][gid], pp_end = a.pre_off[1][gid + 1];
      long long fpos = a.off_front[gid], fend = a.off_front[gid + 1];
      int sp_ = 0;       // walk stack entries
      int npc = 0;       // pending cells
      int nrun = 0;      // pending runs
      int roff = 0;      // particles of run 0 already evaluated
      int npart = 0;     // pending particles (over the runs, less roff)
      __syncwarp();
      for (;;) {
        const bool walked = sp_ == 0 && fpos >= fend;
        int which = -1;  // 0 a cell block, 1 a particle block
        int2 ent = make_int2(0, 0x49 << 22);
        bool v = false;
        if (pc_pos < pc_end) {
          const int ne = (int)min(32LL, pc_end - pc_pos);
          v = lane < ne;
          if (v) ent = a.pre[0][pc_pos + lane];
          pc_pos += ne;
          which = 0;
        } else if (pp_pos < pp_end) {
          const int ne = (int)min(32LL, pp_end - pp_pos);
          v = lane < ne;
          if (v) ent = a.pre[1][pp_pos + lane];
          pp_pos += ne;
          which = 1;
        } else if (npc >= 32 || (walked && npc > 0)) {
          const int ne = min(32, npc);
          v = lane < ne;
          if (v) ent = pcell[warp][lane];
          const int rest = npc - ne;  // at most 31
          const int2 keep = lane < rest ? pcell[warp][ne + lane] : make_int2(0, 0);
          __syncwarp();
          if (lane < rest) pcell[warp][lane] = keep;
          npc = rest;
          which = 0;
        } else if (npart >= 32 || (walked && npart > 0)) {
          /* the next min(32, npart) particles of the queued runs: entry j
           * belongs to the first run whose inclusive end exceeds j */
          const int ne = min(32, npart);
          int cnt = 0;
          int4 run = make_int4(0, 0, 0, 0);
          if (lane < nrun) {
            run = prun[warp][lane];
            cnt = run.y - (lane == 0 ? roff : 0);
          }
          int tot;
          const int excl = warp_excl_scan(cnt, tot);
          const int incl = excl + cnt;
          int owner = 0;
#pragma unroll
          for (int bit = 16; bit > 0; bit >>= 1)
            if (__shfl_sync(kFull, incl, owner + bit - 1) <= lane) owner += bit;
          const int o_excl = __shfl_sync(kFull, excl, owner);
          const int o_first = __shfl_sync(kFull, run.x, owner);
          const int o_code = __shfl_sync(kFull, run.z, owner);
          v = lane < ne;
          if (v) ent = make_int2(o_first + (owner == 0 ? roff : 0) + (lane - o_excl), o_code << 22);
          /* runs used up by the block, and how far into the next one */
          const int done = __popc(__ballot_sync(kFull, lane < nrun && incl <= ne));
          int used = __shfl_sync(kFull, excl, done & 31);
          if (done == 32) used = ne;  // 32 runs of one particle each
          roff = done < nrun ? (done == 0 ? roff : 0) + (ne - used) : 0;
          const int left = nrun - done;  // at most 64
          const int4 k0 = lane < left ? prun[warp][done + lane] : make_int4(0, 0, 0, 0);
          const int4 k1 = lane + 32 < left ? prun[warp][done + lane + 32] : make_int4(0, 0, 0, 0);
          __syncwarp();
          if (lane < left) prun[warp][lane] = k0;
          if (lane + 32 < left) prun[warp][lane + 32] = k1;
          nrun = left;
          npart -= ne;
          which = 1;
        } else if (walked) {
          break;
        }
        if (which == 0) {
          eval_block(ent, v, CellT{});
          continue;
        }
        if (which == 1) {
          eval_block(ent, v, PartT{});
          continue;
        }
        /* one walk step (walk_kernel, phase 2, quadrupole): up to 32 entries
         * tested; opened children pushed, accepted cells and opened source
         * buckets queued */
        int nst;
        int2 e = make_int2(-1, 0);
        if (sp_ > 0) {
          nst = sp_ < 32 ? sp_ : 32;
          const int top = sp_ - nst;
          if (lane < nst) e = stk[warp][top + lane];
          sp_ = top;
        } else {
          nst = (int)(fend - fpos < 32 ? fend - fpos : 32);
          if (lane < nst) {
            const int2 fr = a.front[fpos + lane];
            e = make_int2(fr.x, ((gdepth + 1) << 16) | (fr.y & 0xffff));
          }
          fpos += nst;
        }
        __syncwarp();
        int kind = -1, c0 = -1, c1 = -1, pfirst = 0, pcount = 0;
        const int src = e.x, level = e.y >> 16, code = e.y & 0xffff;
        if (src >= 0 && src < a.n_nodes && level <= depth) {
          const int local = chain[warp][level];
          const bool local_bucket = level == depth;
          const WalkNode nd = a.nodes[src];
          const int open = open_criterion_screened(a, nd, src, local, local_bucket, code);
          if (open == 0) {
            kind = 0;
          } else if (nd.link.x < 0 && nd.link.y < 0) {
            kind = 2;
            pfirst = nd.link.z;
            pcount = nd.link.w;
          } else if (open == 1 || local_bucket) {
            kind = 3;
            c0 = nd.link.x;
            c1 = nd.link.y;
          } else {
            kind = 4;
          }
        }
        const int npush = kind == 3 ? (c0 >= 0) + (c1 >= 0) : (kind == 4 ? 1 : 0);
        int tpush;
        int pos = sp_ + warp_excl_scan(npush, tpush);
        if (sp_ + tpush > STACK) {  // uniform; the host re-runs the launch with the larger stack
          if (lane == 0) atomicExch(a.error, 2);
          return;
        }
        if (kind == 3) {
          if (c1 >= 0) stk[warp][pos++] = make_int2(c1, (level << 16) | code);
          if (c0 >= 0) stk[warp][pos++] = make_int2(c0, (level << 16) | code);
        } else if (kind == 4) {
          stk[warp][pos] = make_int2(src, ((level + 1) << 16) | code);
        }
        sp_ += tpush;
        const unsigned mc = __ballot_sync(kFull, kind == 0);
        const unsigned mr = __ballot_sync(kFull, kind == 2 && pcount > 0);
        if (kind == 0) pcell[warp][npc + __popc(mc & below)] = make_int2(src, code << 22);
        if (kind == 2 && pcount > 0)
          prun[warp][nrun + __popc(mr & below)] = make_int4(pfirst, pcount, code, 0);
        int tpart;
        warp_excl_scan(kind == 2 && pcount > 0 ? pcount : 0, tpart);
        npc += __popc(mc);
        nrun += __popc(mr);
        npart += tpart;
        __syncwarp();  // pushes and queued entries visible to the next step
      }

      if (active) {
        red[warp][0][lane] = (double)sx - (double)cx;
        red[warp][1][lane] = (double)sy - (double)cy;
        red[warp][2][lane] = (double)sz - (double)cz;
        red[warp][3][lane] = (double)sp - (double)cp;
        red[warp][4][lane] = fmax(-(double)idc, (double)idp);
      }
      __syncwarp();
      if (lane < nt) {
        double rx = 0, ry = 0, rz = 0, rp = 0, ri = 0;
        for (int gg = 0; gg < G; ++gg) {
          const int l = gg * nt + lane;
          rx += red[warp][0][l];
          ry += red[warp][1][l];
          rz += red[warp][2][l];
          rp += red[warp][3][l];
          ri = fmax(ri, red[warp][4][l]);
        }
        double* out = f.vars + 5 * (tbase + t0 + lane);
        out[0] = rx;
        out[1] = ry;
        out[2] = rz;
        out[3] = rp;
        out[4] = ri;
      }
      __syncwarp();
    }
  }
}

/* The append pass's chunks into CSR order: entry j of chunk c (rank r of
 * bucket b) goes to off[b] + r kChunk + j when it lies inside b's list. */
__global__ void gather_chunks_kernel(const int2* __restrict__ pool, const int* __restrict__ cb,
                                     const int* __restrict__ cr, long long n_chunks,
                                     const long long* __restrict__ off, int2* __restrict__ out) {
  const long long total = n_chunks * kChunk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / kChunk;
    const int j = (int)(t - c * kChunk);
    const int b = cb[c];
    const long long pos = (long long)cr[c] * kChunk + j;
    if (off[b] + pos < off[b + 1]) out[off[b] + pos] = pool[t];
  }
}

/* Exclusive scan of n int counts into off64[0..n] and off32[0..n]: per-tile
 * sums, a one-block scan of the tile sums, then per-tile scans. */
constexpr int kScanThreads = 1024, kScanPer = 4, kScanTile = kScanThreads * kScanPer;

__global__ void scan_tile_sums_kernel(const int* __restrict__ in, int n, long long* __restrict__ ts) {
  __shared__ long long part[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  long long v = 0;
  for (int k = 0; k < kScanPer; ++k)
    if (base + k < n) v += in[base + k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    long long w = part[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (threadIdx.x == 0) ts[blockIdx.x] = w;
  }
}

__device__ long long block_exclusive_scan(long long v, long long* sh, long long& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    long long z = sh[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    sh[lane] = z;
  }
  __syncthreads();
  total = sh[31];
  const long long before = w ? sh[w - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void scan_tiles_kernel(long long* __restrict__ ts, int nt) {
  __shared__ long long sh[32];
  long long carry = 0;
  for (int b0 = 0; b0 < nt; b0 += kScanThreads) {
    const int i = b0 + threadIdx.x;
    const long long v = i < nt ? ts[i] : 0;
    long long tot;
    const long long ex = block_exclusive_scan(v, sh, tot);
    if (i < nt) ts[i] = carry + ex;
    carry += tot;
  }
}

__global__ void scan_apply_kernel(const int* __restrict__ in, int n, const long long* __restrict__ ts,
                                  long long* __restrict__ off64, int* __restrict__ off32) {
  __shared__ long long sh[32];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int v[kScanPer];
  long long sum = 0;
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    sum += v[k];
  }
  long long tot;
  long long run = ts[blockIdx.x] + block_exclusive_scan(sum, sh, tot);
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) {
      off64[base + k] = run;
      off32[base + k] = (int)run;
    }
    run += v[k];
    if (base + k == n - 1) {
      off64[n] = run;
      off32[n] = (int)run;
    }
  }
}

/* ---- groups for the two-phase walk ---- */

/* First particle of each bucket (buckets are numbered in particle order,
 * so the array rises). */
__global__ void bucket_first_kernel(const int* __restrict__ bucket_node, const int* __restrict__ info,
                                    long long n_nodes, int nb, int* __restrict__ bfirst) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nb;
       b += (long long)gridDim.x * blockDim.x) {
    const int x = bucket_node[b];
    bfirst[b] = (x >= 0 && x < n_nodes) ? info[4 * (size_t)x + 2] : 0;
  }
}

/* Buckets whose first particle lies in [lo, hi): the buckets of the node
 * covering those particles. */
__device__ __forceinline__ int buckets_in(const int* bfirst, int nb, int lo, int hi) {
  int a0 = 0, a1 = nb;  // first index with bfirst >= lo
  while (a0 < a1) {
    const int m = (a0 + a1) >> 1;
    if (bfirst[m] < lo) a0 = m + 1; else a1 = m;
  }
  int b0 = a0, b1 = nb;  // first index with bfirst >= hi
  while (b0 < b1) {
    const int m = (b0 + b1) >> 1;
    if (bfirst[m] < hi) b0 = m + 1; else b1 = m;
  }
  return b0 - a0;
}

/* Each bucket's group node: its highest ancestor whose subtree holds at
 * most gmax buckets (the bucket itself when its parent's holds more). */
__global__ void bucket_group_node_kernel(const int* __restrict__ bucket_node,
                                         const int* __restrict__ parent, const int* __restrict__ info,
                                         const int* __restrict__ bfirst, long long n_nodes, int nb,
                                         int gmax, int* __restrict__ gn) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nb;
       b += (long long)gridDim.x * blockDim.x) {
    int x = bucket_node[b];
    for (int up = 0; up < 64 && x >= 0 && x < n_nodes; ++up) {
      const int q = parent[x];
      if (q < 0 || q >= n_nodes) break;
      const int lo = info[4 * (size_t)q + 2], cnt = info[4 * (size_t)q + 3];
      if (buckets_in(bfirst, nb, lo, lo + cnt) > gmax) break;
      x = q;
    }
    gn[b] = x;
  }
}

/* 1 where a run of buckets with the same group node starts. */
__global__ void group_flag_kernel(const int* __restrict__ gn, int nb, int* __restrict__ flag) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nb;
       b += (long long)gridDim.x * blockDim.x)
    flag[b] = (b == 0 || gn[b] != gn[b - 1]) ? 1 : 0;
}

/* Group id of every bucket and the node of every group, from the
 * exclusive scan of the flags. */
__global__ void group_ids_kernel(const int* __restrict__ gn, const int* __restrict__ flag,
                                 const long long* __restrict__ excl, int nb,
                                 int* __restrict__ bucket_group, int* __restrict__ group_node) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nb;
       b += (long long)gridDim.x * blockDim.x) {
    const int gid = (int)(flag[b] ? excl[b] : excl[b] - 1);
    bucket_group[b] = gid;
    if (flag[b]) group_node[gid] = gn[b];
  }
}

}  // namespace
}  // namespace chg

using namespace chg;

static bool walk_args_ok(const ChangaTreeView* t, const ChangaWalkParams* p) {
  return t && p && t->geom && t->bbox && t->info && t->parent && t->bucket_node &&
         t->n_nodes > 0 && t->n_buckets >= 0 && p->theta > 0 && (p->order == 2 || p->order == 4) &&
         p->n_replicas >= 0 && p->n_replicas <= 3;
}

/* Node records and boxes for the screened tests (stream-ordered scratch,
 * freed by the caller). */
static int walk_setup(const ChangaTreeView* t, const ChangaWalkParams* p, WalkArgs& a, char** block,
                      cudaStream_t s) {
  prepare_pool();
  const size_t nn = (size_t)t->n_nodes;
  CHG_CUDA(cudaMallocAsync((void**)block,
                           256 + nn * (sizeof(WalkNode) + 2 * sizeof(float4) + sizeof(float2)), s));
  int* err = (int*)*block;
  WalkNode* nodes = (WalkNode*)(*block + 256);
  float4* boxf = (float4*)(nodes + nn);
  float2* hexf = (float2*)(boxf + 2 * nn);
  CHG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  long long g = (t->n_nodes + 255) / 256;
  const long long cap = (long long)sm_count() * 8;
  walk_prep_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(
      t->geom, t->bbox, t->info, t->n_nodes, p->theta,
      p->theta * p->theta * p->theta * p->theta, nodes, boxf, hexf);
  count_launch();
  a = WalkArgs{};
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
  a.error = err;
  a.nodes = nodes;
  a.boxf = boxf;
  a.hexf = hexf;
  a.period32 = (float)p->period;
  a.bucket_stride = 1;
  return 0;
}

/* Testing only: the first traversal with a 64-entry stack, so that the
 * re-run with the large stack is taken. */
static std::atomic<int> g_test_small_stack{0};
static std::atomic<long long> g_stack_reruns{0};  // launches re-run with the large stack

template <int STACK, int PHASE>
static void walk_launch_phase(const WalkArgs& a, int mode, int grid, cudaStream_t s) {
  if (mode == kFill) walk_kernel<kFill, STACK, PHASE><<<grid, kWalkWarps * 32, 0, s>>>(a);
  else if (mode == kAppend && PHASE != 1)
    walk_kernel<(PHASE != 1 ? kAppend : kCount), STACK, PHASE><<<grid, kWalkWarps * 32, 0, s>>>(a);
  else walk_kernel<kCount, STACK, PHASE><<<grid, kWalkWarps * 32, 0, s>>>(a);
  count_launch();
}

template <int STACK>
static void walk_launch_mode(const WalkArgs& a, int mode, int phase, int grid, cudaStream_t s) {
  if (phase == 1) walk_launch_phase<STACK, 1>(a, mode, grid, s);
  else if (phase == 2) walk_launch_phase<STACK, 2>(a, mode, grid, s);
  else walk_launch_phase<STACK, 0>(a, mode, grid, s);
}

/* One traversal.  The per-warp stack of kWarpStack entries keeps the
 * blocks' shared memory small enough for register-bound residency; a warp
 * that would exhaust it sets error 2 and stops, and the whole launch then
 * runs once more with kWarpStackLarge entries (every output of a launch is
 * rewritten by the re-run: per-bucket counts and entries, and in append
 * mode the pools, whose counters are reset first). */
static void walk_run(const WalkArgs& a, int mode, cudaStream_t s, int phase = 0) {
  const long long units = phase == 1 ? a.n_groups : a.n_buckets;
  const long long warps = (units + a.bucket_stride - 1) / a.bucket_stride;
  const int grid = (int)((warps + kWalkWarps - 1) / kWalkWarps);
  if (grid <= 0) return;
  if (g_test_small_stack.load()) walk_launch_mode<64>(a, mode, phase, grid, s);
  else walk_launch_mode<kWarpStack>(a, mode, phase, grid, s);
  int h = 0;
  if (cudaMemcpyAsync(&h, a.error, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess || h != 2)
    return;  // launch errors surface at the caller's next check
  if (cudaMemsetAsync(a.error, 0, sizeof(int), s) != cudaSuccess) return;
  if (mode == kAppend && a.pool_next &&
      cudaMemsetAsync(a.pool_next, 0, 64, s) != cudaSuccess)  // pool counters, overflow flag
    return;
  walk_launch_mode<kWarpStackLarge>(a, mode, phase, grid, s);
  g_stack_reruns.fetch_add(1);
}

static int walk_error(int h_err) {
  if (h_err == 3)
    return record_error(CHANGA_E_INVALID_ARG,
                        "walk_forces: a bucket's particles lie outside the particle array",
                        __FILE__, __LINE__);
  return record_error(CHANGA_E_TOO_LARGE, h_err == 1 ? "walk: tree deeper than 64 levels"
                                                     : "walk: traversal stack exhausted",
                      __FILE__, __LINE__);
}

static int walk_launch(const ChangaTreeView* t, const ChangaWalkParams* p, bool fill, int* nc,
                       int* np, int* ns, const long long* oc, const long long* op,
                       const long long* os, ILCell* cells, ILCell* parts, ILCell* soft,
                       cudaStream_t s) {
  if (!walk_args_ok(t, p))
    return record_error(CHANGA_E_INVALID_ARG, "walk: arguments", __FILE__, __LINE__);
  if (t->n_buckets == 0) return 0;
  WalkArgs a;
  char* block = nullptr;
  if (int rc = walk_setup(t, p, a, &block, s)) return rc;
  a.n_cells = nc;
  a.n_parts = np;
  a.n_soft = ns;
  a.off_cells = oc;
  a.off_parts = op;
  a.off_soft = os;
  a.cells = (int2*)cells;
  a.parts = (int2*)parts;
  a.soft = (int2*)soft;
  walk_run(a, fill ? kFill : kCount, s);
  CHG_CUDA(cudaGetLastError());
  int h_err = 0;
  CHG_CUDA(cudaMemcpyAsync(&h_err, a.error, sizeof(int), cudaMemcpyDeviceToHost, s));
  CHG_CUDA(cudaFreeAsync(block, s));
  CHG_CUDA(cudaStreamSynchronize(s));
  return h_err ? walk_error(h_err) : 0;
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

/* ---- both passes and the prefix sums, lists owned by the result ---- */

/* append-pass pool size over the sampled estimate of the entries */
static std::atomic<double> g_pool_factor{1.2};

extern "C" void changa_walk_set_pool_factor(double f) { g_pool_factor.store(f > 0 ? f : 0.0); }

extern "C" void changa_walk_set_test_small_stack(int on) { g_test_small_stack.store(on ? 1 : 0); }

/* Two-phase walk: groups of at most g_group_max buckets, for quadrupole
 * walks of at least g_group_min buckets (0 turns it off). */
static std::atomic<int> g_group_max{32};
static std::atomic<int> g_group_min{4096};

extern "C" void changa_walk_set_groups(int max_buckets, int min_tree_buckets) {
  g_group_max.store(max_buckets > 0 ? max_buckets : 0);
  g_group_min.store(min_tree_buckets > 0 ? min_tree_buckets : 0);
}

extern "C" long long changa_walk_stack_reruns(void) { return g_stack_reruns.load(); }

static void release_lists(ChangaWalkLists* out) {
  for (int k = 0; k < 3; ++k) {
    if (out->list[k]) cudaFreeAsync(out->list[k], 0);
    if (out->markers[k]) cudaFreeAsync(out->markers[k], 0);
    out->list[k] = nullptr;
    out->markers[k] = nullptr;
  }
}

extern "C" void changa_walk_lists_free(ChangaWalkLists* out) {
  if (!out) return;
  cudaDeviceSynchronize();  // the lists may be in use on any stream
  release_lists(out);
  std::memset(out, 0, sizeof(*out));
}

/* Stream-ordered scratch blocks of one call, freed together. */
struct Scratch {
  cudaStream_t s;
  std::vector<void*> blocks;
  void* alloc(size_t bytes) {
    void* q = nullptr;
    if (cudaMallocAsync(&q, bytes < 256 ? 256 : bytes, s) != cudaSuccess) return nullptr;
    blocks.push_back(q);
    return q;
  }
  void release() {
    for (void* q : blocks) cudaFreeAsync(q, s);
    blocks.clear();
  }
};

/* Groups of at most gmax buckets and phase 1 of the two-phase walk.
 * Phase 1 walks each group's node once: its chain down to the group node
 * is shared by all the group's buckets, so the entries accepted on it (the
 * group's prefix lists) and those still undecided at the group node (its
 * frontier) are the same for each of them.  Fills a's group fields and the
 * phase 2 inputs (prefix lists, frontier), in scratch of sc. */
static int walk_phase1(WalkArgs& a, const ChangaTreeView* t, int gmax, Scratch& sc,
                       cudaStream_t s) {
  const int nb = t->n_buckets;
  const int tiles = (nb + kScanTile - 1) / kScanTile;
  long long* ts = (long long*)sc.alloc((size_t)tiles * sizeof(long long));
  if (!ts) return record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__);
  int h_err = 0;
  int* bfirst = (int*)sc.alloc((size_t)nb * sizeof(int));
  int* gn = (int*)sc.alloc((size_t)nb * sizeof(int));
  int* flag = (int*)sc.alloc((size_t)nb * sizeof(int));
  long long* gex = (long long*)sc.alloc((size_t)(nb + 1) * sizeof(long long));
  int* gex32 = (int*)sc.alloc((size_t)(nb + 1) * sizeof(int));
  int* bucket_group = (int*)sc.alloc((size_t)nb * sizeof(int));
  int* group_node = (int*)sc.alloc((size_t)nb * sizeof(int));
  if (!bfirst || !gn || !flag || !gex || !gex32 || !bucket_group || !group_node)
    return record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__);
  const long long gb = ((long long)nb + 255) / 256, cap = (long long)sm_count() * 8;
  const int grid = (int)(gb < cap ? gb : cap);
  bucket_first_kernel<<<grid, 256, 0, s>>>(t->bucket_node, t->info, t->n_nodes, nb, bfirst);
  bucket_group_node_kernel<<<grid, 256, 0, s>>>(t->bucket_node, t->parent, t->info, bfirst,
                                                t->n_nodes, nb, gmax, gn);
  group_flag_kernel<<<grid, 256, 0, s>>>(gn, nb, flag);
  scan_tile_sums_kernel<<<tiles, kScanThreads, 0, s>>>(flag, nb, ts);
  scan_tiles_kernel<<<1, kScanThreads, 0, s>>>(ts, tiles);
  scan_apply_kernel<<<tiles, kScanThreads, 0, s>>>(flag, nb, ts, gex, gex32);
  group_ids_kernel<<<grid, 256, 0, s>>>(gn, flag, gex, nb, bucket_group, group_node);
  count_launch(7);
  long long ng_ll = 0;
  if (cudaMemcpyAsync(&ng_ll, gex + nb, sizeof(long long), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess || ng_ll <= 0 || ng_ll > nb)
    return record_error((int)cudaGetLastError(), "walk: groups", __FILE__, __LINE__);
  const int ng = (int)ng_ll;
  int* gcnt = (int*)sc.alloc((size_t)3 * ng * sizeof(int));
  long long* goff = (long long*)sc.alloc((size_t)3 * (ng + 1) * sizeof(long long));
  int* goff32 = (int*)sc.alloc((size_t)3 * (ng + 1) * sizeof(int));
  if (!gcnt || !goff || !goff32)
    return record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__);
  a.group_node = group_node;
  a.n_groups = ng;
  a.bucket_group = bucket_group;
  a.n_cells = gcnt;
  a.n_parts = gcnt + ng;
  a.n_soft = nullptr;
  a.n_front = gcnt + 2 * (size_t)ng;
  walk_run(a, kCount, s, 1);
  const int gtiles = (ng + kScanTile - 1) / kScanTile;
  for (int k = 0; k < 3; ++k) {
    scan_tile_sums_kernel<<<gtiles, kScanThreads, 0, s>>>(gcnt + (size_t)k * ng, ng, ts);
    scan_tiles_kernel<<<1, kScanThreads, 0, s>>>(ts, gtiles);
    scan_apply_kernel<<<gtiles, kScanThreads, 0, s>>>(gcnt + (size_t)k * ng, ng, ts,
                                                      goff + (size_t)k * (ng + 1),
                                                      goff32 + (size_t)k * (ng + 1));
    count_launch(3);
  }
  long long gtot[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k)
    cudaMemcpyAsync(&gtot[k], goff + (size_t)k * (ng + 1) + ng, sizeof(long long),
                    cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&h_err, a.error, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return record_error((int)cudaGetLastError(), "walk: group count", __FILE__, __LINE__);
  if (h_err) return walk_error(h_err);
  int2* pre_cells = (int2*)sc.alloc((size_t)(gtot[0] > 0 ? gtot[0] : 1) * sizeof(int2));
  int2* pre_parts = (int2*)sc.alloc((size_t)(gtot[1] > 0 ? gtot[1] : 1) * sizeof(int2));
  int2* front = (int2*)sc.alloc((size_t)(gtot[2] > 0 ? gtot[2] : 1) * sizeof(int2));
  if (!pre_cells || !pre_parts || !front)
    return record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__);
  a.off_cells = goff;
  a.off_parts = goff + (ng + 1);
  a.off_soft = nullptr;
  a.off_front = goff + 2 * (size_t)(ng + 1);
  a.cells = pre_cells;
  a.parts = pre_parts;
  a.soft = nullptr;
  a.front = front;
  walk_run(a, kFill, s, 1);
  /* phase 2 reads the group outputs */
  a.pre_off[0] = goff;
  a.pre_off[1] = goff + (ng + 1);
  a.pre[0] = pre_cells;
  a.pre[1] = pre_parts;
  a.off_cells = a.off_parts = a.off_soft = nullptr;
  a.cells = a.parts = a.soft = nullptr;
  a.n_front = nullptr;
  return 0;
}

extern "C" int changa_walk(const ChangaTreeView* t, const ChangaWalkParams* p,
                           ChangaWalkLists* out, cudaStream_t s) {
  if (!out) return record_error(CHANGA_E_INVALID_ARG, "walk: output", __FILE__, __LINE__);
  std::memset(out, 0, sizeof(*out));
  if (!walk_args_ok(t, p))
    return record_error(CHANGA_E_INVALID_ARG, "walk: arguments", __FILE__, __LINE__);
  const int nb = t->n_buckets;
  out->n_buckets = nb;
  out->order = p->order;
  if (nb == 0) return 0;
  const int nl = p->order == 4 ? 3 : 2;
  WalkArgs a;
  char* block = nullptr;
  if (int rc = walk_setup(t, p, a, &block, s)) return rc;
  Scratch sc{s, {block}};
  auto finish = [&](int rc) {
    sc.release();
    if (rc) {
      cudaStreamSynchronize(s);
      release_lists(out);
    }
    return rc;
  };
  auto alloc = [&](size_t bytes) { return sc.alloc(bytes); };
  int* cnt = (int*)alloc((size_t)3 * nb * sizeof(int));
  const int tiles = (nb + kScanTile - 1) / kScanTile;
  long long* ts = (long long*)alloc((size_t)tiles * sizeof(long long));
  long long* off = (long long*)alloc((size_t)3 * (nb + 1) * sizeof(long long));
  unsigned int* ctr = (unsigned int*)alloc(64);
  if (!cnt || !ts || !off || !ctr)
    return finish(record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__));
  int h_err = 0;
  /* Walks of many buckets run in two phases (walk_phase1); phase 2 walks
   * each bucket from its group's frontier, its lists starting with the
   * group's prefix. */
  int phase = 0;
  const int gmax = g_group_max.load();
  if (gmax > 0 && g_group_min.load() > 0 && nb >= g_group_min.load()) {
    if (int rc = walk_phase1(a, t, gmax, sc, s)) return finish(rc);
    phase = 2;
  }
  /* Large trees: one traversal appends the entries into pools of chunks
   * sized from a sampled count (every 16th bucket); small trees (where the
   * sample's fixed costs dominate) count, then fill. */
  bool appended = false;
  long long chunks[3] = {0, 0, 0};
  if (nb >= 16384) {
    const int stride = 16, nsamp = (nb + stride - 1) / stride;
    int* samp = (int*)alloc((size_t)3 * nsamp * sizeof(int));
    if (!samp)
      return finish(record_error(cudaErrorMemoryAllocation, "walk: memory", __FILE__, __LINE__));
    a.n_cells = samp;
    a.n_parts = samp + nsamp;
    a.n_soft = nl == 3 ? samp + 2 * nsamp : nullptr;
    a.bucket_stride = stride;
    walk_run(a, kCount, s, phase);
    a.bucket_stride = 1;
    std::vector<int> hs((size_t)nl * nsamp);
    if (cudaMemcpyAsync(hs.data(), samp, hs.size() * sizeof(int), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return finish(record_error((int)cudaGetLastError(), "walk: sample", __FILE__, __LINE__));
    bool ok = true;
    for (int k = 0; k < nl && ok; ++k) {
      double sum = 0;
      for (int i = 0; i < nsamp; ++i) sum += hs[(size_t)k * nsamp + i];
      chunks[k] = (long long)(sum * ((double)nb / nsamp) * g_pool_factor.load() / kChunk) + nb + 256;
      a.pool[k] = (int2*)alloc((size_t)chunks[k] * kChunk * sizeof(int2));
      a.chunk_bucket[k] = (int*)alloc((size_t)chunks[k] * sizeof(int));
      a.chunk_rank[k] = (int*)alloc((size_t)chunks[k] * sizeof(int));
      a.pool_chunks[k] = chunks[k];
      ok = a.pool[k] && a.chunk_bucket[k] && a.chunk_rank[k];
    }
    if (ok && cudaMemsetAsync(ctr, 0, 64, s) == cudaSuccess) {
      a.pool_next = ctr;
      a.overflow = reinterpret_cast<int*>(ctr + 8);
      a.n_cells = cnt;
      a.n_parts = cnt + nb;
      a.n_soft = nl == 3 ? cnt + 2 * (size_t)nb : nullptr;
      walk_run(a, kAppend, s, phase);
      appended = true;
    } else {
      cudaGetLastError();  // a pool that did not fit: count and fill instead
    }
  }
  if (!appended) {
    a.n_cells = cnt;
    a.n_parts = cnt + nb;
    a.n_soft = nl == 3 ? cnt + 2 * (size_t)nb : nullptr;
    walk_run(a, kCount, s, phase);
  }
  /* offsets (and the int32 markers) of every list */
  for (int k = 0; k < nl; ++k) {
    if (cudaMallocAsync((void**)&out->markers[k], (size_t)(nb + 1) * sizeof(int), s) != cudaSuccess)
      return finish(record_error(cudaErrorMemoryAllocation, "walk: markers", __FILE__, __LINE__));
    scan_tile_sums_kernel<<<tiles, kScanThreads, 0, s>>>(cnt + (size_t)k * nb, nb, ts);
    scan_tiles_kernel<<<1, kScanThreads, 0, s>>>(ts, tiles);
    scan_apply_kernel<<<tiles, kScanThreads, 0, s>>>(cnt + (size_t)k * nb, nb, ts,
                                                     off + (size_t)k * (nb + 1), out->markers[k]);
    count_launch(3);
  }
  long long tot[3] = {0, 0, 0};
  unsigned int hc[16] = {0};
  for (int k = 0; k < nl; ++k)
    cudaMemcpyAsync(&tot[k], off + (size_t)k * (nb + 1) + nb, sizeof(long long),
                    cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(hc, ctr, 64, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&h_err, a.error, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return finish(record_error((int)cudaGetLastError(), "walk: count", __FILE__, __LINE__));
  if (h_err) return finish(walk_error(h_err));
  for (int k = 0; k < nl; ++k) {
    if (tot[k] >= (1LL << 31) - 1)
      return finish(record_error(CHANGA_E_TOO_LARGE, "walk: list exceeds int32 markers", __FILE__,
                                 __LINE__));
    out->n_entries[k] = tot[k];
    if (cudaMallocAsync((void**)&out->list[k], (size_t)(tot[k] > 0 ? tot[k] : 1) * sizeof(ILCell),
                        s) != cudaSuccess)
      return finish(record_error(cudaErrorMemoryAllocation, "walk: lists", __FILE__, __LINE__));
  }
  const bool overflow = appended && hc[8] != 0;
  if (appended && !overflow) {
    for (int k = 0; k < nl; ++k) {
      const long long used = (long long)hc[k] < chunks[k] ? (long long)hc[k] : chunks[k];
      if (used == 0) continue;
      long long g = (used * kChunk + 255) / 256;
      const long long cap = (long long)sm_count() * 16;
      gather_chunks_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(
          a.pool[k], a.chunk_bucket[k], a.chunk_rank[k], used, off + (size_t)k * (nb + 1),
          (int2*)out->list[k]);
      count_launch();
    }
  } else {
    /* entries by a second traversal (small trees, or pools that ran short) */
    a.off_cells = off;
    a.off_parts = off + (nb + 1);
    a.off_soft = nl == 3 ? off + 2 * (size_t)(nb + 1) : nullptr;
    a.cells = (int2*)out->list[0];
    a.parts = (int2*)out->list[1];
    a.soft = nl == 3 ? (int2*)out->list[2] : nullptr;
    walk_run(a, kFill, s, phase);
    cudaMemcpyAsync(&h_err, a.error, sizeof(int), cudaMemcpyDeviceToHost, s);
  }
  out->passes = appended ? (overflow ? 3 : 1) : 2;
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return finish(record_error((int)cudaGetLastError(), "walk: entries", __FILE__, __LINE__));
  if (h_err) return finish(walk_error(h_err));
  return finish(0);
}

/* ---- fused walk and evaluation: the host side ---- */

template <int STACK, int WARPS>
static cudaError_t launch_walk_eval(const WalkArgs& a, const FusedArgs& f, cudaStream_t s) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, walk_eval_kernel<STACK, WARPS>, WARPS * 32, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const long long want = ((long long)a.n_buckets + WARPS - 1) / WARPS;
  const long long cap = (long long)sm_count() * per_sm;
  walk_eval_kernel<STACK, WARPS><<<(int)(want < cap ? want : cap), WARPS * 32, 0, s>>>(a, f);
  count_launch();
  return cudaGetLastError();
}

extern "C" int changa_walk_forces(const ChangaTreeView* t, const ChangaWalkParams* p,
                                  const double* moments, const double* parts, long long n_parts,
                                  const ChangaEwaldParams* ewald, double* vars, cudaStream_t s) {
  if (!walk_args_ok(t, p) || p->order != 2)
    return record_error(CHANGA_E_INVALID_ARG, "walk_forces: arguments (quadrupole trees)",
                        __FILE__, __LINE__);
  if (!moments || !parts || !vars || n_parts <= 0)
    return record_error(CHANGA_E_INVALID_ARG, "walk_forces: arrays", __FILE__, __LINE__);
  if (t->n_buckets == 0) return 0;
  WalkArgs a;
  char* block = nullptr;
  if (int rc = walk_setup(t, p, a, &block, s)) return rc;
  Scratch sc{s, {block}};
  auto finish = [&](int rc) {
    sc.release();
    if (rc) cudaStreamSynchronize(s);
    return rc;
  };
  const size_t cb = (size_t)t->n_nodes * kCellPackF4 * sizeof(float4);
  const size_t pb = (size_t)n_parts * kPartPackF4 * sizeof(float4);
  float4* pc = (float4*)sc.alloc(cb);
  float4* ppk = (float4*)sc.alloc(pb);
  unsigned int* queue = (unsigned int*)sc.alloc(256);
  if (!pc || !ppk || !queue)
    return finish(record_error(cudaErrorMemoryAllocation, "walk_forces: memory", __FILE__, __LINE__));
  cudaError_t e;
  if ((e = launch_pack_cells(moments, t->n_nodes, pc, s)) != cudaSuccess ||
      (e = launch_pack_parts(parts, n_parts, ppk, s)) != cudaSuccess)
    return finish(record_error((int)e, "walk_forces: pack", __FILE__, __LINE__));
  const int gmax = g_group_max.load() > 0 ? g_group_max.load() : 32;
  if (int rc = walk_phase1(a, t, gmax, sc, s)) return finish(rc);
  FusedArgs f{};
  f.cells.src = pc;
  f.cells.n_src = t->n_nodes;
  f.cells.fperiod_f = (float)p->period;
  f.cells.fperiod_d = p->period;
  f.parts.src = ppk;
  f.parts.n_src = n_parts;
  f.parts.fperiod_f = (float)p->period;
  f.parts.fperiod_d = p->period;
  f.vars = vars;
  f.queue = queue;
  /* a warp that would exhaust its stack stops with error 2; the launch
   * then runs again with the larger stack and rewrites every target */
  int h_err = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if ((e = cudaMemsetAsync(queue, 0, sizeof(unsigned int), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(a.error, 0, sizeof(int), s)) != cudaSuccess)
      return finish(record_error((int)e, "walk_forces: reset", __FILE__, __LINE__));
    if (attempt == 1) {
      e = launch_walk_eval<kWarpStackLarge, 2>(a, f, s);
      g_stack_reruns.fetch_add(1);
    } else if (g_test_small_stack.load()) {
      e = launch_walk_eval<32, kFusedWarps>(a, f, s);  // runs out on the first opening steps
    } else {
      e = launch_walk_eval<kWarpStack, kFusedWarps>(a, f, s);
    }
    if (e != cudaSuccess) return finish(record_error((int)e, "walk_forces: launch", __FILE__, __LINE__));
    if ((e = cudaMemcpyAsync(&h_err, a.error, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return finish(record_error((int)e, "walk_forces: status", __FILE__, __LINE__));
    if (h_err != 2) break;
  }
  if (h_err) return finish(walk_error(h_err));
  if (ewald && (e = launch_ewald_fp(kMix, parts, n_parts, nullptr, n_parts, *ewald, vars, s)) !=
                   cudaSuccess)
    return finish(record_error((int)e, "walk_forces: ewald", __FILE__, __LINE__));
  return finish(0);
}
