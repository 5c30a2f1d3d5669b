/*
 * Tree build on the GPU: the host build of changa_gb300/host/tree.cpp
 * (ChaNGa's TreePiece::buildTree path restated for one tree piece), step
 * for step, so the arrays equal the host's:
 *
 *   1. bounding box of the positions in float, made cubical with the key
 *      slop (TreePiece.cpp:141-165);
 *   2. 63-bit Morton keys, 21 bits per axis (the host's own key; ChaNGa's
 *      SFC.h lives in the absent N-BodyShop utility);
 *   3. a stable LSD radix sort of (key, index), 4-bit digits, so equal keys
 *      keep index order exactly as std::sort on (key, index) pairs does;
 *   4. the binary tree level by level: a node of more than nBucket
 *      particles splits where key bit (62 - level) turns on
 *      (GenericTreeNode.h:473-599), nodes are numbered breadth-first with
 *      empty children dropped (DataManager.cpp:768-858), buckets in key
 *      order;
 *   5. per node: mass, mass-weighted softening and centre of mass, second
 *      moments about the centre of mass, the particle bounding box and the
 *      radius rules (bucket: farthest particle, else half the spatial cell's
 *      diagonal; internal: farthest bounding-box corner;
 *      MultipoleMoments.h:206-352, 460-526, GenericTreeNode.h:219-255):
 *      buckets add their particles one at a time (a thread per bucket),
 *      then each level's internal nodes add their children, deepest level
 *      first.
 *
 * The arithmetic is the host build's, in its order, and this file is
 * compiled without FMA contraction (as the host code is), so every array
 * equals the host's bit for bit.
 */
#include <vector>

#include "chg_internal.h"

namespace chg {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortRun = 16;  // elements per thread per tile
constexpr int kSortTile = kSortThreads * kSortRun;
constexpr int kDigits = 16;   // 4-bit digits

__global__ void box_partial_kernel(const double* __restrict__ pos, long long n,
                                   float* __restrict__ part) {
  __shared__ float smin[3][256], smax[3][256];
  float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const float v = (float)pos[3 * i + k];
      lo[k] = fminf(lo[k], v);
      hi[k] = fmaxf(hi[k], v);
    }
  for (int k = 0; k < 3; ++k) {
    smin[k][threadIdx.x] = lo[k];
    smax[k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        smin[k][threadIdx.x] = fminf(smin[k][threadIdx.x], smin[k][threadIdx.x + o]);
        smax[k][threadIdx.x] = fmaxf(smax[k][threadIdx.x], smax[k][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) {
      part[6 * blockIdx.x + k] = smin[k][0];
      part[6 * blockIdx.x + 3 + k] = smax[k][0];
    }
}

/* The cubical box from the partial extents (one thread; the host's float
 * arithmetic). */
__global__ void box_final_kernel(const float* __restrict__ part, int nparts, double* __restrict__ box) {
  float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
  for (int b = 0; b < nparts; ++b)
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], part[6 * b + k]);
      hi[k] = fmaxf(hi[k], part[6 * b + 3 + k]);
    }
  float size[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  float mx = size[0] > size[1] ? size[0] : size[1];
  mx = mx > size[2] ? mx : size[2];
  const float fEps = 1.0f + 1.91e-6f;
  const float half = (float)(fEps * 0.5 * mx);
  for (int k = 0; k < 3; ++k) {
    const float c = 0.5f * (lo[k] + hi[k]);
    box[k] = (double)(c - half);
    box[3 + k] = (double)(c + half);
  }
  if (!(box[3] > box[0]))
    for (int k = 0; k < 3; ++k) {
      box[k] -= 0.5;
      box[3 + k] += 0.5;
    }
}

__device__ __forceinline__ unsigned long long spread3(unsigned long long v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

__global__ void keys_kernel(const double* __restrict__ pos, long long n, const double* __restrict__ box,
                            unsigned long long* __restrict__ keys, int* __restrict__ idx) {
  const double b0 = box[0], b1 = box[1], b2 = box[2], b3 = box[3], b4 = box[4], b5 = box[5];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    unsigned long long q[3];
    const double lo[3] = {b0, b1, b2}, hi[3] = {b3, b4, b5};
    for (int k = 0; k < 3; ++k) {
      double s = (pos[3 * i + k] - lo[k]) / (hi[k] - lo[k]);
      if (s < 0) s = 0;
      const double f = s * 2097152.0;
      q[k] = f >= 2097151.0 ? 2097151ULL : (unsigned long long)f;
    }
    keys[i] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
    idx[i] = (int)i;
  }
}

/* Radix pass 1: per-tile digit counts, counts[digit * tiles + tile]. */
__global__ void __launch_bounds__(kSortThreads) radix_count_kernel(
    const unsigned long long* __restrict__ keys, long long n, int shift, int* __restrict__ counts,
    int tiles) {
  __shared__ int h[kDigits];
  if (threadIdx.x < kDigits) h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortTile + (long long)threadIdx.x * kSortRun;
  int c[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) c[d] = 0;
  for (int j = 0; j < kSortRun; ++j) {
    const long long i = base + j;
    if (i < n) {
      const int d = (int)((keys[i] >> shift) & (kDigits - 1));
#pragma unroll
      for (int dd = 0; dd < kDigits; ++dd) c[dd] += dd == d;
    }
  }
#pragma unroll
  for (int d = 0; d < kDigits; ++d)
    if (c[d]) atomicAdd(&h[d], c[d]);
  __syncthreads();
  if (threadIdx.x < kDigits) counts[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

/* Exclusive scan of the digit-major counts (one block). */
__global__ void scan_kernel(int* __restrict__ v, int n) {
  __shared__ int carry;
  __shared__ int buf[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < n; b0 += 1024) {
    const int i = b0 + threadIdx.x;
    const int x = i < n ? v[i] : 0;
    buf[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int y = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < n) v[i] = carry + buf[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}

/* Radix pass 2: stable scatter.  Each thread owns a run of kSortRun
 * consecutive elements; its offset for digit d is the tile's base for d
 * plus the count of d in the runs of the threads before it. */
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const unsigned long long* __restrict__ keys, const int* __restrict__ vals, long long n,
    int shift, const int* __restrict__ offsets, int tiles, unsigned long long* __restrict__ okeys,
    int* __restrict__ ovals) {
  __shared__ int pre[kDigits][kSortThreads + 1];
  const long long base = (long long)blockIdx.x * kSortTile + (long long)threadIdx.x * kSortRun;
  int c[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) c[d] = 0;
  for (int j = 0; j < kSortRun; ++j) {
    const long long i = base + j;
    if (i < n) {
      const int d = (int)((keys[i] >> shift) & (kDigits - 1));
#pragma unroll
      for (int dd = 0; dd < kDigits; ++dd) c[dd] += dd == d;
    }
  }
#pragma unroll
  for (int d = 0; d < kDigits; ++d) pre[d][threadIdx.x + 1] = c[d];
  if (threadIdx.x == 0)
    for (int d = 0; d < kDigits; ++d) pre[d][0] = 0;
  __syncthreads();
  /* inclusive scan along threads for each digit (threads 0..15 scan one
   * digit each, 256 steps) */
  if (threadIdx.x < kDigits) {
    int acc = 0;
    for (int t = 1; t <= kSortThreads; ++t) {
      acc += pre[threadIdx.x][t];
      pre[threadIdx.x][t] = acc;
    }
  }
  __syncthreads();
  int pos[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) pos[d] = offsets[d * tiles + blockIdx.x] + pre[d][threadIdx.x];
  for (int j = 0; j < kSortRun; ++j) {
    const long long i = base + j;
    if (i < n) {
      const unsigned long long k = keys[i];
      const int d = (int)((k >> shift) & (kDigits - 1));
      int p = 0;
#pragma unroll
      for (int dd = 0; dd < kDigits; ++dd)
        if (dd == d) p = pos[dd]++;
      okeys[p] = k;
      ovals[p] = vals[i];
    }
  }
}

/* Sorted particles in the parts layout. */
__global__ void gather_parts_kernel(const double* __restrict__ pos, const double* __restrict__ mass,
                                    const double* __restrict__ soft, const int* __restrict__ perm,
                                    long long n, double* __restrict__ parts) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long j = perm[i];
    double* o = parts + 5 * i;
    o[0] = mass[j];
    o[1] = soft[j];
    o[2] = pos[3 * j];
    o[3] = pos[3 * j + 1];
    o[4] = pos[3 * j + 2];
  }
}

/* One level of the breadth-first build.  In: the level's nodes {first,
 * count} and split cells; out: per node the number of non-empty children
 * (0 for buckets) and their ranges. */
struct LevelNode {
  int first, count;
};

__global__ void split_kernel(const unsigned long long* __restrict__ keys, const LevelNode* __restrict__ nodes,
                             int n_nodes, int level, int n_bucket, int* __restrict__ nchild,
                             int* __restrict__ mid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  const LevelNode nd = nodes[i];
  if (nd.count <= n_bucket || level >= 60) {
    nchild[i] = 0;
    mid[i] = -1;
    return;
  }
  const unsigned long long mask = 1ULL << (62 - level);
  int lo = nd.first, hi = nd.first + nd.count;
  while (lo < hi) {
    const int md = lo + (hi - lo) / 2;
    if (keys[md] & mask) hi = md;
    else lo = md + 1;
  }
  mid[i] = lo;
  nchild[i] = (lo > nd.first) + (nd.first + nd.count > lo);
}

/* Writes the next level's nodes; nodes of this level get their info. */
__global__ void link_kernel(const LevelNode* __restrict__ nodes, const double* __restrict__ split,
                            int n_nodes, int level, int base, int next_base,
                            const int* __restrict__ nchild_scan, const int* __restrict__ mid,
                            LevelNode* __restrict__ next, double* __restrict__ next_split,
                            int* __restrict__ info, int* __restrict__ parent,
                            double* __restrict__ cell) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  const LevelNode nd = nodes[i];
  const int me = base + i;
  int* f = info + 4 * (size_t)me;
  f[0] = f[1] = -1;
  f[2] = nd.first;
  f[3] = nd.count;
  const double* sp = split + 6 * (size_t)i;
  for (int k = 0; k < 6; ++k) cell[6 * (size_t)me + k] = sp[k];
  if (mid[i] < 0) return;
  const int axis = level % 3;
  const double m = 0.5 * (sp[3 + axis] + sp[axis]);
  int slot = nchild_scan[i];
  const int ranges[2][2] = {{nd.first, mid[i] - nd.first}, {mid[i], nd.first + nd.count - mid[i]}};
  for (int c = 0; c < 2; ++c) {
    if (ranges[c][1] <= 0) continue;
    const int child = next_base + slot;
    next[slot] = LevelNode{ranges[c][0], ranges[c][1]};
    double* ns = next_split + 6 * (size_t)slot;
    for (int k = 0; k < 6; ++k) ns[k] = sp[k];
    if (c == 0) ns[3 + axis] = m;
    else ns[axis] = m;
    f[c] = child;
    parent[child] = me;
    ++slot;
  }
}

/* Moments, box and radius of every node, as the host build forms them:
 * buckets add their particles one at a time, internal nodes add their
 * children (MultipoleMoments.h:206-352; the radius rules of
 * GenericTreeNode.h:219-255 and MultipoleMoments.h:462-476).  The
 * operations and their order are the host's, and this file is compiled
 * without FMA contraction as the host code is, so the results are the
 * host's bit for bit. */
__device__ __forceinline__ void mom_add_particle(double* m, double pm, double ps, const double* p) {
  const double m1 = m[2];
  m[2] += pm;
  if (m[2] == 0.0) {
    m[1] = 0.5 * (m[1] + ps);
    for (int k = 0; k < 3; ++k) m[3 + k] = 0.5 * (m[3 + k] + p[k]);
    return;
  }
  m[1] = (m1 * m[1] + pm * ps) / m[2];
  const double c0 = m[3], c1 = m[4], c2 = m[5];
  m[3] = (m1 * c0 + pm * p[0]) / m[2];
  m[4] = (m1 * c1 + pm * p[1]) / m[2];
  m[5] = (m1 * c2 + pm * p[2]) / m[2];
  double d0 = c0 - m[3], d1 = c1 - m[4], d2 = c2 - m[5];
  m[6] += m1 * d0 * d0;
  m[9] += m1 * d1 * d1;
  m[11] += m1 * d2 * d2;
  m[7] += m1 * d0 * d1;
  m[8] += m1 * d0 * d2;
  m[10] += m1 * d1 * d2;
  d0 = p[0] - m[3];
  d1 = p[1] - m[4];
  d2 = p[2] - m[5];
  m[6] += pm * d0 * d0;
  m[9] += pm * d1 * d1;
  m[11] += pm * d2 * d2;
  m[7] += pm * d0 * d1;
  m[8] += pm * d0 * d2;
  m[10] += pm * d1 * d2;
}

__device__ __forceinline__ void mom_add_node(double* m, const double* c) {
  const double m1 = m[2];
  m[2] += c[2];
  if (m[2] == 0.0) {
    m[1] = 0.5 * (m[1] + c[1]);
    for (int k = 0; k < 3; ++k) m[3 + k] = 0.5 * (m[3 + k] + c[3 + k]);
    return;
  }
  if (m1 == 0.0) {
    for (int k = 0; k < 12; ++k) m[k] = c[k];
    return;
  }
  if (c[2] == 0.0) return;
  m[1] = (m1 * m[1] + c[2] * c[1]) / m[2];
  const double c0 = m[3], c1 = m[4], c2 = m[5];
  m[3] = (m1 * c0 + c[2] * c[3]) / m[2];
  m[4] = (m1 * c1 + c[2] * c[4]) / m[2];
  m[5] = (m1 * c2 + c[2] * c[5]) / m[2];
  double d0 = c0 - m[3], d1 = c1 - m[4], d2 = c2 - m[5];
  m[6] += m1 * d0 * d0;
  m[9] += m1 * d1 * d1;
  m[11] += m1 * d2 * d2;
  m[7] += m1 * d0 * d1;
  m[8] += m1 * d0 * d2;
  m[10] += m1 * d1 * d2;
  d0 = c[3] - m[3];
  d1 = c[4] - m[4];
  d2 = c[5] - m[5];
  m[6] += c[6] + c[2] * d0 * d0;
  m[9] += c[9] + c[2] * d1 * d1;
  m[11] += c[11] + c[2] * d2 * d2;
  m[7] += c[7] + c[2] * d0 * d1;
  m[8] += c[8] + c[2] * d0 * d2;
  m[10] += c[10] + c[2] * d1 * d2;
}

__device__ __forceinline__ void store_node(long long node, const double* m, const double* b,
                                           double* __restrict__ moments, double* __restrict__ bbox,
                                           double* __restrict__ geom) {
  double* o = moments + 12 * node;
#pragma unroll
  for (int k = 0; k < 12; ++k) o[k] = m[k];
  double* ob = bbox + 6 * node;
#pragma unroll
  for (int k = 0; k < 6; ++k) ob[k] = b[k];
  double* g = geom + 6 * node;
  g[0] = m[3];
  g[1] = m[4];
  g[2] = m[5];
  g[3] = m[0];
  g[4] = m[1];
  g[5] = m[2];
}

/* Buckets (one thread each): calculateRadiusBox on the spatial cell, the
 * particles added in key order, then the farthest particle from the centre
 * of mass. */
__global__ void bucket_props_kernel(const double* __restrict__ parts, const int* __restrict__ info,
                                    const double* __restrict__ cell, long long n_nodes,
                                    double* __restrict__ moments, double* __restrict__ bbox,
                                    double* __restrict__ geom) {
  for (long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x; node < n_nodes;
       node += (long long)gridDim.x * blockDim.x) {
    const int* f = info + 4 * node;
    if (f[0] >= 0 || f[1] >= 0) continue;
    const long long first = f[2], count = f[3];
    double m[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = 0.0;
    double b[6] = {HUGE_VAL, HUGE_VAL, HUGE_VAL, -HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    const double* sp = cell + 6 * node;
    const double dx = sp[3] - sp[0], dy = sp[4] - sp[1], dz = sp[5] - sp[2];
    m[0] = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
    if (m[0] <= 0.0) {
      if (count > 1) {
        const double* p1 = parts + 5 * first + 2;
        double r2 = 0.0;
        for (long long i = first + 1; i < first + count; ++i) {
          const double* p = parts + 5 * i + 2;
          const double d = (p1[0] - p[0]) * (p1[0] - p[0]) + (p1[1] - p[1]) * (p1[1] - p[1]) +
                           (p1[2] - p[2]) * (p1[2] - p[2]);
          if (d > r2) r2 = d;
        }
        if (r2 > 0) m[0] = sqrt(r2);
      } else {
        m[0] = 1.0;
      }
    }
    for (long long i = first; i < first + count; ++i) {
      const double* p = parts + 5 * i;
      mom_add_particle(m, p[0], p[1], p + 2);
      for (int k = 0; k < 3; ++k) {
        if (p[2 + k] < b[k]) b[k] = p[2 + k];
        if (p[2 + k] > b[3 + k]) b[3 + k] = p[2 + k];
      }
    }
    if (count > 1) {
      double r2 = 0.0;
      for (long long i = first; i < first + count; ++i) {
        const double* p = parts + 5 * i + 2;
        const double d = (m[3] - p[0]) * (m[3] - p[0]) + (m[4] - p[1]) * (m[4] - p[1]) +
                         (m[5] - p[2]) * (m[5] - p[2]);
        if (d > r2) r2 = d;
      }
      if (r2 > 0.0) m[0] = sqrt(r2);
    }
    store_node(node, m, b, moments, bbox, geom);
  }
}

/* Internal nodes of one level (one thread each), after the level below:
 * the children's moments and boxes added in order, then the farthest
 * corner of the box from the centre of mass. */
__global__ void internal_props_kernel(const int* __restrict__ info, long long first_node, int width,
                                      double* __restrict__ moments, double* __restrict__ bbox,
                                      double* __restrict__ geom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= width) return;
  const long long node = first_node + i;
  const int* f = info + 4 * node;
  if (f[0] < 0 && f[1] < 0) return;
  double m[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) m[k] = 0.0;
  double b[6] = {HUGE_VAL, HUGE_VAL, HUGE_VAL, -HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
  for (int c = 0; c < 2; ++c) {
    const int ch = f[c];
    if (ch < 0) continue;
    double cm[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) cm[k] = moments[12 * (size_t)ch + k];
    mom_add_node(m, cm);
    const double* cb = bbox + 6 * (size_t)ch;
    for (int k = 0; k < 3; ++k) {
      if (cb[k] < b[k]) b[k] = cb[k];
      if (cb[3 + k] > b[3 + k]) b[3 + k] = cb[3 + k];
    }
  }
  double d1[3];
  for (int k = 0; k < 3; ++k) {
    d1[k] = m[3 + k] - b[k];
    const double d2 = b[3 + k] - m[3 + k];
    if (d2 > d1[k]) d1[k] = d2;
  }
  m[0] = sqrt(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
  store_node(node, m, b, moments, bbox, geom);
}

/* Buckets in key order: a bucket starts at particle `first`; every
 * particle learns its bucket. */
__global__ void bucket_mark_kernel(const int* __restrict__ info, long long n_nodes, int* __restrict__ at,
                                   int* __restrict__ leaf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_nodes;
       i += (long long)gridDim.x * blockDim.x) {
    const int* f = info + 4 * i;
    if (f[0] < 0 && f[1] < 0 && f[3] > 0) {
      at[f[2]] = (int)i;
      for (int j = f[2]; j < f[2] + f[3]; ++j) leaf[j] = (int)i;
    }
  }
}

constexpr int kCompactThreads = 1024;
constexpr int kCompactRun = 8;
constexpr int kCompactTile = kCompactThreads * kCompactRun;

/* Stream compaction of the non-negative entries of at[], order kept:
 * pass 1 counts per tile, pass 2 writes. */
__global__ void compact_count_kernel(const int* __restrict__ at, long long n, int* __restrict__ tile_count) {
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kCompactTile + (long long)threadIdx.x * kCompactRun;
  int c = 0;
  for (int j = 0; j < kCompactRun; ++j)
    if (base + j < n && at[base + j] >= 0) ++c;
  if (c) atomicAdd(&total, c);
  __syncthreads();
  if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

__global__ void compact_write_kernel(const int* __restrict__ at, long long n,
                                     const int* __restrict__ tile_off, int* __restrict__ out) {
  __shared__ int pre[kCompactThreads];
  const long long base = (long long)blockIdx.x * kCompactTile + (long long)threadIdx.x * kCompactRun;
  int c = 0;
  for (int j = 0; j < kCompactRun; ++j)
    if (base + j < n && at[base + j] >= 0) ++c;
  pre[threadIdx.x] = c;
  __syncthreads();
  for (int o = 1; o < kCompactThreads; o <<= 1) {
    const int y = threadIdx.x >= o ? pre[threadIdx.x - o] : 0;
    __syncthreads();
    pre[threadIdx.x] += y;
    __syncthreads();
  }
  int w = tile_off[blockIdx.x] + pre[threadIdx.x] - c;
  for (int j = 0; j < kCompactRun; ++j)
    if (base + j < n && at[base + j] >= 0) out[w++] = at[base + j];
}

int grid_n(long long n, int threads, int per_sm = 8) {
  long long g = (n + threads - 1) / threads;
  const long long cap = (long long)sm_count() * per_sm;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace
}  // namespace chg

using namespace chg;

struct ChangaTree {
  long long n = 0, n_nodes = 0;
  int n_buckets = 0, n_bucket = 0;
  int* perm = nullptr;           // n: GPU order -> input index
  double* parts = nullptr;       // n x 5
  double* moments = nullptr;     // n_nodes x 12
  double* geom = nullptr;        // n_nodes x 6
  double* bbox = nullptr;        // n_nodes x 6
  int* info = nullptr;           // n_nodes x 4
  int* parent = nullptr;         // n_nodes
  int* bucket_node = nullptr;    // n_buckets
  int* leaf = nullptr;           // n
  double* box = nullptr;         // 6
  std::vector<void*> blocks;     // from the device's default pool
};

extern "C" void changa_tree_free(ChangaTree* t) {
  if (!t) return;
  /* the arrays may be in use on any stream: wait as cudaFree would, then
   * hand the blocks back to the pool */
  cudaDeviceSynchronize();
  for (void* p : t->blocks)
    if (p) cudaFreeAsync(p, 0);
  delete t;
}

extern "C" ChangaTree* changa_tree_build(const double* pos, const double* mass, const double* soft,
                                         long long n, int n_bucket, cudaStream_t s) {
  if (!pos || !mass || !soft || n <= 0 || n >= (1LL << 31) - 1 || n_bucket <= 0) {
    record_error(CHANGA_E_INVALID_ARG, "changa_tree_build: arguments", __FILE__, __LINE__);
    return nullptr;
  }
  prepare_pool();
  ChangaTree* t = new ChangaTree();
  t->n = n;
  t->n_bucket = n_bucket;
  /* tree arrays live as long as the handle; scratch is freed (back to the
   * pool, stream-ordered) before the build returns */
  std::vector<void*> scratch;
  auto alloc = [&](size_t bytes, bool keep) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes < 256 ? 256 : bytes, s) != cudaSuccess) return nullptr;
    (keep ? t->blocks : scratch).push_back(p);
    return p;
  };
  auto drop = [&](void* p) {
    for (auto& b : scratch)
      if (b == p) {
        cudaFreeAsync(b, s);
        b = nullptr;
      }
  };
  auto release_scratch = [&]() {
    for (void* p : scratch)
      if (p) cudaFreeAsync(p, s);
    scratch.clear();
  };
  auto fail = [&](const char* what) -> ChangaTree* {
    const cudaError_t e = cudaGetLastError();
    record_error(e != cudaSuccess ? (int)e : CHANGA_E_INVALID_ARG, what, __FILE__, __LINE__);
    release_scratch();
    changa_tree_free(t);
    return nullptr;
  };
  /* 1-2: box and keys */
  const int gb = grid_n(n, 256);
  float* part_box = (float*)alloc((size_t)gb * 6 * sizeof(float), false);
  t->box = (double*)alloc(6 * sizeof(double), true);
  unsigned long long* k0 = (unsigned long long*)alloc((size_t)n * 8, false);
  unsigned long long* k1 = (unsigned long long*)alloc((size_t)n * 8, false);
  /* 16 passes: the sorted order ends in the first value buffer */
  int* v0 = (int*)alloc((size_t)n * 4, true);
  int* v1 = (int*)alloc((size_t)n * 4, false);
  const int tiles = (int)((n + kSortTile - 1) / kSortTile);
  int* counts = (int*)alloc((size_t)tiles * kDigits * 4, false);
  if (!part_box || !t->box || !k0 || !k1 || !v0 || !v1 || !counts) return fail("tree: memory");
  box_partial_kernel<<<gb, 256, 0, s>>>(pos, n, part_box);
  box_final_kernel<<<1, 1, 0, s>>>(part_box, gb, t->box);
  keys_kernel<<<grid_n(n, 256), 256, 0, s>>>(pos, n, t->box, k0, v0);
  count_launch(3);
  /* 3: stable radix sort, 16 passes of 4 bits */
  for (int pass = 0; pass < 16; ++pass) {
    const int shift = 4 * pass;
    radix_count_kernel<<<tiles, kSortThreads, 0, s>>>(k0, n, shift, counts, tiles);
    scan_kernel<<<1, 1024, 0, s>>>(counts, tiles * kDigits);
    radix_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(k0, v0, n, shift, counts, tiles, k1, v1);
    count_launch(3);
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  if (cudaGetLastError() != cudaSuccess) return fail("tree: sort");
  t->perm = v0;
  drop(k1);
  drop(v1);
  drop(counts);
  t->parts = (double*)alloc((size_t)n * 5 * sizeof(double), true);
  if (!t->parts) return fail("tree: memory");
  gather_parts_kernel<<<grid_n(n, 256), 256, 0, s>>>(pos, mass, soft, t->perm, n, t->parts);
  count_launch();
  /* 4: levels.  Splits that leave one side empty add single-child nodes,
   * so the node count has no tight bound: the node arrays grow by doubling
   * as the levels are built. */
  long long cap = 4 * (n / n_bucket) + 64;
  t->info = (int*)alloc((size_t)cap * 4 * sizeof(int), true);
  t->parent = (int*)alloc((size_t)cap * sizeof(int), true);
  double* cell = (double*)alloc((size_t)cap * 6 * sizeof(double), false);
  auto grow = [&](long long need) -> bool {
    long long nc = cap;
    while (nc < need) nc *= 2;
    if (nc == cap) return true;
    void* fields[3] = {t->info, t->parent, cell};
    const size_t width[3] = {4 * sizeof(int), sizeof(int), 6 * sizeof(double)};
    const bool keep[3] = {true, true, false};
    void* fresh[3];
    for (int k = 0; k < 3; ++k) {
      fresh[k] = alloc((size_t)nc * width[k], keep[k]);
      if (!fresh[k]) return false;
      if (cudaMemcpyAsync(fresh[k], fields[k], (size_t)cap * width[k], cudaMemcpyDeviceToDevice,
                          s) != cudaSuccess)
        return false;
    }
    for (int k = 0; k < 3; ++k) {
      auto& list = keep[k] ? t->blocks : scratch;
      for (auto& b : list)
        if (b == fields[k]) {
          cudaFreeAsync(b, s);
          b = nullptr;
        }
    }
    t->info = (int*)fresh[0];
    t->parent = (int*)fresh[1];
    cell = (double*)fresh[2];
    cap = nc;
    return true;
  };
  LevelNode* lv[2] = {(LevelNode*)alloc((size_t)n * sizeof(LevelNode) + 16, false),
                      (LevelNode*)alloc((size_t)n * sizeof(LevelNode) + 16, false)};
  double* sp[2] = {(double*)alloc((size_t)n * 6 * sizeof(double) + 64, false),
                   (double*)alloc((size_t)n * 6 * sizeof(double) + 64, false)};
  int* nchild = (int*)alloc((size_t)n * sizeof(int) + 16, false);
  int* mid = (int*)alloc((size_t)n * sizeof(int) + 16, false);
  int* pinned = nullptr;  // per-level read-back: last scan value, mid, node
  if (!t->info || !t->parent || !cell || !lv[0] || !lv[1] || !sp[0] || !sp[1] ||
      !nchild || !mid || cudaMallocHost((void**)&pinned, 4 * sizeof(int)) != cudaSuccess)
    return fail("tree: memory");
  {
    const LevelNode root{0, (int)n};
    const int minus1 = -1;
    if (cudaMemcpyAsync(lv[0], &root, sizeof(root), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(sp[0], t->box, 6 * sizeof(double), cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(t->parent, &minus1, sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      cudaFreeHost(pinned);
      return fail("tree: root");
    }
  }
  std::vector<long long> level_base;
  std::vector<int> level_width;
  long long base = 0;
  int width = 1, cur = 0;
  for (int level = 0; width > 0 && level <= 61; ++level) {
    split_kernel<<<(width + 255) / 256, 256, 0, s>>>(k0, lv[cur], width, level, n_bucket, nchild, mid);
    /* exclusive scan of the children counts; the total gives the next width */
    scan_kernel<<<1, 1024, 0, s>>>(nchild, width);
    cudaMemcpyAsync(pinned, nchild + width - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(pinned + 1, mid + width - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(pinned + 2, lv[cur] + width - 1, sizeof(LevelNode), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      cudaFreeHost(pinned);
      return fail("tree: level");
    }
    const int last_scan = pinned[0], last_mid = pinned[1];
    const LevelNode last_node{pinned[2], pinned[3]};
    int last_n = 0;
    if (last_mid >= 0)
      last_n = (last_mid > last_node.first) + (last_node.first + last_node.count > last_mid);
    const int next_width = last_scan + last_n;
    if (base + width + next_width > cap && !grow(base + width + next_width)) {
      cudaFreeHost(pinned);
      return fail("tree: node memory");
    }
    link_kernel<<<(width + 255) / 256, 256, 0, s>>>(lv[cur], sp[cur], width, level, (int)base,
                                                    (int)(base + width), nchild, mid, lv[cur ^ 1],
                                                    sp[cur ^ 1], t->info, t->parent, cell);
    count_launch(3);
    level_base.push_back(base);
    level_width.push_back(width);
    base += width;
    width = next_width;
    cur ^= 1;
  }
  cudaFreeHost(pinned);
  if (cudaGetLastError() != cudaSuccess) return fail("tree: levels");
  t->n_nodes = base;
  /* 5: node properties, buckets first, then the internal nodes level by
   * level from the deepest up */
  t->moments = (double*)alloc((size_t)base * 12 * sizeof(double), true);
  t->geom = (double*)alloc((size_t)base * 6 * sizeof(double), true);
  t->bbox = (double*)alloc((size_t)base * 6 * sizeof(double), true);
  if (!t->moments || !t->geom || !t->bbox) return fail("tree: memory");
  bucket_props_kernel<<<grid_n(base, 128, 16), 128, 0, s>>>(t->parts, t->info, cell, base,
                                                            t->moments, t->bbox, t->geom);
  count_launch();
  for (int l = (int)level_base.size() - 1; l >= 0; --l) {
    internal_props_kernel<<<(level_width[l] + 127) / 128, 128, 0, s>>>(
        t->info, level_base[l], level_width[l], t->moments, t->bbox, t->geom);
    count_launch();
  }
  /* buckets in key order, and each particle's bucket */
  int* at = (int*)alloc((size_t)n * sizeof(int), false);
  t->bucket_node = (int*)alloc((size_t)n * sizeof(int), true);
  t->leaf = (int*)alloc((size_t)n * sizeof(int), true);
  const int ctiles = (int)((n + kCompactTile - 1) / kCompactTile);
  int* tile_count = (int*)alloc((size_t)(ctiles + 1) * sizeof(int), false);
  if (!at || !t->bucket_node || !t->leaf || !tile_count) return fail("tree: memory");
  cudaMemsetAsync(at, 0xff, (size_t)n * sizeof(int), s);
  bucket_mark_kernel<<<grid_n(base, 256), 256, 0, s>>>(t->info, base, at, t->leaf);
  compact_count_kernel<<<ctiles, kCompactThreads, 0, s>>>(at, n, tile_count);
  cudaMemsetAsync(tile_count + ctiles, 0, sizeof(int), s);
  scan_kernel<<<1, 1024, 0, s>>>(tile_count, ctiles + 1);
  compact_write_kernel<<<ctiles, kCompactThreads, 0, s>>>(at, n, tile_count, t->bucket_node);
  count_launch(4);
  int h_nb = 0;
  cudaMemcpyAsync(&h_nb, tile_count + ctiles, sizeof(int), cudaMemcpyDeviceToHost, s);
  release_scratch();
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail("tree: buckets");
  t->n_buckets = h_nb;
  return t;
}

extern "C" int changa_tree_view(const ChangaTree* t, ChangaTreeArrays* out) {
  if (!t || !out) return record_error(CHANGA_E_INVALID_ARG, "changa_tree_view", __FILE__, __LINE__);
  out->n = t->n;
  out->n_nodes = t->n_nodes;
  out->n_buckets = t->n_buckets;
  out->perm = t->perm;
  out->parts = t->parts;
  out->moments = t->moments;
  out->geom = t->geom;
  out->bbox = t->bbox;
  out->info = t->info;
  out->parent = t->parent;
  out->bucket_node = t->bucket_node;
  out->leaf = t->leaf;
  out->box = t->box;
  return 0;
}
