/*
 * Host side of the gravity path: the caller of the GPU boundary.
 *
 * ChaNGa builds its tree, computes multipole moments, walks the tree and
 * serialises interaction lists on the CPU (TreePiece / ListCompute /
 * DataManager), then hands flat arrays to the GPU entry points declared in
 * HostCUDA.h.  That host code needs Charm++ and is not rebuilt here; this
 * file restates the parts that decide WHAT the GPU computes, for a single
 * tree piece, so the kernels receive exactly the arrays the reference would
 * build:
 *
 *   - cubical bounding box with the 1+1.91e-6 slop (TreePiece.cpp:141-165);
 *   - 63-bit keys, 21 bits per axis, x/y/z interleaved from the top bit.
 *     ChaNGa's key function lives in the N-BodyShop utility (SFC.h), which
 *     is not available; this Morton key is this project's own and is the one
 *     whose top bits match the spatial bisection below;
 *   - binary tree split at the box midpoint along level%3, membership by key
 *     bit (GenericTreeNode.h:473-599), buckets when count <= maxBucketSize
 *     (Compute.cpp:2476-2495), makeBucket radius rules
 *     (GenericTreeNode.h:219-255), children moments and farthest-corner
 *     radius (Compute.cpp:2556-2576, TreePiece.cpp:3540-3546);
 *   - quadrupole moments by the parallel-axis sums of
 *     MultipoleMoments.h:206-352 and the radius rules at 460-526;
 *   - the dual tree walk: ListCompute::doWork with LocalOpt actions
 *     (Compute.cpp:690-891, Opt.h:101-136), LocalTargetWalk::dft
 *     (TreeWalk.cpp:308-397), openCriterionNode (gravity.h:652-723) and the
 *     replica roots on the level-0 check list (TreePiece.cpp:3745-3763);
 *   - serialisation: moments in breadth-first order (DataManager.cpp:
 *     768-858), particles in bucket order (ParallelGravity.h:957-975), cell
 *     lists per bucket as levels 0..lowest (Compute.cpp:1626-1741), particle
 *     lists flattened to one ILCell per source particle (Compute.cpp:
 *     1119-1218); only buckets with a non-empty list appear in a request
 *     (Compute.cpp:1044-1090).
 *
 * A single tree piece has no Boundary/NonLocal nodes (those come from the
 * multi-piece sentinels at GenericTreeNode.h:499-560); every node here is
 * Internal, Bucket or Empty.  The geometry predicates use closed balls, as in
 * oracle/shim/Space.h.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum NodeType { T_BUCKET = 2, T_INTERNAL = 3, T_EMPTY = 6 };

struct Node {
  int first = 0, count = 0;  // particle range [first, first+count)
  int child[2] = {-1, -1};
  int type = T_EMPTY;
  int level = 0;
  double mom[12] = {0};  // radius, soft, totalMass, cm xyz, xx xy xz yy yz zz
  double bbox[6];        // lesser xyz, greater xyz (from particles)
  double split[6];       // spatial cell from the midpoint splits
  int bfs = -1;          // index in the moment array
  int bucket = -1;       // bucket id for buckets
  int first_bucket = 0, n_buckets = 0;
};

struct Entry {
  int node;
  int off;  // 9-bit replica code (x+3)|(y+3)<<3|(z+3)<<6
};

struct Tree {
  long n = 0;
  int n_bucket = 16;
  double theta = 0.7;
  double period = 0.0;
  int n_replicas = 0;
  std::vector<double> pos;   // sorted positions (n x 3)
  std::vector<double> mass;  // sorted
  std::vector<double> soft;  // sorted
  std::vector<long> perm;    // sorted index -> original index
  std::vector<uint64_t> keys;
  std::vector<Node> nodes;
  std::vector<int> bucket_nodes;  // bucket id -> node
  std::vector<int> bfs_nodes;     // bfs index -> node
  double box[6];
  // walk output per bucket
  std::vector<std::vector<int>> cell_idx, cell_off, part_idx, part_off;
  std::vector<long> n_cells, n_parts;  // per bucket list lengths
  /* multipole order of the cell interactions: 2 (quadrupole) or 4
   * (hexadecapole: the walk adds the softening / monopole tests and routes
   * softened cells to their own per-bucket list) */
  int order = 2;
  double theta_mono = 0.0;
  std::vector<std::vector<int>> soft_idx, soft_off;
  std::vector<long> n_soft;
};

/* ---- moments (MultipoleMoments.h:206-352) ---- */

static void mom_add_particle(double* m, double pm, double ps, const double* p) {
  double m1 = m[2];
  m[2] += pm;
  if (m[2] == 0.0) {
    m[1] = 0.5 * (m[1] + ps);
    for (int k = 0; k < 3; ++k) m[3 + k] = 0.5 * (m[3 + k] + p[k]);
    return;
  }
  m[1] = (m1 * m[1] + pm * ps) / m[2];
  double cm1[3] = {m[3], m[4], m[5]};
  for (int k = 0; k < 3; ++k) m[3 + k] = (m1 * cm1[k] + pm * p[k]) / m[2];
  double dr[3] = {cm1[0] - m[3], cm1[1] - m[4], cm1[2] - m[5]};
  m[6] += m1 * dr[0] * dr[0];
  m[9] += m1 * dr[1] * dr[1];
  m[11] += m1 * dr[2] * dr[2];
  m[7] += m1 * dr[0] * dr[1];
  m[8] += m1 * dr[0] * dr[2];
  m[10] += m1 * dr[1] * dr[2];
  dr[0] = p[0] - m[3];
  dr[1] = p[1] - m[4];
  dr[2] = p[2] - m[5];
  m[6] += pm * dr[0] * dr[0];
  m[9] += pm * dr[1] * dr[1];
  m[11] += pm * dr[2] * dr[2];
  m[7] += pm * dr[0] * dr[1];
  m[8] += pm * dr[0] * dr[2];
  m[10] += pm * dr[1] * dr[2];
}

static void mom_add_node(double* m, const double* c) {
  double m1 = m[2];
  m[2] += c[2];
  if (m[2] == 0.0) {
    m[1] = 0.5 * (m[1] + c[1]);
    for (int k = 0; k < 3; ++k) m[3 + k] = 0.5 * (m[3 + k] + c[3 + k]);
    return;
  }
  if (m1 == 0.0) {
    std::memcpy(m, c, 12 * sizeof(double));
    return;
  }
  if (c[2] == 0.0) return;
  m[1] = (m1 * m[1] + c[2] * c[1]) / m[2];
  double cm1[3] = {m[3], m[4], m[5]};
  for (int k = 0; k < 3; ++k) m[3 + k] = (m1 * cm1[k] + c[2] * c[3 + k]) / m[2];
  double dr[3] = {cm1[0] - m[3], cm1[1] - m[4], cm1[2] - m[5]};
  m[6] += m1 * dr[0] * dr[0];
  m[9] += m1 * dr[1] * dr[1];
  m[11] += m1 * dr[2] * dr[2];
  m[7] += m1 * dr[0] * dr[1];
  m[8] += m1 * dr[0] * dr[2];
  m[10] += m1 * dr[1] * dr[2];
  dr[0] = c[3] - m[3];
  dr[1] = c[4] - m[4];
  dr[2] = c[5] - m[5];
  m[6] += c[6] + c[2] * dr[0] * dr[0];
  m[9] += c[9] + c[2] * dr[1] * dr[1];
  m[11] += c[11] + c[2] * dr[2] * dr[2];
  m[7] += c[7] + c[2] * dr[0] * dr[1];
  m[8] += c[8] + c[2] * dr[0] * dr[2];
  m[10] += c[10] + c[2] * dr[1] * dr[2];
}

static inline void bbox_reset(double* b) {
  b[0] = b[1] = b[2] = HUGE_VAL;
  b[3] = b[4] = b[5] = -HUGE_VAL;
}
static inline void bbox_grow_pt(double* b, const double* p) {
  for (int k = 0; k < 3; ++k) {
    if (p[k] < b[k]) b[k] = p[k];
    if (p[k] > b[3 + k]) b[3 + k] = p[k];
  }
}
static inline void bbox_grow_box(double* b, const double* o) {
  for (int k = 0; k < 3; ++k) {
    if (o[k] < b[k]) b[k] = o[k];
    if (o[3 + k] > b[3 + k]) b[3 + k] = o[3 + k];
  }
}

/* ---- keys ---- */

static inline uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

static inline uint64_t make_key(const double* p, const double* box) {
  uint64_t q[3];
  for (int k = 0; k < 3; ++k) {
    double s = (p[k] - box[k]) / (box[3 + k] - box[k]);
    if (s < 0) s = 0;
    double f = s * 2097152.0;
    uint64_t v = f >= 2097151.0 ? 2097151 : (uint64_t)f;
    q[k] = v;
  }
  return (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
}

/* ---- tree build ---- */

static int build_node(Tree& t, int first, int count, int level, const double* split) {
  int id = (int)t.nodes.size();
  t.nodes.emplace_back();
  {
    Node& nd = t.nodes[id];
    nd.first = first;
    nd.count = count;
    nd.level = level;
    std::memcpy(nd.split, split, sizeof(nd.split));
    bbox_reset(nd.bbox);
  }
  if (count == 0) {
    t.nodes[id].type = T_EMPTY;
    return id;
  }
  if (count <= t.n_bucket || level >= 60) {
    Node& nd = t.nodes[id];
    nd.type = T_BUCKET;
    double* m = nd.mom;
    /* calculateRadiusBox on the spatial cell before the particle loop */
    double dx = split[3] - split[0], dy = split[4] - split[1], dz = split[5] - split[2];
    m[0] = 0.5 * std::sqrt(dx * dx + dy * dy + dz * dz);
    if (m[0] <= 0.0) {
      if (count > 1) {
        const double* p1 = &t.pos[3 * (size_t)first];
        double r2 = 0;
        for (int i = first + 1; i < first + count; ++i) {
          const double* p = &t.pos[3 * (size_t)i];
          double d = (p1[0] - p[0]) * (p1[0] - p[0]) + (p1[1] - p[1]) * (p1[1] - p[1]) +
                     (p1[2] - p[2]) * (p1[2] - p[2]);
          if (d > r2) r2 = d;
        }
        if (r2 > 0) m[0] = std::sqrt(r2);
      } else {
        m[0] = 1.0;
      }
    }
    for (int i = first; i < first + count; ++i) {
      mom_add_particle(m, t.mass[i], t.soft[i], &t.pos[3 * (size_t)i]);
      bbox_grow_pt(nd.bbox, &t.pos[3 * (size_t)i]);
    }
    if (count > 1) {
      double r2 = 0;
      for (int i = first; i < first + count; ++i) {
        const double* p = &t.pos[3 * (size_t)i];
        double d = (m[3] - p[0]) * (m[3] - p[0]) + (m[4] - p[1]) * (m[4] - p[1]) +
                   (m[5] - p[2]) * (m[5] - p[2]);
        if (d > r2) r2 = d;
      }
      if (r2 > 0.0) m[0] = std::sqrt(r2);
    }
    return id;
  }
  t.nodes[id].type = T_INTERNAL;
  int axis = level % 3;
  double s0[6], s1[6];
  std::memcpy(s0, split, sizeof(s0));
  std::memcpy(s1, split, sizeof(s1));
  double mid = 0.5 * (split[3 + axis] + split[axis]);
  s0[3 + axis] = mid;
  s1[axis] = mid;
  uint64_t mask = 1ULL << (62 - level);
  /* first particle with the split bit set */
  int lo = first, hi = first + count;
  while (lo < hi) {
    int md = lo + (hi - lo) / 2;
    if (t.keys[md] & mask) hi = md;
    else lo = md + 1;
  }
  int c0 = build_node(t, first, lo - first, level + 1, s0);
  int c1 = build_node(t, lo, first + count - lo, level + 1, s1);
  Node& nd = t.nodes[id];
  nd.child[0] = c0;
  nd.child[1] = c1;
  double* m = nd.mom;
  for (int c = 0; c < 2; ++c) {
    const Node& ch = t.nodes[nd.child[c]];
    if (ch.type == T_EMPTY) continue;
    mom_add_node(m, ch.mom);
    bbox_grow_box(nd.bbox, ch.bbox);
  }
  /* calculateRadiusFarthestCorner (MultipoleMoments.h:462-476) */
  double d1[3], d2[3];
  for (int k = 0; k < 3; ++k) {
    d1[k] = m[3 + k] - nd.bbox[k];
    d2[k] = nd.bbox[3 + k] - m[3 + k];
    if (d2[k] > d1[k]) d1[k] = d2[k];
  }
  m[0] = std::sqrt(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
  return id;
}

static void number_buckets(Tree& t, int id) {
  Node& nd = t.nodes[id];
  nd.first_bucket = (int)t.bucket_nodes.size();
  if (nd.type == T_BUCKET) {
    nd.bucket = (int)t.bucket_nodes.size();
    t.bucket_nodes.push_back(id);
  } else if (nd.type == T_INTERNAL) {
    number_buckets(t, nd.child[0]);
    number_buckets(t, nd.child[1]);
  }
  t.nodes[id].n_buckets = (int)t.bucket_nodes.size() - t.nodes[id].first_bucket;
}

/* ---- walk ---- */

const double kOpenGeom = 2.0 / std::sqrt(3.0);  // TreeNode.h:35

static inline void decode(int off, double period, double* o) {
  o[0] = ((off & 7) - 3) * period;
  o[1] = (((off >> 3) & 7) - 3) * period;
  o[2] = (((off >> 6) & 7) - 3) * period;
}

/* openCriterionNode, gravity.h:652-723 (quadrupole build): 1 = open
 * (CONTAIN), -1 = undecided (INTERSECT), 0 = accept. */
static inline int open_criterion(const Tree& t, const Node& g, const Node& local, int off) {
  if (g.count <= 6) return 1;
  double radius = kOpenGeom * g.mom[0] / t.theta;
  if (radius < g.mom[0]) radius = g.mom[0];
  double o[3];
  decode(off, t.period, o);
  double c[3] = {g.mom[3] + o[0], g.mom[4] + o[1], g.mom[5] + o[2]};
  const double* b = local.bbox;
  double d2 = 0.0, d;
  for (int k = 0; k < 3; ++k) {
    if ((d = b[k] - c[k]) > 0) d2 += d * d;
    else if ((d = c[k] - b[3 + k]) > 0) d2 += d * d;
  }
  double r2 = radius * radius;
  bool inter = d2 <= r2;
  if (local.type == T_BUCKET) return inter ? 1 : 0;
  if (!inter) return 0;
  double f2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double a1 = c[k] - b[k], a2 = b[3 + k] - c[k];
    a1 *= a1;
    a2 *= a2;
    f2 += a1 > a2 ? a1 : a2;
  }
  return f2 <= r2 ? 1 : -1;
}

/* openSoftening, gravity.h:252-260: the cell's softening sphere (twice its
 * softening, at cm + offset) meets the bucket's softening sphere or box. */
static inline bool open_softening(const Tree& t, const Node& g, const Node& local, int off) {
  double o[3];
  decode(off, t.period, o);
  const double c[3] = {g.mom[3] + o[0], g.mom[4] + o[1], g.mom[5] + o[2]};
  const double r = 2.0 * g.mom[1];
  double dx = c[0] - local.mom[3], dy = c[1] - local.mom[4], dz = c[2] - local.mom[5];
  const double rr = r + 2.0 * local.mom[1];
  if (dx * dx + dy * dy + dz * dz <= rr * rr) return true;
  const double* b = local.bbox;
  double d2 = 0.0, d;
  for (int k = 0; k < 3; ++k) {
    if ((d = b[k] - c[k]) > 0) d2 += d * d;
    else if ((d = c[k] - b[3 + k]) > 0) d2 += d * d;
  }
  return d2 <= r * r;
}

/* Hexadecapole form of openCriterionNode (gravity.h:664-722): a
 * well-separated cell whose softening overlaps the local node is opened
 * unless it also passes the monopole angle theta_mono. */
static inline int open_criterion_hex(const Tree& t, const Node& g, const Node& local, int off) {
  if (g.count <= 6) return 1;
  double radius = kOpenGeom * g.mom[0] / t.theta;
  if (radius < g.mom[0]) radius = g.mom[0];
  double o[3];
  decode(off, t.period, o);
  const double c[3] = {g.mom[3] + o[0], g.mom[4] + o[1], g.mom[5] + o[2]};
  const double* b = local.bbox;
  double d2 = 0.0, d;
  for (int k = 0; k < 3; ++k) {
    if ((d = b[k] - c[k]) > 0) d2 += d * d;
    else if ((d = c[k] - b[3 + k]) > 0) d2 += d * d;
  }
  if (d2 <= radius * radius) {
    if (local.type == T_BUCKET) return 1;
    double f2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      double a1 = c[k] - b[k], a2 = b[3 + k] - c[k];
      a1 *= a1;
      a2 *= a2;
      f2 += a1 > a2 ? a1 : a2;
    }
    return f2 <= radius * radius ? 1 : -1;
  }
  if (!open_softening(t, g, local, off)) return 0;
  const double rm = kOpenGeom * g.mom[0] / t.theta_mono;
  return d2 <= rm * rm ? 1 : 0;
}

struct LevelLists {
  std::vector<Entry> clist, plist, und;
};

struct WalkCtx {
  Tree* t;
  std::vector<LevelLists> lv;
};

static void emit(WalkCtx& w, int local, int level) {
  Tree& t = *w.t;
  const Node& ln = t.nodes[local];
  size_t nc = 0, np = 0;
  for (int l = 0; l <= level; ++l) {
    nc += w.lv[l].clist.size();
    for (const Entry& e : w.lv[l].plist) np += t.nodes[e.node].count;
  }
  for (int b = ln.first_bucket; b < ln.first_bucket + ln.n_buckets; ++b) {
    std::vector<int>& ci = t.cell_idx[b];
    std::vector<int>& co = t.cell_off[b];
    std::vector<int>& pi = t.part_idx[b];
    std::vector<int>& po = t.part_off[b];
    ci.reserve(nc);
    co.reserve(nc);
    pi.reserve(np);
    po.reserve(np);
    const Node& bn = t.nodes[t.bucket_nodes[b]];
    for (int l = 0; l <= level; ++l) {
      for (const Entry& e : w.lv[l].clist) {
        /* reqID = reEncodeOffset(bucket, offset) (TreeWalk.cpp:336); the low
         * 22 bits carry the walking bucket, the kernels read only bits 22+ */
        const int code = (e.off << 22) | (ln.first_bucket & 0x3fffff);
        if (t.order == 4 && open_softening(t, t.nodes[e.node], bn, e.off)) {
          /* nodeBucketForce evaluates these as softened point masses
           * (gravity.h:414-421, Compute.cpp:1683-1698) */
          t.soft_idx[b].push_back(t.nodes[e.node].bfs);
          t.soft_off[b].push_back(code);
          continue;
        }
        ci.push_back(t.nodes[e.node].bfs);
        co.push_back(code);
      }
      for (const Entry& e : w.lv[l].plist) {
        const Node& src = t.nodes[e.node];
        for (int k = 0; k < src.count; ++k) {
          pi.push_back(src.first + k);
          po.push_back(e.off << 22);  // encodeOffset(0, x, y, z)
        }
      }
    }
    t.n_cells[b] = (long)ci.size();
    t.n_parts[b] = (long)pi.size();
    if (t.order == 4) t.n_soft[b] = (long)t.soft_idx[b].size();
  }
}

static void process(WalkCtx& w, int local, int level, const Entry& g, std::deque<Entry>& chk) {
  Tree& t = *w.t;
  const Node& gn = t.nodes[g.node];
  if (gn.type == T_EMPTY) return;  // DUMP
  int open = t.order == 4 ? open_criterion_hex(t, gn, t.nodes[local], g.off)
                          : open_criterion(t, gn, t.nodes[local], g.off);
  if (open == 0) {
    w.lv[level].clist.push_back(g);  // COMPUTE
    return;
  }
  if (gn.type == T_BUCKET) {
    w.lv[level].plist.push_back(g);  // KEEP_LOCAL_BUCKET
    return;
  }
  /* KEEP */
  if (open == 1 || t.nodes[local].type == T_BUCKET) {
    chk.push_back(Entry{gn.child[0], g.off});
    chk.push_back(Entry{gn.child[1], g.off});
  } else {
    w.lv[level].und.push_back(g);
  }
}

static void dft(WalkCtx& w, int local, int level, int task_depth) {
  Tree& t = *w.t;
  if ((int)w.lv.size() <= level + 1) w.lv.resize(level + 2);
  LevelLists& L = w.lv[level];
  L.clist.clear();
  L.plist.clear();
  L.und.clear();
  std::deque<Entry> chk;
  if (level == 0) {
    int nr = t.n_replicas;
    for (int x = -nr; x <= nr; ++x)
      for (int y = -nr; y <= nr; ++y)
        for (int z = -nr; z <= nr; ++z)
          chk.push_back(Entry{0, (x + 3) | ((y + 3) << 3) | ((z + 3) << 6)});
  } else {
    const std::vector<Entry>& pu = w.lv[level - 1].und;
    for (size_t i = 0; i < pu.size(); ++i) process(w, local, level, pu[i], chk);
  }
  while (!chk.empty()) {
    Entry e = chk.front();
    chk.pop_front();
    process(w, local, level, e, chk);
  }
  const Node& ln = t.nodes[local];
  if (!w.lv[level].und.empty() && ln.type == T_INTERNAL) {
    for (int c = 0; c < 2; ++c) {
      int ch = ln.child[c];
      if (t.nodes[ch].type == T_EMPTY) continue;
      if (level < task_depth) {
#ifdef _OPENMP
        WalkCtx w2;
        w2.t = w.t;
        w2.lv.assign(w.lv.begin(), w.lv.begin() + level + 1);
#pragma omp task firstprivate(w2, ch, level, task_depth)
        { dft(w2, ch, level + 1, task_depth); }
#else
        dft(w, ch, level + 1, task_depth);
#endif
      } else {
        dft(w, ch, level + 1, task_depth);
      }
    }
  } else {
    emit(w, local, level);
  }
}

}  // namespace

extern "C" {

/* Builds the tree for n particles (pos n x 3, mass, soft: FP64).
 * Returns an opaque handle (NULL on error). */
void* chg_tree_build(const double* pos, const double* mass, const double* soft, long n,
                     int n_bucket, double theta, double period, int n_replicas) {
  if (n <= 0 || n_bucket <= 0 || theta <= 0 || n_replicas < 0 || n_replicas > 3) return nullptr;
  Tree* t = new Tree();
  t->n = n;
  t->n_bucket = n_bucket;
  t->theta = theta;
  t->period = period;
  t->n_replicas = n_replicas;
  /* bounding box in float, made cubical with the key slop (TreePiece.cpp:
   * 141-156) */
  float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
  for (long i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      float v = (float)pos[3 * i + k];
      if (v < lo[k]) lo[k] = v;
      if (v > hi[k]) hi[k] = v;
    }
  float size[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  float mx = size[0] > size[1] ? size[0] : size[1];
  mx = mx > size[2] ? mx : size[2];
  const float fEps = 1.0f + 1.91e-6f;
  float half = (float)(fEps * 0.5 * mx);
  for (int k = 0; k < 3; ++k) {
    float c = 0.5f * (lo[k] + hi[k]);
    t->box[k] = (double)(c - half);
    t->box[3 + k] = (double)(c + half);
  }
  if (!(t->box[3] > t->box[0])) {  // degenerate: all particles coincide
    for (int k = 0; k < 3; ++k) {
      t->box[k] -= 0.5;
      t->box[3 + k] += 0.5;
    }
  }
  std::vector<std::pair<uint64_t, long>> kp((size_t)n);
#ifdef _OPENMP
#pragma omp parallel for
#endif
  for (long i = 0; i < n; ++i) kp[i] = std::make_pair(make_key(&pos[3 * i], t->box), i);
  std::sort(kp.begin(), kp.end());
  t->pos.resize(3 * (size_t)n);
  t->mass.resize(n);
  t->soft.resize(n);
  t->perm.resize(n);
  t->keys.resize(n);
  for (long i = 0; i < n; ++i) {
    long j = kp[i].second;
    t->perm[i] = j;
    t->keys[i] = kp[i].first;
    for (int k = 0; k < 3; ++k) t->pos[3 * i + k] = pos[3 * j + k];
    t->mass[i] = mass[j];
    t->soft[i] = soft[j];
  }
  t->nodes.reserve((size_t)(4 * n / n_bucket + 64));
  build_node(*t, 0, (int)n, 0, t->box);
  number_buckets(*t, 0);
  /* breadth-first moment order, Empty nodes skipped */
  std::deque<int> q;
  q.push_back(0);
  while (!q.empty()) {
    int id = q.front();
    q.pop_front();
    Node& nd = t->nodes[id];
    if (nd.type == T_EMPTY) continue;
    nd.bfs = (int)t->bfs_nodes.size();
    t->bfs_nodes.push_back(id);
    if (nd.type == T_INTERNAL) {
      q.push_back(nd.child[0]);
      q.push_back(nd.child[1]);
    }
  }
  return t;
}

void chg_tree_free(void* h) { delete (Tree*)h; }

long chg_tree_num_moments(void* h) { return (long)((Tree*)h)->bfs_nodes.size(); }
long chg_tree_num_buckets(void* h) { return (long)((Tree*)h)->bucket_nodes.size(); }
long chg_tree_num_nodes(void* h) { return (long)((Tree*)h)->nodes.size(); }

/* perm[k] = original index of the k-th particle in GPU (bucket) order */
void chg_tree_get_order(void* h, long* perm) {
  Tree* t = (Tree*)h;
  std::memcpy(perm, t->perm.data(), t->n * sizeof(long));
}

void chg_tree_get_moments(void* h, double* out) {
  Tree* t = (Tree*)h;
  for (size_t i = 0; i < t->bfs_nodes.size(); ++i)
    std::memcpy(out + 12 * i, t->nodes[t->bfs_nodes[i]].mom, 12 * sizeof(double));
}

void chg_tree_get_root(void* h, double* out12) {
  Tree* t = (Tree*)h;
  std::memcpy(out12, t->nodes[0].mom, 12 * sizeof(double));
}

/* starts/sizes per bucket (GPU particle indices), bbox B x 6, and the
 * moment index of each bucket node */
void chg_tree_get_buckets(void* h, int* starts, int* sizes, double* bbox, int* mom_index) {
  Tree* t = (Tree*)h;
  for (size_t b = 0; b < t->bucket_nodes.size(); ++b) {
    const Node& nd = t->nodes[t->bucket_nodes[b]];
    if (starts) starts[b] = nd.first;
    if (sizes) sizes[b] = nd.count;
    if (bbox) std::memcpy(bbox + 6 * b, nd.bbox, 6 * sizeof(double));
    if (mom_index) mom_index[b] = nd.bfs;
  }
}

/* Tree structure in moment (BFS) indices, for gradients through the moment
 * construction: parent[i] = moment index of node i's parent (-1 at the
 * root); leaf[k] = moment index of the bucket holding GPU particle k. */
void chg_tree_get_structure(void* h, int* parent, int* leaf) {
  Tree* t = (Tree*)h;
  if (parent) {
    for (size_t i = 0; i < t->bfs_nodes.size(); ++i) parent[i] = -1;
    for (size_t i = 0; i < t->bfs_nodes.size(); ++i) {
      const Node& nd = t->nodes[t->bfs_nodes[i]];
      if (nd.type != T_INTERNAL) continue;
      for (int c = 0; c < 2; ++c) {
        const Node& ch = t->nodes[nd.child[c]];
        if (ch.bfs >= 0) parent[ch.bfs] = (int)i;
      }
    }
  }
  if (leaf) {
    for (size_t b = 0; b < t->bucket_nodes.size(); ++b) {
      const Node& nd = t->nodes[t->bucket_nodes[b]];
      for (int k = nd.first; k < nd.first + nd.count; ++k) leaf[k] = nd.bfs;
    }
  }
}

/* Particle range [first, first + count) of every moment (BFS) index, in GPU
 * order: what the device moment refresh reduces over. */
void chg_tree_get_ranges(void* h, int* first, int* count) {
  Tree* t = (Tree*)h;
  for (size_t i = 0; i < t->bfs_nodes.size(); ++i) {
    const Node& nd = t->nodes[t->bfs_nodes[i]];
    first[i] = nd.first;
    count[i] = nd.count;
  }
}

/* Runs the walk; returns 0 on success. */
int chg_tree_walk(void* h, int nthreads) {
  Tree* t = (Tree*)h;
  size_t B = t->bucket_nodes.size();
  t->cell_idx.assign(B, {});
  t->cell_off.assign(B, {});
  t->part_idx.assign(B, {});
  t->part_off.assign(B, {});
  t->n_cells.assign(B, 0);
  t->n_parts.assign(B, 0);
  t->soft_idx.assign(t->order == 4 ? B : 0, {});
  t->soft_off.assign(t->order == 4 ? B : 0, {});
  t->n_soft.assign(B, 0);
  WalkCtx w;
  w.t = t;
  w.lv.resize(64);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int depth = 12;
#pragma omp parallel
#pragma omp single
  dft(w, 0, 0, depth);
#else
  (void)nthreads;
  dft(w, 0, 0, -1);
#endif
  return 0;
}

/* Per-bucket list lengths (B entries each). */
void chg_tree_list_lengths(void* h, long* n_cells, long* n_parts) {
  Tree* t = (Tree*)h;
  size_t B = t->bucket_nodes.size();
  if (n_cells) std::memcpy(n_cells, t->n_cells.data(), B * sizeof(long));
  if (n_parts) std::memcpy(n_parts, t->n_parts.data(), B * sizeof(long));
}

/* Adds one particle's reduced (trace-free) scaled moments up to the
 * hexadecapole to r[21] = {xx xy xz yy yz, xxx xyy xxy yyy xxz yyz xyz,
 * xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz}, for mass m at (x, y, z)
 * from the centre of mass in units of the expansion radius: the moments
 * momEvalFmomrcm consumes (moments.c:772-846 forms the same tensors). */
static void reduced_moment_add(double* r, double m, double x, double y, double z) {
  const double x2 = x * x, y2 = y * y, d2 = x2 + y2 + z * z;
  const double mx2 = m * x2, my2 = m * y2, md2 = m * d2;
  /* quadrupole: m (r_i r_j - delta_ij d2 / 3), xx and yy stored */
  const double mxy = m * x * y;
  r[0] += mx2 - md2 / 3.0;
  r[1] += mxy;
  r[2] += m * x * z;
  r[3] += my2 - md2 / 3.0;
  r[4] += m * y * z;
  /* octupole: m (r_i r_j r_k - d2 (delta r) / 5) */
  const double o = md2 / 5.0;
  r[5] += (mx2 - 3.0 * o) * x;   // xxx
  r[6] += (my2 - o) * x;         // xyy
  r[7] += (mx2 - o) * y;         // xxy
  r[8] += (my2 - 3.0 * o) * y;   // yyy
  r[9] += (mx2 - o) * z;         // xxz
  r[10] += (my2 - o) * z;        // yyz
  r[11] += mxy * z;              // xyz
  /* hexadecapole */
  const double h = md2 / 7.0;
  const double ax = (mx2 - 3.0 * h) * x, ay = (my2 - 3.0 * h) * y;
  const double bx = h * (x2 - 0.1 * d2), by = h * (y2 - 0.1 * d2);
  r[12] += mx2 * x2 - 6.0 * bx;  // xxxx
  r[13] += ay * x;               // xyyy
  r[14] += ax * y;               // xxxy
  r[15] += my2 * y2 - 6.0 * by;  // yyyy
  r[16] += ax * z;               // xxxz
  r[17] += ay * z;               // yyyz
  r[18] += mx2 * y2 - bx - by;   // xxyy
  r[19] += (mx2 - h) * y * z;    // xxyz
  r[20] += (my2 - h) * x * z;    // xyyz
}

/* Hexadecapole moments of every node, breadth-first, 27 doubles each:
 * {radius, soft, totalMass, cm.xyz, xx xy xz yy yz, xxx xyy xxy yyy xxz yyz
 * xyz, xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz} (the hexadecapole
 * CudaMultipoleMoments order, cuda_typedef.h:103-128), the multipole terms
 * scaled by the node radius.  ChaNGa accumulates them child by child with
 * shifts and rescales (MultipoleMoments.h:247-262, 318-330, 460-504);
 * summing each node's particles about its final centre and radius gives
 * the same tensors. */
void chg_tree_get_moments_hex(void* h, double* out) {
  Tree* t = (Tree*)h;
  const long nm = (long)t->bfs_nodes.size();
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (long i = 0; i < nm; ++i) {
    const Node& nd = t->nodes[t->bfs_nodes[i]];
    double* o = out + 27 * i;
    std::memcpy(o, nd.mom, 6 * sizeof(double));
    double* r = o + 6;
    for (int k = 0; k < 21; ++k) r[k] = 0.0;
    const double u = nd.mom[0];
    if (!(u > 0.0)) continue;
    const double iu = 1.0 / u;
    for (int k = nd.first; k < nd.first + nd.count; ++k) {
      const double* p = &t->pos[3 * (size_t)k];
      reduced_moment_add(r, t->mass[k], (p[0] - nd.mom[3]) * iu, (p[1] - nd.mom[4]) * iu,
                         (p[2] - nd.mom[5]) * iu);
    }
  }
}

/* Node arrays for a device-side walk, breadth-first like the moments:
 * geom 6 per node {cm.xyz, radius, soft, mass}, bbox 6 {lesser xyz,
 * greater xyz} from the node's particles, info 4 {child0, child1, first,
 * count} with children as moment indices (-1: none; buckets have none). */
void chg_tree_get_nodes(void* h, double* geom, double* bbox, int* info) {
  Tree* t = (Tree*)h;
  for (size_t i = 0; i < t->bfs_nodes.size(); ++i) {
    const Node& nd = t->nodes[t->bfs_nodes[i]];
    double* g = geom + 6 * i;
    g[0] = nd.mom[3];
    g[1] = nd.mom[4];
    g[2] = nd.mom[5];
    g[3] = nd.mom[0];
    g[4] = nd.mom[1];
    g[5] = nd.mom[2];
    std::memcpy(bbox + 6 * i, nd.bbox, 6 * sizeof(double));
    int* f = info + 4 * i;
    f[0] = f[1] = -1;
    if (nd.type == T_INTERNAL)
      for (int c = 0; c < 2; ++c) f[c] = t->nodes[nd.child[c]].bfs;  // -1 for Empty
    f[2] = nd.first;
    f[3] = nd.count;
  }
}

/* Hexadecapole mode (order 4) or quadrupole (order 2, the default): set
 * before the walk.  theta_mono = theta^4 (ParallelGravity.cpp:993). */
int chg_tree_set_order(void* h, int order) {
  Tree* t = (Tree*)h;
  if (order != 2 && order != 4) return -1;
  t->order = order;
  t->theta_mono = t->theta * t->theta * t->theta * t->theta;
  return 0;
}

/* Per-bucket lengths of the softened-cell lists (order 4; zeros else). */
void chg_tree_soft_lengths(void* h, long* n_soft) {
  Tree* t = (Tree*)h;
  std::memcpy(n_soft, t->n_soft.data(), t->bucket_nodes.size() * sizeof(long));
}

/* Serialises one request of kind 0 (cell lists), 1 (particle lists) or 2
 * (softened cells of the hexadecapole mode, indices into the moments) for
 * the buckets [b0, b1): list (L x 2 int32), markers (nfilled+1), starts,
 * sizes and the bucket ids (nfilled each).  Only buckets with a non-empty
 * list appear.  Returns nfilled.  index_base is added to every list index
 * and start_base to every start (for concatenating independent systems). */
long chg_tree_serialize(void* h, int kind, long b0, long b1, int* list, int* markers, int* starts,
                        int* sizes, int* bucket_ids, long index_base, long start_base) {
  Tree* t = (Tree*)h;
  long filled = 0;
  long pos = 0;
  for (long b = b0; b < b1; ++b) {
    if (kind == 2 && t->order != 4) break;
    const std::vector<int>& ix =
        kind == 0 ? t->cell_idx[b] : (kind == 1 ? t->part_idx[b] : t->soft_idx[b]);
    const std::vector<int>& of =
        kind == 0 ? t->cell_off[b] : (kind == 1 ? t->part_off[b] : t->soft_off[b]);
    if (ix.empty()) continue;
    const Node& nd = t->nodes[t->bucket_nodes[b]];
    markers[filled] = (int)pos;
    starts[filled] = (int)(nd.first + start_base);
    sizes[filled] = nd.count;
    if (bucket_ids) bucket_ids[filled] = (int)b;
    int* dst = list + 2 * pos;
    for (size_t e = 0; e < ix.size(); ++e) {
      dst[2 * e] = (int)(ix[e] + index_base);
      dst[2 * e + 1] = of[e];
    }
    pos += (long)ix.size();
    ++filled;
  }
  markers[filled] = (int)pos;
  return filled;
}

/* Releases the per-bucket walk lists once serialised. */
void chg_tree_drop_lists(void* h) {
  Tree* t = (Tree*)h;
  std::vector<std::vector<int>>().swap(t->cell_idx);
  std::vector<std::vector<int>>().swap(t->cell_off);
  std::vector<std::vector<int>>().swap(t->part_idx);
  std::vector<std::vector<int>>().swap(t->part_off);
}

}  // extern "C"
