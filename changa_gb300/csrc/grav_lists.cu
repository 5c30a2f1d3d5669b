/*
 * Interaction-list force kernels: cell (quadrupole) lists and particle lists.
 *
 * Reference behaviour (HostCUDA.cu:1008-1205 nodeGravityComputation,
 * HostCUDA.cu:1565-1751 particleGravityComputation; CPU gravity.h:267-303,
 * 398-475): for every bucket b of a request, every target particle in
 * [starts[b], starts[b]+sizes[b]) interacts with every list entry in
 * [markers[b], markers[b+1]); results accumulate (+=, max for dtGrav).
 *
 * GB300 design (not the reference's 8x16 thread tile):
 *   - a persistent grid, one warp per bucket at a time, buckets taken from
 *     a device work queue (one atomicAdd per bucket) so uneven list lengths
 *     balance themselves;
 *   - the warp's 32 lanes are split into G = 32/nt groups of nt target
 *     lanes (nt = targets in the current chunk of <= 32), so small buckets
 *     still fill the warp; group g takes list entries g, g+G, g+2G, ...;
 *   - list entries are staged 32 at a time: each lane loads one ILCell
 *     (coalesced) and gathers its source record (the moment array is small
 *     enough to stay resident in the 126 MB L2), adds the replica offset
 *     and writes a ready-to-use record to the warp's shared-memory slice;
 *     every target lane then reads records by broadcast, so the hot loop is
 *     FP32 FMA plus one MUFU rsqrt per interaction;
 *   - targets live in registers; the group partial sums are reduced through
 *     shared memory once per bucket, not per list tile.
 * Three arithmetic forms share the code:
 *   kF32  the drop-in form on the FP32 ABI structs (no accidental FP64);
 *   kF64  plain FP64 on FP64 arrays;
 *   kMix  FP32 arithmetic on bucket-relative coordinates: positions are
 *         packed as float hi + float lo parts, the bucket-centre subtraction
 *         (hi - c_hi) + (lo - c_lo) keeps the result accurate to FP32
 *         rounding of the *relative* vector, and per-tile FP32 partial sums
 *         are folded into Kahan-compensated per-particle totals.
 */
#include <cuda.h>

#include <atomic>
#include <type_traits>
#include <utility>

#include "chg_internal.h"
#include "f32x2.cuh"
#include "list_eval.cuh"

namespace chg {
namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }
__device__ __forceinline__ double max_t(double a, double b) { return fmax(a, b); }

template <typename T>
struct Acc {
  T ax, ay, az, pot, idt2;
};

/* One cell on one target (gravity.h:436-472 / HostCUDA.cu:1091-1164).
 * rec: {sx, sy, sz, M, soft, tr, xx, xy, xz, yy, yz, zz}; r = target - s. */
template <typename T>
__device__ __forceinline__ void pc_interact(const T* rec, T tx, T ty, T tz, T tsoft, T tmass,
                                            Acc<T>& acc) {
  const T rx = tx - rec[0], ry = ty - rec[1], rz = tz - rec[2];
  const T M = rec[3];
  const T rsq = rx * rx + ry * ry + rz * rz;
  if (rsq != T(0)) {
    const T dir = rsqrt_t(rsq);
    const T twoh = rec[4] + tsoft;
    T a, b, c, d;
    if (rsq < twoh * twoh) {
      splineq_near(dir, rsq, twoh, a, b, c, d);
    } else {
      const T dir2 = dir * dir;
      a = dir;
      b = dir2 * dir;
      c = T(3) * b * dir2;
      d = T(5) * c * dir2;
    }
    const T xx = rec[6], xy = rec[7], xz = rec[8], yy = rec[9], yz = rec[10], zz = rec[11];
    const T qirx = xx * rx + xy * ry + xz * rz;
    const T qiry = xy * rx + yy * ry + yz * rz;
    const T qirz = xz * rx + yz * ry + zz * rz;
    const T qir = T(0.5) * (qirx * rx + qiry * ry + qirz * rz);
    const T tr = rec[5];
    const T qir3 = b * M + d * qir - c * tr;
    acc.pot -= M * a + c * qir - b * tr;
    acc.ax -= qir3 * rx - c * qirx;
    acc.ay -= qir3 * ry - c * qiry;
    acc.az -= qir3 * rz - c * qirz;
    acc.idt2 = max_t(acc.idt2, (tmass + M) * b);
  }
}

/* One source particle on one target (gravity.h:276-301 /
 * HostCUDA.cu:1654-1711).  rec: {sx, sy, sz, m, soft}; r = s - target. */
template <typename T>
__device__ __forceinline__ void pp_interact(const T* rec, T tx, T ty, T tz, T tsoft, T tmass,
                                            Acc<T>& acc) {
  const T rx = rec[0] - tx, ry = rec[1] - ty, rz = rec[2] - tz;
  const T m = rec[3];
  const T rsq = rx * rx + ry * ry + rz * rz;
  if (rsq != T(0)) {
    const T twoh = rec[4] + tsoft;
    const T dir = rsqrt_t(rsq);
    const T r1 = rsq * dir;
    T a, b;
    if (r1 < twoh) {
      spline_near(r1, dir, twoh, a, b);
    } else {
      a = dir;
      b = dir * dir * dir;
    }
    const T bm = b * m;
    acc.pot -= m * a;
    acc.ax += rx * bm;
    acc.ay += ry * bm;
    acc.az += rz * bm;
    acc.idt2 = max_t(acc.idt2, (tmass + m) * b);
  }
}

/* One hexadecapole cell on one target: momEvalFmomrcm (moments.c:
 * 1469-1525, CUDAMoments.cu:14-109) for the scaled reduced moments of the
 * hexadecapole build; no softening (softened cells are evaluated as point
 * masses from their own list).  rec: {sx, sy, sz, M, radius, xx xy xz yy yz,
 * xxx xyy xxy yyy xxz yyz xyz, xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz};
 * r = target - s.  onethird is the reference's single-precision 1/3. */
template <typename T>
__device__ __forceinline__ void hex_eval(const T* q, T M, T u, T dir, T x, T y, T z, T& pot,
                                         T& ax, T& ay, T& az) {
  const T onethird = T(0.3333333432674408);
  u *= dir;
  T g0 = dir;
  T g2 = T(3) * dir * u * u;
  T g3 = T(5) * g2 * u;
  T g4 = T(7) * g3 * u;
  x *= dir;
  y *= dir;
  z *= dir;
  T xx = T(0.5) * x * x, xy = x * y, xz = x * z, yy = T(0.5) * y * y, yz = y * z,
    zz = T(0.5) * z * z;
  T xxx = x * (onethird * xx - zz), xxz = z * (xx - onethird * zz);
  T yyy = y * (onethird * yy - zz), yyz = z * (yy - onethird * zz);
  xx -= zz;
  yy -= zz;
  T xxy = y * xx, xyy = x * yy, xyz = xy * z;
  /* q: 0 xx 1 xy 2 xz 3 yy 4 yz 5 xxx 6 xyy 7 xxy 8 yyy 9 xxz 10 yyz 11 xyz
   *    12 xxxx 13 xyyy 14 xxxy 15 yyyy 16 xxxz 17 yyyz 18 xxyy 19 xxyz 20 xyyz */
  const T tx = g4 * (q[12] * xxx + q[13] * yyy + q[14] * xxy + q[16] * xxz + q[18] * xyy +
                     q[19] * xyz + q[20] * yyz);
  const T ty = g4 * (q[13] * xyy + q[14] * xxx + q[15] * yyy + q[17] * yyz + q[18] * xxy +
                     q[19] * xxz + q[20] * xyz);
  const T tz = g4 * (-q[12] * xxz - (q[13] + q[14]) * xyz - q[15] * yyz + q[16] * xxx +
                     q[17] * yyy - q[18] * (xxz + yyz) + q[19] * xxy + q[20] * xyy);
  g4 = T(0.25) * (tx * x + ty * y + tz * z);
  const T o3x = g3 * (q[5] * xx + q[6] * yy + q[7] * xy + q[9] * xz + q[11] * yz);
  const T o3y = g3 * (q[6] * xy + q[7] * xx + q[8] * yy + q[10] * yz + q[11] * xz);
  const T o3z = g3 * (-(q[5] + q[6]) * xz - (q[7] + q[8]) * yz + q[9] * xx + q[10] * yy +
                      q[11] * xy);
  g3 = onethird * (o3x * x + o3y * y + o3z * z);
  const T o2x = g2 * (q[0] * x + q[1] * y + q[2] * z);
  const T o2y = g2 * (q[3] * y + q[1] * x + q[4] * z);
  const T o2z = g2 * (-(q[0] + q[3]) * z + q[2] * x + q[4] * y);
  g2 = T(0.5) * (o2x * x + o2y * y + o2z * z);
  g0 *= M;
  pot -= g0 + g2 + g3 + g4;
  g0 += T(5) * g2 + T(7) * g3 + T(9) * g4;
  ax += dir * (o2x + o3x + tx - x * g0);
  ay += dir * (o2y + o3y + ty - y * g0);
  az += dir * (o2z + o3z + tz - z * g0);
}

template <typename T>
__device__ __forceinline__ void hex_interact(const T* rec, T tx, T ty, T tz, T tmass,
                                             Acc<T>& acc) {
  const T rx = tx - rec[0], ry = ty - rec[1], rz = tz - rec[2];
  const T rsq = rx * rx + ry * ry + rz * rz;
  if (rsq != T(0)) {
    const T dir = rsqrt_t(rsq);
    hex_eval<T>(rec + 5, rec[3], rec[4], dir, rx, ry, rz, acc.pot, acc.ax, acc.ay, acc.az);
    acc.idt2 = max_t(acc.idt2, (tmass + rec[3]) * dir * dir * dir);
  }
}

template <int FORM>
struct FormT {
  using T = float;  // arithmetic
  using A = float;  // reduction / output
};
template <>
struct FormT<kF64> {
  using T = double;
  using A = double;
};
template <>
struct FormT<kMix> {
  using T = float;
  using A = double;
};

/* Builds the staged record of list entry e in dst. */
template <int FORM, bool CELL, bool HEX = false>
__device__ __forceinline__ void stage_entry(const ListArgs& a, int e, float3 chi, float3 clo,
                                            typename FormT<FORM>::T* dst) {
  const int2 ent = __ldg(a.list + e);
  long long idx = ent.x;
  if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;  // memory safety
  const int code = (ent.y >> 22) & 0x1ff;
  const int ox = (code & 7) - 3, oy = ((code >> 3) & 7) - 3, oz = ((code >> 6) & 7) - 3;
  if constexpr (FORM == kF32) {
    const float fp = a.fperiod_f;
    if constexpr (CELL) {
      const float4* m = reinterpret_cast<const float4*>(
          static_cast<const CudaMultipoleMoments*>(a.src) + idx);
      const float4 m0 = __ldg(m), m1 = __ldg(m + 1), m2 = __ldg(m + 2);
      // m0 {radius, soft, M, cm.x}  m1 {cm.y, cm.z, xx, xy}  m2 {xz, yy, yz, zz}
      float4* d4 = reinterpret_cast<float4*>(dst);
      d4[0] = make_float4((float)ox * fp + m0.w, (float)oy * fp + m1.x, (float)oz * fp + m1.y, m0.z);
      d4[1] = make_float4(m0.y, 0.5f * (m1.z + m2.y + m2.w), m1.z, m1.w);
      d4[2] = m2;
    } else {
      const CompactPartData* p = static_cast<const CompactPartData*>(a.src) + idx;
      const float m = __ldg(&p->mass), s = __ldg(&p->soft);
      const float px = __ldg(&p->position.x), py = __ldg(&p->position.y), pz = __ldg(&p->position.z);
      float4* d4 = reinterpret_cast<float4*>(dst);
      d4[0] = make_float4((float)ox * fp + px, (float)oy * fp + py, (float)oz * fp + pz, m);
      d4[1] = make_float4(s, 0.f, 0.f, 0.f);
    }
  } else if constexpr (FORM == kF64) {
    const double fp = a.fperiod_d;
    if constexpr (CELL && HEX) {
      /* hexadecapole moments: 27 doubles per node */
      const double* m = static_cast<const double*>(a.src) + 27 * idx;
      dst[0] = (double)ox * fp + __ldg(m + 3);
      dst[1] = (double)oy * fp + __ldg(m + 4);
      dst[2] = (double)oz * fp + __ldg(m + 5);
      dst[3] = __ldg(m + 2);
      dst[4] = __ldg(m + 0);
#pragma unroll
      for (int k = 0; k < 21; ++k) dst[5 + k] = __ldg(m + 6 + k);
    } else if constexpr (CELL) {
      const double* m = static_cast<const double*>(a.src) + 12 * idx;
      dst[0] = (double)ox * fp + __ldg(m + 3);
      dst[1] = (double)oy * fp + __ldg(m + 4);
      dst[2] = (double)oz * fp + __ldg(m + 5);
      dst[3] = __ldg(m + 2);
      dst[4] = __ldg(m + 1);
      const double xx = __ldg(m + 6), xy = __ldg(m + 7), xz = __ldg(m + 8);
      const double yy = __ldg(m + 9), yz = __ldg(m + 10), zz = __ldg(m + 11);
      dst[5] = 0.5 * (xx + yy + zz);
      dst[6] = xx;
      dst[7] = xy;
      dst[8] = xz;
      dst[9] = yy;
      dst[10] = yz;
      dst[11] = zz;
    } else {
      const double* p = static_cast<const double*>(a.src) + 5 * idx;
      dst[0] = (double)ox * fp + __ldg(p + 2);
      dst[1] = (double)oy * fp + __ldg(p + 3);
      dst[2] = (double)oz * fp + __ldg(p + 4);
      dst[3] = __ldg(p + 0);
      dst[4] = __ldg(p + 1);
    }
  } else {  // kMix
    const float fp = a.fperiod_f;
    float4* d4 = reinterpret_cast<float4*>(dst);
    if constexpr (CELL && HEX) {
      /* packed hexadecapole cell, 8 float4: {hi.xyz, M} {lo.xyz, soft}
       * {radius, xx, xy, xz} {yy, yz, xxx, xyy} {xxy, yyy, xxz, yyz}
       * {xyz, xxxx, xyyy, xxxy} {yyyy, xxxz, yyyz, xxyy} {xxyz, xyyz, 0, 0} */
      const float4* m = static_cast<const float4*>(a.src) + kCellHexPackF4 * idx;
      const float4 h = __ldg(m), l = __ldg(m + 1);
      const float sx = ((h.x - chi.x) + (float)ox * fp) + (l.x - clo.x);
      const float sy = ((h.y - chi.y) + (float)oy * fp) + (l.y - clo.y);
      const float sz = ((h.z - chi.z) + (float)oz * fp) + (l.z - clo.z);
      d4[0] = make_float4(sx, sy, sz, h.w);
      /* rec[4] = radius, rec[5..25] = the 21 moments: the packed words 2..7
       * carry exactly that sequence */
#pragma unroll
      for (int w = 0; w < 6; ++w) d4[1 + w] = __ldg(m + 2 + w);
    } else if constexpr (CELL) {
      const float4* m = static_cast<const float4*>(a.src) + kCellPackF4 * idx;
      const float4 h = __ldg(m), l = __ldg(m + 1), q0 = __ldg(m + 2), q1 = __ldg(m + 3);
      const float sx = ((h.x - chi.x) + (float)ox * fp) + (l.x - clo.x);
      const float sy = ((h.y - chi.y) + (float)oy * fp) + (l.y - clo.y);
      const float sz = ((h.z - chi.z) + (float)oz * fp) + (l.z - clo.z);
      d4[0] = make_float4(sx, sy, sz, h.w);
      d4[1] = make_float4(l.w, q1.z, q0.x, q0.y);
      d4[2] = make_float4(q0.z, q0.w, q1.x, q1.y);
    } else {
      const float4* p = static_cast<const float4*>(a.src) + kPartPackF4 * idx;
      const float4 h = __ldg(p), l = __ldg(p + 1);
      const float sx = ((h.x - chi.x) + (float)ox * fp) + (l.x - clo.x);
      const float sy = ((h.y - chi.y) + (float)oy * fp) + (l.y - clo.y);
      const float sz = ((h.z - chi.z) + (float)oz * fp) + (l.z - clo.z);
      d4[0] = make_float4(sx, sy, sz, h.w);
      d4[1] = make_float4(l.w, 0.f, 0.f, 0.f);
    }
  }
}

template <int FORM, bool CELL, bool HEX = false>
__global__ void __launch_bounds__(kThreads, 2) list_kernel(const ListArgs a) {
  using T = typename FormT<FORM>::T;
  using A = typename FormT<FORM>::A;
  constexpr int RW = CELL ? (HEX ? 28 : 12) : 8;  // record width in T, multiple of 4
  constexpr int SB = HEX ? 16 : 32;                // entries staged per block
  __shared__ __align__(16) T stage[kWarps][SB * RW];
  __shared__ A red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* st = stage[warp];

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 h = __ldg(tp), l = __ldg(tp + 1);
      chi = make_float3(h.x, h.y, h.z);
      clo = make_float3(l.x, l.y, l.z);
    }

    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt;
      const int g = lane / nt;
      const int t = lane - g * nt;
      const bool active = g < G;
      const long long ti = tbase + t0 + t;

      T tx, ty, tz, tsoft, tmass;
      if constexpr (FORM == kF32) {
        const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
        tmass = __ldg(&p->mass);
        tsoft = __ldg(&p->soft);
        tx = __ldg(&p->position.x);
        ty = __ldg(&p->position.y);
        tz = __ldg(&p->position.z);
      } else if constexpr (FORM == kF64) {
        const double* p = static_cast<const double*>(a.tgt) + 5 * ti;
        tmass = __ldg(p);
        tsoft = __ldg(p + 1);
        tx = __ldg(p + 2);
        ty = __ldg(p + 3);
        tz = __ldg(p + 4);
      } else {
        const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
        const float4 h = __ldg(p), l = __ldg(p + 1);
        tx = (h.x - chi.x) + (l.x - clo.x);
        ty = (h.y - chi.y) + (l.y - clo.y);
        tz = (h.z - chi.z) + (l.z - clo.z);
        tmass = h.w;
        tsoft = l.w;
      }

      /* running totals: plain for kF32/kF64, Kahan pairs for kMix */
      T sx = 0, sy = 0, sz = 0, sp = 0, idt2 = 0;
      float cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;

      for (int e0 = e_begin; e0 < e_end; e0 += SB) {
        const int ne = min(SB, e_end - e0);
        if (lane < ne) stage_entry<FORM, CELL, HEX>(a, e0 + lane, chi, clo, st + lane * RW);
        __syncwarp();
        if (active) {
          Acc<T> acc{T(0), T(0), T(0), T(0), idt2};
#pragma unroll 4
          for (int k = g; k < ne; k += G) {
            if constexpr (CELL && HEX) hex_interact<T>(st + k * RW, tx, ty, tz, tmass, acc);
            else if constexpr (CELL) pc_interact<T>(st + k * RW, tx, ty, tz, tsoft, tmass, acc);
            else pp_interact<T>(st + k * RW, tx, ty, tz, tsoft, tmass, acc);
          }
          idt2 = acc.idt2;
          if constexpr (FORM == kMix) {
            kahan_add(sx, cx, acc.ax);
            kahan_add(sy, cy, acc.ay);
            kahan_add(sz, cz, acc.az);
            kahan_add(sp, cp, acc.pot);
          } else {
            sx += acc.ax;
            sy += acc.ay;
            sz += acc.az;
            sp += acc.pot;
          }
        }
        __syncwarp();
      }

      if (active) {
        if constexpr (FORM == kMix) {
          red[warp][0][lane] = (double)sx - (double)cx;
          red[warp][1][lane] = (double)sy - (double)cy;
          red[warp][2][lane] = (double)sz - (double)cz;
          red[warp][3][lane] = (double)sp - (double)cp;
        } else {
          red[warp][0][lane] = sx;
          red[warp][1][lane] = sy;
          red[warp][2][lane] = sz;
          red[warp][3][lane] = sp;
        }
        red[warp][4][lane] = (A)idt2;
      }
      __syncwarp();
      if (lane < nt) {
        A rx = 0, ry = 0, rz = 0, rp = 0, ri = 0;
        for (int gg = 0; gg < G; ++gg) {
          const int l = gg * nt + lane;
          rx += red[warp][0][l];
          ry += red[warp][1][l];
          rz += red[warp][2][l];
          rp += red[warp][3][l];
          ri = max_t(ri, red[warp][4][l]);
        }
        const long long to = tbase + t0 + lane;
        if constexpr (FORM == kF32) {
          VariablePartData* v = static_cast<VariablePartData*>(a.vars) + to;
          v->a.x += rx;
          v->a.y += ry;
          v->a.z += rz;
          v->potential += rp;
          v->dtGrav = fmaxf(ri, v->dtGrav);
        } else {
          double* v = static_cast<double*>(a.vars) + 5 * to;
          v[0] += rx;
          v[1] += ry;
          v[2] += rz;
          v[3] += rp;
          v[4] = fmax(ri, v[4]);
        }
      }
      __syncwarp();
    }
  }
}

/* ------------------------------------------------------------------ */
/* Source-parallel kernel for the FP32 arithmetic forms (kF32, kMix).  */
/*                                                                    */
/* Lanes own list entries instead of targets: each lane holds one     */
/* source record in registers and the bucket's targets are broadcast  */
/* from shared memory in chunks of kTC.  A tile of 32 sources x kTC   */
/* targets leaves every lane with kTC x 4 partial sums, which a       */
/* butterfly reduce-scatter (31 shuffles) turns into one warp total   */
/* per lane: lane l ends with target l/4, quantity l%4.  Every lane   */
/* works whatever the bucket size (buckets average ~0.7 of nBucket),  */
/* and one broadcast LDS.128 per interaction feeds ~40 FP32 ops.      */
/* ------------------------------------------------------------------ */

constexpr int kTC = 8;   // targets per reduction chunk
constexpr int kTB = 32;  // targets staged per block; larger buckets loop

/* v[k] summed over the warp; lane l returns the total of index l. */
__device__ __forceinline__ float reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s, h = 16 >> s;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const float send = up ? v[i] : v[i + h];
      const float keep = up ? v[i + h] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  return v[0];
}

/* max over the warp of v[k], k < 8; lane l returns the max of index l/4. */
__device__ __forceinline__ float max_scatter8(float (&v)[8], int lane) {
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const int o = 16 >> s, h = 4 >> s;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const float send = up ? v[i] : v[i + h];
      const float keep = up ? v[i + h] : v[i];
      v[i] = fmaxf(keep, __shfl_xor_sync(kFull, send, o));
    }
  }
  v[0] = fmaxf(v[0], __shfl_xor_sync(kFull, v[0], 2));
  v[0] = fmaxf(v[0], __shfl_xor_sync(kFull, v[0], 1));
  return v[0];
}

/* Source record held by one lane (FP32). */
struct SrcRec {
  float x, y, z, m, soft;
  float tr, xx, xy, xz, yy, yz, zz;  // cells only
};

/* ---- asynchronous gathers (cp.async, sm_80+) ---- */

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

/* Words of one source record: 16-byte words (kMix cells 4, kF32 cells 3,
 * kMix particles 2) or, for the 20-byte kF32 particles, 5 single words.
 * Stored per lane as structure of arrays, so reads are conflict-free. */
template <int FORM, bool CELL>
struct RawWords {
  static constexpr int kWords = FORM == kMix ? (CELL ? 4 : 2) : (CELL ? 3 : 5);
  static constexpr bool kWide = !(FORM == kF32 && !CELL);
};

/* Issues the asynchronous copy of source record idx into this lane's slot. */
template <int FORM, bool CELL>
__device__ __forceinline__ void fetch_source(const ListArgs& a, long long idx, float4* buf4,
                                             float* buf1, int lane) {
  using R = RawWords<FORM, CELL>;
  if constexpr (R::kWide) {
    const float4* src;
    if constexpr (FORM == kF32)
      src = reinterpret_cast<const float4*>(static_cast<const CudaMultipoleMoments*>(a.src) + idx);
    else
      src = static_cast<const float4*>(a.src) + (CELL ? kCellPackF4 : kPartPackF4) * idx;
#pragma unroll
    for (int w = 0; w < R::kWords; ++w) cp_async16(buf4 + w * 32 + lane, src + w);
  } else {
    const float* src =
        reinterpret_cast<const float*>(static_cast<const CompactPartData*>(a.src) + idx);
#pragma unroll
    for (int w = 0; w < R::kWords; ++w) cp_async4(buf1 + w * 32 + lane, src + w);
  }
}

/* Builds the lane's record from its landed words, the replica code and the
 * bucket centre (kMix: (hi - c_hi + offset) + (lo - c_lo)). */
template <int FORM, bool CELL>
__device__ __forceinline__ SrcRec finish_source(const ListArgs& a, const float4* buf4,
                                                const float* buf1, int lane, int code, float3 chi,
                                                float3 clo) {
  const float fp = a.fperiod_f;
  const float ox = (float)((code & 7) - 3) * fp, oy = (float)(((code >> 3) & 7) - 3) * fp,
              oz = (float)(((code >> 6) & 7) - 3) * fp;
  SrcRec r;
  if constexpr (FORM == kF32) {
    if constexpr (CELL) {
      const float4 m0 = buf4[lane], m1 = buf4[32 + lane], m2 = buf4[64 + lane];
      // m0 {radius, soft, M, cm.x}  m1 {cm.y, cm.z, xx, xy}  m2 {xz, yy, yz, zz}
      r.x = ox + m0.w;
      r.y = oy + m1.x;
      r.z = oz + m1.y;
      r.m = m0.z;
      r.soft = m0.y;
      r.xx = m1.z;
      r.xy = m1.w;
      r.xz = m2.x;
      r.yy = m2.y;
      r.yz = m2.z;
      r.zz = m2.w;
      r.tr = 0.5f * (r.xx + r.yy + r.zz);
    } else {
      r.m = buf1[lane];
      r.soft = buf1[32 + lane];
      r.x = ox + buf1[64 + lane];
      r.y = oy + buf1[96 + lane];
      r.z = oz + buf1[128 + lane];
    }
  } else {
    const float4 h = buf4[lane], l = buf4[32 + lane];
    r.x = ((h.x - chi.x) + ox) + (l.x - clo.x);
    r.y = ((h.y - chi.y) + oy) + (l.y - clo.y);
    r.z = ((h.z - chi.z) + oz) + (l.z - clo.z);
    r.m = h.w;
    r.soft = l.w;
    if constexpr (CELL) {
      const float4 q0 = buf4[64 + lane], q1 = buf4[96 + lane];
      r.xx = q0.x;
      r.xy = q0.y;
      r.xz = q0.z;
      r.yy = q0.w;
      r.yz = q1.x;
      r.zz = q1.y;
      r.tr = q1.z;
    }
  }
  return r;
}

/* Variants of the source-parallel kernel, chosen at run time (by the
 * autotuner or changa_gb300_set_list_variant): MINB resident blocks per SM
 * (the register cap) x GROUP source chunks per reduction (the list tile). */
struct Variant {
  int minb, group;
  int tp;  // 0 source-parallel, 1 target-parallel (list_kernel_tp), 2 paired (list_kernel_tp2),
           // 3 paired with TMA-staged cell records (list_kernel_tma; FP32-mixed cell lists,
           //   list_kernel_tp2 for the others), 4 register-blocked paired (list_kernel_rb,
           //   group = the most targets per lane)
};
constexpr Variant kVariants[] = {{2, 16, 0}, {3, 16, 0}, {4, 16, 0}, {3, 32, 0}, {2, 32, 0},
                                 {2, 0, 1},  {3, 0, 1},  {4, 0, 1},  {2, 0, 2},  {3, 0, 2},
                                 {4, 0, 2},  {2, 0, 3},  {1, 0, 3},  {2, 3, 4},  {2, 2, 4},
                                 {3, 2, 4},  {1, 3, 4}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

/* Source-parallel list kernel of the FP32 forms.  Per warp and bucket: the
 * targets (kTB at a time) sit in shared memory; for each chunk of kTC
 * targets the list streams 32 entries at a time, one per lane.  The record
 * of chunk k+1 travels to shared memory by cp.async while chunk k computes,
 * and its ILCell was loaded one chunk earlier still, so neither the list
 * stream from HBM nor the gather from L2 waits on the critical path. */
template <int FORM, bool CELL, int MINB, int GROUP>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_src(const ListArgs a) {
  static_assert(FORM != kF64, "FP32 arithmetic forms only");
  using R = RawWords<FORM, CELL>;
  constexpr int kW = R::kWords;
  constexpr int kGroup = GROUP;
  __shared__ __align__(16) float4 tpos[kWarps][kTB];  // target x, y, z, mass
  __shared__ float tsoft[kWarps][kTB];
  __shared__ __align__(16) float4 rbuf4[kWarps][2][R::kWide ? kW * 32 : 1];
  __shared__ float rbuf1[kWarps][2][R::kWide ? 1 : kW * 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 h = __ldg(tp), l = __ldg(tp + 1);
      chi = make_float3(h.x, h.y, h.z);
      clo = make_float3(l.x, l.y, l.z);
    }

    for (int tb0 = 0; tb0 < n; tb0 += kTB) {
      const int nt = min(kTB, n - tb0);
      __syncwarp();
      if (lane < nt) {
        const long long ti = tbase + tb0 + lane;
        if constexpr (FORM == kF32) {
          const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
          tpos[warp][lane] = make_float4(__ldg(&p->position.x), __ldg(&p->position.y),
                                         __ldg(&p->position.z), __ldg(&p->mass));
          tsoft[warp][lane] = __ldg(&p->soft);
        } else {
          const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
          const float4 h = __ldg(p), l = __ldg(p + 1);
          tpos[warp][lane] = make_float4((h.x - chi.x) + (l.x - clo.x),
                                         (h.y - chi.y) + (l.y - clo.y),
                                         (h.z - chi.z) + (l.z - clo.z), h.w);
          tsoft[warp][lane] = l.w;
        }
      }
      __syncwarp();
      const int nch = (nt + kTC - 1) / kTC;
      for (int c = 0; c < nch; ++c) {
        const int t0 = c * kTC;
        const int ntc = min(kTC, nt - t0);
        /* largest target softening of the chunk: pairs beyond
         * (source soft + this)^2 cannot be inside the spline */
        float smax = 0.f;
        for (int tt = 0; tt < ntc; ++tt) smax = fmaxf(smax, tsoft[warp][t0 + tt]);
        float tot = 0.f, comp = 0.f, idt = 0.f;
        for (int g0 = e_begin; g0 < e_end; g0 += 32 * kGroup) {
          const int g1 = min(e_end, g0 + 32 * kGroup);
          const int nk = (g1 - g0 + 31) >> 5;  // chunks in this group (uniform)
          float v[32], id[8];
#pragma unroll
          for (int k = 0; k < 32; ++k) v[k] = 0.f;
#pragma unroll
          for (int k = 0; k < 8; ++k) id[k] = 0.f;
          /* prologue: chunk 0's record in flight, chunk 1's ILCell loaded */
          int e = g0 + lane;
          int2 ent = e < g1 ? __ldg(a.list + e) : make_int2(0, 0);
          {
            long long idx = ent.x;
            if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;  // memory safety
            if (e < g1) fetch_source<FORM, CELL>(a, idx, rbuf4[warp][0], rbuf1[warp][0], lane);
            cp_commit();
          }
          int2 ent_next = e + 32 < g1 ? __ldg(a.list + e + 32) : make_int2(0, 0);
          for (int k = 0; k < nk; ++k, e += 32) {
            const int buf = k & 1;
            const bool valid = e < g1;
            const int code = (ent.y >> 22) & 0x1ff;
            /* start chunk k+1's gather, then wait for chunk k's */
            if (k + 1 < nk) {
              long long idx = ent_next.x;
              if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;
              if (e + 32 < g1)
                fetch_source<FORM, CELL>(a, idx, rbuf4[warp][buf ^ 1], rbuf1[warp][buf ^ 1], lane);
              cp_commit();
              ent = ent_next;
              ent_next = e + 64 < g1 ? __ldg(a.list + e + 64) : make_int2(0, 0);
              cp_wait<1>();
            } else {
              cp_wait<0>();
            }
            if (valid) {
              const SrcRec s = finish_source<FORM, CELL>(a, rbuf4[warp][buf], rbuf1[warp][buf],
                                                         lane, code, chi, clo);
              const float tw = s.soft + smax;
              const float near2 = tw * tw;
#pragma unroll
              for (int tt = 0; tt < kTC; ++tt) {
                if (tt < ntc) {
                  const float4 tp = tpos[warp][t0 + tt];
                  if constexpr (CELL) {
                    /* gravity.h:436-472: r = target - cell */
                    const float rx = tp.x - s.x, ry = tp.y - s.y, rz = tp.z - s.z;
                    const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    const float dir = rsqrtf(rsq);
                    const float dir2 = dir * dir;
                    float av = dir, bv = dir2 * dir;
                    float cv = bv * (3.f * dir2), dv = cv * (5.f * dir2);
                    if (rsq <= near2) {
                      const float twoh = s.soft + tsoft[warp][t0 + tt];
                      if (rsq == 0.f) {
                        av = bv = cv = dv = 0.f;
                      } else if (rsq < twoh * twoh) {
                        const float4 kk = splineq_near_f(dir, rsq, twoh);
                        av = kk.x;
                        bv = kk.y;
                        cv = kk.z;
                        dv = kk.w;
                      }
                    }
                    const float qirx = fmaf(s.xx, rx, fmaf(s.xy, ry, s.xz * rz));
                    const float qiry = fmaf(s.xy, rx, fmaf(s.yy, ry, s.yz * rz));
                    const float qirz = fmaf(s.xz, rx, fmaf(s.yz, ry, s.zz * rz));
                    const float qir = 0.5f * fmaf(qirx, rx, fmaf(qiry, ry, qirz * rz));
                    const float bM = bv * s.m;
                    const float qir3 = fmaf(dv, qir, fmaf(-cv, s.tr, bM));
                    v[4 * tt + 3] -= fmaf(s.m, av, fmaf(cv, qir, -bv * s.tr));
                    v[4 * tt + 0] = fmaf(cv, qirx, fmaf(-qir3, rx, v[4 * tt + 0]));
                    v[4 * tt + 1] = fmaf(cv, qiry, fmaf(-qir3, ry, v[4 * tt + 1]));
                    v[4 * tt + 2] = fmaf(cv, qirz, fmaf(-qir3, rz, v[4 * tt + 2]));
                    id[tt] = fmaxf(id[tt], fmaf(tp.w, bv, bM));
                  } else {
                    /* gravity.h:276-301: r = source - target */
                    const float rx = s.x - tp.x, ry = s.y - tp.y, rz = s.z - tp.z;
                    const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    const float dir = rsqrtf(rsq);
                    float av = dir, bv = dir * dir * dir;
                    if (rsq <= near2) {
                      const float twoh = s.soft + tsoft[warp][t0 + tt];
                      if (rsq == 0.f) {
                        av = bv = 0.f;
                      } else {
                        const float r1 = rsq * dir;
                        if (r1 < twoh) {
                          const float2 kk = spline_near_f(r1, dir, twoh);
                          av = kk.x;
                          bv = kk.y;
                        }
                      }
                    }
                    const float bm = bv * s.m;
                    v[4 * tt + 3] = fmaf(-s.m, av, v[4 * tt + 3]);
                    v[4 * tt + 0] = fmaf(rx, bm, v[4 * tt + 0]);
                    v[4 * tt + 1] = fmaf(ry, bm, v[4 * tt + 1]);
                    v[4 * tt + 2] = fmaf(rz, bm, v[4 * tt + 2]);
                    id[tt] = fmaxf(id[tt], fmaf(tp.w, bv, bm));
                  }
                }
              }
            }
          }
          /* 32 sources' partials -> lane l holds target t0 + l/4, quantity
           * l%4; groups of kGroup chunks are combined with Kahan
           * compensation (the mixed form) */
          const float r = reduce_scatter32(v, lane);
          const float mx = max_scatter8(id, lane);
          if constexpr (FORM == kMix) kahan_add(tot, comp, r);
          else tot += r;
          idt = fmaxf(idt, mx);
        }
        const int t = lane >> 2;
        if (t < ntc) {
          const int q = lane & 3;
          const long long to = tbase + tb0 + t0 + t;
          if constexpr (FORM == kF32) {
            float* vo = reinterpret_cast<float*>(static_cast<VariablePartData*>(a.vars) + to);
            vo[q] += tot;
            if (q == 0) vo[4] = fmaxf(idt, vo[4]);
          } else {
            double* vo = static_cast<double*>(a.vars) + 5 * to;
            vo[q] += (double)tot - (double)comp;
            if (q == 0) vo[4] = fmax((double)idt, vo[4]);
          }
        }
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Target-parallel kernel for the FP32 arithmetic forms (kF32, kMix).  */
/*                                                                    */
/* Lanes own targets, in G = 32 / nt groups for buckets of nt < 32     */
/* targets (group g takes the staged entries g, g + G, ...).  The list */
/* streams in blocks of 32 entries: each lane gathers one entry's raw  */
/* source record into registers a block ahead, finishes it (replica    */
/* offset, bucket-relative split coordinates) and stores it to the     */
/* warp's shared-memory slice, from where every lane reads it by       */
/* broadcast.  Accumulation is in registers with no cross-lane         */
/* reduction inside the list; the spline test runs against one         */
/* near-field radius per block ((max source soft + max target soft)^2)  */
/* and only pairs inside it take the exact per-pair test.              */
/* ------------------------------------------------------------------ */

template <int FORM, bool CELL>
__device__ __forceinline__ void gather_raw(const ListArgs& a, int e, int e_end,
                                           RawRec<FORM, CELL>& r) {
  long long idx = 0;
  r.code = 0x49;  // replica (0, 0, 0)
  if (e < e_end) {
    const int2 ent = __ldg(a.list + e);
    idx = ent.x;
    if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;  // memory safety
    r.code = (ent.y >> 22) & 0x1ff;
  }
  if constexpr (FORM == kF32) {
    if constexpr (CELL) {
      const float4* m = reinterpret_cast<const float4*>(
          static_cast<const CudaMultipoleMoments*>(a.src) + idx);
      r.w0 = __ldg(m);
      r.w1 = __ldg(m + 1);
      r.w2 = __ldg(m + 2);
    } else {
      const CompactPartData* p = static_cast<const CompactPartData*>(a.src) + idx;
      r.w0 = make_float4(__ldg(&p->position.x), __ldg(&p->position.y), __ldg(&p->position.z),
                         __ldg(&p->mass));
      r.f4 = __ldg(&p->soft);
    }
  } else {
    const float4* p = static_cast<const float4*>(a.src) + (CELL ? kCellPackF4 : kPartPackF4) * idx;
    r.w0 = __ldg(p);
    r.w1 = __ldg(p + 1);
    if constexpr (CELL) {
      r.w2 = __ldg(p + 2);
      r.w3 = __ldg(p + 3);
    }
  }
}

template <int FORM, bool CELL, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_tp(const ListArgs a) {
  static_assert(FORM != kF64, "FP32 arithmetic forms only");
  constexpr int RW = CELL ? 3 : 1;  // float4 words per staged record
  __shared__ __align__(16) float4 stage[kWarps][2][32 * RW];
  __shared__ float ssoft[kWarps][2][32];
  __shared__ double red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 h = __ldg(tp), l = __ldg(tp + 1);
      chi = make_float3(h.x, h.y, h.z);
      clo = make_float3(l.x, l.y, l.z);
    }

    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt;
      const int g = lane / nt;
      const int t = lane - g * nt;
      const bool active = g < G;
      const long long ti = tbase + t0 + t;

      float tx, ty, tz, tsoft, tmass;
      if constexpr (FORM == kF32) {
        const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
        tmass = __ldg(&p->mass);
        tsoft = __ldg(&p->soft);
        tx = __ldg(&p->position.x);
        ty = __ldg(&p->position.y);
        tz = __ldg(&p->position.z);
      } else {
        const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
        const float4 h = __ldg(p), l = __ldg(p + 1);
        tx = (h.x - chi.x) + (l.x - clo.x);
        ty = (h.y - chi.y) + (l.y - clo.y);
        tz = (h.z - chi.z) + (l.z - clo.z);
        tmass = h.w;
        tsoft = l.w;
      }
      const float tsmax = warp_max(active ? tsoft : 0.f);

      /* running totals: plain for kF32, Kahan pairs for kMix */
      float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, idt2 = 0.f;
      float cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;

      RawRec<FORM, CELL> raw;
      gather_raw<FORM, CELL>(a, e_begin + lane, e_end, raw);
      int buf = 0;
      for (int e0 = e_begin; e0 < e_end; e0 += 32, buf ^= 1) {
        const int ne = min(32, e_end - e0);
        float4* st = stage[warp][buf];
        const float ls = finish_raw<FORM, CELL>(a, raw, lane < ne, chi, clo, st + lane * RW);
        ssoft[warp][buf][lane] = ls;
        const float ss = warp_max(ls) + tsmax;
        const float near2 = ss * ss;
        __syncwarp();
        if (e0 + 32 < e_end) gather_raw<FORM, CELL>(a, e0 + 32 + lane, e_end, raw);
        float ax = 0.f, ay = 0.f, az = 0.f, pot = 0.f;
        /* one staged entry on this lane's target; entries past the list
         * end are massless records at 1e30 and add exact zeros, so every
         * block runs its full 32 slots */
        auto body = [&](int k) {
          const float4 s0 = st[k * RW];
          if constexpr (CELL) {
            /* gravity.h:436-472: r = target - cell */
            const float4 q0 = st[k * RW + 1], q1 = st[k * RW + 2];
            const float rx = tx - s0.x, ry = ty - s0.y, rz = tz - s0.z;
            const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            const float dir = rsqrt_ftz(rsq);
            const float dir2 = dir * dir;
            float av = dir, bv = dir2 * dir;
            float cv = bv * (3.f * dir2), dv = cv * (5.f * dir2);
            if (rsq <= near2) {
              const float twoh = q1.w + tsoft;
              if (rsq == 0.f) {
                av = bv = cv = dv = 0.f;
              } else if (rsq < twoh * twoh) {
                const float4 kk = splineq_near_f(dir, rsq, twoh);
                av = kk.x;
                bv = kk.y;
                cv = kk.z;
                dv = kk.w;
              }
            }
            const float qirx = fmaf(q0.x, rx, fmaf(q0.y, ry, q0.z * rz));
            const float qiry = fmaf(q0.y, rx, fmaf(q0.w, ry, q1.x * rz));
            const float qirz = fmaf(q0.z, rx, fmaf(q1.x, ry, q1.y * rz));
            const float qir = 0.5f * fmaf(qirx, rx, fmaf(qiry, ry, qirz * rz));
            const float bM = bv * s0.w;
            const float qir3 = fmaf(dv, qir, fmaf(-cv, q1.z, bM));
            pot -= fmaf(s0.w, av, fmaf(cv, qir, -bv * q1.z));
            ax = fmaf(cv, qirx, fmaf(-qir3, rx, ax));
            ay = fmaf(cv, qiry, fmaf(-qir3, ry, ay));
            az = fmaf(cv, qirz, fmaf(-qir3, rz, az));
            idt2 = fmaxf(idt2, fmaf(tmass, bv, bM));
          } else {
            /* gravity.h:276-301: r = source - target */
            const float rx = s0.x - tx, ry = s0.y - ty, rz = s0.z - tz;
            const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            const float dir = rsqrt_ftz(rsq);
            float av = dir, bv = dir * dir * dir;
            if (rsq <= near2) {
              const float twoh = ssoft[warp][buf][k] + tsoft;
              if (rsq == 0.f) {
                av = bv = 0.f;
              } else {
                const float r1 = rsq * dir;
                if (r1 < twoh) {
                  const float2 kk = spline_near_f(r1, dir, twoh);
                  av = kk.x;
                  bv = kk.y;
                }
              }
            }
            const float bm = bv * s0.w;
            pot = fmaf(-s0.w, av, pot);
            ax = fmaf(rx, bm, ax);
            ay = fmaf(ry, bm, ay);
            az = fmaf(rz, bm, az);
            idt2 = fmaxf(idt2, fmaf(tmass, bv, bm));
          }
        };
        if (G == 1) {
#pragma unroll 8
          for (int k = 0; k < 32; ++k) body(k);
        } else if (active) {
#pragma unroll 4
          for (int k = g; k < 32; k += G) body(k);
        }
        if constexpr (FORM == kMix) {
          kahan_add(sx, cx, ax);
          kahan_add(sy, cy, ay);
          kahan_add(sz, cz, az);
          kahan_add(sp, cp, pot);
        } else {
          sx += ax;
          sy += ay;
          sz += az;
          sp += pot;
        }
      }

      if (active) {
        red[warp][0][lane] = (double)sx - (double)cx;
        red[warp][1][lane] = (double)sy - (double)cy;
        red[warp][2][lane] = (double)sz - (double)cz;
        red[warp][3][lane] = (double)sp - (double)cp;
        red[warp][4][lane] = (double)idt2;
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
        const long long to = tbase + t0 + lane;
        if constexpr (FORM == kF32) {
          VariablePartData* v = static_cast<VariablePartData*>(a.vars) + to;
          v->a.x += (float)rx;
          v->a.y += (float)ry;
          v->a.z += (float)rz;
          v->potential += (float)rp;
          v->dtGrav = fmaxf((float)ri, v->dtGrav);
        } else {
          double* v = static_cast<double*>(a.vars) + 5 * to;
          v[0] += rx;
          v[1] += ry;
          v[2] += rz;
          v[3] += rp;
          v[4] = fmax(ri, v[4]);
        }
      }
      __syncwarp();
    }
  }
}

/* ------------------------------------------------------------------ */
/* Paired target-parallel kernel: list_kernel_tp with the FP32 math of  */
/* two staged sources in one packed instruction (add/mul/fma .f32x2).  */
/* The list kernels are issue-bound; packed ops issue half as many     */
/* instructions for the same FMA-pipe work.  Staged records are laid   */
/* out in pairs ({x0, x1, y0, y1} ...) so each 128-bit shared load     */
/* yields two ready operand pairs.                                     */
/* Particle lists: a block whose sources all lie beyond the softening  */
/* bound of the targets' bounding box runs a loop with no softening    */
/* test; in the other blocks the pairs within the bound are zeroed by  */
/* selects and marked, and each lane evaluates its marked sources with */
/* the spline after the block.  Neither loop branches per pair, so the */
/* compiler overlaps consecutive pairs.                                */
/* ------------------------------------------------------------------ */


template <int FORM, bool CELL, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_tp2(const ListArgs a) {
  static_assert(FORM != kF64, "FP32 arithmetic forms only");
  constexpr int NF = CELL ? 12 : 4;  // fields: x y z m [xx xy xz yy yz zz tr soft]
  constexpr int PW = NF / 2;         // float4 words per pair
  __shared__ __align__(16) float4 stage[kWarps][2][16 * PW];
  __shared__ float ssoft[kWarps][2][32];
  __shared__ double red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 h = __ldg(tp), l = __ldg(tp + 1);
      chi = make_float3(h.x, h.y, h.z);
      clo = make_float3(l.x, l.y, l.z);
    }

    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt;
      const int g = lane / nt;
      const int t = lane - g * nt;
      const bool active = g < G;
      const long long ti = tbase + t0 + t;

      float tx, ty, tz, tsoft, tmass;
      if constexpr (FORM == kF32) {
        const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
        tmass = __ldg(&p->mass);
        tsoft = __ldg(&p->soft);
        tx = __ldg(&p->position.x);
        ty = __ldg(&p->position.y);
        tz = __ldg(&p->position.z);
      } else {
        const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
        const float4 h = __ldg(p), l = __ldg(p + 1);
        tx = (h.x - chi.x) + (l.x - clo.x);
        ty = (h.y - chi.y) + (l.y - clo.y);
        tz = (h.z - chi.z) + (l.z - clo.z);
        tmass = h.w;
        tsoft = l.w;
      }
      const float tsmax = warp_max(active ? tsoft : 0.f);
      /* the targets' bounding box, against which each block's sources are
       * tested for the softening bound */
      const float3 blo = make_float3(warp_min(active ? tx : 3.4e38f),
                                     warp_min(active ? ty : 3.4e38f),
                                     warp_min(active ? tz : 3.4e38f));
      const float3 bhi = make_float3(warp_max(active ? tx : -3.4e38f),
                                     warp_max(active ? ty : -3.4e38f),
                                     warp_max(active ? tz : -3.4e38f));
      const float tms = CELL ? -tmass : tmass;  // pc_pair takes the target mass negated
      const f2 tx2 = pk2(tx, tx), ty2 = pk2(ty, ty), tz2 = pk2(tz, tz), tm2 = pk2(tms, tms);

      /* running sums (Kahan pairs in the mixed form) and dtGrav's running
       * maximum, kept negated (a running minimum) for cells as pc_pair
       * keeps it */
      float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, idt2 = 0.f;
      float cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;

      /* records one block ahead, their list entries two blocks ahead */
      RawRec<FORM, CELL> raw;
      int2 ent = load_entry(a, e_begin + lane, e_end);
      gather_raw_entry<FORM, CELL>(a, ent, raw);
      ent = load_entry(a, e_begin + 32 + lane, e_end);
      int buf = 0;
      for (int e0 = e_begin; e0 < e_end; e0 += 32, buf ^= 1) {
        const int ne = min(32, e_end - e0);
        float4 rec[3];
        const float ls = finish_raw<FORM, CELL>(a, raw, lane < ne, chi, clo, rec);
        {
          /* this lane's record into its half of pair lane/2 */
          float* pb = reinterpret_cast<float*>(stage[warp][buf] + (lane >> 1) * PW);
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
        ssoft[warp][buf][lane] = ls;
        /* no source of the block within its own softening plus the
         * targets' largest of the targets' box (then no pair of the block
         * is softened; the margin covers the rounding of the box distance);
         * the block-wide bound for the marked pairs only where some source
         * is near */
        bool far_block;
        {
          const float bx = fmaxf(fmaxf(blo.x - rec[0].x, rec[0].x - bhi.x), 0.f);
          const float by = fmaxf(fmaxf(blo.y - rec[0].y, rec[0].y - bhi.y), 0.f);
          const float bz = fmaxf(fmaxf(blo.z - rec[0].z, rec[0].z - bhi.z), 0.f);
          const float own = ls + tsmax;
          far_block = __all_sync(kFull, fmaf(bx, bx, fmaf(by, by, bz * bz)) > own * own * 1.0001f);
        }
        float near2 = 0.f;
        if (!far_block) {
          const float ss = warp_max(ls) + tsmax;
          near2 = ss * ss;
        }
        __syncwarp();
        if (e0 + 32 < e_end) {
          gather_raw_entry<FORM, CELL>(a, ent, raw);
          ent = load_entry(a, e0 + 64 + lane, e_end);
        }
        const float4* st = stage[warp][buf];
        f2 ax2 = 0ull, ay2 = 0ull, az2 = 0ull, pot2 = 0ull;  // +0.0f in both halves
        f2 pw2 = 0ull;
        unsigned nmask = 0;  // particles: sources left for the softened pass
        using Far = std::integral_constant<bool, false>;
        using Mark = std::integral_constant<bool, true>;
        /* one staged cell pair on this lane's target, with or without the
         * softening test */
        auto body = [&](int p, auto near) {
          pc_pair<decltype(near)::value>(st + p * PW, &ssoft[warp][buf][2 * p], tx2, ty2, tz2,
                                         tm2, tsoft, near2, pot2, pw2, ax2, ay2, az2, idt2);
        };
        /* a staged particle pair without branches: with MARK, halves within
         * the softening bound get a = b = 0 (selects) and their bit in nmask,
         * for the softened pass after the block */
        auto part_body = [&](int p, auto mark) {
          pp_pair<decltype(mark)::value>(st + p * PW, p, tx2, ty2, tz2, tm2, near2, pot2, ax2, ay2,
                                         az2, idt2, nmask);
        };
        if constexpr (CELL) {
          if (far_block) {
            if (G == 1) {
#pragma unroll 4
              for (int p = 0; p < 16; ++p) body(p, Far{});
            } else if (active) {
#pragma unroll 2
              for (int p = g; p < 16; p += G) body(p, Far{});
            }
          } else if (G == 1) {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) body(p, Mark{});
          } else if (active) {
#pragma unroll 2
            for (int p = g; p < 16; p += G) body(p, Mark{});
          }
        } else if (far_block) {
          if (G == 1) {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) part_body(p, Far{});
          } else if (active) {
#pragma unroll 2
            for (int p = g; p < 16; p += G) part_body(p, Far{});
          }
        } else {
          if (G == 1) {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) part_body(p, Mark{});
          } else if (active) {
#pragma unroll 2
            for (int p = g; p < 16; p += G) part_body(p, Mark{});
          }
        }
        /* the marked sources (within the softening bound of the block),
         * each lane its own, all lanes at once: gravity.h:276-301 with the
         * spline inside 2h, zero at r = 0 */
        float ex = 0.f, ey = 0.f, ez = 0.f, ep = 0.f;
        if constexpr (!CELL) {
          pp_soft_pass(st, ssoft[warp][buf], nmask, tx, ty, tz, tsoft, tmass, ex, ey, ez, ep,
                       idt2);
        }
        float x0, x1, y0, y1, z0, z1, p0, p1;
        up2(ax2, x0, x1);
        up2(ay2, y0, y1);
        up2(az2, z0, z1);
        up2(pot2, p0, p1);
        float pb_;  // this block's potential
        if constexpr (CELL) {
          float w0_, w1_;
          up2(pw2, w0_, w1_);
          pb_ = (p0 + p1) - 0.5f * (w0_ + w1_);
        } else {
          pb_ = -((p0 + p1) + ep);
        }
        if constexpr (FORM == kMix) {
          kahan_add(sx, cx, (x0 + x1) + ex);
          kahan_add(sy, cy, (y0 + y1) + ey);
          kahan_add(sz, cz, (z0 + z1) + ez);
          kahan_add(sp, cp, pb_);
        } else {
          sx += (x0 + x1) + ex;
          sy += (y0 + y1) + ey;
          sz += (z0 + z1) + ez;
          sp += pb_;
        }
      }

      if (active) {
        red[warp][0][lane] = (double)sx - (double)cx;
        red[warp][1][lane] = (double)sy - (double)cy;
        red[warp][2][lane] = (double)sz - (double)cz;
        red[warp][3][lane] = (double)sp - (double)cp;
        red[warp][4][lane] = CELL ? -(double)idt2 : (double)idt2;
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
        const long long to = tbase + t0 + lane;
        if constexpr (FORM == kF32) {
          VariablePartData* v = static_cast<VariablePartData*>(a.vars) + to;
          v->a.x += (float)rx;
          v->a.y += (float)ry;
          v->a.z += (float)rz;
          v->potential += (float)rp;
          v->dtGrav = fmaxf((float)ri, v->dtGrav);
        } else {
          double* v = static_cast<double*>(a.vars) + 5 * to;
          v[0] += rx;
          v[1] += ry;
          v[2] += rz;
          v[3] += rp;
          v[4] = fmax(ri, v[4]);
        }
      }
      __syncwarp();
    }
  }
}

/* ------------------------------------------------------------------ */
/* Register-blocked paired kernel: list_kernel_tp2's staging and pair   */
/* arithmetic with R targets per lane.  A chunk of nt targets is split  */
/* into c = ceil(nt / R) slots of R targets each (slot s holds targets  */
/* s, s + c, ...), and G = 32 / c groups of c lanes take the staged     */
/* pairs g, g + G, ...  With one target per lane, 32 - G nt lanes sit   */
/* idle (nt = 20: 12 of 32); R is chosen per chunk to minimise the pair */
/* steps per 32-entry block, R ceil(16 / G) (nt = 20: R = 2, 30 lanes;  */
/* nt = 24: R = 3, all 32), and each staged pair read from shared       */
/* memory serves all R targets of a lane.  The last block of a list     */
/* runs only its own pairs.                                             */
/* ------------------------------------------------------------------ */

/* targets per lane for a chunk of nt <= 32 targets, at most RMAX */
template <int RMAX>
__device__ __forceinline__ int rb_targets_per_lane(int nt) {
  int best = 1, cost = 1 << 30;
#pragma unroll
  for (int r = 1; r <= RMAX; ++r) {
    const int c = (nt + r - 1) / r, G = 32 / c;
    const int k = r * ((16 + G - 1) / G);
    if (k < cost) {
      cost = k;
      best = r;
    }
  }
  return best;
}

/* One target of a lane: packed position and mass (negated for cells, as
 * pc_pair takes it), softening, and whether it is a target of the chunk
 * (a lane's spare slots compute on target 0's data and are discarded). */
struct RbTarget {
  f2 x2, y2, z2, m2;
  float soft;
  bool valid;
};

/* running per-target sums: Kahan pairs in the mixed form, and dtGrav's
 * running maximum (kept negated, a running minimum, for cells) */
struct RbSums {
  float sx, sy, sz, sp, cx, cy, cz, cp, idt;
};

template <int FORM, bool CELL, int R>
__device__ __forceinline__ void rb_chunk(const ListArgs& a, const int lane, const int e_begin,
                                         const int e_end, const long long tb, const int nt,
                                         const float3 chi, const float3 clo,
                                         float4 (&stage)[2][16 * (CELL ? 6 : 2)],
                                         float (&ssoft)[2][32], double (&red)[5][32]) {
  constexpr int PW = CELL ? 6 : 2;  // float4 words per staged pair
  const int c = (nt + R - 1) / R;
  const int G = 32 / c;
  const int g = lane / c, s = lane - g * c;
  const bool active = g < G;

  RbTarget T[R];
  float tsm = 0.f;
  float3 blo = make_float3(3.4e38f, 3.4e38f, 3.4e38f), bhi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int t = s + k * c;
    T[k].valid = active && t < nt;
    const long long ti = tb + (T[k].valid ? t : 0);
    float tx, ty, tz, tmass, tsoft;
    if constexpr (FORM == kF32) {
      const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
      tmass = __ldg(&p->mass);
      tsoft = __ldg(&p->soft);
      tx = __ldg(&p->position.x);
      ty = __ldg(&p->position.y);
      tz = __ldg(&p->position.z);
    } else {
      const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
      const float4 h = __ldg(p), l = __ldg(p + 1);
      tx = (h.x - chi.x) + (l.x - clo.x);
      ty = (h.y - chi.y) + (l.y - clo.y);
      tz = (h.z - chi.z) + (l.z - clo.z);
      tmass = h.w;
      tsoft = l.w;
    }
    if (T[k].valid) {
      tsm = fmaxf(tsm, tsoft);
      blo = make_float3(fminf(blo.x, tx), fminf(blo.y, ty), fminf(blo.z, tz));
      bhi = make_float3(fmaxf(bhi.x, tx), fmaxf(bhi.y, ty), fmaxf(bhi.z, tz));
    }
    const float tms = CELL ? -tmass : tmass;
    T[k].x2 = pk2(tx, tx);
    T[k].y2 = pk2(ty, ty);
    T[k].z2 = pk2(tz, tz);
    T[k].m2 = pk2(tms, tms);
    T[k].soft = tsoft;
  }
  const float tsmax = warp_max(tsm);
  blo = make_float3(warp_min(blo.x), warp_min(blo.y), warp_min(blo.z));
  bhi = make_float3(warp_max(bhi.x), warp_max(bhi.y), warp_max(bhi.z));

  RbSums S[R];
#pragma unroll
  for (int k = 0; k < R; ++k) S[k] = RbSums{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};

  /* records one block ahead, their list entries two blocks ahead */
  RawRec<FORM, CELL> raw;
  int2 ent = load_entry(a, e_begin + lane, e_end);
  gather_raw_entry<FORM, CELL>(a, ent, raw);
  ent = load_entry(a, e_begin + 32 + lane, e_end);
  int buf = 0;
  for (int e0 = e_begin; e0 < e_end; e0 += 32, buf ^= 1) {
    const int ne = min(32, e_end - e0);
    const int np = (ne + 1) >> 1;  // staged pairs of this block
    float4 rec[3];
    const float ls = finish_raw<FORM, CELL>(a, raw, lane < ne, chi, clo, rec);
    {
      /* this lane's record into its half of pair lane/2 */
      float* pb = reinterpret_cast<float*>(stage[buf] + (lane >> 1) * PW);
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
    ssoft[buf][lane] = ls;
    /* no source of the block within its own softening plus the targets'
     * largest of the targets' box; the block-wide bound only where some
     * source is near */
    bool far_block;
    {
      const float bx = fmaxf(fmaxf(blo.x - rec[0].x, rec[0].x - bhi.x), 0.f);
      const float by = fmaxf(fmaxf(blo.y - rec[0].y, rec[0].y - bhi.y), 0.f);
      const float bz = fmaxf(fmaxf(blo.z - rec[0].z, rec[0].z - bhi.z), 0.f);
      const float own = ls + tsmax;
      far_block = __all_sync(kFull, fmaf(bx, bx, fmaf(by, by, bz * bz)) > own * own * 1.0001f);
    }
    float near2 = 0.f;
    if (!far_block) {
      const float ss = warp_max(ls) + tsmax;
      near2 = ss * ss;
    }
    __syncwarp();
    if (e0 + 32 < e_end) {
      gather_raw_entry<FORM, CELL>(a, ent, raw);
      ent = load_entry(a, e0 + 64 + lane, e_end);
    }
    const float4* st = stage[buf];
    const float* sf = ssoft[buf];
    f2 ax[R], ay[R], az[R], pt[R], pw[R];
    unsigned nm[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      ax[k] = ay[k] = az[k] = pt[k] = pw[k] = 0ull;  // +0.0f in both halves
      nm[k] = 0u;
    }
    /* staged pair p on every target of the lane, with or without the
     * softening test (cells) or the marking of softened pairs (particles) */
    auto step = [&](int p, auto near) {
      constexpr bool NEAR = decltype(near)::value;
      if constexpr (CELL) {
        const CellPair cpw = load_cell_pair(st + p * PW);
#pragma unroll
        for (int k = 0; k < R; ++k)
          pc_pair_w<NEAR>(cpw, sf + 2 * p, T[k].x2, T[k].y2, T[k].z2, T[k].m2, T[k].soft, near2,
                          pt[k], pw[k], ax[k], ay[k], az[k], S[k].idt);
      } else {
        const float4 w0 = st[p * PW], w1 = st[p * PW + 1];
        const f2 sx2 = pk2(w0.x, w0.y), sy2 = pk2(w0.z, w0.w), sz2 = pk2(w1.x, w1.y);
        const f2 pm = pk2(w1.z, w1.w);
#pragma unroll
        for (int k = 0; k < R; ++k) {
          /* gravity.h:276-301: r = source - target */
          const f2 rx = sub2(sx2, T[k].x2), ry = sub2(sy2, T[k].y2), rz = sub2(sz2, T[k].z2);
          const f2 rsq = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
          float q0, q1;
          up2(rsq, q0, q1);
          float a0 = rsqrt_ftz(q0), a1 = rsqrt_ftz(q1);
          if constexpr (NEAR) {
            const bool n0 = q0 <= near2, n1 = q1 <= near2;
            nm[k] |= ((n0 ? 1u : 0u) | (n1 ? 2u : 0u)) << (2 * p);
            a0 = n0 ? 0.f : a0;
            a1 = n1 ? 0.f : a1;
          }
          const f2 av = pk2(a0, a1);
          const f2 bv = mul2(mul2(av, av), av);
          const f2 bm = mul2(bv, pm);
          pt[k] = fma2(pm, av, pt[k]);  // opposite sign, negated at the fold
          ax[k] = fma2(rx, bm, ax[k]);
          ay[k] = fma2(ry, bm, ay[k]);
          az[k] = fma2(rz, bm, az[k]);
          float d0, d1;
          up2(fma2(T[k].m2, bv, bm), d0, d1);
          S[k].idt = fmax3(S[k].idt, d0, d1);
        }
      }
    };
    using Far = std::integral_constant<bool, false>;
    using Near = std::integral_constant<bool, true>;
    if (G == 1) {
      if (far_block) {
#pragma unroll(R == 1 ? 2 : 1)
        for (int p = 0; p < np; ++p) step(p, Far{});
      } else {
#pragma unroll(R == 1 ? 2 : 1)
        for (int p = 0; p < np; ++p) step(p, Near{});
      }
    } else if (active) {
      if (far_block) {
#pragma unroll 1
        for (int p = g; p < np; p += G) step(p, Far{});
      } else {
#pragma unroll 1
        for (int p = g; p < np; p += G) step(p, Near{});
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
      /* the marked sources (within the softening bound of the block), each
       * lane its own: gravity.h:276-301 with the spline inside 2h, zero at
       * r = 0 */
      float ex = 0.f, ey = 0.f, ez = 0.f, ep = 0.f;
      if constexpr (!CELL) {
        float tx, ty, tz, tm, d_;
        up2(T[k].x2, tx, d_);
        up2(T[k].y2, ty, d_);
        up2(T[k].z2, tz, d_);
        up2(T[k].m2, tm, d_);
        unsigned m = T[k].valid ? nm[k] : 0u;
        while (m) {
          const int jb = __ffs(m) - 1;
          m &= m - 1u;
          const float* pb = reinterpret_cast<const float*>(st + (jb >> 1) * PW);
          const int h = jb & 1;
          const float dx = pb[pair_slot(0, h)] - tx, dy = pb[pair_slot(1, h)] - ty,
                      dz = pb[pair_slot(2, h)] - tz, sm = pb[pair_slot(3, h)];
          const float q = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          float av = 0.f, bv = 0.f;
          if (q != 0.f) {
            av = rsqrt_ftz(q);
            bv = (av * av) * av;
            const float twoh = sf[jb] + T[k].soft;
            const float r1 = q * av;
            if (r1 < twoh) spline_near(r1, av, twoh, av, bv);
          }
          const float bm = bv * sm;
          ep = fmaf(sm, av, ep);
          ex = fmaf(dx, bm, ex);
          ey = fmaf(dy, bm, ey);
          ez = fmaf(dz, bm, ez);
          S[k].idt = fmaxf(S[k].idt, fmaf(tm, bv, bm));
        }
      }
      float x0, x1, y0, y1, z0, z1, p0, p1;
      up2(ax[k], x0, x1);
      up2(ay[k], y0, y1);
      up2(az[k], z0, z1);
      up2(pt[k], p0, p1);
      float pb_;  // this block's potential
      if constexpr (CELL) {
        float w0_, w1_;
        up2(pw[k], w0_, w1_);
        pb_ = (p0 + p1) - 0.5f * (w0_ + w1_);
      } else {
        pb_ = -((p0 + p1) + ep);
      }
      if constexpr (FORM == kMix) {
        kahan_add(S[k].sx, S[k].cx, (x0 + x1) + ex);
        kahan_add(S[k].sy, S[k].cy, (y0 + y1) + ey);
        kahan_add(S[k].sz, S[k].cz, (z0 + z1) + ez);
        kahan_add(S[k].sp, S[k].cp, pb_);
      } else {
        S[k].sx += (x0 + x1) + ex;
        S[k].sy += (y0 + y1) + ey;
        S[k].sz += (z0 + z1) + ez;
        S[k].sp += pb_;
      }
    }
  }

  /* per target slot k: the G groups' partial sums of each target */
#pragma unroll
  for (int k = 0; k < R; ++k) {
    if (T[k].valid) {
      red[0][lane] = (double)S[k].sx - (double)S[k].cx;
      red[1][lane] = (double)S[k].sy - (double)S[k].cy;
      red[2][lane] = (double)S[k].sz - (double)S[k].cz;
      red[3][lane] = (double)S[k].sp - (double)S[k].cp;
      red[4][lane] = CELL ? -(double)S[k].idt : (double)S[k].idt;
    }
    __syncwarp();
    const int t = lane + k * c;
    if (lane < c && t < nt) {
      double rx = 0, ry = 0, rz = 0, rp = 0, ri = 0;
      for (int gg = 0; gg < G; ++gg) {
        const int l = gg * c + lane;
        rx += red[0][l];
        ry += red[1][l];
        rz += red[2][l];
        rp += red[3][l];
        ri = fmax(ri, red[4][l]);
      }
      const long long to = tb + t;
      if constexpr (FORM == kF32) {
        VariablePartData* v = static_cast<VariablePartData*>(a.vars) + to;
        v->a.x += (float)rx;
        v->a.y += (float)ry;
        v->a.z += (float)rz;
        v->potential += (float)rp;
        v->dtGrav = fmaxf((float)ri, v->dtGrav);
      } else {
        double* v = static_cast<double*>(a.vars) + 5 * to;
        v[0] += rx;
        v[1] += ry;
        v[2] += rz;
        v[3] += rp;
        v[4] = fmax(ri, v[4]);
      }
    }
    __syncwarp();
  }
}

template <int FORM, bool CELL, int MINB, int RMAX>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_rb(const ListArgs a) {
  static_assert(FORM != kF64, "FP32 arithmetic forms only");
  static_assert(RMAX >= 1 && RMAX <= 3, "1 to 3 targets per lane");
  constexpr int PW = CELL ? 6 : 2;
  __shared__ __align__(16) float4 stage[kWarps][2][16 * PW];
  __shared__ float ssoft[kWarps][2][32];
  __shared__ double red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 h = __ldg(tp), l = __ldg(tp + 1);
      chi = make_float3(h.x, h.y, h.z);
      clo = make_float3(l.x, l.y, l.z);
    }
    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int r = rb_targets_per_lane<RMAX>(nt);
      if (RMAX >= 3 && r == 3) {
        rb_chunk<FORM, CELL, (RMAX >= 3 ? 3 : 1)>(a, lane, e_begin, e_end, tbase + t0, nt, chi,
                                                  clo, stage[warp], ssoft[warp], red[warp]);
      } else if (RMAX >= 2 && r == 2) {
        rb_chunk<FORM, CELL, (RMAX >= 2 ? 2 : 1)>(a, lane, e_begin, e_end, tbase + t0, nt, chi,
                                                  clo, stage[warp], ssoft[warp], red[warp]);
      } else {
        rb_chunk<FORM, CELL, 1>(a, lane, e_begin, e_end, tbase + t0, nt, chi, clo, stage[warp],
                                ssoft[warp], red[warp]);
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Paired cell kernel with TMA staging (FP32-mixed form): the packed    */
/* cell records (64 bytes, one row of a 2-D tensor map) of each         */
/* 32-entry block arrive in shared memory by eight tile::gather4 bulk   */
/* tensor copies (four rows by index each) on a per-warp mbarrier; the  */
/* next block's copy runs while the current block computes.  Each lane  */
/* then turns its raw record into its half of a staged pair, and the    */
/* arithmetic is list_kernel_tp2's (pc_pair).                           */
/* ------------------------------------------------------------------ */

/* Device status word of this library (one per device): kStatusTmaWait is
 * set when a TMA-staged list kernel gave up waiting for its copies, so its
 * forces are incomplete.  read_device_status() returns and clears it. */
__device__ unsigned int g_device_status = 0;
constexpr unsigned kStatusTmaWait = 1u;
/* polls of the wait that drains a copy still in flight after a timeout: it
 * must outlast any copy, so it never takes the test limit */
constexpr int kDrainPolls = 1 << 26;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

/* Waits for phase `parity` of the mbarrier, at most `polls` polls. */
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int polls) {
  for (int it = 0; it < polls; ++it) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

/* Lane 0: the 32 rows of one block (row indices from the lanes) into raw. */
__device__ __forceinline__ void tma_issue_block(const CUtensorMap* tmap, unsigned raw, unsigned bar,
                                                int row) {
  const unsigned full = 0xffffffffu;
  int r[32];
#pragma unroll
  for (int l = 0; l < 32; ++l) r[l] = __shfl_sync(full, row, l);
  if ((threadIdx.x & 31) == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(32 * 64)
                 : "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
          " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(raw + q * 256),
          "l"(tmap), "r"(0), "r"(r[4 * q]), "r"(r[4 * q + 1]), "r"(r[4 * q + 2]), "r"(r[4 * q + 3]),
          "r"(bar)
          : "memory");
  }
}

template <int MINB>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_tma(const ListArgs a,
                                                                  const __grid_constant__ CUtensorMap tmap,
                                                                  const int wait_polls) {
  constexpr int PW = 6;  // float4 words per staged pair
  __shared__ __align__(1024) float4 raw[kWarps][32 * kCellPackF4];
  __shared__ __align__(16) float4 stage[kWarps][16 * PW];
  __shared__ float ssoft[kWarps][32];
  __shared__ __align__(8) unsigned long long bars[kWarps];
  __shared__ double red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const unsigned bar = smem_u32(&bars[warp]), rawa = smem_u32(raw[warp]);
  if (lane == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  unsigned phase = 0;
  bool ok = true;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(full, b, 0);
    if (b >= a.n_buckets || !ok) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    const float4* tp0 = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
    const float4 ch = __ldg(tp0), cl = __ldg(tp0 + 1);
    const float3 chi = make_float3(ch.x, ch.y, ch.z), clo = make_float3(cl.x, cl.y, cl.z);

    for (int t0 = 0; t0 < n && ok; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt;
      const int g = lane / nt;
      const int t = lane - g * nt;
      const bool active = g < G;
      const long long ti = tbase + t0 + t;
      const float4* pp = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
      const float4 h = __ldg(pp), l = __ldg(pp + 1);
      const float tx = (h.x - chi.x) + (l.x - clo.x);
      const float ty = (h.y - chi.y) + (l.y - clo.y);
      const float tz = (h.z - chi.z) + (l.z - clo.z);
      const float tmass = h.w, tsoft = l.w;
      const float tsmax = warp_max(active ? tsoft : 0.f);
      const f2 tx2 = pk2(tx, tx), ty2 = pk2(ty, ty), tz2 = pk2(tz, tz), tm2 = pk2(-tmass, -tmass);

      float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, idt2 = 0.f;
      float cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;
      /* this lane's entry of the first block: its row and replica code */
      auto entry = [&](int e, int& row, int& code) {
        row = 0;
        code = 0x49;  // replica (0, 0, 0)
        if (e < e_end) {
          const int2 ent = __ldg(a.list + e);
          row = ent.x;
          if ((unsigned long long)row >= (unsigned long long)a.n_src) row = 0;  // memory safety
          code = (ent.y >> 22) & 0x1ff;
        }
      };
      int row = 0, code = 0x49;
      if (e_begin < e_end) {  // uniform; every issued block is waited for below
        entry(e_begin + lane, row, code);
        tma_issue_block(&tmap, rawa, bar, row);
      }
      for (int e0 = e_begin; e0 < e_end; e0 += 32) {
        const int ne = min(32, e_end - e0);
        if (!mbar_wait(bar, phase, wait_polls)) {
          if (lane == 0) atomicOr(&g_device_status, kStatusTmaWait);
          /* the block's copy is still in flight into this warp's raw buffer:
           * wait for it (long, bounded) before the warp stops and the CTA can
           * end */
          mbar_wait(bar, phase, kDrainPolls);
          ok = false;
          break;
        }
        phase ^= 1u;
        /* this lane's raw record into its half of pair lane/2 */
        {
          const float4* rr = raw[warp] + lane * kCellPackF4;
          const float4 w0 = rr[0], w1 = rr[1], w2 = rr[2], w3 = rr[3];
          const float fp = a.fperiod_f;
          const float ox = (float)((code & 7) - 3) * fp, oy = (float)(((code >> 3) & 7) - 3) * fp,
                      oz = (float)(((code >> 6) & 7) - 3) * fp;
          const bool valid = lane < ne;
          const float4 p = valid ? make_float4(((w0.x - chi.x) + ox) + (w1.x - clo.x),
                                               ((w0.y - chi.y) + oy) + (w1.y - clo.y),
                                               ((w0.z - chi.z) + oz) + (w1.z - clo.z), w0.w)
                                 : make_float4(1e30f, 1e30f, 1e30f, 0.f);
          const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
          // w2 {xx, xy, xz, yy}  w3 {yz, zz, tr, 0}
          const float4 q1 = valid ? w2 : zero, q2 = valid ? make_float4(w3.x, w3.y, w3.z, 0.f) : zero;
          float* pb = reinterpret_cast<float*>(stage[warp] + (lane >> 1) * PW);
          stage_cell_half(pb, lane & 1, p, q1, q2);
          const float ls = valid ? w1.w : 0.f;
          ssoft[warp][lane] = ls;
          const float ss = warp_max(ls) + tsmax;
          /* the raw buffer is free again: order the reads above before the
           * next block's bulk copies into it */
          __syncwarp();
          if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (e0 + 32 < e_end) {
            entry(e0 + 32 + lane, row, code);
            tma_issue_block(&tmap, rawa, bar, row);
          }
          const float near2 = ss * ss;
          const float4* st = stage[warp];
          f2 ax2 = 0ull, ay2 = 0ull, az2 = 0ull, pot2 = 0ull, pw2 = 0ull;
          if (G == 1) {
#pragma unroll 4
            for (int q = 0; q < 16; ++q)
              pc_pair(st + q * PW, &ssoft[warp][2 * q], tx2, ty2, tz2, tm2, tsoft, near2, pot2,
                      pw2, ax2, ay2, az2, idt2);
          } else if (active) {
#pragma unroll 2
            for (int q = g; q < 16; q += G)
              pc_pair(st + q * PW, &ssoft[warp][2 * q], tx2, ty2, tz2, tm2, tsoft, near2, pot2,
                      pw2, ax2, ay2, az2, idt2);
          }
          __syncwarp();  // the stage is rewritten by the next block
          float x0, x1, y0, y1, z0, z1, p0, p1;
          up2(ax2, x0, x1);
          up2(ay2, y0, y1);
          up2(az2, z0, z1);
          up2(pot2, p0, p1);
          float w0_, w1_;
          up2(pw2, w0_, w1_);
          kahan_add(sx, cx, x0 + x1);
          kahan_add(sy, cy, y0 + y1);
          kahan_add(sz, cz, z0 + z1);
          kahan_add(sp, cp, (p0 + p1) - 0.5f * (w0_ + w1_));
        }
      }
      if (!ok) break;

      if (active) {
        red[warp][0][lane] = (double)sx - (double)cx;
        red[warp][1][lane] = (double)sy - (double)cy;
        red[warp][2][lane] = (double)sz - (double)cz;
        red[warp][3][lane] = (double)sp - (double)cp;
        red[warp][4][lane] = -(double)idt2;  // pc_pair keeps dtGrav negated
      }
      __syncwarp();
      if (lane < nt) {
        double rx = 0, ry = 0, rz = 0, rp = 0, ri = 0;
        for (int gg = 0; gg < G; ++gg) {
          const int l2 = gg * nt + lane;
          rx += red[warp][0][l2];
          ry += red[warp][1][l2];
          rz += red[warp][2][l2];
          rp += red[warp][3][l2];
          ri = fmax(ri, red[warp][4][l2]);
        }
        double* v = static_cast<double*>(a.vars) + 5 * (tbase + t0 + lane);
        v[0] += rx;
        v[1] += ry;
        v[2] += rz;
        v[3] += rp;
        v[4] = fmax(ri, v[4]);
      }
      __syncwarp();
    }
  }
}

/* ------------------------------------------------------------------ */
/* Paired target-parallel kernel for hexadecapole cells (FP32-mixed):  */
/* list_kernel_tp2's structure with momEvalFmomrcm (hex_eval) on two    */
/* staged cells per .f32x2 instruction.  Staged pair: 26 fields {x y z */
/* M radius, 21 moments} of both cells, 13 float4 words; hexadecapole  */
/* cells carry no softening (softened cells have their own list), so   */
/* there is no near-field branch.  One staging buffer per warp (the    */
/* record is 2.2x the quadrupole's); the next block's packed records   */
/* are loaded into registers while the current block computes.        */
/* ------------------------------------------------------------------ */

struct RawHex {
  float4 w[kCellHexPackF4];
  int code;
};

/* Raw record of entry e: kMix, the packed cell (8 float4); kF32 (the
 * drop-in of the hexadecapole build), the 108-byte CudaMultipoleMoments
 * (27 floats, 4-byte aligned) rearranged into the same words with a zero
 * low part. */
template <int FORM>
__device__ __forceinline__ void gather_hex(const ListArgs& a, int e, int e_end, RawHex& r) {
  long long idx = 0;
  r.code = 0x49;  // replica (0, 0, 0)
  if (e < e_end) {
    const int2 ent = __ldg(a.list + e);
    idx = ent.x;
    if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;  // memory safety
    r.code = (ent.y >> 22) & 0x1ff;
  }
  if constexpr (FORM == kMix) {
    const float4* p = static_cast<const float4*>(a.src) + kCellHexPackF4 * idx;
#pragma unroll
    for (int k = 0; k < kCellHexPackF4; ++k) r.w[k] = __ldg(p + k);
  } else {
#ifdef HEXADECAPOLE
    /* {radius, soft, totalMass, cm.xyz, then the 21 moments} */
    const float* m = reinterpret_cast<const float*>(static_cast<const CudaMultipoleMoments*>(a.src) + idx);
    float v[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) v[k] = __ldg(m + k);
    r.w[0] = make_float4(v[3], v[4], v[5], v[2]);
    r.w[1] = make_float4(0.f, 0.f, 0.f, v[1]);
    float q[24];
    q[0] = v[0];
#pragma unroll
    for (int k = 0; k < 21; ++k) q[1 + k] = v[6 + k];
    q[22] = q[23] = 0.f;
#pragma unroll
    for (int w = 0; w < 6; ++w) r.w[2 + w] = make_float4(q[4 * w], q[4 * w + 1], q[4 * w + 2], q[4 * w + 3]);
#else
    static_assert(FORM == kMix, "the FP32 hexadecapole drop-in exists in the HEXADECAPOLE build");
#endif
  }
}

/* One record into half h of a staged pair (kHexFields fields): the source
 * position with the replica offset (kMix: relative to the bucket's centre,
 * as stage_entry forms it; kF32: offset + cm as the reference forms it,
 * HostCUDA.cu:1094-1099), M, then the 21 reduced moments each scaled by its
 * order's gamma factor at unit distance (second order 3 R^2, third 15 R^3,
 * fourth 105 R^4, R the radius), so that the pair evaluation multiplies
 * them by 1/r^3, 1/r^4, 1/r^5 only, and four sums of scaled moments the
 * traces need (the first negated).  Entries past the list end become massless cells far away
 * (they add exact zeros). */
constexpr int kHexFields = 30;  // 15 float4 words per staged pair

template <int FORM>
__device__ __forceinline__ void stage_hex(const ListArgs& a, const RawHex& r, bool valid,
                                          float3 chi, float3 clo, float* pb, int h) {
  const float fp = a.fperiod_f;
  const float4 hi = r.w[0], lo = r.w[1];
  const float ox = (float)((r.code & 7) - 3) * fp, oy = (float)(((r.code >> 3) & 7) - 3) * fp,
              oz = (float)(((r.code >> 6) & 7) - 3) * fp;
  float f[kHexFields];
  if constexpr (FORM == kMix) {
    f[0] = ((hi.x - chi.x) + ox) + (lo.x - clo.x);
    f[1] = ((hi.y - chi.y) + oy) + (lo.y - clo.y);
    f[2] = ((hi.z - chi.z) + oz) + (lo.z - clo.z);
  } else {
    f[0] = ox + hi.x;
    f[1] = oy + hi.y;
    f[2] = oz + hi.z;
  }
  f[3] = hi.w;
  /* raw words 2..7: the radius, then the 21 moments (two zeros after) */
  float q[24];
#pragma unroll
  for (int w = 0; w < 6; ++w) {
    const float4 v = r.w[2 + w];
    q[4 * w] = v.x;
    q[4 * w + 1] = v.y;
    q[4 * w + 2] = v.z;
    q[4 * w + 3] = v.w;
  }
  const float R = q[0];
  const float R2 = R * R;
  const float s2 = 3.f * R2, s3 = 5.f * s2 * R, s4 = 7.f * s3 * R;
#pragma unroll
  for (int k = 0; k < 21; ++k) f[4 + k] = q[1 + k] * (k < 5 ? s2 : (k < 12 ? s3 : s4));
  f[25] = -(f[4] + f[7]);  // -(Q0 + Q3)
  f[26] = f[9] + f[10];   // Q5 + Q6
  f[27] = f[11] + f[12];  // Q7 + Q8
  f[28] = f[17] + f[18];  // Q13 + Q14
  f[29] = 0.f;
  if (!valid) {
    f[0] = f[1] = f[2] = 1e30f;
#pragma unroll
    for (int k = 3; k < kHexFields; ++k) f[k] = 0.f;
  }
#pragma unroll
  for (int k = 0; k < kHexFields; ++k) pb[pair_slot(k, h)] = f[k];
}

__device__ __forceinline__ f2 lo2(float4 v) { return pk2(v.x, v.y); }
__device__ __forceinline__ f2 hi2(float4 v) { return pk2(v.z, v.w); }

/* hex_eval (momEvalFmomrcm, moments.c) on the two cells of staged pair w
 * (15 words, stage_hex's fields) for one target, r = target - cell.  Field
 * k of the pair sits in word k/2, in its low half for even k and its high
 * half for odd k.  With x = r/|r| and the staged moments Q' already scaled
 * by the gamma factor of their order at unit distance, the gammas are
 * d3 = 1/r^3, d4 = 1/r^4, d5 = 1/r^5:
 *   P2 = Q'2 x (quadrupole), P3 = Q'3 xx (octupole), P4 = Q'4 xxx
 *   (hexadecapole), a_n = P_n . x,
 *   pot -= M/r + d3 a2 / 2 + d4 a3 / 3 + d5 a4 / 4,
 *   acc += (d3 P2 + d4 P3 + d5 P4 - x G) / r,
 *   G = M/r + 5/2 d3 a2 + 7/3 d4 a3 + 9/4 d5 a4,
 * which is the reference's evaluation with its gammas g2 = 3 R^2/r^3,
 * g3 = 5 g2 R/r, g4 = 7 g3 R/r folded into the moments. */
__device__ __forceinline__ void hex_pair(const float4* __restrict__ w, f2 tx2, f2 ty2, f2 tz2,
                                         f2 tm2, f2& pot2, f2& ax2, f2& ay2, f2& az2,
                                         float& idt2) {
  const f2 CH = pk2(0.5f, 0.5f), CMH = pk2(-0.5f, -0.5f), CQ = pk2(0.25f, 0.25f);
  const float third = 0.3333333432674408f;  // the reference's single-precision 1/3
  const f2 C13 = pk2(third, third);
  const f2 K2 = pk2(2.5f, 2.5f), K3 = pk2(7.f * third, 7.f * third), K4 = pk2(2.25f, 2.25f);
  const float4 w0 = w[0], w1 = w[1];
  const f2 rx = sub2(tx2, lo2(w0)), ry = sub2(ty2, hi2(w0)), rz = sub2(tz2, lo2(w1));
  const f2 M = hi2(w1);
  const f2 rsq = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
  float q0, q1;
  up2(rsq, q0, q1);
  /* rsq = 0 (a cell at the target) contributes nothing, as in
   * hex_interact; the far padding records give rsq = inf and dir = 0 */
  const f2 dir = pk2(q0 > 0.f ? rsqrt_ftz(q0) : 0.f, q1 > 0.f ? rsqrt_ftz(q1) : 0.f);
  const f2 d2 = mul2(dir, dir);
  const f2 d3 = mul2(d2, dir), d4 = mul2(d2, d2);
  const f2 d5 = mul2(d4, dir);
  const f2 x = mul2(rx, dir), y = mul2(ry, dir), z = mul2(rz, dir);
  f2 xx = mul2(mul2(CH, x), x), yy = mul2(mul2(CH, y), y);
  const f2 xy = mul2(x, y), xz = mul2(x, z), yz = mul2(y, z);
  const f2 nzz = mul2(mul2(CMH, z), z);  // -zz
  const f2 xxx = mul2(x, fma2(C13, xx, nzz)), xxz = mul2(z, fma2(C13, nzz, xx));
  const f2 yyy = mul2(y, fma2(C13, yy, nzz)), yyz = mul2(z, fma2(C13, nzz, yy));
  xx = add2(xx, nzz);
  yy = add2(yy, nzz);
  const f2 xxy = mul2(y, xx), xyy = mul2(x, yy), xyz = mul2(xy, z);
  const float4 w2 = w[2], w3 = w[3], w4 = w[4], w5 = w[5], w6 = w[6], w7 = w[7], w8 = w[8],
               w9 = w[9], w10 = w[10], w11 = w[11], w12 = w[12], w13 = w[13], w14 = w[14];
  /* scaled moment k is field 4 + k */
  const f2 Q0 = lo2(w2), Q1 = hi2(w2), Q2 = lo2(w3), Q3 = hi2(w3), Q4 = lo2(w4), Q5 = hi2(w4),
           Q6 = lo2(w5), Q7 = hi2(w5), Q8 = lo2(w6), Q9 = hi2(w6), Q10 = lo2(w7), Q11 = hi2(w7),
           Q12 = lo2(w8), Q13 = hi2(w8), Q14 = lo2(w9), Q15 = hi2(w9), Q16 = lo2(w10),
           Q17 = hi2(w10), Q18 = lo2(w11), Q19 = hi2(w11), Q20 = lo2(w12);
  const f2 nQ03 = hi2(w12), Q56 = lo2(w13), Q78 = hi2(w13), Q1314 = lo2(w14);
  /* hexadecapole */
  f2 t = mul2(Q12, xxx);
  t = fma2(Q13, yyy, t);
  t = fma2(Q14, xxy, t);
  t = fma2(Q16, xxz, t);
  t = fma2(Q18, xyy, t);
  t = fma2(Q19, xyz, t);
  const f2 p4x = fma2(Q20, yyz, t);
  t = mul2(Q13, xyy);
  t = fma2(Q14, xxx, t);
  t = fma2(Q15, yyy, t);
  t = fma2(Q17, yyz, t);
  t = fma2(Q18, xxy, t);
  t = fma2(Q19, xxz, t);
  const f2 p4y = fma2(Q20, xyz, t);
  t = mul2(Q16, xxx);
  t = fma2(Q17, yyy, t);
  t = fma2(Q19, xxy, t);
  t = fma2(Q20, xyy, t);
  f2 sm = mul2(Q12, xxz);
  sm = fma2(Q1314, xyz, sm);
  sm = fma2(Q15, yyz, sm);
  sm = fma2(Q18, add2(xxz, yyz), sm);
  const f2 p4z = sub2(t, sm);
  const f2 b4 = mul2(d5, fma2(p4x, x, fma2(p4y, y, mul2(p4z, z))));
  /* octupole */
  t = mul2(Q5, xx);
  t = fma2(Q6, yy, t);
  t = fma2(Q7, xy, t);
  t = fma2(Q9, xz, t);
  const f2 p3x = fma2(Q11, yz, t);
  t = mul2(Q6, xy);
  t = fma2(Q7, xx, t);
  t = fma2(Q8, yy, t);
  t = fma2(Q10, yz, t);
  const f2 p3y = fma2(Q11, xz, t);
  t = mul2(Q9, xx);
  t = fma2(Q10, yy, t);
  t = fma2(Q11, xy, t);
  const f2 p3z = sub2(t, fma2(Q56, xz, mul2(Q78, yz)));
  const f2 b3 = mul2(d4, fma2(p3x, x, fma2(p3y, y, mul2(p3z, z))));
  /* quadrupole */
  const f2 p2x = fma2(Q0, x, fma2(Q1, y, mul2(Q2, z)));
  const f2 p2y = fma2(Q3, y, fma2(Q1, x, mul2(Q4, z)));
  const f2 p2z = fma2(Q2, x, fma2(Q4, y, mul2(nQ03, z)));
  const f2 b2 = mul2(d3, fma2(p2x, x, fma2(p2y, y, mul2(p2z, z))));
  const f2 g0 = mul2(dir, M);
  /* pot -= g0 + b2/2 + b3/3 + b4/4: accumulated with the opposite sign */
  pot2 = add2(pot2, fma2(CH, b2, fma2(C13, b3, fma2(CQ, b4, g0))));
  const f2 ng = sub2(pk2(0.f, 0.f), fma2(K2, b2, fma2(K3, b3, fma2(K4, b4, g0))));
  const f2 sx = fma2(d5, p4x, fma2(d4, p3x, mul2(d3, p2x)));
  const f2 sy = fma2(d5, p4y, fma2(d4, p3y, mul2(d3, p2y)));
  const f2 sz = fma2(d5, p4z, fma2(d4, p3z, mul2(d3, p2z)));
  ax2 = fma2(dir, fma2(x, ng, sx), ax2);
  ay2 = fma2(dir, fma2(y, ng, sy), ay2);
  az2 = fma2(dir, fma2(z, ng, sz), az2);
  float e0, e1;
  up2(mul2(add2(tm2, M), d3), e0, e1);
  idt2 = fmax3(idt2, e0, e1);
}

template <int FORM, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) list_kernel_hex2(const ListArgs a) {
  static_assert(FORM == kMix || FORM == kF32, "FP32 arithmetic forms only");
  constexpr int PW = kHexFields / 2;  // float4 words per staged pair
  __shared__ __align__(16) float4 stage[kWarps][16 * PW];
  __shared__ double red[kWarps][5][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);  // memory safety
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;  // memory safety

    float3 chi = make_float3(0.f, 0.f, 0.f), clo = chi;
    if constexpr (FORM == kMix) {
      const float4* tp = static_cast<const float4*>(a.tgt) + kPartPackF4 * tbase;
      const float4 ch = __ldg(tp), cl = __ldg(tp + 1);
      chi = make_float3(ch.x, ch.y, ch.z);
      clo = make_float3(cl.x, cl.y, cl.z);
    }

    for (int t0 = 0; t0 < n; t0 += 32) {
      const int nt = min(32, n - t0);
      const int G = 32 / nt;
      const int g = lane / nt;
      const int t = lane - g * nt;
      const bool active = g < G;
      const long long ti = tbase + t0 + t;
      float tx, ty, tz, tmass;
      if constexpr (FORM == kMix) {
        const float4* p = static_cast<const float4*>(a.tgt) + kPartPackF4 * ti;
        const float4 h = __ldg(p), l = __ldg(p + 1);
        tx = (h.x - chi.x) + (l.x - clo.x);
        ty = (h.y - chi.y) + (l.y - clo.y);
        tz = (h.z - chi.z) + (l.z - clo.z);
        tmass = h.w;
      } else {
        const CompactPartData* p = static_cast<const CompactPartData*>(a.tgt) + ti;
        tmass = __ldg(&p->mass);
        tx = __ldg(&p->position.x);
        ty = __ldg(&p->position.y);
        tz = __ldg(&p->position.z);
      }
      const f2 tx2 = pk2(tx, tx), ty2 = pk2(ty, ty), tz2 = pk2(tz, tz), tm2 = pk2(tmass, tmass);

      float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, idt2 = 0.f;
      float cx = 0.f, cy = 0.f, cz = 0.f, cp = 0.f;
      RawHex raw;
      gather_hex<FORM>(a, e_begin + lane, e_end, raw);
      for (int e0 = e_begin; e0 < e_end; e0 += 32) {
        const int ne = min(32, e_end - e0);
        stage_hex<FORM>(a, raw, lane < ne, chi, clo,
                        reinterpret_cast<float*>(stage[warp] + (lane >> 1) * PW), lane & 1);
        __syncwarp();
        if (e0 + 32 < e_end) gather_hex<FORM>(a, e0 + 32 + lane, e_end, raw);
        f2 ax2 = 0ull, ay2 = 0ull, az2 = 0ull, pot2 = 0ull;  // +0.0f in both halves
        const float4* st = stage[warp];
        if (G == 1) {
#pragma unroll 2
          for (int q = 0; q < 16; ++q)
            hex_pair(st + q * PW, tx2, ty2, tz2, tm2, pot2, ax2, ay2, az2, idt2);
        } else if (active) {
          for (int q = g; q < 16; q += G)
            hex_pair(st + q * PW, tx2, ty2, tz2, tm2, pot2, ax2, ay2, az2, idt2);
        }
        __syncwarp();  // the stage is rewritten by the next block
        float x0, x1, y0, y1, z0, z1, p0, p1;
        up2(ax2, x0, x1);
        up2(ay2, y0, y1);
        up2(az2, z0, z1);
        up2(pot2, p0, p1);
        if constexpr (FORM == kMix) {
          kahan_add(sx, cx, x0 + x1);
          kahan_add(sy, cy, y0 + y1);
          kahan_add(sz, cz, z0 + z1);
          kahan_add(sp, cp, -(p0 + p1));
        } else {
          sx += x0 + x1;
          sy += y0 + y1;
          sz += z0 + z1;
          sp -= p0 + p1;
        }
      }

      if (active) {
        red[warp][0][lane] = (double)sx - (double)cx;
        red[warp][1][lane] = (double)sy - (double)cy;
        red[warp][2][lane] = (double)sz - (double)cz;
        red[warp][3][lane] = (double)sp - (double)cp;
        red[warp][4][lane] = (double)idt2;
      }
      __syncwarp();
      if (lane < nt) {
        double rx = 0, ry = 0, rz = 0, rp = 0, ri = 0;
        for (int gg = 0; gg < G; ++gg) {
          const int l2 = gg * nt + lane;
          rx += red[warp][0][l2];
          ry += red[warp][1][l2];
          rz += red[warp][2][l2];
          rp += red[warp][3][l2];
          ri = fmax(ri, red[warp][4][l2]);
        }
        const long long to = tbase + t0 + lane;
        if constexpr (FORM == kF32) {
          VariablePartData* v = static_cast<VariablePartData*>(a.vars) + to;
          v->a.x += (float)rx;
          v->a.y += (float)ry;
          v->a.z += (float)rz;
          v->potential += (float)rp;
          v->dtGrav = fmaxf((float)ri, v->dtGrav);
        } else {
          double* v = static_cast<double*>(a.vars) + 5 * to;
          v[0] += rx;
          v[1] += ry;
          v[2] += rz;
          v[3] += rp;
          v[4] = fmax(ri, v[4]);
        }
      }
      __syncwarp();
    }
  }
}

__global__ void pack_cells_kernel(const double* __restrict__ m, long long n, float4* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double* r = m + 12 * i;
    const double x = r[3], y = r[4], z = r[5];
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    out[4 * i + 0] = make_float4(hx, hy, hz, (float)r[2]);
    out[4 * i + 1] = make_float4((float)(x - (double)hx), (float)(y - (double)hy),
                                 (float)(z - (double)hz), (float)r[1]);
    out[4 * i + 2] = make_float4((float)r[6], (float)r[7], (float)r[8], (float)r[9]);
    out[4 * i + 3] = make_float4((float)r[10], (float)r[11], (float)(0.5 * (r[6] + r[9] + r[11])), 0.f);
  }
}

__global__ void pack_parts_kernel(const double* __restrict__ p, long long n, float4* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double* r = p + 5 * i;
    const double x = r[2], y = r[3], z = r[4];
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    out[2 * i + 0] = make_float4(hx, hy, hz, (float)r[0]);
    out[2 * i + 1] = make_float4((float)(x - (double)hx), (float)(y - (double)hy),
                                 (float)(z - (double)hz), (float)r[1]);
  }
}

/* Packed hexadecapole cells (FP32-mixed form) from 27-double moments. */
__global__ void pack_cells_hex_kernel(const double* __restrict__ m, long long n,
                                      float4* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double* r = m + 27 * i;
    const double x = r[3], y = r[4], z = r[5];
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    float4* o = out + kCellHexPackF4 * i;
    o[0] = make_float4(hx, hy, hz, (float)r[2]);
    o[1] = make_float4((float)(x - (double)hx), (float)(y - (double)hy), (float)(z - (double)hz),
                       (float)r[1]);
    float w[24];
    w[0] = (float)r[0];
#pragma unroll
    for (int k = 0; k < 21; ++k) w[1 + k] = (float)r[6 + k];
    w[22] = 0.f;
    w[23] = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) o[2 + k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
}

/* Cells as point masses {M, soft, cm} in the particle layout: the sources
 * of the softened-cell list. */
__global__ void cells_as_parts_kernel(const double* __restrict__ m, int stride, long long n,
                                      double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double* r = m + (size_t)stride * i;
    double* o = out + 5 * i;
    o[0] = r[2];
    o[1] = r[1];
    o[2] = r[3];
    o[3] = r[4];
    o[4] = r[5];
  }
}

/* The FP64 form runs list_kernel (its cost is the FP64 pipe); the FP32
 * forms run one of the variants below: paired target-parallel by default
 * (the fastest on the measured workloads), the others on request or by the
 * autotuner. */
template <typename K>
int blocks_per_sm(K kernel, std::atomic<int>* cache) {
  int nb = cache->load(std::memory_order_relaxed);
  if (!nb) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kThreads, 0) != cudaSuccess ||
        nb < 1)
      nb = 1;
    cache->store(nb, std::memory_order_relaxed);
  }
  return nb;
}

template <typename K>
cudaError_t launch_kernel(K kernel, std::atomic<int>* occ_cache, int kid, const ListArgs& a,
                          cudaStream_t s) {
  if (a.n_buckets <= 0) return cudaSuccess;
  long long want = ((long long)a.n_buckets + kWarps - 1) / kWarps;
  long long cap = (long long)sm_count() * blocks_per_sm(kernel, occ_cache);
  int grid = (int)(want < cap ? want : cap);
  TimingScope ts(kid, s);
  kernel<<<grid, kThreads, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

/* current variant per list kernel id (FP32 forms); several host threads
 * may launch while another sets a variant, so each launch loads its id's
 * variant once, atomically */
std::atomic<int> g_variant[6] = {{8}, {10}, {0}, {0}, {8}, {10}};
/* poll limit of the TMA variants' mbarrier waits (a test hook lowers it) */
constexpr int kDefaultWaitPolls = 1 << 22;
std::atomic<int> g_tma_wait_polls{kDefaultWaitPolls};
/* TMA-variant launches since load: an entry that synchronises compares it
 * before and after to know whether to read the device status word */
std::atomic<unsigned long long> g_tma_launches{0};

/* cuTensorMapEncodeTiled, resolved through the runtime (the library
 * loads on machines without a driver). */
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)f;
    else
      cudaGetLastError();
    tried = true;
  }
  return fn;
}

/* The packed cell records as a 2-D tensor: rows of 16 floats (64 bytes),
 * one row per box (tile::gather4 takes one-row boxes). */
static bool make_cell_tmap(const void* base, long long rows, CUtensorMap* tm) {
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc || !base || rows <= 0 || rows > 0x7fffffffLL || ((uintptr_t)base & 15)) return false;
  const cuuint64_t dims[2] = {16, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {16 * sizeof(float)};
  const cuuint32_t box[2] = {16, 1};
  const cuuint32_t estr[2] = {1, 1};
  return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int MINB>
cudaError_t launch_tma(const ListArgs& a, const CUtensorMap& tm, cudaStream_t s) {
  static std::atomic<int> occ{0};
  if (a.n_buckets <= 0) return cudaSuccess;
  long long want = ((long long)a.n_buckets + kWarps - 1) / kWarps;
  long long cap = (long long)sm_count() * blocks_per_sm(list_kernel_tma<MINB>, &occ);
  int grid = (int)(want < cap ? want : cap);
  TimingScope ts(list_kernel_id(kMix, true), s);
  g_tma_launches.fetch_add(1);
  list_kernel_tma<MINB><<<grid, kThreads, 0, s>>>(a, tm, g_tma_wait_polls.load());
  count_launch();
  return cudaGetLastError();
}

template <int FORM, bool CELL, int V>
cudaError_t launch_variant(const ListArgs& a, cudaStream_t s) {
  static std::atomic<int> occ{0};
  constexpr Variant var = kVariants[V];
  if constexpr (var.tp == 3) {
    if constexpr (FORM == kMix && CELL) {
      CUtensorMap tm;
      if (make_cell_tmap(a.src, a.n_src, &tm)) return launch_tma<var.minb>(a, tm, s);
    }
    return launch_kernel(list_kernel_tp2<FORM, CELL, var.minb>, &occ, list_kernel_id(FORM, CELL),
                         a, s);
  } else if constexpr (var.tp == 4)
    return launch_kernel(list_kernel_rb<FORM, CELL, var.minb, var.group>, &occ,
                         list_kernel_id(FORM, CELL), a, s);
  else if constexpr (var.tp == 2)
    return launch_kernel(list_kernel_tp2<FORM, CELL, var.minb>, &occ, list_kernel_id(FORM, CELL),
                         a, s);
  else if constexpr (var.tp == 1)
    return launch_kernel(list_kernel_tp<FORM, CELL, var.minb>, &occ, list_kernel_id(FORM, CELL),
                         a, s);
  else
    return launch_kernel(list_kernel_src<FORM, CELL, var.minb, var.group>, &occ,
                         list_kernel_id(FORM, CELL), a, s);
}

template <int FORM, bool CELL, int... V>
cudaError_t launch_src(int v, const ListArgs& a, cudaStream_t s, std::integer_sequence<int, V...>) {
  cudaError_t e = cudaErrorInvalidValue;
  ((v == V ? (e = launch_variant<FORM, CELL, V>(a, s), 0) : 0), ...);
  return e;
}

/* the drop-in cell lists of the hexadecapole build: momEvalFmomrcm on the
 * 108-byte CudaMultipoleMoments (nodeGravityComputation with HEXADECAPOLE,
 * HostCUDA.cu:1106-1112); the quadrupole build's FP32 cell kernels are not
 * instantiated there */
#ifdef HEXADECAPOLE
constexpr bool kHexDropIn = true;
#else
constexpr bool kHexDropIn = false;
#endif

template <int FORM, bool CELL>
cudaError_t launch_t(const ListArgs& a, cudaStream_t s) {
  if constexpr (FORM == kF64) {
    static std::atomic<int> occ{0};
    return launch_kernel(list_kernel<FORM, CELL>, &occ, list_kernel_id(FORM, CELL), a, s);
  } else if constexpr (kHexDropIn && FORM == kF32 && CELL) {
    static std::atomic<int> occ{0};
    return launch_kernel(list_kernel_hex2<kF32, 2>, &occ, list_kernel_id(kF32, true), a, s);
  } else {
    return launch_src<FORM, CELL>(g_variant[list_kernel_id(FORM, CELL)].load(), a, s,
                                  std::make_integer_sequence<int, kNumVariants>{});
  }
}

}  // namespace

int list_variant_count() { return kNumVariants; }

int set_list_variant(int kernel, int variant) {
  if (kernel < 0 || kernel >= 6 || kernel == kKidListF64Cell || kernel == kKidListF64Part)
    return -1;
  if (variant < 0 || variant >= kNumVariants) return -1;
  g_variant[kernel].store(variant);
  return 0;
}

int get_list_variant(int kernel) {
  if (kernel < 0 || kernel >= 6) return -1;
  return g_variant[kernel].load();
}

void set_tma_wait_polls(int polls) { g_tma_wait_polls.store(polls >= 0 ? polls : kDefaultWaitPolls); }

unsigned long long tma_launches() { return g_tma_launches.load(); }

cudaError_t read_device_status(unsigned* bits) {
  *bits = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return e;
  unsigned v = 0;
  e = cudaMemcpyFromSymbol(&v, g_device_status, sizeof v);
  if (e == cudaSuccess && v) {
    const unsigned z = 0;
    e = cudaMemcpyToSymbol(g_device_status, &z, sizeof z);
  }
  *bits = v;
  return e;
}

cudaError_t launch_list(int form, bool cell, const ListArgs& a, cudaStream_t s) {
  switch (form) {
    case kF32: return cell ? launch_t<kF32, true>(a, s) : launch_t<kF32, false>(a, s);
    case kF64: return cell ? launch_t<kF64, true>(a, s) : launch_t<kF64, false>(a, s);
    case kMix: return cell ? launch_t<kMix, true>(a, s) : launch_t<kMix, false>(a, s);
  }
  return cudaErrorInvalidValue;
}

static int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  long long cap = (long long)sm_count() * 8;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

cudaError_t launch_pack_cells(const double* moments, long long n, float4* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  TimingScope ts(kKidPack, s);
  pack_cells_kernel<<<grid_for(n, 256), 256, 0, s>>>(moments, n, out);
  count_launch();
  return cudaGetLastError();
}

/* hexadecapole FP32-mixed cell kernel: 0 synchronous staging
 * (list_kernel<kMix, true, true>), 1/2 paired (list_kernel_hex2, 1/2
 * resident blocks per SM) */
std::atomic<int> g_hex_variant{2};

cudaError_t launch_list_hex(int form, const ListArgs& a, cudaStream_t s) {
  if (form == kF64) {
    static std::atomic<int> occ{0};
    return launch_kernel(list_kernel<kF64, true, true>, &occ, list_kernel_id(kF64, true), a, s);
  }
  if (form == kMix) {
    const int kid = list_kernel_id(kMix, true);
    const int hv = g_hex_variant.load();
    if (hv == 1) {
      static std::atomic<int> occ{0};
      return launch_kernel(list_kernel_hex2<kMix, 1>, &occ, kid, a, s);
    }
    if (hv == 2) {
      static std::atomic<int> occ{0};
      return launch_kernel(list_kernel_hex2<kMix, 2>, &occ, kid, a, s);
    }
    static std::atomic<int> occ{0};
    return launch_kernel(list_kernel<kMix, true, true>, &occ, kid, a, s);
  }
  return cudaErrorInvalidValue;
}

int set_hex_variant(int v) {
  if (v < 0 || v > 2) return -1;
  g_hex_variant.store(v);
  return 0;
}

int get_hex_variant() { return g_hex_variant.load(); }

cudaError_t launch_pack_cells_hex(const double* moments, long long n, float4* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  TimingScope ts(kKidPack, s);
  pack_cells_hex_kernel<<<grid_for(n, 256), 256, 0, s>>>(moments, n, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_cells_as_parts(const double* moments, int stride, long long n, double* out,
                                  cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  TimingScope ts(kKidPack, s);
  cells_as_parts_kernel<<<grid_for(n, 256), 256, 0, s>>>(moments, stride, n, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pack_parts(const double* parts, long long n, float4* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  TimingScope ts(kKidPack, s);
  pack_parts_kernel<<<grid_for(n, 256), 256, 0, s>>>(parts, n, out);
  count_launch();
  return cudaGetLastError();
}

}  // namespace chg
