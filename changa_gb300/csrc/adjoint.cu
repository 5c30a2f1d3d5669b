/*
 * Adjoint (vector-Jacobian product) of the tree accelerations, FP32-mixed.
 *
 * No reference counterpart: ChaNGa has no differentiable force path.  Given
 * lambda_i = dL/da_i for every particle, these kernels return dL/dx_k and
 * dL/dm_k through the same interaction lists the forward pass used, with the
 * tree topology and the lists held fixed:
 *
 *   particle lists (gravity.h:276-301): a_i += m_j b(r) r, r = x_j - x_i;
 *     d(b r)/dr = b I - c r r^T with c = -(1/r) db/dr (SPLINEQ's c), so with
 *     g = m_j (b lambda - c (r.lambda) r):  dL/dx_j += g, dL/dx_i -= g,
 *     dL/dm_j += b (r.lambda);
 *   cell lists (gravity.h:436-472): a_i = -(b M + d qir - c tr) r + c Q r,
 *     r = x_i - X_c, qir = r.Q.r/2, tr = trace(Q)/2; differentiating with
 *     db/dr = -c r, dc/dr = -d r, dd/dr = -e r needs one spline coefficient
 *     beyond SPLINEQ's d: e = -(1/r) dd/dr (far field 105/r^9, and derived
 *     below for both softened branches);
 *       g = (tr c - M b - qir d) lambda
 *           + (rl (M c + qir e - tr d) - d lQr) r - d rl Qr + c Q lambda
 *     (rl = r.lambda, lQr = lambda.Q.r) gives dL/dx_i += g, dL/dX_c -= g,
 *     dL/dM_c += -b rl, and dL/dQ_ab from the Q terms;
 *   the cell gradients then flow to the particles through the moment
 *     definitions X = sum m x / M, M = sum m, Q = sum m (x - X)(x - X)^T
 *     (MultipoleMoments.h:206-352 builds exactly these sums): for every
 *     ancestor node c of particle k, with d = x_k - X_c,
 *       dL/dx_k += (m_k / M_c) gX + m_k G d,   G = [[2gxx gxy gxz] ...],
 *       dL/dm_k += gM + gX.d / M_c + d^T Gh d,  Gh = G / 2.
 *
 * Kernel design.  One warp per bucket from a device work queue; the
 * bucket's targets (position relative to the bucket centre, softening,
 * lambda) sit in shared memory.  Targets go in tiles of 16 split between
 * the two half-warps (ceil/floor), and both halves walk the same 16 list
 * entries per step, so a lane pair (l, l + 16) sees every target of the
 * tile against one source: one shuffle completes the source's gradient,
 * which is then added once per entry.  The next step's list entry and
 * source record are loaded into registers while the current step computes.
 * Per-lane target partials accumulate over the whole list and are reduced
 * once per tile with a 16-lane butterfly reduce-scatter.
 * Source gradients go out as vector FP32 reductions (red.global.add.v4.f32:
 * 3 per cell entry, 1 per particle entry) into kReplicas copies of the
 * accumulators (chosen by warp), which bounds the terms per FP32 sum; a
 * finishing kernel adds the copies in FP64.  The moment chain then runs on
 * per-node coefficients: for particle k under node c,
 *   dL/dx_k += m_k (A_c + G_c x_k),
 *   dL/dm_k += c0_c + A_c . x_k + x_k^T G_c x_k / 2,
 * with A_c = gX/M - G_c X, c0_c = gM - gX.X/M + X^T G_c X / 2, so the sums
 * over a particle's ancestors become prefix sums down the tree (FP64).
 */
#include "chg_internal.h"

namespace chg {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kTB = 32;      // targets staged per shared-memory tile
constexpr int kReplicas = 4; // copies of the FP32 source-gradient accumulators
constexpr int kCellAcc = 12; // floats per cell accumulator {gX, gM} {gQ xx xy xz yy} {yz zz - -}
constexpr int kPartAcc = 4;  // floats per particle accumulator {gX, gm}
constexpr int kCoef = 10;    // FP64 per node coefficient set {A(3), G(6), c0}

/* a, b, c, d, e of the quadrupole spline kernel inside the softening
 * length (gravity.h:27-59 for a..d; e = -(1/r) dd/dr derived from them:
 * u < 1: e = 3/2 dih^6 / r^3; 1 <= u < 2: e = -7/r^9 + 9 dih^4 / r^5 -
 * dih^6 / (2 r^3); both meet 105/r^9 at u = 2). */
struct Spl5 {
  float b, c, d, e;
};

__device__ __noinline__ Spl5 spline5_near(float dir, float rsq, float twoh) {
  const float dih = __fdividef(2.0f, twoh);
  const float u = dih * (rsq * dir);
  const float dih2 = dih * dih, dih3 = dih2 * dih, dih4 = dih2 * dih2, dih5 = dih4 * dih,
              dih6 = dih3 * dih3;
  const float u2 = u * u;
  const float dir2 = dir * dir, dir3 = dir2 * dir;
  Spl5 k;
  if (u < 1.0f) {
    k.b = dih3 * (4.0f / 3.0f - 6.0f / 5.0f * u2 + 0.5f * u2 * u);
    k.c = dih5 * (12.0f / 5.0f - 1.5f * u);
    k.d = 1.5f * dih6 * dir;
    k.e = 1.5f * dih6 * dir3;
  } else {
    const float dir5 = dir3 * dir2, dir7 = dir5 * dir2, dir9 = dir7 * dir2;
    k.b = -1.0f / 15.0f * dir3 +
          dih3 * (8.0f / 3.0f - 3.0f * u + 6.0f / 5.0f * u2 - 1.0f / 6.0f * u2 * u);
    k.c = -1.0f / 5.0f * dir5 + 3.0f * dih4 * dir + dih5 * (-12.0f / 5.0f + 0.5f * u);
    k.d = -dir7 + 3.0f * dih4 * dir3 - 0.5f * dih6 * dir;
    k.e = -7.0f * dir9 + 9.0f * dih4 * dir5 - 0.5f * dih6 * dir3;
  }
  return k;
}

/* Butterfly reduce-scatter of 32 values over the 16 lanes of a half-warp
 * (offsets 8, 4, 2, 1): lane l ends with the totals of values
 * 2 (l & 15) and 2 (l & 15) + 1 in v[0], v[1]. */
__device__ __forceinline__ void reduce_scatter16(float (&v)[32], int lane) {
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int o = 8 >> s, h = 16 >> s;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const float send = up ? v[i] : v[i + h];
      const float keep = up ? v[i + h] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
}

__device__ __forceinline__ void red_add4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

__device__ __forceinline__ void red_add2(float* p, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(a), "f"(b) : "memory");
}

struct VjpArgs {
  const float4* src;  // packed cells (4 float4) or particles (2 float4)
  long long n_src;
  const float4* tgt;  // packed particles
  const float4* lam;  // lambda per target {x, y, z, 0}
  long long n_tgt;
  const int2* list;
  long long n_entries;
  const int* markers;
  const int* starts;
  const int* sizes;
  int n_buckets;
  float fperiod;
  double* grad_tgt;  // n_tgt x 4 {dx, dy, dz, dm}; each row written by its bucket's warp only
  float* acc;        // kReplicas x n_src x (kCellAcc | kPartAcc)
  unsigned int* queue;
};

/* One list entry as a lane holds it. */
template <bool CELL>
struct Src {
  float4 h, l, q0, q1;
  int code;
  bool valid;
  long long idx;
};

template <bool CELL>
__device__ __forceinline__ void load_src(const VjpArgs& a, int e, int e_end, Src<CELL>& s) {
  s.valid = e < e_end;
  s.idx = 0;
  s.code = 0;
  if (s.valid) {
    const int2 ent = __ldg(a.list + e);
    s.idx = ent.x;
    if ((unsigned long long)s.idx >= (unsigned long long)a.n_src) s.idx = 0;
    s.code = (ent.y >> 22) & 0x1ff;
  }
  const float4* sp = a.src + (CELL ? 4 : 2) * s.idx;
  s.h = __ldg(sp);
  s.l = __ldg(sp + 1);
  if constexpr (CELL) {
    s.q0 = __ldg(sp + 2);
    s.q1 = __ldg(sp + 3);
  }
}

template <bool CELL>
__global__ void __launch_bounds__(kThreads, 4) vjp_kernel(const VjpArgs a) {
  __shared__ __align__(16) float4 tpos[kWarps][kTB];
  __shared__ __align__(16) float4 tlam[kWarps][kTB];
  __shared__ float tsoft[kWarps][kTB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4, hl = lane & 15;
  constexpr int kStride = CELL ? kCellAcc : kPartAcc;
  float* acc = a.acc + (size_t)((blockIdx.x * kWarps + warp) % kReplicas) * a.n_src * kStride;

  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(a.queue, 1u);
    b = __shfl_sync(kFull, b, 0);
    if (b >= a.n_buckets) break;
    const int e_begin = max(__ldg(a.markers + b), 0);
    const int e_end = (int)min((long long)__ldg(a.markers + b + 1), a.n_entries);
    const long long tbase = __ldg(a.starts + b);
    const int n = __ldg(a.sizes + b);
    if (n <= 0 || tbase < 0 || tbase + n > a.n_tgt) continue;
    const float4 c0 = __ldg(a.tgt + 2 * tbase), c1 = __ldg(a.tgt + 2 * tbase + 1);
    const float3 chi = make_float3(c0.x, c0.y, c0.z), clo = make_float3(c1.x, c1.y, c1.z);

    for (int tb0 = 0; tb0 < n; tb0 += kTB) {
      const int nt = min(kTB, n - tb0);
      __syncwarp();
      if (lane < nt) {
        const long long ti = tbase + tb0 + lane;
        const float4 h = __ldg(a.tgt + 2 * ti), l = __ldg(a.tgt + 2 * ti + 1);
        tpos[warp][lane] = make_float4((h.x - chi.x) + (l.x - clo.x), (h.y - chi.y) + (l.y - clo.y),
                                       (h.z - chi.z) + (l.z - clo.z), h.w);
        tsoft[warp][lane] = l.w;
        tlam[warp][lane] = __ldg(a.lam + ti);
      }
      __syncwarp();
      for (int t16 = 0; t16 < nt; t16 += 16) {
        const int ntile = min(16, nt - t16);
        const int nh0 = (ntile + 1) >> 1;
        const int my0 = t16 + (half ? nh0 : 0);
        const int myn = half ? ntile - nh0 : nh0;
        /* the tile's bounding box and largest softening: a step whose
         * sources all lie beyond (source softening + that softening) of the
         * box has no softened pair and no pair at r = 0 */
        float blo[3], bhi[3], tsm;
        {
          const bool in = hl < ntile;
          const float4 tp = tpos[warp][t16 + (in ? hl : 0)];
          const float ts = in ? tsoft[warp][t16 + hl] : 0.f;
          const float c3[3] = {tp.x, tp.y, tp.z};
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            float lo_ = in ? c3[k] : 3.4e38f, hi_ = in ? c3[k] : -3.4e38f;
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
              lo_ = fminf(lo_, __shfl_xor_sync(kFull, lo_, o));
              hi_ = fmaxf(hi_, __shfl_xor_sync(kFull, hi_, o));
            }
            blo[k] = lo_;
            bhi[k] = hi_;
          }
          float m = ts;
#pragma unroll
          for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(kFull, m, o));
          tsm = m;
        }
        float v[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) v[k] = 0.f;
        Src<CELL> cur;
        load_src<CELL>(a, e_begin + hl, e_end, cur);
        for (int e0 = e_begin; e0 < e_end; e0 += 16) {
          Src<CELL> nxt;
          load_src<CELL>(a, e0 + 16 + hl, e_end, nxt);
          const float ox = (float)((cur.code & 7) - 3) * a.fperiod,
                      oy = (float)(((cur.code >> 3) & 7) - 3) * a.fperiod,
                      oz = (float)(((cur.code >> 6) & 7) - 3) * a.fperiod;
          float sx = ((cur.h.x - chi.x) + ox) + (cur.l.x - clo.x);
          float sy = ((cur.h.y - chi.y) + oy) + (cur.l.y - clo.y);
          float sz = ((cur.h.z - chi.z) + oz) + (cur.l.z - clo.z);
          float sm = cur.h.w;
          const float ss = cur.l.w;
          float xx = 0.f, xy = 0.f, xz = 0.f, yy = 0.f, yz = 0.f, zz = 0.f, tr = 0.f;
          if constexpr (CELL) {
            xx = cur.q0.x;
            xy = cur.q0.y;
            xz = cur.q0.z;
            yy = cur.q0.w;
            yz = cur.q1.x;
            zz = cur.q1.y;
            tr = cur.q1.z;
          }
          if (!cur.valid) {
            /* past the list end: a source without mass or moments far away
             * (r^2 stays finite in FP32), whose every term is an exact zero */
            sx = sy = sz = 1e15f;
            sm = xx = xy = xz = yy = yz = zz = tr = 0.f;
          }
          /* this source's gradient over this half's targets */
          float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
          float q_xx = 0.f, q_xy = 0.f, q_xz = 0.f, q_yy = 0.f, q_yz = 0.f, q_zz = 0.f;
          bool far_src;
          {
            const float bx = fmaxf(fmaxf(blo[0] - sx, sx - bhi[0]), 0.f);
            const float by = fmaxf(fmaxf(blo[1] - sy, sy - bhi[1]), 0.f);
            const float bz = fmaxf(fmaxf(blo[2] - sz, sz - bhi[2]), 0.f);
            const float bound = ss + tsm;
            far_src = !cur.valid ||
                      fmaf(bx, bx, fmaf(by, by, bz * bz)) > bound * bound * 1.0001f;
          }
          if (__all_sync(kFull, far_src)) {
            /* no softened pair and r > 0 for every pair of the step: the
             * far-field coefficients without per-pair tests (invalid
             * entries are discarded below) */
#pragma unroll
            for (int tt = 0; tt < 8; ++tt) {
              if (tt < myn) {
                const float4 tp = tpos[warp][my0 + tt];
                const float4 la = tlam[warp][my0 + tt];
                if constexpr (CELL) {
                  const float rx = tp.x - sx, ry = tp.y - sy, rz = tp.z - sz;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  const float dir = rsqrtf(rsq);
                  const float dir2 = dir * dir;
                  const float bv = dir2 * dir, cv = bv * (3.f * dir2), dv = cv * (5.f * dir2),
                              ev = dv * (7.f * dir2);
                  const float Qrx = fmaf(xx, rx, fmaf(xy, ry, xz * rz));
                  const float Qry = fmaf(xy, rx, fmaf(yy, ry, yz * rz));
                  const float Qrz = fmaf(xz, rx, fmaf(yz, ry, zz * rz));
                  const float Qlx = fmaf(xx, la.x, fmaf(xy, la.y, xz * la.z));
                  const float Qly = fmaf(xy, la.x, fmaf(yy, la.y, yz * la.z));
                  const float Qlz = fmaf(xz, la.x, fmaf(yz, la.y, zz * la.z));
                  const float qir = 0.5f * fmaf(Qrx, rx, fmaf(Qry, ry, Qrz * rz));
                  const float rl = fmaf(rx, la.x, fmaf(ry, la.y, rz * la.z));
                  const float lQr = fmaf(la.x, Qrx, fmaf(la.y, Qry, la.z * Qrz));
                  const float cl = tr * cv - sm * bv - qir * dv;
                  const float cr = rl * (sm * cv + qir * ev - tr * dv) - dv * lQr;
                  const float cq = -dv * rl;
                  const float gx = cl * la.x + cr * rx + cq * Qrx + cv * Qlx;
                  const float gy = cl * la.y + cr * ry + cq * Qry + cv * Qly;
                  const float gz = cl * la.z + cr * rz + cq * Qrz + cv * Qlz;
                  v[4 * tt + 0] += gx;
                  v[4 * tt + 1] += gy;
                  v[4 * tt + 2] += gz;
                  g0 -= gx;
                  g1 -= gy;
                  g2 -= gz;
                  g3 -= bv * rl;
                  const float hr = -0.5f * dv * rl;
                  const float ht = 0.5f * cv * rl;
                  const float hrx = hr * rx, hry = hr * ry;
                  q_xx += fmaf(hrx, rx, fmaf(cv * la.x, rx, ht));
                  q_yy += fmaf(hry, ry, fmaf(cv * la.y, ry, ht));
                  q_zz += fmaf(hr * rz, rz, fmaf(cv * la.z, rz, ht));
                  q_xy += fmaf(2.f * hrx, ry, cv * fmaf(la.x, ry, la.y * rx));
                  q_xz += fmaf(2.f * hrx, rz, cv * fmaf(la.x, rz, la.z * rx));
                  q_yz += fmaf(2.f * hry, rz, cv * fmaf(la.y, rz, la.z * ry));
                } else {
                  const float rx = sx - tp.x, ry = sy - tp.y, rz = sz - tp.z;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  const float dir = rsqrtf(rsq);
                  const float dir2 = dir * dir;
                  const float bv = dir2 * dir, cv = bv * (3.f * dir2);
                  const float rl = fmaf(rx, la.x, fmaf(ry, la.y, rz * la.z));
                  const float crl = cv * rl;
                  const float gx = sm * fmaf(bv, la.x, -crl * rx);
                  const float gy = sm * fmaf(bv, la.y, -crl * ry);
                  const float gz = sm * fmaf(bv, la.z, -crl * rz);
                  v[4 * tt + 0] -= gx;
                  v[4 * tt + 1] -= gy;
                  v[4 * tt + 2] -= gz;
                  g0 += gx;
                  g1 += gy;
                  g2 += gz;
                  g3 += bv * rl;
                }
              }
            }
          } else if (cur.valid) {
#pragma unroll
            for (int tt = 0; tt < 8; ++tt) {
              if (tt < myn) {
                const float4 tp = tpos[warp][my0 + tt];
                const float4 la = tlam[warp][my0 + tt];
                const float twoh = ss + tsoft[warp][my0 + tt];
                if constexpr (CELL) {
                  const float rx = tp.x - sx, ry = tp.y - sy, rz = tp.z - sz;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  if (rsq > 0.f) {
                    const float dir = rsqrtf(rsq);
                    const float dir2 = dir * dir;
                    float bv = dir2 * dir, cv = bv * (3.f * dir2), dv = cv * (5.f * dir2),
                          ev = dv * (7.f * dir2);
                    if (rsq < twoh * twoh) {
                      const Spl5 k = spline5_near(dir, rsq, twoh);
                      bv = k.b;
                      cv = k.c;
                      dv = k.d;
                      ev = k.e;
                    }
                    const float Qrx = fmaf(xx, rx, fmaf(xy, ry, xz * rz));
                    const float Qry = fmaf(xy, rx, fmaf(yy, ry, yz * rz));
                    const float Qrz = fmaf(xz, rx, fmaf(yz, ry, zz * rz));
                    const float Qlx = fmaf(xx, la.x, fmaf(xy, la.y, xz * la.z));
                    const float Qly = fmaf(xy, la.x, fmaf(yy, la.y, yz * la.z));
                    const float Qlz = fmaf(xz, la.x, fmaf(yz, la.y, zz * la.z));
                    const float qir = 0.5f * fmaf(Qrx, rx, fmaf(Qry, ry, Qrz * rz));
                    const float rl = fmaf(rx, la.x, fmaf(ry, la.y, rz * la.z));
                    const float lQr = fmaf(la.x, Qrx, fmaf(la.y, Qry, la.z * Qrz));
                    const float cl = tr * cv - sm * bv - qir * dv;
                    const float cr = rl * (sm * cv + qir * ev - tr * dv) - dv * lQr;
                    const float cq = -dv * rl;
                    const float gx = cl * la.x + cr * rx + cq * Qrx + cv * Qlx;
                    const float gy = cl * la.y + cr * ry + cq * Qry + cv * Qly;
                    const float gz = cl * la.z + cr * rz + cq * Qrz + cv * Qlz;
                    v[4 * tt + 0] += gx;
                    v[4 * tt + 1] += gy;
                    v[4 * tt + 2] += gz;
                    g0 -= gx;
                    g1 -= gy;
                    g2 -= gz;
                    g3 -= bv * rl;
                    /* dL/dQ for the stored components (off-diagonals appear
                     * twice in the forward formula) */
                    const float hr = -0.5f * dv * rl;
                    const float ht = 0.5f * cv * rl;
                    const float hrx = hr * rx, hry = hr * ry;
                    q_xx += fmaf(hrx, rx, fmaf(cv * la.x, rx, ht));
                    q_yy += fmaf(hry, ry, fmaf(cv * la.y, ry, ht));
                    q_zz += fmaf(hr * rz, rz, fmaf(cv * la.z, rz, ht));
                    q_xy += fmaf(2.f * hrx, ry, cv * fmaf(la.x, ry, la.y * rx));
                    q_xz += fmaf(2.f * hrx, rz, cv * fmaf(la.x, rz, la.z * rx));
                    q_yz += fmaf(2.f * hry, rz, cv * fmaf(la.y, rz, la.z * ry));
                  }
                } else {
                  const float rx = sx - tp.x, ry = sy - tp.y, rz = sz - tp.z;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  if (rsq > 0.f) {
                    const float dir = rsqrtf(rsq);
                    const float dir2 = dir * dir;
                    float bv = dir2 * dir, cv = bv * (3.f * dir2);
                    if (rsq < twoh * twoh) {
                      const Spl5 k = spline5_near(dir, rsq, twoh);
                      bv = k.b;
                      cv = k.c;
                    }
                    const float rl = fmaf(rx, la.x, fmaf(ry, la.y, rz * la.z));
                    const float crl = cv * rl;
                    const float gx = sm * fmaf(bv, la.x, -crl * rx);
                    const float gy = sm * fmaf(bv, la.y, -crl * ry);
                    const float gz = sm * fmaf(bv, la.z, -crl * rz);
                    v[4 * tt + 0] -= gx;
                    v[4 * tt + 1] -= gy;
                    v[4 * tt + 2] -= gz;
                    g0 += gx;
                    g1 += gy;
                    g2 += gz;
                    g3 += bv * rl;
                  }
                }
              }
            }
          }
          /* lanes l and l + 16 hold the same entry */
          g0 += __shfl_xor_sync(kFull, g0, 16);
          g1 += __shfl_xor_sync(kFull, g1, 16);
          g2 += __shfl_xor_sync(kFull, g2, 16);
          g3 += __shfl_xor_sync(kFull, g3, 16);
          if constexpr (CELL) {
            q_xx += __shfl_xor_sync(kFull, q_xx, 16);
            q_xy += __shfl_xor_sync(kFull, q_xy, 16);
            q_xz += __shfl_xor_sync(kFull, q_xz, 16);
            q_yy += __shfl_xor_sync(kFull, q_yy, 16);
            q_yz += __shfl_xor_sync(kFull, q_yz, 16);
            q_zz += __shfl_xor_sync(kFull, q_zz, 16);
          }
          if (cur.valid && half == 0) {
            float* gs = acc + kStride * cur.idx;
            red_add4(gs, g0, g1, g2, g3);
            if constexpr (CELL) {
              red_add4(gs + 4, q_xx, q_xy, q_xz, q_yy);
              red_add2(gs + 8, q_yz, q_zz);
            }
          }
          cur = nxt;
        }
        reduce_scatter16(v, lane);
        const int t = hl >> 1, q = 2 * (hl & 1);
        if (t < myn) {
          double* gt = a.grad_tgt + 4 * (tbase + tb0 + my0 + t) + q;
          gt[0] += (double)v[0];
          if (q == 0) gt[1] += (double)v[1];
        }
      }
    }
  }
}

__global__ void pack_lambda_kernel(const double* __restrict__ lam, long long n,
                                   float4* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = make_float4((float)lam[3 * i], (float)lam[3 * i + 1], (float)lam[3 * i + 2], 0.f);
}

/* Sums the particle accumulator copies into grad (FP64). */
__global__ void finish_parts_kernel(const float* __restrict__ acc, long long n,
                                    double* __restrict__ grad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 4 * n;
       i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < kReplicas; ++r) s += (double)acc[(size_t)r * 4 * n + i];
    grad[i] += s;
  }
}

/* Per node: the coefficient set {A, G, c0} of the moment chain from the
 * node's summed gradients {gX, gM, gQ} and its moments (FP64). */
__device__ void node_coef(const double* __restrict__ moments, const float* __restrict__ acc,
                          long long n_moments, long long node, double (&c)[kCoef]) {
  double g[10];
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < kReplicas; ++r)
      s += (double)acc[((size_t)r * n_moments + node) * kCellAcc + k];
    g[k] = s;
  }
  const double* mo = moments + 12 * node;
  const double M = mo[2];
  if (!(M > 0.0)) {
#pragma unroll
    for (int k = 0; k < kCoef; ++k) c[k] = 0.0;
    return;
  }
  const double X = mo[3], Y = mo[4], Z = mo[5];
  const double iM = 1.0 / M;
  /* G = [[2gxx gxy gxz] [gxy 2gyy gyz] [gxz gyz 2gzz]] */
  const double Gxx = 2 * g[4], Gxy = g[5], Gxz = g[6], Gyy = 2 * g[7], Gyz = g[8], Gzz = 2 * g[9];
  const double GX = Gxx * X + Gxy * Y + Gxz * Z;
  const double GY = Gxy * X + Gyy * Y + Gyz * Z;
  const double GZ = Gxz * X + Gyz * Y + Gzz * Z;
  const double ux = g[0] * iM, uy = g[1] * iM, uz = g[2] * iM;
  c[0] = ux - GX;
  c[1] = uy - GY;
  c[2] = uz - GZ;
  c[3] = Gxx;
  c[4] = Gxy;
  c[5] = Gxz;
  c[6] = Gyy;
  c[7] = Gyz;
  c[8] = Gzz;
  c[9] = g[3] - (ux * X + uy * Y + uz * Z) + 0.5 * (GX * X + GY * Y + GZ * Z);
}

__global__ void node_coef_kernel(const double* __restrict__ moments, const float* __restrict__ acc,
                                 long long n_moments, double* __restrict__ coef) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_moments;
       i += (long long)gridDim.x * blockDim.x) {
    double c[kCoef];
    node_coef(moments, acc, n_moments, i, c);
#pragma unroll
    for (int k = 0; k < kCoef; ++k) coef[kCoef * i + k] = c[k];
  }
}

/* prefix[i] = sum of the coefficient sets of node i and all its ancestors. */
__global__ void node_prefix_kernel(const double* __restrict__ coef, const int* __restrict__ parent,
                                   long long n_moments, double* __restrict__ prefix) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_moments;
       i += (long long)gridDim.x * blockDim.x) {
    double p[kCoef];
#pragma unroll
    for (int k = 0; k < kCoef; ++k) p[k] = 0.0;
    long long node = i;
    for (int depth = 0; node >= 0 && node < n_moments && depth < 256; ++depth) {
#pragma unroll
      for (int k = 0; k < kCoef; ++k) p[k] += coef[kCoef * node + k];
      node = parent[node];
    }
#pragma unroll
    for (int k = 0; k < kCoef; ++k) prefix[kCoef * i + k] = p[k];
  }
}

/* Moment chain to the particles from their bucket's prefix coefficients. */
__global__ void moment_grad_kernel(const double* __restrict__ prefix, const int* __restrict__ leaf,
                                   const double* __restrict__ parts, long long n,
                                   long long n_moments, double* __restrict__ grad) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int node = leaf[k];
    if (node < 0 || node >= n_moments) continue;
    const double* c = prefix + kCoef * node;
    const double mk = parts[5 * k], x = parts[5 * k + 2], y = parts[5 * k + 3], z = parts[5 * k + 4];
    const double Gx = c[3] * x + c[4] * y + c[5] * z;
    const double Gy = c[4] * x + c[6] * y + c[7] * z;
    const double Gz = c[5] * x + c[7] * y + c[8] * z;
    grad[4 * k] += mk * (c[0] + Gx);
    grad[4 * k + 1] += mk * (c[1] + Gy);
    grad[4 * k + 2] += mk * (c[2] + Gz);
    grad[4 * k + 3] += c[9] + c[0] * x + c[1] * y + c[2] * z + 0.5 * (Gx * x + Gy * y + Gz * z);
  }
}

int grid_of(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  long long cap = (long long)sm_count() * 16;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace
}  // namespace chg

using namespace chg;

extern "C" int changa_gravity_vjp_mixed(const double* moments, long long n_moments,
                                        const double* parts, long long n_parts,
                                        const ChangaListRequest* cells,
                                        const ChangaListRequest* plist, double fperiod,
                                        const int* parent, const int* leaf, const double* lam,
                                        double* grad, cudaStream_t s) {
  if (!moments || !parts || !lam || !grad || !parent || !leaf || n_moments < 0 || n_parts < 0)
    return record_error(CHANGA_E_INVALID_ARG, "vjp: arrays", __FILE__, __LINE__);
  const ChangaListRequest* reqs[2] = {cells, plist};
  for (const ChangaListRequest* r : reqs)
    if (r && (r->n_buckets < 0 || r->n_entries < 0 ||
              (r->n_buckets > 0 && (!r->markers || !r->starts || !r->sizes || !r->list))))
      return record_error(CHANGA_E_INVALID_ARG, "vjp: request", __FILE__, __LINE__);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t cb = al((size_t)n_moments * kCellPackF4 * sizeof(float4));
  const size_t pb = al((size_t)n_parts * kPartPackF4 * sizeof(float4));
  const size_t lb = al((size_t)n_parts * sizeof(float4));
  const size_t fb = al((size_t)n_moments * kCoef * sizeof(double)) * 2;  // coef + prefix
  const size_t ab = al((size_t)kReplicas * n_moments * kCellAcc * sizeof(float));
  const size_t qb = al((size_t)kReplicas * n_parts * kPartAcc * sizeof(float));
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, cb + pb + lb + fb + ab + qb + 512, s));
  float4* pc = (float4*)block;
  float4* pp = (float4*)(block + cb);
  float4* pl = (float4*)(block + cb + pb);
  double* coef = (double*)(block + cb + pb + lb);
  double* prefix = coef + (size_t)n_moments * kCoef;
  float* acc_cell = (float*)(block + cb + pb + lb + fb);
  float* acc_part = (float*)(block + cb + pb + lb + fb + ab);
  unsigned int* q = (unsigned int*)(block + cb + pb + lb + fb + ab + qb);
  CHG_CUDA(cudaMemsetAsync(acc_cell, 0, ab + qb + 512, s));
  CHG_CUDA(launch_pack_cells(moments, n_moments, pc, s));
  CHG_CUDA(launch_pack_parts(parts, n_parts, pp, s));
  {
    TimingScope ts(kKidPack, s);
    pack_lambda_kernel<<<grid_of(n_parts, 256), 256, 0, s>>>(lam, n_parts, pl);
  }
  count_launch();
  for (int k = 0; k < 2; ++k) {
    const ChangaListRequest* r = reqs[k];
    if (!r || r->n_buckets == 0 || n_parts == 0 || (k == 0 ? n_moments : n_parts) == 0) continue;
    VjpArgs va;
    va.src = k == 0 ? pc : pp;
    va.n_src = k == 0 ? n_moments : n_parts;
    va.tgt = pp;
    va.lam = pl;
    va.n_tgt = n_parts;
    va.list = (const int2*)r->list;
    va.n_entries = r->n_entries;
    va.markers = r->markers;
    va.starts = r->starts;
    va.sizes = r->sizes;
    va.n_buckets = r->n_buckets;
    va.fperiod = (float)fperiod;
    va.grad_tgt = grad;
    va.acc = k == 0 ? acc_cell : acc_part;
    va.queue = q + 64 * k;
    const int grid = grid_of(((long long)r->n_buckets + kWarps - 1) / kWarps, 1);
    {
      TimingScope ts(k == 0 ? kKidVjpCell : kKidVjpPart, s);
      if (k == 0) vjp_kernel<true><<<grid, kThreads, 0, s>>>(va);
      else vjp_kernel<false><<<grid, kThreads, 0, s>>>(va);
    }
    count_launch();
    CHG_CUDA(cudaGetLastError());
  }
  {
    TimingScope ts(kKidMoments, s);
    finish_parts_kernel<<<grid_of(4 * n_parts, 256), 256, 0, s>>>(acc_part, n_parts, grad);
    if (n_moments > 0) {
      node_coef_kernel<<<grid_of(n_moments, 64), 64, 0, s>>>(moments, acc_cell, n_moments, coef);
      node_prefix_kernel<<<grid_of(n_moments, 64), 64, 0, s>>>(coef, parent, n_moments, prefix);
      moment_grad_kernel<<<grid_of(n_parts, 256), 256, 0, s>>>(prefix, leaf, parts, n_parts,
                                                              n_moments, grad);
    }
  }
  count_launch(n_moments > 0 ? 4 : 1);
  CHG_CUDA(cudaGetLastError());
  CHG_CUDA(cudaFreeAsync(block, s));
  return 0;
}
