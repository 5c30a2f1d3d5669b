/*
 * FP32 evaluation pieces shared by the interaction-list kernels
 * (grav_lists.cu) and the fused walk-and-evaluate kernel (walk.cu): the
 * spline-softening branches, the raw-record gather and finishing step of
 * the list entries, and the paired (.f32x2) cell and particle bodies on
 * staged source pairs.
 */
#pragma once

#include "chg_internal.h"
#include "f32x2.cuh"

namespace chg {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float two_over(float t) { return __fdividef(2.0f, t); }
__device__ __forceinline__ double two_over(double t) { return 2.0 / t; }

/* SPLINEQ inside the softening radius (gravity.h:27-59): both branches. */
template <typename T>
__device__ __forceinline__ void splineq_near(T dir, T rsq, T twoh, T& a, T& b, T& c, T& d) {
  const T dih = two_over(twoh);
  const T u = dih * (rsq * dir);
  const T dih2 = dih * dih, dih3 = dih2 * dih, dih5 = dih3 * dih2;
  const T u2 = u * u;
  if (u < T(1)) {
    a = dih * (T(7.0 / 5.0) - T(2.0 / 3.0) * u2 + T(3.0 / 10.0) * u2 * u2 -
               T(1.0 / 10.0) * u2 * u2 * u);
    b = dih3 * (T(4.0 / 3.0) - T(6.0 / 5.0) * u2 + T(0.5) * u2 * u);
    c = dih5 * (T(12.0 / 5.0) - T(1.5) * u);
    d = T(1.5) * dih5 * dih * dir;
  } else {
    const T dir2 = dir * dir, dir3 = dir2 * dir;
    a = T(-1.0 / 15.0) * dir +
        dih * (T(8.0 / 5.0) - T(4.0 / 3.0) * u2 + u2 * u - T(3.0 / 10.0) * u2 * u2 +
               T(1.0 / 30.0) * u2 * u2 * u);
    b = T(-1.0 / 15.0) * dir3 +
        dih3 * (T(8.0 / 3.0) - T(3) * u + T(6.0 / 5.0) * u2 - T(1.0 / 6.0) * u2 * u);
    c = T(-1.0 / 5.0) * dir3 * dir2 + T(3) * dih2 * dih2 * dir + dih5 * (T(-12.0 / 5.0) + T(0.5) * u);
    d = -dir3 * dir3 * dir + T(3) * dih2 * dih2 * dir3 - T(0.5) * dih5 * dih * dir;
  }
}

/* SPLINE inside the softening radius (gravity.h:152-176). */
template <typename T>
__device__ __forceinline__ void spline_near(T r, T dir, T twoh, T& a, T& b) {
  const T dih = two_over(twoh);
  const T u = r * dih;
  const T u2 = u * u, dih3 = dih * dih * dih;
  if (u < T(1)) {
    a = dih * (T(7.0 / 5.0) - T(2.0 / 3.0) * u2 + T(3.0 / 10.0) * u2 * u2 -
               T(1.0 / 10.0) * u2 * u2 * u);
    b = dih3 * (T(4.0 / 3.0) - T(6.0 / 5.0) * u2 + T(0.5) * u2 * u);
  } else {
    a = T(-1.0 / 15.0) * dir +
        dih * (T(8.0 / 5.0) - T(4.0 / 3.0) * u2 + u2 * u - T(3.0 / 10.0) * u2 * u2 +
               T(1.0 / 30.0) * u2 * u2 * u);
    b = T(-1.0 / 15.0) * dir * dir * dir +
        dih3 * (T(8.0 / 3.0) - T(3) * u + T(6.0 / 5.0) * u2 - T(1.0 / 6.0) * u2 * u);
  }
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float x) {
  const float y = x - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

/* The near-field spline branches of the FP32 forms, out of line: they are
 * rare, and inlining them at every unrolled call site would multiply the
 * hot loop's code size past the instruction cache. */
__device__ __noinline__ float4 splineq_near_f(float dir, float rsq, float twoh) {
  float4 k;
  splineq_near(dir, rsq, twoh, k.x, k.y, k.z, k.w);
  return k;
}
__device__ __noinline__ float2 spline_near_f(float r, float dir, float twoh) {
  float2 k;
  spline_near(r, dir, twoh, k.x, k.y);
  return k;
}

/* Raw words of one list entry as a lane holds them between the gather
 * and the finishing step. */
template <int FORM, bool CELL>
struct RawRec {
  float4 w0, w1, w2, w3;
  float f4;
  int code;
};

/* List entry e (a massless entry at replica (0, 0, 0) past the end), and the
 * raw record of a loaded entry: gather_raw in two steps, so the entries can
 * be loaded a block ahead of their records. */
__device__ __forceinline__ int2 load_entry(const ListArgs& a, int e, int e_end) {
  return e < e_end ? __ldg(a.list + e) : make_int2(0, 0x49 << 22);
}

template <int FORM, bool CELL>
__device__ __forceinline__ void gather_raw_entry(const ListArgs& a, int2 ent,
                                                 RawRec<FORM, CELL>& r) {
  long long idx = ent.x;
  if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;  // memory safety
  r.code = (ent.y >> 22) & 0x1ff;
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

/* Finished record words: cells {x, y, z, M} {xx, xy, xz, yy} {yz, zz, tr,
 * soft}; particles {x, y, z, m} and the softening.  Entries past the list
 * end become massless records far away (they add exact zeros). */
template <int FORM, bool CELL>
__device__ __forceinline__ float finish_raw(const ListArgs& a, const RawRec<FORM, CELL>& r,
                                            bool valid, float3 chi, float3 clo, float4* dst) {
  const float fp = a.fperiod_f;
  const float ox = (float)((r.code & 7) - 3) * fp, oy = (float)(((r.code >> 3) & 7) - 3) * fp,
              oz = (float)(((r.code >> 6) & 7) - 3) * fp;
  float4 p0;
  float soft;
  if constexpr (FORM == kF32) {
    if constexpr (CELL) {
      // w0 {radius, soft, M, cm.x}  w1 {cm.y, cm.z, xx, xy}  w2 {xz, yy, yz, zz}
      p0 = make_float4(ox + r.w0.w, oy + r.w1.x, oz + r.w1.y, r.w0.z);
      soft = r.w0.y;
      dst[1] = make_float4(r.w1.z, r.w1.w, r.w2.x, r.w2.y);
      dst[2] = make_float4(r.w2.z, r.w2.w, 0.5f * (r.w1.z + r.w2.y + r.w2.w), soft);
    } else {
      p0 = make_float4(ox + r.w0.x, oy + r.w0.y, oz + r.w0.z, r.w0.w);
      soft = r.f4;
    }
  } else {
    p0 = make_float4(((r.w0.x - chi.x) + ox) + (r.w1.x - clo.x),
                     ((r.w0.y - chi.y) + oy) + (r.w1.y - clo.y),
                     ((r.w0.z - chi.z) + oz) + (r.w1.z - clo.z), r.w0.w);
    soft = r.w1.w;
    if constexpr (CELL) {
      // w2 {xx, xy, xz, yy}  w3 {yz, zz, tr, 0}
      dst[1] = r.w2;
      dst[2] = make_float4(r.w3.x, r.w3.y, r.w3.z, soft);
    }
  }
  if (!valid) {
    p0 = make_float4(1e30f, 1e30f, 1e30f, 0.f);
    soft = 0.f;
    if constexpr (CELL) {
      dst[1] = make_float4(0.f, 0.f, 0.f, 0.f);
      dst[2] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  dst[0] = p0;
  return soft;
}

/* Hardware reciprocal square root, flushing subnormal inputs (the
 * squared separations here are zero or far above the subnormal range):
 * one MUFU instruction. */
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

/* f2, pk2/up2 and the packed add2/sub2/mul2/fma2: f32x2.cuh */

/* float index of field f of pair half h inside a pair block */
__device__ __forceinline__ int pair_slot(int f, int h) { return 4 * (f >> 1) + 2 * (f & 1) + h; }

/* max of three (one instruction on sm_100 and later; NaN operands are
 * ignored as fmaxf ignores them) */
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

/* One lane's cell record into its half h of a staged pair (pc_pair's
 * layout): {x0 x1 y0 y1} {z0 z1 -M0 -M1} {Sxx Sxy} {Sxz Syy} {Syz Szz}
 * {tr tr3} with S = 3Q and tr3 = 3 tr (each two-field word as pair halves);
 * the softening goes to a side array. */
__device__ __forceinline__ void stage_cell_half(float* pb, int h, float4 p, float4 q1, float4 q2) {
  // p {x, y, z, M}  q1 {xx, xy, xz, yy}  q2 {yz, zz, tr, soft}
  pb[pair_slot(0, h)] = p.x;
  pb[pair_slot(1, h)] = p.y;
  pb[pair_slot(2, h)] = p.z;
  pb[pair_slot(3, h)] = -p.w;
  pb[pair_slot(4, h)] = 3.f * q1.x;
  pb[pair_slot(5, h)] = 3.f * q1.y;
  pb[pair_slot(6, h)] = 3.f * q1.z;
  pb[pair_slot(7, h)] = 3.f * q1.w;
  pb[pair_slot(8, h)] = 3.f * q2.x;
  pb[pair_slot(9, h)] = 3.f * q2.y;
  pb[pair_slot(10, h)] = q2.z;
  pb[pair_slot(11, h)] = 3.f * q2.z;
}

/* One staged pair of quadrupole cells on one target, FP32 (gravity.h:
 * 436-472, r = target - cell), for the paired kernels, on records staged by
 * stage_cell_half.  With s = 1/r^2, c3 = c/3 and u = d/15 (far field:
 * c3 = b s, u = c3 s), q = S r = 3 Q r and w = r.q = 6 qir, the terms of
 * the reference read
 *   c Q r = c3 q,  2 c qir = c3 w,  d qir = 2.5 u w,  c tr = c3 tr3,
 * so no constant factor is applied per pair.  Accumulators: pa2 gets
 * -M a + b tr and pw2 gets c3 w (the potential is pa2 - pw2 / 2), the
 * acceleration adds c Q r - qir3 r (qir3 = b M + d qir - c tr), and idtn
 * keeps the minimum of -(m_t b + M b) (dtGrav's maximum, negated).  sft
 * holds the pair's two softenings.  NEAR = false leaves out the softening
 * test (for blocks whose cells all lie beyond the softening bound). */
/* A staged cell pair's six words, read from shared memory once and used
 * for every target of a lane (pc_pair_w). */
struct CellPair {
  float4 w0, w1, w2, w3, w4, w5;
};
__device__ __forceinline__ CellPair load_cell_pair(const float4* __restrict__ w) {
  return CellPair{w[0], w[1], w[2], w[3], w[4], w[5]};
}

template <bool NEAR = true>
__device__ __forceinline__ void pc_pair_w(const CellPair& cp, const float* __restrict__ sft,
                                          f2 tx2, f2 ty2, f2 tz2, f2 tmn2, float tsoft,
                                          float near2, f2& pa2, f2& pw2, f2& ax2, f2& ay2, f2& az2,
                                          float& idtn) {
  const float4 w0 = cp.w0, w1 = cp.w1;
  const f2 px = pk2(w0.x, w0.y), py = pk2(w0.z, w0.w), pz = pk2(w1.x, w1.y), mn = pk2(w1.z, w1.w);
  const float4 w2 = cp.w2, w3 = cp.w3, w4 = cp.w4, w5 = cp.w5;
  const f2 sxx = pk2(w2.x, w2.y), sxy = pk2(w2.z, w2.w), sxz = pk2(w3.x, w3.y),
           syy = pk2(w3.z, w3.w), syz = pk2(w4.x, w4.y), szz = pk2(w4.z, w4.w),
           tr = pk2(w5.x, w5.y), tr3 = pk2(w5.z, w5.w);
  const f2 rx = sub2(tx2, px), ry = sub2(ty2, py), rz = sub2(tz2, pz);
  const f2 rsq = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
  float q0, q1;
  up2(rsq, q0, q1);
  f2 av = pk2(rsqrt_ftz(q0), rsqrt_ftz(q1));
  const f2 s2 = mul2(av, av);
  f2 bv = mul2(s2, av);
  f2 cv = mul2(bv, s2);  // c / 3
  f2 uv = mul2(cv, s2);  // d / 15
  if (NEAR && fminf(q0, q1) <= near2) {
    float a_[2], b_[2], c_[2], u_[2], r_[2] = {q0, q1};
    up2(av, a_[0], a_[1]);
    up2(bv, b_[0], b_[1]);
    up2(cv, c_[0], c_[1]);
    up2(uv, u_[0], u_[1]);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (r_[h] > near2) continue;
      const float twoh = sft[h] + tsoft;
      if (r_[h] == 0.f) {
        a_[h] = b_[h] = c_[h] = u_[h] = 0.f;
      } else if (r_[h] < twoh * twoh) {
        const float4 kk = splineq_near_f(a_[h], r_[h], twoh);
        a_[h] = kk.x;
        b_[h] = kk.y;
        c_[h] = kk.z * (1.f / 3.f);
        u_[h] = kk.w * (1.f / 15.f);
      }
    }
    av = pk2(a_[0], a_[1]);
    bv = pk2(b_[0], b_[1]);
    cv = pk2(c_[0], c_[1]);
    uv = pk2(u_[0], u_[1]);
  }
  const f2 qx = fma2(sxx, rx, fma2(sxy, ry, mul2(sxz, rz)));
  const f2 qy = fma2(sxy, rx, fma2(syy, ry, mul2(syz, rz)));
  const f2 qz = fma2(sxz, rx, fma2(syz, ry, mul2(szz, rz)));
  const f2 wq = fma2(qx, rx, fma2(qy, ry, mul2(qz, rz)));
  const f2 bmn = mul2(bv, mn);  // -b M
  /* -qir3 = -b M - 2.5 u w + c3 tr3 */
  const f2 nq3 = fma2(uv, mul2(wq, pk2(-2.5f, -2.5f)), fma2(cv, tr3, bmn));
  pa2 = fma2(bv, tr, fma2(mn, av, pa2));
  pw2 = fma2(cv, wq, pw2);
  ax2 = fma2(cv, qx, fma2(nq3, rx, ax2));
  ay2 = fma2(cv, qy, fma2(nq3, ry, ay2));
  az2 = fma2(cv, qz, fma2(nq3, rz, az2));
  float d0, d1;
  up2(fma2(tmn2, bv, bmn), d0, d1);
  idtn = fmin3(idtn, d0, d1);
}

template <bool NEAR = true>
__device__ __forceinline__ void pc_pair(const float4* __restrict__ w, const float* __restrict__ sft,
                                        f2 tx2, f2 ty2, f2 tz2, f2 tmn2, float tsoft, float near2,
                                        f2& pa2, f2& pw2, f2& ax2, f2& ay2, f2& az2, float& idtn) {
  pc_pair_w<NEAR>(load_cell_pair(w), sft, tx2, ty2, tz2, tmn2, tsoft, near2, pa2, pw2, ax2, ay2,
                  az2, idtn);
}

/* One staged particle pair (two sources of one 32-entry block) on this
 * lane's target, without branches (gravity.h:276-301, r = source - target,
 * FP32 on bucket-relative coordinates).  Accumulators: pot2 gets m a (the
 * potential's opposite sign, negated at the fold), the acceleration adds
 * r m b, idt2 keeps dtGrav's running maximum (m_t + m) b.  With MARK,
 * halves within the softening bound near2 get a = b = 0 (selects) and their
 * bit (2p + half) in nmask, for pp_soft_pass after the block. */
template <bool MARK>
__device__ __forceinline__ void pp_pair(const float4* __restrict__ w, int p, f2 tx2, f2 ty2,
                                        f2 tz2, f2 tm2, float near2, f2& pot2, f2& ax2, f2& ay2,
                                        f2& az2, float& idt2, unsigned& nmask) {
  const float4 w0 = w[0], w1 = w[1];
  const f2 pm = pk2(w1.z, w1.w);
  const f2 rx = sub2(pk2(w0.x, w0.y), tx2), ry = sub2(pk2(w0.z, w0.w), ty2),
           rz = sub2(pk2(w1.x, w1.y), tz2);
  const f2 rsq = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
  float q0, q1;
  up2(rsq, q0, q1);
  float a0 = rsqrt_ftz(q0), a1 = rsqrt_ftz(q1);
  if constexpr (MARK) {
    const bool n0 = q0 <= near2, n1 = q1 <= near2;
    nmask |= ((n0 ? 1u : 0u) | (n1 ? 2u : 0u)) << (2 * p);
    a0 = n0 ? 0.f : a0;
    a1 = n1 ? 0.f : a1;
  }
  const f2 av = pk2(a0, a1);
  const f2 bv = mul2(mul2(av, av), av);
  const f2 bm = mul2(bv, pm);
  pot2 = fma2(pm, av, pot2);
  ax2 = fma2(rx, bm, ax2);
  ay2 = fma2(ry, bm, ay2);
  az2 = fma2(rz, bm, az2);
  float d0, d1;
  up2(fma2(tm2, bv, bm), d0, d1);
  idt2 = fmax3(idt2, d0, d1);
}

/* The sources marked by pp_pair in nmask, each lane its own, all lanes at
 * once: gravity.h:276-301 with the spline inside 2h, zero at r = 0.  st:
 * the staged pairs (two float4 per pair), ss: the block's 32 softenings. */
__device__ __forceinline__ void pp_soft_pass(const float4* __restrict__ st,
                                             const float* __restrict__ ss, unsigned nmask,
                                             float tx, float ty, float tz, float tsoft,
                                             float tmass, float& ex, float& ey, float& ez,
                                             float& ep, float& idt2) {
  while (nmask) {
    const int jb = __ffs(nmask) - 1;
    nmask &= nmask - 1u;
    const float* pb = reinterpret_cast<const float*>(st + (jb >> 1) * 2);
    const int h = jb & 1;
    const float dx = pb[pair_slot(0, h)] - tx, dy = pb[pair_slot(1, h)] - ty,
                dz = pb[pair_slot(2, h)] - tz, sm = pb[pair_slot(3, h)];
    const float q = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float av = 0.f, bv = 0.f;
    if (q != 0.f) {
      av = rsqrt_ftz(q);
      bv = (av * av) * av;
      const float twoh = ss[jb] + tsoft;
      const float r1 = q * av;
      if (r1 < twoh) spline_near(r1, av, twoh, av, bv);
    }
    const float bm = bv * sm;
    ep = fmaf(sm, av, ep);
    ex = fmaf(dx, bm, ex);
    ey = fmaf(dy, bm, ey);
    ez = fmaf(dz, bm, ez);
    idt2 = fmaxf(idt2, fmaf(tmass, bv, bm));
  }
}

}  // namespace
}  // namespace chg
