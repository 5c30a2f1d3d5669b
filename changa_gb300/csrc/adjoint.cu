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
 * Kernel design mirrors the forward source-parallel kernel: lanes own list
 * entries, targets (position, mass, lambda) are broadcast from shared memory
 * in chunks of 8, target gradients are reduced with the butterfly
 * reduce-scatter, and each lane adds its source's gradient (summed over the
 * chunk's targets) with one set of FP64 atomics.  Cell softening is treated
 * as a constant (its mass derivative only matters inside the spline, where
 * cells are almost never evaluated).
 */
#include "chg_internal.h"

namespace chg {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kTC = 8;
constexpr int kTB = 32;

/* a, b, c, d, e of the quadrupole spline kernel inside the softening
 * length (gravity.h:27-59 for a..d; e = -(1/r) dd/dr derived from them:
 * u < 1: e = 3/2 dih^6 / r^3; 1 <= u < 2: e = -7/r^9 + 9 dih^4 / r^5 -
 * dih^6 / (2 r^3); both meet 105/r^9 at u = 2). */
struct Spl5 {
  float a, b, c, d, e;
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
    k.a = dih * (7.0f / 5.0f - 2.0f / 3.0f * u2 + 3.0f / 10.0f * u2 * u2 - 1.0f / 10.0f * u2 * u2 * u);
    k.b = dih3 * (4.0f / 3.0f - 6.0f / 5.0f * u2 + 0.5f * u2 * u);
    k.c = dih5 * (12.0f / 5.0f - 1.5f * u);
    k.d = 1.5f * dih6 * dir;
    k.e = 1.5f * dih6 * dir3;
  } else {
    const float dir5 = dir3 * dir2, dir7 = dir5 * dir2, dir9 = dir7 * dir2;
    k.a = -1.0f / 15.0f * dir +
          dih * (8.0f / 5.0f - 4.0f / 3.0f * u2 + u2 * u - 3.0f / 10.0f * u2 * u2 +
                 1.0f / 30.0f * u2 * u2 * u);
    k.b = -1.0f / 15.0f * dir3 +
          dih3 * (8.0f / 3.0f - 3.0f * u + 6.0f / 5.0f * u2 - 1.0f / 6.0f * u2 * u);
    k.c = -1.0f / 5.0f * dir5 + 3.0f * dih4 * dir + dih5 * (-12.0f / 5.0f + 0.5f * u);
    k.d = -dir7 + 3.0f * dih4 * dir3 - 0.5f * dih6 * dir;
    k.e = -7.0f * dir9 + 9.0f * dih4 * dir5 - 0.5f * dih6 * dir3;
  }
  return k;
}

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
  double* grad_tgt;  // n_tgt x 4 {dx, dy, dz, dm}
  double* grad_src;  // particles: n_src x 4; cells: n_src x 10 {X(3), M, xx xy xz yy yz zz}
  unsigned int* queue;
};

template <bool CELL>
__global__ void __launch_bounds__(kThreads, 2) vjp_kernel(const VjpArgs a) {
  __shared__ __align__(16) float4 tpos[kWarps][kTB];
  __shared__ __align__(16) float4 tlam[kWarps][kTB];
  __shared__ float tsoft[kWarps][kTB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

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
      const int nch = (nt + kTC - 1) / kTC;
      for (int c = 0; c < nch; ++c) {
        const int t0 = c * kTC;
        const int ntc = min(kTC, nt - t0);
        float tot = 0.f;
        for (int e0 = e_begin; e0 < e_end; e0 += 32) {
          const int e = e0 + lane;
          const bool valid = e < e_end;
          float v[32];
#pragma unroll
          for (int k = 0; k < 32; ++k) v[k] = 0.f;
          /* this lane's source */
          long long idx = 0;
          int code = 0;
          if (valid) {
            const int2 ent = __ldg(a.list + e);
            idx = ent.x;
            if ((unsigned long long)idx >= (unsigned long long)a.n_src) idx = 0;
            code = (ent.y >> 22) & 0x1ff;
          }
          const float ox = (float)((code & 7) - 3) * a.fperiod,
                      oy = (float)(((code >> 3) & 7) - 3) * a.fperiod,
                      oz = (float)(((code >> 6) & 7) - 3) * a.fperiod;
          const float4* sp = a.src + (CELL ? 4 : 2) * idx;
          const float4 h = __ldg(sp), l = __ldg(sp + 1);
          const float sx = ((h.x - chi.x) + ox) + (l.x - clo.x);
          const float sy = ((h.y - chi.y) + oy) + (l.y - clo.y);
          const float sz = ((h.z - chi.z) + oz) + (l.z - clo.z);
          const float sm = h.w, ss = l.w;
          float xx = 0.f, xy = 0.f, xz = 0.f, yy = 0.f, yz = 0.f, zz = 0.f, tr = 0.f;
          if constexpr (CELL) {
            const float4 q0 = __ldg(sp + 2), q1 = __ldg(sp + 3);
            xx = q0.x;
            xy = q0.y;
            xz = q0.z;
            yy = q0.w;
            yz = q1.x;
            zz = q1.y;
            tr = q1.z;
          }
          /* source gradient accumulated over this chunk's targets */
          float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
          float q_xx = 0.f, q_xy = 0.f, q_xz = 0.f, q_yy = 0.f, q_yz = 0.f, q_zz = 0.f;
          if (valid) {
#pragma unroll
            for (int tt = 0; tt < kTC; ++tt) {
              if (tt < ntc) {
                const float4 tp = tpos[warp][t0 + tt];
                const float4 la = tlam[warp][t0 + tt];
                if constexpr (CELL) {
                  const float rx = tp.x - sx, ry = tp.y - sy, rz = tp.z - sz;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  if (rsq > 0.f) {
                    const float dir = rsqrtf(rsq);
                    const float dir2 = dir * dir;
                    float bv = dir2 * dir, cv = bv * (3.f * dir2), dv = cv * (5.f * dir2),
                          ev = dv * (7.f * dir2);
                    const float twoh = ss + tsoft[warp][t0 + tt];
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
                    q_xx += hr * rx * rx + ht + cv * la.x * rx;
                    q_yy += hr * ry * ry + ht + cv * la.y * ry;
                    q_zz += hr * rz * rz + ht + cv * la.z * rz;
                    q_xy += 2.f * hr * rx * ry + cv * (la.x * ry + la.y * rx);
                    q_xz += 2.f * hr * rx * rz + cv * (la.x * rz + la.z * rx);
                    q_yz += 2.f * hr * ry * rz + cv * (la.y * rz + la.z * ry);
                  }
                } else {
                  const float rx = sx - tp.x, ry = sy - tp.y, rz = sz - tp.z;
                  const float rsq = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                  if (rsq > 0.f) {
                    const float dir = rsqrtf(rsq);
                    const float dir2 = dir * dir;
                    float bv = dir2 * dir, cv = bv * (3.f * dir2);
                    const float twoh = ss + tsoft[warp][t0 + tt];
                    if (rsq < twoh * twoh) {
                      const Spl5 k = spline5_near(dir, rsq, twoh);
                      bv = k.b;
                      cv = k.c;
                    }
                    const float rl = fmaf(rx, la.x, fmaf(ry, la.y, rz * la.z));
                    const float gx = sm * (bv * la.x - cv * rl * rx);
                    const float gy = sm * (bv * la.y - cv * rl * ry);
                    const float gz = sm * (bv * la.z - cv * rl * rz);
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
            double* gs = a.grad_src + (CELL ? 10 : 4) * idx;
            atomicAdd(gs + 0, (double)g0);
            atomicAdd(gs + 1, (double)g1);
            atomicAdd(gs + 2, (double)g2);
            atomicAdd(gs + 3, (double)g3);
            if constexpr (CELL) {
              atomicAdd(gs + 4, (double)q_xx);
              atomicAdd(gs + 5, (double)q_xy);
              atomicAdd(gs + 6, (double)q_xz);
              atomicAdd(gs + 7, (double)q_yy);
              atomicAdd(gs + 8, (double)q_yz);
              atomicAdd(gs + 9, (double)q_zz);
            }
          }
          tot += reduce_scatter32(v, lane);
        }
        const int t = lane >> 2, q = lane & 3;
        if (t < ntc && q < 3) a.grad_tgt[4 * (tbase + tb0 + t0 + t) + q] += (double)tot;
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

/* Cell gradients to particles: every particle walks its ancestors (FP64). */
__global__ void moment_grad_kernel(const double* __restrict__ moments,
                                   const double* __restrict__ gcell, const int* __restrict__ parent,
                                   const int* __restrict__ leaf, const double* __restrict__ parts,
                                   long long n, long long n_moments, double* __restrict__ grad) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const double mk = parts[5 * k], x = parts[5 * k + 2], y = parts[5 * k + 3], z = parts[5 * k + 4];
    double gx = 0, gy = 0, gz = 0, gm = 0;
    int node = leaf[k];
    for (int depth = 0; node >= 0 && node < n_moments && depth < 256; ++depth) {
      const double* gc = gcell + 10 * node;
      const double* mo = moments + 12 * node;
      const double M = mo[2];
      if (M > 0.0) {
        const double dx = x - mo[3], dy = y - mo[4], dz = z - mo[5];
        const double gxx = gc[4], gxy = gc[5], gxz = gc[6], gyy = gc[7], gyz = gc[8], gzz = gc[9];
        /* G d with G = [[2gxx gxy gxz] [gxy 2gyy gyz] [gxz gyz 2gzz]] */
        const double Gx = 2 * gxx * dx + gxy * dy + gxz * dz;
        const double Gy = gxy * dx + 2 * gyy * dy + gyz * dz;
        const double Gz = gxz * dx + gyz * dy + 2 * gzz * dz;
        gx += mk * (gc[0] / M + Gx);
        gy += mk * (gc[1] / M + Gy);
        gz += mk * (gc[2] / M + Gz);
        gm += gc[3] + (gc[0] * dx + gc[1] * dy + gc[2] * dz) / M + 0.5 * (Gx * dx + Gy * dy + Gz * dz);
      }
      node = parent[node];
    }
    grad[4 * k] += gx;
    grad[4 * k + 1] += gy;
    grad[4 * k + 2] += gz;
    grad[4 * k + 3] += gm;
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
  const size_t gb = al((size_t)n_moments * 10 * sizeof(double));
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, cb + pb + lb + gb + 512, s));
  float4* pc = (float4*)block;
  float4* pp = (float4*)(block + cb);
  float4* pl = (float4*)(block + cb + pb);
  double* gcell = (double*)(block + cb + pb + lb);
  unsigned int* q = (unsigned int*)(block + cb + pb + lb + gb);
  CHG_CUDA(cudaMemsetAsync(gcell, 0, gb + 512, s));
  CHG_CUDA(launch_pack_cells(moments, n_moments, pc, s));
  CHG_CUDA(launch_pack_parts(parts, n_parts, pp, s));
  pack_lambda_kernel<<<grid_of(n_parts, 256), 256, 0, s>>>(lam, n_parts, pl);
  count_launch();
  for (int k = 0; k < 2; ++k) {
    const ChangaListRequest* r = reqs[k];
    if (!r || r->n_buckets == 0) continue;
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
    va.grad_src = k == 0 ? gcell : grad;
    va.queue = q + 64 * k;
    const int grid = grid_of(((long long)r->n_buckets + kWarps - 1) / kWarps, 1);
    if (k == 0) vjp_kernel<true><<<grid, kThreads, 0, s>>>(va);
    else vjp_kernel<false><<<grid, kThreads, 0, s>>>(va);
    count_launch();
    CHG_CUDA(cudaGetLastError());
  }
  moment_grad_kernel<<<grid_of(n_parts, 256), 256, 0, s>>>(moments, gcell, parent, leaf, parts,
                                                          n_parts, n_moments, grad);
  count_launch();
  CHG_CUDA(cudaGetLastError());
  CHG_CUDA(cudaFreeAsync(block, s));
  return 0;
}
