// cylinder.cuh — device helpers of the point-level cylinder fit shared by
// models.cu (hypotheses, the learned proposals' pass) and cylqueue.cu (the
// persistent work-queue kernel): the prior-axis frame of a tree, the
// projection of its points on that frame, where its points live, the
// Philox three-point circle hypothesis and the LS model's normal frame.
#pragma once
#include "common.cuh"
#include "internal.h"

namespace sg {

struct CylFrame {
  float ox, oy, oz;
  float ax, ay, az;
  float e1x, e1y, e1z, e2x, e2y, e2z;
};

__device__ __forceinline__ CylFrame make_frame(const Dev& d, const CylD& c) {
  CylFrame f;
  const float* vx = d.lm_vxyz + 3 * (size_t)d.lm_vbeg[c.landmark];
  f.ox = vx[3]; f.oy = vx[4]; f.oz = vx[5];
  float ax = (float)c.ray[0], ay = (float)c.ray[1], az = (float)c.ray[2];
  if (az < 0) { ax = -ax; ay = -ay; az = -az; }
  float tx = 1.0f, ty = 0.0f, tz = 0.0f;
  if (!(fabsf(ax) < 0.9f)) { tx = 0.0f; ty = 1.0f; }
  float e1x = fsub(fmul(ay, tz), fmul(az, ty)), e1y = fsub(fmul(az, tx), fmul(ax, tz)),
        e1z = fsub(fmul(ax, ty), fmul(ay, tx));
  const float e1n = fsqrt(fadd(fadd(fmul(e1x, e1x), fmul(e1y, e1y)), fmul(e1z, e1z)));
  e1x = fdiv(e1x, e1n); e1y = fdiv(e1y, e1n); e1z = fdiv(e1z, e1n);
  f.e2x = fsub(fmul(ay, e1z), fmul(az, e1y));
  f.e2y = fsub(fmul(az, e1x), fmul(ax, e1z));
  f.e2z = fsub(fmul(ax, e1y), fmul(ay, e1x));
  f.ax = ax; f.ay = ay; f.az = az;
  f.e1x = e1x; f.e1y = e1y; f.e1z = e1z;
  return f;
}

__device__ __forceinline__ float2 project_uv(const CylFrame& f, float4 q) {
  const float dx = fsub(q.x, f.ox), dy = fsub(q.y, f.oy), dz = fsub(q.z, f.oz);
  const float u = fadd(fadd(fmul(dx, f.e1x), fmul(dy, f.e1y)), fmul(dz, f.e1z));
  const float v = fadd(fadd(fmul(dx, f.e2x), fmul(dy, f.e2y)), fmul(dz, f.e2z));
  return make_float2(u, v);
}

// The tree's points: its CC cluster, or its vertex points when no cluster;
// *uv = where their projections live in lm_uv.
__device__ __forceinline__ void tree_points(const Dev& d, int l, const float4** pts, int* n,
                                            const float2** uv) {
  const int c0 = d.lm_cbeg[l], c1 = d.lm_cbeg[l + 1];
  if (c1 > c0) {
    *pts = d.lm_cpts + c0;
    *n = c1 - c0;
    *uv = d.lm_uv + c0;
  } else {
    const int vb = d.lm_vbeg[l], ve = d.lm_vbeg[l + 1];
    *pts = d.lm_pts + d.lm_pbeg[vb];
    *n = d.lm_pbeg[ve] - d.lm_pbeg[vb];
    *uv = d.lm_uv + d.cap_cluster + d.lm_pbeg[vb];
  }
}

__device__ __forceinline__ bool fit_eligible(const CylD& c) {
  return c.stage == 1 && c.radius != -1.0;
}

struct Hyp {
  float cu, cv, r, lo2, hi2;
  bool ok;
};

template <typename UV>
__device__ __forceinline__ Hyp make_hyp(const KParams& kp, int h, int tree_id, int n, UV uv) {
  Hyp H{};
  H.ok = false;
  uint32_t u[4], id[3];
  philox(kp.seed, (uint32_t)h, (uint32_t)tree_id, 1u, 0u, u);
  draw_distinct(u, (uint32_t)n, 3, id);
  const float2 p0 = uv(id[0]), p1 = uv(id[1]), p2 = uv(id[2]);
  const float bx = fsub(p1.x, p0.x), by = fsub(p1.y, p0.y);
  const float cx = fsub(p2.x, p0.x), cy = fsub(p2.y, p0.y);
  const float t1 = fmul(bx, cy), t2 = fmul(by, cx);
  const float den = fmul(2.0f, fsub(t1, t2));
  if (den == 0.0f) return H;
  const float b2 = fadd(fmul(bx, bx), fmul(by, by)), c2 = fadd(fmul(cx, cx), fmul(cy, cy));
  const float ox = fdiv(fsub(fmul(cy, b2), fmul(by, c2)), den);
  const float oy = fdiv(fsub(fmul(bx, c2), fmul(cx, b2)), den);
  const float r = fsqrt(fadd(fmul(ox, ox), fmul(oy, oy)));
  if (!(r <= kp.max_hyp_r)) return H;
  H.cu = fadd(p0.x, ox);
  H.cv = fadd(p0.y, oy);
  H.r = r;
  const float lo = fsub(r, kp.tau), hi = fadd(r, kp.tau);
  H.lo2 = lo > 0.0f ? fmul(lo, lo) : -1.0f;
  H.hi2 = fmul(hi, hi);
  H.ok = true;
  return H;
}

// Normal frame of the LS model st (centre st[0..2], unit direction
// st[3..5], radius st[6]): b1 = dir x t / |dir x t| (t = x unless
// |dir_x| >= 0.9, then y), b2 = dir x b1, in double into st[8..13], and the
// float copies every thread uses into sf.
__device__ __forceinline__ void ls_frame(double* st, float* sf) {
  const d3 dd = mk3(st[3], st[4], st[5]);
  const d3 t = fabs(dd.x) < 0.9 ? mk3(1, 0, 0) : mk3(0, 1, 0);
  d3 b1 = cross3(dd, t);
  b1 = scl3(1.0 / norm3(b1), b1);
  const d3 b2 = cross3(dd, b1);
  st[8] = b1.x; st[9] = b1.y; st[10] = b1.z;
  st[11] = b2.x; st[12] = b2.y; st[13] = b2.z;
  for (int j = 0; j < 6; ++j) sf[j] = (float)st[j];
  sf[6] = (float)b1.x; sf[7] = (float)b1.y; sf[8] = (float)b1.z;
  sf[9] = (float)b2.x; sf[10] = (float)b2.y; sf[11] = (float)b2.z;
  sf[12] = (float)st[6];
}
// ls_frame on a whole warp: lane i < 3 computes component i of b1 and b2
// (the same expressions, component by component; lanes 3..31 repeat lane
// 0's), so each FP64 instruction serves three components: the FP64 pipe
// takes about as long for one active lane as for 32.
__device__ __forceinline__ void warp_ls_frame(double* st, float* sf) {
  const int lane = threadIdx.x & 31;
  const int i = lane < 3 ? lane : 0;
  const d3 dd = mk3(st[3], st[4], st[5]);
  const d3 t = fabs(dd.x) < 0.9 ? mk3(1, 0, 0) : mk3(0, 1, 0);
  const int i1 = i == 2 ? 0 : i + 1, i2 = i == 0 ? 2 : i - 1;  // the cross product's indices
  const double da[3] = {dd.x, dd.y, dd.z}, ta[3] = {t.x, t.y, t.z};
  double b1 = da[i1] * ta[i2] - da[i2] * ta[i1];
  const double b1x = __shfl_sync(0xffffffffu, b1, 0), b1y = __shfl_sync(0xffffffffu, b1, 1),
               b1z = __shfl_sync(0xffffffffu, b1, 2);
  b1 = (1.0 / norm3(mk3(b1x, b1y, b1z))) * b1;
  const double n0 = __shfl_sync(0xffffffffu, b1, 0), n1 = __shfl_sync(0xffffffffu, b1, 1),
               n2 = __shfl_sync(0xffffffffu, b1, 2);
  const double ba[3] = {n0, n1, n2};
  const double b2 = da[i1] * ba[i2] - da[i2] * ba[i1];
  __syncwarp();
  if (lane < 3) {
    st[8 + i] = b1;
    st[11 + i] = b2;
    sf[6 + i] = (float)b1;
    sf[9 + i] = (float)b2;
  }
  if (lane < 6) sf[lane] = (float)st[lane];
  if (lane == 0) sf[12] = (float)st[6];
  __syncwarp();
}

// The LS model update on a whole warp (st in shared memory, x the 5x5
// solution): centre += x0 b1 + x1 b2, direction += x2 b1 + x3 b2 then
// normalised, radius += x4, then the new frame -- the expressions of the
// one-thread update, component by component on lanes 0..2.
__device__ __forceinline__ void warp_model_update(double* st, const double* x, float* sf) {
  const int lane = threadIdx.x & 31;
  const int i = lane < 3 ? lane : 0;
  const double b1 = st[8 + i], b2 = st[11 + i];
  const double c2 = (st[i] + x[0] * b1) + x[1] * b2;
  double d2 = (st[3 + i] + x[2] * b1) + x[3] * b2;
  const double dx = __shfl_sync(0xffffffffu, d2, 0), dy = __shfl_sync(0xffffffffu, d2, 1),
               dz = __shfl_sync(0xffffffffu, d2, 2);
  d2 = (1.0 / norm3(mk3(dx, dy, dz))) * d2;
  const double r = st[6] + x[4];
  __syncwarp();
  if (lane < 3) {
    st[i] = c2;
    st[3 + i] = d2;
  }
  if (lane == 0) st[6] = r;
  __syncwarp();
  warp_ls_frame(st, sf);
}
}  // namespace sg
