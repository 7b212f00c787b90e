// pose.cu — a9-a11: association, pose update, re-projection and map
// association of sloam::sloam::RunSloam (sloam.cpp:453-532).
//
// a9  matchFeatures (sloam.cpp:257-296): the map's axis points at the three
//     sample heights of Cylinder::distance (cylinder.cpp:175-194) are
//     computed once per keyframe; then one block per current object, its
//     threads over the map, FP64 distances, argmin with first-index ties.
// a10 pose (replacing Ceres LM, sloam.cpp:33-255): fixed gn_iters
//     Gauss-Newton iterations with IRLS Huber weights in one block; the
//     residual table (sensor point, anchored model) is built once, residuals
//     and Jacobians are FP32 in a frame anchored at the pose estimate's
//     translation, J^T J / J^T r are reduced with warp shuffles, the normal
//     equations solved and the SE(3) update applied in FP64.  Joint mode:
//     left SO(3) perturbation + translation (6x6).  Two-step mode: the
//     reference's angle-axis 6-vector with {x, y, yaw} then {z, roll, pitch}
//     free (3x3 each) and its angle-axis recombination.
// a11 projectModels + matchModels (sloam.cpp:298-328, 438-451) and the
//     prevGPlanes_ update.
#include <cfloat>

#include "internal.h"
#include "scan_util.cuh"

namespace sg {

namespace {

constexpr int kAssocThreads = 128;
constexpr int kGN = 256;
constexpr int kResStride = 12;

__device__ __forceinline__ Pose pose_at(const double* p) {
  sloam_se3 s;
  for (int j = 0; j < 4; ++j) s.q[j] = p[j];
  for (int j = 0; j < 3; ++j) s.t[j] = p[4 + j];
  return pose_from(s);
}
__device__ __forceinline__ void pose_store(double* p, const Pose& T) {
  const sloam_se3 s = pose_to(T);
  for (int j = 0; j < 4; ++j) p[j] = s.q[j];
  for (int j = 0; j < 3; ++j) p[4 + j] = s.t[j];
}

// Axis points of a cylinder at z = 0, 3, 6 (Cylinder::distance's samples).
__device__ __forceinline__ void axis_points(d3 root, d3 ray, d3* pts) {
  const double hs[3] = {0.0, 3.0, 6.0};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double t = (hs[k] - root.z) / ray.z;
    pts[k] = add3(root, scl3(t, ray));
  }
}
__device__ __forceinline__ double axis_dist(const double* mp, const d3* tp) {
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    acc += norm3(mk3(mp[3 * k] - tp[k].x, mp[3 * k + 1] - tp[k].y, mp[3 * k + 2] - tp[k].z));
  return acc / 3.0;
}

// Cylinder::project, cylinder.cpp:205-211
__device__ __forceinline__ void cyl_project(const Pose& T, d3& root, d3& ray) {
  const d3 other = xform(T, add3(root, ray));
  root = xform(T, root);
  ray = sub3(other, root);
}

// block-wide argmin (value, then index) of non-negative, non-NaN doubles:
// their bit patterns order as unsigned integers, so the comparisons need no
// FP64 instruction
__device__ __forceinline__ void block_argmin(double& v, int& i, double* sv, int* si) {
  unsigned long long key = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (ok < key || (ok == key && oi < i)) {
      key = ok;
      i = oi;
    }
  }
  unsigned long long* sk = reinterpret_cast<unsigned long long*>(sv);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sk[w] = key; si[w] = i; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
      if (sk[k] < sk[0] || (sk[k] == sk[0] && si[k] < si[0])) { sk[0] = sk[k]; si[0] = si[k]; }
  }
  __syncthreads();
  v = __longlong_as_double((long long)sk[0]);
  i = si[0];
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_map_prep(Dev d) {
  const int n = d.in->n_map;
  const sloam_cylinder* map = d.in->map;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const sloam_cylinder& m = map[k];
    d3 pts[3];
    axis_points(mk3(m.root[0], m.root[1], m.root[2]), mk3(m.ray[0], m.ray[1], m.ray[2]), pts);
    float f[12];
    float cmax = 0.0f;
    for (int j = 0; j < 3; ++j) {
      d.map_pts[9 * k + 3 * j] = pts[j].x;
      d.map_pts[9 * k + 3 * j + 1] = pts[j].y;
      d.map_pts[9 * k + 3 * j + 2] = pts[j].z;
      f[3 * j] = (float)pts[j].x;
      f[3 * j + 1] = (float)pts[j].y;
      f[3 * j + 2] = (float)pts[j].z;
      cmax = fmaxf(cmax, fmaxf(fabsf(f[3 * j]), fmaxf(fabsf(f[3 * j + 1]), fabsf(f[3 * j + 2]))));
    }
    f[9] = cmax;  // NaN coordinates make every bound NaN: never a candidate
    if (!(cmax < INFINITY)) f[9] = __int_as_float(0x7fc00000);
    f[10] = f[11] = 0.0f;
    for (int j = 0; j < 3; ++j)
      d.map_f[3 * (size_t)k + j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
  }
}

// The current cylinder's axis points, shared by the block (written by one
// thread): FP64, FP32 copies and their max |coordinate|.
struct AxisPts {
  double tp[9];
  float tf[9];
  float tmax;
};

__device__ __forceinline__ void set_axis_pts(AxisPts* a, d3 root, d3 ray) {
  d3 tp[3];
  axis_points(root, ray, tp);
  float cmax = 0.0f;
  for (int k = 0; k < 3; ++k) {
    a->tp[3 * k] = tp[k].x; a->tp[3 * k + 1] = tp[k].y; a->tp[3 * k + 2] = tp[k].z;
    a->tf[3 * k] = (float)tp[k].x; a->tf[3 * k + 1] = (float)tp[k].y;
    a->tf[3 * k + 2] = (float)tp[k].z;
    cmax = fmaxf(cmax, fmaxf(fabsf(a->tf[3 * k]), fmaxf(fabsf(a->tf[3 * k + 1]),
                                                         fabsf(a->tf[3 * k + 2]))));
  }
  a->tmax = cmax < INFINITY ? cmax : __int_as_float(0x7fc00000);
}

// FP32 axis distance of map entry k (its three float4 records) and a bound
// on |it - the exact distance|: coordinates rounded to float (u = 2^-24 each)
// move each of the three norms by at most sqrt(3) u (|m| + |t|)max, the float
// differences, squares, sums, root and mean add a few u relative; the bound
// takes 3e-7 * (2 (|m|max + |t|max) + 8 d) (about 2x these).  NaN or
// infinite inputs give a NaN bound.
__device__ __forceinline__ float axis_dist_f(const float4* mf, const float* tf, float tmax,
                                             float* eps) {
  const float4 a = mf[0], b = mf[1], c = mf[2];
  const float m[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dx = m[3 * k] - tf[3 * k], dy = m[3 * k + 1] - tf[3 * k + 1],
                dz = m[3 * k + 2] - tf[3 * k + 2];
    acc += sqrtf(dx * dx + dy * dy + dz * dz);
  }
  const float dist = acc * (1.0f / 3.0f);
  *eps = 3e-7f * (2.0f * (c.y + tmax) + 8.0f * dist);
  return dist;
}

// argmin over the map of the distance to the current cylinder whose axis
// points are in *a: the smallest FP64 distance below `init`, first index on
// ties (bi = 0 when none), exactly as an FP64 scan of the whole map.  The
// FP64 distance is evaluated only for entries whose FP32 lower bound
// (distance - eps) is at most the smallest FP32 upper bound (distance + eps,
// or init): the exact minimum and every entry tied with it are among them.
__device__ void map_argmin(const Dev& d, const AxisPts* a, double init, double& bd, int& bi,
                           double* sv, int* si, float* su) {
  const int n_map = d.in->n_map;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float tf[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) tf[j] = a->tf[j];
  const float tmax = a->tmax;
  float U = (float)init * (1.0f + 1e-6f);
  for (int k = threadIdx.x; k < n_map; k += blockDim.x) {
    float eps;
    const float df = axis_dist_f(d.map_f + 3 * (size_t)k, tf, tmax, &eps);
    U = fminf(U, df + eps);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) U = fminf(U, __shfl_xor_sync(0xffffffffu, U, o));
  if (lane == 0) su[w] = U;
  __syncthreads();
  U = su[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); ++q) U = fminf(U, su[q]);
  bd = init;
  bi = 0;
  for (int k = threadIdx.x; k < n_map; k += blockDim.x) {
    float eps;
    const float df = axis_dist_f(d.map_f + 3 * (size_t)k, tf, tmax, &eps);
    if (!(df - eps <= U)) continue;
    d3 tp[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) tp[j] = mk3(a->tp[3 * j], a->tp[3 * j + 1], a->tp[3 * j + 2]);
    const double dist = axis_dist(d.map_pts + 9 * (size_t)k, tp);
    if (dist < bd) { bd = dist; bi = k; }
  }
  block_argmin(bd, bi, sv, si);
}

__global__ void __launch_bounds__(kAssocThreads) k_assoc(Dev d, KParams kp) {
  __shared__ double sv[kAssocThreads / 32];
  __shared__ int si[kAssocThreads / 32];
  __shared__ float su[kAssocThreads / 32];
  __shared__ AxisPts ax;
  __shared__ Pose sT;
  __shared__ double sc[3];
  const int nc = d.cnt->n_cyl, np = d.cnt->n_planes, nprev = d.cnt->n_prev;
  if (threadIdx.x == 0) sT = pose_at(d.pose_io);  // FP64 once per block
  __syncthreads();
  const Pose& T = sT;
  for (int it = blockIdx.x; it < nc + np; it += gridDim.x) {
    double bd;
    int bi;
    if (it < nc) {
      if (threadIdx.x == 0) {
        const CylD c = d.cyls[it];
        d3 root = mk3(c.root[0], c.root[1], c.root[2]), ray = mk3(c.ray[0], c.ray[1], c.ray[2]);
        cyl_project(T, root, ray);
        set_axis_pts(&ax, root, ray);
      }
      __syncthreads();
      map_argmin(d, &ax, kp.tree_match_thresh + 100, bd, bi, sv, si, su);
      if (threadIdx.x == 0)
        d.cyl_match[it] = (d.in->n_map > 0 && bd < kp.tree_match_thresh) ? bi : -1;
    } else {
      const int p = it - nc;
      if (threadIdx.x == 0) {
        const PlaneD P = d.planes[p];
        const d3 c0 = xform(T, mk3(P.centroid[0], P.centroid[1], P.centroid[2]));
        sc[0] = c0.x; sc[1] = c0.y; sc[2] = c0.z;
      }
      __syncthreads();
      const d3 c = mk3(sc[0], sc[1], sc[2]);
      bd = kp.plane_match_thresh + 100;
      bi = 0;
      for (int k = threadIdx.x; k < nprev; k += blockDim.x) {
        const PlaneD& Q = d.prev_planes[k];
        const double dist = norm3(sub3(mk3(Q.centroid[0], Q.centroid[1], Q.centroid[2]), c));
        if (dist < bd) { bd = dist; bi = k; }
      }
      block_argmin(bd, bi, sv, si);
      if (threadIdx.x == 0)
        d.plane_match[p] = (nprev > 0 && bd < kp.plane_match_thresh) ? bi : -1;
    }
  }
}

__device__ __forceinline__ float huber_w(float r, float delta) {
  const float a = fabsf(r);
  return a <= delta ? 1.0f : delta / a;
}

// Ceres QuaternionToAngleAxis / AngleAxisToQuaternion (rotation.h), restated.
__device__ void quat_to_aa(const double* qwxyz, double* aa) {
  const double q1 = qwxyz[1], q2 = qwxyz[2], q3 = qwxyz[3];
  const double s2 = q1 * q1 + q2 * q2 + q3 * q3;
  if (s2 > 0.0) {
    const double s = sqrt(s2), c = qwxyz[0];
    const double two_theta = 2.0 * ((c < 0.0) ? atan2(-s, -c) : atan2(s, c));
    const double k = two_theta / s;
    aa[0] = q1 * k; aa[1] = q2 * k; aa[2] = q3 * k;
  } else {
    aa[0] = q1 * 2.0; aa[1] = q2 * 2.0; aa[2] = q3 * 2.0;
  }
}
__device__ void aa_to_quat(const double* aa, double* qwxyz) {
  const double t2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (t2 > 0.0) {
    const double th = sqrt(t2), h = th * 0.5, k = sin(h) / th;
    qwxyz[0] = cos(h); qwxyz[1] = aa[0] * k; qwxyz[2] = aa[1] * k; qwxyz[3] = aa[2] * k;
  } else {
    qwxyz[0] = 1.0; qwxyz[1] = aa[0] * 0.5; qwxyz[2] = aa[1] * 0.5; qwxyz[3] = aa[2] * 0.5;
  }
}

// Rotation (Rm: the point map) and the pieces of d(R(r)p)/dr = -Rj [p]x Jr for
// an angle-axis vector r (Ceres AngleAxisRotatePoint semantics, including its
// first-order branch for theta^2 <= DBL_EPSILON).
__device__ void aa_mats(const double* r, double* Rm, double* Rj, double* Jr) {
  const double th2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (th2 > DBL_EPSILON) {
    const double th = sqrt(th2);
    so3_exp(mk3(r[0], r[1], r[2]), Rm);
    for (int k = 0; k < 9; ++k) Rj[k] = Rm[k];
    const double A = (1.0 - cos(th)) / th2, B = (th - sin(th)) / (th2 * th);
    const double K[9] = {0, -r[2], r[1], r[2], 0, -r[0], -r[1], r[0], 0};
    double K2[9];
    matmul3(K, K, K2);
    for (int i = 0; i < 9; ++i) Jr[i] = (i % 4 == 0 ? 1.0 : 0.0) - A * K[i] + B * K2[i];
  } else {
    const double K[9] = {0, -r[2], r[1], r[2], 0, -r[0], -r[1], r[0], 0};
    for (int i = 0; i < 9; ++i) {
      Rm[i] = (i % 4 == 0 ? 1.0 : 0.0) + K[i];
      Rj[i] = (i % 4 == 0 ? 1.0 : 0.0);
      Jr[i] = (i % 4 == 0 ? 1.0 : 0.0);
    }
  }
}

// aa_mats on one warp, as floats for the residual pass: lane i < 9 writes
// Rm_i and Rj_i, lane 9 + i writes Jr_i, each entry by the formulas of
// aa_mats and so3_exp (all 32 lanes call it; lanes 18..31 write nothing).
// Every lane takes the same sin, cos and quotients, so the FP64 work is one
// warp instruction per step for all 18 entries: the narrow FP64 pipe costs
// the same for one lane or 32, and aa_mats on one thread runs its 27
// entries one after another with sin and cos twice.
__device__ void warp_aa_mats_f(const double* r, float* sRm, float* sRj, float* sJr) {
  const int lane = threadIdx.x & 31;
  const double th2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double K[9] = {0, -r[2], r[1], r[2], 0, -r[0], -r[1], r[0], 0};
  const int i = lane < 9 ? lane : (lane < 18 ? lane - 9 : 0);
  const int a = i / 3, b = i - 3 * a;
  const double k2 = K[3 * a] * K[b] + K[3 * a + 1] * K[3 + b] + K[3 * a + 2] * K[6 + b];
  const double id = (i % 4 == 0) ? 1.0 : 0.0;
  double rm, rj, jr;
  if (th2 > DBL_EPSILON) {
    const double th = sqrt(th2);
    const double sn = sin(th), cs = cos(th);
    double A, B;  // exp([r]x) = I + A K + B K^2 (so3_exp)
    if (th2 < 1e-2) {
      A = 1.0 - th2 / 6.0 * (1.0 - th2 / 20.0 * (1.0 - th2 / 42.0));
      B = 0.5 - th2 / 24.0 * (1.0 - th2 / 30.0 * (1.0 - th2 / 56.0));
    } else {
      A = sn / th;
      B = (1.0 - cs) / th2;
    }
    const double Aj = (1.0 - cs) / th2, Bj = (th - sn) / (th2 * th);
    rm = id + A * K[i] + B * k2;
    rj = rm;
    jr = id - Aj * K[i] + Bj * k2;
  } else {
    rm = id + K[i];
    rj = id;
    jr = id;
  }
  if (lane < 9) {
    sRm[i] = (float)rm;
    sRj[i] = (float)rj;
  } else if (lane < 18) {
    sJr[i] = (float)jr;
  }
}

// Residual table entry i: [kind, px, py, pz, m0..m7] with kind 0 = none,
// 1 = cylinder (root - anchor, ray, 1/ray.ray, radius), 2 = plane (n, d + n.anchor, 1/|n|).
__device__ void build_residual(const Dev& d, const KParams& kp, int i, int nc, const double* a,
                               float* e) {
  e[0] = 0.f;
  if (i < nc * kp.F) {
    const int c = i / kp.F;
    const int m = d.cyl_match[c];
    if (m < 0) return;
    const float4 f = d.cyl_feat[(size_t)c * kp.F + (i - c * kp.F)];
    const sloam_cylinder& M = d.in->map[m];
    e[0] = 1.f;
    e[1] = f.x; e[2] = f.y; e[3] = f.z;
    e[4] = (float)(M.root[0] - a[0]); e[5] = (float)(M.root[1] - a[1]);
    e[6] = (float)(M.root[2] - a[2]);
    e[7] = (float)M.ray[0]; e[8] = (float)M.ray[1]; e[9] = (float)M.ray[2];
    e[10] = (float)(1.0 / (M.ray[0] * M.ray[0] + M.ray[1] * M.ray[1] + M.ray[2] * M.ray[2]));
    e[11] = (float)M.radius;
    return;
  }
  i -= nc * kp.F;
  const int p = i / kp.G;
  const int m = d.plane_match[p];
  if (m < 0) return;
  const float4 f = d.plane_feat[(size_t)p * kp.G + (i - p * kp.G)];
  const PlaneD& Q = d.prev_planes[m];
  e[0] = 2.f;
  e[1] = f.x; e[2] = f.y; e[3] = f.z;
  e[4] = (float)Q.plane[0]; e[5] = (float)Q.plane[1]; e[6] = (float)Q.plane[2];
  e[7] = (float)(Q.plane[3] + Q.plane[0] * a[0] + Q.plane[1] * a[1] + Q.plane[2] * a[2]);
  e[8] = (float)(1.0 / sqrt(Q.plane[0] * Q.plane[0] + Q.plane[1] * Q.plane[1] +
                            Q.plane[2] * Q.plane[2]));
}

// residual and its gradient w.r.t. the transformed point lp (FP32)
__device__ __forceinline__ float residual_eval(const float* e, float lx, float ly, float lz,
                                               float* J) {
  if (e[0] == 1.f) {
    const float vx = lx - e[4], vy = ly - e[5], vz = lz - e[6];
    const float s = (vx * e[7] + vy * e[8] + vz * e[9]) * e[10];
    const float wx = vx - s * e[7], wy = vy - s * e[8], wz = vz - s * e[9];
    const float nw = sqrtf(wx * wx + wy * wy + wz * wz);
    if (nw > 0.f) {
      const float inv = 1.0f / nw;
      J[0] = wx * inv; J[1] = wy * inv; J[2] = wz * inv;
    } else {
      J[0] = J[1] = J[2] = 0.f;
    }
    return nw - e[11];
  }
  const float num = e[4] * lx + e[5] * ly + e[6] * lz + e[7];
  const float sg = num > 0.f ? e[8] : (num < 0.f ? -e[8] : 0.f);
  J[0] = sg * e[4]; J[1] = sg * e[5]; J[2] = sg * e[6];
  return fabsf(num) * e[8];
}

// block reduction of NV floats over kGN threads into s_out (FP64)
template <int NV>
__device__ __forceinline__ void reduce_normal(const float* acc, float (*red)[kGN / 32],
                                              double* s_out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const float v = warp_sum(acc[j]);
    if (lane == 0) red[j][w] = v;
  }
  __syncthreads();
  if (w == 0 && lane < NV) {
    double s = 0;
#pragma unroll
    for (int q = 0; q < kGN / 32; ++q) s += red[lane][q];
    s_out[lane] = s;
  }
  __syncthreads();
}

// ---- pose_solver 1: trust-region Levenberg-Marquardt (the rules of the
// oracle's lm_minimize: the solver settings the reference gives Ceres,
// sloam.cpp:91-97, 149-155).  The bookkeeping runs on one thread in FP64;
// the residual passes use the whole block.
template <int N>
struct LMDev {
  double H[N * N], g[N], cost;  // linearisation at the current point
  double radius, factor, model;
  double d[N];                  // the step proposed last
  int done;
};
__device__ __forceinline__ float huber_rho_f(float r, float delta) {
  const float a = fabsf(r);
  return a <= delta ? r * r : 2.0f * delta * a - delta * delta;
}
// H (upper triangle, row by row), g and the cost from a block reduction;
// `sc` scales the parameters (the joint mode steps half rotation vectors)
template <int N>
__device__ void lm_load(LMDev<N>& L, const double* s_out, const double* sc) {
  int k = 0;
  for (int a = 0; a < N; ++a)
    for (int b = a; b < N; ++b) {
      L.H[N * a + b] = L.H[N * b + a] = sc[a] * s_out[k] * sc[b];
      ++k;
    }
  for (int a = 0; a < N; ++a) L.g[a] = sc[a] * s_out[k + a];
  L.cost = s_out[k + N];
}
template <int N>
__device__ bool lm_gsmall(const LMDev<N>& L) {
  double m = 0.0;
  for (int i = 0; i < N; ++i) m = fmax(m, fabs(L.g[i]));
  return m <= 1e-10;
}
// One proposal: 1 = a candidate step in L.d, -1 = the damped system failed
// (the radius shrank), 0 = stopped (step below the parameter tolerance, or
// the radius below 1e-32).
template <int N>
__device__ int lm_propose(LMDev<N>& L, double xnorm) {
  double sc[N], A[N * N], b[N], ds[N];
  for (int i = 0; i < N; ++i) sc[i] = 1.0 / (1.0 + sqrt(L.H[i * N + i]));
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) A[i * N + j] = sc[i] * L.H[i * N + j] * sc[j];
  for (int i = 0; i < N; ++i) {
    const double dg = fmin(fmax(A[i * N + i], 1e-6), 1e32);
    A[i * N + i] += dg / L.radius;
    b[i] = -sc[i] * L.g[i];
  }
  if (!chol_solve(N, A, b, ds)) {
    L.radius /= L.factor;
    L.factor *= 2.0;
    return L.radius < 1e-32 ? 0 : -1;
  }
  double step2 = 0.0, gd = 0.0, dHd = 0.0;
  for (int i = 0; i < N; ++i) {
    L.d[i] = sc[i] * ds[i];
    step2 += L.d[i] * L.d[i];
  }
  for (int i = 0; i < N; ++i) {
    gd += L.g[i] * L.d[i];
    for (int j = 0; j < N; ++j) dHd += L.d[i] * L.H[i * N + j] * L.d[j];
  }
  L.model = -(gd + 0.5 * dHd);
  if (sqrt(step2) <= 1e-8 * (xnorm + 1e-8)) return 0;
  return 1;
}
// The candidate's linearisation in s_out: true when the step is taken;
// sets L.done when the solve stops.
template <int N>
__device__ bool lm_decide(LMDev<N>& L, const double* s_out, const double* sc) {
  LMDev<N> C;
  lm_load<N>(C, s_out, sc);
  if (fabs(L.cost - C.cost) <= 1e-6 * L.cost) {
    L.done = 1;
    return false;
  }
  const double ratio = (L.cost - C.cost) / L.model;
  if (L.model > 0.0 && ratio > 1e-3) {
    for (int i = 0; i < N * N; ++i) L.H[i] = C.H[i];
    for (int i = 0; i < N; ++i) L.g[i] = C.g[i];
    L.cost = C.cost;
    const double t = 2.0 * ratio - 1.0;
    L.radius = fmin(1e16, L.radius / fmax(1.0 / 3.0, 1.0 - t * t * t));
    L.factor = 2.0;
    if (lm_gsmall<N>(L)) L.done = 1;
    return true;
  }
  L.radius /= L.factor;
  L.factor *= 2.0;
  if (L.radius < 1e-32) L.done = 1;
  return false;
}

template <bool kLM>
__global__ void __launch_bounds__(kGN) k_gn(Dev d, KParams kp) {
  __shared__ float red[28][kGN / 32];
  __shared__ double s_out[28];
  __shared__ LMDev<6> lm6;
  __shared__ LMDev<3> lm3;
  __shared__ double c_R[9], c_t[3], c_x[6];
  __shared__ int s_flag;
  __shared__ float sR[9], sT[3], sRj[9], sJr[9];
  __shared__ double s_R[9], s_t[3], s_x[6], s_anchor[3];
  __shared__ int s_ok, s_checks[2];
  __shared__ int sm[33];
  const int nc = d.cnt->n_cyl, np = d.cnt->n_planes;
  const int nitems = nc * kp.F + np * kp.G;
  // ---- counts and gates (sloam.cpp:499-500)
  {
    int mc = 0, mp = 0;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) mc += d.cyl_match[c] >= 0;
    for (int p = threadIdx.x; p < np; p += blockDim.x) mp += d.plane_match[p] >= 0;
    int tc, tp;
    block_excl_scan(mc, sm, &tc);
    block_excl_scan(mp, sm, &tp);
    if (threadIdx.x == 0) {
      const int ntm = tc * kp.F, npm = tp * kp.G;
      d.cnt->n_tm = ntm;
      d.cnt->n_pm = npm;
      const int tchk = nc > kp.min_tree_models && ntm > 5.0 * kp.F;
      const int gchk = npm > kp.min_ground_models && np > kp.min_planes;
      d.cnt->tree_check = tchk;
      d.cnt->ground_check = gchk;
      s_checks[0] = tchk;
      s_checks[1] = gchk;
      const Pose E = pose_at(d.pose_io);
      for (int k = 0; k < 9; ++k) s_R[k] = E.R[k];
      s_anchor[0] = E.t.x; s_anchor[1] = E.t.y; s_anchor[2] = E.t.z;
      s_t[0] = s_t[1] = s_t[2] = 0.0;
      s_ok = 1;
      d.cnt->status = (np == 0 || nc == 0) ? SLOAM_ERR_NO_MODELS : SLOAM_OK;
      for (int j = 0; j < 7; ++j) d.pose_io[7 + j] = d.pose_io[j];
      for (int j = 0; j < 7; ++j) d.pose_io[14 + j] = (j == 3) ? 1.0 : 0.0;
      d.cnt->success = 1;
    }
    __syncthreads();
  }
  if (np == 0 || nc == 0) return;
  // ---- residual table (each thread builds and later reads its own entries)
  for (int i = threadIdx.x; i < nitems; i += blockDim.x)
    build_residual(d, kp, i, nc, s_anchor, d.res_tab + (size_t)kResStride * i);
  const int tchk = s_checks[0], gchk = s_checks[1];
  const float delta = (float)kp.huber;
  if (!kp.two_step) {
    if (!(tchk && gchk)) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if constexpr (kLM) {
      // ------------------------------------------ joint, trust-region LM
      const double sc6[6] = {2.0, 2.0, 2.0, 1.0, 1.0, 1.0};  // d = omega / 2
      auto pass = [&]() {  // cost, H, g at (sR, sT)
        float acc[28];
#pragma unroll
        for (int j = 0; j < 28; ++j) acc[j] = 0.f;
        for (int i = threadIdx.x; i < nitems; i += blockDim.x) {
          const float* e = d.res_tab + (size_t)kResStride * i;
          if (e[0] == 0.f) continue;
          const float px = e[1], py = e[2], pz = e[3];
          const float qx = sR[0] * px + sR[1] * py + sR[2] * pz;
          const float qy = sR[3] * px + sR[4] * py + sR[5] * pz;
          const float qz = sR[6] * px + sR[7] * py + sR[8] * pz;
          float Jl[3];
          const float res = residual_eval(e, qx + sT[0], qy + sT[1], qz + sT[2], Jl);
          const float J[6] = {qy * Jl[2] - qz * Jl[1], qz * Jl[0] - qx * Jl[2],
                              qx * Jl[1] - qy * Jl[0], Jl[0], Jl[1], Jl[2]};
          const float wgt = huber_w(res, delta);
          int k = 0;
#pragma unroll
          for (int a = 0; a < 6; ++a) {
            const float wa = wgt * J[a];
#pragma unroll
            for (int b = a; b < 6; ++b) acc[k++] += wa * J[b];
            acc[21 + a] += wa * res;
          }
          acc[27] += 0.5f * huber_rho_f(res, delta);
        }
        reduce_normal<28>(acc, red, s_out);
      };
      if (w == 0 && lane < 12) {
        if (lane < 9) sR[lane] = (float)s_R[lane];
        else sT[lane - 9] = (float)s_t[lane - 9];
      }
      __syncthreads();
      pass();
      if (threadIdx.x == 0) {
        lm_load<6>(lm6, s_out, sc6);
        lm6.radius = 1e4;
        lm6.factor = 2.0;
        lm6.done = lm_gsmall<6>(lm6) ? 1 : 0;
      }
      __syncthreads();
      for (int itn = 0; itn < kp.lm_iters; ++itn) {
        if (threadIdx.x == 0) {
          int r = 0;
          if (!lm6.done) {
            const double ta[3] = {s_t[0] + s_anchor[0], s_t[1] + s_anchor[1], s_t[2] + s_anchor[2]};
            r = lm_propose<6>(lm6, sqrt(1.0 + ta[0] * ta[0] + ta[1] * ta[1] + ta[2] * ta[2]));
          }
          if (r == 1) {
            double dR[9];
            so3_exp(mk3(2.0 * lm6.d[0], 2.0 * lm6.d[1], 2.0 * lm6.d[2]), dR);
            matmul3(dR, s_R, c_R);
            for (int k = 0; k < 3; ++k) c_t[k] = s_t[k] + lm6.d[3 + k];
            for (int k = 0; k < 9; ++k) sR[k] = (float)c_R[k];
            for (int k = 0; k < 3; ++k) sT[k] = (float)c_t[k];
          }
          s_flag = r;
        }
        __syncthreads();
        const int r = s_flag;
        if (r == 1) {
          pass();
          if (threadIdx.x == 0 && lm_decide<6>(lm6, s_out, sc6)) {
            for (int k = 0; k < 9; ++k) s_R[k] = c_R[k];
            for (int k = 0; k < 3; ++k) s_t[k] = c_t[k];
          }
        }
        __syncthreads();
        if (r == 0) break;
      }
      if (threadIdx.x == 0) {
        d.cnt->success = 1;
        Pose T;
        for (int k = 0; k < 9; ++k) T.R[k] = s_R[k];
        T.t = mk3(s_t[0] + s_anchor[0], s_t[1] + s_anchor[1], s_t[2] + s_anchor[2]);
        pose_store(d.pose_io + 7, T);
        pose_store(d.pose_io + 14, T);
      }
      return;
    } else {
      // ---------------------------------------------------------- joint
      for (int itn = 0; itn < kp.gn_iters; ++itn) {
        // float copies of the pose, one lane per entry
        if (w == 0 && lane < 12) {
          if (lane < 9) sR[lane] = (float)s_R[lane];
          else sT[lane - 9] = (float)s_t[lane - 9];
        }
        __syncthreads();
        float acc[27];
  #pragma unroll
        for (int j = 0; j < 27; ++j) acc[j] = 0.f;
        for (int i = threadIdx.x; i < nitems; i += blockDim.x) {
          const float* e = d.res_tab + (size_t)kResStride * i;
          if (e[0] == 0.f) continue;
          const float px = e[1], py = e[2], pz = e[3];
          const float qx = sR[0] * px + sR[1] * py + sR[2] * pz;
          const float qy = sR[3] * px + sR[4] * py + sR[5] * pz;
          const float qz = sR[6] * px + sR[7] * py + sR[8] * pz;
          float Jl[3];
          const float res = residual_eval(e, qx + sT[0], qy + sT[1], qz + sT[2], Jl);
          const float J[6] = {qy * Jl[2] - qz * Jl[1], qz * Jl[0] - qx * Jl[2],
                              qx * Jl[1] - qy * Jl[0], Jl[0], Jl[1], Jl[2]};
          const float wgt = huber_w(res, delta);
          int k = 0;
  #pragma unroll
          for (int a = 0; a < 6; ++a) {
            const float wa = wgt * J[a];
  #pragma unroll
            for (int b = a; b < 6; ++b) acc[k++] += wa * J[b];
            acc[21 + a] += wa * res;
          }
        }
        reduce_normal<27>(acc, red, s_out);
        // FP64 6x6 solve by warp 0; the SE(3) update R <- exp([x0..2]) R,
        // t <- t + x3..5 on nine lanes of the same warp (each FP64 warp
        // instruction costs the pipe the same for one lane or nine)
        if (w == 0) {
          // H x = -g (s_out: H's upper triangle, then g) on the whole warp
          const bool solved = s_ok && warp_chol_solve<6>(s_out, s_out + 21, s_x);
          __syncwarp();
          if (lane == 0 && !solved) s_ok = 0;
          __syncwarp();
          if (s_ok && lane < 9) {
            const int r = lane / 3, c = lane - 3 * r;
            double dRr[3];
            so3_exp_row(mk3(s_x[0], s_x[1], s_x[2]), r, dRr);
            const double v = dRr[0] * s_R[c] + dRr[1] * s_R[3 + c] + dRr[2] * s_R[6 + c];
            const double tn = lane < 3 ? s_t[lane] + s_x[3 + lane] : 0.0;
            __syncwarp(0x1ffu);
            s_R[lane] = v;
            if (lane < 3) s_t[lane] = tn;
          }
        }
        __syncthreads();
        if (!s_ok) break;
      }
      if (threadIdx.x == 0) {
        d.cnt->success = s_ok;
        if (s_ok) {
          Pose T;
          for (int k = 0; k < 9; ++k) T.R[k] = s_R[k];
          T.t = mk3(s_t[0] + s_anchor[0], s_t[1] + s_anchor[1], s_t[2] + s_anchor[2]);
          pose_store(d.pose_io + 7, T);
          pose_store(d.pose_io + 14, T);
        } else {
          d.cnt->status = SLOAM_ERR_NOT_CONVERGED;
        }
      }
      return;
    }
  }
  // -------------------------------------------------------- two-step
  double rpy[3];
  double out_tree[3], out_ground[3];
  {
    const sloam_se3 e = pose_to(pose_at(d.pose_io));
    const double qwxyz[4] = {e.q[3], e.q[0], e.q[1], e.q[2]};
    quat_to_aa(qwxyz, rpy);
  }
  for (int step = 0; step < 2; ++step) {
    const bool opt = step == 0 ? tchk : gchk;
    const int f0 = step == 0 ? 0 : 2, f1 = step == 0 ? 1 : 3, f2 = step == 0 ? 5 : 4;
    if (threadIdx.x == 0) {
      s_x[0] = s_anchor[0]; s_x[1] = s_anchor[1]; s_x[2] = s_anchor[2];
      s_x[3] = rpy[0]; s_x[4] = rpy[1]; s_x[5] = rpy[2];
      s_ok = opt ? 1 : 0;
    }
    __syncthreads();
    const int lo = step == 0 ? 0 : nc * kp.F;
    const int hi = step == 0 ? nc * kp.F : nitems;
    if constexpr (kLM) {
      // ------------------------------------- subset, trust-region LM
      const double sc3[3] = {1.0, 1.0, 1.0};
      auto set_point = [&](const double* xv) {  // thread 0: the pass's matrices at xv
        double Rm[9], Rj[9], Jr[9];
        aa_mats(xv + 3, Rm, Rj, Jr);
        for (int k = 0; k < 9; ++k) {
          sR[k] = (float)Rm[k];
          sRj[k] = (float)Rj[k];
          sJr[k] = (float)Jr[k];
        }
        for (int k = 0; k < 3; ++k) sT[k] = (float)(xv[k] - s_anchor[k]);
      };
      auto pass = [&]() {  // cost, H, g of the free entries at (sR, sRj, sJr, sT)
        float acc[10];
#pragma unroll
        for (int j = 0; j < 10; ++j) acc[j] = 0.f;
        for (int i = threadIdx.x; i < nitems; i += blockDim.x) {
          if (i < lo || i >= hi) continue;
          const float* e = d.res_tab + (size_t)kResStride * i;
          if (e[0] == 0.f) continue;
          const float px = e[1], py = e[2], pz = e[3];
          const float qx = sR[0] * px + sR[1] * py + sR[2] * pz;
          const float qy = sR[3] * px + sR[4] * py + sR[5] * pz;
          const float qz = sR[6] * px + sR[7] * py + sR[8] * pz;
          float Jl[3];
          const float res = residual_eval(e, qx + sT[0], qy + sT[1], qz + sT[2], Jl);
          float Jfull[6] = {Jl[0], Jl[1], Jl[2], 0.f, 0.f, 0.f};
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float vx = sJr[k], vy = sJr[3 + k], vz = sJr[6 + k];
            const float cx = py * vz - pz * vy, cy = pz * vx - px * vz, cz = px * vy - py * vx;
            const float mx = -(sRj[0] * cx + sRj[1] * cy + sRj[2] * cz);
            const float my = -(sRj[3] * cx + sRj[4] * cy + sRj[5] * cz);
            const float mz = -(sRj[6] * cx + sRj[7] * cy + sRj[8] * cz);
            Jfull[3 + k] = Jl[0] * mx + Jl[1] * my + Jl[2] * mz;
          }
          const float J[3] = {Jfull[f0], Jfull[f1], Jfull[f2]};
          const float wgt = huber_w(res, delta);
          acc[0] += wgt * J[0] * J[0]; acc[1] += wgt * J[0] * J[1]; acc[2] += wgt * J[0] * J[2];
          acc[3] += wgt * J[1] * J[1]; acc[4] += wgt * J[1] * J[2]; acc[5] += wgt * J[2] * J[2];
          acc[6] += wgt * J[0] * res; acc[7] += wgt * J[1] * res; acc[8] += wgt * J[2] * res;
          acc[9] += 0.5f * huber_rho_f(res, delta);
        }
        reduce_normal<10>(acc, red, s_out);
      };
      if (threadIdx.x == 0 && s_ok) set_point(s_x);
      __syncthreads();
      if (s_ok) {
        pass();
        if (threadIdx.x == 0) {
          lm_load<3>(lm3, s_out, sc3);
          lm3.radius = 1e4;
          lm3.factor = 2.0;
          lm3.done = lm_gsmall<3>(lm3) ? 1 : 0;
        }
        __syncthreads();
        for (int itn = 0; itn < kp.lm_iters; ++itn) {
          if (threadIdx.x == 0) {
            int r = 0;
            if (!lm3.done) {
              double xn = 0.0;
              for (int k = 0; k < 6; ++k) xn += s_x[k] * s_x[k];
              r = lm_propose<3>(lm3, sqrt(xn));
            }
            if (r == 1) {
              for (int k = 0; k < 6; ++k) c_x[k] = s_x[k];
              c_x[f0] += lm3.d[0];
              c_x[f1] += lm3.d[1];
              c_x[f2] += lm3.d[2];
              set_point(c_x);
            }
            s_flag = r;
          }
          __syncthreads();
          const int r = s_flag;
          if (r == 1) {
            pass();
            if (threadIdx.x == 0 && lm_decide<3>(lm3, s_out, sc3))
              for (int k = 0; k < 6; ++k) s_x[k] = c_x[k];
          }
          __syncthreads();
          if (r == 0) break;
        }
      }
    } else {
      for (int itn = 0; itn < kp.gn_iters && s_ok; ++itn) {
        if (threadIdx.x < 32) {
          warp_aa_mats_f(s_x + 3, sR, sRj, sJr);
          if (threadIdx.x >= 18 && threadIdx.x < 21)
            sT[threadIdx.x - 18] = (float)(s_x[threadIdx.x - 18] - s_anchor[threadIdx.x - 18]);
        }
        __syncthreads();
        float acc[9];
  #pragma unroll
        for (int j = 0; j < 9; ++j) acc[j] = 0.f;
        // residuals i == threadIdx.x (mod kGN): the entries this thread built
        for (int i = threadIdx.x; i < nitems; i += blockDim.x) {
          if (i < lo || i >= hi) continue;
          const float* e = d.res_tab + (size_t)kResStride * i;
          if (e[0] == 0.f) continue;
          const float px = e[1], py = e[2], pz = e[3];
          const float qx = sR[0] * px + sR[1] * py + sR[2] * pz;
          const float qy = sR[3] * px + sR[4] * py + sR[5] * pz;
          const float qz = sR[6] * px + sR[7] * py + sR[8] * pz;
          float Jl[3];
          const float res = residual_eval(e, qx + sT[0], qy + sT[1], qz + sT[2], Jl);
          // d lp / d r_k = -Rj (p x Jr[:,k])
          float Jfull[6] = {Jl[0], Jl[1], Jl[2], 0.f, 0.f, 0.f};
  #pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float vx = sJr[k], vy = sJr[3 + k], vz = sJr[6 + k];
            const float cx = py * vz - pz * vy, cy = pz * vx - px * vz, cz = px * vy - py * vx;
            const float mx = -(sRj[0] * cx + sRj[1] * cy + sRj[2] * cz);
            const float my = -(sRj[3] * cx + sRj[4] * cy + sRj[5] * cz);
            const float mz = -(sRj[6] * cx + sRj[7] * cy + sRj[8] * cz);
            Jfull[3 + k] = Jl[0] * mx + Jl[1] * my + Jl[2] * mz;
          }
          const float J[3] = {Jfull[f0], Jfull[f1], Jfull[f2]};
          const float wgt = huber_w(res, delta);
          acc[0] += wgt * J[0] * J[0]; acc[1] += wgt * J[0] * J[1]; acc[2] += wgt * J[0] * J[2];
          acc[3] += wgt * J[1] * J[1]; acc[4] += wgt * J[1] * J[2]; acc[5] += wgt * J[2] * J[2];
          acc[6] += wgt * J[0] * res; acc[7] += wgt * J[1] * res; acc[8] += wgt * J[2] * res;
        }
        reduce_normal<9>(acc, red, s_out);
        if (threadIdx.x == 0) {
          const double Hm[9] = {s_out[0], s_out[1], s_out[2], s_out[1], s_out[3],
                                s_out[4], s_out[2], s_out[4], s_out[5]};
          const double g[3] = {-s_out[6], -s_out[7], -s_out[8]};
          double x[3];
          if (chol_solve(3, Hm, g, x)) {
            s_x[f0] += x[0]; s_x[f1] += x[1]; s_x[f2] += x[2];
          } else {
            s_ok = 0;
          }
        }
        __syncthreads();
      }
    }
    if (step == 0) {
      if (s_ok) { out_tree[0] = s_x[0]; out_tree[1] = s_x[1]; out_tree[2] = s_x[5]; }
      else { out_tree[0] = s_anchor[0]; out_tree[1] = s_anchor[1]; out_tree[2] = rpy[2]; }
    } else {
      if (s_ok) { out_ground[0] = s_x[2]; out_ground[1] = s_x[3]; out_ground[2] = s_x[4]; }
      else { out_ground[0] = s_anchor[2]; out_ground[1] = rpy[0]; out_ground[2] = rpy[1]; }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double aa[3] = {out_ground[1], out_ground[2], out_tree[2]};
    double q[4];
    aa_to_quat(aa, q);
    sloam_se3 o;
    o.q[0] = q[1]; o.q[1] = q[2]; o.q[2] = q[3]; o.q[3] = q[0];
    o.t[0] = out_tree[0]; o.t[1] = out_tree[1]; o.t[2] = out_ground[0];
    const Pose T = pose_from(o);
    pose_store(d.pose_io + 7, T);
    d.cnt->success = 1;
  }
}

// projectModels + matchModels + prevGPlanes_ (first scan: projection by the
// estimate, no matching).  One block per cylinder.
__global__ void __launch_bounds__(kAssocThreads) k_finalize(Dev d, KParams kp, int first,
                                                            int update) {
  __shared__ double sv[kAssocThreads / 32];
  __shared__ int si[kAssocThreads / 32];
  __shared__ float su[kAssocThreads / 32];
  __shared__ AxisPts ax;
  const int nc = d.cnt->n_cyl, np = d.cnt->n_planes;
  if (first) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      for (int j = 0; j < 7; ++j) d.pose_io[7 + j] = d.pose_io[j];
      for (int j = 0; j < 7; ++j) d.pose_io[14 + j] = (j == 3) ? 1.0 : 0.0;
      d.cnt->status = SLOAM_OK;
      d.cnt->success = 1;
      d.cnt->n_tm = d.cnt->n_pm = 0;
      d.cnt->tree_check = d.cnt->ground_check = 0;
    }
  } else if (d.cnt->status == SLOAM_ERR_NO_MODELS) {
    return;
  }
  __shared__ Pose sT;
  if (threadIdx.x == 0) sT = pose_at(d.pose_io + (first ? 0 : 7));  // FP64 once per block
  __syncthreads();
  const Pose& T = sT;
  if (blockIdx.x == 0) {
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
      PlaneD P = d.planes[p];
      const d3 n2 = rot3(T.R, mk3(P.plane[0], P.plane[1], P.plane[2]));
      const double d2 = P.plane[3] - dot3(T.t, n2);
      const d3 c2 = xform(T, mk3(P.centroid[0], P.centroid[1], P.centroid[2]));
      P.plane[0] = n2.x; P.plane[1] = n2.y; P.plane[2] = n2.z; P.plane[3] = d2;
      P.centroid[0] = c2.x; P.centroid[1] = c2.y; P.centroid[2] = c2.z;
      d.planes[p] = P;
      if (update) d.prev_planes[p] = P;
    }
    if (threadIdx.x == 0 && update) d.cnt->n_prev = np;
  }
  for (int c = blockIdx.x; c < nc; c += gridDim.x) {
    if (threadIdx.x == 0) {
      CylD C = d.cyls[c];
      d3 root = mk3(C.root[0], C.root[1], C.root[2]), ray = mk3(C.ray[0], C.ray[1], C.ray[2]);
      cyl_project(T, root, ray);
      set_axis_pts(&ax, root, ray);
      C.root[0] = root.x; C.root[1] = root.y; C.root[2] = root.z;
      C.ray[0] = ray.x; C.ray[1] = ray.y; C.ray[2] = ray.z;
      d.cyls[c] = C;
    }
    __syncthreads();
    int out = -1;
    if (!first) {
      double bd;
      int bi;
      map_argmin(d, &ax, kp.tree_match_thresh + 100, bd, bi, sv, si, su);
      out = (d.in->n_map > 0 && bd < kp.add_new_tree_thresh) ? bi : -1;
    }
    if (threadIdx.x == 0) d.match_out[c] = out;
    __syncthreads();
  }
}

}  // namespace

// The pose solve alone over the last keyframe's residual table, for timing
// (it reads the estimate and writes the result into separate slots).
int launch_pose_kernel(const Dev& d, const KParams& kp, cudaStream_t st) {
  if (kp.pose_lm)
    k_gn<true><<<1, kGN, 0, st>>>(d, kp);
  else
    k_gn<false><<<1, kGN, 0, st>>>(d, kp);
  return 1;
}

// The submap's per-cylinder prep (needs the map input only).
int launch_map_prep(const Dev& d, cudaStream_t st) {
  k_map_prep<<<16, 256, 0, st>>>(d);
  return 1;
}

int launch_run(const Dev& d, const KParams& kp, bool first_scan, bool update, cudaStream_t st,
               bool map_prepped) {
  if (first_scan) {
    k_finalize<<<64, kAssocThreads, 0, st>>>(d, kp, 1, update ? 1 : 0);
    return 1;
  }
  int n = 3;
  if (!map_prepped) {
    k_map_prep<<<16, 256, 0, st>>>(d);
    ++n;
  }
  k_assoc<<<96, kAssocThreads, 0, st>>>(d, kp);
  if (kp.pose_lm)
    k_gn<true><<<1, kGN, 0, st>>>(d, kp);
  else
    k_gn<false><<<1, kGN, 0, st>>>(d, kp);
  k_finalize<<<64, kAssocThreads, 0, st>>>(d, kp, 0, update ? 1 : 0);
  return n;
}

}  // namespace sg
