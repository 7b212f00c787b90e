// models.cu — a6-a8: sloam::computeModels (sloam.cpp:388-436).
//
// a7 binGroundPoints (sloam.cpp:330-386) + Plane (plane.cpp:3-17, 96-128) +
//    the angle/height gates (sloam.cpp:394-412): per-point bins from exact
//    float boundary tables (theta is the correctly rounded float atan2, same
//    fast/slow scheme as the projection), one block per bin selects the
//    lowest int(n / retainNum) points by (z, index) with a shared-memory
//    bitonic sort (radix select first when a bin exceeds the staging size),
//    float centroid in that order, FP64 scatter + Jacobi normal (with the
//    sign Eigen's JacobiSVD gives it: eigen_normal_opposes).
// a8 landmark -> nearest plane (sloam.cpp:418-431), and
// a6 Cylinder (cylinder.cpp:3-173): one warp per landmark runs the
//    vertex-line RANSAC (Philox hypotheses, PCL's sequential stopping rule),
//    the PCL-style PCA refit, the radius median and the gates; the optional
//    point-level cylinder RANSAC spreads each tree's hypotheses over blocks
//    that stage the tree's projected points in shared memory, then one block
//    per tree runs the least-squares refinement (FP32 sums, FP64 5x5 solve).
#include <cfloat>
#include <climits>

#include "internal.h"
#include "proposal.cuh"
#include "scan_util.cuh"
#include "cylinder.cuh"

namespace sg {

KParams make_kparams(const sloam_params& p) {
  KParams k{};
  k.cc_iter_limit = kCCIterLimitDefault;
  const float fov_up = (float)(p.fov_up_deg / 180.0 * 3.14159265358979323846);
  const float fov_down = (float)(p.fov_down_deg / 180.0 * 3.14159265358979323846);
  k.fov_down_abs = fov_down < 0 ? -fov_down : fov_down;
  k.fov = k.fov_down_abs + (fov_up < 0 ? -fov_up : fov_up);
  k.img_w = p.img_w;
  k.img_h = p.img_h;
  k.do_destagger = p.do_destagger;
  k.cc_thr = p.cc_dist_threshold;
  k.min_cluster = p.trellis_min_cluster;
  k.min_beam = p.trellis_min_beam_points;
  k.min_vertices = p.trellis_min_vertices;
  k.max_vertices = p.trellis_max_vertices;
  k.max_d_centroid = p.max_dist_to_centroid;
  k.Rb = p.ground_radii_bins;
  k.Tb = p.ground_theta_bins;
  k.retain_num = 1 / p.ground_retain_thresh;
  k.G = p.num_ground_features;
  k.F = p.features_per_tree;
  k.max_lidar_dist = p.max_lidar_dist;
  k.min_tree_height_sq = p.min_tree_height_sq;
  k.root_plane_max_dist = p.root_plane_max_dist;
  k.max_tree_radius = p.max_tree_radius;
  k.max_axis_theta = p.max_axis_theta;
  k.default_tree_radius = p.default_tree_radius;
  k.line_thr = p.line_ransac_thresh;
  k.line_max_iter = p.line_ransac_max_iter;
  k.line_prob = p.line_ransac_probability;
  k.seed = p.seed;
  k.cyl_mode = p.cyl_mode;
  k.prop_S = p.prop_samples;
  k.prop_ratio = p.prop_min_inlier_ratio;
  k.K = p.cyl_hypotheses;
  k.ls_iters = p.cyl_ls_iters;
  k.tau = p.cyl_inlier_thresh;
  k.max_hyp_r = p.cyl_max_hyp_radius;
  k.tree_match_thresh = p.tree_match_thresh;
  k.plane_match_thresh = p.plane_match_thresh;
  k.add_new_tree_thresh = p.add_new_tree_thresh_dist;
  k.min_tree_models = p.min_tree_models;
  k.min_ground_models = p.min_ground_models;
  k.min_planes = p.min_planes;
  k.two_step = p.two_step_optim;
  k.gn_iters = p.gn_iters;
  k.pose_lm = p.pose_solver == 1 ? 1 : 0;
  k.lm_iters = p.lm_max_iters;
  k.huber = p.huber_delta;
  k.q_chunk = p.cyl_chunk_points;
  k.q_tile = p.cyl_hyp_tile;
  // persistent blocks: the given count, else 76 (half the SMs; with 32
  // keyframes in flight fewer, longer-lived blocks did best)
  k.q_blocks = p.cyl_queue_blocks > 0 ? p.cyl_queue_blocks : 76;
  return k;
}

namespace {

// ============================================================ ground bins
__device__ __forceinline__ int bin_from_table(const float* __restrict__ tab, float v, int nb) {
  int k = 0;
  while (k < nb - 1 && v >= tab[k + 1]) ++k;
  return k;
}

__device__ __forceinline__ uint32_t zkey(float z) {
  if (z == 0.0f) z = 0.0f;  // -0 == +0
  const uint32_t u = __float_as_uint(z);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Bin counts are combined per warp (match on the bin) and per block (shared
// histogram) before one global atomicAdd per bin and block: the ground list
// falls into a few dozen bins, so plain global atomics serialise.
constexpr int kMaxBins = 4096;

__device__ __forceinline__ int warp_bin_add(int* hist, int bin, int lane) {
  const unsigned peers = __match_any_sync(0xffffffffu, bin);
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (bin >= 0 && lane == leader) base = atomicAdd(hist + bin, __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// The ground binning kernels take kGbinPer points per thread (slices of 256
// in point order), all of their loads issued before use.
constexpr int kGbinPer = 4;
constexpr int kGbinSpan = 256 * kGbinPer;

__global__ void __launch_bounds__(256, 5) k_gbin(Dev d, KParams kp) {
  __shared__ int hist[kMaxBins];
  const GroundView ground = ground_view(d.in);
  const int n = d.cnt->n_ground;
  if (blockIdx.x * kGbinSpan >= n) return;
  const int lane = threadIdx.x & 31;
  for (int b = threadIdx.x; b < d.n_bins; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  int slow = 0;
  for (int i0 = blockIdx.x * kGbinSpan; i0 < n; i0 += gridDim.x * kGbinSpan) {
    float4 pts[kGbinPer];
#pragma unroll
    for (int u = 0; u < kGbinPer; ++u) {
      const int i = i0 + u * 256 + threadIdx.x;
      if (i < n) pts[u] = ground[i];
    }
#pragma unroll
    for (int u = 0; u < kGbinPer; ++u) {
      const int i = i0 + u * 256 + threadIdx.x;
      int bin = -1;
      if (i < n) {
        const float4 p = pts[u];
        const float dx = fsub(0.0f, p.x), dy = fsub(0.0f, p.y);
        const float r = fsqrt(fadd(fmul(dx, dx), fmul(dy, dy)));
        if (r >= d.r_lo && r <= d.r_hi) {
          const float y = fsub(p.y, 0.0f), x = fsub(p.x, 0.0f);
          float th = atan2f(y, x);
          int tb;
          bool need = !(isfinite(x) && isfinite(y)) || x == 0.0f || y == 0.0f;
          if (!need) {
            const float m = fmaxf(fabsf(th) * 1.2e-6f, 1e-30f);
            tb = bin_from_table(d.tb_tab, th - m, kp.Tb);
            need = tb != bin_from_table(d.tb_tab, th + m, kp.Tb);
          }
          if (need) {
            th = (float)atan2((double)y, (double)x);
            tb = bin_from_table(d.tb_tab, th, kp.Tb);
            ++slow;
          }
          const int rb = bin_from_table(d.rb_tab, r, kp.Rb);
          bin = rb * kp.Tb + tb;
        }
        d.bin_of[i] = bin;
      }
      warp_bin_add(hist, bin, lane);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < d.n_bins; b += blockDim.x)
    if (hist[b]) atomicAdd(d.bin_cnt + b, hist[b]);
  slow = warp_sumi(slow);
  if (lane == 0 && slow) atomicAdd(&d.cnt->n_slow_theta, slow);
}

__global__ void __launch_bounds__(1024) k_gbin_scan(Dev d) {
  __shared__ int sm[33];
  int base = 0;
  for (int b0 = 0; b0 < d.n_bins; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    const int v = b < d.n_bins ? d.bin_cnt[b] : 0;
    int total;
    const int ex = block_excl_scan(v, sm, &total);
    if (b < d.n_bins) {
      d.bin_off[b] = base + ex;
      d.bin_cnt[b] = base + ex;  // becomes the scatter cursor
    }
    base += total;
  }
  if (threadIdx.x == 0) d.bin_off[d.n_bins] = base;
}

// Scatter of (z key, index) into the bins; the order inside a bin is free
// (k_plane orders the keys it retains).
__global__ void __launch_bounds__(256) k_gbin_scatter(Dev d) {
  __shared__ int hist[kMaxBins];
  const GroundView ground = ground_view(d.in);
  const int n = d.cnt->n_ground;
  if (blockIdx.x * kGbinSpan >= n) return;
  const int lane = threadIdx.x & 31;
  for (int i0 = blockIdx.x * kGbinSpan; i0 < n; i0 += gridDim.x * kGbinSpan) {
    int bin[kGbinPer], local[kGbinPer];
    float z[kGbinPer];
#pragma unroll
    for (int u = 0; u < kGbinPer; ++u) {
      const int i = i0 + u * 256 + threadIdx.x;
      bin[u] = -1;
      z[u] = 0.0f;
      if (i < n) {
        bin[u] = d.bin_of[i];
        z[u] = ground[i].z;
      }
    }
    for (int b = threadIdx.x; b < d.n_bins; b += blockDim.x) hist[b] = 0;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kGbinPer; ++u) local[u] = warp_bin_add(hist, bin[u], lane);
    __syncthreads();
    for (int b = threadIdx.x; b < d.n_bins; b += blockDim.x)
      if (hist[b]) hist[b] = atomicAdd(d.bin_cnt + b, hist[b]);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kGbinPer; ++u) {
      const int i = i0 + u * 256 + threadIdx.x;
      if (bin[u] >= 0)
        d.bin_keys[hist[bin[u]] + local[u]] =
            ((unsigned long long)zkey(z[u]) << 32) | (uint32_t)i;
    }
    __syncthreads();
  }
}

// ------------------------------------------------ Eigen euler gate (FP64)
// Quaternion::setFromTwoVectors + toRotationMatrix + eulerAngles(0,1,2),
// restated (Eigen 3.3); returns the three angles.
__device__ void euler_two_vectors(d3 a, d3 b, double* ang) {
  d3 v0 = scl3(1.0 / norm3(a), a), v1 = scl3(1.0 / norm3(b), b);
  double c = dot3(v1, v0);
  double qx, qy, qz, qw;
  if (c < -1.0 + 1e-12) {
    c = fmax(c, -1.0);
    d3 axis = fabs(v0.x) < 0.9 ? cross3(v0, mk3(1, 0, 0)) : cross3(v0, mk3(0, 1, 0));
    axis = scl3(1.0 / norm3(axis), axis);
    const double w2 = (1.0 + c) * 0.5;
    qw = sqrt(w2);
    const double s = sqrt(1.0 - w2);
    qx = axis.x * s; qy = axis.y * s; qz = axis.z * s;
  } else {
    const d3 axis = cross3(v0, v1);
    const double s = sqrt((1.0 + c) * 2.0), invs = 1.0 / s;
    qx = axis.x * invs; qy = axis.y * invs; qz = axis.z * invs;
    qw = s * 0.5;
  }
  const double tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
  const double twx = tx * qw, twy = ty * qw, twz = tz * qw;
  const double txx = tx * qx, txy = ty * qx, txz = tz * qx;
  const double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  const double M00 = 1 - (tyy + tzz), M01 = txy - twz, M02 = txz + twy;
  const double M10 = txy + twz, M11 = 1 - (txx + tzz), M12 = tyz - twx;
  const double M20 = txz - twy, M21 = tyz + twx, M22 = 1 - (txx + tyy);
  double r0 = atan2(M12, M22);
  const double c2 = hypot(M00, M01);
  double r1;
  if (r0 > 0) {
    r0 -= 3.14159265358979323846;
    r1 = atan2(-M02, -c2);
  } else {
    r1 = atan2(-M02, c2);
  }
  const double s1 = sin(r0), c1 = cos(r0);
  const double r2 = atan2(s1 * M20 - c1 * M10, c1 * M11 - s1 * M21);
  ang[0] = -r0; ang[1] = -r1; ang[2] = -r2;
}

constexpr int kBinCap = 4096;   // keys of one bin staged in shared memory
constexpr int kPlaneThreads = 512;
constexpr int kPlaneStage = kBinCap / 2;  // retained points that fit over the keys as float4
constexpr int kSelCap = 256;              // retained keys sorted apart from the bin
static_assert(kPlaneStage % kPlaneThreads == 0, "whole passes");
constexpr int kScatterWarps = 4;

__device__ void bitonic_sort(unsigned long long* a, int n2) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const unsigned long long x = a[i], y = a[l];
          if ((x > y) == up) { a[i] = y; a[l] = x; }
        }
      }
      __syncthreads();
    }
  }
}

// The sign Eigen's JacobiSVD gives the plane normal (the third column of U
// of the 3 x n centred matrix A, plane.cpp:113-115; Eigen 3.3.7): true when
// it points against `nrm`.  Same steps as Eigen, in a form that needs only
// the Gram matrix S = A A^T (6 entries, upper triangle row by row) and the
// first three centred points a[0..2] (rows of A^T):
//  - the column-pivoted Householder QR of A^T (ColPivHouseholderQR with its
//    norm downdates), FP64: a reflection's inner products with the columns
//    follow from S and the rows it leaves in place, S shrinks by the R row
//    each step produces, and the pivot (c0) of step k is row k of the
//    reflected column, so only the first three rows are carried;
//  - the two-sided Jacobi sweep on W = R^T (real_2x2_jacobi_svd, makeJacobi),
//    the positive-diagonal fix of U and the descending sort, FP32: every
//    right rotation has a positive cosine, so the sign of u3 = A v3 / s3 does
//    not depend on where the sweep stops.
// Only the sign is used; the normal itself comes from the scatter's Jacobi.
__device__ bool eigen_normal_opposes(const double* S6, const double a[3][3], int n, d3 nrm) {
  double S[3][3] = {{S6[0], S6[1], S6[2]}, {S6[1], S6[3], S6[4]}, {S6[2], S6[4], S6[5]}};
  double row[3][3];  // rows 0..2 of the working matrix (the first three points)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) row[i][j] = a[i][j];
  double R[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double nu[3], nd[3];
  for (int j = 0; j < 3; ++j) nd[j] = nu[j] = sqrt(S[j][j]);
  int trans[3];
  const double kMinD = 2.2250738585072014e-308, kEpsD = 2.220446049250313e-16;
  for (int k = 0; k < 3; ++k) {
    int big = k;
    for (int j = k + 1; j < 3; ++j)
      if (nu[j] > nu[big]) big = j;
    trans[k] = big;
    if (big != k) {
      for (int i = 0; i < 3; ++i) {  // the whole column: S, the rows, R above
        const double t = S[i][k]; S[i][k] = S[i][big]; S[i][big] = t;
      }
      for (int i = 0; i < 3; ++i) {
        const double t = S[k][i]; S[k][i] = S[big][i]; S[big][i] = t;
      }
      for (int i = 0; i < 3; ++i) {
        const double t = row[i][k]; row[i][k] = row[i][big]; row[i][big] = t;
      }
      for (int i = 0; i < k; ++i) {
        const double t = R[i][k]; R[i][k] = R[i][big]; R[i][big] = t;
      }
      double t = nu[k]; nu[k] = nu[big]; nu[big] = t;
      t = nd[k]; nd[k] = nd[big]; nd[big] = t;
    }
    // S now holds the Gram matrix of rows k.. of the working columns
    const double c0 = row[k][k];
    const double tail = (k == 2 && n == 3) ? 0.0 : S[k][k] - c0 * c0;
    double tau = 0.0, beta = c0, den = 1.0;
    if (tail > kMinD) {
      beta = sqrt(S[k][k]);
      if (c0 >= 0.0) beta = -beta;
      den = c0 - beta;
      tau = (beta - c0) / beta;
    }
    R[k][k] = beta;
    double rk[3] = {0, 0, 0};
    for (int j = k + 1; j < 3; ++j) {
      if (tau != 0.0) {
        // v^T x over rows k..: x_k + (S_kj - c0 x_k) / (c0 - beta)
        const double vtx = row[k][j] + (S[k][j] - c0 * row[k][j]) / den;
        rk[j] = row[k][j] - tau * vtx;
        for (int i = k + 1; i < 3; ++i) row[i][j] -= tau * (row[i][k] / den) * vtx;
      } else {
        rk[j] = row[k][j];
      }
      R[k][j] = rk[j];
    }
    for (int j = k + 1; j < 3; ++j)
      for (int l = k + 1; l < 3; ++l) S[j][l] -= rk[j] * rk[l];
    for (int j = k + 1; j < 3; ++j) {
      if (nu[j] != 0.0) {
        double t = fabs(rk[j]) / nu[j];
        t = (1.0 + t) * (1.0 - t);
        t = t < 0.0 ? 0.0 : t;
        const double r = nu[j] / nd[j];
        if (t * r * r <= sqrt(kEpsD)) {
          nd[j] = nu[j] = sqrt(S[j][j] > 0.0 ? S[j][j] : 0.0);
        } else {
          nu[j] *= sqrt(t);
        }
      }
    }
  }
  int idx[3] = {0, 1, 2};
  for (int k = 0; k < 3; ++k) {
    const int t = idx[k]; idx[k] = idx[trans[k]]; idx[trans[k]] = t;
  }
  // the Jacobi sweep on W = R^T, U from the permutation (FP32)
  float W[3][3], U[3][3];
  float scale = 0.f;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) scale = fmaxf(scale, fabsf((float)R[i][j]));
  if (!(scale > 0.f)) return false;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      W[i][j] = j <= i ? (float)(R[j][i] / (double)scale) : 0.f;
      U[i][j] = 0.f;
    }
  for (int i = 0; i < 3; ++i) U[idx[i]][i] = 1.f;
  float maxd = fmaxf(fabsf(W[0][0]), fmaxf(fabsf(W[1][1]), fabsf(W[2][2])));
  bool finished = false;
  for (int sweep = 0; !finished && sweep < 30; ++sweep) {
    finished = true;
    for (int p = 1; p < 3; ++p) {
      for (int q = 0; q < p; ++q) {
        const float thr = fmaxf(FLT_MIN, 2.f * FLT_EPSILON * maxd);
        if (!(fabsf(W[p][q]) > thr || fabsf(W[q][p]) > thr)) continue;
        finished = false;
        float m00 = W[p][p], m01 = W[p][q], m10 = W[q][p], m11 = W[q][q];
        const float t = m00 + m11, dd = m10 - m01;
        float c1 = 1.f, s1 = 0.f;
        if (!(fabsf(dd) < FLT_MIN)) {
          const float u = t / dd, tmp = sqrtf(1.f + u * u);
          s1 = 1.f / tmp;
          c1 = u / tmp;
        }
        const float x0 = m00, x1 = m01;
        m00 = c1 * x0 + s1 * m10;
        m01 = c1 * x1 + s1 * m11;
        m11 = -s1 * x1 + c1 * m11;
        float cr = 1.f, sr = 0.f;
        const float deno = 2.f * fabsf(m01);
        if (!(deno < FLT_MIN)) {
          const float tau = (m00 - m11) / deno, w = sqrtf(tau * tau + 1.f);
          const float tt = tau > 0.f ? 1.f / (tau + w) : 1.f / (tau - w);
          const float sign_t = tt > 0.f ? 1.f : -1.f;
          const float nn = 1.f / sqrtf(tt * tt + 1.f);
          sr = -sign_t * (m01 > 0.f ? 1.f : -1.f) * fabsf(tt) * nn;
          cr = nn;
        }
        const float lc = c1 * cr + s1 * sr, ls = -c1 * sr + s1 * cr;
        for (int i = 0; i < 3; ++i) {  // W rows p, q by j_left
          const float x = W[p][i], y = W[q][i];
          W[p][i] = lc * x + ls * y;
          W[q][i] = -ls * x + lc * y;
        }
        for (int i = 0; i < 3; ++i) {  // U columns p, q by j_left^T
          const float x = U[i][p], y = U[i][q];
          U[i][p] = lc * x + ls * y;
          U[i][q] = -ls * x + lc * y;
        }
        for (int i = 0; i < 3; ++i) {  // W columns p, q by j_right
          const float x = W[i][p], y = W[i][q];
          W[i][p] = cr * x - sr * y;
          W[i][q] = sr * x + cr * y;
        }
        maxd = fmaxf(maxd, fmaxf(fabsf(W[p][p]), fabsf(W[q][q])));
      }
    }
  }
  float sv[3];
  for (int i = 0; i < 3; ++i) {
    sv[i] = fabsf(W[i][i]);
    if (W[i][i] < 0.f)
      for (int r = 0; r < 3; ++r) U[r][i] = -U[r][i];
  }
  // the descending sort (first maximum moved forward); its last column
  int ord[3] = {0, 1, 2};
  for (int i = 0; i < 3; ++i) {
    int pos = i;
    for (int j = i + 1; j < 3; ++j)
      if (sv[j] > sv[pos]) pos = j;
    if (pos != i) {
      const float t = sv[i]; sv[i] = sv[pos]; sv[pos] = t;
      const int o = ord[i]; ord[i] = ord[pos]; ord[pos] = o;
    }
  }
  const int last = ord[2];
  const double dot = nrm.x * U[0][last] + nrm.y * U[1][last] + nrm.z * U[2][last];
  return dot < 0.0;
}

// Plane::computeModel (plane.cpp:96-128) over points at(0..n-1) by the whole
// block: float centroid accumulated sequentially in feature order
// (utils.h:14-28), FP64 scatter about it, normal = eigenvector of the
// smallest eigenvalue (FP32 Jacobi), with the sign Eigen's JacobiSVD gives
// it (eigen_normal_opposes), d = -n.c.  `cen` (3 floats) and `red` (6 * 32
// doubles) are shared memory; the model lands in `out` of thread 0.
template <typename At>
__device__ void fit_plane_block(At at, int n, float* cen, double* red, PlaneD& out) {
  if (threadIdx.x == 0) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int i = 0; i < n; ++i) {
      const float4 p = at(i);
      sx = fadd(sx, p.x);
      sy = fadd(sy, p.y);
      sz = fadd(sz, p.z);
    }
    cen[0] = (float)((double)sx / (double)n);
    cen[1] = (float)((double)sy / (double)n);
    cen[2] = (float)((double)sz / (double)n);
  }
  __syncthreads();
  // FP64 scatter by the first kScatterWarps warps only: every FP64 warp
  // instruction and warp reduction costs the same pipe time whatever the
  // number of points, so fewer warps cost less
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (w < kScatterWarps) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += 32 * kScatterWarps) {
      const float4 p = at(i);
      const double a0 = (double)fsub(p.x, cen[0]), a1 = (double)fsub(p.y, cen[1]),
                   a2 = (double)fsub(p.z, cen[2]);
      s[0] += a0 * a0; s[1] += a0 * a1; s[2] += a0 * a2;
      s[3] += a1 * a1; s[4] += a1 * a2; s[5] += a2 * a2;
    }
    for (int j = 0; j < 6; ++j) {
      const double v = warp_sumd(s[j]);
      if (lane == 0) red[j * 32 + w] = v;
    }
  }
  __syncthreads();
  // sum j over the warps by lane j of warp 0 (the order of one thread's sum)
  if (w == 0) {
    if (lane < 6) {
      double t = 0;
      for (int q = 0; q < kScatterWarps; ++q) t += red[lane * 32 + q];
      red[lane * 32 + 31] = t;  // slot 31: at most 16 warps write partials
    }
    __syncwarp();
  }
  if (threadIdx.x == 0) {
    double S6[6];
    for (int j = 0; j < 6; ++j) S6[j] = red[j * 32 + 31];
    const float S[9] = {(float)S6[0], (float)S6[1], (float)S6[2], (float)S6[1], (float)S6[3],
                        (float)S6[4], (float)S6[2], (float)S6[4], (float)S6[5]};
    float ev[3], V[9];
    jacobi3f(S, ev, V);
    d3 nrm = mk3(V[0], V[3], V[6]);
    double a[3][3];
    for (int i = 0; i < 3; ++i) {
      const float4 p = at(i);
      a[i][0] = (double)fsub(p.x, cen[0]);
      a[i][1] = (double)fsub(p.y, cen[1]);
      a[i][2] = (double)fsub(p.z, cen[2]);
    }
    if (eigen_normal_opposes(S6, a, n, nrm)) nrm = scl3(-1.0, nrm);
    const double dd = -(nrm.x * cen[0] + nrm.y * cen[1] + nrm.z * cen[2]);
    out.plane[0] = nrm.x; out.plane[1] = nrm.y; out.plane[2] = nrm.z; out.plane[3] = dd;
    out.centroid[0] = cen[0]; out.centroid[1] = cen[1]; out.centroid[2] = cen[2];
  }
}

// Block-wide radix select: the k-th smallest (k >= 1) of n distinct 64-bit
// keys at(0..n-1), 8 bits at a time from the top; it stops once the chosen
// digit prefix holds a single key and finds that key.  Every thread calls
// it and gets the key.  The keys of a bin share their high bytes (nearby
// z), so histogram increments are combined per warp and digit.
struct SelState {
  unsigned long long prefix, found;
  int k, unique;
};
template <typename At>
__device__ unsigned long long radix_select(At at, int n, int k, unsigned* hist, SelState* ss) {
  if (threadIdx.x == 0) {
    ss->prefix = 0;
    ss->k = k;
    ss->unique = 0;
  }
  __syncthreads();
  int shift = 56;
  for (; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const unsigned long long pre = ss->prefix;
    const unsigned long long hmask = shift == 56 ? 0ull : (~0ull << (shift + 8));
    for (int i0 = 0; i0 < n; i0 += blockDim.x) {
      const int i = i0 + threadIdx.x;
      int dg = -1;
      if (i < n) {
        const unsigned long long v = at(i);
        if ((v & hmask) == pre) dg = (int)((v >> shift) & 255u);
      }
      const unsigned peers = __match_any_sync(0xffffffffu, dg);
      if (dg >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1)
        atomicAdd(hist + dg, (unsigned)__popc(peers));
    }
    __syncthreads();
    // the digit where the running count reaches k: warp 0, 8 bins a lane, a
    // scan of the lane sums, then the owning lane's 8 bins
    if (threadIdx.x < 32) {
      const int ln = threadIdx.x;
      unsigned sum = 0;
      for (int j = 0; j < 8; ++j) sum += hist[ln * 8 + j];
      unsigned incl = sum;
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (ln >= o) incl += y;
      }
      const int rem = ss->k;
      if (rem > (int)(incl - sum) && rem <= (int)incl) {
        int r = rem - (int)(incl - sum), dg = ln * 8;
        for (int j = 0; j < 8; ++j, ++dg) {
          const int cj = (int)hist[dg];
          if (r <= cj) break;
          r -= cj;
        }
        ss->prefix = pre | ((unsigned long long)dg << shift);
        ss->k = r;
        ss->unique = hist[dg] == 1u;
      }
    }
    __syncthreads();
    if (ss->unique) break;  // block-uniform
  }
  if (shift < 0) return ss->prefix;  // every byte chosen: the key itself
  const unsigned long long m = ~0ull << shift, pre = ss->prefix;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long v = at(i);
    if ((v & m) == pre) ss->found = v;  // exactly one key
  }
  __syncthreads();
  return ss->found;
}
// The keys <= T of at(0..n-1) into out[0 ..), in any order; one counter
// update per warp.
template <typename At>
__device__ void take_le(At at, int n, unsigned long long T, unsigned long long* out, int* cnt) {
  if (threadIdx.x == 0) *cnt = 0;
  __syncthreads();
  for (int i0 = 0; i0 < n; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    unsigned long long v = 0;
    bool take = false;
    if (i < n) {
      v = at(i);
      take = v <= T;
    }
    const unsigned b = __ballot_sync(0xffffffffu, take);
    int base = 0;
    if ((threadIdx.x & 31) == 0 && b) base = atomicAdd(cnt, __popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (take) out[base + __popc(b & ((1u << (threadIdx.x & 31)) - 1u))] = v;
  }
  __syncthreads();
}

// One block per bin: retained points, plane model, gates, features.
__global__ void __launch_bounds__(kPlaneThreads, 3) k_plane(Dev d, KParams kp) {
  __shared__ unsigned long long keys[kBinCap];
  __shared__ unsigned int hist[256];
  __shared__ double red[6 * 32];
  __shared__ float cen[3];
  __shared__ unsigned long long sel[kSelCap];
  __shared__ SelState ss;
  __shared__ int s_cnt;
  const GroundView ground = ground_view(d.in);
  const int b = blockIdx.x;
  if (b >= d.n_bins) return;
  const int off = d.bin_off[b], n = d.bin_off[b + 1] - off;
  const unsigned long long* src = d.bin_keys + off;
  PlaneD out{};
  out.bin = b;
  out.valid = 0;
  const bool retain = n > 0 && kp.retain_num < (double)n;
  const int k = n == 0 ? 0 : (retain ? (int)((double)n / kp.retain_num) : n);
  // the retained set sorted by (z, index); without retention, by index
  int kk = k;
  if (n > 0 && k > 0) {
    if (n <= kBinCap && retain && k <= kSelCap) {
      // the k lowest of the staged keys: select the k-th, take the keys at
      // or below it, sort those k (distinct keys: the same set and order as
      // sorting all n)
      for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = src[i];
      __syncthreads();
      auto at = [&](int i) { return keys[i]; };
      const unsigned long long T = radix_select(at, n, k, hist, &ss);
      take_le(at, n, T, sel, &s_cnt);
      int m2 = 1;
      while (m2 < k) m2 <<= 1;
      for (int i = k + threadIdx.x; i < m2; i += blockDim.x) sel[i] = ~0ull;
      __syncthreads();
      bitonic_sort(sel, m2);
      for (int i = threadIdx.x; i < k; i += blockDim.x) keys[i] = sel[i];
    } else if (n <= kBinCap) {
      int n2 = 1;
      while (n2 < n) n2 <<= 1;
      for (int i = threadIdx.x; i < n2; i += blockDim.x)
        keys[i] = i < n ? (retain ? src[i] : (src[i] & 0xffffffffull)) : ~0ull;
      __syncthreads();
      bitonic_sort(keys, n2);
    } else if (k > kBinCap) {
      if (threadIdx.x == 0) atomicOr(&d.cnt->overflow, 8);
      kk = 0;
    } else {
      // the same from global memory, the k keys sorted in the key array
      auto at = [&](int i) { return src[i]; };
      const unsigned long long T = radix_select(at, n, k, hist, &ss);
      take_le(at, n, T, keys, &s_cnt);
      int n2 = 1;
      while (n2 < k) n2 <<= 1;
      for (int i = k + threadIdx.x; i < n2; i += blockDim.x) keys[i] = ~0ull;
      __syncthreads();
      bitonic_sort(keys, n2);
    }
  }
  __syncthreads();
  const bool enough = kk > 0 && kk >= kp.G && kk >= 3;
  if (enough && kk <= kPlaneStage) {
    // the retained points gathered once into shared memory (over the key
    // array: every key is read into registers before the first point is
    // written), so that the sequential centroid, the scatter and the
    // features read shared memory instead of two dependent global loads
    float4* sp = reinterpret_cast<float4*>(keys);
    uint32_t gi[kPlaneStage / kPlaneThreads];
#pragma unroll
    for (int q = 0; q < kPlaneStage / kPlaneThreads; ++q) {
      const int i = threadIdx.x + q * kPlaneThreads;
      gi[q] = i < kk ? (uint32_t)keys[i] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPlaneStage / kPlaneThreads; ++q) {
      const int i = threadIdx.x + q * kPlaneThreads;
      if (i < kk) sp[i] = ground[gi[q]];
    }
    __syncthreads();
    fit_plane_block([&](int i) { return sp[i]; }, kk, cen, red, out);
    if (threadIdx.x == 0) {
      out.valid = 1;  // fitted; the gates follow in k_plane_compact
      d.plane_all[b] = out;
    }
    for (int i = threadIdx.x; i < kp.G; i += blockDim.x)
      d.plane_feat_all[(size_t)b * kp.G + i] = sp[i];
  } else if (enough) {
    fit_plane_block([&](int i) { return ground[(uint32_t)keys[i]]; }, kk, cen, red, out);
    if (threadIdx.x == 0) {
      out.valid = 1;
      d.plane_all[b] = out;
    }
    for (int i = threadIdx.x; i < kp.G; i += blockDim.x)
      d.plane_feat_all[(size_t)b * kp.G + i] = ground[(uint32_t)keys[i]];
  } else if (threadIdx.x == 0) {
    d.plane_all[b] = out;
  }
}

// Plane(points, params) (plane.cpp:3-17) over the input block's ground
// view: the model of all n points; valid iff n >= numGroundFeatures; the
// features are the first numGroundFeatures points.  Result in plane_all[0],
// plane_feat_all[0 .. G).
__global__ void __launch_bounds__(kPlaneThreads) k_plane_points(Dev d, KParams kp, int n) {
  __shared__ double red[6 * 32];
  __shared__ float cen[3];
  const float4* __restrict__ pts = d.in->ground;
  PlaneD out{};
  out.bin = -1;
  out.valid = 0;
  if (n > 0 && n >= kp.G) {
    fit_plane_block([&](int i) { return pts[i]; }, n, cen, red, out);
    if (threadIdx.x == 0) {
      out.valid = 1;
      d.plane_all[0] = out;
    }
    for (int i = threadIdx.x; i < kp.G; i += blockDim.x) d.plane_feat_all[i] = pts[i];
  } else if (threadIdx.x == 0) {
    d.plane_all[0] = out;
  }
}

// Gates of a fitted bin plane (sloam.cpp:394-408): the normal in the map
// frame (R n) within 0.1 rad of +-z by its Euler angles, and the centroid
// below the sensor.  FP64, one bin per thread.
// euler_two_vectors((0, 0, 1), b) in FP32 with the same steps (CUDA's float
// atan2, hypot, sin, cos): angles within about 1e-6 rad of the FP64 ones.
// Returns false when the gate's decision could differ from the FP64 one: b
// nearly opposite to z (the FP64 path takes its other formula), the first
// angle within `eps` of 0 or of +-pi (its branch and wrap), or an angle
// within `eps` of a gate threshold (0.1, pi - 0.1).
__device__ bool euler_z_to_f(d3 b, float eps, float* ang) {
  const float nb = sqrtf((float)b.x * (float)b.x + (float)b.y * (float)b.y +
                         (float)b.z * (float)b.z);
  const float vx = (float)b.x / nb, vy = (float)b.y / nb, vz = (float)b.z / nb;
  const float c = vz;
  if (!(c > -1.0f + 1e-5f)) return false;
  const float s = sqrtf((1.0f + c) * 2.0f), invs = 1.0f / s;
  const float qx = -vy * invs, qy = vx * invs, qz = 0.0f, qw = s * 0.5f;
  const float tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
  const float twx = tx * qw, twy = ty * qw, twz = tz * qw;
  const float txx = tx * qx, txy = ty * qx, txz = tz * qx;
  const float tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  const float M00 = 1 - (tyy + tzz), M01 = txy - twz, M02 = txz + twy;
  const float M10 = txy + twz, M11 = 1 - (txx + tzz);
  const float M20 = txz - twy, M21 = tyz + twx, M22 = 1 - (txx + tyy), M12 = tyz - twx;
  const float PIf = 3.14159265f;
  float r0 = atan2f(M12, M22);
  if (fabsf(r0) < eps || fabsf(PIf - fabsf(r0)) < eps) return false;
  const float c2 = hypotf(M00, M01);
  float r1;
  if (r0 > 0) {
    r0 -= PIf;
    r1 = atan2f(-M02, -c2);
  } else {
    r1 = atan2f(-M02, c2);
  }
  const float s1 = sinf(r0), c1 = cosf(r0);
  const float r2 = atan2f(s1 * M20 - c1 * M10, c1 * M11 - s1 * M21);
  ang[0] = -r0; ang[1] = -r1; ang[2] = -r2;
  for (int i = 0; i < 3; ++i)
    if (fabsf(ang[i] - 0.1f) < eps || fabsf(PIf - fabsf(ang[i]) - 0.1f) < eps) return false;
  return true;
}

__device__ bool plane_gates(const Dev& d, const PlaneD& pl) {
  const d3 nrm = mk3(pl.plane[0], pl.plane[1], pl.plane[2]);
  sloam_se3 pe;
  for (int j = 0; j < 4; ++j) pe.q[j] = d.pose_io[j];
  for (int j = 0; j < 3; ++j) pe.t[j] = d.pose_io[4 + j];
  const Pose T = pose_from(pe);
  const d3 nw = rot3(T.R, nrm);
  const double PI = 3.14159265358979323846;
  // the angle gate from FP32 angles where their decision is certain (a
  // 1e-4 rad margin, about 100 times their error), else from FP64
  bool angle_ok;
  float af[3];
  if (euler_z_to_f(nw, 1e-4f, af)) {
    const float PIf = 3.14159265f;
    angle_ok = (af[0] < 0.1f && af[1] < 0.1f && af[2] < 0.1f) ||
               (PIf - fabsf(af[0]) < 0.1f && PIf - fabsf(af[1]) < 0.1f &&
                PIf - fabsf(af[2]) < 0.1f);
  } else {
    double ang[3];
    euler_two_vectors(mk3(0, 0, 1), nw, ang);
    angle_ok = (ang[0] < 0.1 && ang[1] < 0.1 && ang[2] < 0.1) ||
               (PI - fabs(ang[0]) < 0.1 && PI - fabs(ang[1]) < 0.1 &&
                PI - fabs(ang[2]) < 0.1);
  }
  const bool height_ok =
      xform(T, mk3(pl.centroid[0], pl.centroid[1], pl.centroid[2])).z < T.t.z;
  return angle_ok && height_ok;
}

__global__ void __launch_bounds__(1024) k_plane_compact(Dev d, KParams kp) {
  __shared__ int sm[33];
  int base = 0;
  for (int b0 = 0; b0 < d.n_bins; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    const bool v = b < d.n_bins && d.plane_all[b].valid && plane_gates(d, d.plane_all[b]);
    int total;
    const int ex = block_excl_scan(v ? 1 : 0, sm, &total);
    if (v) {
      d.planes[base + ex] = d.plane_all[b];
      for (int j = 0; j < kp.G; ++j)
        d.plane_feat[(size_t)(base + ex) * kp.G + j] = d.plane_feat_all[(size_t)b * kp.G + j];
    }
    base += total;
  }
  if (threadIdx.x == 0) d.cnt->n_planes = base;
}

// ============================================================ cylinders
__device__ __forceinline__ float euclid2d_f(float ax, float ay, float bx, float by) {
  const float dx = fsub(ax, bx), dy = fsub(ay, by);
  return fsqrt(fadd(fmul(dx, dx), fmul(dy, dy)));
}

// PCL line refit direction with pcl::computeCorrespondingEigenVector's sign
// (the largest cross product of the rows of S - lambda_max I), FP32.
__device__ d3 pcl_line_direction(const double* Sd) {
  float S[9], ev[3], V[9];
  for (int k = 0; k < 9; ++k) S[k] = (float)Sd[k];
  jacobi3f(S, ev, V);
  const float lam = ev[2];
  float scale = 0.f;
  for (int k = 0; k < 9; ++k) scale = fmaxf(scale, fabsf(S[k]));
  if (scale <= FLT_MIN) scale = 1.0f;
  const float is = 1.0f / scale;
  float M[9];
  for (int k = 0; k < 9; ++k) M[k] = S[k] * is;
  M[0] -= lam * is; M[4] -= lam * is; M[8] -= lam * is;
  auto crs = [](const float* a, const float* b, float* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  float c1[3], c2[3], c3[3];
  crs(M, M + 3, c1);
  crs(M, M + 6, c2);
  crs(M + 3, M + 6, c3);
  const float l1 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
  const float l2 = c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2];
  const float l3 = c3[0] * c3[0] + c3[1] * c3[1] + c3[2] * c3[2];
  const float* c;
  float l;
  if (l1 >= l2 && l1 >= l3) { c = c1; l = l1; }
  else if (l2 >= l1 && l2 >= l3) { c = c2; l = l2; }
  else { c = c3; l = l3; }
  const float r = rsqrtf(l);
  d3 v = mk3(c[0] * r, c[1] * r, c[2] * r);
  if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && l > 0.f)) v = mk3(V[2], V[5], V[8]);
  return v;
}

__device__ __forceinline__ int line_count(const float* vx, int V, float ax, float ay, float az,
                                          float dx, float dy, float dz, float thr2, int j0,
                                          int step) {
  int cnt = 0;
  for (int j = j0; j < V; j += step) {
    const float vxj = fsub(ax, vx[3 * j]), vyj = fsub(ay, vx[3 * j + 1]),
                vzj = fsub(az, vx[3 * j + 2]);
    const float cx = fsub(fmul(vyj, dz), fmul(vzj, dy));
    const float cy = fsub(fmul(vzj, dx), fmul(vxj, dz));
    const float cz = fsub(fmul(vxj, dy), fmul(vyj, dx));
    const float sq = fadd(fadd(fmul(cx, cx), fmul(cy, cy)), fmul(cz, cz));
    cnt += sq < thr2;
  }
  return cnt;
}

// One warp per landmark: vertex-line RANSAC model, radius, features.
// Writes cyl_all[l] with stage 1 when a model exists.  The plane gates of
// the same reference code (a model needs a ground plane, and the nearest
// plane's centroid within max_lidar_dist) are applied by k_cyl_gate once
// the planes exist: nothing here reads a plane, so the ground planes are
// fitted beside the Trellis and this fit.
constexpr int kCylWarps = 4;
constexpr int kMaxLineHyp = 256;

__global__ void __launch_bounds__(kCylWarps * 32) k_cyl_fit(Dev d, KParams kp) {
  __shared__ int scnt[kCylWarps][kMaxLineHyp];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int nl = d.cnt->n_lm;
  for (int l = wg; l < nl; l += nw) {
    CylD c{};
    c.landmark = l;
    c.plane = -1;
    c.stage = 0;
    c.valid = 0;
    c.radius = -1;
    if (lane == 0) d.cyl_best[l] = 0ull;
    const int vb = d.lm_vbeg[l], V = d.lm_vbeg[l + 1] - vb;
    const float* vx = d.lm_vxyz + 3 * (size_t)vb;
    c.id = d.lm_tree[l];
    // features (cylinder.cpp:82-91, 172): the first F vertex points
    {
      const int p0 = d.lm_pbeg[vb], p1 = d.lm_pbeg[vb + V];
      for (int f = lane; f < kp.F; f += 32) {
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p0 + f < p1) {
          q = d.lm_pts[p0 + f];
          q.w = (float)c.id;
        }
        d.cyl_feat_all[(size_t)l * kp.F + f] = q;
      }
    }
    if (V < 3) {
      if (lane == 0) d.cyl_all[l] = c;
      continue;
    }
    c.root[0] = vx[3]; c.root[1] = vx[4]; c.root[2] = vx[5];
    // ---- validRadii median (cylinder.cpp:141-163)
    int nvalid = 0, nle0 = 0;
    for (int j = lane; j < V; j += 32) {
      const int npj = d.lm_pbeg[vb + j + 1] - d.lm_pbeg[vb + j];
      if (npj > 3) {
        ++nvalid;
        if (!((float)d.lm_vrad[vb + j] > 0.0f)) ++nle0;
      }
    }
    nvalid = warp_sumi(nvalid);
    nle0 = warp_sumi(nle0);
    float rad_med = -1.0f;
    if (nvalid > 0) {
      const int dd = nle0;
      const int middle = min(nvalid - 1, (dd + 1) + (nvalid - dd) / 2);
      float found = -FLT_MAX;
      for (int j = lane; j < V; j += 32) {
        const int npj = d.lm_pbeg[vb + j + 1] - d.lm_pbeg[vb + j];
        if (npj <= 3) continue;
        const float rj = (float)d.lm_vrad[vb + j];
        int rank = 0;
        for (int k = 0; k < V; ++k) {
          const int npk = d.lm_pbeg[vb + k + 1] - d.lm_pbeg[vb + k];
          if (npk <= 3) continue;
          const float rk = (float)d.lm_vrad[vb + k];
          rank += (rk < rj) || (rk == rj && k < j);
        }
        if (rank == middle) found = rj;
      }
      for (int o = 16; o > 0; o >>= 1) found = fmaxf(found, __shfl_xor_sync(0xffffffffu, found, o));
      rad_med = found;
    }
    // ---- tree height (cylinder.cpp:101-113)
    const float* top = vx + 3 * (V - 2);
    if (eigen_sqnorm3(vx[3], vx[4], vx[5], top[0], top[1], top[2]) < kp.min_tree_height_sq) {
      if (lane == 0) d.cyl_all[l] = c;  // radius -1: invalid
      continue;
    }
    // ---- vertex-line RANSAC (PCL SACMODEL_LINE semantics)
    const float thr2 = (float)(kp.line_thr * kp.line_thr);
    const int K = min(kp.line_max_iter, kMaxLineHyp);
    for (int h = lane; h < K; h += 32) {
      uint32_t u[4], id[2];
      philox(kp.seed, (uint32_t)h, (uint32_t)c.id, 0u, 0u, u);
      draw_distinct(u, (uint32_t)V, 2, id);
      const float ax = vx[3 * id[0]], ay = vx[3 * id[0] + 1], az = vx[3 * id[0] + 2];
      float dx = fsub(vx[3 * id[1]], ax), dy = fsub(vx[3 * id[1] + 1], ay),
            dz = fsub(vx[3 * id[1] + 2], az);
      const float nn = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
      int cnt = -1;
      if (nn != 0.0f) {
        const float nr = fsqrt(nn);
        dx = fdiv(dx, nr); dy = fdiv(dy, nr); dz = fdiv(dz, nr);
        cnt = line_count(vx, V, ax, ay, az, dx, dy, dz, thr2, 0, 1);
      }
      scnt[w][h] = cnt;
    }
    __syncwarp();
    int best = -1, best_count = 0;
    if (lane == 0) {
      double k = 1.0;
      int itn = 0;
      const double eps = DBL_EPSILON;
      for (int h = 0; h < K; ++h) {
        if (!(itn < k)) break;
        const int cnt = scnt[w][h];
        if (cnt < 0) continue;
        if (cnt > best_count) {
          best_count = cnt;
          best = h;
          if (V <= kLineKMax) {  // the host's value of the reference's expression
            k = d.line_k[V * (kLineKMax + 1) + best_count];
          } else {
            const double wgt = (double)best_count / V;
            double p_no = 1.0 - wgt * wgt;
            p_no = fmax(eps, fmin(1.0 - eps, p_no));
            k = log(1.0 - kp.line_prob) / log(p_no);
          }
        }
        ++itn;
      }
    }
    best = __shfl_sync(0xffffffffu, best, 0);
    best_count = __shfl_sync(0xffffffffu, best_count, 0);
    c.inliers = best_count;
    if (best < 0) {
      if (lane == 0) d.cyl_all[l] = c;
      continue;
    }
    uint32_t u[4], id[2];
    philox(kp.seed, (uint32_t)best, (uint32_t)c.id, 0u, 0u, u);
    draw_distinct(u, (uint32_t)V, 2, id);
    const float ax = vx[3 * id[0]], ay = vx[3 * id[0] + 1], az = vx[3 * id[0] + 2];
    float dx = fsub(vx[3 * id[1]], ax), dy = fsub(vx[3 * id[1] + 1], ay),
          dz = fsub(vx[3 * id[1] + 2], az);
    {
      const float nr = fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
      dx = fdiv(dx, nr); dy = fdiv(dy, nr); dz = fdiv(dz, nr);
    }
    // inliers of the best model -> PCA refit (FP64)
    int ni = 0;
    double sx = 0, sy = 0, sz = 0;
    unsigned inl_lo = 0, inl_hi = 0;  // V <= 64 inlier bit mask
    for (int j = lane; j < V; j += 32) {
      const float vxj = fsub(ax, vx[3 * j]), vyj = fsub(ay, vx[3 * j + 1]),
                  vzj = fsub(az, vx[3 * j + 2]);
      const float cx = fsub(fmul(vyj, dz), fmul(vzj, dy));
      const float cy = fsub(fmul(vzj, dx), fmul(vxj, dz));
      const float cz = fsub(fmul(vxj, dy), fmul(vyj, dx));
      const float sq = fadd(fadd(fmul(cx, cx), fmul(cy, cy)), fmul(cz, cz));
      if (sq < thr2) {
        ++ni;
        sx += vx[3 * j]; sy += vx[3 * j + 1]; sz += vx[3 * j + 2];
        if (j < 32) inl_lo |= 1u << j;
        else inl_hi |= 1u << (j - 32);
      }
    }
    ni = warp_sumi(ni);
    sx = warp_sumd(sx); sy = warp_sumd(sy); sz = warp_sumd(sz);
    for (int o = 16; o > 0; o >>= 1) {
      inl_lo |= __shfl_xor_sync(0xffffffffu, inl_lo, o);
      inl_hi |= __shfl_xor_sync(0xffffffffu, inl_hi, o);
    }
    d3 cpt = mk3(ax, ay, az), dir = mk3(dx, dy, dz);
    if (ni > 2) {
      const d3 m = mk3(sx / ni, sy / ni, sz / ni);
      double s6[6] = {0, 0, 0, 0, 0, 0};
      for (int j = lane; j < V; j += 32) {
        const bool in = j < 32 ? ((inl_lo >> j) & 1u) : ((inl_hi >> (j - 32)) & 1u);
        if (!in) continue;
        const double q0 = vx[3 * j] - m.x, q1 = vx[3 * j + 1] - m.y, q2 = vx[3 * j + 2] - m.z;
        s6[0] += q0 * q0; s6[1] += q0 * q1; s6[2] += q0 * q2;
        s6[3] += q1 * q1; s6[4] += q1 * q2; s6[5] += q2 * q2;
      }
      for (int j = 0; j < 6; ++j) s6[j] = warp_sumd(s6[j]);
      const double S[9] = {s6[0], s6[1], s6[2], s6[1], s6[3], s6[4], s6[2], s6[4], s6[5]};
      cpt = m;
      dir = pcl_line_direction(S);
    }
    int reinl = 0;
    for (int j = lane; j < V; j += 32) {
      const d3 q = sub3(mk3(vx[3 * j], vx[3 * j + 1], vx[3 * j + 2]), cpt);
      const d3 x = cross3(q, dir);
      reinl += dot3(x, x) < kp.line_thr * kp.line_thr;
    }
    reinl = warp_sumi(reinl);
    if (reinl == 0) {
      if (lane == 0) d.cyl_all[l] = c;
      continue;
    }
    c.ray[0] = (double)(float)dir.x;
    c.ray[1] = (double)(float)dir.y;
    c.ray[2] = (double)(float)dir.z;
    double radius = -1.0;
    if (nvalid > 0) {
      radius = rad_med;
      if (radius == 0) radius = -1;
      else if (radius < kp.default_tree_radius) radius = kp.default_tree_radius;
    }
    c.radius = radius;
    c.stage = 1;
    if (lane == 0) d.cyl_all[l] = c;
  }
}

// The plane gates of the cylinder model (sloam.cpp:420-431 nearest plane to
// vertex[1]; cylinder.cpp:11-13 within maxLidarDist of its centroid), one
// warp per landmark, after the planes and the cylinder fits: a landmark
// without a plane, or too far from its plane, gets the record the model
// code gives it at that point (no model, radius -1, the plane index);
// otherwise the record keeps its fit and gets the plane.
__device__ __forceinline__ CylD no_model(int l, int id, int plane) {
  CylD c{};
  c.landmark = l;
  c.plane = plane;
  c.stage = 0;
  c.valid = 0;
  c.radius = -1;
  c.id = id;
  return c;
}
// One landmark's gates, by a whole warp (the nearest plane by a warp argmin).
__device__ __forceinline__ void cyl_gate_one(const Dev& d, const KParams& kp, int l, int np,
                                             int lane) {
  const int vb = d.lm_vbeg[l], V = d.lm_vbeg[l + 1] - vb;
  if (V < 3) return;  // no model and no plane either way
  CylD c = d.cyl_all[l];
  if (np == 0) {
    if (lane == 0) d.cyl_all[l] = no_model(l, c.id, -1);
    return;
  }
  const float* vx = d.lm_vxyz + 3 * (size_t)vb;
  const d3 v1 = mk3(vx[3], vx[4], vx[5]);
  double bd = 100000.0;
  int bi = 0;
  for (int k = lane; k < np; k += 32) {
    const PlaneD& P = d.planes[k];
    const double dist = fabs(P.plane[0] * v1.x + P.plane[1] * v1.y + P.plane[2] * v1.z + P.plane[3]) /
                        norm3(mk3(P.plane[0], P.plane[1], P.plane[2]));
    if (dist < bd) { bd = dist; bi = k; }
  }
  warp_argmin(bd, bi);
  if (!(bd < 100000.0)) bi = 0;
  const PlaneD P = d.planes[bi];
  const float cxf = (float)P.centroid[0], cyf = (float)P.centroid[1];
  const bool within = (double)euclid2d_f(vx[3], vx[4], cxf, cyf) < kp.max_lidar_dist;
  if (lane == 0) {
    if (within) {
      c.plane = bi;
      d.cyl_all[l] = c;
    } else {
      d.cyl_all[l] = no_model(l, c.id, bi);
    }
  }
}

// ---------------------------------------------- point-level cylinder fit

// Projection of each eligible tree's points on its prior-axis frame.
__global__ void __launch_bounds__(256) k_cyl_uv(Dev d) {
  const int nl = d.cnt->n_lm;
  for (int l = blockIdx.x; l < nl; l += gridDim.x) {
    const CylD c = d.cyl_all[l];
    if (!fit_eligible(c)) continue;
    const float4* pts;
    const float2* uv;
    int n;
    tree_points(d, l, &pts, &n, &uv);
    const CylFrame f = make_frame(d, c);
    float2* out = const_cast<float2*>(uv);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = project_uv(f, pts[i]);
  }
}

// Hypothesis table: one thread per (tree, hypothesis); clears the counts.
// An invalid hypothesis gets hi2 = -1 (no point can be an inlier).  With a
// mask (`only`), only the masked trees' rows are written (the queue reads no
// other), and nothing at all when the learned pass kept every tree.
__global__ void __launch_bounds__(256) k_cyl_hypgen(Dev d, KParams kp,
                                                    const int32_t* __restrict__ only) {
  const int nl = d.cnt->n_lm, K = kp.K;
  if (only && d.cnt->n_fallback == 0) return;  // no tree for the RANSAC pass
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nl * K;
       it += gridDim.x * blockDim.x) {
    const int l = it / K, h = it - l * K;
    if (only && !only[l]) continue;  // only the queued trees' rows are read
    d.hyp_cnt[it] = 0;
    float4 e = make_float4(0.f, 0.f, 0.f, -1.f);
    const CylD c = d.cyl_all[l];
    if (fit_eligible(c) && (!only || only[l])) {
      const float4* pts;
      const float2* uv;
      int n;
      tree_points(d, l, &pts, &n, &uv);
      if (n >= 3) {
        const Hyp H = make_hyp(kp, h, c.id, n, [&](uint32_t i) { return uv[i]; });
        if (H.ok) e = make_float4(H.cu, H.cv, H.lo2, H.hi2);
      }
    }
    d.hyp[it] = e;
  }
}

// ----------------------------------------- learned proposals (cyl_mode 2)
// 8 (prop_S) samples of 128 points per eligible tree, drawn with
// replacement from the tree's points (Philox keyed by tree id, sample and
// point), centred and scaled by the trimmed frame the network was trained
// with (prop::sample_frame).
__global__ void __launch_bounds__(128) k_prop_gather(Dev d, KParams kp) {
  __shared__ float red[4];
  const int nl = d.cnt->n_lm, S = kp.prop_S;
  const int i = threadIdx.x;
  for (int it = blockIdx.x; it < nl * S; it += gridDim.x) {
    const int l = it / S, j = it - l * S;
    const CylD c = d.cyl_all[l];
    const float4* pts;
    const float2* uv;
    int n;
    tree_points(d, l, &pts, &n, &uv);
    if (!fit_eligible(c) || n < 1) {  // scale 0: the network skips the tree
      if (i == 0) d.prop_f[it] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    uint32_t u[4];
    philox(kp.seed, (uint32_t)c.id, (uint32_t)j, 3u, (uint32_t)i, u);
    const float4 p = pts[mulhi_idx(u[0], (uint32_t)n)];
    float mm[3], sc;
    prop::sample_frame(p.x, p.y, p.z, red, mm, &sc);
    const float mx = mm[0], my = mm[1], mz = mm[2];
    const float dx = p.x - mx, dy = p.y - my, dz = p.z - mz;
    float* x = d.prop_x + (size_t)it * 384;
    x[3 * i] = dx / sc;
    x[3 * i + 1] = dy / sc;
    x[3 * i + 2] = dz / sc;
    if (i == 0) d.prop_f[it] = make_float4(mx, my, mz, sc);
  }
}

// Network output -> circle hypothesis on the tree's prior-axis frame: the
// proposed axis point nearest the sample mean, projected along the prior
// axis, and the proposed radius with the inlier band +-tau; (0, 0, 0, -1)
// (no inlier) when the output gives no usable circle.
__device__ __forceinline__ float4 prop_hyp(const Dev& d, const KParams& kp, int it,
                                           const CylFrame& f) {
  float4 e = make_float4(0.f, 0.f, 0.f, -1.f);
  const float* o = d.prop_out + (size_t)it * 8;
  const float4 fm = d.prop_f[it];
  float ax = o[0], ay = o[1], az = o[2];
  const float an = sqrtf(ax * ax + ay * ay + az * az);
  if (an > 0.f && fabsf(az) > 1e-3f * an) {
    ax /= an; ay /= an; az /= an;
    const float cz = -(o[3] * ax + o[4] * ay) / az;
    const float4 C = make_float4(fm.x + fm.w * o[3], fm.y + fm.w * o[4], fm.z + fm.w * cz, 0.f);
    const float r = fm.w * expf(o[5]);
    const float2 cuv = project_uv(f, C);
    if (r > 0.f && r <= kp.max_hyp_r && isfinite(cuv.x) && isfinite(cuv.y)) {
      const float lo = fsub(r, kp.tau), hi = fadd(r, kp.tau);
      e = make_float4(cuv.x, cuv.y, lo > 0.0f ? fmul(lo, lo) : -1.0f, fmul(hi, hi));
    }
  }
  return e;
}

// The learned proposals' pass (cyl_mode 2), one block per tree: the tree's
// prop_S circle hypotheses from the network outputs, their inlier counts
// over the tree's projected points (|(u, v) - centre|^2 strictly inside the
// band), the best (most inliers, the lowest proposal on ties, none without
// an inlier), then LS refinement from it with the inliers re-selected by
// the current model; the refined model is kept when its inliers (|distance
// to the refined axis - radius| < tau) are at least prop_ratio of the
// tree's points, else the tree is flagged for the RANSAC pass (the cylinder
// work queue).  The proposals are few and their trees all alike in cost, so
// one block per tree does the whole pass with no launch in between.
constexpr int kLsThreads = 256, kMaxProp = 8;
__global__ void __launch_bounds__(kLsThreads, 4) k_prop_fit(Dev d, KParams kp) {
  __shared__ int s_in[kLsThreads / 32];
  __shared__ float red[20][kLsThreads / 32];
  __shared__ double st[14];  // c(3), dir(3), r, ok, b1(3), b2(3)
  __shared__ double ssum[20];
  __shared__ double sxls[5];
  __shared__ float sf[13];   // c(3), dir(3), b1(3), b2(3), r as float
  __shared__ float4 s_hyp[kMaxProp];
  __shared__ int s_cnt[kLsThreads / 32][kMaxProp];
  __shared__ unsigned long long s_best;
  const int nl = d.cnt->n_lm, S = kp.prop_S;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int l = blockIdx.x; l < nl; l += gridDim.x) {
    CylD c = d.cyl_all[l];
    const bool elig = fit_eligible(c);
    if (threadIdx.x == 0) {
      d.pflag[l] = 0;
      if (elig) atomicAdd(&d.cnt->n_fit, 1);
    }
    if (!elig) continue;
    const float4* pts;
    const float2* uvs;
    int n;
    tree_points(d, l, &pts, &n, &uvs);
    const CylFrame f = make_frame(d, c);
    if (threadIdx.x < S) s_hyp[threadIdx.x] = prop_hyp(d, kp, l * S + threadIdx.x, f);
    __syncthreads();
    {
      int cnt[kMaxProp];
#pragma unroll
      for (int h = 0; h < kMaxProp; ++h) cnt[h] = 0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float2 p = uvs[i];
#pragma unroll
        for (int h = 0; h < kMaxProp; ++h) {
          if (h >= S) break;
          const float4 e = s_hyp[h];
          const float du = fsub(p.x, e.x), dv = fsub(p.y, e.y);
          const float d2 = fadd(fmul(du, du), fmul(dv, dv));
          cnt[h] += (d2 > e.z) && (d2 < e.w) ? 1 : 0;
        }
      }
#pragma unroll
      for (int h = 0; h < kMaxProp; ++h) {
        const int v = warp_sumi(cnt[h]);
        if (lane == 0) s_cnt[w][h] = v;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long best = 0ull;
        for (int h = 0; h < S; ++h) {
          int t = 0;
          for (int q2 = 0; q2 < kLsThreads / 32; ++q2) t += s_cnt[q2][h];
          if (t > 0) {
            const unsigned long long key =
                ((unsigned long long)t << 32) | (unsigned long long)(0xFFFFFFFFu - (uint32_t)h);
            best = key > best ? key : best;
          }
        }
        s_best = best;
      }
      __syncthreads();
    }
    const unsigned long long key = s_best;
    if (key == 0ull) {
      if (threadIdx.x == 0) {
        d.pflag[l] = 1;
        atomicAdd(&d.cnt->n_fallback, 1);
      }
      __syncthreads();
      continue;
    }
    const int h = (int)(0xFFFFFFFFu - (uint32_t)(key & 0xffffffffull));
    const int best_cnt = (int)(key >> 32);
    Hyp H;
    {
      const float4 e = s_hyp[h];
      H.cu = e.x;
      H.cv = e.y;
      H.lo2 = e.z;
      H.hi2 = e.w;
      H.r = fsub(fsqrt(e.w), kp.tau);
      H.ok = true;
    }
    if (threadIdx.x == 0) {
      st[0] = f.ox + (double)H.cu * f.e1x + (double)H.cv * f.e2x;
      st[1] = f.oy + (double)H.cu * f.e1y + (double)H.cv * f.e2y;
      st[2] = f.oz + (double)H.cu * f.e1z + (double)H.cv * f.e2z;
      const double an = sqrt((double)f.ax * f.ax + (double)f.ay * f.ay + (double)f.az * f.az);
      st[3] = f.ax / an; st[4] = f.ay / an; st[5] = f.az / an;
      st[6] = H.r;
      st[7] = 1.0;
      ls_frame(st, sf);
    }
    __syncthreads();
    for (int itn = 0; itn < kp.ls_iters; ++itn) {
      if (st[7] == 0.0) break;
      // the model and its normal frame, as floats (computed once by thread 0)
      const float cx = sf[0], cy = sf[1], cz = sf[2];
      const float dx = sf[3], dy = sf[4], dz = sf[5];
      const float b1x = sf[6], b1y = sf[7], b1z = sf[8];
      const float b2x = sf[9], b2y = sf[10], b2z = sf[11];
      const float rf = sf[12];
      float acc[20];
#pragma unroll
      for (int j = 0; j < 20; ++j) acc[j] = 0.f;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 q = pts[i];
        const float wx = q.x - cx, wy = q.y - cy, wz = q.z - cz;
        const float wd = wx * dx + wy * dy + wz * dz;
        const float px_ = wx - wd * dx, py_ = wy - wd * dy, pz_ = wz - wd * dz;
        const float rho = sqrtf(px_ * px_ + py_ * py_ + pz_ * pz_);
        if (!(rho > 0.f)) continue;
        // a proposal starts coarser: its inliers follow the current model,
        // in a band of 2 tau on the first iteration and tau after it
        if (!(fabsf(rho - rf) < (itn == 0 ? 2.0f : 1.0f) * kp.tau)) continue;
        const float res = rho - rf;
        const float a1 = (px_ * b1x + py_ * b1y + pz_ * b1z) / rho;
        const float a2 = (px_ * b2x + py_ * b2y + pz_ * b2z) / rho;
        const float J[5] = {-a1, -a2, -wd * a1, -wd * a2, -1.0f};
        int k = 0;
#pragma unroll
        for (int p = 0; p < 5; ++p)
#pragma unroll
          for (int q2 = p; q2 < 5; ++q2) acc[k++] += J[p] * J[q2];
#pragma unroll
        for (int p = 0; p < 5; ++p) acc[15 + p] += J[p] * res;
      }
#pragma unroll
      for (int j = 0; j < 20; ++j) {
        const float v = warp_sum(acc[j]);
        if (lane == 0) red[j][w] = v;
      }
      __syncthreads();
      // sum j over the warps by lane j of warp 0 (the same order as one
      // thread summing them)
      if (w == 0) {
        if (lane < 20) {
          double t2 = 0;
          for (int q2 = 0; q2 < kLsThreads / 32; ++q2) t2 += red[lane][q2];
          ssum[lane] = t2;
        }
        __syncwarp();
        // the 5x5 normal equations (ssum: upper triangle, then J^T r) and
        // the model update on the warp
        const bool solved = warp_chol_solve<5>(ssum, ssum + 15, sxls);
        __syncwarp();
        if (solved) {
          warp_model_update(st, sxls, sf);
        } else if (lane == 0) {
          st[7] = 0.0;
        }
      }
      __syncthreads();
    }
    {
      // inliers of the refined model over all the tree's points
      const float cx = sf[0], cy = sf[1], cz = sf[2];
      const float dx = sf[3], dy = sf[4], dz = sf[5];
      const float rf = sf[12];
      int cnt = 0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 q = pts[i];
        const float wx = q.x - cx, wy = q.y - cy, wz = q.z - cz;
        const float wd = wx * dx + wy * dy + wz * dz;
        const float px_ = wx - wd * dx, py_ = wy - wd * dy, pz_ = wz - wd * dz;
        const float rho = sqrtf(px_ * px_ + py_ * py_ + pz_ * pz_);
        cnt += fabsf(rho - rf) < kp.tau ? 1 : 0;
      }
      cnt = warp_sumi(cnt);
      if (lane == 0) s_in[w] = cnt;
      __syncthreads();
      int tot = 0;
      for (int q2 = 0; q2 < kLsThreads / 32; ++q2) tot += s_in[q2];
      const bool keep = st[7] != 0.0 && (float)tot >= kp.prop_ratio * (float)n;
      __syncthreads();
      if (!keep) {
        if (threadIdx.x == 0) {
          d.pflag[l] = 1;
          atomicAdd(&d.cnt->n_fallback, 1);
        }
        continue;
      }
    }
    if (threadIdx.x == 0) {
      d3 cc = mk3(st[0], st[1], st[2]), dd = mk3(st[3], st[4], st[5]);
      if (dd.z < 0) dd = scl3(-1.0, dd);
      const float* vx = d.lm_vxyz + 3 * (size_t)d.lm_vbeg[l];
      const d3 b = mk3(vx[3], vx[4], vx[5]);
      const d3 root = add3(cc, scl3(dot3(sub3(b, cc), dd), dd));
      c.root[0] = root.x; c.root[1] = root.y; c.root[2] = root.z;
      c.ray[0] = dd.x; c.ray[1] = dd.y; c.ray[2] = dd.z;
      c.radius = st[6] > 0 ? st[6] : -1.0;
      c.inliers = best_cnt;
      c.stage = 2;
      d.cyl_all[l] = c;
    }
    __syncthreads();
  }
}

// One landmark's ground-based root and validity, by one thread:
// groundBasedRoot (cylinder.cpp:41-55), validNorm, filter (cylinder.cpp:57-73).
__device__ __forceinline__ void cyl_finalize_one(const Dev& d, const KParams& kp, int l) {
  CylD c = d.cyl_all[l];
  if (c.stage == 0) {
    c.valid = 0;
    d.cyl_all[l] = c;
    return;
  }
  const PlaneD P = d.planes[c.plane];
  const d3 n = mk3(P.plane[0], P.plane[1], P.plane[2]);
  d3 root = mk3(c.root[0], c.root[1], c.root[2]);
  const d3 ray = mk3(c.ray[0], c.ray[1], c.ray[2]);
  const float dist = (float)(fabs(P.plane[0] * root.x + P.plane[1] * root.y +
                                  P.plane[2] * root.z + P.plane[3]) / norm3(n));
  bool validZ = false;
  if (dist < kp.root_plane_max_dist) {
    // rayPlaneIntersection, utils.h:41-51
    const float denom = (float)dot3(n, ray);
    if (fabsf(denom) > 0.001f) {
      const float t = (float)(dot3(sub3(mk3(P.centroid[0], P.centroid[1], P.centroid[2]), root), n) /
                              (double)denom);
      if (t >= 0.001f) root = add3(root, scl3((double)t, ray));
    }
    validZ = true;
  }
  c.root[0] = root.x; c.root[1] = root.y; c.root[2] = root.z;
  const bool validNorm = norm3(root) > 0.01;
  const bool validRadius = c.radius > 0.0;
  bool validTree = false;
  if (c.radius != -1.0) {
    const double theta = (180.0 / kPIDEF) * acos(dot3(ray, n) / (norm3(ray) * norm3(n)));
    validTree = (c.radius < kp.max_tree_radius) &&
                ((theta <= kp.max_axis_theta) || (theta >= 180.0 - kp.max_axis_theta));
  }
  c.valid = validZ && validRadius && validTree && validNorm;
  d.cyl_all[l] = c;
}

// The plane gates and then the ground-based root and validity of each
// landmark, one warp per landmark over the grid (the FP64 of both spread
// over the SMs: one block of 1024 threads doing all of it, fused with the
// compaction below, ran the cylinder stage 7 us longer).
__global__ void __launch_bounds__(kCylWarps * 32) k_cyl_gate(Dev d, KParams kp) {
  const int lane = threadIdx.x & 31;
  const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int nl = d.cnt->n_lm, np = d.cnt->n_planes;
  for (int l = wg; l < nl; l += nw) {
    cyl_gate_one(d, kp, l, np, lane);
    if (lane == 0) cyl_finalize_one(d, kp, l);  // reads the record lane 0 wrote
  }
}

// The ordered list of the valid cylinders, one block.
__global__ void __launch_bounds__(1024) k_cyl_compact(Dev d, KParams kp) {
  __shared__ int sm[33];
  const int nl = d.cnt->n_lm;
  int base = 0;
  for (int l0 = 0; l0 < nl; l0 += blockDim.x) {
    const int l = l0 + threadIdx.x;
    const bool v = l < nl && d.cyl_all[l].valid;
    int total;
    const int ex = block_excl_scan(v ? 1 : 0, sm, &total);
    if (v) {
      d.cyls[base + ex] = d.cyl_all[l];
      for (int f = 0; f < kp.F; ++f)
        d.cyl_feat[(size_t)(base + ex) * kp.F + f] = d.cyl_feat_all[(size_t)l * kp.F + f];
    }
    base += total;
  }
  if (threadIdx.x == 0) d.cnt->n_cyl = base;
}

__global__ void k_zero_bins(Dev d) {
  for (int b = threadIdx.x; b < d.n_bins; b += blockDim.x) d.bin_cnt[b] = 0;
}

}  // namespace

// one wave of warps for the per-landmark kernels (grid-stride beyond it)
constexpr int kCylBlocks = 64;

int launch_cyl_fit_kernel(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_cyl_fit<<<kCylBlocks, kCylWarps * 32, 0, st>>>(d, kp);
  return 1;
}

constexpr int kCountBlocks = 304;

// The inputs of the cylinder work queue (vertex-line models, projected
// points, hypothesis table), for timing the queue alone.
int launch_cyl_count_prep(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_cyl_fit<<<kCylBlocks, kCylWarps * 32, 0, st>>>(d, kp);
  k_cyl_uv<<<kCylBlocks, 256, 0, st>>>(d);
  k_cyl_hypgen<<<kCylBlocks, 256, 0, st>>>(d, kp, nullptr);
  return 3;
}

// mode 1: K random 3-point circles per tree, LS refinement of the best.
// mode 2: prop_S network proposals per tree (one tensor-core launch over
// every sample), inliers counted, the best LS-refined; trees whose refined
// model holds less than prop_ratio of their points as inliers run the K
// random circles and their LS refinement.
int launch_fit_cylinder_points(const Dev& d, const KParams& kp, bool, cudaStream_t st) {
  int n = 0;
  k_cyl_uv<<<kCylBlocks, 256, 0, st>>>(d);
  ++n;
  const int32_t* only = nullptr;
  if (kp.cyl_mode == 2) {
    k_prop_gather<<<kCountBlocks, 128, 0, st>>>(d, kp);
    n += 1 + prop::launch_prop_infer_trees(d.prop_tc, d.prop_x, &d.cnt->n_lm, kp.prop_S,
                                           d.prop_cap, d.prop_f, d.prop_out, d.prop_err, st);
    k_prop_fit<<<kCylBlocks, kLsThreads, 0, st>>>(d, kp);
    n += 1;
    only = d.pflag;
  }
  k_cyl_hypgen<<<kCylBlocks, 256, 0, st>>>(d, kp, only);
  return n + 1 + launch_cyl_queue(d, kp, only, st);
}

int launch_plane_points(const Dev& d, const KParams& kp, int n, cudaStream_t st) {
  k_plane_points<<<1, kPlaneThreads, 0, st>>>(d, kp, n);
  return 1;
}

// The cylinder models before the plane gates: the vertex-line fit and, in
// modes 1 and 2, the point-level fit.  Needs the landmarks only.
int launch_cylinder_fits(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st) {
  int n = 1;
  k_cyl_fit<<<kCylBlocks, kCylWarps * 32, 0, st>>>(d, kp);
  if (kp.cyl_mode >= 1) n += launch_fit_cylinder_points(d, kp, from_trellis, st);
  return n;
}
// The plane gates, the ground-based roots and the valid-cylinder list:
// needs the fits and the planes.
int launch_cylinder_close(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_cyl_gate<<<kCylBlocks, kCylWarps * 32, 0, st>>>(d, kp);
  k_cyl_compact<<<1, 1024, 0, st>>>(d, kp);
  return 2;
}

int launch_cylinders(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st) {
  const int n = launch_cylinder_fits(d, kp, from_trellis, st);
  return n + launch_cylinder_close(d, kp, st);
}

// The ground planes (a7): ground bins, plane fits and gates.  Needs the
// ground list only.
int launch_planes(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_zero_bins<<<1, 256, 0, st>>>(d);
  const int gg = (d.cap_ground + kGbinSpan - 1) / kGbinSpan;
  k_gbin<<<gg < 1 ? 1 : gg, 256, 0, st>>>(d, kp);
  k_gbin_scan<<<1, 1024, 0, st>>>(d);
  k_gbin_scatter<<<gg < 1 ? 1 : gg, 256, 0, st>>>(d);
  k_plane<<<d.n_bins, kPlaneThreads, 0, st>>>(d, kp);
  k_plane_compact<<<1, 1024, 0, st>>>(d, kp);
  return 6;
}

int launch_models(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st) {
  const int n = launch_planes(d, kp, st);
  return n + launch_cylinders(d, kp, from_trellis, st);
}

void init_kernel_attributes() {
  prop::init_attributes();
  init_queue_attributes();
  init_trellis_attributes();
}

}  // namespace sg
