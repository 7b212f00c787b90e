// sloam_oracle.cpp — TEST INFRASTRUCTURE ONLY (see sloam_oracle.h).
//
// A std-only C++17 restatement of the SLOAM per-keyframe path.  Each function
// cites the reference file:line it follows (paths relative to the
// KumarRobotics/sloam repository).  Where the reference delegates to a
// third-party library that is absent here (PCL 1.10, Eigen 3.3, Ceres
// @206061a), the published behaviour of that library is restated and the
// choice is named in the comment (Eigen's JacobiSVD, down to the sign of the
// plane normal, is restated step by step).  Where the reference is not
// deterministic or its library is not restated (std::sort ties, PCL's
// internal RANSAC RNG, Ceres LM) the contract of this project is stated
// instead; the GPU kernels follow the same
// contract and are checked bit-exact on integers against this file.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared (see build.py);
// -ffp-contract=off keeps every float expression unfused, as the reference's
// x86-64 build computes it.

#include "sloam_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <type_traits>
#include <vector>

namespace {

constexpr double kPIDEF = 3.14159265;  // definitions.h:28
const float kNaNf = std::numeric_limits<float>::quiet_NaN();

struct Pt {
  float x, y, z, i;
};
struct Vtx {  // TreeVertex, definitions.h:56-66 (+ row)
  int treeId = 0;
  double radius = 0;
  bool isValid = false;
  Pt coords{0, 0, 0, 0};
  std::vector<Pt> points;
  int row = 0;
};
using Tree = std::vector<Vtx>;

// std::min / std::max exactly as the reference calls them: a NaN second
// argument returns the first argument (inference.cpp:120-126).
inline float ref_min(float a, float b) { return (b < a) ? b : a; }
inline float ref_max(float a, float b) { return (a < b) ? b : a; }

// ------------------------------------------------------------------ RNG
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
// as easy as 1, 2, 3").  key = 64-bit seed, counter = (hypothesis, tree id,
// stream, 0).  Stream 0 = vertex-line RANSAC, stream 1 = point cylinder.
void philox(uint64_t key64, const uint32_t in[4], uint32_t out[4]) {
  uint32_t k0 = (uint32_t)key64, k1 = (uint32_t)(key64 >> 32);
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
inline uint32_t mulhi_idx(uint32_t u, uint32_t n) {
  return (uint32_t)(((uint64_t)u * n) >> 32);
}
// Distinct indices from one Philox block: i0 in [0,n), i1 in [0,n)\{i0},
// i2 in [0,n)\{i0,i1} (successive skip).
void draw_distinct(const uint32_t u[4], uint32_t n, int k, uint32_t* idx) {
  uint32_t a = mulhi_idx(u[0], n);
  idx[0] = a;
  if (k < 2) return;
  uint32_t b = mulhi_idx(u[1], n - 1);
  if (b >= a) ++b;
  idx[1] = b;
  if (k < 3) return;
  uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
  uint32_t c = mulhi_idx(u[2], n - 2);
  if (c >= lo) ++c;
  if (c >= hi) ++c;
  idx[2] = c;
}

// ------------------------------------------------------- small FP64 algebra
struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

struct SE3 {
  double R[9];  // row-major
  V3 t;
};
SE3 se3_from(const sloam_se3& p) {
  double x = p.q[0], y = p.q[1], z = p.q[2], w = p.q[3];
  double n = std::sqrt(x * x + y * y + z * z + w * w);
  x /= n; y /= n; z /= n; w /= n;
  SE3 T;
  T.R[0] = 1 - 2 * (y * y + z * z); T.R[1] = 2 * (x * y - w * z); T.R[2] = 2 * (x * z + w * y);
  T.R[3] = 2 * (x * y + w * z); T.R[4] = 1 - 2 * (x * x + z * z); T.R[5] = 2 * (y * z - w * x);
  T.R[6] = 2 * (x * z - w * y); T.R[7] = 2 * (y * z + w * x); T.R[8] = 1 - 2 * (x * x + y * y);
  T.t = {p.t[0], p.t[1], p.t[2]};
  return T;
}
inline V3 rot(const double* R, V3 p) {
  return {R[0] * p.x + R[1] * p.y + R[2] * p.z, R[3] * p.x + R[4] * p.y + R[5] * p.z,
          R[6] * p.x + R[7] * p.y + R[8] * p.z};
}
inline V3 xf(const SE3& T, V3 p) { return rot(T.R, p) + T.t; }
// Rotation matrix -> unit quaternion (x, y, z, w), Shepperd's method.
void quat_from_R(const double* R, double* q) {
  double tr = R[0] + R[4] + R[8];
  double x, y, z, w;
  if (tr > 0) {
    double s = std::sqrt(tr + 1.0) * 2;
    w = 0.25 * s; x = (R[7] - R[5]) / s; y = (R[2] - R[6]) / s; z = (R[3] - R[1]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    double s = std::sqrt(1.0 + R[0] - R[4] - R[8]) * 2;
    w = (R[7] - R[5]) / s; x = 0.25 * s; y = (R[1] + R[3]) / s; z = (R[2] + R[6]) / s;
  } else if (R[4] > R[8]) {
    double s = std::sqrt(1.0 + R[4] - R[0] - R[8]) * 2;
    w = (R[2] - R[6]) / s; x = (R[1] + R[3]) / s; y = 0.25 * s; z = (R[5] + R[7]) / s;
  } else {
    double s = std::sqrt(1.0 + R[8] - R[0] - R[4]) * 2;
    w = (R[3] - R[1]) / s; x = (R[2] + R[6]) / s; y = (R[5] + R[7]) / s; z = 0.25 * s;
  }
  double n = std::sqrt(x * x + y * y + z * z + w * w);
  q[0] = x / n; q[1] = y / n; q[2] = z / n; q[3] = w / n;
}
sloam_se3 se3_to(const SE3& T) {
  sloam_se3 o;
  quat_from_R(T.R, o.q);
  o.t[0] = T.t.x; o.t[1] = T.t.y; o.t[2] = T.t.z;
  return o;
}
sloam_se3 se3_identity() {
  sloam_se3 o{};
  o.q[3] = 1.0;
  return o;
}

// Symmetric 3x3 eigen-decomposition, cyclic Jacobi in FP64.  Eigenvalues
// ascending; columns of V are the eigenvectors.
void jacobi3(const double A_in[9], double evals[3], double V[9]) {
  double A[9];
  std::memcpy(A, A_in, sizeof(A));
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 32; ++sweep) {
    double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    double diag = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off <= 1e-300 || off <= diag * 1e-32) break;
    for (int p = 0; p < 2; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        double apq = A[3 * p + q];
        if (apq == 0.0) continue;
        double app = A[3 * p + p], aqq = A[3 * q + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) /
                   (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {  // A = J^T A J
          double akp = A[3 * k + p], akq = A[3 * k + q];
          A[3 * k + p] = c * akp - s * akq;
          A[3 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = A[3 * p + k], aqk = A[3 * q + k];
          A[3 * p + k] = c * apk - s * aqk;
          A[3 * q + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[3 * k + p], vkq = V[3 * k + q];
          V[3 * k + p] = c * vkp - s * vkq;
          V[3 * k + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  int order[3] = {0, 1, 2};
  double d[3] = {A[0], A[4], A[8]};
  std::sort(order, order + 3, [&](int a, int b) { return d[a] < d[b]; });
  double Vs[9];
  for (int c = 0; c < 3; ++c) {
    evals[c] = d[order[c]];
    for (int r = 0; r < 3; ++r) Vs[3 * r + c] = V[3 * r + order[c]];
  }
  std::memcpy(V, Vs, sizeof(Vs));
}

// Cholesky solve of the n x n SPD system H x = b (row-major).  false if H is
// not positive definite or the result is not finite.
bool chol_solve(int n, const double* H, const double* b, double* x) {
  double L[36];
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = H[i * n + j];
      for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[i * n + i] = std::sqrt(s);
      } else {
        L[i * n + j] = s / L[j * n + j];
      }
    }
  }
  double y[6];
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * n + k] * y[k];
    y[i] = s / L[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
    x[i] = s / L[i * n + i];
  }
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

// pcl::euclideanDistance / squaredEuclideanDistance (pcl/common/distances.h):
// float, ((dx*dx + dy*dy) + dz*dz).
inline float pcl_euclid(const Pt& a, const Pt& b) {
  float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}
// Eigen Vector3f (a - b).squaredNorm(): fixed-size redux, dx^2 + (dy^2 + dz^2).
inline float eigen_sqnorm3f(const Pt& a, const Pt& b) {
  float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + (dy * dy + dz * dz);
}
// utils.h:9-14  pow_2 takes a double and returns float.
inline float pow_2(double x) { return (float)(x * x); }
inline float euclid2d(const Pt& a, const Pt& b) {  // utils.h:11-14
  return std::sqrt(pow_2(a.x - b.x) + pow_2(a.y - b.y));
}

// ==================================================================== a1/a2
struct Projection {
  std::vector<int32_t> px, py;
};

// Segmentation::_doProjection, inference.cpp:80-165 (pixel of each point).
void project_points(const sloam_params& P, const float* s, int n, int variant,
                    Projection& pr, std::vector<float>& ranges) {
  const float fov_up = P.fov_up_deg / 180.0 * M_PI;      // inference.cpp:7
  const float fov_down = P.fov_down_deg / 180.0 * M_PI;  // inference.cpp:8
  const float fov = std::abs(fov_down) + std::abs(fov_up);
  const int W = P.img_w, H = P.img_h;
  pr.px.resize(n);
  pr.py.resize(n);
  ranges.resize(n);
  for (int i = 0; i < n; ++i) {
    float x = s[4 * i], y = s[4 * i + 1], z = s[4 * i + 2];
    float range = std::sqrt(x * x + y * y + z * z);  // :99
    float yaw, pitch;
    if (variant == ORACLE_LIBM) {
      yaw = -std::atan2(y, x);      // :107
      pitch = std::asin(z / range);  // :108
    } else {
      // contract: correctly rounded float atan2 / asin
      yaw = -(float)std::atan2((double)y, (double)x);
      pitch = (float)std::asin((double)(z / range));
    }
    float proj_x = 0.5 * (yaw / M_PI + 1.0);                       // :111
    float proj_y = 1.0 - (pitch + std::abs(fov_down)) / fov;       // :112
    proj_x *= W;                                                   // :115
    proj_y *= H;                                                   // :116
    proj_x = std::floor(proj_x);                                   // :119
    proj_x = ref_min(W - 1.0f, proj_x);
    proj_x = ref_max(0.0f, proj_x);
    proj_y = std::floor(proj_y);
    proj_y = ref_min(H - 1.0f, proj_y);
    proj_y = ref_max(0.0f, proj_y);
    pr.px[i] = (int32_t)proj_x;
    pr.py[i] = (int32_t)proj_y;
    ranges[i] = range;
  }
}

// Pixel winners: the reference sorts ranges descending (sort_indexes,
// inference.h:233-243) and scatters, so the nearest point wins a pixel.
// Contract: ties (equal range) go to the lowest point index; a NaN range
// loses to every number.
void pixel_winners(const sloam_params& P, const Projection& pr,
                   const std::vector<float>& ranges, int variant,
                   std::vector<int32_t>& winner) {
  const int W = P.img_w, H = P.img_h, n = (int)ranges.size();
  winner.assign((size_t)W * H, -1);
  bool any_nan = false;
  for (float r : ranges) any_nan |= std::isnan(r);
  if (variant == ORACLE_LIBM && !any_nan) {
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(),
              [&](size_t a, size_t b) { return ranges[a] > ranges[b]; });
    for (size_t k : idx) winner[(size_t)pr.py[k] * W + pr.px[k]] = (int32_t)k;
    return;
  }
  auto key = [&](int i) -> uint64_t {
    uint32_t b;
    float r = ranges[i];
    if (std::isnan(r)) b = 0x7fc00000u;
    else std::memcpy(&b, &r, 4);
    return ((uint64_t)b << 32) | (uint32_t)i;
  };
  std::vector<uint64_t> best((size_t)W * H, ~0ull);
  for (int i = 0; i < n; ++i) {
    size_t p = (size_t)pr.py[i] * W + pr.px[i];
    uint64_t k = key(i);
    if (k < best[p]) {
      best[p] = k;
      winner[p] = i;
    }
  }
}

// ==================================================================== a3
// pcl::OrganizedConnectedComponentSegmentation<PointT, Label>::segment with
// pcl::EuclideanClusterComparator (PCL 1.10, organized_connected_component_
// segmentation.hpp; called at trellis.cpp:15-28).  Two-pass run labelling:
// a pixel is valid iff its x is finite; it joins its left and upper
// neighbours when |p - q| < threshold (Eigen Vector3f norm, float); runs are
// merged towards the smaller run id; final labels are numbered by the run
// order of each component's root, i.e. by the raster position of each
// component's first pixel.  label_indices has max_id + 1 entries (the last
// one empty), as PCL returns.
void organized_cc(const float* c, int H, int W, float thr,
                  std::vector<uint32_t>& labels,
                  std::vector<std::vector<int>>& label_indices) {
  const uint32_t INV = 0xFFFFFFFFu;
  labels.assign((size_t)H * W, INV);
  std::vector<uint32_t> run_ids;
  auto fin = [&](size_t i) { return std::isfinite(c[4 * i]); };
  auto cmp = [&](size_t a, size_t b) {
    float dx = c[4 * a] - c[4 * b], dy = c[4 * a + 1] - c[4 * b + 1],
          dz = c[4 * a + 2] - c[4 * b + 2];
    float d = std::sqrt(dx * dx + (dy * dy + dz * dz));
    return d < thr;
  };
  auto root = [&](uint32_t r) {
    while (run_ids[r] != r) r = run_ids[r];
    return r;
  };
  uint32_t clust = 0;
  if (fin(0)) {
    labels[0] = clust++;
    run_ids.push_back(labels[0]);
  }
  for (int col = 1; col < W; ++col) {
    if (!fin(col)) continue;
    if (cmp(col, col - 1)) {
      labels[col] = labels[col - 1];
    } else {
      labels[col] = clust++;
      run_ids.push_back(labels[col]);
    }
  }
  for (int row = 1; row < H; ++row) {
    size_t cur = (size_t)row * W, prev = cur - W;
    if (fin(cur)) {
      if (cmp(cur, prev)) {
        labels[cur] = labels[prev];
      } else {
        labels[cur] = clust++;
        run_ids.push_back(labels[cur]);
      }
    }
    for (int col = 1; col < W; ++col) {
      size_t i = cur + col;
      if (!fin(i)) continue;
      if (cmp(i, i - 1)) labels[i] = labels[i - 1];
      if (cmp(i, prev + col)) {
        if (labels[i] == INV) {
          labels[i] = labels[prev + col];
        } else if (labels[prev + col] != INV) {
          uint32_t r1 = root(labels[i]), r2 = root(labels[prev + col]);
          if (r1 < r2) run_ids[r2] = r1;
          else run_ids[r1] = r2;
        }
      }
      if (labels[i] == INV) {
        labels[i] = clust++;
        run_ids.push_back(labels[i]);
      }
    }
  }
  std::vector<uint32_t> map(clust);
  uint32_t max_id = 0;
  for (uint32_t r = 0; r < run_ids.size(); ++r)
    map[r] = (run_ids[r] == r) ? max_id++ : map[root(r)];
  label_indices.assign(max_id + 1, {});
  for (size_t i = 0; i < labels.size(); ++i) {
    if (labels[i] != INV) {
      labels[i] = map[labels[i]];
      label_indices[labels[i]].push_back((int)i);
    }
  }
}

// ==================================================================== a4/a5
// Instance::computeVertexProperties, trellis.cpp:63-102.  The per-axis
// median is the value at index (int)(n/2.0) of each sorted axis (unique
// whatever the sort).  Contract for the point order (which std::sort leaves
// unspecified on ties beyond 16 points): (z, y, x, column) ascending, which
// equals libstdc++'s result whenever n <= 16 (insertion sort, stable).
bool vertex_props(std::vector<Pt>& pts, int variant, float max_d,
                  std::vector<Pt>& kept, Pt& median, double& radius) {
  const int n = (int)pts.size();
  const int mid = (int)(n / 2.0);
  if (variant == ORACLE_LIBM) {
    std::sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& b) { return a.x < b.x; });
    median.x = pts[mid].x;
    std::sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& b) { return a.y < b.y; });
    median.y = pts[mid].y;
    std::sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& b) { return a.z < b.z; });
    median.z = pts[mid].z;
  } else {
    std::vector<float> v(n);
    for (int k = 0; k < n; ++k) v[k] = pts[k].x;
    std::nth_element(v.begin(), v.begin() + mid, v.end());
    median.x = v[mid];
    for (int k = 0; k < n; ++k) v[k] = pts[k].y;
    std::nth_element(v.begin(), v.begin() + mid, v.end());
    median.y = v[mid];
    for (int k = 0; k < n; ++k) v[k] = pts[k].z;
    std::nth_element(v.begin(), v.begin() + mid, v.end());
    median.z = v[mid];
    std::stable_sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& b) {
      if (a.z < b.z) return true;
      if (b.z < a.z) return false;
      if (a.y < b.y) return true;
      if (b.y < a.y) return false;
      return a.x < b.x;
    });
  }
  median.i = 0.0f;
  kept.clear();
  for (const Pt& p : pts)
    if (pcl_euclid(p, median) < max_d) kept.push_back(p);  // :89-93
  if (kept.size() > 1) {
    radius = pcl_euclid(kept.front(), kept.back());  // :95-99
    return true;
  }
  radius = 0.0;
  return false;
}

// Instance::findTrees, trellis.cpp:104-132 (+ computeTreeVertex :45-61).
void find_trees(const sloam_params& P, const float* c, int H, int W,
                const std::vector<uint32_t>& labels,
                const std::vector<std::vector<int>>& label_indices, int variant,
                bool radius_half, std::vector<Tree>& trees,
                std::vector<int>& tree_label) {
  for (size_t i = 0; i < label_indices.size(); ++i) {
    if ((int)label_indices[i].size() <= P.trellis_min_cluster) continue;
    Tree tree;
    for (int row = H - 1; row >= 0; --row) {
      std::vector<Pt> beam;
      for (int col = 0; col < W; ++col) {
        size_t k = (size_t)row * W + col;
        if (labels[k] == i) beam.push_back({c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]});
      }
      if ((int)beam.size() > P.trellis_min_beam_points) {
        Vtx v;
        v.treeId = (int)i;
        v.row = row;
        v.isValid = vertex_props(beam, variant, P.max_dist_to_centroid, v.points, v.coords, v.radius);
        if (radius_half) v.radius *= 0.5;
        if (v.isValid) tree.push_back(std::move(v));
      }
    }
    if ((int)tree.size() > P.trellis_min_vertices) {
      if ((int)tree.size() > P.trellis_max_vertices) tree.resize(P.trellis_max_vertices);
      trees.push_back(std::move(tree));
      tree_label.push_back((int)i);
    }
  }
}

int write_landmarks(const std::vector<Tree>& trees, sloam_landmarks* out) {
  int nl = (int)trees.size(), nv = 0, np = 0;
  for (auto& t : trees) {
    nv += (int)t.size();
    for (auto& v : t) np += (int)v.points.size();
  }
  out->n_landmarks = nl;
  out->n_vertices = nv;
  out->n_points = np;
  if (nl > out->cap_landmarks || nv > out->cap_vertices || np > out->cap_points)
    return SLOAM_ERR_CAPACITY;
  int vi = 0, pi = 0;
  for (int l = 0; l < nl; ++l) {
    out->tree_id[l] = trees[l][0].treeId;
    out->vertex_begin[l] = vi;
    for (auto& v : trees[l]) {
      out->vertex_xyz[3 * vi] = v.coords.x;
      out->vertex_xyz[3 * vi + 1] = v.coords.y;
      out->vertex_xyz[3 * vi + 2] = v.coords.z;
      out->vertex_radius[vi] = v.radius;
      if (out->vertex_row) out->vertex_row[vi] = v.row;
      out->point_begin[vi] = pi;
      for (auto& p : v.points) {
        out->point_xyzi[4 * pi] = p.x;
        out->point_xyzi[4 * pi + 1] = p.y;
        out->point_xyzi[4 * pi + 2] = p.z;
        out->point_xyzi[4 * pi + 3] = p.i;
        ++pi;
      }
      ++vi;
    }
  }
  out->vertex_begin[nl] = vi;
  out->point_begin[vi] = pi;
  return SLOAM_OK;
}

std::vector<Tree> read_landmarks(const sloam_landmarks* lm) {
  std::vector<Tree> trees(lm->n_landmarks);
  for (int l = 0; l < lm->n_landmarks; ++l) {
    for (int v = lm->vertex_begin[l]; v < lm->vertex_begin[l + 1]; ++v) {
      Vtx x;
      x.treeId = lm->tree_id[l];
      x.isValid = true;
      x.coords = {lm->vertex_xyz[3 * v], lm->vertex_xyz[3 * v + 1], lm->vertex_xyz[3 * v + 2], 0.0f};
      x.radius = lm->vertex_radius[v];
      x.row = lm->vertex_row ? lm->vertex_row[v] : 0;
      for (int p = lm->point_begin[v]; p < lm->point_begin[v + 1]; ++p)
        x.points.push_back({lm->point_xyzi[4 * p], lm->point_xyzi[4 * p + 1],
                            lm->point_xyzi[4 * p + 2], lm->point_xyzi[4 * p + 3]});
      trees[l].push_back(std::move(x));
    }
  }
  return trees;
}

// ==================================================================== a7
struct PlaneObj {  // Plane, plane.h / plane.cpp
  double plane[4] = {0, 0, 0, 0};
  V3 centroid{0, 0, 0};
  std::vector<Pt> features;
  bool isValid = false;
  int bin = 0;
};

// The sign of the normal Plane::computeModel gets from
// `JacobiSVD<MatrixX>(centeredGf, ComputeThinU | ComputeThinV).matrixU()
// .col(2)` (plane.cpp:113-115), restated from Eigen 3.3.7 (Ubuntu 20.04's
// libeigen3-dev, the version ROS Noetic builds against; not in the
// reference tree): JacobiSVD::compute (scaling by the largest |entry|), the
// ColPivHouseholderQR preconditioner for more columns than rows (QR of the
// adjoint with column pivoting and norm downdates; work matrix = R^T; U
// starts as the column permutation), the two-sided Jacobi sweep
// (real_2x2_jacobi_svd, JacobiRotation::makeJacobi), the positive-diagonal
// sign fix of U and the descending sort.  Only the third column of U is
// returned; its sign decides the plane gate (sloam.cpp:402-406), where a
// downward normal fails the Euler-angle test.  `a` holds the 3 x n centred
// coordinates row by row.
void eigen_jacobi_svd_u3(const std::vector<double>& a_in, int n, double u3[3]) {
  const double kMin = std::numeric_limits<double>::min();
  const double kEps = std::numeric_limits<double>::epsilon();
  double scale = 0.0;
  for (double v : a_in) scale = std::max(scale, std::fabs(v));
  if (scale == 0.0) scale = 1.0;
  // m = (A / scale)^T, n x 3, column-major: m[j * n + i]
  std::vector<double> m((size_t)3 * n);
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < n; ++i) m[(size_t)r * n + i] = a_in[(size_t)r * n + i] / scale;
  auto col = [&](int j) { return m.data() + (size_t)j * n; };
  // ColPivHouseholderQR::computeInPlace
  double nu[3], nd[3];
  for (int j = 0; j < 3; ++j) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += col(j)[i] * col(j)[i];
    nd[j] = nu[j] = std::sqrt(s);
  }
  const double downdate_thr = std::sqrt(kEps);
  int trans[3];
  const int size = std::min(n, 3);
  for (int k = 0; k < size; ++k) {
    int big = k;
    for (int j = k + 1; j < 3; ++j)
      if (nu[j] > nu[big]) big = j;  // maxCoeff: first index of the maximum
    trans[k] = big;
    if (big != k) {
      for (int i = 0; i < n; ++i) std::swap(col(k)[i], col(big)[i]);
      std::swap(nu[k], nu[big]);
      std::swap(nd[k], nd[big]);
    }
    // makeHouseholderInPlace on col(k)[k..n)
    double* c = col(k);
    double tail = 0;
    for (int i = k + 1; i < n; ++i) tail += c[i] * c[i];
    const double c0 = c[k];
    double tau, beta;
    if (tail <= kMin) {
      tau = 0.0;
      beta = c0;
      for (int i = k + 1; i < n; ++i) c[i] = 0.0;
    } else {
      beta = std::sqrt(c0 * c0 + tail);
      if (c0 >= 0.0) beta = -beta;
      for (int i = k + 1; i < n; ++i) c[i] = c[i] / (c0 - beta);
      tau = (beta - c0) / beta;
    }
    c[k] = beta;
    // applyHouseholderOnTheLeft to the columns right of k, rows k..n
    if (tau != 0.0) {
      for (int j = k + 1; j < 3; ++j) {
        double* x = col(j);
        double tmp = 0;
        for (int i = k + 1; i < n; ++i) tmp += c[i] * x[i];
        tmp += x[k];
        x[k] -= tau * tmp;
        for (int i = k + 1; i < n; ++i) x[i] -= tau * c[i] * tmp;
      }
    }
    for (int j = k + 1; j < 3; ++j) {
      if (nu[j] != 0.0) {
        double t = std::fabs(col(j)[k]) / nu[j];
        t = (1.0 + t) * (1.0 - t);
        t = t < 0.0 ? 0.0 : t;
        const double t2 = t * (nu[j] / nd[j]) * (nu[j] / nd[j]);
        if (t2 <= downdate_thr) {
          double s = 0;
          for (int i = k + 1; i < n; ++i) s += col(j)[i] * col(j)[i];
          nd[j] = nu[j] = std::sqrt(s);
        } else {
          nu[j] *= std::sqrt(t);
        }
      }
    }
  }
  int idx[3] = {0, 1, 2};
  for (int k = 0; k < size; ++k) std::swap(idx[k], idx[trans[k]]);
  // W = R^T (lower triangular), U = the permutation matrix
  double W[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, U[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j <= i; ++j) W[i][j] = col(i)[j];
  for (int i = 0; i < 3; ++i) U[idx[i]][i] = 1.0;
  // rotations: (c, s) applied as x' = c x + s y, y' = -s x + c y
  auto rows = [&](double M[3][3], int p, int q, double c, double s) {
    for (int i = 0; i < 3; ++i) {
      const double x = M[p][i], y = M[q][i];
      M[p][i] = c * x + s * y;
      M[q][i] = -s * x + c * y;
    }
  };
  auto cols = [&](double M[3][3], int p, int q, double c, double s) {  // applyOnTheRight(j)
    for (int i = 0; i < 3; ++i) {
      const double x = M[i][p], y = M[i][q];
      M[i][p] = c * x - s * y;
      M[i][q] = s * x + c * y;
    }
  };
  double maxd = std::max({std::fabs(W[0][0]), std::fabs(W[1][1]), std::fabs(W[2][2])});
  const double precision = 2.0 * kEps;
  bool finished = false;
  for (int sweep = 0; !finished && sweep < 100; ++sweep) {
    finished = true;
    for (int p = 1; p < 3; ++p) {
      for (int q = 0; q < p; ++q) {
        const double thr = std::max(kMin, precision * maxd);
        if (!(std::fabs(W[p][q]) > thr || std::fabs(W[q][p]) > thr)) continue;
        finished = false;
        // real_2x2_jacobi_svd
        double mm[2][2] = {{W[p][p], W[p][q]}, {W[q][p], W[q][q]}};
        const double t = mm[0][0] + mm[1][1], d = mm[1][0] - mm[0][1];
        double c1, s1;
        if (std::fabs(d) < kMin) {
          c1 = 1.0;
          s1 = 0.0;
        } else {
          const double u = t / d, tmp = std::sqrt(1.0 + u * u);
          s1 = 1.0 / tmp;
          c1 = u / tmp;
        }
        for (int i = 0; i < 2; ++i) {
          const double x = mm[0][i], y = mm[1][i];
          mm[0][i] = c1 * x + s1 * y;
          mm[1][i] = -s1 * x + c1 * y;
        }
        // makeJacobi(m(0,0), m(0,1), m(1,1))
        double cr = 1.0, sr = 0.0;
        {
          const double x = mm[0][0], y = mm[0][1], z = mm[1][1];
          const double deno = 2.0 * std::fabs(y);
          if (!(deno < kMin)) {
            const double tau = (x - z) / deno, w = std::sqrt(tau * tau + 1.0);
            const double tt = tau > 0.0 ? 1.0 / (tau + w) : 1.0 / (tau - w);
            const double sign_t = tt > 0.0 ? 1.0 : -1.0;
            const double nn = 1.0 / std::sqrt(tt * tt + 1.0);
            sr = -sign_t * (y / std::fabs(y)) * std::fabs(tt) * nn;
            cr = nn;
          }
        }
        // j_left = rot1 * j_right^T, with j_right^T = (cr, -sr)
        const double lc = c1 * cr - s1 * (-sr), ls = c1 * (-sr) + s1 * cr;
        rows(W, p, q, lc, ls);
        cols(U, p, q, lc, -ls);  // U.applyOnTheRight(p, q, j_left^T)
        cols(W, p, q, cr, sr);
        maxd = std::max({maxd, std::fabs(W[p][p]), std::fabs(W[q][q])});
      }
    }
  }
  double sv[3];
  for (int i = 0; i < 3; ++i) {
    sv[i] = std::fabs(W[i][i]);
    if (W[i][i] < 0.0)
      for (int r = 0; r < 3; ++r) U[r][i] = -U[r][i];
  }
  for (int i = 0; i < 3; ++i) {
    int pos = i;
    for (int j = i + 1; j < 3; ++j)
      if (sv[j] > sv[pos]) pos = j;
    if (sv[pos] == 0.0) break;
    if (pos != i) {
      std::swap(sv[i], sv[pos]);
      for (int r = 0; r < 3; ++r) std::swap(U[r][i], U[r][pos]);
    }
  }
  for (int r = 0; r < 3; ++r) u3[r] = U[r][2];
}

// Plane::computeModel, plane.cpp:96-128.  Centroid accumulated in float in
// feature order (utils.h:14-28); the 3xN SVD normal (left singular vector of
// the smallest singular value) is the eigenvector of the smallest eigenvalue
// of the FP64 scatter matrix, with the sign Eigen's JacobiSVD gives it
// (eigen_jacobi_svd_u3 above).
void plane_model(PlaneObj& pl) {
  Pt cen{0, 0, 0, 0};
  for (const Pt& p : pl.features) {
    cen.x += p.x;
    cen.y += p.y;
    cen.z += p.z;
  }
  double n = (double)pl.features.size();
  cen.x = (float)(cen.x / n);
  cen.y = (float)(cen.y / n);
  cen.z = (float)(cen.z / n);
  double S[9] = {0};
  for (const Pt& p : pl.features) {
    double a[3] = {(double)(p.x - cen.x), (double)(p.y - cen.y), (double)(p.z - cen.z)};
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) S[3 * r + q] += a[r] * a[q];
  }
  double ev[3], V[9];
  jacobi3(S, ev, V);
  V3 nrm{V[0], V[3], V[6]};
  // centeredGf (plane.cpp:102-110): float differences stored as double
  const int nf = (int)pl.features.size();
  std::vector<double> a((size_t)3 * nf);
  for (int i = 0; i < nf; ++i) {
    const Pt& p = pl.features[i];
    a[i] = (double)(p.x - cen.x);
    a[(size_t)nf + i] = (double)(p.y - cen.y);
    a[(size_t)2 * nf + i] = (double)(p.z - cen.z);
  }
  double u3[3];
  eigen_jacobi_svd_u3(a, nf, u3);
  if (nrm.x * u3[0] + nrm.y * u3[1] + nrm.z * u3[2] < 0) nrm = -1.0 * nrm;
  double d = -(nrm.x * cen.x + nrm.y * cen.y + nrm.z * cen.z);
  pl.plane[0] = nrm.x; pl.plane[1] = nrm.y; pl.plane[2] = nrm.z; pl.plane[3] = d;
  pl.centroid = {cen.x, cen.y, cen.z};
}

// Plane::Plane, plane.cpp:3-17
PlaneObj make_plane(const std::vector<Pt>& pts, const sloam_params& P) {
  PlaneObj pl;
  pl.features = pts;
  if ((int)pl.features.size() < P.num_ground_features || pl.features.size() < 3) {
    pl.isValid = false;  // (< 3 points: the reference's thin SVD is undefined)
  } else {
    plane_model(pl);
    pl.features.resize(P.num_ground_features);
    pl.isValid = true;
  }
  return pl;
}

// Plane::distance(point), plane.cpp:136-151
double plane_dist_point(const PlaneObj& pl, V3 p) {
  return std::abs(pl.plane[0] * p.x + pl.plane[1] * p.y + pl.plane[2] * p.z + pl.plane[3]) /
         norm({pl.plane[0], pl.plane[1], pl.plane[2]});
}

// Plane::project, plane.cpp:153-176 (model part): plane' = T^-T plane,
// centroid' = T centroid.
void plane_project(PlaneObj& pl, const SE3& T) {
  V3 n{pl.plane[0], pl.plane[1], pl.plane[2]};
  V3 n2 = rot(T.R, n);
  double d2 = pl.plane[3] - dot(T.t, n2);
  pl.plane[0] = n2.x; pl.plane[1] = n2.y; pl.plane[2] = n2.z; pl.plane[3] = d2;
  pl.centroid = xf(T, pl.centroid);
}

// sloam::binGroundPoints, sloam.cpp:330-386, pose = identity (as called at
// :392).  theta uses the float atan2 overload (contract: correctly rounded).
// Retained points of a bin are its lowest int(size/retainNum) by z; contract
// for ties in z: lower point index first.
void bin_ground(const sloam_params& P, const float* g, int n, int variant,
                std::vector<std::vector<Pt>>& bins) {
  const int Rb = P.ground_radii_bins, Tb = P.ground_theta_bins;
  bins.assign((size_t)Rb * Tb, {});
  std::vector<std::vector<int>> idx((size_t)Rb * Tb);
  Pt origin{0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    Pt p{g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]};
    double r = euclid2d(origin, p);
    if (r < P.max_ground_lidar_dist && r > P.min_ground_lidar_dist) {
      float th_f = (variant == ORACLE_LIBM)
                       ? std::atan2(p.y - origin.y, p.x - origin.x)
                       : (float)std::atan2((double)(p.y - origin.y), (double)(p.x - origin.x));
      double th = th_f;
      int rb = (int)std::floor(r / (P.max_ground_lidar_dist / (double)Rb));
      int tb = (int)std::floor((kPIDEF + th) / (2 * kPIDEF / (double)Tb));
      rb = std::max(0, std::min(rb, Rb - 1));
      tb = std::max(0, std::min(tb, Tb - 1));
      bins[(size_t)rb * Tb + tb].push_back(p);
      idx[(size_t)rb * Tb + tb].push_back(i);
    }
  }
  for (size_t b = 0; b < bins.size(); ++b) {
    auto& v = bins[b];
    if (v.empty()) continue;
    double retainNum = 1 / P.ground_retain_thresh;
    if (retainNum < v.size()) {
      int bottom = (int)(v.size() / retainNum);
      std::vector<int> ord(v.size());
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return v[a].z < v[c].z; });
      std::vector<Pt> s;
      for (int k = 0; k < bottom; ++k) s.push_back(v[ord[k]]);
      v.swap(s);
    }
  }
}

// Eigen Quaternion::setFromTwoVectors + toRotationMatrix + eulerAngles(0,1,2)
// (Eigen 3.3 Quaternion.h / EulerAngles.h, restated).  Returns the three
// Euler angles of the rotation taking a to b.
void euler_from_two_vectors(V3 a, V3 b, double ang[3]) {
  V3 v0 = (1.0 / norm(a)) * a, v1 = (1.0 / norm(b)) * b;
  double c = dot(v1, v0);
  double qx, qy, qz, qw;
  if (c < -1.0 + 1e-12) {
    c = std::max(c, -1.0);
    V3 axis = std::fabs(v0.x) < 0.9 ? cross(v0, {1, 0, 0}) : cross(v0, {0, 1, 0});
    axis = (1.0 / norm(axis)) * axis;
    double w2 = (1.0 + c) * 0.5;
    qw = std::sqrt(w2);
    double s = std::sqrt(1.0 - w2);
    qx = axis.x * s; qy = axis.y * s; qz = axis.z * s;
  } else {
    V3 axis = cross(v0, v1);
    double s = std::sqrt((1.0 + c) * 2.0);
    double invs = 1.0 / s;
    qx = axis.x * invs; qy = axis.y * invs; qz = axis.z * invs;
    qw = s * 0.5;
  }
  double tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
  double twx = tx * qw, twy = ty * qw, twz = tz * qw;
  double txx = tx * qx, txy = ty * qx, txz = tz * qx;
  double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  double M[3][3] = {{1 - (tyy + tzz), txy - twz, txz + twy},
                    {txy + twz, 1 - (txx + tzz), tyz - twx},
                    {txz - twy, tyz + twx, 1 - (txx + tyy)}};
  // eulerAngles(0,1,2): i=0, j=1, k=2, odd=0 (Graphics Gems IV)
  double r0 = std::atan2(M[1][2], M[2][2]);
  double c2 = std::hypot(M[0][0], M[0][1]);
  double r1;
  if (r0 > 0) {
    r0 -= M_PI;
    r1 = std::atan2(-M[0][2], -c2);
  } else {
    r1 = std::atan2(-M[0][2], c2);
  }
  double s1 = std::sin(r0), c1 = std::cos(r0);
  double r2 = std::atan2(s1 * M[2][0] - c1 * M[1][0], c1 * M[1][1] - s1 * M[2][1]);
  ang[0] = -r0; ang[1] = -r1; ang[2] = -r2;
}

// sloam::computeModels ground part, sloam.cpp:390-412.
void ground_planes(const sloam_params& P, const SE3& pose, const float* g, int n,
                   int variant, std::vector<PlaneObj>& planes) {
  std::vector<std::vector<Pt>> bins;
  bin_ground(P, g, n, variant, bins);
  const int Rb = P.ground_radii_bins, Tb = P.ground_theta_bins;
  for (int r = 0; r < Rb; ++r) {
    for (int t = 0; t < Tb; ++t) {
      PlaneObj pl = make_plane(bins[(size_t)r * Tb + t], P);
      pl.bin = r * Tb + t;
      if (!pl.isValid) continue;
      V3 nw = rot(pose.R, {pl.plane[0], pl.plane[1], pl.plane[2]});  // (T^-1)^T plane
      double ang[3];
      euler_from_two_vectors({0, 0, 1}, nw, ang);
      bool angleCheck = (ang[0] < 0.1 && ang[1] < 0.1 && ang[2] < 0.1) ||
                        (M_PI - std::abs(ang[0]) < 0.1 && M_PI - std::abs(ang[1]) < 0.1 &&
                         M_PI - std::abs(ang[2]) < 0.1);
      bool heightCheck = xf(pose, pl.centroid).z < pose.t.z;
      if (angleCheck && heightCheck) planes.push_back(std::move(pl));
    }
  }
}

// ==================================================================== a6
struct CylObj {  // Cylinder, cylinder.h / cylinder.cpp
  V3 root{0, 0, 0}, ray{0, 0, 0};
  double radius = 0;
  std::vector<Pt> features;
  int id = 0;
  bool isValid = false;
  int inliers = 0;
};

// rayPlaneIntersection, utils.h:41-51
V3 ray_plane(V3 c, V3 nrm, V3 o, V3 d) {
  float denom = dot(nrm, d);
  if (std::abs(denom) > 0.001f) {
    float t = dot(c - o, nrm) / denom;
    if (t >= 0.001f) return o + (double)t * d;
  }
  return o;
}

// PCL SampleConsensusModelLine::optimizeModelCoefficients restated: the line
// through the inliers' centroid along the eigenvector of the largest
// eigenvalue of their scatter matrix; the eigenvector's sign follows
// pcl::computeCorrespondingEigenVector (the largest of the three row cross
// products of (S - lambda I)), computed here in FP64.
V3 pcl_line_direction(const double S[9]) {
  double ev[3], V[9];
  jacobi3(S, ev, V);
  double lam = ev[2];
  double scale = 0;
  for (int k = 0; k < 9; ++k) scale = std::max(scale, std::fabs(S[k]));
  if (scale <= std::numeric_limits<double>::min()) scale = 1.0;
  double M[9];
  for (int k = 0; k < 9; ++k) M[k] = S[k] / scale;
  M[0] -= lam / scale; M[4] -= lam / scale; M[8] -= lam / scale;
  V3 r0{M[0], M[1], M[2]}, r1{M[3], M[4], M[5]}, r2{M[6], M[7], M[8]};
  V3 c1 = cross(r0, r1), c2 = cross(r0, r2), c3 = cross(r1, r2);
  double l1 = dot(c1, c1), l2 = dot(c2, c2), l3 = dot(c3, c3);
  V3 v;
  if (l1 >= l2 && l1 >= l3) v = (1.0 / std::sqrt(l1)) * c1;
  else if (l2 >= l1 && l2 >= l3) v = (1.0 / std::sqrt(l2)) * c2;
  else v = (1.0 / std::sqrt(l3)) * c3;
  if (!(std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z)))
    v = {V[2], V[5], V[8]};
  return v;
}

// Vertex-line RANSAC replacing pcl::SACSegmentation(SACMODEL_LINE, SAC_RANSAC,
// threshold 0.25, optimise) at cylinder.cpp:115-139.  Contract:
//  - hypothesis h (0 <= h < line_ransac_max_iter) samples two distinct
//    vertices with Philox(seed, (h, tree id, 0, 0));
//  - identical points are a degenerate sample (skipped, not an iteration);
//  - inliers: |(p1 - c) x dir|^2 < thr^2 in float, dir = (p2-p1)/|p2-p1|;
//  - PCL's sequential RandomSampleConsensus stopping rule is applied over
//    the hypotheses in order (k = log(1-p) / log(1 - w^2));
//  - refinement as pcl_line_direction through the best model's inliers, then
//    the inliers are re-selected with the refined line (FP64).
// Returns false where PCL returns no inliers.
bool line_ransac(const sloam_params& P, const std::vector<Pt>& C, int tree_id,
                 V3& dir_out, int& best_count_out) {
  const int V = (int)C.size();
  if (V < 2) return false;
  const float thr2 = (float)(P.line_ransac_thresh * P.line_ransac_thresh);
  const int K = P.line_ransac_max_iter;
  int best = -1, best_count = 0, it = 0;
  double k = 1.0;
  const double log_p = std::log(1.0 - P.line_ransac_probability);
  const double eps = std::numeric_limits<double>::epsilon();
  float bdx = 0, bdy = 0, bdz = 0;
  for (int h = 0; h < K; ++h) {
    if (!(it < k)) break;
    uint32_t ctr[4] = {(uint32_t)h, (uint32_t)tree_id, 0u, 0u}, u[4], id[2];
    philox(P.seed, ctr, u);
    draw_distinct(u, (uint32_t)V, 2, id);
    const Pt& a = C[id[0]];
    const Pt& b = C[id[1]];
    float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    float nn = (dx * dx + dy * dy) + dz * dz;
    if (nn == 0.0f) continue;  // degenerate sample
    float nr = std::sqrt(nn);
    dx = dx / nr; dy = dy / nr; dz = dz / nr;
    int cnt = 0;
    for (int j = 0; j < V; ++j) {
      float vx = a.x - C[j].x, vy = a.y - C[j].y, vz = a.z - C[j].z;
      float cx = vy * dz - vz * dy, cy = vz * dx - vx * dz, cz = vx * dy - vy * dx;
      float sq = (cx * cx + cy * cy) + cz * cz;
      if (sq < thr2) ++cnt;
    }
    if (cnt > best_count) {
      best_count = cnt;
      best = h;
      bdx = dx; bdy = dy; bdz = dz;
      double w = (double)best_count / V;
      double p_no = 1.0 - w * w;
      p_no = std::max(eps, std::min(1.0 - eps, p_no));
      k = log_p / std::log(p_no);
    }
    ++it;
  }
  best_count_out = best_count;
  if (best < 0) return false;
  // best model's inliers
  uint32_t ctr[4] = {(uint32_t)best, (uint32_t)tree_id, 0u, 0u}, u[4], id[2];
  philox(P.seed, ctr, u);
  draw_distinct(u, (uint32_t)V, 2, id);
  const Pt& a = C[id[0]];
  std::vector<int> inl;
  for (int j = 0; j < V; ++j) {
    float vx = a.x - C[j].x, vy = a.y - C[j].y, vz = a.z - C[j].z;
    float cx = vy * bdz - vz * bdy, cy = vz * bdx - vx * bdz, cz = vx * bdy - vy * bdx;
    float sq = (cx * cx + cy * cy) + cz * cz;
    if (sq < thr2) inl.push_back(j);
  }
  V3 c{a.x, a.y, a.z}, d{bdx, bdy, bdz};
  if (inl.size() > 2) {  // PCL keeps the raw model for <= sample size inliers
    V3 m{0, 0, 0};
    for (int j : inl) m = m + V3{C[j].x, C[j].y, C[j].z};
    m = (1.0 / inl.size()) * m;
    double S[9] = {0};
    for (int j : inl) {
      double q[3] = {C[j].x - m.x, C[j].y - m.y, C[j].z - m.z};
      for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s) S[3 * r + s] += q[r] * q[s];
    }
    c = m;
    d = pcl_line_direction(S);
  }
  int reinl = 0;
  for (int j = 0; j < V; ++j) {
    V3 q = V3{C[j].x, C[j].y, C[j].z} - c;
    V3 x = cross(q, d);
    if (dot(x, x) < P.line_ransac_thresh * P.line_ransac_thresh) ++reinl;
  }
  if (reinl == 0) return false;
  // pcl::ModelCoefficients stores floats (cylinder.cpp:137-139)
  dir_out = {(double)(float)d.x, (double)(float)d.y, (double)(float)d.z};
  return true;
}

// Point-level cylinder RANSAC + LS refinement (this project's extension of
// the cylinder fit; no reference counterpart).  Contract:
//  - frame: o = the landmark's vertex[1] median, prior axis a = the vertex
//    line direction (float, z >= 0); e1 = normalize(a x t) with
//    t = (1,0,0) if |a.x| < 0.9 else (0,1,0), e2 = a x e1;
//    u_i = (q_i - o).e1, v_i = (q_i - o).e2 (float, left-to-right sums);
//  - hypothesis h samples 3 distinct points with Philox(seed,(h,tree,1,0)),
//    fits the circle through them in (u,v); degenerate when the determinant
//    is 0 or the radius is not <= cyl_max_hyp_radius;
//  - inlier: lo2 < du^2 + dv^2 < hi2 with lo = r - tau (lo2 = -1 if lo <= 0),
//    hi = r + tau; best = most inliers, lowest h on ties;
//  - cyl_ls_iters Gauss-Newton steps (FP64 here) over the best inliers on
//    (axis point, axis direction, radius); a failed solve stops early.
// Returns the best inlier count (0 if no hypothesis).
int point_cylinder(const sloam_params& P, const std::vector<Pt>& Q, Pt o, V3 prior,
                   int tree_id, V3& c_out, V3& d_out, double& r_out) {
  const int n = (int)Q.size();
  if (n < 3 || P.cyl_hypotheses <= 0) return 0;
  float ax = (float)prior.x, ay = (float)prior.y, az = (float)prior.z;
  if (az < 0) { ax = -ax; ay = -ay; az = -az; }
  float tx = 1.0f, ty = 0.0f, tz = 0.0f;
  if (!(std::fabs(ax) < 0.9f)) { tx = 0.0f; ty = 1.0f; }
  float e1x = ay * tz - az * ty, e1y = az * tx - ax * tz, e1z = ax * ty - ay * tx;
  float e1n = std::sqrt((e1x * e1x + e1y * e1y) + e1z * e1z);
  e1x = e1x / e1n; e1y = e1y / e1n; e1z = e1z / e1n;
  float e2x = ay * e1z - az * e1y, e2y = az * e1x - ax * e1z, e2z = ax * e1y - ay * e1x;
  std::vector<float> U(n), Vv(n);
  for (int i = 0; i < n; ++i) {
    float dx = Q[i].x - o.x, dy = Q[i].y - o.y, dz = Q[i].z - o.z;
    U[i] = (dx * e1x + dy * e1y) + dz * e1z;
    Vv[i] = (dx * e2x + dy * e2y) + dz * e2z;
  }
  const float tau = P.cyl_inlier_thresh;
  int best = -1, best_cnt = 0;
  float bcu = 0, bcv = 0, br = 0, blo2 = 0, bhi2 = 0;
  for (int h = 0; h < P.cyl_hypotheses; ++h) {
    uint32_t ctr[4] = {(uint32_t)h, (uint32_t)tree_id, 1u, 0u}, u[4], id[3];
    philox(P.seed, ctr, u);
    draw_distinct(u, (uint32_t)n, 3, id);
    float p0u = U[id[0]], p0v = Vv[id[0]];
    float bx_ = U[id[1]] - p0u, by_ = Vv[id[1]] - p0v;
    float cx_ = U[id[2]] - p0u, cy_ = Vv[id[2]] - p0v;
    float t1 = bx_ * cy_, t2 = by_ * cx_;
    float den = 2.0f * (t1 - t2);
    if (den == 0.0f) continue;
    float b2 = bx_ * bx_ + by_ * by_, c2 = cx_ * cx_ + cy_ * cy_;
    float ox = (cy_ * b2 - by_ * c2) / den;
    float oy = (bx_ * c2 - cx_ * b2) / den;
    float r = std::sqrt(ox * ox + oy * oy);
    if (!(r <= P.cyl_max_hyp_radius)) continue;
    float cu = p0u + ox, cv = p0v + oy;
    float lo = r - tau, hi = r + tau;
    float lo2 = lo > 0.0f ? lo * lo : -1.0f;
    float hi2 = hi * hi;
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
      float du = U[i] - cu, dv = Vv[i] - cv;
      float d2 = du * du + dv * dv;
      if (d2 > lo2 && d2 < hi2) ++cnt;
    }
    if (cnt > best_cnt) {
      best_cnt = cnt; best = h;
      bcu = cu; bcv = cv; br = r; blo2 = lo2; bhi2 = hi2;
    }
  }
  if (best < 0) return 0;
  std::vector<int> inl;
  for (int i = 0; i < n; ++i) {
    float du = U[i] - bcu, dv = Vv[i] - bcv;
    float d2 = du * du + dv * dv;
    if (d2 > blo2 && d2 < bhi2) inl.push_back(i);
  }
  // LS refinement, FP64
  V3 d{ax, ay, az};
  d = (1.0 / norm(d)) * d;
  V3 e1{e1x, e1y, e1z}, e2{e2x, e2y, e2z};
  V3 c = V3{o.x, o.y, o.z} + (double)bcu * e1 + (double)bcv * e2;
  double r = br;
  for (int itn = 0; itn < P.cyl_ls_iters; ++itn) {
    V3 t = std::fabs(d.x) < 0.9 ? V3{1, 0, 0} : V3{0, 1, 0};
    V3 b1 = cross(d, t);
    b1 = (1.0 / norm(b1)) * b1;
    V3 b2 = cross(d, b1);
    double H[25] = {0}, g[5] = {0};
    for (int i : inl) {
      V3 w = V3{Q[i].x, Q[i].y, Q[i].z} - c;
      double wd = dot(w, d);
      V3 wp = w - wd * d;
      double rho = norm(wp);
      if (!(rho > 0)) continue;
      double res = rho - r;
      double a1 = dot(wp, b1) / rho, a2 = dot(wp, b2) / rho;
      double J[5] = {-a1, -a2, -wd * a1, -wd * a2, -1.0};
      for (int p = 0; p < 5; ++p) {
        g[p] += J[p] * res;
        for (int q = 0; q < 5; ++q) H[5 * p + q] += J[p] * J[q];
      }
    }
    double mg[5] = {-g[0], -g[1], -g[2], -g[3], -g[4]}, dx[5];
    if (!chol_solve(5, H, mg, dx)) break;
    c = c + dx[0] * b1 + dx[1] * b2;
    d = d + dx[2] * b1 + dx[3] * b2;
    d = (1.0 / norm(d)) * d;
    r = r + dx[4];
  }
  if (d.z < 0) d = -1.0 * d;
  c_out = c; d_out = d; r_out = r;
  return best_cnt;
}

// Cylinder::Cylinder + computeModel + groundBasedRoot + filter,
// cylinder.cpp:3-28, 41-173.
CylObj make_cylinder(const sloam_params& P, const Tree& vt, const PlaneObj& gp,
                     const std::vector<Pt>* cluster) {
  CylObj cy;
  cy.isValid = false;
  const int V = (int)vt.size();
  if (V < 3) return cy;  // the reference indexes vertices[1], [2], [V-2]
  Pt centroid{(float)gp.centroid.x, (float)gp.centroid.y, (float)gp.centroid.z, 0};
  bool within = euclid2d(vt[1].coords, centroid) < P.max_lidar_dist;  // :11-13
  if (!within) return cy;
  // ---- computeModel, :75-173
  const Vtx& firstVtx = vt[2];
  std::vector<float> validRadii;
  std::vector<Pt> coords;
  for (const Vtx& v : vt) {
    coords.push_back(v.coords);
    for (Pt p : v.points) {
      p.i = (float)firstVtx.treeId;
      cy.features.push_back(p);
    }
    if (v.points.size() > 3) validRadii.push_back((float)v.radius);
  }
  cy.id = firstVtx.treeId;
  Pt bottom = vt[1].coords, top = vt[V - 2].coords;
  cy.root = {bottom.x, bottom.y, bottom.z};
  bool model_ok = true;
  if (eigen_sqnorm3f(bottom, top) < P.min_tree_height_sq || coords.empty()) {
    cy.radius = -1;
    model_ok = false;
  }
  V3 dir{0, 0, 1};
  if (model_ok) {
    if (!line_ransac(P, coords, cy.id, dir, cy.inliers)) {
      cy.radius = -1;
      model_ok = false;
    }
  }
  if (model_ok) {
    cy.ray = dir;
    if (!validRadii.empty()) {
      std::sort(validRadii.begin(), validRadii.end());
      int d = (int)(std::find_if(validRadii.begin(), validRadii.end(),
                                 [](float x) { return x > 0; }) - validRadii.begin());
      int middle = std::min((int)(validRadii.size() - 1),
                            (d + 1) + (int)((validRadii.size() - d) / 2));
      cy.radius = validRadii[middle];
      if (cy.radius == 0) cy.radius = -1;
      else if (cy.radius < P.default_tree_radius) cy.radius = P.default_tree_radius;
    } else {
      cy.radius = -1;
    }
    if (P.cyl_mode == 1 && cy.radius != -1) {
      std::vector<Pt> pts;
      if (cluster && !cluster->empty()) pts = *cluster;
      else
        for (const Vtx& v : vt) pts.insert(pts.end(), v.points.begin(), v.points.end());
      V3 c, d;
      double r;
      int cnt = point_cylinder(P, pts, vt[1].coords, dir, cy.id, c, d, r);
      if (cnt > 0) {
        cy.inliers = cnt;
        cy.ray = d;
        cy.radius = r > 0 ? r : -1;
        V3 b{vt[1].coords.x, vt[1].coords.y, vt[1].coords.z};
        cy.root = c + dot(b - c, d) * d;
      }
    }
    cy.features.resize(P.features_per_tree, Pt{0, 0, 0, 0});  // :172
  }
  // ---- groundBasedRoot, :41-55
  bool validZ = false;
  {
    const double* g = gp.plane;
    V3 n{g[0], g[1], g[2]};
    float dist = std::abs(g[0] * cy.root.x + g[1] * cy.root.y + g[2] * cy.root.z + g[3]) / norm(n);
    if (dist < P.root_plane_max_dist) {
      cy.root = ray_plane(gp.centroid, n, cy.root, cy.ray);
      validZ = true;
    }
  }
  bool validNorm = norm(cy.root) > 0.01;
  bool validRadius = cy.radius > 0.0;
  // ---- filter, :57-73
  bool validTree = false;
  if (cy.radius != -1) {
    V3 up{gp.plane[0], gp.plane[1], gp.plane[2]};
    double theta = (180 / kPIDEF) * std::acos(dot(cy.ray, up) / (norm(cy.ray) * norm(up)));
    validTree = (cy.radius < P.max_tree_radius) &&
                ((theta <= P.max_axis_theta) || (theta >= 180 - P.max_axis_theta));
  }
  cy.isValid = validZ && validRadius && validTree && validNorm;
  return cy;
}

// Cylinder::distance(model), cylinder.cpp:175-194 (self = map object)
double cyl_dist_model(const CylObj& self, const CylObj& tgt) {
  const double hs[3] = {0.0, 3.0, 6.0};
  double dsum = 0.0;
  for (double h : hs) {
    double st = (h - self.root.z) / self.ray.z;
    V3 mp = self.root + st * self.ray;
    double tt = (h - tgt.root.z) / tgt.ray.z;
    V3 tp = tgt.root + tt * tgt.ray;
    dsum += norm(mp - tp);
  }
  return dsum / 3.0;
}
// Cylinder::distance(point), cylinder.cpp:196-203
double cyl_dist_point(const CylObj& c, V3 p) {
  V3 pp = c.root + (dot(p - c.root, c.ray) / dot(c.ray, c.ray)) * c.ray;
  return norm(p - pp) - c.radius;
}
// Cylinder::project, cylinder.cpp:205-211
void cyl_project(CylObj& c, const SE3& T) {
  V3 other = c.root + c.ray;
  c.root = xf(T, c.root);
  other = xf(T, other);
  c.ray = other - c.root;
}

// sloam::computeModels, sloam.cpp:388-436
void compute_models(const sloam_params& P, const SE3& pose, const float* g, int ng,
                    const std::vector<Tree>& trees,
                    const std::vector<std::vector<Pt>>* clusters,
                    std::vector<PlaneObj>& planes, std::vector<CylObj>& cyls) {
  ground_planes(P, pose, g, ng, ORACLE_CONTRACT, planes);
  if (planes.empty()) return;  // :414-415
  for (size_t l = 0; l < trees.size(); ++l) {
    const Tree& t = trees[l];
    if (t.size() < 2) continue;
    V3 pos{t[1].coords.x, t[1].coords.y, t[1].coords.z};
    double bestDist = 100000;
    size_t best = 0;
    for (size_t k = 0; k < planes.size(); ++k) {
      double d = plane_dist_point(planes[k], pos);
      if (d < bestDist) {
        bestDist = d;
        best = k;
      }
    }
    const std::vector<Pt>* cl = (clusters && l < clusters->size()) ? &(*clusters)[l] : nullptr;
    CylObj c = make_cylinder(P, t, planes[best], cl);
    if (c.isValid) cyls.push_back(std::move(c));
  }
}

// ==================================================================== a9
struct Match {
  V3 feat;
  int obj;  // index into the map list
};

// matchFeatures<T> + addFeatureMatches, sloam.cpp:257-296.  Contract: an
// empty map gives no matches (the reference indexes mapObjects[0]).
template <typename T, typename DistFn, typename ProjFn>
std::vector<Match> match_features(const SE3& tf, const std::vector<T>& cur,
                                  const std::vector<T>& map, double thr, DistFn dist,
                                  ProjFn proj) {
  std::vector<Match> m;
  if (map.empty()) return m;
  for (const T& co : cur) {
    T pobj = co;
    proj(pobj, tf);
    double bestDist = thr + 100;
    int best = 0;
    for (size_t k = 0; k < map.size(); ++k) {
      double d = dist(map[k], pobj);
      if (d < bestDist) {
        bestDist = d;
        best = (int)k;
      }
    }
    if (bestDist < thr)
      for (const Pt& f : co.features) m.push_back({{f.x, f.y, f.z}, best});
  }
  return m;
}

// ==================================================================== a10
// Pose update contract (replaces Ceres LM at sloam.cpp:33-255): fixed
// gn_iters Gauss-Newton iterations with IRLS Huber weights
// (w = 1 if |r| <= delta else delta/|r|), FP64 normal equations solved by
// Cholesky.  Residuals: point-to-cylinder |lp - proj_axis(lp)| - radius
// (cylinder.h:42-132), point-to-plane |n.lp + d| / |n| (plane.h:34-116).
// Computation is done in a frame anchored at the pose estimate's translation.
struct CylRes {
  V3 p, root, ray;
  double radius;
};
struct PlaneRes {
  V3 p, n;
  double d;
};

inline double huber_w(double r, double delta) {
  double a = std::fabs(r);
  return a <= delta ? 1.0 : delta / a;
}
// residual + gradient wrt lp
inline double cyl_res(const CylRes& m, V3 lp, V3& J) {
  V3 v = lp - m.root;
  double s = dot(v, m.ray) / dot(m.ray, m.ray);
  V3 w = v - s * m.ray;
  double nw = norm(w);
  J = nw > 0 ? (1.0 / nw) * w : V3{0, 0, 0};
  return nw - m.radius;
}
inline double plane_res(const PlaneRes& m, V3 lp, V3& J) {
  double num = dot(m.n, lp) + m.d;
  double nn = norm(m.n);
  double sg = num > 0 ? 1.0 : (num < 0 ? -1.0 : 0.0);
  J = (sg / nn) * m.n;
  return std::fabs(num) / nn;
}

void so3_exp(V3 w, double* R) {
  double th2 = dot(w, w), th = std::sqrt(th2);
  double A, B;
  if (th2 < 1e-24) {
    A = 1.0; B = 0.5;
  } else {
    A = std::sin(th) / th;
    B = (1.0 - std::cos(th)) / th2;
  }
  double K[9] = {0, -w.z, w.y, w.z, 0, -w.x, -w.y, w.x, 0};
  double K2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += K[3 * i + k] * K[3 * k + j];
      K2[3 * i + j] = s;
    }
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0 ? 1.0 : 0.0) + A * K[i] + B * K2[i];
}
void matmul3(const double* A, const double* B, double* C) {
  double T[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += A[3 * i + k] * B[3 * k + j];
      T[3 * i + j] = s;
    }
  std::memcpy(C, T, sizeof(T));
}

bool optimize_joint_lm(const sloam_params& P, const SE3& est, const std::vector<CylRes>& cr,
                       const std::vector<PlaneRes>& pr, SE3& out);

// OptimizePose (joint, quaternion + translation), sloam.cpp:174-255.
bool optimize_joint(const sloam_params& P, const SE3& est, const std::vector<CylRes>& cr,
                    const std::vector<PlaneRes>& pr, SE3& out) {
  if (P.pose_solver == 1) return optimize_joint_lm(P, est, cr, pr, out);
  V3 a = est.t;
  double R[9];
  std::memcpy(R, est.R, sizeof(R));
  V3 t{0, 0, 0};
  std::vector<CylRes> C = cr;
  std::vector<PlaneRes> Pl = pr;
  for (auto& m : C) m.root = m.root - a;
  for (auto& m : Pl) m.d = m.d + dot(m.n, a);
  const double delta = P.huber_delta;
  for (int it = 0; it < P.gn_iters; ++it) {
    double H[36] = {0}, g[6] = {0};
    auto acc = [&](double res, V3 Jl, V3 q) {
      V3 Jw = cross(q, Jl);
      double J[6] = {Jw.x, Jw.y, Jw.z, Jl.x, Jl.y, Jl.z};
      double w = huber_w(res, delta);
      for (int i = 0; i < 6; ++i) {
        g[i] += w * J[i] * res;
        for (int j = 0; j < 6; ++j) H[6 * i + j] += w * J[i] * J[j];
      }
    };
    for (auto& m : C) {
      V3 q = rot(R, m.p), lp = q + t, J;
      double r = cyl_res(m, lp, J);
      acc(r, J, q);
    }
    for (auto& m : Pl) {
      V3 q = rot(R, m.p), lp = q + t, J;
      double r = plane_res(m, lp, J);
      acc(r, J, q);
    }
    double mg[6], dx[6];
    for (int i = 0; i < 6; ++i) mg[i] = -g[i];
    if (!chol_solve(6, H, mg, dx)) return false;
    double dR[9];
    so3_exp({dx[0], dx[1], dx[2]}, dR);
    matmul3(dR, R, R);
    t = t + V3{dx[3], dx[4], dx[5]};
  }
  std::memcpy(out.R, R, sizeof(R));
  out.t = t + a;
  return true;
}

// Ceres QuaternionToAngleAxis / AngleAxisToQuaternion (rotation.h), restated.
void quat_to_aa(const double* qwxyz, double* aa) {
  double q1 = qwxyz[1], q2 = qwxyz[2], q3 = qwxyz[3];
  double s2 = q1 * q1 + q2 * q2 + q3 * q3;
  if (s2 > 0.0) {
    double s = std::sqrt(s2), c = qwxyz[0];
    double two_theta = 2.0 * ((c < 0.0) ? std::atan2(-s, -c) : std::atan2(s, c));
    double k = two_theta / s;
    aa[0] = q1 * k; aa[1] = q2 * k; aa[2] = q3 * k;
  } else {
    aa[0] = q1 * 2.0; aa[1] = q2 * 2.0; aa[2] = q3 * 2.0;
  }
}
void aa_to_quat(const double* aa, double* qwxyz) {
  double t2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (t2 > 0.0) {
    double th = std::sqrt(t2), h = th * 0.5, k = std::sin(h) / th;
    qwxyz[0] = std::cos(h); qwxyz[1] = aa[0] * k; qwxyz[2] = aa[1] * k; qwxyz[3] = aa[2] * k;
  } else {
    qwxyz[0] = 1.0; qwxyz[1] = aa[0] * 0.5; qwxyz[2] = aa[1] * 0.5; qwxyz[3] = aa[2] * 0.5;
  }
}
// R(r) (Rodrigues) and d(R(r) p)/dr = -R [p]x Jr(r).
void aa_rotate_jac(const double* r, V3 p, V3& out, double Jr3[9]) {
  double th2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (th2 > std::numeric_limits<double>::epsilon()) {
    double th = std::sqrt(th2);
    double R[9];
    so3_exp({r[0], r[1], r[2]}, R);
    out = rot(R, p);
    double A = (1.0 - std::cos(th)) / th2, B = (th - std::sin(th)) / (th2 * th);
    double K[9] = {0, -r[2], r[1], r[2], 0, -r[0], -r[1], r[0], 0}, K2[9], Jr[9];
    matmul3(K, K, K2);
    for (int i = 0; i < 9; ++i) Jr[i] = (i % 4 == 0 ? 1.0 : 0.0) - A * K[i] + B * K2[i];
    double Px[9] = {0, -p.z, p.y, p.z, 0, -p.x, -p.y, p.x, 0}, T1[9];
    matmul3(R, Px, T1);
    matmul3(T1, Jr, Jr3);
    for (int i = 0; i < 9; ++i) Jr3[i] = -Jr3[i];
  } else {
    V3 w{r[0], r[1], r[2]};
    out = p + cross(w, p);
    double Px[9] = {0, -p.z, p.y, p.z, 0, -p.x, -p.y, p.x, 0};
    for (int i = 0; i < 9; ++i) Jr3[i] = -Px[i];
  }
}

// ---- a10 with pose_solver 1: trust-region Levenberg-Marquardt ----------
// The solver settings the reference gives Ceres (sloam.cpp:91-97,
// 149-155: at most max_num_iterations = 50, the rest default), restated
// from Ceres' documented behaviour:
//  - cost 1/2 sum rho(r^2), Huber rho with delta = huber_delta; residuals
//    and Jacobian rows rescaled by sqrt(rho'), which for a loss with
//    rho'' <= 0 (Huber) is the whole robust correction: H = sum w J J^T,
//    g = sum w J r with w = rho'(r^2) (the IRLS weight of the GN path);
//  - Jacobi scaling: column i scaled by 1 / (1 + sqrt(H_ii));
//  - LM step: (Hs + D / radius) ds = -gs, D = diag(Hs) clamped to
//    [1e-6, 1e32]; predicted decrease -(g.d + d.H.d / 2);
//  - ratio = actual / predicted decrease; a step is taken when it is above
//    1e-3: radius /= max(1/3, 1 - (2 ratio - 1)^3) (at most 1e16) and the
//    shrink factor returns to 2; otherwise radius /= factor, factor *= 2
//    (stop below 1e-32);
//  - stop when |g|_inf <= 1e-10, when |step| <= 1e-8 (|x| + 1e-8), when a
//    step changes the cost by at most 1e-6 of it (not taken), or after
//    lm_max_iters iterations; initial radius 1e4.
// The joint mode's quaternion is stepped as Ceres' quaternion plus does,
// q <- [cos|d|, sin|d| d/|d|] q: a rotation by 2|d|, so its step is half
// the rotation vector of the GN path.
struct LMLin {
  double cost = 0.0;
  double H[36] = {0};
  double g[6] = {0};
};

inline double huber_rho(double r, double delta) {
  const double s2 = r * r;
  return s2 <= delta * delta ? s2 : 2.0 * delta * std::fabs(r) - delta * delta;
}

template <int N, typename State, typename Lin, typename Plus, typename XNorm>
void lm_minimize(int max_iters, State& x, Lin lin, Plus plus, XNorm xnorm) {
  LMLin L = lin(x);
  double radius = 1e4, factor = 2.0;
  auto gmax = [](const LMLin& l) {
    double m = 0.0;
    for (int i = 0; i < N; ++i) m = std::max(m, std::fabs(l.g[i]));
    return m;
  };
  if (gmax(L) <= 1e-10) return;
  for (int it = 0; it < max_iters; ++it) {
    double sc[N], A[N * N], b[N], ds[N], d[N];
    for (int i = 0; i < N; ++i) sc[i] = 1.0 / (1.0 + std::sqrt(L.H[i * N + i]));
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) A[i * N + j] = sc[i] * L.H[i * N + j] * sc[j];
    for (int i = 0; i < N; ++i) {
      const double dg = std::min(std::max(A[i * N + i], 1e-6), 1e32);
      A[i * N + i] += dg / radius;
      b[i] = -sc[i] * L.g[i];
    }
    if (!chol_solve(N, A, b, ds)) {
      radius /= factor;
      factor *= 2.0;
      if (radius < 1e-32) return;
      continue;
    }
    double step2 = 0.0, gd = 0.0, dHd = 0.0;
    for (int i = 0; i < N; ++i) {
      d[i] = sc[i] * ds[i];
      step2 += d[i] * d[i];
    }
    for (int i = 0; i < N; ++i) {
      gd += L.g[i] * d[i];
      for (int j = 0; j < N; ++j) dHd += d[i] * L.H[i * N + j] * d[j];
    }
    const double model = -(gd + 0.5 * dHd);
    if (std::sqrt(step2) <= 1e-8 * (xnorm(x) + 1e-8)) return;
    const State xn = plus(x, d);
    const LMLin Ln = lin(xn);
    if (std::fabs(L.cost - Ln.cost) <= 1e-6 * L.cost) return;
    const double ratio = (L.cost - Ln.cost) / model;
    if (model > 0.0 && ratio > 1e-3) {
      x = xn;
      L = Ln;
      const double t = 2.0 * ratio - 1.0;
      radius = std::min(1e16, radius / std::max(1.0 / 3.0, 1.0 - t * t * t));
      factor = 2.0;
      if (gmax(L) <= 1e-10) return;
    } else {
      radius /= factor;
      factor *= 2.0;
      if (radius < 1e-32) return;
    }
  }
}

struct JointState {
  double R[9];
  V3 t;  // in the frame anchored at the estimate's translation
};

bool optimize_joint_lm(const sloam_params& P, const SE3& est, const std::vector<CylRes>& cr,
                       const std::vector<PlaneRes>& pr, SE3& out) {
  const V3 a = est.t;
  JointState x;
  std::memcpy(x.R, est.R, sizeof(x.R));
  x.t = V3{0, 0, 0};
  std::vector<CylRes> C = cr;
  std::vector<PlaneRes> Pl = pr;
  for (auto& m : C) m.root = m.root - a;
  for (auto& m : Pl) m.d = m.d + dot(m.n, a);
  const double delta = P.huber_delta;
  auto lin = [&](const JointState& s) {
    LMLin L;
    auto acc = [&](double res, V3 Jl, V3 q) {
      const V3 Jw = cross(q, Jl);
      const double J[6] = {2 * Jw.x, 2 * Jw.y, 2 * Jw.z, Jl.x, Jl.y, Jl.z};
      const double w = huber_w(res, delta);
      L.cost += 0.5 * huber_rho(res, delta);
      for (int i = 0; i < 6; ++i) {
        L.g[i] += w * J[i] * res;
        for (int j = 0; j < 6; ++j) L.H[6 * i + j] += w * J[i] * J[j];
      }
    };
    for (auto& m : C) {
      V3 q = rot(s.R, m.p), lp = q + s.t, J;
      double r = cyl_res(m, lp, J);
      acc(r, J, q);
    }
    for (auto& m : Pl) {
      V3 q = rot(s.R, m.p), lp = q + s.t, J;
      double r = plane_res(m, lp, J);
      acc(r, J, q);
    }
    return L;
  };
  auto plus = [](const JointState& s, const double* d) {
    JointState n;
    double dR[9];
    so3_exp({2 * d[0], 2 * d[1], 2 * d[2]}, dR);
    matmul3(dR, s.R, n.R);
    n.t = s.t + V3{d[3], d[4], d[5]};
    return n;
  };
  auto xnorm = [&](const JointState& s) {
    const V3 ta = s.t + a;
    return std::sqrt(1.0 + dot(ta, ta));
  };
  lm_minimize<6>(P.lm_max_iters, x, lin, plus, xnorm);
  std::memcpy(out.R, x.R, sizeof(x.R));
  out.t = x.t + a;
  return true;
}

struct SubsetState {
  double v[6];
};

template <typename ResT>
bool optimize_subset_lm(const sloam_params& P, double x[6], const int free_idx[3],
                        const std::vector<ResT>& res, V3 a) {
  const double delta = P.huber_delta;
  SubsetState st;
  for (int i = 0; i < 6; ++i) st.v[i] = x[i];
  auto lin = [&](const SubsetState& s) {
    LMLin L;
    for (const auto& m0 : res) {
      ResT m = m0;
      V3 q, Jl;
      double J3[9];
      aa_rotate_jac(s.v + 3, m.p, q, J3);
      V3 lp = q + V3{s.v[0] - a.x, s.v[1] - a.y, s.v[2] - a.z};
      double r;
      if constexpr (std::is_same<ResT, CylRes>::value) r = cyl_res(m, lp, Jl);
      else r = plane_res(m, lp, Jl);
      const double Jfull[6] = {Jl.x, Jl.y, Jl.z,
                               Jl.x * J3[0] + Jl.y * J3[3] + Jl.z * J3[6],
                               Jl.x * J3[1] + Jl.y * J3[4] + Jl.z * J3[7],
                               Jl.x * J3[2] + Jl.y * J3[5] + Jl.z * J3[8]};
      const double J[3] = {Jfull[free_idx[0]], Jfull[free_idx[1]], Jfull[free_idx[2]]};
      const double w = huber_w(r, delta);
      L.cost += 0.5 * huber_rho(r, delta);
      for (int i = 0; i < 3; ++i) {
        L.g[i] += w * J[i] * r;
        for (int j = 0; j < 3; ++j) L.H[3 * i + j] += w * J[i] * J[j];
      }
    }
    return L;
  };
  auto plus = [&](const SubsetState& s, const double* d) {
    SubsetState n = s;
    for (int i = 0; i < 3; ++i) n.v[free_idx[i]] += d[i];
    return n;
  };
  auto xnorm = [](const SubsetState& s) {
    double q = 0.0;
    for (int i = 0; i < 6; ++i) q += s.v[i] * s.v[i];
    return std::sqrt(q);
  };
  lm_minimize<3>(P.lm_max_iters, st, lin, plus, xnorm);
  for (int i = 0; i < 6; ++i) x[i] = st.v[i];
  return true;
}

// OptimizeXYYaw / OptimizeZRollPitch, sloam.cpp:55-172: the 6-vector
// (tx,ty,tz,rx,ry,rz) with angle-axis rotation, `free` the three optimised
// entries.  Returns false if a solve fails.
template <typename ResT>
bool optimize_subset(const sloam_params& P, double x[6], const int free_idx[3],
                     const std::vector<ResT>& res, V3 a) {
  if (P.pose_solver == 1) return optimize_subset_lm(P, x, free_idx, res, a);
  const double delta = P.huber_delta;
  for (int it = 0; it < P.gn_iters; ++it) {
    double H[9] = {0}, g[3] = {0};
    for (const auto& m0 : res) {
      ResT m = m0;
      V3 q, Jl;
      double J3[9];
      aa_rotate_jac(x + 3, m.p, q, J3);
      V3 lp = q + V3{x[0] - a.x, x[1] - a.y, x[2] - a.z};
      double r;
      if constexpr (std::is_same<ResT, CylRes>::value) r = cyl_res(m, lp, Jl);
      else r = plane_res(m, lp, Jl);
      double Jfull[6] = {Jl.x, Jl.y, Jl.z,
                         Jl.x * J3[0] + Jl.y * J3[3] + Jl.z * J3[6],
                         Jl.x * J3[1] + Jl.y * J3[4] + Jl.z * J3[7],
                         Jl.x * J3[2] + Jl.y * J3[5] + Jl.z * J3[8]};
      double J[3] = {Jfull[free_idx[0]], Jfull[free_idx[1]], Jfull[free_idx[2]]};
      double w = huber_w(r, delta);
      for (int i = 0; i < 3; ++i) {
        g[i] += w * J[i] * r;
        for (int j = 0; j < 3; ++j) H[3 * i + j] += w * J[i] * J[j];
      }
    }
    double mg[3] = {-g[0], -g[1], -g[2]}, dx[3];
    if (!chol_solve(3, H, mg, dx)) return false;
    for (int i = 0; i < 3; ++i) x[free_idx[i]] += dx[i];
  }
  return true;
}

void two_step(const sloam_params& P, const SE3& est, bool optTrees, bool optGround,
              const std::vector<CylRes>& cr, const std::vector<PlaneRes>& pr, SE3& out) {
  sloam_se3 e = se3_to(est);
  double qwxyz[4] = {e.q[3], e.q[0], e.q[1], e.q[2]}, rpy[3];
  quat_to_aa(qwxyz, rpy);
  V3 a = est.t;
  std::vector<CylRes> C = cr;
  std::vector<PlaneRes> Pl = pr;
  for (auto& m : C) m.root = m.root - a;
  for (auto& m : Pl) m.d = m.d + dot(m.n, a);
  double treeOut[3], groundOut[3];
  {
    double x[6] = {e.t[0], e.t[1], e.t[2], rpy[0], rpy[1], rpy[2]};
    const int fr[3] = {0, 1, 5};
    bool ok = optTrees && optimize_subset(P, x, fr, C, a);
    if (ok) { treeOut[0] = x[0]; treeOut[1] = x[1]; treeOut[2] = x[5]; }
    else { treeOut[0] = e.t[0]; treeOut[1] = e.t[1]; treeOut[2] = rpy[2]; }
  }
  {
    double x[6] = {e.t[0], e.t[1], e.t[2], rpy[0], rpy[1], rpy[2]};
    const int fr[3] = {2, 3, 4};
    bool ok = optGround && optimize_subset(P, x, fr, Pl, a);
    if (ok) { groundOut[0] = x[2]; groundOut[1] = x[3]; groundOut[2] = x[4]; }
    else { groundOut[0] = e.t[2]; groundOut[1] = rpy[0]; groundOut[2] = rpy[1]; }
  }
  double aa[3] = {groundOut[1], groundOut[2], treeOut[2]}, q[4];
  aa_to_quat(aa, q);  // (w, x, y, z)
  sloam_se3 o;
  o.q[0] = q[1]; o.q[1] = q[2]; o.q[2] = q[3]; o.q[3] = q[0];
  o.t[0] = treeOut[0]; o.t[1] = treeOut[1]; o.t[2] = groundOut[0];
  out = se3_from(o);  // Sophus setQuaternion normalises
}

// ==================================================================== a11
void write_models(const sloam_params& P, const std::vector<PlaneObj>& planes,
                  const std::vector<CylObj>& cyls, sloam_models_out* out, int& status) {
  out->n_planes = (int)planes.size();
  out->n_cylinders = (int)cyls.size();
  if (out->n_planes > out->cap_planes || out->n_cylinders > out->cap_cylinders) {
    status = SLOAM_ERR_CAPACITY;
    return;
  }
  for (size_t k = 0; k < planes.size(); ++k) {
    sloam_plane& o = out->planes[k];
    for (int j = 0; j < 4; ++j) o.plane[j] = planes[k].plane[j];
    o.centroid[0] = planes[k].centroid.x;
    o.centroid[1] = planes[k].centroid.y;
    o.centroid[2] = planes[k].centroid.z;
    o.bin = planes[k].bin;
    o.valid = 1;
  }
  const int F = P.features_per_tree;
  for (size_t k = 0; k < cyls.size(); ++k) {
    sloam_cylinder& o = out->cylinders[k];
    const CylObj& c = cyls[k];
    o.root[0] = c.root.x; o.root[1] = c.root.y; o.root[2] = c.root.z;
    o.ray[0] = c.ray.x; o.ray[1] = c.ray.y; o.ray[2] = c.ray.z;
    o.radius = c.radius;
    o.id = c.id;
    o.valid = 1;
    if (out->cyl_inliers) out->cyl_inliers[k] = c.inliers;
    if (out->cyl_features)
      for (int f = 0; f < F; ++f) {
        const Pt& p = c.features[f];
        float* d = out->cyl_features + ((size_t)k * F + f) * 4;
        d[0] = p.x; d[1] = p.y; d[2] = p.z; d[3] = p.i;
      }
  }
}

CylObj cyl_from(const sloam_cylinder& c) {
  CylObj o;
  o.root = {c.root[0], c.root[1], c.root[2]};
  o.ray = {c.ray[0], c.ray[1], c.ray[2]};
  o.radius = c.radius;
  o.id = c.id;
  o.isValid = c.valid != 0;
  return o;
}

std::vector<std::vector<Pt>> read_clusters(const sloam_landmarks* lm) {
  std::vector<std::vector<Pt>> cl;
  const int32_t* cb = lm->cluster_begin;
  const float* cx = lm->cluster_xyzi;
  if (!cb || !cx) return cl;
  cl.resize(lm->n_landmarks);
  for (int l = 0; l < lm->n_landmarks; ++l)
    for (int k = cb[l]; k < cb[l + 1]; ++k)
      cl[l].push_back({cx[4 * k], cx[4 * k + 1], cx[4 * k + 2], cx[4 * k + 3]});
  return cl;
}

}  // namespace

// ================================================================ state
struct oracle_state {
  sloam_params P;
  bool firstScan = true;
  std::vector<PlaneObj> prevPlanes;
};

extern "C" {

void oracle_philox(uint64_t key, const uint32_t ctr[4], uint32_t out[4]) {
  philox(key, ctr, out);
}

void oracle_eigen_svd_u3(const double* a, int32_t n, double u3[3]) {
  eigen_jacobi_svd_u3(std::vector<double>(a, a + (size_t)3 * n), n, u3);
}

int oracle_project_mask(const sloam_params* p, const float* xyzi, int32_t n,
                        const uint8_t* point_labels, const uint8_t* mask_image,
                        int variant, sloam_scan_out* out) {
  const sloam_params& P = *p;
  const int W = P.img_w, H = P.img_h;
  if (n != W * H || (!point_labels && !mask_image)) return SLOAM_ERR_ARG;
  Projection pr;
  std::vector<float> ranges;
  project_points(P, xyzi, n, variant, pr, ranges);
  std::vector<int32_t> win;
  pixel_winners(P, pr, ranges, variant, win);
  std::vector<uint8_t> mask((size_t)W * H, 0);
  for (size_t k = 0; k < mask.size(); ++k) {
    if (mask_image) mask[k] = mask_image[k];
    else mask[k] = win[k] >= 0 ? point_labels[win[k]] : 0;
  }
  if (out->px) std::memcpy(out->px, pr.px.data(), sizeof(int32_t) * n);
  if (out->py) std::memcpy(out->py, pr.py.data(), sizeof(int32_t) * n);
  if (out->range_image)
    for (size_t k = 0; k < mask.size(); ++k) out->range_image[k] = win[k] >= 0 ? ranges[win[k]] : 0.0f;
  if (out->mask_out) std::memcpy(out->mask_out, mask.data(), mask.size());
  // maskCloud (inference.cpp:230-273): val = 1, sparse -> ground list
  int ng = 0;
  std::vector<Pt> temp((size_t)n);
  for (int i = 0; i < n; ++i) {
    size_t proj_idx = (size_t)pr.py[i] * W + pr.px[i];
    uint8_t m = mask[proj_idx];
    if (m == 1 && out->ground_idx) out->ground_idx[ng] = i;
    if (m == 1) ++ng;
    if (m == 255) temp[i] = {xyzi[4 * i], xyzi[4 * i + 1], xyzi[4 * i + 2], xyzi[4 * i + 3]};
    else temp[i] = {kNaNf, kNaNf, kNaNf, 0.0f};
  }
  out->n_ground = ng;
  // val = 255, dense -> organised tree cloud (+ _destaggerCloud :200-228)
  if (out->tree_cloud) {
    std::vector<Pt> oc = temp;
    if (P.do_destagger) {
      bool col_valid = true;
      for (int irow = 0; irow < H; ++irow) {
        for (int icol = 0; icol < W; ++icol) {
          int im_col = icol;
          if (irow % 2 == 0) {
            im_col += 32;
            if (im_col < 0 || im_col > W) {
              col_valid = false;
              im_col = im_col % W;
            }
          }
          size_t dst = (size_t)irow * W + im_col;
          if (col_valid && dst < oc.size()) {  // (H odd: the reference writes past the end)
            oc[dst].x = temp[(size_t)irow * W + icol].x;
            oc[dst].y = temp[(size_t)irow * W + icol].y;
            oc[dst].z = temp[(size_t)irow * W + icol].z;
          }
          col_valid = true;
        }
      }
    }
    std::memcpy(out->tree_cloud, oc.data(), sizeof(Pt) * oc.size());
  }
  return SLOAM_OK;
}

int oracle_trellis(const sloam_params* p, const float* tree_cloud, int32_t H, int32_t W,
                   int sort_variant, int radius_half, uint32_t* cc_labels,
                   int32_t* n_components, sloam_landmarks* out) {
  std::vector<uint32_t> labels;
  std::vector<std::vector<int>> li;
  organized_cc(tree_cloud, H, W, p->cc_dist_threshold, labels, li);
  if (cc_labels) std::memcpy(cc_labels, labels.data(), sizeof(uint32_t) * labels.size());
  if (n_components) *n_components = (int32_t)li.size() - 1;
  std::vector<Tree> trees;
  std::vector<int> tl;
  find_trees(*p, tree_cloud, H, W, labels, li, sort_variant, radius_half != 0, trees, tl);
  int st = write_landmarks(trees, out);
  out->n_cluster = 0;
  if (out->cluster_begin && st == SLOAM_OK) {
    int k = 0;
    for (size_t l = 0; l < tl.size(); ++l) {
      out->cluster_begin[l] = k;
      for (int idx : li[tl[l]]) {
        if (k < out->cap_cluster && out->cluster_xyzi)
          std::memcpy(out->cluster_xyzi + 4 * (size_t)k, tree_cloud + 4 * (size_t)idx, 16);
        ++k;
      }
    }
    out->cluster_begin[tl.size()] = k;
    out->n_cluster = k;
    if (k > out->cap_cluster) st = SLOAM_ERR_CAPACITY;
  }
  return st;
}

oracle_state* oracle_create(const sloam_params* p) {
  oracle_state* s = new oracle_state;
  s->P = *p;
  return s;
}
void oracle_destroy(oracle_state* s) { delete s; }
void oracle_set_params(oracle_state* s, const sloam_params* p) { s->P = *p; }
void oracle_reset(oracle_state* s) {
  s->firstScan = true;
  s->prevPlanes.clear();
}

int oracle_compute_models(oracle_state* s, const sloam_se3* pose, const float* g,
                          int32_t ng, const sloam_landmarks* lm, sloam_models_out* out) {
  std::vector<Tree> trees = read_landmarks(lm);
  auto cl = read_clusters(lm);
  std::vector<PlaneObj> planes;
  std::vector<CylObj> cyls;
  compute_models(s->P, se3_from(*pose), g, ng, trees, cl.empty() ? nullptr : &cl, planes, cyls);
  int st = SLOAM_OK;
  write_models(s->P, planes, cyls, out, st);
  return st;
}

int oracle_run(oracle_state* s, const sloam_se3* pose_in, const float* g, int32_t ng,
               const sloam_landmarks* lm, const sloam_cylinder* map_in, int32_t n_map,
               sloam_run_out* out) {
  const sloam_params& P = s->P;
  std::vector<Tree> trees = read_landmarks(lm);
  auto cl = read_clusters(lm);
  std::vector<PlaneObj> planes;
  std::vector<CylObj> cyls;
  SE3 pose = se3_from(*pose_in);
  compute_models(P, pose, g, ng, trees, cl.empty() ? nullptr : &cl, planes, cyls);
  out->first_scan = s->firstScan ? 1 : 0;
  out->T_Delta = se3_identity();
  out->n_tree_matches = out->n_plane_matches = 0;
  out->tree_check = out->ground_check = 0;
  int st = SLOAM_OK;
  if (s->firstScan) {
    for (auto& p : planes) plane_project(p, pose);
    for (auto& c : cyls) cyl_project(c, pose);
    out->T_Map_Curr = *pose_in;
    write_models(P, planes, cyls, &out->models, st);
    for (size_t k = 0; k < cyls.size() && (int)k < out->models.cap_cylinders; ++k)
      out->matches[k] = -1;
    s->prevPlanes = planes;
    s->firstScan = false;
    out->success = 1;
    return st;
  }
  if (n_map == 0) {
    out->success = 0;
    return SLOAM_ERR_EMPTY_MAP;
  }
  if (planes.empty() || cyls.empty()) {
    out->success = 0;
    return SLOAM_ERR_NO_MODELS;
  }
  std::vector<CylObj> map;
  for (int k = 0; k < n_map; ++k) map.push_back(cyl_from(map_in[k]));
  auto tm = match_features(
      pose, cyls, map, P.tree_match_thresh,
      [](const CylObj& a, const CylObj& b) { return cyl_dist_model(a, b); },
      [](CylObj& c, const SE3& T) { cyl_project(c, T); });
  auto pm = match_features(
      pose, planes, s->prevPlanes, P.plane_match_thresh,
      [](const PlaneObj& a, const PlaneObj& b) { return norm(a.centroid - b.centroid); },
      [](PlaneObj& p, const SE3& T) { plane_project(p, T); });
  out->n_tree_matches = (int)tm.size();
  out->n_plane_matches = (int)pm.size();
  std::vector<CylRes> cr;
  for (auto& m : tm) cr.push_back({m.feat, map[m.obj].root, map[m.obj].ray, map[m.obj].radius});
  std::vector<PlaneRes> pr;
  for (auto& m : pm) {
    const PlaneObj& o = s->prevPlanes[m.obj];
    pr.push_back({m.feat, {o.plane[0], o.plane[1], o.plane[2]}, o.plane[3]});
  }
  bool treeCheck = cyls.size() > P.min_tree_models && tm.size() > 5.0 * P.features_per_tree;
  bool groundCheck = pm.size() > P.min_ground_models && planes.size() > P.min_planes;
  out->tree_check = treeCheck;
  out->ground_check = groundCheck;
  SE3 curr = pose;
  bool success = true;
  if (P.two_step_optim) {
    two_step(P, pose, treeCheck, groundCheck, cr, pr, curr);
  } else if (treeCheck && groundCheck) {
    SE3 res;
    success = optimize_joint(P, pose, cr, pr, res);
    if (success) {
      curr = res;
      out->T_Delta = se3_to(res);
    }
  }
  for (auto& p : planes) plane_project(p, curr);
  for (auto& c : cyls) cyl_project(c, curr);
  // matchModels, sloam.cpp:298-328
  for (size_t i = 0; i < cyls.size(); ++i) {
    double bestDist = P.tree_match_thresh + 100;
    int bestKey = 0;
    for (size_t k = 0; k < map.size(); ++k) {
      double d = cyl_dist_model(map[k], cyls[i]);
      if (d < bestDist) {
        bestDist = d;
        bestKey = (int)k;
      }
    }
    if ((int)i < out->models.cap_cylinders)
      out->matches[i] = bestDist < P.add_new_tree_thresh_dist ? bestKey : -1;
  }
  s->prevPlanes = planes;
  out->T_Map_Curr = se3_to(curr);
  write_models(P, planes, cyls, &out->models, st);
  out->success = success ? 1 : 0;
  if (st != SLOAM_OK) return st;
  return success ? SLOAM_OK : SLOAM_ERR_NOT_CONVERGED;
}

int oracle_keyframe(oracle_state* s, const float* xyzi, int32_t n, const uint8_t* labels,
                    const uint8_t* mask_image, const sloam_se3* pose,
                    const sloam_cylinder* map, int32_t n_map, sloam_run_out* out) {
  const sloam_params& P = s->P;
  const int W = P.img_w, H = P.img_h;
  std::vector<int32_t> gidx(n);
  std::vector<float> tree((size_t)4 * n);
  sloam_scan_out so{};
  so.ground_idx = gidx.data();
  so.tree_cloud = tree.data();
  int st = oracle_project_mask(&P, xyzi, n, labels, mask_image, ORACLE_CONTRACT, &so);
  if (st) return st;
  std::vector<float> ground((size_t)4 * so.n_ground);
  for (int k = 0; k < so.n_ground; ++k) std::memcpy(&ground[4 * k], xyzi + 4 * (size_t)gidx[k], 16);
  std::vector<uint32_t> labels_cc;
  std::vector<std::vector<int>> li;
  organized_cc(tree.data(), H, W, P.cc_dist_threshold, labels_cc, li);
  std::vector<Tree> trees;
  std::vector<int> tl;
  find_trees(P, tree.data(), H, W, labels_cc, li, ORACLE_CONTRACT, false, trees, tl);
  int nv = 0, np = 0;
  for (auto& t : trees) {
    nv += (int)t.size();
    for (auto& v : t) np += (int)v.points.size();
  }
  std::vector<int32_t> tid(trees.size() + 1), vb(trees.size() + 1), vr(nv + 1), pb(nv + 1);
  std::vector<float> vx((size_t)3 * nv + 3), px((size_t)4 * np + 4);
  std::vector<double> vrad(nv + 1);
  sloam_landmarks lm{};
  lm.cap_landmarks = (int)trees.size();
  lm.cap_vertices = nv;
  lm.cap_points = np;
  lm.tree_id = tid.data(); lm.vertex_begin = vb.data(); lm.vertex_xyz = vx.data();
  lm.vertex_radius = vrad.data(); lm.vertex_row = vr.data(); lm.point_begin = pb.data();
  lm.point_xyzi = px.data();
  write_landmarks(trees, &lm);
  std::vector<int32_t> cb(trees.size() + 1);
  std::vector<float> cx;
  int k = 0;
  for (size_t l = 0; l < tl.size(); ++l) {
    cb[l] = k;
    for (int idx : li[tl[l]]) {
      cx.insert(cx.end(), tree.begin() + 4 * (size_t)idx, tree.begin() + 4 * (size_t)idx + 4);
      ++k;
    }
  }
  cb[tl.size()] = k;
  lm.cap_cluster = lm.n_cluster = k;
  lm.cluster_begin = cb.data();
  lm.cluster_xyzi = cx.data();
  return oracle_run(s, pose, ground.data(), so.n_ground, &lm, map, n_map, out);
}

int oracle_plane(const sloam_params* p, const float* xyzi, int32_t n, sloam_plane* out,
                 float* features) {
  std::vector<Pt> pts(n);
  for (int i = 0; i < n; ++i) pts[i] = {xyzi[4 * i], xyzi[4 * i + 1], xyzi[4 * i + 2], xyzi[4 * i + 3]};
  PlaneObj pl = make_plane(pts, *p);
  for (int j = 0; j < 4; ++j) out->plane[j] = pl.plane[j];
  out->centroid[0] = pl.centroid.x; out->centroid[1] = pl.centroid.y; out->centroid[2] = pl.centroid.z;
  out->valid = pl.isValid;
  out->bin = 0;
  if (features && pl.isValid)
    for (size_t k = 0; k < pl.features.size(); ++k) std::memcpy(features + 4 * k, &pl.features[k], 16);
  return SLOAM_OK;
}

int oracle_cylinder(const sloam_params* p, const sloam_landmarks* lm, int32_t landmark,
                    const sloam_plane* plane, sloam_cylinder* out, float* features,
                    int32_t* inliers) {
  std::vector<Tree> trees = read_landmarks(lm);
  if (landmark < 0 || landmark >= (int)trees.size()) return SLOAM_ERR_ARG;
  PlaneObj pl;
  for (int j = 0; j < 4; ++j) pl.plane[j] = plane->plane[j];
  pl.centroid = {plane->centroid[0], plane->centroid[1], plane->centroid[2]};
  CylObj c = make_cylinder(*p, trees[landmark], pl, nullptr);
  out->root[0] = c.root.x; out->root[1] = c.root.y; out->root[2] = c.root.z;
  out->ray[0] = c.ray.x; out->ray[1] = c.ray.y; out->ray[2] = c.ray.z;
  out->radius = c.radius;
  out->id = c.id;
  out->valid = c.isValid;
  if (inliers) *inliers = c.inliers;
  if (features)
    for (size_t k = 0; k < c.features.size() && (int)k < p->features_per_tree; ++k)
      std::memcpy(features + 4 * k, &c.features[k], 16);
  return SLOAM_OK;
}

double oracle_cylinder_distance_model(const sloam_cylinder* self, const sloam_cylinder* tgt) {
  return cyl_dist_model(cyl_from(*self), cyl_from(*tgt));
}
double oracle_cylinder_distance_point(const sloam_cylinder* self, const float* xyz) {
  return cyl_dist_point(cyl_from(*self), {xyz[0], xyz[1], xyz[2]});
}
void oracle_cylinder_project(sloam_cylinder* c, const sloam_se3* tf) {
  CylObj o = cyl_from(*c);
  cyl_project(o, se3_from(*tf));
  c->root[0] = o.root.x; c->root[1] = o.root.y; c->root[2] = o.root.z;
  c->ray[0] = o.ray.x; c->ray[1] = o.ray.y; c->ray[2] = o.ray.z;
}
double oracle_plane_distance_point(const sloam_plane* self, const float* xyz) {
  PlaneObj pl;
  for (int j = 0; j < 4; ++j) pl.plane[j] = self->plane[j];
  return plane_dist_point(pl, {xyz[0], xyz[1], xyz[2]});
}
void oracle_plane_project(sloam_plane* p, const sloam_se3* tf) {
  PlaneObj pl;
  for (int j = 0; j < 4; ++j) pl.plane[j] = p->plane[j];
  pl.centroid = {p->centroid[0], p->centroid[1], p->centroid[2]};
  plane_project(pl, se3_from(*tf));
  for (int j = 0; j < 4; ++j) p->plane[j] = pl.plane[j];
  p->centroid[0] = pl.centroid.x; p->centroid[1] = pl.centroid.y; p->centroid[2] = pl.centroid.z;
}

}  // extern "C"
