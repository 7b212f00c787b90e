// common.cuh — device helpers shared by the SLOAM kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sloam_gb300.h"

#define SLOAM_HD __host__ __device__ __forceinline__
#define SLOAM_D __device__ __forceinline__

namespace sg {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr double kPIDEF = 3.14159265;  // definitions.h:28

// ---------------------------------------------------------- exact float ops
// Bit-exact paths use these so nvcc never contracts them into FMA: they are
// IEEE single operations with round-to-nearest, like the host's SSE/NEON code
// built with -ffp-contract=off.
SLOAM_D float fadd(float a, float b) { return __fadd_rn(a, b); }
SLOAM_D float fsub(float a, float b) { return __fsub_rn(a, b); }
SLOAM_D float fmul(float a, float b) { return __fmul_rn(a, b); }
SLOAM_D float fdiv(float a, float b) { return __fdiv_rn(a, b); }
SLOAM_D float fsqrt(float a) { return __fsqrt_rn(a); }

// pcl::euclideanDistance: sqrt((dx*dx + dy*dy) + dz*dz), float.
SLOAM_D float pcl_euclid(float ax, float ay, float az, float bx, float by, float bz) {
  float dx = fsub(bx, ax), dy = fsub(by, ay), dz = fsub(bz, az);
  return fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
}
// Eigen Vector3f (a-b).squaredNorm(): dx*dx + (dy*dy + dz*dz).
SLOAM_D float eigen_sqnorm3(float ax, float ay, float az, float bx, float by, float bz) {
  float dx = fsub(ax, bx), dy = fsub(ay, by), dz = fsub(az, bz);
  return fadd(fmul(dx, dx), fadd(fmul(dy, dy), fmul(dz, dz)));
}

// Orderable key of a float range (range >= 0 or NaN): NaN sorts last.
SLOAM_D uint32_t range_key(float r) {
  return isnan(r) ? 0x7fc00000u : __float_as_uint(r);
}

// ------------------------------------------------------------------- RNG
// Philox4x32-10 (Salmon et al., SC'11).  key = seed, counter = 4 words.
SLOAM_HD void philox(uint64_t key64, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                     uint32_t out[4]) {
  uint32_t k0 = (uint32_t)key64, k1 = (uint32_t)(key64 >> 32);
#pragma unroll
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
SLOAM_HD uint32_t mulhi_idx(uint32_t u, uint32_t n) {
  return (uint32_t)(((uint64_t)u * n) >> 32);
}
// k (<= 3) distinct indices in [0, n) from one Philox block.
SLOAM_HD void draw_distinct(const uint32_t u[4], uint32_t n, int k, uint32_t* idx) {
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

// --------------------------------------------------------- warp helpers
SLOAM_D float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
SLOAM_D double warp_sumd(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
SLOAM_D int warp_sumi(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// argmin over (value, index): smallest value, then smallest index.
SLOAM_D void warp_argmin(double& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (ov < v || (ov == v && oi < i) || (isnan(v) && !isnan(ov))) {
      v = ov;
      i = oi;
    }
  }
}

// ------------------------------------------------------------ FP64 algebra
struct d3 {
  double x, y, z;
};
SLOAM_HD d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
SLOAM_HD d3 add3(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
SLOAM_HD d3 sub3(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
SLOAM_HD d3 scl3(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
SLOAM_HD double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SLOAM_HD d3 cross3(d3 a, d3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
SLOAM_HD double norm3(d3 a) { return sqrt(dot3(a, a)); }

struct Pose {  // rotation (row-major) + translation, FP64
  double R[9];
  d3 t;
};
SLOAM_HD Pose pose_from(const sloam_se3& p) {
  double x = p.q[0], y = p.q[1], z = p.q[2], w = p.q[3];
  double n = sqrt(x * x + y * y + z * z + w * w);
  x /= n; y /= n; z /= n; w /= n;
  Pose T;
  T.R[0] = 1 - 2 * (y * y + z * z); T.R[1] = 2 * (x * y - w * z); T.R[2] = 2 * (x * z + w * y);
  T.R[3] = 2 * (x * y + w * z); T.R[4] = 1 - 2 * (x * x + z * z); T.R[5] = 2 * (y * z - w * x);
  T.R[6] = 2 * (x * z - w * y); T.R[7] = 2 * (y * z + w * x); T.R[8] = 1 - 2 * (x * x + y * y);
  T.t = {p.t[0], p.t[1], p.t[2]};
  return T;
}
SLOAM_HD d3 rot3(const double* R, d3 p) {
  return {R[0] * p.x + R[1] * p.y + R[2] * p.z, R[3] * p.x + R[4] * p.y + R[5] * p.z,
          R[6] * p.x + R[7] * p.y + R[8] * p.z};
}
SLOAM_HD d3 xform(const Pose& T, d3 p) { return add3(rot3(T.R, p), T.t); }
SLOAM_HD void quat_from_R(const double* R, double* q) {
  double tr = R[0] + R[4] + R[8];
  double x, y, z, w;
  if (tr > 0) {
    double s = sqrt(tr + 1.0) * 2;
    w = 0.25 * s; x = (R[7] - R[5]) / s; y = (R[2] - R[6]) / s; z = (R[3] - R[1]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    double s = sqrt(1.0 + R[0] - R[4] - R[8]) * 2;
    w = (R[7] - R[5]) / s; x = 0.25 * s; y = (R[1] + R[3]) / s; z = (R[2] + R[6]) / s;
  } else if (R[4] > R[8]) {
    double s = sqrt(1.0 + R[4] - R[0] - R[8]) * 2;
    w = (R[2] - R[6]) / s; x = (R[1] + R[3]) / s; y = 0.25 * s; z = (R[5] + R[7]) / s;
  } else {
    double s = sqrt(1.0 + R[8] - R[0] - R[4]) * 2;
    w = (R[3] - R[1]) / s; x = (R[2] + R[6]) / s; y = (R[5] + R[7]) / s; z = 0.25 * s;
  }
  double n = sqrt(x * x + y * y + z * z + w * w);
  q[0] = x / n; q[1] = y / n; q[2] = z / n; q[3] = w / n;
}
SLOAM_HD sloam_se3 pose_to(const Pose& T) {
  sloam_se3 o;
  quat_from_R(T.R, o.q);
  o.t[0] = T.t.x; o.t[1] = T.t.y; o.t[2] = T.t.z;
  return o;
}
SLOAM_HD void matmul3(const double* A, const double* B, double* C) {
  double T[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      T[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
  for (int k = 0; k < 9; ++k) C[k] = T[k];
}
// Row r of exp([w]x) = I + A K + B K^2, K = [w]x, K^2 = w w^T - |w|^2 I;
// A = sin(t)/t, B = (1 - cos(t))/t^2 by their Taylor series for t < 0.1
// (truncation < 3e-14 relative; multiplications by the series' reciprocal
// constants), else the library functions.
SLOAM_HD void so3_exp_row(d3 w, int r, double* out) {
  const double th2 = dot3(w, w);
  double A, B;
  if (th2 < 1e-2) {
    A = 1.0 - th2 * (1.0 / 6.0) * (1.0 - th2 * (1.0 / 20.0) * (1.0 - th2 * (1.0 / 42.0)));
    B = 0.5 - th2 * (1.0 / 24.0) * (1.0 - th2 * (1.0 / 30.0) * (1.0 - th2 * (1.0 / 56.0)));
  } else {
    const double th = sqrt(th2);
    A = sin(th) / th;
    B = (1.0 - cos(th)) / th2;
  }
  const double wv[3] = {w.x, w.y, w.z};
  // K row r: r = 0: (0, -wz, wy); r = 1: (wz, 0, -wx); r = 2: (-wy, wx, 0)
  const double K[3][3] = {{0.0, -w.z, w.y}, {w.z, 0.0, -w.x}, {-w.y, w.x, 0.0}};
  for (int k = 0; k < 3; ++k)
    out[k] = (r == k ? 1.0 : 0.0) + A * K[r][k] + B * (wv[r] * wv[k] - (r == k ? th2 : 0.0));
}

SLOAM_HD void so3_exp(d3 w, double* R) {
  const double th2 = dot3(w, w);
  double A, B;
  if (th2 < 1e-2) {
    // sin(t)/t and (1-cos(t))/t^2 by their Taylor series (truncation
    // < 3e-14 relative for t < 0.1): no FP64 transcendental on the GN path
    A = 1.0 - th2 / 6.0 * (1.0 - th2 / 20.0 * (1.0 - th2 / 42.0));
    B = 0.5 - th2 / 24.0 * (1.0 - th2 / 30.0 * (1.0 - th2 / 56.0));
  } else {
    const double th = sqrt(th2);
    A = sin(th) / th;
    B = (1.0 - cos(th)) / th2;
  }
  double K[9] = {0, -w.z, w.y, w.z, 0, -w.x, -w.y, w.x, 0}, K2[9];
  matmul3(K, K, K2);
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0 ? 1.0 : 0.0) + A * K[i] + B * K2[i];
}

// Cholesky solve of N x N normal equations H x = -g (N <= 6) by one warp
// (all 32 lanes call it): lanes 0..T-1 (T = N(N+1)/2) hold the lower
// triangle of H row by row (lane i(i+1)/2 + j holds H_ij, j <= i), lanes
// T..T+N-1 the right-hand side.  Column k: the pivot's reciprocal square
// root (every lane computes it: an FP64 warp instruction costs the pipe the
// same for one lane or 32), L_ik scaled on their lanes, y_k = b_k / L_kk,
// then the trailing entries and right-hand sides updated together, one fma
// per lane.  Back substitution one unknown at a time.  The same eliminations
// as chol_solve in the same order (the back substitution sums in the
// opposite order).  `H` is the upper triangle row by row (H_ab, a <= b).
// Returns false (on every lane) when a pivot is not positive or x is not
// finite; lane T + i writes x[i].
template <int N>
__device__ bool warp_chol_solve(const double* H, const double* g, double* x) {
  constexpr int T = N * (N + 1) / 2;
  static_assert(T + N <= 32, "one warp");
  const int lane = threadIdx.x & 31;
  int ri = -1, rj = -1;  // this lane's matrix entry (ri, rj), or rhs row ri (rj = -1)
  double v = 0.0;
  if (lane < T) {
    int i = 0;
    while ((i + 1) * (i + 2) / 2 <= lane) ++i;
    ri = i;
    rj = lane - i * (i + 1) / 2;
    const int a = rj, b = ri;  // upper index of (a, b), a <= b
    v = H[a * N - a * (a - 1) / 2 + (b - a)];
  } else if (lane < T + N) {
    ri = lane - T;
    v = -g[ri];
  }
  double inv[N];
  bool ok = true;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const double piv = __shfl_sync(0xffffffffu, v, k * (k + 1) / 2 + k);
    ok = ok && piv > 0.0;
    inv[k] = rsqrt(piv);
    // L_kk (the pivot's own lane, v == piv), L_ik (i > k) and y_k: one
    // predicated multiply for all three
    if ((rj == k && ri >= k) || (rj < 0 && ri == k)) v *= inv[k];
    // trailing update: matrix (i, j), k < j <= i: -= L_ik L_jk;
    // rhs i > k: -= L_ik y_k
    int s1 = 0, s2 = 0;
    const bool upd = (rj > k) || (rj < 0 && ri > k);
    if (upd) {
      s1 = ri * (ri + 1) / 2 + k;
      s2 = rj >= 0 ? rj * (rj + 1) / 2 + k : T + k;
    }
    const double a1 = __shfl_sync(0xffffffffu, v, s1);
    const double a2 = __shfl_sync(0xffffffffu, v, s2);
    if (upd) v = fma(-a1, a2, v);
  }
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    if (rj < 0 && ri == i) v *= inv[i];                // x_i
    const double xi = __shfl_sync(0xffffffffu, v, T + i);
    const int src = (rj < 0 && ri >= 0 && ri < i) ? i * (i + 1) / 2 + ri : 0;
    const double lij = __shfl_sync(0xffffffffu, v, src);
    if (rj < 0 && ri >= 0 && ri < i) v = fma(-lij, xi, v);
  }
  const bool fin = rj >= 0 || ri < 0 || isfinite(v);
  ok = ok && __all_sync(0xffffffffu, fin);
  if (rj < 0 && ri >= 0) x[ri] = v;
  return ok;
}

// Cholesky solve of an n x n SPD system (n <= 6, row-major), FP64.  One
// reciprocal square root per pivot; everything else multiplies (the FP64
// divide and square root are long dependent sequences on this part).
SLOAM_HD bool chol_solve(int n, const double* H, const double* b, double* x) {
  double L[36], inv[6];
  for (int j = 0; j < n; ++j) {
    double s = H[j * n + j];
    for (int k = 0; k < j; ++k) s -= L[j * n + k] * L[j * n + k];
    if (!(s > 0.0)) return false;
#ifdef __CUDA_ARCH__
    inv[j] = rsqrt(s);
#else
    inv[j] = 1.0 / sqrt(s);
#endif
    L[j * n + j] = s * inv[j];
    for (int i = j + 1; i < n; ++i) {
      double t = H[i * n + j];
      for (int k = 0; k < j; ++k) t -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = t * inv[j];
    }
  }
  double y[6];
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * n + k] * y[k];
    y[i] = s * inv[i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
    x[i] = s * inv[i];
  }
  for (int i = 0; i < n; ++i)
    if (!isfinite(x[i])) return false;
  return true;
}

// Symmetric 3x3 eigen-decomposition, cyclic Jacobi in FP32 (the plane
// normals and line directions: well-separated spectra, ~1e-7 rad accurate).
// Eigenvalues ascending; eigenvectors as columns of V.
SLOAM_D void jacobi3f(const float* A_in, float* evals, float* V) {
  float A[9];
  for (int i = 0; i < 9; ++i) A[i] = A_in[i];
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0f : 0.0f;
  for (int sweep = 0; sweep < 16; ++sweep) {
    const float off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    const float diag = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off <= 1e-36f || off <= diag * 1e-16f) break;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
#pragma unroll
      for (int q = p + 1; q < 3; ++q) {
        const float apq = A[3 * p + q];
        if (apq == 0.0f) continue;
        const float app = A[3 * p + p], aqq = A[3 * q + q];
        const float theta = (aqq - app) / (2.0f * apq);
        const float t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
        const float c = rsqrtf(t * t + 1.0f), s = t * c;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float akp = A[3 * k + p], akq = A[3 * k + q];
          A[3 * k + p] = c * akp - s * akq;
          A[3 * k + q] = s * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float apk = A[3 * p + k], aqk = A[3 * q + k];
          A[3 * p + k] = c * apk - s * aqk;
          A[3 * q + k] = s * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float vkp = V[3 * k + p], vkq = V[3 * k + q];
          V[3 * k + p] = c * vkp - s * vkq;
          V[3 * k + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  float d[3] = {A[0], A[4], A[8]};
  int o0 = 0, o1 = 1, o2 = 2, tmp;
  if (d[o1] < d[o0]) { tmp = o0; o0 = o1; o1 = tmp; }
  if (d[o2] < d[o1]) { tmp = o1; o1 = o2; o2 = tmp; }
  if (d[o1] < d[o0]) { tmp = o0; o0 = o1; o1 = tmp; }
  const int ord[3] = {o0, o1, o2};
  float Vs[9];
  for (int c = 0; c < 3; ++c) {
    evals[c] = d[ord[c]];
    for (int r = 0; r < 3; ++r) Vs[3 * r + c] = V[3 * r + ord[c]];
  }
  for (int i = 0; i < 9; ++i) V[i] = Vs[i];
}

}  // namespace sg
