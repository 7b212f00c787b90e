// proposal.cu — the learned cylinder proposal (network layout in
// proposal.cuh): synthetic training clusters, FP32 training kernels
// (forward + backward per cluster, a deterministic gradient reduction,
// Adam), and BF16 inference -- every layer of the shared MLP and the head
// on the 5th-generation tensor cores (tcgen05.mma, operands in shared
// memory by bulk copy, accumulators in TMEM), with a SIMT kernel of the same
// bf16 operands as the reference it is checked against.
//
// Training clusters: a trunk of radius U(0.05, 0.8) m, axis tilt U(0, 15)
// deg, 2-20 m from the sensor, the arc that faces the sensor minus an
// occluding azimuth wedge of 0-30 % of it, range noise sigma U(1, 5) cm
// along the beam, and a fraction U(0, 0.15) of range outliers moved
// U(-1, 1) m along the beam (as segmentation keeps them in the trunk's
// cluster); 128 points; targets from the generator's own trunk.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "bulk.cuh"
#include "common.cuh"
#include "internal.h"
#include "proposal.cuh"

namespace sg {
namespace prop {
namespace {

constexpr float kPi = 3.14159265358979f;

SLOAM_D float u01(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }
SLOAM_D float gauss(uint32_t a, uint32_t b) {  // Box-Muller
  const float r = sqrtf(-2.0f * logf(fmaxf(u01(a), 1e-7f)));
  return r * cospif(2.0f * u01(b));
}

// ------------------------------------------------------------ samples
// One block (128 threads) per cluster id; thread i makes point i.
__global__ void __launch_bounds__(128) k_prop_sample(uint64_t seed, int64_t first_id,
                                                     float* __restrict__ X,
                                                     float* __restrict__ T) {
  __shared__ float red[4];
  const int64_t g = first_id + blockIdx.x;
  const uint32_t g0 = (uint32_t)g, g1 = (uint32_t)(g >> 32);
  uint32_t u[4], v[4], w[4];
  philox(seed, g0, g1, 0, 0, u);
  philox(seed, g0, g1, 1, 0, v);
  philox(seed, g0, g1, 2, 0, w);
  const float r = 0.05f + 0.75f * u01(u[0]);
  const float th = u01(u[1]) * (15.0f * kPi / 180.0f), ph = 2.0f * kPi * u01(u[2]);
  const float D = 2.0f + 18.0f * u01(u[3]), ps = 2.0f * kPi * u01(v[0]);
  const float sig = 0.01f + 0.04f * u01(v[1]), occ = 0.3f * u01(v[2]);
  const float h = 1.0f + 3.0f * u01(w[0]), zb = -(1.2f + 0.8f * u01(w[1]));
  const float ax = sinf(th) * cosf(ph), ay = sinf(th) * sinf(ph), az = cosf(th);
  const float bx = D * cosf(ps), by = D * sinf(ps), bz = zb;
  // frame around the axis: e1 towards the sensor (origin), e2 = a x e1
  float sx = -bx, sy = -by, sz = -bz;
  const float sa = sx * ax + sy * ay + sz * az;
  sx -= sa * ax; sy -= sa * ay; sz -= sa * az;
  const float dp = sqrtf(sx * sx + sy * sy + sz * sz);
  const float e1x = sx / dp, e1y = sy / dp, e1z = sz / dp;
  const float e2x = ay * e1z - az * e1y, e2y = az * e1x - ax * e1z, e2z = ax * e1y - ay * e1x;
  const float A = acosf(fminf(1.0f, r / dp));       // visible half-arc
  const float wdg = occ * 2.0f * A;
  const float ws = -A + u01(v[3]) * (2.0f * A - wdg);
  const int i = threadIdx.x;
  uint32_t q[4];
  philox(seed, g0, g1, 3 + i, 0, q);
  float al = -A + u01(q[0]) * (2.0f * A - wdg);
  if (al >= ws) al += wdg;
  const float t = u01(q[1]) * h;
  const float ca = cosf(al), sn = sinf(al);
  float px = bx + t * ax + r * (ca * e1x + sn * e2x);
  float py = by + t * ay + r * (ca * e1y + sn * e2y);
  float pz = bz + t * az + r * (ca * e1z + sn * e2z);
  {
    // range noise, and outliers, along the beam (the sensor is the origin)
    uint32_t o[4];
    philox(seed, g0, g1, 3 + i, 1, o);
    const float fo = 0.15f * u01(w[2]);
    const float dr = u01(o[0]) < fo ? 2.0f * u01(o[1]) - 1.0f : sig * gauss(q[2], q[3]);
    const float rn = sqrtf(px * px + py * py + pz * pz);
    const float k = (rn + dr) / rn;
    px *= k; py *= k; pz *= k;
  }
  float mm[3], s;
  sample_frame(px, py, pz, red, mm, &s);
  const float mx = mm[0], my = mm[1], mz = mm[2];
  const float dx = px - mx, dy = py - my, dz = pz - mz;
  float* x = X + (size_t)blockIdx.x * kPts * 3;
  x[3 * i] = dx / s;
  x[3 * i + 1] = dy / s;
  x[3 * i + 2] = dz / s;
  if (i == 0) {
    // axis point nearest the mean, relative to the mean, in units of s
    const float k = (mx - bx) * ax + (my - by) * ay + (mz - bz) * az;
    float* tg = T + (size_t)blockIdx.x * kTgt;
    tg[0] = ax; tg[1] = ay; tg[2] = az;
    tg[3] = (bx + k * ax - mx) / s;
    tg[4] = (by + k * ay - my) / s;
    tg[5] = logf(r / s);
    tg[6] = s;
    tg[7] = r;
  }
}

__global__ void k_prop_init(float* __restrict__ W, uint64_t seed) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNumParams) return;
  int fan_in = 0;
  float gain = 1.0f;
  if (p < kB1) fan_in = 3;
  else if (p >= kW2 && p < kB2) fan_in = kD1;
  else if (p >= kW3 && p < kB3) fan_in = kD2;
  else if (p >= kW4 && p < kB4) fan_in = kD3;
  else if (p >= kW5 && p < kB5) { fan_in = kD4; gain = 0.1f; }
  if (!fan_in) { W[p] = 0.0f; return; }  // biases
  uint32_t u[4];
  philox(seed, (uint32_t)p, 0x70726f70u, 0, 0, u);
  const float bound = gain * sqrtf(6.0f / fan_in);
  W[p] = (2.0f * u01(u[0]) - 1.0f) * bound;
}

// ------------------------------------------------------------ training
// One block per cluster: forward, loss, backward; the cluster's gradient
// (every parameter, written once) goes to its own slot G[b][*].
constexpr int kTrainThreads = 256;
constexpr int kW2Pad = kD1 + 1;  // W2 staged transposed, [128][65]
constexpr size_t kTrainSmemFloats = 384 + kPts * kD1 + 2 * kPts * kD2 + kD2 * kW2Pad + 256 + 256 +
                                    128 + 8 + 128 + 256 + 8 + 64;

__global__ void __launch_bounds__(kTrainThreads) k_prop_train(const float* __restrict__ W,
                                                              const float* __restrict__ X,
                                                              const float* __restrict__ T,
                                                              float* __restrict__ G,
                                                              float* __restrict__ loss) {
  extern __shared__ float sm[];
  float* x = sm;                       // [128][3]
  float* a1 = x + 384;                 // [128][64]
  float* a2 = a1 + kPts * kD1;         // [128][128]; later dA1 / dZ1 [128][64]
  float* da2 = a2 + kPts * kD2;        // [128][128]
  float* w2t = da2 + kPts * kD2;       // W2^T padded [128][65]
  float* h = w2t + kD2 * kW2Pad;       // [256]
  int* arg = reinterpret_cast<int*>(h + kD3);  // [256]
  float* y1 = reinterpret_cast<float*>(arg + kD3);  // [128]
  float* out = y1 + kD4;               // [8]
  float* dy1 = out + 8;                // [128]
  float* dh = dy1 + kD4;               // [256]
  float* dout = dh + kD3;              // [8]
  const int tid = threadIdx.x;
  const int b = blockIdx.x;
  float* g = G + (size_t)b * kNumParams;

  for (int i = tid; i < 384; i += kTrainThreads) x[i] = X[(size_t)b * 384 + i];
  for (int i = tid; i < kD1 * kD2; i += kTrainThreads) {
    const int k = i / kD2, j = i % kD2;
    w2t[j * kW2Pad + k] = W[kW2 + i];
  }
  for (int i = tid; i < kPts * kD2; i += kTrainThreads) da2[i] = 0.0f;
  __syncthreads();
  // layer 1
  for (int i = tid; i < kPts * kD1; i += kTrainThreads) {
    const int r = i / kD1, j = i % kD1;
    const float z = W[kB1 + j] + x[3 * r] * W[kW1 + j] + x[3 * r + 1] * W[kW1 + kD1 + j] +
                    x[3 * r + 2] * W[kW1 + 2 * kD1 + j];
    a1[i] = fmaxf(z, 0.0f);
  }
  __syncthreads();
  // layer 2: column j, 64 rows per thread in tiles of 16
  {
    const int j = tid & (kD2 - 1), rh = tid >> 7;
    for (int r0 = rh * 64; r0 < rh * 64 + 64; r0 += 16) {
      float acc[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = W[kB2 + j];
      for (int k = 0; k < kD1; ++k) {
        const float w = w2t[j * kW2Pad + k];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += a1[(r0 + q) * kD1 + k] * w;
      }
#pragma unroll
      for (int q = 0; q < 16; ++q) a2[(r0 + q) * kD2 + j] = fmaxf(acc[q], 0.0f);
    }
  }
  __syncthreads();
  // layer 3 + max-pool: thread c, rows in tiles of 16
  {
    const int c = tid;
    float best = -INFINITY;
    int br = -1;
    for (int r0 = 0; r0 < kPts; r0 += 16) {
      float acc[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = W[kB3 + c];
      for (int k = 0; k < kD2; ++k) {
        const float w = W[kW3 + k * kD3 + c];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += a2[(r0 + q) * kD2 + k] * w;
      }
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (acc[q] > best) { best = acc[q]; br = r0 + q; }
    }
    h[c] = fmaxf(best, 0.0f);
    arg[c] = best > 0.0f ? br : -1;
  }
  __syncthreads();
  // head
  if (tid < kD4) {
    float z = W[kB4 + tid];
    for (int c = 0; c < kD3; ++c) z += h[c] * W[kW4 + c * kD4 + tid];
    y1[tid] = fmaxf(z, 0.0f);
  }
  __syncthreads();
  if (tid < kD5) {
    float z = W[kB5 + tid];
    for (int j = 0; j < kD4; ++j) z += y1[j] * W[kW5 + j * kD5 + tid];
    out[tid] = z;
  }
  __syncthreads();
  if (tid == 0) {
    const float* tg = T + (size_t)b * kTgt;
    float L = 0.0f;
    for (int q = 0; q < 6; ++q) {
      const float d = out[q] - tg[q];
      L += d * d;
      dout[q] = 2.0f * d;
    }
    const float ec = (out[3] - tg[3]) * (out[3] - tg[3]) + (out[4] - tg[4]) * (out[4] - tg[4]) +
                     (out[5] - tg[5]) * (out[5] - tg[5]);
    const float ct = expf(-ec / 0.01f);  // confidence target: the proposal is good
    const float p = 1.0f / (1.0f + expf(-out[6]));
    L += 0.1f * -(ct * logf(fmaxf(p, 1e-7f)) + (1.0f - ct) * logf(fmaxf(1.0f - p, 1e-7f)));
    dout[6] = 0.1f * (p - ct);
    loss[b] = L;
  }
  __syncthreads();
  // ---- backward: head
  for (int i = tid; i < kD4 * kD5; i += kTrainThreads)
    g[kW5 + i] = y1[i / kD5] * dout[i % kD5];
  if (tid < kD5) g[kB5 + tid] = dout[tid];
  if (tid < kD4) {
    float s = 0.0f;
    for (int o = 0; o < kD5; ++o) s += dout[o] * W[kW5 + tid * kD5 + o];
    dy1[tid] = y1[tid] > 0.0f ? s : 0.0f;
  }
  __syncthreads();
  for (int i = tid; i < kD3 * kD4; i += kTrainThreads) g[kW4 + i] = h[i / kD4] * dy1[i % kD4];
  if (tid < kD4) g[kB4 + tid] = dy1[tid];
  {
    const int c = tid;
    float s = 0.0f;
    for (int j = 0; j < kD4; ++j) s += dy1[j] * W[kW4 + c * kD4 + j];
    dh[c] = s;
  }
  __syncthreads();
  // layer 3 (the max routes the gradient to one row per column)
  {
    const int c = tid, r = arg[c];
    const float gc = r >= 0 ? dh[c] : 0.0f;
    g[kB3 + c] = gc;
    for (int k = 0; k < kD2; ++k) {
      g[kW3 + k * kD3 + c] = r >= 0 ? a2[r * kD2 + k] * gc : 0.0f;
      if (r >= 0 && gc != 0.0f) atomicAdd(&da2[r * kD2 + k], W[kW3 + k * kD3 + c] * gc);
    }
  }
  __syncthreads();
  for (int i = tid; i < kPts * kD2; i += kTrainThreads)
    if (!(a2[i] > 0.0f)) da2[i] = 0.0f;  // dZ2
  __syncthreads();
  // layer 2: dW2[k][j] = sum_r a1[r][k] dZ2[r][j]; db2
  {
    const int j = tid & (kD2 - 1), kh = tid >> 7;
    float acc[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) acc[q] = 0.0f;
    float sb = 0.0f;
    for (int r = 0; r < kPts; ++r) {
      const float d = da2[r * kD2 + j];
      sb += d;
#pragma unroll
      for (int q = 0; q < 32; ++q) acc[q] += a1[r * kD1 + kh * 32 + q] * d;
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) g[kW2 + (kh * 32 + q) * kD2 + j] = acc[q];
    if (kh == 0) g[kB2 + j] = sb;
  }
  // dA1[r][k] = sum_j dZ2[r][j] W2[k][j], into the a2 region
  float* da1 = a2;
  {
    const int k = tid & (kD1 - 1), rq = tid >> 6;
    for (int r = rq * 32; r < rq * 32 + 32; ++r) {
      float s = 0.0f;
      for (int j = 0; j < kD2; ++j) s += da2[r * kD2 + j] * w2t[j * kW2Pad + k];
      da1[r * kD1 + k] = s;
    }
  }
  __syncthreads();
  for (int i = tid; i < kPts * kD1; i += kTrainThreads)
    if (!(a1[i] > 0.0f)) da1[i] = 0.0f;  // dZ1
  __syncthreads();
  if (tid < 3 * kD1) {
    const int dd = tid / kD1, k = tid % kD1;
    float s = 0.0f;
    for (int r = 0; r < kPts; ++r) s += x[3 * r + dd] * da1[r * kD1 + k];
    g[kW1 + dd * kD1 + k] = s;
  } else {
    const int k = tid - 3 * kD1;
    float s = 0.0f;
    for (int r = 0; r < kPts; ++r) s += da1[r * kD1 + k];
    g[kB1 + k] = s;
  }
}

// Mean gradient over the B slots (fixed order: deterministic).
__global__ void k_prop_reduce(const float* __restrict__ G, int B, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNumParams) return;
  float s = 0.0f;
  for (int b = 0; b < B; ++b) s += G[(size_t)b * kNumParams + p];
  grad[p] = s / (float)B;
}

__global__ void k_prop_adam(float* __restrict__ W, const float* __restrict__ grad,
                            float* __restrict__ m, float* __restrict__ v, float lr, float c1,
                            float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNumParams) return;
  const float gr = grad[p];
  const float mm = 0.9f * m[p] + 0.1f * gr, vv = 0.999f * v[p] + 0.001f * gr * gr;
  m[p] = mm;
  v[p] = vv;
  W[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
}

__global__ void k_prop_loss_mean(const float* __restrict__ loss, int B, float* __restrict__ out) {
  __shared__ float red[32];
  float s = 0.0f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) s += loss[b];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    *out = t / (float)B;
  }
}

// ----------------------------------------------------------- inference
SLOAM_D float bfr(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// BF16 operands in the tensor-core layout + bf16-rounded fp32 copies.
__global__ void k_prop_pack(const float* __restrict__ W, unsigned char* __restrict__ tcw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  __nv_bfloat16* b2 = reinterpret_cast<__nv_bfloat16*>(tcw);
  __nv_bfloat16* b3 = reinterpret_cast<__nv_bfloat16*>(tcw + kTcW2Bytes);
  float* f = reinterpret_cast<float*>(tcw + kTcF32Off);
  if (i < kD1 * kD2) {  // W2[k][j] -> W2^T (j, k), K = 64
    const int k = i / kD2, j = i % kD2;
    b2[core_offset(j, k, kD1) / 2] = __float2bfloat16_rn(W[kW2 + i]);
  }
  if (i < kD2 * kD3) {  // W3[k][c] -> W3^T (c, k), K = 128
    const int k = i / kD3, c = i % kD3;
    b3[core_offset(c, k, kD2) / 2] = __float2bfloat16_rn(W[kW3 + i]);
  }
  if (i < kNumParams) f[i] = bfr(W[i]);
  if (i < kD3 * kD4) {  // W4[c][j] -> W4^T (j, c), K = 256
    __nv_bfloat16* b4 = reinterpret_cast<__nv_bfloat16*>(tcw + kTcW4Off);
    const int c = i / kD4, j = i % kD4;
    b4[core_offset(j, c, kD3) / 2] = __float2bfloat16_rn(W[kW4 + i]);
  }
  if (i < kD4 * kD5)  // W5 [128][7] in bf16
    reinterpret_cast<__nv_bfloat16*>(tcw + kTcW5hOff)[i] = __float2bfloat16_rn(W[kW5 + i]);
  if (i < kSmallFloats) {  // W1 / b1 as float4 rows, b2, b3, b4, b5, pad, W5
    float v = 0.0f;
    if (i < kSfB2) {
      const int j = i >> 2, q = i & 3;
      v = W[q < 3 ? kW1 + q * kD1 + j : kB1 + j];
    } else if (i < kSfB3) {
      v = W[kB2 + i - kSfB2];
    } else if (i < kSfB4) {
      v = W[kB3 + i - kSfB3];
    } else if (i < kSfB5) {
      v = W[kB4 + i - kSfB4];
    } else if (i < kSfB5 + kD5) {
      v = W[kB5 + i - kSfB5];
    } else if (i >= kSfW5) {
      v = W[kW5 + i - kSfW5];
    }
    reinterpret_cast<float*>(tcw + kTcSmallOff)[i] = bfr(v);
  }
  if (i < kD2 * kK2x) {  // W2^T | b2 (128 x 80), K-major core matrices
    const int j = i / kK2x, k = i % kK2x;
    const float v = k < kD1 ? W[kW2 + k * kD2 + j] : (k == kD1 ? W[kB2 + j] : 0.0f);
    reinterpret_cast<__nv_bfloat16*>(tcw + kTcB2xOff)[core_offset(j, k, kK2x) / 2] =
        __float2bfloat16_rn(v);
  }
  if (i < kD1 * kK1) {  // B1 (64 x 16): W1 rows for the hi, mid, lo terms, b1
    const int j = i / kK1, k = i % kK1;
    const float v = k < 9 ? W[kW1 + (k % 3) * kD1 + j] : (k == 9 ? W[kB1 + j] : 0.0f);
    reinterpret_cast<__nv_bfloat16*>(tcw + kTcB1Off)[core_offset(j, k, kK1) / 2] =
        __float2bfloat16_rn(v);
  }
}

// SIMT reference of the tensor-core kernel: the same bf16 operands and
// roundings, FP32 accumulation.  One block (128 threads) per sample.
constexpr size_t kRefSmem = sizeof(float) * (kPts * kD1 + kPts * (kD2 + 1) + kD3 + kD4);

__global__ void __launch_bounds__(128) k_prop_infer_ref(const unsigned char* __restrict__ tcw,
                                                        const float* __restrict__ X, int S,
                                                        float* __restrict__ out) {
  extern __shared__ float rsm[];
  float* a1 = rsm;                       // [128][64]
  float* a2 = a1 + kPts * kD1;           // [128][129]
  float* h = a2 + kPts * (kD2 + 1);      // [256]
  float* y1 = h + kD3;                   // [128]
  const __nv_bfloat16* b2 = reinterpret_cast<const __nv_bfloat16*>(tcw);
  const __nv_bfloat16* b3 = reinterpret_cast<const __nv_bfloat16*>(tcw + kTcW2Bytes);
  const float* f = reinterpret_cast<const float*>(tcw + kTcF32Off);
  const int r = threadIdx.x;
  for (int s = blockIdx.x; s < S; s += gridDim.x) {
    const float* x = X + (size_t)s * kPts * 3;
    const float x0 = x[3 * r], x1 = x[3 * r + 1], x2 = x[3 * r + 2];
    for (int j = 0; j < kD1; ++j)
      a1[r * kD1 + j] = bfr(fmaxf(f[kB1 + j] + x0 * f[kW1 + j] + x1 * f[kW1 + kD1 + j] +
                                      x2 * f[kW1 + 2 * kD1 + j], 0.0f));
    __syncthreads();
    for (int j = 0; j < kD2; ++j) {
      float z = 0.0f;
      for (int k = 0; k < kD1; ++k)
        z += a1[r * kD1 + k] * __bfloat162float(b2[core_offset(j, k, kD1) / 2]);
      a2[r * (kD2 + 1) + j] = bfr(fmaxf(z + f[kB2 + j], 0.0f));
    }
    __syncthreads();
    for (int c = r; c < kD3; c += 128) {
      float best = 0.0f;
      for (int q = 0; q < kPts; ++q) {
        float z = 0.0f;
        for (int k = 0; k < kD2; ++k)
          z += a2[q * (kD2 + 1) + k] * __bfloat162float(b3[core_offset(c, k, kD2) / 2]);
        best = fmaxf(best, z + f[kB3 + c]);
      }
      h[c] = best;
    }
    __syncthreads();
    float z = f[kB4 + r];
    for (int c = 0; c < kD3; ++c) z += h[c] * f[kW4 + c * kD4 + r];
    y1[r] = fmaxf(z, 0.0f);
    __syncthreads();
    if (r < kD5) {
      float o = f[kB5 + r];
      for (int j = 0; j < kD4; ++j) o += y1[j] * f[kW5 + j * kD5 + r];
      out[(size_t)s * 8 + r] = o;
    }
    __syncthreads();
  }
}

// ------------------------------------------------- tcgen05 primitives
// shared-memory matrix descriptor: K-major, no swizzle; LBO = byte stride
// between core matrices along K, SBO = along M/N; version 1 (bit 46)
SLOAM_D uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor, kind::f16: D f32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
SLOAM_D void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
SLOAM_D void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   saddr(mbar))
               : "memory");
}
SLOAM_D void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
SLOAM_D void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
constexpr int kMbarSpin = 1 << 20;  // bounded wait (the MMAs take microseconds)

#define SG_TMEM_LD32(taddr, v)                                                                 \
  asm volatile(                                                                                \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"      \
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),   \
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),            \
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),         \
        "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),         \
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),         \
        "=r"(v[31])                                                                            \
      : "r"(taddr))
SLOAM_D void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory layout of the tensor-core inference kernel below, which runs
// with WG warpgroups (one sample each at a time): four for large standalone
// launches (one CTA per SM, the SM to itself), two inside the keyframe
// pipeline (the CTA leaves registers and shared memory for other kernels).
constexpr int kMaxGroup = 8;     // samples per group (one tree's proposals)
// Per warpgroup one 32 KB operand buffer: A1 [128 x 80] (the ones column
// at 64 carries b2) at its start and A0 [128 x 16] (layer-1 input) after
// it while layers 1 and 2 run, then A2 [128 x 128] (written once the
// layer-2 MMAs, which read A1, have completed).  Between groups the
// operand buffers hold the head's W4^T (64 KB, bulk copy), and the head's
// outputs go to Ht once the head MMA, which reads Ht, has completed.
// W2^T | b2, W3^T, B1, the biases and W5 arrive by bulk copy from the
// packed device layout.  Ht [16 x 256] is the head's B operand: the
// max-pooled features of sample k split exactly into bf16 hi (row k) and
// lo (row 8 + k) terms.
constexpr uint32_t kSmB2 = 0, kSmB3 = kSmB2 + kTcB2xBytes,
                   kSmA2 = kSmB3 + kTcW3Bytes,                    // [wg][32 KB]
                   kSmallCopy = 4 * (kSfW5 - kSfB3);
constexpr uint32_t kOpA0 = kPts * kK2x * 2;                       // A0 inside the buffer
template <int WG>
struct TcLayout {
  static constexpr int kThreads = 128 * WG;
  static constexpr uint32_t kB1 = kSmA2 + WG * kPts * kD2 * 2,   // [64 x 16] bf16
      kHt = kB1 + kTcB1Bytes,                                     // [16 x 256] bf16
      kSmall = kHt + 2 * kMaxGroup * kD3 * 2,                     // b3, b4, b5
      kW5h = kSmall + kSmallCopy,                                 // W5 [128][7] bf16
      kMisc = kW5h + kTcW5hBytes,
      kSmem = kMisc + 64;
  static constexpr uint32_t kTmemCols = 128 * WG;                 // 128 columns per warpgroup
  static_assert(WG == 2 || WG == 4, "TMEM allocation: a power of two");
  static_assert(kB1 % 128 == 0 && kHt % 128 == 0, "operand alignment");
  static_assert(kSmall % 16 == 0 && kW5h % 16 == 0 && kMisc % 16 == 0, "16-byte alignment");
  static_assert(kSmem <= 227 * 1024, "shared memory");
  static_assert(kTcW4Bytes <= WG * kPts * kD2 * 2, "W4^T inside the operand buffers");
};
static_assert(kSmA2 % 128 == 0 && kSmB3 % 128 == 0 && kOpA0 % 128 == 0, "operand alignment");
static_assert(kOpA0 + kPts * kK1 * 2 <= kPts * kD2 * 2, "A1 and A0 inside the A2 buffer");
static_assert(kMaxGroup * kD4 * 4 <= 2 * kMaxGroup * kD3 * 2, "head outputs inside Ht");
static_assert(2 * kMaxGroup == 16, "head MMA: N = 16 (hi and lo rows of 8 samples)");
// the descriptors address at most: A0 [128 x 16], A1 [128 x 80], A2
// [128 x 128], B1 [64 x 16], W2^T | b2 [128 x 80], W3^T [256 x 128], W4^T
// [128 x 256], Ht [16 x 256]; every core matrix lies inside its buffer
static_assert(core_offset(kPts - 1, kK1 - 1, kK1) + 2 <= kPts * kK1 * 2, "A0 extent");
static_assert(core_offset(kPts - 1, kK2x - 1, kK2x) + 2 <= kOpA0, "A1 extent");
static_assert(core_offset(kD1 - 1, kK1 - 1, kK1) + 2 <= kTcB1Bytes, "B1 extent");
static_assert(core_offset(kD2 - 1, kK2x - 1, kK2x) + 2 <= kTcB2xBytes, "W2 extent");
static_assert(core_offset(kD3 - 1, kD2 - 1, kD2) + 2 <= kTcW3Bytes, "W3 extent");
static_assert(core_offset(kD4 - 1, kD3 - 1, kD3) + 2 <= kTcW4Bytes, "W4 extent");
static_assert(core_offset(2 * kMaxGroup - 1, kD3 - 1, kD3) + 2 <= 2 * kMaxGroup * kD3 * 2,
              "Ht extent");

SLOAM_D bool mbar_wait_bounded(uint64_t* m, uint32_t phase, int* err, int* abort_flag) {
  int it = 0;
  while (!mbar_test(m, phase) && ++it < kMbarSpin) {
  }
  if (it >= kMbarSpin) {
    atomicOr(err, 1);
    *abort_flag = 1;
    return false;
  }
  return true;
}
// ReLU, round to bf16 and pack: lo in the low half, hi in the high half
SLOAM_D uint32_t relu_bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}
SLOAM_D float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
// barrier of one warpgroup (128 threads); ids 1..kTcWg (0 is __syncthreads)
SLOAM_D void wg_sync(int wg) { asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory"); }
// the same barrier, returning the OR of p over the warpgroup: a decision
// every thread of the warpgroup takes alike
SLOAM_D bool wg_any(int wg, bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, d;\n\tsetp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred d, %2, 128, q;\n\tselp.u32 %0, 1, 0, d;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(1 + wg)
      : "memory");
  return r != 0;
}

// Tensor-core inference.  Persistent CTAs (one per SM at most: the shared
// memory allows no second) over groups of `group` samples -- in the
// pipeline one tree's proposals; groups whose frame scale is 0 (trees not
// fitted) are skipped.  kTcWg warpgroups: warpgroup g takes samples
// g, g + kTcWg, ... of the group with its own operand buffer, TMEM columns
// [128 g, 128 g + 128), mbarrier and barrier, so that one warpgroup's MMAs
// overlap the others' CUDA-core work; its next sample's points are loaded
// while it works on the current one.  Per sample (thread r = point r):
// layer 1 as one tcgen05.mma M=128 points, N=64, K=16 -- each FP32
// coordinate split exactly into three bf16 terms (hi + mid + lo) against
// W1 repeated three times, and a ones column against b1 -- then ReLU and
// bf16 into A1; layer 2 as M=128 points, N=128, K=80 (A1's ones column
// against b2); ReLU and bf16 into A2; layer 3 transposed, M=128 features
// (two halves of W3^T), N=128 points, K=128, so that TMEM lane r holds
// feature r of a half and the max over the points is a register reduction
// of the thread's own row; bias and ReLU, and the feature goes to Ht as
// bf16 hi and lo terms.  The head is one MMA per group, M=128 outputs,
// N=16 (hi and lo of 8 samples), K=256, A = W4^T; then bias and ReLU, and
// one warp per (sample, output) for the last layer.  bf16 operands in
// shared memory, fp32 accumulators in TMEM.
template <int kTcWg>
__global__ void __launch_bounds__(128 * kTcWg, 4 / kTcWg) k_prop_infer_tc(
    const unsigned char* __restrict__ tcw, const float* __restrict__ X, int S,
    const int* __restrict__ n_groups_dev, int group, const float4* __restrict__ frames,
    float* __restrict__ out, int* __restrict__ err) {
  using L = TcLayout<kTcWg>;
  constexpr int kTcThreads = L::kThreads;
  constexpr uint32_t kSmB1 = L::kB1, kSmHt = L::kHt, kSmSmall = L::kSmall, kSmW5h = L::kW5h,
                     kSmMisc = L::kMisc, kTmemCols = L::kTmemCols;
  extern __shared__ __align__(128) unsigned char smem[];
  const float* sb3 = reinterpret_cast<const float*>(smem + kSmSmall);  // b3, b4, b5
  const float* sb4 = sb3 + (kSfB4 - kSfB3);
  const float* sb5 = sb3 + (kSfB5 - kSfB3);
  const __nv_bfloat16* sw5 = reinterpret_cast<const __nv_bfloat16*>(smem + kSmW5h);
  unsigned char* htb = smem + kSmHt;
  float* y1 = reinterpret_cast<float*>(htb);  // [group][128], after the head MMA
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kSmMisc);  // [kTcWg]
  uint64_t* lbar = mbar + kTcWg;  // bulk copies and the head MMA
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kSmMisc + 8 * kTcWg + 8);
  int* abort_flag = reinterpret_cast<int*>(smem + kSmMisc + 8 * kTcWg + 12);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid >> 7, lt = tid & 127, wq = warp & 3;
  unsigned char* a2b = smem + kSmA2 + wg * kPts * kD2 * 2;
  unsigned char* a1b = a2b;
  unsigned char* a0b = a2b + kOpA0;
  // groups: ceil(S / group), or the device count of groups when given
  int ng = (S + group - 1) / group;
  if (n_groups_dev) ng = min(ng, *n_groups_dev);
  if ((int)blockIdx.x >= ng) return;
  // this warpgroup's next sample and its point (row lt), loaded ahead
  int pf_s = -1;
  float px0 = 0.f, px1 = 0.f, px2 = 0.f;
  auto prefetch = [&](int s) {
    pf_s = s;
    if (s >= 0) {
      const float* x = X + (size_t)s * kPts * 3 + 3 * lt;
      px0 = x[0];
      px1 = x[1];
      px2 = x[2];
    }
  };
  {
    const int s = blockIdx.x * group + wg;
    prefetch(wg < min(group, S - (int)blockIdx.x * group) ? s : -1);
  }

  if (tid == 0) {
    for (int q = 0; q < kTcWg; ++q) mbar_init(mbar + q, 1);
    mbar_init(lbar, 1);
    *abort_flag = 0;
    mbar_init_fence();
    mbar_expect_tx(lbar, kTcB2xBytes + kTcW3Bytes + kTcB1Bytes + kSmallCopy + kTcW5hBytes);
    bulk_load(saddr(smem + kSmB2), tcw + kTcB2xOff, kTcB2xBytes, lbar);
    bulk_load(saddr(smem + kSmB3), tcw + kTcW2Bytes, kTcW3Bytes, lbar);
    bulk_load(saddr(smem + kSmB1), tcw + kTcB1Off, kTcB1Bytes, lbar);
    bulk_load(saddr(smem + kSmSmall), tcw + kTcSmallOff + 4 * kSfB3, kSmallCopy, lbar);
    bulk_load(saddr(smem + kSmW5h), tcw + kTcW5hOff, kTcW5hBytes, lbar);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tslot)), "n"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  uint32_t lph = 0;  // parity of lbar's next phase
  mbar_wait_bounded(lbar, lph, err, abort_flag);
  lph ^= 1u;
  if (__syncthreads_or(*abort_flag != 0)) {
    // the copies may still be in flight: wait for them (bounded) before the
    // shared memory is given up
    mbar_wait_bounded(lbar, 0, err, abort_flag);
    ng = 0;
  }
  const uint32_t tmem0 = *tslot;
  const uint32_t tmem = tmem0 + (uint32_t)(wg * 128);  // 128 columns per warpgroup
  const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
  const uint32_t sA0 = saddr(a0b), sA1 = saddr(a1b), sA2 = saddr(a2b);
  const uint32_t sB1 = saddr(smem + kSmB1), sB2 = saddr(smem + kSmB2),
                 sB3 = saddr(smem + kSmB3), sW4 = saddr(smem + kSmA2), sHt = saddr(htb);
  uint64_t* mb = mbar + wg;
  uint32_t phase = 0;

  for (int g = blockIdx.x; g < ng; g += gridDim.x) {
    const int s0 = g * group, gs = min(group, S - s0);
    if (frames && !(frames[s0].w > 0.0f)) {  // block-uniform
      const int g2 = g + gridDim.x;
      if (g2 < ng && wg < min(group, S - g2 * group)) prefetch(g2 * group + wg);
      continue;
    }
    for (int k = wg; k < gs; k += kTcWg) {
      const int s = s0 + k;
      if (pf_s != s) prefetch(s);
      const float x0 = px0, x1 = px1, x2 = px2;
      {  // the next sample of this warpgroup: in this group, else the next group's
        const int g2 = g + gridDim.x;
        if (k + kTcWg < gs) prefetch(s + kTcWg);
        else if (g2 < ng && wg < min(group, S - g2 * group)) prefetch(g2 * group + wg);
      }
      // A0 row lt: x = hi + mid + lo in bf16 (exact), then 1 (b1)
      {
        const float xv[3] = {x0, x1, x2};
        uint32_t t[9];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float v = xv[d];
          const __nv_bfloat16 hi = __float2bfloat16_rn(v);
          const float r1 = v - __bfloat162float(hi);
          const __nv_bfloat16 mi = __float2bfloat16_rn(r1);
          const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mi));
          t[d] = __bfloat16_as_ushort(hi);
          t[3 + d] = __bfloat16_as_ushort(mi);
          t[6 + d] = __bfloat16_as_ushort(lo);
        }
        *reinterpret_cast<uint4*>(a0b + core_offset(lt, 0, kK1)) =
            make_uint4(t[0] | (t[1] << 16), t[2] | (t[3] << 16), t[4] | (t[5] << 16),
                       t[6] | (t[7] << 16));
        *reinterpret_cast<uint4*>(a0b + core_offset(lt, 8, kK1)) =
            make_uint4(t[8] | (0x3F80u << 16), 0u, 0u, 0u);
      }
      fence_async_smem();
      fence_before();
      wg_sync(wg);
      fence_after();
      if (lt == 0) {
        mma_bf16(tmem, smem_desc(sA0, 128, (kK1 / 8) * 128), smem_desc(sB1, 128, (kK1 / 8) * 128),
                 idesc_bf16(128, kD1), 0);
        mma_commit(mb);
      }
      mbar_wait_bounded(mb, phase, err, abort_flag);
      phase ^= 1u;
      fence_after();
      // epilogue 1: ReLU, bf16 -> A1 columns 0..63; column 64 = 1 (b2)
#pragma unroll
      for (int cc = 0; cc < kD1 / 32; ++cc) {
        uint32_t v[32];
        SG_TMEM_LD32(tmem + lane_base + cc * 32, v);
        tmem_wait_ld();
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) {
          uint4 pk;
          pk.x = relu_bf16x2(__uint_as_float(v[k0]), __uint_as_float(v[k0 + 1]));
          pk.y = relu_bf16x2(__uint_as_float(v[k0 + 2]), __uint_as_float(v[k0 + 3]));
          pk.z = relu_bf16x2(__uint_as_float(v[k0 + 4]), __uint_as_float(v[k0 + 5]));
          pk.w = relu_bf16x2(__uint_as_float(v[k0 + 6]), __uint_as_float(v[k0 + 7]));
          *reinterpret_cast<uint4*>(a1b + core_offset(lt, cc * 32 + k0, kK2x)) = pk;
        }
      }
      *reinterpret_cast<uint4*>(a1b + core_offset(lt, kD1, kK2x)) = make_uint4(0x3F80u, 0u, 0u, 0u);
      *reinterpret_cast<uint4*>(a1b + core_offset(lt, kD1 + 8, kK2x)) = make_uint4(0u, 0u, 0u, 0u);
      fence_async_smem();
      fence_before();
      wg_sync(wg);
      fence_after();
      if (lt == 0) {
        for (int ks = 0; ks < kK2x / 16; ++ks)
          mma_bf16(tmem, smem_desc(sA1 + ks * 256, 128, (kK2x / 8) * 128),
                   smem_desc(sB2 + ks * 256, 128, (kK2x / 8) * 128), idesc_bf16(128, kD2), ks > 0);
        mma_commit(mb);
      }
      mbar_wait_bounded(mb, phase, err, abort_flag);
      phase ^= 1u;
      fence_after();
      // epilogue 2: ReLU, bf16 -> A2 (b2 came with the MMA)
      for (int cc = 0; cc < kD2 / 32; ++cc) {
        uint32_t v[32];
        SG_TMEM_LD32(tmem + lane_base + cc * 32, v);
        tmem_wait_ld();
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) {
          uint4 pk;
          pk.x = relu_bf16x2(__uint_as_float(v[k0]), __uint_as_float(v[k0 + 1]));
          pk.y = relu_bf16x2(__uint_as_float(v[k0 + 2]), __uint_as_float(v[k0 + 3]));
          pk.z = relu_bf16x2(__uint_as_float(v[k0 + 4]), __uint_as_float(v[k0 + 5]));
          pk.w = relu_bf16x2(__uint_as_float(v[k0 + 6]), __uint_as_float(v[k0 + 7]));
          *reinterpret_cast<uint4*>(a2b + core_offset(lt, cc * 32 + k0, kD2)) = pk;
        }
      }
      fence_async_smem();
      fence_before();
      if (wg_any(wg, *abort_flag != 0)) break;  // uniform over the warpgroup
      fence_after();
      // layer 3 transposed: D^T[feature][point] = W3^T[feature][:] . A2[point][:],
      // one M = 128 feature half at a time (A = W3^T rows, B = A2, N = 128
      // points) into the warpgroup's 128 TMEM columns.  Thread (TMEM lane)
      // = feature: the max over the points is a register reduction of its
      // row, then bias and ReLU (both monotone, so max then bias/ReLU equals
      // the max of the biased ReLU outputs).
      bool ab = false;
      for (int hf = 0; hf < 2 && !ab; ++hf) {
        if (lt == 0) {
          for (int ks = 0; ks < kD2 / 16; ++ks)
            mma_bf16(tmem,
                     smem_desc(sB3 + hf * (kPts * kD2 * 2) + ks * 256, 128, (kD2 / 8) * 128),
                     smem_desc(sA2 + ks * 256, 128, (kD2 / 8) * 128), idesc_bf16(128, kPts),
                     ks > 0);
          mma_commit(mb);
        }
        mbar_wait_bounded(mb, phase, err, abort_flag);
        phase ^= 1u;
        fence_after();
        float m = -INFINITY;
#pragma unroll 1
        for (int cc = 0; cc < kPts / 32; ++cc) {
          uint32_t v[32];
          SG_TMEM_LD32(tmem + lane_base + cc * 32, v);
          tmem_wait_ld();
#pragma unroll
          for (int q = 0; q < 32; q += 2)
            m = max3f(m, __uint_as_float(v[q]), __uint_as_float(v[q + 1]));
        }
        // feature c of sample k -> Ht rows k (hi) and 8 + k (lo)
        const int c = hf * kPts + lt;
        const float hv = fmaxf(m + sb3[c], 0.0f);
        const __nv_bfloat16 hh = __float2bfloat16_rn(hv);
        const __nv_bfloat16 hl = __float2bfloat16_rn(hv - __bfloat162float(hh));
        *reinterpret_cast<__nv_bfloat16*>(htb + core_offset(k, c, kD3)) = hh;
        *reinterpret_cast<__nv_bfloat16*>(htb + core_offset(kMaxGroup + k, c, kD3)) = hl;
        fence_async_smem();
        // barrier: the next half's MMAs (or the next sample's) overwrite
        // these columns
        fence_before();
        ab = wg_any(wg, *abort_flag != 0);
        fence_after();
      }
      if (ab) break;
    }
    fence_before();
    const int ab_all = __syncthreads_or(*abort_flag != 0);
    fence_after();
    if (ab_all) break;
    // head: W4^T into the operand buffers (free: every MMA that read them
    // has completed), then D[j][n] = W4^T[j][:] . Ht[n][:] into warpgroup
    // 0's TMEM columns 0..15
    if (tid == 0) {
      mbar_expect_tx(lbar, kTcW4Bytes);
      bulk_load(sW4, tcw + kTcW4Off, kTcW4Bytes, lbar);
      mbar_wait_bounded(lbar, lph, err, abort_flag);
      fence_after();
      if (!*abort_flag) {
        for (int ks = 0; ks < kD3 / 16; ++ks)
          mma_bf16(tmem0, smem_desc(sW4 + ks * 256, 128, (kD3 / 8) * 128),
                   smem_desc(sHt + ks * 256, 128, (kD3 / 8) * 128), idesc_bf16(128, 2 * kMaxGroup),
                   ks > 0);
        mma_commit(lbar);
      }
    }
    fence_before();
    if (__syncthreads_or(*abort_flag != 0)) {
      // the copy may still be in flight (its wait timed out): wait for it
      // (bounded) before the shared memory is given up
      if (tid == 0) mbar_wait_bounded(lbar, lph, err, abort_flag);
      __syncthreads();
      break;
    }
    lph ^= 1u;
    mbar_wait_bounded(lbar, lph, err, abort_flag);  // the head MMA
    lph ^= 1u;
    fence_after();
    if (wg == 0) {
      // lane j = output j: y1[k][j] = ReLU(b4[j] + hi part + lo part)
      uint32_t v[32];
      SG_TMEM_LD32(tmem0 + lane_base, v);
      tmem_wait_ld();
      const float b = sb4[lt];
#pragma unroll
      for (int k = 0; k < kMaxGroup; ++k)
        if (k < gs)
          y1[k * kD4 + lt] =
              fmaxf(b + (__uint_as_float(v[k]) + __uint_as_float(v[kMaxGroup + k])), 0.0f);
    }
    fence_before();
    if (__syncthreads_or(*abort_flag != 0)) break;
    fence_after();
    // last layer: warp w takes the (sample, output) pairs w + 16 i, i < 4,
    // side by side
    {
      constexpr int kPairW = (kMaxGroup * kD5 + kTcThreads / 32 - 1) / (kTcThreads / 32);
      float z[kPairW];
#pragma unroll
      for (int i = 0; i < kPairW; ++i) {
        const int p = warp + i * (kTcThreads / 32);
        z[i] = 0.0f;
        if (p < gs * kD5) {
          const int k = p / kD5, o = p - k * kD5;
#pragma unroll
          for (int j = lane; j < kD4; j += 32)
            z[i] += y1[k * kD4 + j] * __bfloat162float(sw5[j * kD5 + o]);
        }
      }
#pragma unroll
      for (int i = 0; i < kPairW; ++i) z[i] = warp_sum(z[i]);
#pragma unroll
      for (int i = 0; i < kPairW; ++i) {
        const int p = warp + i * (kTcThreads / 32);
        if (lane == 0 && p < gs * kD5) {
          const int k = p / kD5, o = p - k * kD5;
          out[(size_t)(s0 + k) * 8 + o] = z[i] + sb5[o];
        }
      }
    }
    fence_before();
    __syncthreads();
    fence_after();
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot),
                 "n"(kTmemCols)
                 : "memory");
}

int g_tc_attr = 0;
// Persistent CTAs of the per-keyframe launch, two warpgroups each (160 KB of
// shared memory and 256 threads: the rest of the SM stays open to the
// batch's other kernels, where four warpgroups filled it and every CTA
// waited for an SM to drain).  On the 32-slot 64x2048 batch two warpgroups
// ran the learned path 1.3-1.7 % faster than four; 24 CTAs, two trees each for
// the scene's ~40 trees, beat 16, 20, 30, 36 and 48.
constexpr int kTreeWg = 2;
constexpr int kTreeCtas = 24;
// standalone launches (many groups): four warpgroups, one CTA per SM
constexpr int kBulkWg = 4;

}  // namespace

void init_attributes() {
  if (g_tc_attr) return;
  cudaFuncSetAttribute(k_prop_infer_tc<kTreeWg>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)TcLayout<kTreeWg>::kSmem);
  cudaFuncSetAttribute(k_prop_infer_tc<kBulkWg>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)TcLayout<kBulkWg>::kSmem);
  cudaFuncSetAttribute(k_prop_infer_ref, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kRefSmem);
  g_tc_attr = 1;
}

static int sm_count() {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

int launch_prop_infer_trees(const unsigned char* d_tcw, const float* d_x, const int* d_n_trees,
                            int per_tree, int cap, const float4* d_frames, float* d_out,
                            int* d_err, cudaStream_t st) {
  init_attributes();
  // persistent CTAs over the trees: at most kTreeCtas, each of which needs
  // a whole SM, so that the many CTAs of a large capacity do not each wait
  // for an empty SM only to exit
  const int groups = (cap + per_tree - 1) / per_tree;
  const int lim = sm_count() < kTreeCtas ? sm_count() : kTreeCtas;
  const int grid = groups < lim ? (groups > 0 ? groups : 1) : lim;
  k_prop_infer_tc<kTreeWg><<<grid, TcLayout<kTreeWg>::kThreads, TcLayout<kTreeWg>::kSmem, st>>>(
      d_tcw, d_x, cap, d_n_trees, per_tree, d_frames, d_out, d_err);
  return 1;
}

int launch_prop_pack(const float* d_w, unsigned char* d_tcw, cudaStream_t st) {
  k_prop_pack<<<(kNumParams + 255) / 256, 256, 0, st>>>(d_w, d_tcw);
  return 1;
}

int launch_prop_infer(const unsigned char* d_tcw, const float* d_x, int n, float* d_out,
                      int* d_err, int mode, cudaStream_t st) {
  if (n <= 0) return 0;
  init_attributes();
  if (mode == 1) {
    k_prop_infer_ref<<<n, 128, kRefSmem, st>>>(d_tcw, d_x, n, d_out);
    return 1;
  }
  const int groups = (n + kMaxGroup - 1) / kMaxGroup;
  const int grid = groups < sm_count() ? groups : sm_count();
  k_prop_infer_tc<kBulkWg><<<grid, TcLayout<kBulkWg>::kThreads, TcLayout<kBulkWg>::kSmem, st>>>(
      d_tcw, d_x, n, nullptr, kMaxGroup, nullptr, d_out, d_err);
  return 1;
}

}  // namespace prop
}  // namespace sg

using namespace sg::prop;

namespace {
int prop_fail(const char* what, cudaError_t e) {
  std::fprintf(stderr, "sloam proposal: %s: %s\n", what, cudaGetErrorString(e));
  return SLOAM_ERR_CUDA;
}
#define PCK(call)                                  \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return prop_fail(#call, e_); \
  } while (0)
}  // namespace

extern "C" int sloam_prop_num_params(void) { return kNumParams; }

extern "C" int sloam_prop_sample(uint64_t seed, int64_t first_id, int32_t n, float* d_points,
                                 float* d_targets) {
  if (n < 0 || (n > 0 && (!d_points || !d_targets))) return SLOAM_ERR_ARG;
  if (n == 0) return SLOAM_OK;
  k_prop_sample<<<n, 128>>>(seed, first_id, d_points, d_targets);
  PCK(cudaGetLastError());
  PCK(cudaDeviceSynchronize());
  return SLOAM_OK;
}

extern "C" int sloam_prop_train(const float* init, int32_t steps, int32_t batch, float lr,
                                uint64_t seed, int64_t first_id, float* weights_out,
                                float* loss_out) {
  if (steps < 0 || batch < 1 || !weights_out) return SLOAM_ERR_ARG;
  float *W = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *G = nullptr, *X = nullptr,
        *T = nullptr, *L = nullptr, *Lm = nullptr;
  auto release = [&]() {
    for (float* p : {W, m, v, grad, G, X, T, L, Lm})
      if (p) cudaFree(p);
  };
  const size_t np = kNumParams;
  cudaError_t e = cudaSuccess;
  for (auto pp : {&W, &m, &v, &grad}) {
    if (e == cudaSuccess) e = cudaMalloc(pp, sizeof(float) * np);
  }
  if (e == cudaSuccess) e = cudaMalloc(&G, sizeof(float) * np * batch);
  if (e == cudaSuccess) e = cudaMalloc(&X, sizeof(float) * 384 * batch);
  if (e == cudaSuccess) e = cudaMalloc(&T, sizeof(float) * kTgt * batch);
  if (e == cudaSuccess) e = cudaMalloc(&L, sizeof(float) * batch);
  if (e == cudaSuccess) e = cudaMalloc(&Lm, sizeof(float) * (steps > 0 ? steps : 1));
  if (e != cudaSuccess) {
    release();
    return prop_fail("allocation", e);
  }
  cudaMemset(m, 0, sizeof(float) * np);
  cudaMemset(v, 0, sizeof(float) * np);
  if (init)
    e = cudaMemcpy(W, init, sizeof(float) * np, cudaMemcpyHostToDevice);
  else
    k_prop_init<<<(kNumParams + 255) / 256, 256>>>(W, seed);
  const size_t smem = sizeof(float) * kTrainSmemFloats;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_prop_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  float c1 = 1.0f, c2 = 1.0f;
  for (int s = 0; s < steps && e == cudaSuccess; ++s) {
    k_prop_sample<<<batch, 128>>>(seed ^ 0x5a5a5a5aull, first_id + (int64_t)s * batch, X, T);
    k_prop_train<<<batch, kTrainThreads, smem>>>(W, X, T, G, L);
    k_prop_reduce<<<(kNumParams + 255) / 256, 256>>>(G, batch, grad);
    c1 *= 0.9f;
    c2 *= 0.999f;
    k_prop_adam<<<(kNumParams + 255) / 256, 256>>>(W, grad, m, v, lr, 1.0f - c1, 1.0f - c2);
    k_prop_loss_mean<<<1, 256>>>(L, batch, Lm + s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(weights_out, W, sizeof(float) * np, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss_out && steps > 0)
    e = cudaMemcpy(loss_out, Lm, sizeof(float) * steps, cudaMemcpyDeviceToHost);
  release();
  if (e != cudaSuccess) return prop_fail("training", e);
  return SLOAM_OK;
}

// One training step's backward pass alone: the per-cluster forward, loss and
// gradient of k_prop_train over n samples (device arrays of 384 and kTgt
// floats each), then their mean (k_prop_reduce).  grad_out receives the
// kNumParams mean gradient, loss_out (may be NULL) the n per-cluster losses.
extern "C" int sloam_prop_grad(const float* weights, const float* d_points,
                               const float* d_targets, int32_t n, float* grad_out,
                               float* loss_out) {
  if (!weights || !grad_out || n < 1 || !d_points || !d_targets) return SLOAM_ERR_ARG;
  float *W = nullptr, *G = nullptr, *grad = nullptr, *L = nullptr;
  cudaError_t e = cudaMalloc(&W, sizeof(float) * kNumParams);
  if (e == cudaSuccess) e = cudaMalloc(&G, sizeof(float) * kNumParams * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&grad, sizeof(float) * kNumParams);
  if (e == cudaSuccess) e = cudaMalloc(&L, sizeof(float) * n);
  if (e == cudaSuccess)
    e = cudaMemcpy(W, weights, sizeof(float) * kNumParams, cudaMemcpyHostToDevice);
  const size_t smem = sizeof(float) * kTrainSmemFloats;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_prop_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    k_prop_train<<<n, kTrainThreads, smem>>>(W, d_points, d_targets, G, L);
    k_prop_reduce<<<(kNumParams + 255) / 256, 256>>>(G, n, grad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemcpy(grad_out, grad, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss_out)
    e = cudaMemcpy(loss_out, L, sizeof(float) * n, cudaMemcpyDeviceToHost);
  for (float* p : {W, G, grad, L})
    if (p) cudaFree(p);
  if (e != cudaSuccess) return prop_fail("gradient", e);
  return SLOAM_OK;
}

extern "C" int sloam_prop_infer(const float* weights, const float* d_points, int32_t n,
                                float* d_out, int32_t mode) {
  if (!weights || n < 0 || (n > 0 && (!d_points || !d_out)) || mode < 0 || mode > 1)
    return SLOAM_ERR_ARG;
  float* W = nullptr;
  unsigned char* tcw = nullptr;
  int* err = nullptr;
  cudaError_t e = cudaMalloc(&W, sizeof(float) * kNumParams);
  if (e == cudaSuccess) e = cudaMalloc(&tcw, kTcBytes);
  if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(W, weights, sizeof(float) * kNumParams, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
  int herr = 0;
  if (e == cudaSuccess) {
    sg::prop::launch_prop_pack(W, tcw, 0);
    sg::prop::launch_prop_infer(tcw, d_points, n, d_out, err, mode, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
  }
  if (W) cudaFree(W);
  if (tcw) cudaFree(tcw);
  if (err) cudaFree(err);
  if (e != cudaSuccess) return prop_fail("inference", e);
  return herr ? SLOAM_ERR_TIMEOUT : SLOAM_OK;
}
