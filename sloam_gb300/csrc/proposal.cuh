// proposal.cuh — the learned cylinder proposal: a point-set network over
// 128 points of one trunk cluster (centred, scale-normalised), shared MLP
// 3 -> 64 -> 128 -> 256 (ReLU), max-pool over the points, head
// 256 -> 128 (ReLU) -> 7: axis (3, unnormalised), centre xy (2: the axis
// point nearest the cluster mean, in the normalised frame; z follows from
// orthogonality to the axis), log(radius / scale), confidence logit.
// 75 399 parameters, FP32 master copy in this order (row-major W[in][out]).
#pragma once
#include <stdint.h>

namespace sg {
namespace prop {

constexpr int kPts = 128, kD1 = 64, kD2 = 128, kD3 = 256, kD4 = 128, kD5 = 7;
constexpr int kW1 = 0;                       // [3][64]
constexpr int kB1 = kW1 + 3 * kD1;           // [64]
constexpr int kW2 = kB1 + kD1;               // [64][128]
constexpr int kB2 = kW2 + kD1 * kD2;         // [128]
constexpr int kW3 = kB2 + kD2;               // [128][256]
constexpr int kB3 = kW3 + kD2 * kD3;         // [256]
constexpr int kW4 = kB3 + kD3;               // [256][128]
constexpr int kB4 = kW4 + kD3 * kD4;         // [128]
constexpr int kW5 = kB4 + kD4;               // [128][7]
constexpr int kB5 = kW5 + kD4 * kD5;         // [7]
constexpr int kNumParams = kB5 + kD5;        // 75 399
static_assert(kNumParams == 75399, "parameter count");

// Per-sample target / frame record: axis (3), centre xy (2), log radius,
// scale, spare.  The pipeline's samples carry the cluster mean instead.
constexpr int kTgt = 8;

// Inference operands in shared memory, bf16, "K-major, no swizzle" core
// matrices: element (r, k) of an R x K operand at byte
// ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
__host__ __device__ constexpr uint32_t core_offset(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// bf16 inference weights, one device block: W2^T (128 x 64) and W3^T
// (256 x 128) in the core-matrix layout, then fp32 copies of W1, b1, b2,
// b3, W4, b4, W5, b5 rounded to bf16 values.
constexpr int kTcW2Bytes = kD2 * kD1 * 2;           // 16 KB
constexpr int kTcW3Bytes = kD3 * kD2 * 2;           // 64 KB
constexpr int kTcF32Off = kTcW2Bytes + kTcW3Bytes;  // fp32 part after the bf16 operands
constexpr int kTcBytes = kTcF32Off + 4 * kNumParams;

}  // namespace prop
}  // namespace sg

#include "common.cuh"

namespace sg {
namespace prop {

// Centre and scale of a 128-point sample, by the 128 threads of a block
// (thread i holds point i): mean and RMS radius, then once more over the
// points within 2.5 RMS of that mean, so that range outliers move neither
// much.  `red` is 4 floats of shared memory.  Used identically by the
// training generator and by the pipeline.
__device__ __forceinline__ float block_sum128(float v, float* red) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  const float t = red[0] + red[1] + red[2] + red[3];
  __syncthreads();
  return t;
}
__device__ __forceinline__ void sample_frame(float px, float py, float pz, float* red, float* m,
                                             float* s) {
  float mx = block_sum128(px, red) / kPts, my = block_sum128(py, red) / kPts,
        mz = block_sum128(pz, red) / kPts;
  float dx = px - mx, dy = py - my, dz = pz - mz;
  const float s1 = sqrtf(block_sum128(dx * dx + dy * dy + dz * dz, red) / kPts);
  const float in = (dx * dx + dy * dy + dz * dz <= 6.25f * s1 * s1) ? 1.0f : 0.0f;
  const float n = fmaxf(block_sum128(in, red), 1.0f);
  mx = block_sum128(in * px, red) / n;
  my = block_sum128(in * py, red) / n;
  mz = block_sum128(in * pz, red) / n;
  dx = px - mx; dy = py - my; dz = pz - mz;
  m[0] = mx; m[1] = my; m[2] = mz;
  *s = sqrtf(block_sum128(in * (dx * dx + dy * dy + dz * dz), red) / n) + 1e-6f;
}

}  // namespace prop
}  // namespace sg
