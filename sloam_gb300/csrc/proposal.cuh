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
// (256 x 128) in the core-matrix layout; fp32 copies of all parameters
// rounded to bf16 values (parameter order); W4^T (128 x 256) in the
// core-matrix layout; the small fp32 block (W1 and b1 as float4 (w0j, w1j,
// w2j, b1j), b2, b3, b4, b5 (+1 pad), W5, of which the tensor-core kernel
// copies b3, b4 and b5; the rest is spare); and the tensor-core kernel's
// own operands: W2^T extended by b2 as column 64 (128 x 80, K = 80: A1
// carries a ones column there), B1 (64 x 16): W1 rows 0-2 repeated three
// times (for the three bf16 terms of each FP32 coordinate) and b1 as
// column 9, so that layer 1 is one MMA; and W5 in bf16 ([128][7]).
constexpr int kTcW2Bytes = kD2 * kD1 * 2;           // 16 KB
constexpr int kTcW3Bytes = kD3 * kD2 * 2;           // 64 KB
constexpr int kTcF32Off = kTcW2Bytes + kTcW3Bytes;  // fp32 part after the bf16 operands
constexpr int kTcW4Off = (kTcF32Off + 4 * kNumParams + 15) / 16 * 16;
constexpr int kTcW4Bytes = kD3 * kD4 * 2;           // 64 KB
constexpr int kTcSmallOff = kTcW4Off + kTcW4Bytes;
constexpr int kSfW1 = 0, kSfB2 = kSfW1 + 4 * kD1, kSfB3 = kSfB2 + kD2, kSfB4 = kSfB3 + kD3,
              kSfB5 = kSfB4 + kD4, kSfW5 = kSfB5 + 8,
              kSmallFloats = kSfW5 + kD4 * kD5;     // float offsets in the small block
constexpr int kTcSmallBytes = 4 * kSmallFloats;
constexpr int kK2x = kD1 + 16;                      // layer-2 K with the bias column
constexpr int kK1 = 16;                             // layer-1 K: 3 x 3 terms + bias
constexpr int kTcB2xOff = kTcSmallOff + kTcSmallBytes;
constexpr int kTcB2xBytes = kD2 * kK2x * 2;         // 20 KB
constexpr int kTcB1Off = kTcB2xOff + kTcB2xBytes;
constexpr int kTcB1Bytes = kD1 * kK1 * 2;           // 2 KB
constexpr int kTcW5hOff = kTcB1Off + kTcB1Bytes;
constexpr int kTcW5hBytes = kD4 * kD5 * 2;          // 1792 B
constexpr int kTcBytes = kTcW5hOff + kTcW5hBytes;
static_assert(kTcW4Off % 16 == 0 && kTcSmallOff % 16 == 0 && kTcSmallBytes % 16 == 0 &&
                  kTcB2xOff % 16 == 0 && kTcB1Off % 16 == 0 && kTcW5hOff % 16 == 0 &&
                  kTcW5hBytes % 16 == 0 && kTcW2Bytes % 16 == 0 && kTcW3Bytes % 16 == 0 &&
                  kTcW4Bytes % 16 == 0 && (4 * kSfB3) % 16 == 0 && (4 * kSfW5) % 16 == 0,
              "bulk-copy alignment");

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
