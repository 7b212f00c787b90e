// project.cu — a1/a2: spherical range-image projection of the labelled scan
// (Segmentation::_doProjection, inference.cpp:80-165) and mask -> ground list
// + organised tree cloud (Segmentation::maskCloud / _destaggerCloud,
// inference.cpp:200-273).
//
// Arithmetic contract: range, z/range and the pixel row are IEEE float with
// round-to-nearest, unfused, in the reference's order; yaw and pitch are the
// correctly rounded float atan2/asin.  Yaw enters the column through a double
// expression, so the column is read from an exact boundary table built on the
// host (px_tab[k] = smallest float yaw whose column is >= k).  The fast path
// evaluates atan2f/asinf in FP32 and accepts the result when a +-1.2e-6
// relative margin (about 10 ulp, above the documented error of the CUDA
// functions) cannot change the pixel; otherwise the point takes the FP64
// path.  The nearest point wins its pixel (64-bit atomicMin on
// range-bits:index), ties to the lowest index.
#include "internal.h"
#include "scan_util.cuh"

namespace sg {

namespace {

__device__ __forceinline__ int px_from_yaw(const float* __restrict__ tab, float yaw, int W) {
  if (isnan(yaw)) return W - 1;  // std::min/max with NaN keep the bound
  float e = (yaw * 0.318309886f + 1.0f) * 0.5f * (float)W;
  int k = (int)floorf(fminf(fmaxf(e, -1.0f), (float)W));
  k = max(0, min(W - 1, k));
  while (k < W - 1 && yaw >= __ldg(tab + k + 1)) ++k;
  while (k > 0 && yaw < __ldg(tab + k)) --k;
  return k;
}

__device__ __forceinline__ int py_from_pitch(float pitch, float fd_abs, float fov, int H) {
  float t = fdiv(fadd(pitch, fd_abs), fov);
  float y = fmul(fsub(1.0f, t), (float)H);  // (float)(1.0 - (double)t) == 1.0f - t
  y = floorf(y);
  y = (y < H - 1.0f) ? y : (H - 1.0f);       // std::min(H - 1.0f, y)
  y = (0.0f < y) ? y : 0.0f;                 // std::max(0.0f, y)
  return (int)y;
}

__global__ void __launch_bounds__(256) k_project(Dev d, KParams kp) {
  const int N = d.N, W = kp.img_w, H = kp.img_h;
  int slow = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const float4 p = __ldcs(d.in->xyzi + i);
    const float x = p.x, y = p.y, z = p.z;
    const float range = fsqrt(fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z)));
    // ---- column
    int px;
    {
      float yaw = -atan2f(y, x);
      bool need = !(isfinite(x) && isfinite(y)) || x == 0.0f || y == 0.0f;
      if (!need) {
        float m = fmaxf(fabsf(yaw) * 1.2e-6f, 1e-30f);
        px = px_from_yaw(d.px_tab, yaw - m, W);
        need = px != px_from_yaw(d.px_tab, yaw + m, W);
      }
      if (need) {
        yaw = -(float)atan2((double)y, (double)x);
        px = px_from_yaw(d.px_tab, yaw, W);
        ++slow;
      }
    }
    // ---- row
    int py;
    {
      const float q = fdiv(z, range);
      float pitch = asinf(q);
      bool need = !(fabsf(q) < 1.0f);
      if (!need) {
        float m = fmaxf(fabsf(pitch) * 1.2e-6f, 1e-30f);
        py = py_from_pitch(pitch - m, kp.fov_down_abs, kp.fov, H);
        need = py != py_from_pitch(pitch + m, kp.fov_down_abs, kp.fov, H);
      }
      if (need) {
        pitch = (float)asin((double)q);
        py = py_from_pitch(pitch, kp.fov_down_abs, kp.fov, H);
        ++slow;
      }
    }
    const int pix = py * W + px;
    d.pix[i] = pix;
    const unsigned long long key = ((unsigned long long)range_key(range) << 32) | (uint32_t)i;
    atomicMin(d.pkey + pix, key);
  }
  slow = warp_sumi(slow);
  if ((threadIdx.x & 31) == 0 && slow) atomicAdd(&d.cnt->n_slow_px, slow);
}

// Per pixel: range image and mask from the winner; re-arms the winner key.
__global__ void __launch_bounds__(256) k_resolve(Dev d, int point_labels) {
  const int N = d.N;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const unsigned long long key = d.pkey[p];
    d.pkey[p] = ~0ull;
    float r = 0.0f;
    uint8_t m = 0;
    if (key != ~0ull) {
      r = __uint_as_float((uint32_t)(key >> 32));
      if (point_labels) m = d.in->plabel[(uint32_t)key];
    }
    if (!point_labels) m = d.in->mask_in[p];
    d.range_img[p] = r;
    d.mask[p] = m;
  }
}

// maskCloud: organised tree cloud (with the Ouster destagger as a gather:
// even rows take x,y,z from column c-32 for c >= 32 and keep their own
// intensity; inference.cpp:200-228) and the ground membership bits.
__global__ void __launch_bounds__(1024) k_mask(Dev d, KParams kp) {
  __shared__ int sm[33];
  const int N = d.N, W = kp.img_w;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  bool ground = false;
  if (o < N) {
    const uint8_t mo = d.mask[d.pix[o]];
    ground = (mo == 1);
    const float nan = __int_as_float(0x7fc00000);
    const float4* X = d.in->xyzi;
    float4 src = X[o];
    float4 t = (mo == 255) ? src : make_float4(nan, nan, nan, 0.0f);
    const int row = o / W, c = o - row * W;
    if (kp.do_destagger && (row & 1) == 0 && c >= 32) {
      const int s = o - 32;
      const uint8_t ms = d.mask[d.pix[s]];
      float4 q = X[s];
      t.x = (ms == 255) ? q.x : nan;
      t.y = (ms == 255) ? q.y : nan;
      t.z = (ms == 255) ? q.z : nan;
    }
    d.tree[o] = t;
  }
  const unsigned b = __ballot_sync(0xffffffffu, ground);
  if ((threadIdx.x & 31) == 0 && o < N + 31) d.gbits[o >> 5] = b;
  int total;
  block_excl_scan(ground ? 1 : 0, sm, &total);
  if (threadIdx.x == 0) d.blk[blockIdx.x] = total;
}

// Ordered compaction of the ground points (point order).
__global__ void __launch_bounds__(1024) k_ground_compact(Dev d) {
  __shared__ int sm[33];
  const int N = d.N;
  const int base = block_sum_prefix(d.blk, blockIdx.x, sm);
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned b = (o < N + 31) ? d.gbits[o >> 5] : 0u;
  const bool g = o < N && ((b >> (threadIdx.x & 31)) & 1u);
  int total;
  const int ex = block_excl_scan(g ? 1 : 0, sm, &total);
  const int pos = base + ex;
  if (g) {
    d.ground_idx[pos] = o;
    if (pos < d.cap_ground) d.ground[pos] = d.in->xyzi[o];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    const int n = base + total;
    d.cnt->n_ground = n < d.cap_ground ? n : d.cap_ground;
    if (n > d.cap_ground) atomicOr(&d.cnt->overflow, 1);
  }
}

__global__ void k_begin(Dev d, int n_ground, int n_lm, int n_v, int n_p, int n_cluster) {
  Counters* c = d.cnt;
  const int n_prev = c->n_prev;
  int32_t* w = reinterpret_cast<int32_t*>(c);
  for (int i = threadIdx.x; i < (int)(sizeof(Counters) / 4); i += blockDim.x) w[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    c->n_prev = n_prev;
    if (n_ground >= 0) c->n_ground = n_ground;
    if (n_lm >= 0) c->n_lm = n_lm;
    if (n_v >= 0) c->n_v = n_v;
    if (n_p >= 0) c->n_p = n_p;
    if (n_cluster >= 0) c->n_cluster = n_cluster;
  }
}

}  // namespace

int launch_begin(const Dev& d, int n_ground, int n_lm, int n_v, int n_p, int n_cluster,
                 cudaStream_t st) {
  k_begin<<<1, 64, 0, st>>>(d, n_ground, n_lm, n_v, n_p, n_cluster);
  return 1;
}

int launch_project_kernel(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_project<<<(d.N + 255) / 256, 256, 0, st>>>(d, kp);
  return 1;
}
int launch_resolve_kernel(const Dev& d, bool point_labels, cudaStream_t st) {
  k_resolve<<<(d.N + 255) / 256, 256, 0, st>>>(d, point_labels ? 1 : 0);
  return 1;
}

int launch_project(const Dev& d, const KParams& kp, bool point_labels, cudaStream_t st) {
  const int N = d.N;
  const int g256 = (N + 255) / 256;
  k_project<<<g256, 256, 0, st>>>(d, kp);
  k_resolve<<<g256, 256, 0, st>>>(d, point_labels ? 1 : 0);
  const int g1k = (N + 1023) / 1024;
  k_mask<<<g1k, 1024, 0, st>>>(d, kp);
  k_ground_compact<<<g1k, 1024, 0, st>>>(d);
  return 4;
}

}  // namespace sg
