// project.cu — a1/a2: spherical range-image projection of the labelled scan
// (Segmentation::_doProjection, inference.cpp:80-165) and mask -> ground list
// + organised tree cloud (Segmentation::maskCloud / _destaggerCloud,
// inference.cpp:200-273).
//
// Arithmetic contract: range, z/range and the pixel row are IEEE float with
// round-to-nearest, unfused, in the reference's order; yaw and pitch are the
// correctly rounded float atan2/asin.  Yaw enters the column through a double
// expression, so the column is read from an exact boundary table built on the
// host (px_tab[k] = smallest float yaw whose column is >= k).  The first try
// evaluates yaw with the FP32 polynomial of fastpoly.cuh (at most 4.9e-7
// relative from the correctly rounded angle), reads the table entry the
// column formula estimates, and accepts it when the whole +-1.2e-6 relative
// margin (about 10 ulp) lies inside that entry; otherwise the column takes
// the FP64 path.  The row is monotone in q = z / range (asin and the row
// formula both are), so its boundary table is on q itself (py_tab[k] =
// smallest float q whose row is <= H-1-k): q is exact, and the row is exact
// comparisons, with no angle evaluated.
// The nearest point wins its pixel: 64-bit minimum reduction on
// range bits (32) : point index (24) : point label (8), ties to the lowest
// index; the label rides in the key so the winner's label needs no gather.
//
// Two forms: one keyframe on the context's own buffers (inputs read through
// the context's input block, so a captured graph can be replayed on new
// inputs): k_project, k_label, k_ground_compact; or a chunk of batch
// keyframes, blockIdx.y selecting the keyframe's FrontRef: k_project,
// k_label_batch, k_compact_batch (warp by warp, no block barrier).
#include <algorithm>

#include "internal.h"
#include "scan_util.cuh"
#include "fastpoly.cuh"

namespace sg {

namespace {

// Index k in [0, n-1] with tab[k] <= v < tab[k+1] (tab[0] = -inf, tab[n] =
// +inf, non-decreasing), searched from the estimate e.
__device__ __forceinline__ int table_index(const float* __restrict__ tab, float v, float e,
                                           int n) {
  int k = (int)floorf(fminf(fmaxf(e, -1.0f), (float)n));
  k = max(0, min(n - 1, k));
  while (k < n - 1 && v >= __ldg(tab + k + 1)) ++k;
  while (k > 0 && v < __ldg(tab + k)) --k;
  return k;
}
// Entry k = the estimate e truncated into [0, n-1] when the whole interval
// [v - m, v + m] lies in it (tab[k] <= v - m and v + m < tab[k+1]), else
// -1: two loads and no search.
__device__ __forceinline__ int table_guess(const float* __restrict__ tab, float v, float m,
                                           float e, int n) {
  const int k = min(n - 1, max(0, __float2int_rz(e)));
  return (__ldg(tab + k) <= v - m && v + m < __ldg(tab + k + 1)) ? k : -1;
}
// Column of a yaw: px_tab[k] = smallest yaw of column k (inference.cpp:111-121;
// NaN: std::min/max keep the bound, W - 1).
__device__ __forceinline__ float col_estimate(float yaw, int W) {
  return (yaw * 0.318309886f + 1.0f) * 0.5f * (float)W;
}
// Row of q = z / range: py_tab[k] = smallest q of row H-1-k
// (inference.cpp:108-126 through the correctly rounded asinf); the estimate
// takes asin(q) ~ q (1 + q^2 / 6 + 3 q^4 / 40), and the exact table decides.
__device__ __forceinline__ float row_estimate_q(float q, const KParams& kp) {
  const float q2 = q * q;
  const float pitch = q * (1.0f + q2 * (0.16666667f + q2 * 0.075f));
  return (pitch + kp.fov_down_abs) * (1.0f / kp.fov) * (float)kp.img_h;
}

// 64-bit minimum without a returned value (a reduction, not an atomic with
// a result): nothing waits for it, so a thread's next point does not wait
// for the previous point's round trip to L2.
__device__ __forceinline__ void red_min_u64(unsigned long long* a, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.min.u64 [%0], %1;" ::"l"(a), "l"(v) : "memory");
}

// The buffers of the keyframe this block works on.
template <bool kBatch>
__device__ __forceinline__ FrontRef front(const Dev& d, const FrontRef* refs, int kf0) {
  if (kBatch) return refs[kf0 + blockIdx.y];
  const InPtrs* in = d.in;
  FrontRef f;
  f.xyzi = in->xyzi;
  f.plabel = in->plabel;
  f.mask_in = in->mask_in;
  f.pix = d.pix;
  f.pkey = d.pkey;
  f.range_img = d.range_img;
  f.mask = d.mask;
  f.tree = d.tree;
  f.tflag = nullptr;
  f.gbits = d.gbits;
  f.blk = d.blk;
  f.ground_idx = d.ground_idx;
  f.ground = d.ground;
  f.fe = nullptr;
  return f;
}
// projection counters: the context's counters, or the keyframe's fe block
template <bool kBatch>
__device__ __forceinline__ int32_t* fe_slot(const Dev& d, const FrontRef& f, int which) {
  if (kBatch) return f.fe + which;
  return which == 0 ? &d.cnt->n_ground : which == 1 ? &d.cnt->overflow : &d.cnt->n_slow_px;
}

// In an organised scan the points of a warp fall on distinct pixels, so each
// point makes its own 64-bit minimum reduction (no returned value, so the
// thread's next point does not wait for it).  Pixel (H-1, W-1), where every
// no-return (NaN) point lands, is the exception: its keys are reduced over
// the warp (two full-warp min reductions), kept as a running minimum per
// warp, and sent by one atomic per block.  The minimum is the same, so the
// winner is unchanged.
template <bool kBatch>
__global__ void __launch_bounds__(256) k_project(Dev d, KParams kp, const FrontRef* refs,
                                                 int kf0, int point_labels) {
  __shared__ unsigned long long hot_w[8];
  const FrontRef f = front<kBatch>(d, refs, kf0);
  const int N = d.N, W = kp.img_w, H = kp.img_h;
  const int hot = N - 1;  // the pixel of NaN points: row H - 1, column W - 1
  const int lane = threadIdx.x & 31;
  unsigned long long hot_acc = ~0ull;  // this warp's least key at `hot`
  int slow = 0;
  // a grid of resident blocks: each thread walks its points at the grid's
  // stride, the next point's loads issued before this point's arithmetic
  const int stride = gridDim.x * blockDim.x;
  float4 p_next = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t lab_next = 0u;
  {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) {
      p_next = f.xyzi[i];
      lab_next = point_labels ? f.plabel[i] : 0u;
    }
  }
  for (int i0 = blockIdx.x * blockDim.x; i0 < N; i0 += stride) {
    const int i = i0 + threadIdx.x;
    const bool valid = i < N;
    int pix = -1;
    unsigned long long key = ~0ull;
    const float4 p = p_next;
    const uint32_t lab = lab_next;
    if (i + stride < N) {
      p_next = f.xyzi[i + stride];  // kept in L2 for the label pass
      lab_next = point_labels ? f.plabel[i + stride] : 0u;
    }
    if (valid) {
      const float x = p.x, y = p.y, z = p.z;
      const float range = fsqrt(fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z)));
      // ---- first try: own polynomial angles, the table entry the formula
      // estimates, accepted when the margin interval lies inside it
      const bool nan_xy = isnan(x) || isnan(y);
      const float mx = fmaxf(fabsf(x), fabsf(y)), mn = fminf(fabsf(x), fabsf(y));
      const float yaw0 = -atan2_poly(y, x);
      int px = (mn >= 1e-18f && mx <= 1e18f)
                   ? table_guess(d.px_tab, yaw0, fmaxf(fabsf(yaw0) * 1.2e-6f, 1e-30f),
                                 col_estimate(yaw0, W), W)
                   : -1;
      px = nan_xy ? W - 1 : px;  // NaN in, NaN out: column W - 1
      // ---- the row: exact comparisons of q with its boundary table (a NaN
      // q, or |q| > 1 after rounding, has a NaN pitch: row H - 1)
      const float q = fdiv(z, range);
      const int g = fabsf(q) <= 1.0f ? table_index(d.py_tab, q, row_estimate_q(q, kp), H) : 0;
      // ---- exact column: correctly rounded yaw from FP64
      if (px < 0) {
        const float yaw = -(float)atan2((double)y, (double)x);
        px = table_index(d.px_tab, yaw, col_estimate(yaw, W), W);
        ++slow;
      }
      const int py = H - 1 - g;
      pix = py * W + px;
      f.pix[i] = pix;
      key = ((unsigned long long)range_key(range) << 32) | ((uint32_t)i << 8) | lab;
    }
    const bool at_hot = valid && pix == hot;
    if (valid && !at_hot) red_min_u64(f.pkey + pix, key);
    if (__any_sync(0xffffffffu, at_hot)) {
      const uint32_t hi = at_hot ? (uint32_t)(key >> 32) : 0xffffffffu;
      const uint32_t hmin = __reduce_min_sync(0xffffffffu, hi);
      const uint32_t lmin =
          __reduce_min_sync(0xffffffffu, (at_hot && hi == hmin) ? (uint32_t)key : 0xffffffffu);
      const unsigned long long kmin = ((unsigned long long)hmin << 32) | lmin;
      hot_acc = kmin < hot_acc ? kmin : hot_acc;
    }
  }
  if (lane == 0) hot_w[threadIdx.x >> 5] = hot_acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = hot_w[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = hot_w[w] < m ? hot_w[w] : m;
    if (m != ~0ull) red_min_u64(f.pkey + hot, m);
  }
  slow = warp_sumi(slow);
  if (lane == 0 && slow) atomicAdd(fe_slot<kBatch>(d, f, 2), slow);
}

// Label of pixel `pix`'s winner: the point label carried in the key of the
// nearest point (the pixel holds at least the caller's point), or the given
// mask image.
__device__ __forceinline__ uint8_t pixel_label(const FrontRef& f, int pix, int point_labels) {
  if (!point_labels) return f.mask_in[pix];
  return (uint8_t)f.pkey[pix];
}

// The label stage works in blocks of 1024 pixels / points (the ground
// bits, 32 per word, and the per-block ground counts); 256 threads take 4
// each, at a stride of 256, all loads issued before use.
constexpr int kLabelThreads = 256, kLabelPer = 4, kLabelWarps = kLabelThreads / 32;
static_assert(kLabelThreads * kLabelPer == 1024, "label block");

// One keyframe on the context.  Index o is pixel o and point o.  Pixel:
// range image and mask from the winner.  Point: maskCloud -- the ground bit
// and the organised tree cloud, both from the label of the point's pixel,
// with the Ouster destagger as a gather: even rows take x,y,z from column
// c-32 for c >= 32 and keep their own intensity (inference.cpp:200-228).
__global__ void __launch_bounds__(kLabelThreads) k_label(Dev d, KParams kp, int point_labels) {
  __shared__ int sm[33];
  const FrontRef f = front<false>(d, nullptr, 0);
  const int N = d.N, W = kp.img_w;
  const int o0 = blockIdx.x * 1024 + threadIdx.x;
  const float nan = __int_as_float(0x7fc00000);
  unsigned long long key[kLabelPer];
  int pix[kLabelPer], spix[kLabelPer];
  float4 src[kLabelPer], sq[kLabelPer];
  bool stag[kLabelPer];
  uint8_t min_[kLabelPer];
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    key[j] = ~0ull;
    pix[j] = 0;
    stag[j] = false;
    if (o < N) {
      key[j] = f.pkey[o];
      pix[j] = f.pix[o];
      min_[j] = point_labels ? 0 : f.mask_in[o];
      src[j] = f.xyzi[o];
      const int row = o / W, c = o - row * W;
      stag[j] = kp.do_destagger && (row & 1) == 0 && c >= 32;
      if (stag[j]) {
        spix[j] = f.pix[o - 32];
        sq[j] = f.xyzi[o - 32];
      }
    }
  }
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    bool ground = false;
    if (o < N) {
      float r = 0.0f;
      uint8_t m = 0;
      if (key[j] != ~0ull) {
        r = __uint_as_float((uint32_t)(key[j] >> 32));
        if (point_labels) m = (uint8_t)key[j];
      }
      if (!point_labels) m = min_[j];
      f.range_img[o] = r;
      f.mask[o] = m;
      const uint8_t mo = pixel_label(f, pix[j], point_labels);
      ground = (mo == 1);
      float4 t = (mo == 255) ? src[j] : make_float4(nan, nan, nan, 0.0f);
      if (stag[j]) {
        const uint8_t ms = pixel_label(f, spix[j], point_labels);
        t.x = (ms == 255) ? sq[j].x : nan;
        t.y = (ms == 255) ? sq[j].y : nan;
        t.z = (ms == 255) ? sq[j].z : nan;
      }
      f.tree[o] = t;
    }
    const unsigned b = __ballot_sync(0xffffffffu, ground);
    if ((threadIdx.x & 31) == 0 && o < N + 31) f.gbits[o >> 5] = b;
    cnt += ground ? 1 : 0;
  }
  int total;
  block_excl_scan(cnt, sm, &total);
  if (threadIdx.x == 0) f.blk[blockIdx.x] = total;
}

// One keyframe on the context: ordered compaction of the ground points
// (point order: the 4 slices of a block in turn), their indices and points;
// re-arms the pixel keys for the next scan.
__global__ void __launch_bounds__(kLabelThreads) k_ground_compact(Dev d) {
  __shared__ int sm[33];
  const FrontRef f = front<false>(d, nullptr, 0);
  const int N = d.N;
  const int o0 = blockIdx.x * 1024 + threadIdx.x;
  bool g[kLabelPer];
  float4 v[kLabelPer];
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    const unsigned b = (o < N + 31) ? f.gbits[o >> 5] : 0u;
    g[j] = o < N && ((b >> (threadIdx.x & 31)) & 1u);
    v[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g[j]) v[j] = f.xyzi[o];  // issued before the prefix sums
    if (o < N) f.pkey[o] = ~0ull;
  }
  int run = block_sum_prefix(f.blk, blockIdx.x, sm);
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    int total;
    const int pos = run + block_excl_scan(g[j] ? 1 : 0, sm, &total);
    if (g[j]) {
      f.ground_idx[pos] = o;
      if (pos < d.cap_ground) f.ground[pos] = v[j];
    }
    run += total;
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    d.cnt->n_ground = run < d.cap_ground ? run : d.cap_ground;
    if (run > d.cap_ground) atomicOr(&d.cnt->overflow, 1);
  }
}

// Batch keyframes.  The label pass: block c covers points [1024 c,
// 1024 c + 1024), 4 per thread at a stride of 256; it writes the range image,
// mask and tree flag, the ground bits (one ballot word per 32 points) and
// the chunk's ground count (the warps' ballot counts added once), so the
// compaction's prefix needs no block scan.
__global__ void __launch_bounds__(kLabelThreads) k_label_batch(Dev d, const FrontRef* refs,
                                                               int kf0, int point_labels) {
  const FrontRef f = refs[kf0 + blockIdx.y];
  const int N = d.N;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int o0 = blockIdx.x * 1024 + threadIdx.x;
  unsigned long long key[kLabelPer];
  int pix[kLabelPer];
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    key[j] = o < N ? f.pkey[o] : ~0ull;
    pix[j] = o < N ? f.pix[o] : 0;
  }
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < kLabelPer; ++j) {
    const int o = o0 + j * kLabelThreads;
    bool ground = false;
    if (o < N) {
      float r = 0.0f;
      uint8_t m = point_labels ? 0 : f.mask_in[o];
      if (key[j] != ~0ull) {
        r = __uint_as_float((uint32_t)(key[j] >> 32));
        if (point_labels) m = (uint8_t)key[j];
      }
      f.range_img[o] = r;
      f.mask[o] = m;
      // a point that won its own pixel (the common case in an organised
      // scan) has the pixel's label in the key already loaded
      const uint8_t mo = (point_labels && pix[j] == o) ? (uint8_t)key[j]
                                                       : pixel_label(f, pix[j], point_labels);
      f.tflag[o] = mo == 255 ? 1 : 0;
      ground = (mo == 1);
    }
    const unsigned b = __ballot_sync(0xffffffffu, ground);
    if (lane == 0 && o < N + 31) f.gbits[o >> 5] = b;
    cnt += __popc(b);
  }
  __shared__ int wc[kLabelWarps];
  if (lane == 0) wc[w] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
#pragma unroll
    for (int q = 0; q < kLabelWarps; ++q) t += wc[q];
    f.blk[blockIdx.x] = t;
  }
}

// Batch keyframes: the ordered ground compaction, one warp per 1024-point
// chunk.  Its first position is the sum of the counts of the chunks before
// it; inside the chunk, a warp scan of the 32 ground words' bit
// counts places each word's points, written word by word (coalesced); the
// warp then re-arms the chunk's pixel keys, and the last chunk's warp
// writes the keyframe's ground count.
__global__ void __launch_bounds__(kLabelThreads) k_compact_batch(Dev d, const FrontRef* refs,
                                                                 int kf0) {
  const FrontRef f = refs[kf0 + blockIdx.y];
  const int N = d.N, nch = (N + 1023) >> 10;
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * kLabelWarps + (threadIdx.x >> 5);
  if (c >= nch) return;  // the whole warp
  const int wi = c * 32 + lane;  // this lane's ground word: points 32 wi .. 32 wi + 31
  const unsigned word = (wi << 5) < N ? f.gbits[wi] : 0u;
  // the counts of the chunks before this one, eight independent loads per
  // lane at a time
  int s = 0;
  const int lim = c;
  for (int base = 0; base < lim; base += 256) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int k = base + r * 32 + lane;
      s += k < lim ? f.blk[k] : 0;
    }
  }
  const int run = warp_sumi(s);
  const int pc = __popc(word);
  int incl = pc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  // word by word in point order, so each word's ground points go out as
  // one coalesced store: lane l writes point 32 i + l of word i
  const int excl = run + incl - pc;
  for (int i = 0; i < 32; ++i) {
    const unsigned wd = __shfl_sync(0xffffffffu, word, i);
    const int e = __shfl_sync(0xffffffffu, excl, i);
    if ((wd >> lane) & 1u)
      f.ground_idx[e + __popc(wd & ((1u << lane) - 1u))] = ((c * 32 + i) << 5) + lane;
  }
  // re-arm the chunk's keys for the next scan in this slot
  const int p0 = c << 10, p1 = min(p0 + 1024, N);
  if (p1 - p0 == 1024 && ((reinterpret_cast<uintptr_t>(f.pkey + p0) & 15) == 0)) {
    ulonglong2* k2 = reinterpret_cast<ulonglong2*>(f.pkey + p0);
    const ulonglong2 ones = make_ulonglong2(~0ull, ~0ull);
#pragma unroll 4
    for (int q = lane; q < 512; q += 32) k2[q] = ones;
  } else {
    for (int q = p0 + lane; q < p1; q += 32) f.pkey[q] = ~0ull;
  }
  if (c == nch - 1) {
    const int total = __shfl_sync(0xffffffffu, run + incl, 31);
    if (lane == 0) {
      f.fe[0] = total < d.cap_ground ? total : d.cap_ground;
      if (total > d.cap_ground) atomicOr(f.fe + 1, 1);
    }
  }
}

// The organised tree cloud of a batch keyframe, written out from its view
// (the per-point tree flags and the scan), for the caller.
__global__ void k_tree_out(TreeView v, float4* out, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = v[i];
}

// Per-keyframe counter reset.  A keyframe whose projection ran in a batch
// launch takes the counts of that launch from its fe block.
__global__ void k_begin(Dev d, int n_ground, int n_lm, int n_v, int n_p, int n_cluster) {
  Counters* c = d.cnt;
  const int n_prev = c->n_prev;
  int32_t* w = reinterpret_cast<int32_t*>(c);
  for (int i = threadIdx.x; i < (int)(sizeof(Counters) / 4); i += blockDim.x) w[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    c->n_prev = n_prev;
    const int32_t* fe = d.in->fe;
    if (fe) {
      c->n_ground = fe[0];
      c->overflow = fe[1];
      c->n_slow_px = fe[2];
    }
    if (n_ground >= 0) c->n_ground = n_ground;
    if (n_lm >= 0) c->n_lm = n_lm;
    if (n_v >= 0) c->n_v = n_v;
    if (n_p >= 0) c->n_p = n_p;
    if (n_cluster >= 0) c->n_cluster = n_cluster;
  }
}

}  // namespace

// Blocks per keyframe of a batch projection launch: the resident blocks of
// the whole GPU shared among the launch's keyframes, rounded down so that the
// whole grid is resident in one wave (a block left for a second wave would
// walk its points after all the others), at most one point per thread.
constexpr int kProjBlocksPerSm = 6;
static int project_blocks_per_kf(int N, int nkf) {
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project<true>, 256, 0);
    // at most kProjBlocksPerSm per SM, the rest of each SM left to the
    // previous chunk's label kernels, which run alongside
    resident = std::max(1, sms) * std::max(1, std::min(per_sm, kProjBlocksPerSm));
  }
  const int full = (N + 255) / 256;
  const int share = resident / std::max(1, nkf);
  return std::max(1, std::min(full, share));
}

size_t front_gbits_words(int N) { return (size_t)((N + 1023) / 1024) * 32 + 32; }
int front_blocks(int N) { return (N + 1023) / 1024; }

int launch_tree_out(const FrontRef& f, const KParams& kp, int N, float4* out, cudaStream_t st) {
  const TreeView v{nullptr, f.xyzi, f.tflag, kp.img_w, kp.do_destagger ? 1 : 0};
  k_tree_out<<<(N + 255) / 256, 256, 0, st>>>(v, out, N);
  return 1;
}

int launch_begin(const Dev& d, int n_ground, int n_lm, int n_v, int n_p, int n_cluster,
                 cudaStream_t st) {
  k_begin<<<1, 64, 0, st>>>(d, n_ground, n_lm, n_v, n_p, n_cluster);
  return 1;
}

int launch_project_kernel(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_project<false><<<(d.N + 255) / 256, 256, 0, st>>>(d, kp, nullptr, 0, 1);
  return 1;
}
int launch_project_rest(const Dev& d, const KParams& kp, bool point_labels, cudaStream_t st) {
  const int g1k = front_blocks(d.N);
  k_label<<<g1k, kLabelThreads, 0, st>>>(d, kp, point_labels ? 1 : 0);
  k_ground_compact<<<g1k, kLabelThreads, 0, st>>>(d);
  return 2;
}

int launch_project(const Dev& d, const KParams& kp, bool point_labels, cudaStream_t st) {
  k_project<false><<<(d.N + 255) / 256, 256, 0, st>>>(d, kp, nullptr, 0, point_labels ? 1 : 0);
  return 1 + launch_project_rest(d, kp, point_labels, st);
}

int launch_project_batch_points(const Dev& d, const KParams& kp, const FrontRef* refs,
                                int kf0, int nkf, bool point_labels, cudaStream_t st) {
  if (nkf <= 0) return 0;
  const dim3 g256(project_blocks_per_kf(d.N, nkf), nkf);
  k_project<true><<<g256, 256, 0, st>>>(d, kp, refs, kf0, point_labels ? 1 : 0);
  return 1;
}
int launch_project_batch_labels(const Dev& d, const FrontRef* refs, int kf0, int nkf,
                                bool point_labels, cudaStream_t st) {
  if (nkf <= 0) return 0;
  const dim3 g1k(front_blocks(d.N), nkf);
  k_label_batch<<<g1k, kLabelThreads, 0, st>>>(d, refs, kf0, point_labels ? 1 : 0);
  const dim3 gw((front_blocks(d.N) + kLabelWarps - 1) / kLabelWarps, nkf);
  k_compact_batch<<<gw, kLabelThreads, 0, st>>>(d, refs, kf0);
  return 2;
}

}  // namespace sg
