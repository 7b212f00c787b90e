// trellis.cu — a3-a5: Instance::computeGraph (trellis.cpp:134-139).
//
// a3 organised connected components (PCL OrganizedConnectedComponentSegmentation
//    + EuclideanClusterComparator(1.0), trellis.cpp:15-43): a pixel is valid
//    iff x is finite; 4-neighbours join when |p - q| < thr (float,
//    sqrt(dx^2 + (dy^2 + dz^2))).  Lock-free union-find whose roots are the
//    minimum pixel index of each component, so ranking the roots in raster
//    order reproduces PCL's label numbering.
// a4 Instance::findTrees (trellis.cpp:104-132): the pixels of every component
//    with > min_cluster points are bucketed per (component, row) in column
//    order in one pass over each component's column span (instead of a scan
//    of the whole image per component).
// a5 computeTreeVertex / computeVertexProperties (trellis.cpp:45-102): one
//    warp per (component, row) bucket; medians and the (z, y, x, column)
//    order by rank counting in shared memory.
#include <climits>

#include "internal.h"
#include "scan_util.cuh"

namespace sg {

namespace {

__device__ __forceinline__ bool cc_close(const float4& a, const float4& b, float thr) {
  const float dx = fsub(a.x, b.x), dy = fsub(a.y, b.y), dz = fsub(a.z, b.z);
  const float dd = fadd(fmul(dx, dx), fadd(fmul(dy, dy), fmul(dz, dz)));
  return fsqrt(dd) < thr;
}

__device__ __forceinline__ uint32_t cc_find(volatile uint32_t* P, uint32_t x) {
  uint32_t p = P[x];
  while (p != x) {
    const uint32_t gp = P[p];
    if (gp != p) P[x] = gp;  // path halving: parents only ever decrease
    x = p;
    p = P[x];
  }
  return x;
}

// Union of the components of u and v in parent array P (roots are the
// minimum index: the larger root is linked under the smaller by CAS).
// Returns false when the retry limit (`limit` rounds) ran out.
template <typename T, typename Find>
__device__ __forceinline__ bool cc_union(T* P, T u, T v, Find find, int limit) {
  for (int it = 0; it < limit; ++it) {
    T ru = find(u), rv = find(v);
    if (ru == rv) return true;
    if (ru > rv) { const T t = ru; ru = rv; rv = t; }
    const T old = atomicCAS(P + rv, rv, ru);
    if (old == rv) return true;
    u = ru;
    v = old;
  }
  return false;
}

// a3, first level: one block per 32 x 32 pixel tile, one warp per tile row
// (lane = column).  Horizontal runs come from one ballot: every valid pixel
// points at the first pixel of its run.  Vertical neighbours then join the
// run roots in a shared-memory union-find, once per stretch of overlapping
// runs (where the pixel, or its upper neighbour, starts a run, or the left
// pair was not joined vertically).  Roots are minimum pixel indices (local
// indices are row-major like global ones); each pixel writes the global index
// of its tile root to the global parent array.
constexpr int kCCTile = 32;

__global__ void __launch_bounds__(256) k_cc_local(Dev d, float thr, int limit) {
  __shared__ int lp[kCCTile * kCCTile];
  __shared__ float4 pt[kCCTile * kCCTile];
  __shared__ unsigned vbits[kCCTile], hbits[kCCTile];
  const TreeView tree = tree_view(d.in, d.W);
  const int W = d.W, H = d.H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int tiles_x = (W + kCCTile - 1) / kCCTile;
  const int r0 = (blockIdx.x / tiles_x) * kCCTile, c0 = (blockIdx.x % tiles_x) * kCCTile;
  for (int row = warp; row < kCCTile; row += nwarp) {
    const int r = r0 + row, c = c0 + lane;
    float4 a = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
    if (r < H && c < W) a = tree[r * W + c];
    pt[row * kCCTile + lane] = a;
    const bool v = isfinite(a.x);
    const unsigned vb = __ballot_sync(0xffffffffu, v);
    // left neighbour: the previous lane's point
    const float lx = __shfl_up_sync(0xffffffffu, a.x, 1), ly = __shfl_up_sync(0xffffffffu, a.y, 1),
                lz = __shfl_up_sync(0xffffffffu, a.z, 1);
    const bool h = v && lane > 0 && ((vb >> (lane - 1)) & 1u) &&
                   cc_close(a, make_float4(lx, ly, lz, 0.f), thr);
    const unsigned hb = __ballot_sync(0xffffffffu, h);
    const unsigned starts = vb & ~hb;
    const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
    lp[row * kCCTile + lane] = v ? row * kCCTile + (31 - __clz(starts & upto)) : -1;
    if (lane == 0) {
      vbits[row] = vb;
      hbits[row] = hb;
    }
  }
  __syncthreads();
  volatile int* P = lp;
  auto find = [P](int x) {
    int p = P[x];
    while (p != x) {
      const int gp = P[p];
      if (gp != p) P[x] = gp;  // path halving: parents only ever decrease
      x = p;
      p = P[x];
    }
    return x;
  };
  bool ok = true;
  for (int row = 1 + warp; row < kCCTile; row += nwarp) {
    const int l = row * kCCTile + lane;
    const unsigned vb = vbits[row], vbu = vbits[row - 1];
    bool up = ((vb & vbu) >> lane) & 1u;
    if (up) up = cc_close(pt[l], pt[l - kCCTile], thr);
    const unsigned ub = __ballot_sync(0xffffffffu, up);
    const bool joined_left = lane > 0 && ((hbits[row] >> lane) & 1u) &&
                             ((hbits[row - 1] >> lane) & 1u) && ((ub >> (lane - 1)) & 1u);
    if (up && !joined_left) ok &= cc_union(lp, l, l - kCCTile, find, limit);
  }
  if (!ok) atomicOr(&d.cnt->cc_iter_exceeded, 1);
  __syncthreads();
  for (int l = threadIdx.x; l < kCCTile * kCCTile; l += blockDim.x) {
    const int r = r0 + l / kCCTile, c = c0 + l % kCCTile;
    if (r >= H || c >= W) continue;
    uint32_t g = kInvalid;
    if (P[l] >= 0) {
      const int root = find(l);
      g = (uint32_t)((r0 + root / kCCTile) * W + c0 + root % kCCTile);
    }
    d.parent[r * W + c] = g;
  }
}

// a3, second level: pixel pairs across tile borders (left neighbour across a
// vertical border, upper neighbour across a horizontal one) join in the
// global parent array.
__global__ void __launch_bounds__(256) k_cc_border(Dev d, float thr, int limit) {
  const TreeView tree = tree_view(d.in, d.W);
  const int W = d.W, H = d.H;
  const int nv = ((W + kCCTile - 1) / kCCTile - 1) * H;
  const int nh = ((H + kCCTile - 1) / kCCTile - 1) * W;
  uint32_t* P = d.parent;
  auto find = [P](uint32_t x) { return cc_find(P, x); };
  bool ok = true;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nv + nh; t += gridDim.x * blockDim.x) {
    int p, q;
    if (t < nv) {
      const int k = t / H + 1, r = t - (k - 1) * H;
      p = r * W + k * kCCTile;
      q = p - 1;
    } else {
      const int u = t - nv, k = u / W + 1, c = u - (k - 1) * W;
      p = k * kCCTile * W + c;
      q = p - W;
    }
    if (P[p] == kInvalid || P[q] == kInvalid) continue;
    if (!cc_close(tree[p], tree[q], thr)) continue;
    ok &= cc_union(P, (uint32_t)p, (uint32_t)q, find, limit);
  }
  if (!ok) atomicOr(&d.cnt->cc_iter_exceeded, 1);
}

int cc_border_pairs(int W, int H) {
  return ((W + kCCTile - 1) / kCCTile - 1) * H + ((H + kCCTile - 1) / kCCTile - 1) * W;
}

// The whole-image passes below take blocks of 1024 pixels with 256 threads,
// 4 slices of 256 pixels in turn (so raster order within a block is slice
// order, then thread order).
constexpr int kCCThreads = 256, kCCSlices = 4;
static_assert(kCCThreads * kCCSlices == 1024, "CC block");

// Roots -> per-block counts; every valid pixel stores its root in label[].
__global__ void __launch_bounds__(kCCThreads) k_cc_flatten(Dev d) {
  __shared__ int sm[33];
  int roots = 0;
#pragma unroll
  for (int j = 0; j < kCCSlices; ++j) {
    const int p = blockIdx.x * 1024 + j * kCCThreads + threadIdx.x;
    if (p < d.N) {
      const uint32_t par = d.parent[p];
      if (par != kInvalid) {
        const uint32_t r = cc_find(d.parent, (uint32_t)p);
        d.label[p] = r;
        roots += r == (uint32_t)p ? 1 : 0;
      } else {
        d.label[p] = kInvalid;
      }
    }
  }
  int total;
  block_excl_scan(roots, sm, &total);
  if (threadIdx.x == 0) d.blk[blockIdx.x] = total;
}

// Rank of each root in raster order = the component label.
__global__ void __launch_bounds__(kCCThreads) k_cc_rank(Dev d) {
  __shared__ int sm[33];
  int base = block_sum_prefix(d.blk, blockIdx.x, sm);
#pragma unroll
  for (int j = 0; j < kCCSlices; ++j) {
    const int p = blockIdx.x * 1024 + j * kCCThreads + threadIdx.x;
    const bool root = p < d.N && d.label[p] == (uint32_t)p;
    int total;
    const int ex = block_excl_scan(root ? 1 : 0, sm, &total);
    if (root) {
      const int r = base + ex;
      d.rank[p] = (uint32_t)r;
      d.comp_size[r] = 0;
      d.comp_cmin[r] = INT_MAX;
      d.comp_cmax[r] = -1;
    }
    base += total;
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) d.cnt->n_comp = base;
}

// Final labels + component size and column span (warp-aggregated atomics).
__global__ void __launch_bounds__(kCCThreads) k_cc_label(Dev d) {
  const int W = d.W;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kCCSlices; ++j) {
    const int p = blockIdx.x * 1024 + j * kCCThreads + threadIdx.x;
    uint32_t l = kInvalid;
    if (p < d.N) {
      const uint32_t r = d.label[p];
      if (r != kInvalid) {
        l = d.rank[r];
        d.label[p] = l;
      }
    }
    const bool valid = l != kInvalid;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(act, l);
      const int leader = __ffs(peers) - 1;
      if (lane == leader) {
        const int last = 31 - __clz(peers);
        const int p0 = p, p1 = p + (last - lane);
        int c0 = p0 % W, c1 = p1 % W;
        // a warp may straddle two rows (W % 32 != 0): fall back to per-lane span
        if (p0 / W != p1 / W) { c0 = 0; c1 = W - 1; }
        atomicAdd(d.comp_size + l, __popc(peers));
        atomicMin(d.comp_cmin + l, c0);
        atomicMax(d.comp_cmax + l, c1);
      }
    }
  }
}

// Ordered selection of the candidate components (size > min_cluster).
__global__ void __launch_bounds__(1024) k_cands(Dev d, int min_cluster) {
  __shared__ int sm[33];
  const int nc = d.cnt->n_comp;
  int base = 0;
  for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const bool cand = c < nc && d.comp_size[c] > min_cluster;
    int total;
    const int ex = block_excl_scan(cand ? 1 : 0, sm, &total);
    if (c < nc) {
      const int k = base + ex;
      if (cand && k < d.cap_cand) {
        d.cand_comp[k] = c;
        d.comp_cand[c] = k;
      } else {
        d.comp_cand[c] = -1;
      }
    }
    base += total;
  }
  if (threadIdx.x == 0) {
    d.cnt->n_cand = base < d.cap_cand ? base : d.cap_cand;
    if (base > d.cap_cand) atomicOr(&d.cnt->overflow, 2);
  }
}

// One warp per (candidate, row): count (pass 0) or scatter (pass 1) the
// component's pixels of that row in column order.
template <int PASS>
__global__ void __launch_bounds__(256) k_rows(Dev d) {
  const int H = d.H, W = d.W;
  const int lane = threadIdx.x & 31;
  const int nitems = d.cnt->n_cand * H;
  const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int it = wg; it < nitems; it += nw) {
    const int cand = it / H, row = it - cand * H;
    const int comp = d.cand_comp[cand];
    const int c0 = d.comp_cmin[comp], c1 = d.comp_cmax[comp];
    const uint32_t* lab = d.label + (size_t)row * W;
    int run = 0;
    int out = PASS ? d.roff[it] : 0;
    for (int c = c0; c <= c1; c += 32) {
      const int col = c + lane;
      const bool hit = col <= c1 && lab[col] == (uint32_t)comp;
      const unsigned b = __ballot_sync(0xffffffffu, hit);
      if (PASS && hit) d.bucket[out + run + __popc(b & ((1u << lane) - 1u))] = row * W + col;
      run += __popc(b);
    }
    if (!PASS && lane == 0) d.rc[it] = run;
  }
}

// Exclusive scan of the (candidate, row) counts; single block.
__global__ void __launch_bounds__(1024) k_rowscan(Dev d) {
  __shared__ int sm[33];
  const int n = d.cnt->n_cand * d.H;
  int base = 0;
  for (int i0 = 0; i0 < n; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    const int v = i < n ? d.rc[i] : 0;
    int total;
    const int ex = block_excl_scan(v, sm, &total);
    if (i < n) d.roff[i] = base + ex;
    base += total;
  }
  if (threadIdx.x == 0) {
    d.roff[n] = base;
    d.cnt->n_bucket = base;
  }
}

constexpr int kVtxCap = 256;   // points per vertex staged in shared memory
constexpr int kWideCap = 2048; // wider rows (up to this) run one block each in k_vertex_wide
constexpr int kVtxWarps = 4;

__device__ __forceinline__ bool zless(float4 a, int ia, float4 b, int ib) {
  if (a.z < b.z) return true;
  if (b.z < a.z) return false;
  if (a.y < b.y) return true;
  if (b.y < a.y) return false;
  if (a.x < b.x) return true;
  if (b.x < a.x) return false;
  return ia < ib;
}

// Order-preserving key of a float (x < y <=> key(x) < key(y); -0 and +0
// equal, as the float comparison has them).
__device__ __forceinline__ uint32_t fkey(float v) {
  if (v == 0.0f) v = 0.0f;
  const uint32_t u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Value of the element at position k of the stable order by value of the
// warp's n (<= 32 * kVtxSlots) keys, slot s of lane l holding element
// 32 s + l: warp quickselect (pivot = a pseudo-random remaining candidate,
// counts by ballot; each round removes the pivot's key, so at most n
// rounds), then the k'-th element, in index order, among those with the
// selected key -- the element the rank count (b < a, or b == a and k < j)
// puts at position k.
// kSlots = 4 for buckets of at most 128 points, 8 for at most 256 (the
// wider form costs registers and instructions on every call, so the common
// narrow buckets keep the narrow one).
constexpr int kVtxSortMax = 256;
template <int kVtxSlots>
__device__ __forceinline__ float warp_select(const float4* P, int axis, int n, int k, int lane) {
  const int ns = (n + 31) >> 5;
  uint32_t key[kVtxSlots];
  float val[kVtxSlots];
#pragma unroll
  for (int s = 0; s < kVtxSlots; ++s) {
    const int j = s * 32 + lane;
    float v = 0.0f;
    if (j < n) {
      const float4 a = P[j];
      v = axis == 0 ? a.x : axis == 1 ? a.y : a.z;
    }
    val[s] = v;
    key[s] = fkey(v);
  }
  unsigned cb[kVtxSlots];  // remaining candidates, one ballot word per slot
  int nc = n;
#pragma unroll
  for (int s = 0; s < kVtxSlots; ++s) {
    const int left = n - 32 * s;
    cb[s] = left >= 32 ? 0xffffffffu : left > 0 ? ((1u << left) - 1u) : 0u;
  }
  unsigned seed = 0x2545f491u;
  uint32_t K = 0;
  for (int round = 0; round <= n; ++round) {
    seed = seed * 1664525u + 1013904223u;
    int r = (int)(((unsigned long long)(seed >> 8) * (unsigned)nc) >> 24);
    uint32_t piv = 0;
#pragma unroll
    for (int s = 0; s < kVtxSlots; ++s) {
      if (s < ns) {
        const int c = __popc(cb[s]);
        if (r >= 0 && r < c) {  // warp-uniform
          unsigned e = cb[s];
          for (int q = 0; q < r; ++q) e &= e - 1;
          piv = __shfl_sync(0xffffffffu, key[s], __ffs(e) - 1);
        }
        r -= c;
      }
    }
    int cl = 0, ce = 0;
    unsigned lt[kVtxSlots], gt[kVtxSlots];
#pragma unroll
    for (int s = 0; s < kVtxSlots; ++s) {
      lt[s] = gt[s] = 0u;
      if (s < ns) {
        const bool in = (cb[s] >> lane) & 1u;
        lt[s] = __ballot_sync(0xffffffffu, in && key[s] < piv);
        const unsigned eq = __ballot_sync(0xffffffffu, in && key[s] == piv);
        gt[s] = cb[s] & ~lt[s] & ~eq;
        cl += __popc(lt[s]);
        ce += __popc(eq);
      }
    }
    if (k < cl) {
#pragma unroll
      for (int s = 0; s < kVtxSlots; ++s) cb[s] = lt[s];
      nc = cl;
    } else if (k < cl + ce) {
      K = piv;
      k -= cl;
      break;
    } else {
#pragma unroll
      for (int s = 0; s < kVtxSlots; ++s) cb[s] = gt[s];
      k -= cl + ce;
      nc -= cl + ce;
    }
  }
  float out = 0.0f;
#pragma unroll
  for (int s = 0; s < kVtxSlots; ++s) {
    if (s < ns) {
      const unsigned eq = __ballot_sync(0xffffffffu, s * 32 + lane < n && key[s] == K);
      const int c = __popc(eq);
      if (k >= 0 && k < c) {  // warp-uniform
        unsigned e = eq;
        for (int q = 0; q < k; ++q) e &= e - 1;  // drop the k lowest set bits
        out = __shfl_sync(0xffffffffu, val[s], __ffs(e) - 1);
      }
      k -= c;
    }
  }
  return out;
}

// Warp bitonic sort of m (power of two, <= kVtxCap) indices in shared memory
// by `less`; indices >= n are placed last.
template <typename Less>
__device__ __forceinline__ void warp_bitonic(int* a, int m, int n, int lane, Less less) {
  auto lt = [&](int x, int y) { return x < n && (y >= n || less(x, y)); };
  for (int k = 2; k <= m; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < (m >> 1); t += 32) {
        const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i | j;
        const int x = a[i], y = a[l];
        const bool up = (i & k) == 0;
        if (up ? lt(y, x) : lt(x, y)) {
          a[i] = y;
          a[l] = x;
        }
      }
      __syncwarp();
    }
  }
}

// One warp per (candidate, row) bucket with > min_beam points.
__global__ void __launch_bounds__(kVtxWarps * 32) k_vertex(Dev d, KParams kp) {
  __shared__ float4 spts[kVtxWarps][kVtxCap];
  __shared__ int srank[kVtxWarps][kVtxCap];
  const TreeView tree = tree_view(d.in, d.W);
  const int H = d.H;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nitems = d.cnt->n_cand * H;
  const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int it = wg; it < nitems; it += nw) {
    const int n = d.rc[it];
    const int off = d.roff[it];
    if (n <= kp.min_beam) {
      if (lane == 0) d.vkept[it] = 0;
      continue;
    }
    // stage: shared memory when it fits, else the global scratch `kept`
    // region is read directly (rank pass) - bucket points from the cloud
    if (n > kVtxCap && n <= kWideCap) {  // listed for k_vertex_wide
      if (lane == 0) {
        const int q = atomicAdd(&d.cnt->n_wide, 1);
        if (q < d.cap_cand * H) d.wide_list[q] = it;
      }
      continue;
    }
    const bool inshm = n <= kVtxCap;
    float4* P = spts[w];
    if (inshm)
      for (int j = lane; j < n; j += 32) P[j] = tree[d.bucket[off + j]];
    __syncwarp();
    auto pt = [&](int j) -> float4 { return inshm ? P[j] : tree[d.bucket[off + j]]; };
    const int mid = n / 2;  // (int)(n / 2.0)
    if (inshm && n > 32 && n <= kVtxSortMax) {
      // medians by quickselect; kept points in (z, y, x, column) order
      // by a bitonic sort -- the same elements and order as the rank counts
      // below, in O(n log^2 n) instead of O(n^2)
      float mx, my, mz;
      if (n <= 128) {
        mx = warp_select<4>(P, 0, n, mid, lane);
        my = warp_select<4>(P, 1, n, mid, lane);
        mz = warp_select<4>(P, 2, n, mid, lane);
      } else {
        mx = warp_select<8>(P, 0, n, mid, lane);
        my = warp_select<8>(P, 1, n, mid, lane);
        mz = warp_select<8>(P, 2, n, mid, lane);
      }
      int m = 32;
      while (m < n) m <<= 1;
      int* idx = srank[w];
      int nkept = 0;
      for (int j = lane; j < m; j += 32) {
        bool keep = false;
        if (j < n) {
          const float4 a = P[j];
          keep = pcl_euclid(a.x, a.y, a.z, mx, my, mz) < kp.max_d_centroid;
        }
        idx[j] = keep ? j : n;
        nkept += __popc(__ballot_sync(0xffffffffu, keep));  // m is a multiple of 32
      }
      __syncwarp();
      warp_bitonic(idx, m, n, lane, [&](int x, int y) { return zless(P[x], x, P[y], y); });
      for (int r = lane; r < nkept; r += 32) d.kept[off + r] = P[idx[r]];
      if (lane == 0) {
        const bool valid = nkept > 1;
        double rad = 0.0;
        if (valid) {
          const float4 a = P[idx[0]], b = P[idx[nkept - 1]];
          rad = (double)pcl_euclid(a.x, a.y, a.z, b.x, b.y, b.z);
        }
        d.vmed[it] = make_float4(mx, my, mz, 0.0f);
        d.vrad[it] = rad;
        d.vkept[it] = valid ? nkept : 0;
      }
      __syncwarp();
      continue;
    }
    // per-axis medians by rank
    float mx = __int_as_float(0x7fc00000), my = mx, mz = mx;
    for (int j = lane; j < n; j += 32) {
      const float4 a = pt(j);
      int rx = 0, ry = 0, rz = 0;
      for (int k = 0; k < n; ++k) {
        const float4 b = pt(k);
        rx += (b.x < a.x) || (b.x == a.x && k < j);
        ry += (b.y < a.y) || (b.y == a.y && k < j);
        rz += (b.z < a.z) || (b.z == a.z && k < j);
      }
      if (rx == mid) mx = a.x;
      if (ry == mid) my = a.y;
      if (rz == mid) mz = a.z;
    }
    // gather the medians (exactly one lane holds each)
    for (int o = 16; o > 0; o >>= 1) {
      float ox = __shfl_xor_sync(0xffffffffu, mx, o);
      float oy = __shfl_xor_sync(0xffffffffu, my, o);
      float oz = __shfl_xor_sync(0xffffffffu, mz, o);
      if (isnan(mx)) mx = ox;
      if (isnan(my)) my = oy;
      if (isnan(mz)) mz = oz;
    }
    // keep test and (z, y, x, column) rank
    int nkept = 0;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      bool keep = false;
      if (j < n) {
        const float4 a = pt(j);
        keep = pcl_euclid(a.x, a.y, a.z, mx, my, mz) < kp.max_d_centroid;
        if (inshm) {
          int r = 0;
          for (int k = 0; k < n; ++k) r += zless(P[k], k, a, j);
          srank[w][j] = keep ? r : -1;
        }
      }
      nkept += __popc(__ballot_sync(0xffffffffu, keep));
    }
    __syncwarp();
    const bool valid = nkept > 1;
    if (!inshm) {
      // a row wider than k_vertex_wide takes (images wider than kWideCap):
      // serial fallback by lane 0
      if (lane == 0) {
        int first = -1, last = -1, wr = 0;
        // emit kept points in (z,y,x,col) order by repeated minimum search
        int prev = -1;
        for (int c = 0; c < nkept; ++c) {
          int best = -1;
          for (int j = 0; j < n; ++j) {
            const float4 a = pt(j);
            if (!(pcl_euclid(a.x, a.y, a.z, mx, my, mz) < kp.max_d_centroid)) continue;
            if (prev >= 0 && !zless(pt(prev), prev, a, j)) continue;
            if (best < 0 || zless(a, j, pt(best), best)) best = j;
          }
          if (c == 0) first = best;
          last = best;
          d.kept[off + wr++] = pt(best);
          prev = best;
        }
        double rad = 0.0;
        if (valid) {
          const float4 a = pt(first), b = pt(last);
          rad = (double)pcl_euclid(a.x, a.y, a.z, b.x, b.y, b.z);
        }
        d.vmed[it] = make_float4(mx, my, mz, 0.0f);
        d.vrad[it] = rad;
        d.vkept[it] = valid ? nkept : 0;
      }
      __syncwarp();
      continue;
    }
    // kept rank among kept points -> output slot
    int ifirst = -1, ilast = -1;
    for (int j = lane; j < n; j += 32) {
      const int rj = srank[w][j];
      if (rj < 0) continue;
      int kr = 0;
      for (int k = 0; k < n; ++k) {
        const int rk = srank[w][k];
        kr += (rk >= 0 && rk < rj);
      }
      d.kept[off + kr] = P[j];
      if (kr == 0) ifirst = j;
      if (kr == nkept - 1) ilast = j;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const int a = __shfl_xor_sync(0xffffffffu, ifirst, o);
      const int b = __shfl_xor_sync(0xffffffffu, ilast, o);
      ifirst = max(ifirst, a);
      ilast = max(ilast, b);
    }
    if (lane == 0) {
      double rad = 0.0;
      if (valid) {
        const float4 a = P[ifirst], b = P[ilast];
        rad = (double)pcl_euclid(a.x, a.y, a.z, b.x, b.y, b.z);
      }
      d.vmed[it] = make_float4(mx, my, mz, 0.0f);
      d.vrad[it] = rad;
      d.vkept[it] = valid ? nkept : 0;
    }
    __syncwarp();
  }
}

// Rows of kVtxCap < n <= kWideCap points (the near trees of wide clusters),
// which k_vertex lists: one block of 256 threads per row at a time, the
// listed rows spread over the blocks, everything in shared memory.  Each
// axis median is element `mid` of the order by (value, index) -- the
// element the rank count selects -- by a block bitonic sort of 64-bit
// (order-preserving value key, index) words; the kept points' (z, y, x,
// column) order by a block bitonic sort of their indices with the same
// comparison as the narrow path.
constexpr int kWideThreads = 256;
__device__ __forceinline__ void block_bitonic_u64(unsigned long long* a, int m) {
  for (int k = 2; k <= m; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < (m >> 1); t += blockDim.x) {
        const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i | j;
        const unsigned long long x = a[i], y = a[l];
        const bool up = (i & k) == 0;
        if (up ? (y < x) : (x < y)) {
          a[i] = y;
          a[l] = x;
        }
      }
      __syncthreads();
    }
  }
}
constexpr size_t kWideSmem = (size_t)kWideCap * (sizeof(float4) + sizeof(unsigned long long));
__global__ void __launch_bounds__(kWideThreads) k_vertex_wide(Dev d, KParams kp) {
  extern __shared__ __align__(16) unsigned char wsm[];  // P [kWideCap], key [kWideCap]
  float4* P = reinterpret_cast<float4*>(wsm);
  unsigned long long* key =
      reinterpret_cast<unsigned long long*>(wsm + (size_t)kWideCap * sizeof(float4));
  __shared__ float med[3];
  __shared__ int s_kept[kWideThreads / 32];
  const TreeView tree = tree_view(d.in, d.W);
  // the wide items k_vertex listed, one per block at a time (the list's
  // order does not matter: each item writes only its own outputs)
  const int nwide = min(d.cnt->n_wide, d.cap_cand * d.H);
  {
    for (int q = blockIdx.x; q < nwide; q += gridDim.x) {
      const int it = d.wide_list[q];
      const int n = d.rc[it];
      const int off = d.roff[it];
      for (int j = threadIdx.x; j < n; j += blockDim.x) P[j] = tree[d.bucket[off + j]];
      int m = 1;
      while (m < n) m <<= 1;
      __syncthreads();
      const int mid = n / 2;
      for (int axis = 0; axis < 3; ++axis) {
        for (int j = threadIdx.x; j < m; j += blockDim.x) {
          unsigned long long k = ~0ull;
          if (j < n) {
            const float4 a = P[j];
            k = ((unsigned long long)fkey(axis == 0 ? a.x : axis == 1 ? a.y : a.z) << 32) |
                (uint32_t)j;
          }
          key[j] = k;
        }
        __syncthreads();
        block_bitonic_u64(key, m);
        if (threadIdx.x == 0) {
          const float4 a = P[(int)(uint32_t)key[mid]];
          med[axis] = axis == 0 ? a.x : axis == 1 ? a.y : a.z;
        }
        __syncthreads();
      }
      const float mx = med[0], my = med[1], mz = med[2];
      // kept flags, then the kept indices by (z, y, x, column); key holds the
      // indices (the kept ones first, n for the others) as 64-bit words
      int nk = 0;
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        bool keep = false;
        if (j < n) {
          const float4 a = P[j];
          keep = pcl_euclid(a.x, a.y, a.z, mx, my, mz) < kp.max_d_centroid;
        }
        key[j] = keep ? (unsigned long long)j : (unsigned long long)n;
        nk += keep ? 1 : 0;
      }
      nk = warp_sumi(nk);
      if ((threadIdx.x & 31) == 0) s_kept[threadIdx.x >> 5] = nk;
      __syncthreads();
      int nkept = 0;
      for (int w = 0; w < kWideThreads / 32; ++w) nkept += s_kept[w];
      auto lt = [&](int x, int y) { return x < n && (y >= n || zless(P[x], x, P[y], y)); };
      for (int k = 2; k <= m; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int t = threadIdx.x; t < (m >> 1); t += blockDim.x) {
            const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i | j;
            const int x = (int)key[i], y = (int)key[l];
            const bool up = (i & k) == 0;
            if (up ? lt(y, x) : lt(x, y)) {
              key[i] = (unsigned long long)y;
              key[l] = (unsigned long long)x;
            }
          }
          __syncthreads();
        }
      }
      for (int r = threadIdx.x; r < nkept; r += blockDim.x) d.kept[off + r] = P[(int)key[r]];
      if (threadIdx.x == 0) {
        const bool valid = nkept > 1;
        double rad = 0.0;
        if (valid) {
          const float4 a = P[(int)key[0]], b = P[(int)key[nkept - 1]];
          rad = (double)pcl_euclid(a.x, a.y, a.z, b.x, b.y, b.z);
        }
        d.vmed[it] = make_float4(mx, my, mz, 0.0f);
        d.vrad[it] = rad;
        d.vkept[it] = valid ? nkept : 0;
      }
      __syncthreads();
    }
  }
}

__global__ void k_clear_wide(Dev d) {
  if (threadIdx.x == 0) d.cnt->n_wide = 0;
}

// Per candidate (thread c): vertex count of the landmark (0 = rejected),
// its kept-point count and its cluster size, rows walked bottom (H-1) to
// top; then the landmark numbering and offsets in candidate (= label)
// order.  Single block: the counts feed the scans with no launch between.
__global__ void __launch_bounds__(1024) k_lm_scan(Dev d, KParams kp, int32_t* cand_vb,
                                                  int32_t* cand_pb) {
  __shared__ int sm[33];
  const int nc = d.cnt->n_cand;
  const int H = d.H;
  int bl = 0, bv = 0, bp = 0, bc = 0;
  for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    int nv = 0, np = 0, ncl = 0;
    if (c < nc) {
      for (int row = H - 1; row >= 0; --row) {
        const int it = c * H + row;
        ncl += d.rc[it];
        const int k = d.vkept[it];
        if (k > 0) {
          if (nv < kp.max_vertices) np += k;
          ++nv;
        }
      }
      if (nv <= kp.min_vertices) { nv = 0; np = 0; }
      if (nv > kp.max_vertices) nv = kp.max_vertices;
      if (nv == 0) ncl = 0;
      d.cand_nv[c] = nv;
    }
    int tl, tv, tp, tc;
    const int el = block_excl_scan(nv > 0 ? 1 : 0, sm, &tl);
    const int ev = block_excl_scan(nv, sm, &tv);
    const int ep = block_excl_scan(np, sm, &tp);
    const int ec = block_excl_scan(ncl, sm, &tc);
    if (c < nc) {
      const bool ok = nv > 0 && bl + el < d.cap_lm && bv + ev + nv <= d.cap_v &&
                      bp + ep + np <= d.cap_p && bc + ec + ncl <= d.cap_cluster;
      d.cand_lm[c] = ok ? bl + el : -1;
      cand_vb[c] = bv + ev;
      cand_pb[c] = bp + ep;
      if (ok) {
        const int l = bl + el;
        d.lm_tree[l] = d.cand_comp[c];
        d.lm_vbeg[l] = bv + ev;
        d.lm_cbeg[l] = bc + ec;
      } else if (nv > 0) {
        atomicOr(&d.cnt->overflow, 4);
      }
    }
    bl += tl; bv += tv; bp += tp; bc += tc;
  }
  if (threadIdx.x == 0) {
    const int nl = bl < d.cap_lm ? bl : d.cap_lm;
    d.cnt->n_lm = nl;
    d.cnt->n_v = bv < d.cap_v ? bv : d.cap_v;
    d.cnt->n_p = bp < d.cap_p ? bp : d.cap_p;
    d.cnt->n_cluster = bc < d.cap_cluster ? bc : d.cap_cluster;
    d.lm_vbeg[nl] = d.cnt->n_v;
    d.lm_pbeg[d.cnt->n_v] = d.cnt->n_p;
    d.lm_cbeg[nl] = d.cnt->n_cluster;
  }
}

// One warp per landmark candidate: vertex records, kept points and the
// cluster points (raster order) into the compact landmark arrays.
__global__ void __launch_bounds__(256) k_lm_write(Dev d, const int32_t* cand_vb,
                                                  const int32_t* cand_pb) {
  const int H = d.H;
  const int lane = threadIdx.x & 31;
  const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int c = wg; c < d.cnt->n_cand; c += nw) {
    const int l = d.cand_lm[c];
    if (l < 0) continue;
    const int nv = d.cand_nv[c];
    int vbase = cand_vb[c], pbase = cand_pb[c];
    int vi = 0;
    for (int r0 = H - 1; r0 >= 0 && vi < nv; r0 -= 32) {
      const int row = r0 - lane;
      const int it = c * H + row;
      const int k = row >= 0 ? d.vkept[it] : 0;
      const bool v = k > 0;
      const unsigned b = __ballot_sync(0xffffffffu, v);
      const int my = vi + __popc(b & ((1u << lane) - 1u));
      // kept-point prefix inside this chunk
      int kp = v && my < nv ? k : 0, incl = kp;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int pstart = pbase + incl - kp;
      if (v && my < nv) {
        const int vv = vbase + my;
        const float4 m = d.vmed[it];
        d.lm_vxyz[3 * vv] = m.x;
        d.lm_vxyz[3 * vv + 1] = m.y;
        d.lm_vxyz[3 * vv + 2] = m.z;
        d.lm_vrad[vv] = d.vrad[it];
        d.lm_vrow[vv] = row;
        d.lm_pbeg[vv] = pstart;
        d.lm_vsrc[vv] = d.roff[it];
      }
      pbase += __shfl_sync(0xffffffffu, incl, 31);
      vi += __popc(b);
    }
  }
}

// Point copies of the landmarks, spread over the whole grid: one warp per
// vertex for the kept points, one thread per bucket slot for the cluster
// points (raster order; the candidate of a slot found by binary search).
// One warp per (candidate, row) bucket instead, which needs no search, was
// measured slower (11.6 against 8.7 us per launch): the wide buckets of near
// trees leave most warps idle while a few walk long rows.
__global__ void __launch_bounds__(256) k_lm_copy(Dev d) {
  const TreeView tree = tree_view(d.in, d.W);
  const int H = d.H;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = gridDim.x * blockDim.x;
  const int nv = d.cnt->n_v;
  for (int v = gt >> 5; v < nv; v += nt >> 5) {
    const int src = d.lm_vsrc[v], dst = d.lm_pbeg[v], cnt = d.lm_pbeg[v + 1] - dst;
    for (int q = lane; q < cnt; q += 32) d.lm_pts[dst + q] = d.kept[src + q];
  }
  const int nc = d.cnt->n_cand;
  const int total = d.roff[nc * H];
  for (int q = gt; q < total; q += nt) {
    int lo = 0, hi = nc - 1;  // last candidate whose first slot <= q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (d.roff[mid * H] <= q) lo = mid;
      else hi = mid - 1;
    }
    const int l = d.cand_lm[lo];
    if (l < 0) continue;
    d.lm_cpts[d.lm_cbeg[l] + (q - d.roff[lo * H])] = tree[d.bucket[q]];
  }
}

}  // namespace

// k_vertex alone over the last keyframe's (component, row) buckets, for timing.
int launch_vertex_kernel(const Dev& d, const KParams& kp, cudaStream_t st) {
  k_clear_wide<<<1, 32, 0, st>>>(d);  // repeated timing runs: the list starts empty each time
  k_vertex<<<4 * 152, kVtxWarps * 32, 0, st>>>(d, kp);
  k_vertex_wide<<<152, kWideThreads, kWideSmem, st>>>(d, kp);
  return 3;
}

// The wide-row kernel's 48 KB of dynamic shared memory plus its static
// words exceed the default per-block limit: opt in once per process.
void init_trellis_attributes() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_vertex_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kWideSmem);
  done = true;
}

int launch_trellis(const Dev& d, const KParams& kp, cudaStream_t st) {
  const int N = d.N;
  const int g1k = (N + 1023) / 1024;
  const int tiles = ((d.W + kCCTile - 1) / kCCTile) * ((d.H + kCCTile - 1) / kCCTile);
  k_cc_local<<<tiles, 256, 0, st>>>(d, kp.cc_thr, kp.cc_iter_limit);
  k_cc_border<<<(cc_border_pairs(d.W, d.H) + 255) / 256 + 1, 256, 0, st>>>(d, kp.cc_thr,
                                                                          kp.cc_iter_limit);
  k_cc_flatten<<<g1k, kCCThreads, 0, st>>>(d);
  k_cc_rank<<<g1k, kCCThreads, 0, st>>>(d);
  k_cc_label<<<g1k, kCCThreads, 0, st>>>(d);
  k_cands<<<1, 1024, 0, st>>>(d, kp.min_cluster);
  // warp-per-item kernels stride over the (candidate, row) items: one wave
  // of 1216 warps on the 152 SMs, leaving room for concurrent keyframes
  const int gw = 152;
  k_rows<0><<<gw, 256, 0, st>>>(d);
  k_rowscan<<<1, 1024, 0, st>>>(d);
  k_rows<1><<<gw, 256, 0, st>>>(d);
  // k_vertex on twice that many warps: a (component, row) item is a long
  // dependent chain, and fewer items per warp shorten the keyframe (measured
  // 1.5 % more keyframes/s in the batch than 2 * 152 blocks)
  // (the wide list starts empty: k_begin cleared the counters)
  k_vertex<<<4 * gw, kVtxWarps * 32, 0, st>>>(d, kp);
  k_vertex_wide<<<gw, kWideThreads, kWideSmem, st>>>(d, kp);
  // scratch for the landmark offsets lives in the (now unused) rank array
  int32_t* cand_vb = reinterpret_cast<int32_t*>(d.rank);
  int32_t* cand_pb = cand_vb + d.cap_cand;
  k_lm_scan<<<1, 1024, 0, st>>>(d, kp, cand_vb, cand_pb);
  // the kept-point copies spread over the grid (k_lm_copy) rather than in
  // the record-writing warps: the merged kernel walked each candidate's
  // vertices one after the other and ran the Trellis 23 us longer
  k_lm_write<<<32, 256, 0, st>>>(d, cand_vb, cand_pb);
  k_lm_copy<<<gw, 256, 0, st>>>(d);
  return 14;
}

}  // namespace sg
