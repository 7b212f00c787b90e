// cylqueue.cu — the point-level cylinder fit of a keyframe (cyl_mode 1, and
// the RANSAC fallback pass of cyl_mode 2) as one persistent work-queue
// kernel: inlier counting of the tree's hypotheses, the best hypothesis, and
// the least-squares refinement, over trees of very uneven size.
//
// The reference fits its trees one after the other (sloam.cpp:418-434, one
// Cylinder per landmark).  Here the trees are queued largest first and
// blocks take work items from one atomic counter.  A tree of at most
// kSplitChunks chunks (chunk = `cyl_chunk_points` points; one chunk in the
// fallback pass, whose one or two trees would otherwise leave most blocks
// idle) is one item: one block counts, selects and refines it with no wait.
// A larger tree is cut
// into chunks, and every (phase, chunk) of it is an item:
//   phase 0        count the inliers of all K hypotheses on the chunk
//                  (ballot + popcount per 32 points, integer atomics);
//   phase 1..L     one LS iteration: the 20 normal-equation sums of one
//                  1024-point slice of the tree.
// The block that completes the last chunk of (tree, phase) finishes the
// phase: after phase 0 the best hypothesis (most inliers, lowest index on
// ties) and the initial model; after an LS phase the slice sums in slice
// order, the FP64 5x5 solve on one warp and the model update; after the
// last phase the cylinder record.  Both kinds of tree use the same slice
// sums (each thread's 4 points in FP32 in a fixed order, warp-shuffle sums,
// the warps in order) added in slice order in FP64, so the result depends
// neither on the split, nor on which block ran which item, the chunk size,
// the hypothesis tile or the block count.
//
// Item order: the split trees' phase-0 chunks, then the whole trees, then
// the split trees' phases 1..L, so the phase-0 finishers have run by the
// time their trees' LS items are claimed.  An item of phase p > 0 waits until
// its tree has finished phase p - 1.  Items are claimed in increasing order
// and a block never waits while it holds an unfinished item, so the lowest
// unfinished item always belongs to a running block whose dependencies are
// done: the waits end.  Each wait is still bounded (kQueueWaitPolls); when
// one runs out the kernel sets the counters' error flag and its blocks stop.
#include "cylinder.cuh"
#include "internal.h"
#include "scan_util.cuh"

namespace sg {

namespace {

constexpr int kQThreads = 256;
constexpr int kQWarps = kQThreads / 32;
constexpr int kSlicePer = 4;              // points per thread of one LS slice
constexpr int kSlice = kSlicePer * kQThreads;  // points of one LS slice
constexpr int kSplitChunks = 4;           // larger trees are split over blocks
constexpr int kQSortCap = 4096;           // trees per keyframe the queue orders
constexpr long long kQueueWaitPolls = 1ll << 22;  // x ~100 ns: about 0.4 s

__device__ __forceinline__ bool queue_eligible(const Dev& d, const CylD& c, int l,
                                               const int32_t* only) {
  return c.stage == 1 && c.radius != -1.0 && (!only || only[l]);
}

// One block: the eligible trees with points, ordered by decreasing point
// count (ties by index); the split trees (more than kSplitChunks chunks)
// come first, with their chunk and slice offsets, then the whole trees; the
// per-tree phase state of the split trees is reset.
__global__ void __launch_bounds__(1024) k_cyl_queue_prep(Dev d, KParams kp,
                                                         const int32_t* __restrict__ only,
                                                         int chunk) {
  __shared__ unsigned long long key[kQSortCap];
  __shared__ int sm[33];
  const int nl = d.cnt->n_lm;
  QueueCtl* q = d.qctl;
  if (only && d.cnt->n_fallback == 0) {  // the learned pass kept every tree
    if (threadIdx.x == 0) {
      d.q_off[0] = 0;
      d.q_soff[0] = 0;
      q->tc = 0;
      q->ts = 0;
      q->nq = 0;
      q->nsplit = 0;
      q->phases = 1 + kp.ls_iters;
      q->head = 0;
    }
    return;
  }
  if (nl > kQSortCap) {
    if (threadIdx.x == 0) {
      atomicOr(&d.cnt->overflow, 64);
      q->tc = 0;
      q->ts = 0;
      q->nq = 0;
      q->nsplit = 0;
      q->phases = 1;
      q->head = 0;
    }
    return;
  }
  int n2 = 1;
  while (n2 < nl) n2 <<= 1;
  for (int l = threadIdx.x; l < n2; l += blockDim.x) {
    unsigned long long k = ~0ull;
    if (l < nl) {
      const CylD c = d.cyl_all[l];
      if (queue_eligible(d, c, l, only)) {
        const float4* pts;
        const float2* uv;
        int n;
        tree_points(d, l, &pts, &n, &uv);
        if (n > 0) k = ((unsigned long long)(0xFFFFFFFFu - (uint32_t)n) << 32) | (uint32_t)l;
      }
    }
    key[l] = k;
  }
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int m = i ^ j;
        if (m > i) {
          const bool up = (i & k) == 0;
          const unsigned long long x = key[i], y = key[m];
          if ((x > y) == up) { key[i] = y; key[m] = x; }
        }
      }
      __syncthreads();
    }
  }
  const int P = 1 + kp.ls_iters;
  int base = 0, sbase = 0, nq = 0, nsplit = 0;
  for (int i0 = 0; i0 < n2; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    const bool valid = i < n2 && key[i] != ~0ull;
    const int n = valid ? (int)(0xFFFFFFFFu - (uint32_t)(key[i] >> 32)) : 0;
    const int nc = valid ? (n + chunk - 1) / chunk : 0;
    // the RANSAC pass after the learned proposals has a tree or two on 76
    // blocks: split every tree of more than one chunk, so that its counting
    // spreads over blocks (the results are the same either way)
    const bool split = nc > (only ? 1 : kSplitChunks);
    if (valid) {
      const int l = (int)(uint32_t)key[i];
      d.q_order[i] = l;
      if (split) {
        d.q_ready[l] = 0;
        for (int p = 0; p < P; ++p) d.q_done[(size_t)l * kQueuePhases + p] = 0;
      }
      if (!only) atomicAdd(&d.cnt->n_fit_pts, n);
    }
    // sizes decrease along the order: the split trees are a prefix
    int total, stotal;
    const int ex = block_excl_scan(split ? nc : 0, sm, &total);
    const int sex = block_excl_scan(split ? (n + kSlice - 1) / kSlice : 0, sm, &stotal);
    if (split) {
      d.q_off[i] = base + ex;
      d.q_soff[i] = sbase + sex;
    }
    base += total;
    sbase += stotal;
    nq += __syncthreads_count(valid);
    nsplit += __syncthreads_count(split);
  }
  if (threadIdx.x == 0) {
    d.q_off[nsplit] = base;
    d.q_soff[nsplit] = sbase;
    q->tc = base;
    q->ts = sbase;
    q->nq = nq;
    q->nsplit = nsplit;
    q->phases = P;
    q->head = 0;
    if (!only) d.cnt->n_fit = nq;
  }
}

// Final record of a refined tree (the tail of the LS refinement): the axis
// point nearest the tree's second vertex as root, the axis pointing up, the
// radius, the best hypothesis's inlier count.
__device__ void queue_write_cylinder(Dev& d, int l, const double* st, int best_cnt) {
  CylD c = d.cyl_all[l];
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

// Dynamic shared memory of the worker: the hypothesis tile and the per-warp
// counts of the tile.
template <int kTile>
struct QueueSmem {
  float4 hyp[kTile];
  int cnt[kQWarps][kTile];
};

// Small per-block state in static shared memory.
struct QueueBlock {
  float red[20][kQWarps];
  double st[16];  // c(3), dir(3), r, ok, b1(3), b2(3), best count, best h
  float sf[16];   // float copies of the model and its frame (ls_frame)
  double ssum[20];
  double sxls[5];
  unsigned long long sk[kQWarps];
  float4 hyp;     // the best hypothesis's circle
  int idx, last, stop;
};

// Inlier counts of hypotheses [0, nt) staged in S.hyp over the points
// [i0, i1) of the tree, 32 points per warp at a time; lane j of each warp
// adds the count of hypothesis hb * 32 + j to acc[hb].
template <int kTile>
__device__ __forceinline__ void count_tile(const QueueSmem<kTile>& S, int nt,
                                           const float2* __restrict__ uvs, int i0, int i1,
                                           int* acc) {
  const int lane = threadIdx.x & 31;
  for (int b = i0; b < i1; b += kQThreads) {
    const int i = b + (int)threadIdx.x;
    const bool mine = i < i1;
    const float2 pu = mine ? uvs[i] : make_float2(0.f, 0.f);
#pragma unroll
    for (int hb = 0; hb < kTile / 32; ++hb) {
      if (hb * 32 >= nt) break;  // block-uniform
      const int jn = min(32, nt - hb * 32);
#pragma unroll 4
      for (int j = 0; j < jn; ++j) {
        const float4 e = S.hyp[hb * 32 + j];
        const float du = fsub(pu.x, e.x), dv = fsub(pu.y, e.y);
        const float d2 = fadd(fmul(du, du), fmul(dv, dv));
        const unsigned bal = __ballot_sync(0xffffffffu, mine && (d2 > e.z) && (d2 < e.w));
        if (lane == j) acc[hb] += __popc(bal);
      }
    }
  }
}

// Inlier counts of all K hypotheses of tree l over points [i0, i1), tile by
// tile: `whole` keeps the best key (most inliers, lowest index) of the
// block, otherwise the counts go to hyp_cnt by atomics.
template <int kTile>
__device__ unsigned long long count_points(const float4* __restrict__ hyp_tab,
                                           int* __restrict__ cnt_tab, QueueSmem<kTile>& S,
                                           int l, int K, const float2* __restrict__ uvs, int i0,
                                           int i1, bool whole) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned long long best = 0ull;
  for (int t0 = 0; t0 < K; t0 += kTile) {
    const int nt = min(kTile, K - t0);
    for (int i = tid; i < kTile; i += kQThreads)
      S.hyp[i] = i < nt ? hyp_tab[(size_t)l * K + t0 + i] : make_float4(0.f, 0.f, 0.f, -1.f);
    __syncthreads();
    int acc[kTile / 32];
#pragma unroll
    for (int hb = 0; hb < kTile / 32; ++hb) acc[hb] = 0;
    count_tile<kTile>(S, nt, uvs, i0, i1, acc);
#pragma unroll
    for (int hb = 0; hb < kTile / 32; ++hb) S.cnt[w][hb * 32 + lane] = acc[hb];
    __syncthreads();
    for (int h = tid; h < nt; h += kQThreads) {
      int s = 0;
#pragma unroll
      for (int k = 0; k < kQWarps; ++k) s += S.cnt[k][h];
      if (!whole) {
        if (s) atomicAdd(cnt_tab + (size_t)l * K + t0 + h, s);
      } else if (s > 0) {
        const unsigned long long kk = ((unsigned long long)s << 32) |
                                      (unsigned long long)(0xFFFFFFFFu - (uint32_t)(t0 + h));
        best = kk > best ? kk : best;
      }
    }
    __syncthreads();
  }
  return best;
}

// The 20 LS sums of slice `sl` of the tree (points sl*1024 .. +1023 that are
// inliers of the fixed hypothesis B.hyp), for the model in B.sf: FP32 per
// point (each thread's 4 points in order), warp-shuffle sums, the warps
// summed in order; threads 0..19 return sum j = tid, other threads 0.
__device__ __forceinline__ float slice_sums(QueueBlock& B, const float4* __restrict__ pts,
                                            const float2* __restrict__ uvs, int n, int sl) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const float* sf = B.sf;
  const float4 H = B.hyp;
  float acc[20];
#pragma unroll
  for (int j = 0; j < 20; ++j) acc[j] = 0.f;
#pragma unroll
  for (int k = 0; k < kSlicePer; ++k) {
    const int i = sl * kSlice + k * kQThreads + tid;
    bool use = i < n;
    float4 qp = make_float4(0.f, 0.f, 0.f, 0.f);
    if (use) {
      const float2 uv = uvs[i];
      const float du = fsub(uv.x, H.x), dv = fsub(uv.y, H.y);
      const float d2 = fadd(fmul(du, du), fmul(dv, dv));
      use = (d2 > H.z) & (d2 < H.w);
      if (use) qp = pts[i];
    }
    const float wx = qp.x - sf[0], wy = qp.y - sf[1], wz = qp.z - sf[2];
    const float dx = sf[3], dy = sf[4], dz = sf[5];
    const float wd = wx * dx + wy * dy + wz * dz;
    const float px_ = wx - wd * dx, py_ = wy - wd * dy, pz_ = wz - wd * dz;
    const float rho = sqrtf(px_ * px_ + py_ * py_ + pz_ * pz_);
    if (use && rho > 0.f) {
      const float res = rho - sf[12];
      const float a1 = (px_ * sf[6] + py_ * sf[7] + pz_ * sf[8]) / rho;
      const float a2 = (px_ * sf[9] + py_ * sf[10] + pz_ * sf[11]) / rho;
      const float J[5] = {-a1, -a2, -wd * a1, -wd * a2, -1.0f};
      int m = 0;
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = a; b < 5; ++b) acc[m++] += J[a] * J[b];
#pragma unroll
      for (int a = 0; a < 5; ++a) acc[15 + a] += J[a] * res;
    }
  }
#pragma unroll
  for (int j = 0; j < 20; ++j) {
    const float v = warp_sum(acc[j]);
    if (lane == 0) B.red[j][w] = v;
  }
  __syncthreads();
  float t = 0.0f;
  if (tid < 20)
    for (int q2 = 0; q2 < kQWarps; ++q2) t += B.red[tid][q2];
  __syncthreads();
  return t;
}

// The tree's initial model from its best hypothesis key into B.st, B.sf
// and B.hyp.  Thread 0.
__device__ void init_model(Dev& d, const KParams& kp, QueueBlock& B, int l, int n,
                           const float2* __restrict__ uvs, unsigned long long best) {
  const int K = kp.K;
  const int h = (int)(0xFFFFFFFFu - (uint32_t)(best & 0xffffffffull));
  const CylD cy = d.cyl_all[l];
  const CylFrame f = make_frame(d, cy);
  const float4 e = d.hyp[(size_t)l * K + h];
  double* st = B.st;
  st[0] = f.ox + (double)e.x * f.e1x + (double)e.y * f.e2x;
  st[1] = f.oy + (double)e.x * f.e1y + (double)e.y * f.e2y;
  st[2] = f.oz + (double)e.x * f.e1z + (double)e.y * f.e2z;
  const double an = sqrt((double)f.ax * f.ax + (double)f.ay * f.ay + (double)f.az * f.az);
  st[3] = f.ax / an; st[4] = f.ay / an; st[5] = f.az / an;
  const Hyp Hh = make_hyp(kp, h, cy.id, n, [&](uint32_t i) { return uvs[i]; });
  st[6] = Hh.r;
  st[7] = 1.0;
  st[14] = (double)(int)(best >> 32);
  st[15] = (double)h;
  ls_frame(st, B.sf);
  B.hyp = e;
}

// The 5x5 normal equations in B.ssum solved on warp 0, the model updated
// on the same warp (three components at a time); st[7] = 0 when the solve
// fails.  Called by all of warp 0.
__device__ __noinline__ void solve_update(QueueBlock& B) {
  const int lane = threadIdx.x & 31;
  const bool solved = warp_chol_solve<5>(B.ssum, B.ssum + 15, B.sxls);
  __syncwarp();
  if (solved) {
    warp_model_update(B.st, B.sxls, B.sf);
  } else {
    if (lane == 0) B.st[7] = 0.0;
    __syncwarp();
  }
}

__device__ __forceinline__ unsigned long long block_max_key(QueueBlock& B, unsigned long long v) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x > v ? x : v;
  }
  if (lane == 0) B.sk[w] = v;
  __syncthreads();
  unsigned long long m = B.sk[0];
  for (int k = 1; k < kQWarps; ++k) m = B.sk[k] > m ? B.sk[k] : m;
  __syncthreads();
  return m;
}

template <int kTile>
__global__ void __launch_bounds__(kQThreads, 4) k_cyl_queue(Dev d, KParams kp) {
  extern __shared__ __align__(16) unsigned char q_smem[];
  QueueSmem<kTile>& S = *reinterpret_cast<QueueSmem<kTile>*>(q_smem);
  __shared__ QueueBlock B;
  const int kC = kp.q_chunk;  // points per counting item
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  QueueCtl* q = d.qctl;
  const int TC = q->tc, TS = q->ts, P = q->phases, nq = q->nq, nsplit = q->nsplit;
  const int K = kp.K;
  const float4* __restrict__ hyp_tab = d.hyp;
  int* __restrict__ cnt_tab = d.hyp_cnt;
  const int nwhole = nq - nsplit;
  const long long total = (long long)TC + nwhole + (long long)TS * (P - 1);
  for (;;) {
    if (tid == 0) {
      B.idx = atomicAdd(&q->head, 1);
      B.stop = 0;
    }
    __syncthreads();
    const int idx = B.idx;
    if ((long long)idx >= total) break;  // block-uniform
    if (idx >= TC && idx < TC + nwhole) {
      // ---------------- a whole tree: count, best, LS, record
      const int l = d.q_order[nsplit + (idx - TC)];
      const float4* pts;
      const float2* uvs;
      int n;
      tree_points(d, l, &pts, &n, &uvs);
      const unsigned long long best =
          block_max_key(B, count_points<kTile>(hyp_tab, cnt_tab, S, l, K, uvs, 0, n, true));
      if (tid == 0) d.cyl_best[l] = best;
      if (best != 0ull) {
        if (tid == 0) init_model(d, kp, B, l, n, uvs, best);
        __syncthreads();
        const int ns = (n + kSlice - 1) / kSlice;
        for (int p = 1; p < P; ++p) {
          if (B.st[7] == 0.0) break;  // block-uniform
          double t = 0.0;
          for (int sl = 0; sl < ns; ++sl) t += (double)slice_sums(B, pts, uvs, n, sl);
          if (tid < 20) B.ssum[tid] = t;
          __syncthreads();
          if (w == 0) solve_update(B);
          __syncthreads();
        }
        if (tid == 0) queue_write_cylinder(d, l, B.st, (int)B.st[14]);
      }
      __syncthreads();
      continue;
    }
    // ---------------- one chunk (counting) or slice (LS) of a split tree
    const int p = idx < TC ? 0 : 1 + (idx - TC - nwhole) / TS;
    const int r = idx < TC ? idx : (idx - TC - nwhole) % TS;
    const int32_t* offs = p == 0 ? d.q_off : d.q_soff;
    int lo = 0, hi = nsplit - 1;  // the tree whose chunks / slices hold r
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (offs[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    const int l = d.q_order[lo];
    const int c0 = d.q_off[lo], nc = d.q_off[lo + 1] - c0;   // counting chunks
    const int s0 = d.q_soff[lo], ns = d.q_soff[lo + 1] - s0;  // LS slices
    const int c = r - offs[lo];  // this item's chunk (p == 0) or slice (p > 0)
    const int n_items = p == 0 ? nc : ns;
    const float4* pts;
    const float2* uvs;
    int n;
    tree_points(d, l, &pts, &n, &uvs);
    if (p > 0) {
      // the tree must have finished phase p - 1
      if (tid == 0) {
        long long it = 0;
        while (*reinterpret_cast<volatile int*>(d.q_ready + l) < p) {
          if (++it > kQueueWaitPolls || *reinterpret_cast<volatile int*>(&d.cnt->queue_err)) {
            atomicOr(&d.cnt->queue_err, 1);
            B.stop = 1;
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
      }
      __syncthreads();
      if (B.stop) break;
    }
    if (p == 0) {
      // ---- inlier counts of the chunk for every hypothesis of the tree
      count_points<kTile>(hyp_tab, cnt_tab, S, l, K, uvs, c * kC, min(n, c * kC + kC), false);
    } else {
      const double* gst = d.q_st + (size_t)l * 16;
      const bool live = __ldcg(gst + 15) >= 0.0 && __ldcg(gst + 7) != 0.0;
      if (live) {
        if (tid < 13) B.sf[tid] = __ldcg(d.q_sf + (size_t)l * 16 + tid);
        if (tid == 0) B.hyp = __ldcg(d.q_hyp + l);
        __syncthreads();
        // ---- one LS iteration's sums over the slice
        const float t = slice_sums(B, pts, uvs, n, c);
        if (tid < 20) d.q_part[(size_t)(s0 + c) * 20 + tid] = t;
      }
    }
    // ---- arrival; the last chunk's block finishes the phase for the tree
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      B.last = atomicAdd(d.q_done + (size_t)l * kQueuePhases + p, 1) == n_items - 1;
    }
    __syncthreads();
    if (B.last) {
      __threadfence();
      if (p == 0) {
        unsigned long long best = 0ull;
        for (int h = tid; h < K; h += kQThreads) {
          const int cn = __ldcg(cnt_tab + (size_t)l * K + h);
          if (cn > 0) {
            const unsigned long long kk =
                ((unsigned long long)cn << 32) | (unsigned long long)(0xFFFFFFFFu - (uint32_t)h);
            best = kk > best ? kk : best;
          }
        }
        best = block_max_key(B, best);
        if (tid == 0) {
          d.cyl_best[l] = best;
          double* gst = d.q_st + (size_t)l * 16;
          if (best == 0ull) {
            gst[7] = 0.0;
            gst[15] = -1.0;  // no hypothesis with inliers: the vertex-line model stays
          } else {
            init_model(d, kp, B, l, n, uvs, best);
            for (int j = 0; j < 16; ++j) gst[j] = B.st[j];
            for (int j = 0; j < 13; ++j) d.q_sf[(size_t)l * 16 + j] = B.sf[j];
            d.q_hyp[l] = B.hyp;
            if (P == 1) queue_write_cylinder(d, l, B.st, (int)(best >> 32));
          }
        }
      } else {
        if (tid < 16) B.st[tid] = __ldcg(d.q_st + (size_t)l * 16 + tid);
        __syncthreads();
        const bool has_model = B.st[15] >= 0.0;
        if (has_model && B.st[7] != 0.0 && w == 0) {
          if (lane < 20) {
            double t = 0.0;
            for (int k = 0; k < ns; ++k)
              t += (double)__ldcg(d.q_part + (size_t)(s0 + k) * 20 + lane);
            B.ssum[lane] = t;
          }
          __syncwarp();
          solve_update(B);
          if (lane == 0) {
            double* gst = d.q_st + (size_t)l * 16;
            for (int j = 0; j < 16; ++j) gst[j] = B.st[j];
            for (int j = 0; j < 13; ++j) d.q_sf[(size_t)l * 16 + j] = B.sf[j];
          }
        }
        __syncthreads();
        if (tid == 0 && has_model && p == P - 1) queue_write_cylinder(d, l, B.st, (int)B.st[14]);
      }
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        atomicExch(d.q_ready + l, p + 1);
      }
    }
    __syncthreads();
  }
}

template <int kTile>
void set_queue_attr() {
  cudaFuncSetAttribute(k_cyl_queue<kTile>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(QueueSmem<kTile>));
}

template <int kTile>
void launch_queue_t(const Dev& d, const KParams& kp, int blocks, cudaStream_t st) {
  k_cyl_queue<kTile><<<blocks, kQThreads, sizeof(QueueSmem<kTile>), st>>>(d, kp);
}

bool launch_queue_tile(const Dev& d, const KParams& kp, int tile, int blocks, cudaStream_t st) {
  switch (tile) {
    case 64: launch_queue_t<64>(d, kp, blocks, st); return true;
    case 128: launch_queue_t<128>(d, kp, blocks, st); return true;
    case 256: launch_queue_t<256>(d, kp, blocks, st); return true;
    case 512: launch_queue_t<512>(d, kp, blocks, st); return true;
    case 1024: launch_queue_t<1024>(d, kp, blocks, st); return true;
  }
  return false;
}

}  // namespace

void init_queue_attributes() {
  set_queue_attr<64>();
  set_queue_attr<128>();
  set_queue_attr<256>();
  set_queue_attr<512>();
  set_queue_attr<1024>();
}

bool queue_shape_valid(int chunk_points, int hyp_tile) {
  const bool c = chunk_points == 256 || chunk_points == 512 || chunk_points == 1024;
  const bool t = hyp_tile == 64 || hyp_tile == 128 || hyp_tile == 256 || hyp_tile == 512 ||
                 hyp_tile == 1024;
  return c && t;
}

// Counting, best hypothesis and LS refinement of the trees `only` marks
// (every eligible tree when NULL), from the hypothesis table of
// k_cyl_hypgen.  Two launches: the ordering and the persistent queue.
int launch_cyl_queue(const Dev& d, const KParams& kp, const int32_t* only, cudaStream_t st) {
  k_cyl_queue_prep<<<1, 1024, 0, st>>>(d, kp, only, kp.q_chunk);
  return launch_queue_tile(d, kp, kp.q_tile, kp.q_blocks, st) ? 2 : 1;
}

}  // namespace sg
